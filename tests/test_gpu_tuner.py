"""The face-tile tuner of the mixed and split lattice solvers: the widths it
picks are valid candidates, and every width gives the same bits (only the
shared-memory staging differs between them)."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [1, 2])
def test_face_tile_widths_change_no_bit(ctx, precision):
    from cfd_gb300 import cases, runtime
    c = cases.taylor_green(n=20, shape=(20, 18, 22))
    s = runtime.Solver(ctx, c, precision=precision)
    ti, tjk = s.info().face_tiles
    assert ti in (32, 64, 128) and tjk in (8, 16, 32)
    s.close()
    ref = None
    for ti, tjk in itertools.product((32, 64, 128), (8, 16, 32)):
        s = runtime.Solver(ctx, c, precision=precision)
        s.set_face_tiles(ti, tjk)
        assert s.info().face_tiles == (ti, tjk)
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 2)
        u = s.get_u0()
        s.close()
        if ref is None:
            ref = u
        assert np.array_equal(u, ref), (ti, tjk)


def test_face_tiles_refused_for_fp64(ctx):
    from cfd_gb300 import abi, cases, runtime
    c = cases.taylor_green(n=10)
    s = runtime.Solver(ctx, c)
    assert s.info().face_tiles == (0, 0)
    with pytest.raises(abi.CfdError) as e:
        s.set_face_tiles(64, 16)
    assert e.value.status == abi.EUNSUPPORTED
    s.close()
