"""The face-pass tuners of the lattice solvers -- the face-tile widths of the
mixed and split forms, the FP64 form's register budgets: the choices they
make are valid candidates, and every candidate gives the same bits (only the
staging or the register allocation differs between them)."""
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


def test_fp64_face_budgets_change_no_bit(ctx, oracle_mod):
    """The FP64 face passes' register budgets (blocks per SM, tuned per
    direction at creation): every budget gives the same bits, equal to the
    oracle's (an inviscid case: no LES cube root)."""
    from cfd_gb300 import abi, cases, runtime
    from helpers import copy_arrays
    c = cases.isentropic_vortex(n=20, shape=(20, 18, 22))
    s = runtime.Solver(ctx, c)
    assert all(b in (2, 3, 4) for b in s.info().face_blocks)
    assert s.info().face_tiles == (0, 0)
    s.close()
    a = copy_arrays(c.arrays)
    oracle_mod.rk3_steps(a, c.g_node, c.sd_node, c.params, c.dt, 2)
    own = slice(1, c.sd_node + 1)
    for b in (2, 3, 4):
        s = runtime.Solver(ctx, c)
        s.set_face_blocks(b, b, b)
        assert s.info().face_blocks == (b, b, b)
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 2)
        assert np.array_equal(s.get_u0()[own], a["U0"][own]), b
        s.close()
    s = runtime.Solver(ctx, c, precision=1)
    with pytest.raises(abi.CfdError) as e:
        s.set_face_blocks(3, 3, 3)
    assert e.value.status == abi.EUNSUPPORTED
    assert s.info().face_blocks == (0, 0, 0)
    s.close()
