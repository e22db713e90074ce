"""The FP64 form bit for bit against the oracle.

The FP64 kernels evaluate every expression in the reference's order
(no FMA contraction) and every division, reciprocal, square root and
integer-pipe routine they use returns the IEEE result, as does the oracle
(plain C, no contraction).  The one function outside IEEE 754's correctly
rounded set on the path is the LES filter width's cube root (Viscous.cl:
1/cbrt(det)), whose last bit may differ between the device's and the
host's libm.  Without the LES term the lattice path's state after whole
steps, and the drop-in path's right-hand side, must therefore equal the
oracle's bit for bit -- inviscid (the vortex) and viscous (Taylor-Green
with the LES model off): a sharper check than the 1e-12 parity budget of
the other tests, and the one that would catch a routine off by one ulp in
rare cases."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import copy_arrays

pytestmark = pytest.mark.gpu


def _mismatch(a, b):
    d = a != b
    return f"{int(d.sum())} of {d.size} values differ; max |diff| {float(np.max(np.abs(a - b))):.3e}"


def _case(name):
    from cfd_gb300 import cases
    return cases.isentropic_vortex(n=32) if name == "vortex" else cases.taylor_green(n=24, les=0)


@pytest.mark.parametrize("name,steps", [("vortex", 5), ("tgv_viscous", 3)])
def test_lattice_steps_equal_oracle_bitwise(ctx, oracle_mod, name, steps):
    from cfd_gb300 import runtime
    c = _case(name)
    s = runtime.Solver(ctx, c)
    assert s.info().path == "structured"
    s.set_flow(c.arrays["flow"])
    s.step(c.dt, steps)
    flow, u0 = s.get_flow(), s.get_u0()
    s.close()
    a = copy_arrays(c.arrays)
    oracle_mod.rk3_steps(a, c.g_node, c.sd_node, c.params, c.dt, steps)
    own = slice(1, c.sd_node + 1)
    assert np.array_equal(u0[own], a["U0"][own]), _mismatch(u0[own], a["U0"][own])
    cols = [0, 1, 2, 3, 4, 5, 7, 8]   # u v w p t rho a e (mu is the viscous pass's output)
    assert np.array_equal(flow[own][:, cols], a["flow"][own][:, cols]), _mismatch(flow[own], a["flow"][own])


@pytest.mark.parametrize("name", ["vortex", "tgv_viscous"])
def test_dropin_rhs_equals_oracle_bitwise(ctx, oracle_mod, name):
    c = _case(name)
    dev = ctx.upload_case(c.arrays)
    own = slice(1, c.sd_node + 1)
    try:
        ctx.stage(dev, c.g_node, c.sd_node, c.params, 0, c.dt, want_L=True)
        L = ctx.download(dev, "L", np.zeros((c.g_node + 1, 5)))
    finally:
        for p in dev.values():
            ctx.free(p)
    a = copy_arrays(c.arrays)
    Lo = oracle_mod.stage(a, c.g_node, c.sd_node, c.params, 0, c.dt, want_L=True)
    assert np.array_equal(L[own], Lo[own]), _mismatch(L[own], Lo[own])
