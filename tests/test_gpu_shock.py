"""The shocked case: a high-pressure slab on the perturbed curvilinear
periodic lattice (cases.shock_slab), shocks and contacts running out of both
edges.  FP64 against the oracle at <= 1e-12 relative L2 (FLOW and U0), and
the two reduced-precision forms against FP64 across the discontinuities,
where the FP32 WENO weights matter most (Weno.cl:1056-2186)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import copy_arrays, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def shock_front(flow, shape):
    """Largest pressure jump between i-neighbours, averaged over j and k:
    (index of the jump, ratio of the pressures across it)."""
    from cfd_gb300 import layout
    ni, nj, nk = shape
    p = flow[1:, layout.FLOW["p"]].reshape(nk, nj, ni).mean(axis=(0, 1))
    jump = np.abs(np.roll(p, -1) - p)
    i = int(np.argmax(jump))
    hi, lo = max(p[i], p[(i + 1) % ni]), min(p[i], p[(i + 1) % ni])
    return i, hi / lo


def test_shock_fp64_matches_oracle(ctx, oracle_mod):
    from cfd_gb300 import cases, runtime
    c = cases.shock_slab(shape=(32, 8, 8))
    s = runtime.Solver(ctx, c)
    assert s.info().path == "structured"
    s.set_flow(c.arrays["flow"])
    s.step(c.dt, 5)
    flow, u0 = s.get_flow(), s.get_u0()
    s.close()
    a = copy_arrays(c.arrays)
    oracle_mod.rk3_steps(a, c.g_node, c.sd_node, c.params, c.dt, 5)
    own = slice(1, c.sd_node + 1)
    errs = {"flow": rel_l2(flow[own], a["flow"][own]), "U0": rel_l2(u0[own], a["U0"][own])}
    print("shock slab 32x8x8, 5 steps, fp64 vs oracle:", {k: f"{v:.2e}" for k, v in errs.items()})
    for k, v in errs.items():
        assert v <= TOL, f"{k}: {v:.3e}"
    i, ratio = shock_front(flow, c.shape)
    assert ratio > 1.3          # a discontinuity is present (spread over two cells at this resolution)


@pytest.mark.parametrize("precision", [1, 2])
def test_shock_reduced_forms_against_fp64(ctx, precision):
    from cfd_gb300 import cases, layout, runtime
    c = cases.shock_slab(shape=(64, 16, 16))
    res = {}
    for prec in (0, precision):
        s = runtime.Solver(ctx, c, precision=prec)
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 40)
        res[prec] = s.get_flow()
        s.close()
    own = slice(1, c.sd_node + 1)
    assert np.isfinite(res[precision][own]).all()
    errs = {}
    for name in ("rho", "p"):
        k = layout.FLOW[name]
        a, b = res[precision][own, k], res[0][own, k]
        errs[name] = (rel_l2(a, b), float(np.abs(a - b).max() / np.abs(b).max()))
    f64 = shock_front(res[0], c.shape)
    red = shock_front(res[precision], c.shape)
    print(f"shock slab 64x16x16, 40 steps, form {precision} vs fp64 (L2, Linf):",
          {k: f"{v[0]:.2e}, {v[1]:.2e}" for k, v in errs.items()}, "front fp64", f64, "reduced", red)
    assert f64[1] > 1.5 and red[0] == f64[0]
    for name, (l2, _) in errs.items():
        assert l2 <= 1e-6, f"{name}: {l2:.3e}"
