"""Resident solver (face-based structured path and gather path) on the GPU
against the oracle, plus size-independent properties at the benchmark sizes.
FP64 tolerance: relative L2 <= 1e-12.  Mixed precision: <= 1e-6 against FP64."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import copy_arrays, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def make(kind, **kw):
    from cfd_gb300 import cases
    if kind == "vortex":
        return cases.isentropic_vortex(**kw)
    if kind == "tgv":
        return cases.taylor_green(**kw)
    return cases.ghost_box(**kw)


@pytest.mark.parametrize("kind,kw,path", [
    ("vortex", dict(n=16, shape=(16, 12, 10)), "structured"),
    ("tgv", dict(n=12, shape=(12, 10, 14)), "structured"),
    ("tgv", dict(n=9, shape=(9, 1, 7)), "structured"),
    ("box", dict(shape=(8, 7, 6), seed=2), "gather"),
])
def test_stage_rhs_matches_oracle(ctx, oracle_mod, kind, kw, path):
    from cfd_gb300 import runtime
    c = make(kind, **kw)
    s = runtime.Solver(ctx, c)
    assert s.info().path == path
    s.set_flow(c.arrays["flow"])
    a = copy_arrays(c.arrays)
    own = np.arange(1, c.sd_node + 1)
    stages = 1 if kind == "box" else 3
    if kind == "box":
        P = copy_arrays(c.arrays)
        oracle_mod.set_poison(True)
        try:
            oracle_mod.stage(P, c.g_node, c.sd_node, c.params, 0, c.dt)
        finally:
            oracle_mod.set_poison(False)
        own = own[np.isfinite(P["U1"][own]).all(axis=1)]
    for j in range(stages):
        Lg = s.stage(j, c.dt)
        Lo = oracle_mod.stage(a, c.g_node, c.sd_node, c.params, j, c.dt, want_L=True)
        assert rel_l2(Lg[own], Lo[own]) <= TOL, f"stage {j} L"
    flow = s.get_flow()
    assert rel_l2(flow[own], a["flow"][own]) <= TOL
    s.close()


@pytest.mark.parametrize("kind,kw,force", [
    ("vortex", dict(n=12), -1),
    ("tgv", dict(n=10), -1),
    ("tgv", dict(n=10), 0),
])
def test_steps_match_oracle(ctx, oracle_mod, kind, kw, force):
    from cfd_gb300 import runtime
    c = make(kind, **kw)
    s = runtime.Solver(ctx, c, force_path=force)
    s.set_flow(c.arrays["flow"])
    s.step(c.dt, 5)
    a = copy_arrays(c.arrays)
    oracle_mod.rk3_steps(a, c.g_node, c.sd_node, c.params, c.dt, 5)
    own = np.arange(1, c.sd_node + 1)
    assert rel_l2(s.get_flow()[own], a["flow"][own]) <= TOL
    assert rel_l2(s.get_u0()[own], a["U0"][own]) <= TOL
    s.close()


def test_structured_and_gather_paths_agree_at_64cubed(ctx):
    """Full configuration size (64^3 vortex): two independent GPU paths."""
    from cfd_gb300 import runtime
    c = make("vortex", n=64)
    out = []
    for force in (1, 0):
        s = runtime.Solver(ctx, c, force_path=force)
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 2)
        out.append(s.get_u0()[1:])
        s.close()
    assert rel_l2(out[0], out[1]) <= TOL


@pytest.mark.parametrize("kind,n", [("vortex", 64), ("tgv", 128)])
def test_conservation_at_full_size(ctx, kind, n):
    """Periodic conservative form: sum of U over the domain is invariant
    (face fluxes telescope; Fv[0] = 0), for mass, momentum and energy in
    the inviscid vortex and mass in the viscous TGV."""
    from cfd_gb300 import runtime
    c = make(kind, n=n)
    s = runtime.Solver(ctx, c)
    s.set_flow(c.arrays["flow"])
    s.step(c.dt, 1)
    u_a = s.get_u0()[1:].sum(axis=0)
    s.step(c.dt, 3)
    u_b = s.get_u0()[1:].sum(axis=0)
    comps = range(5) if kind == "vortex" else [0]
    for q in comps:
        scale = np.abs(s.get_u0()[1:, q]).sum()
        assert abs(u_b[q] - u_a[q]) <= 1e-12 * scale, q
    s.close()


def test_free_stream_preserved_at_64cubed(ctx):
    from cfd_gb300 import runtime
    c = make("vortex", n=64)
    f = c.arrays["flow"]
    f[1:, 0], f[1:, 1], f[1:, 2], f[1:, 3], f[1:, 5] = 0.5, 0.1, -0.2, 1.0, 1.0
    s = runtime.Solver(ctx, c)
    s.set_flow(f)
    L = s.stage(0, c.dt)
    assert np.abs(L[1:]).max() < 1e-12
    s.close()


def test_mixed_precision_error_budget(ctx):
    """Characteristic projection, WENO and LLF in FP32, state/RK/metric
    terms FP64: relative L2 of U after 10 steps <= 1e-6 against FP64."""
    from cfd_gb300 import runtime
    c = make("tgv", n=32)
    res = []
    for prec in (0, 1):
        s = runtime.Solver(ctx, c, precision=prec)
        assert s.info().precision == ("mixed" if prec else "fp64")
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 10)
        res.append(s.get_u0()[1:])
        s.close()
    err = rel_l2(res[1], res[0])
    assert err <= 1e-6, err


def test_mixed_precision_rejected_on_gather_path(ctx):
    from cfd_gb300 import abi, runtime
    c = make("box", shape=(6, 6, 6))
    with pytest.raises(abi.CfdError) as e:
        runtime.Solver(ctx, c, precision=1)
    assert e.value.status == abi.EUNSUPPORTED


def test_config1_vortex_64_rhs_and_100_steps(ctx, oracle_mod):
    """The 64^3 isentropic vortex at its full size: the RHS of the 64^3 vortex against the
    oracle, then 100 SSP-RK3 steps of the face-based path against the drop-in
    (gather) path, an independent GPU implementation of the same kernels."""
    from cfd_gb300 import runtime
    c = make("vortex", n=64)
    s = runtime.Solver(ctx, c)
    s.set_flow(c.arrays["flow"])
    Lg = s.stage(0, c.dt)
    a = copy_arrays(c.arrays)
    Lo = oracle_mod.stage(a, c.g_node, c.sd_node, c.params, 0, c.dt, want_L=True)
    own = slice(1, c.sd_node + 1)
    assert rel_l2(Lg[own], Lo[own]) <= TOL
    s.close()
    out = []
    for force in (1, 0):
        s = runtime.Solver(ctx, c, force_path=force)
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 100)
        out.append((s.get_flow()[own], s.get_u0()[own]))
        s.close()
    assert rel_l2(out[0][0], out[1][0]) <= TOL
    assert rel_l2(out[0][1], out[1][1]) <= TOL
    m0 = c.arrays["det"][own] @ c.arrays["flow"][own][:, 5]
    assert abs(out[0][1][:, 0].sum() - m0) <= 1e-12 * m0        # mass conserved over 100 steps


def test_tgv_kinetic_energy_and_enstrophy_mixed_vs_fp64(ctx):
    """The Taylor-Green diagnostics on a reduced grid: kinetic energy and enstrophy
    of the mixed form track the FP64 form to within 1e-6 relative."""
    from cfd_gb300 import diagnostics, runtime
    c = make("tgv", n=24)
    hist = []
    for prec in (0, 1):
        s = runtime.Solver(ctx, c, precision=prec)
        s.set_flow(c.arrays["flow"])
        h = []
        for _ in range(4):
            s.step(c.dt, 5)
            h.append(diagnostics.kinetic_energy_enstrophy(s.get_flow(), c.arrays["metric"], c.arrays["det"], c.shape))
        hist.append(np.array(h))
        s.close()
    err = np.abs(hist[1] - hist[0]) / np.abs(hist[0])
    assert err.max() <= 1e-6, err
    assert hist[0][-1, 0] < hist[0][0, 0]                  # kinetic energy decays (viscous + SGS)
