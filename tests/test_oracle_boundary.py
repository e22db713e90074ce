"""The boundary routine (reference intialise(), Flow_Initialisation.cpp:23-1394)
restated in the oracle: against the reference's own routine compiled from
its source (oracle/_ref, where the reference checkout exists) and against
the golden vectors that build wrote (tests/golden/bc_ghostbox.npz).  Pure
copies and the reference's own formulas: bit-exact."""
from __future__ import annotations

import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "bc_ghostbox.npz"


def golden_inputs():
    from cfd_gb300 import cases, layout
    z = np.load(GOLDEN)
    n = z["in_grid"].shape[0]
    a = layout.empty_arrays(n)
    a["grid"][...] = z["in_grid"]
    a["flow"][...] = z["in_flow"]
    bc = cases.BoundaryLists(**{t: z[f"list_{t}"] for t in ("outlet", "inlet", "boundary", "wall")})
    return z, a, bc


@pytest.mark.parametrize("initial", [1, 0])
def test_boundary_fill_matches_golden(oracle_mod, initial):
    z, a, bc = golden_inputs()
    oracle_mod.boundary_fill(a, bc, float(z["mach"]), initial, int(z["sd_node"]))
    assert np.array_equal(a["flow"], z[f"out_flow_initial{initial}"])


def test_golden_covers_every_type_and_code(oracle_mod):
    z, a, bc = golden_inputs()
    loc = a["grid"]["loc"]
    for t in ("outlet", "inlet", "boundary", "wall"):
        rows = getattr(bc, t)
        assert rows.size > 0
        codes = set(loc[rows].tolist())
        assert codes & set(range(1, 7)) and codes & set(range(7, 27)), t
    assert set(loc[np.concatenate([bc.outlet, bc.inlet, bc.boundary, bc.wall])].tolist()) == set(range(1, 27))


@pytest.mark.parametrize("initial", [1, 0])
def test_boundary_fill_matches_reference_build(oracle_mod, initial):
    if not oracle_mod.ref_available():
        pytest.skip("reference build absent")
    from cfd_gb300 import cases
    c = cases.ghost_box(shape=(7, 6, 5), seed=11, bc=True)
    rng = np.random.default_rng(7)
    a = c.copy().arrays
    a["flow"][1:] = rng.uniform(0.5, 1.5, a["flow"][1:].shape)
    b = {k: v.copy() for k, v in a.items()}
    oracle_mod.boundary_fill(a, c.bc, 0.6, initial, c.sd_node)
    oracle_mod.ref_boundary_fill(b, c.bc, 0.6, initial, c.sd_node)
    assert np.array_equal(a["flow"], b["flow"])


def test_singular_wall_node_is_rejected(oracle_mod):
    z, a, bc = golden_inputs()
    a["grid"]["ID"][bc.wall[0]] = 10        # the reference's singular-node marker
    before = a["flow"].copy()
    with pytest.raises(ValueError):
        oracle_mod.boundary_fill(a, bc, 0.8, 1, int(z["sd_node"]))
    assert np.array_equal(a["flow"], before)


def test_channel_steps_with_boundary_match_reference(oracle_mod):
    """Two SSP-RK3 steps of the wall-bounded channel (lattice with ghost
    layers, wall/inlet/outlet lists), the boundary routine after every
    stage: the restatement against the reference's kernels and routine.
    FLOW is bit-identical; U0 too except on boundary rows, where the
    reference's Weno kernel reads an uninitialised branch (masked by the
    poison mode) that the next stage's U_Q overwrites."""
    if not oracle_mod.ref_available():
        pytest.skip("reference build absent")
    from cfd_gb300 import cases
    c = cases.channel(ni=12, nj=10, nk=6)
    a, b, p = c.copy().arrays, c.copy().arrays, c.copy().arrays
    oracle_mod.rk3_steps_bc(a, c.g_node, c.sd_node, c.params, c.dt, 2, c.bc)
    for _ in range(2):
        for j in range(3):
            oracle_mod.ref_stage(b, c.g_node, c.sd_node, c.params, j, c.dt)
            oracle_mod.ref_boundary_fill(b, c.bc, c.params.mach, 1, c.sd_node)
    oracle_mod.set_poison(True)
    try:
        oracle_mod.rk3_steps_bc(p, c.g_node, c.sd_node, c.params, c.dt, 2, c.bc)
    finally:
        oracle_mod.set_poison(False)
    assert np.array_equal(a["flow"], b["flow"])
    for k in ("U1", "U2"):
        assert np.array_equal(a[k], b[k])
    defined = np.isfinite(p["U0"]).all(axis=1)
    assert defined.sum() > 0.8 * c.g_node
    assert np.array_equal(a["U0"][defined], b["U0"][defined])
    undefined_locs = set(c.arrays["grid"]["loc"][~defined].tolist())
    assert undefined_locs <= {1, 3}
