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


# ---------------------------------------------------------------- singular --
# The wall rules of the singular-node table (Flow_Initialisation.cpp
# :1194-1392: codes 29/30 from the node beyond singular[b][3]; ID 10 the node
# from singular[b][3] and three mirror passes; codes 33..52 the node from
# singular[b][0], then per pass the node from singular[b][k] and a mirror
# pass) and the tip rows (Solver.cpp:660-683).

SINGULAR_GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "bc_singular.npz"


def singular_golden_inputs():
    from cfd_gb300 import cases, layout
    z = np.load(SINGULAR_GOLDEN)
    n = z["in_grid"].shape[0]
    a = layout.empty_arrays(n)
    a["grid"][...] = z["in_grid"]
    a["flow"][...] = z["in_flow"]
    bc = cases.BoundaryLists(*(z[f"list_{t}"] for t in ("outlet", "inlet", "boundary", "wall")),
                             singular=z["singular"])
    return z, a, bc


@pytest.mark.parametrize("initial", [1, 0])
def test_singular_wall_matches_golden(oracle_mod, initial):
    z, a, bc = singular_golden_inputs()
    oracle_mod.boundary_fill(a, bc, float(z["mach"]), initial, int(z["sd_node"]))
    assert np.array_equal(a["flow"], z[f"out_flow_initial{initial}"])


def test_singular_golden_covers_every_branch(oracle_mod):
    """Every singular code, ID 10 over a face code, over an edge code and
    over codes 33..52; and the table changes the result."""
    from cfd_gb300 import cases
    z, a, bc = singular_golden_inputs()
    g = a["grid"]
    wall = bc.wall
    assert set(cases.SINGULAR_CODES) <= set(g["loc"][wall].tolist())
    id10 = wall[g["ID"][wall] == 10]
    codes10 = set(g["loc"][id10].tolist())
    assert 3 in codes10 and codes10 & set(range(7, 27)) and codes10 & set(range(33, 53))
    other = bc.singular.copy()
    other[other != 0] = np.roll(other[other != 0], 1)
    b = {k: v.copy() for k, v in a.items()}
    oracle_mod.boundary_fill(b, cases.BoundaryLists(bc.outlet, bc.inlet, bc.boundary, bc.wall, singular=other),
                             float(z["mach"]), 1, int(z["sd_node"]))
    assert not np.array_equal(b["flow"], z["out_flow_initial1"])


@pytest.mark.parametrize("seed", [0, 1])
def test_singular_wall_matches_reference_build(oracle_mod, seed):
    if not oracle_mod.ref_available():
        pytest.skip("reference build absent")
    from cfd_gb300 import cases
    c = cases.singular_box(shape=(10, 9, 8), seed=seed)
    bc = cases.BoundaryLists(c.bc.outlet, c.bc.inlet, c.bc.boundary, c.bc.wall, singular=c.bc.singular)
    rng = np.random.default_rng(seed + 3)
    a = c.copy().arrays
    a["flow"][1:] = rng.uniform(0.5, 1.5, a["flow"][1:].shape)
    b = {k: v.copy() for k, v in a.items()}
    oracle_mod.boundary_fill(a, bc, 0.7, 1, c.sd_node)
    oracle_mod.ref_boundary_fill(b, bc, 0.7, 1, c.sd_node)
    assert np.array_equal(a["flow"], b["flow"])


def test_tips_after_the_routine(oracle_mod):
    """Each tip row: zero velocity, p and t of its slot-3 neighbour, rho and e
    derived, a untouched -- applied after every list."""
    from cfd_gb300 import cases, layout
    c = cases.singular_box(seed=2)
    F = layout.FLOW
    rng = np.random.default_rng(9)
    a = c.copy().arrays
    a["flow"][1:] = rng.uniform(0.5, 1.5, a["flow"][1:].shape)
    notips = cases.BoundaryLists(c.bc.outlet, c.bc.inlet, c.bc.boundary, c.bc.wall, singular=c.bc.singular)
    b = {k: v.copy() for k, v in a.items()}
    oracle_mod.boundary_fill(a, c.bc, 0.7, 1, c.sd_node)
    oracle_mod.boundary_fill(b, notips, 0.7, 1, c.sd_node)
    m = 0.7
    for t in c.bc.tips:
        s = int(b["grid"]["N3"][t])
        exp = b["flow"][t].copy()
        exp[[F["u"], F["v"], F["w"]]] = 0.0
        exp[F["p"]], exp[F["t"]] = b["flow"][s, F["p"]], b["flow"][s, F["t"]]
        exp[F["rho"]] = (1.4 * m * m) * (exp[F["p"]] / exp[F["t"]])
        exp[F["e"]] = exp[F["p"]] / (0.4 * exp[F["rho"]])
        b["flow"][t] = exp
    assert np.array_equal(a["flow"], b["flow"])


def test_unset_singular_codes_are_rejected(oracle_mod):
    """Codes 53..56 run the routine's mirror passes with slots it never set."""
    from cfd_gb300 import cases
    c = cases.singular_box(seed=0)
    a = c.copy().arrays
    r = int(c.bc.wall[np.flatnonzero(a["grid"]["loc"][c.bc.wall] == 3)[0]])
    a["grid"]["loc"][r] = 54
    before = a["flow"].copy()
    with pytest.raises(ValueError):
        oracle_mod.boundary_fill(a, c.bc, 0.8, 1, c.sd_node)
    assert np.array_equal(a["flow"], before)
