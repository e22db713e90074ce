"""The boundary routine's singular-node wall branches and tip rows on the GPU
(cfd_bc_create_singular): wall nodes with ID 10 or codes 29/30/33..52 take
the routine's rules from the singular-node table after the rule of their
code (Flow_Initialisation.cpp:1194-1392), tips the wall rule from their
slot-3 neighbour after the lists (Solver.cpp:660-683).

* cfd_boundary_fill against the golden vectors of the reference's own
  routine with its singular table (bit-exact), and with tips against the
  oracle (bit-exact);
* the gather path (a ghost box) and the lattice path (the wall-bounded
  channel, FP64 and both reduced forms) with the routine after every stage:
  FP64 against the oracle (relative L2 <= 1e-12), the reduced forms within
  1e-6 of FP64 on the fields the next stage reads."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2
from test_oracle_boundary import singular_golden_inputs

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _fill(ctx, grid, flow, bc, mach, initial, sd_node):
    from cfd_gb300 import runtime
    bnd = runtime.Boundary(ctx, grid, bc)
    dev = ctx.alloc(flow.nbytes)
    try:
        ctx.write(dev, flow)
        n0 = ctx.launch_count
        bnd.fill(dev, mach, initial, sd_node)
        launches = ctx.launch_count - n0
        out = np.empty_like(flow)
        ctx.read(out, dev)
    finally:
        ctx.free(dev)
        bnd.close()
    return out, launches


@pytest.mark.parametrize("initial", [1, 0])
def test_singular_fill_matches_reference_golden(ctx, initial):
    z, a, bc = singular_golden_inputs()
    out, _ = _fill(ctx, a["grid"], a["flow"], bc, float(z["mach"]), initial, int(z["sd_node"]))
    assert np.array_equal(out, z[f"out_flow_initial{initial}"])


@pytest.mark.parametrize("seed", [0, 1])
def test_singular_fill_with_tips_matches_oracle(ctx, oracle_mod, seed):
    from cfd_gb300 import cases
    c = cases.singular_box(seed=seed)
    a = c.copy().arrays
    a["flow"][1:] = np.random.default_rng(seed).uniform(0.5, 1.5, a["flow"][1:].shape)
    out, launches = _fill(ctx, a["grid"], a["flow"], c.bc, 0.7, 1, c.sd_node)
    oracle_mod.boundary_fill(a, c.bc, 0.7, 1, c.sd_node)
    assert np.array_equal(out, a["flow"])
    assert launches >= 1


def test_singular_codes_without_slots_are_unsupported(ctx):
    from cfd_gb300 import abi, cases, runtime
    c = cases.singular_box(seed=0)
    g = c.arrays["grid"]
    r = int(c.bc.wall[np.flatnonzero(g["loc"][c.bc.wall] == 3)[0]])
    g["loc"][r] = 55
    with pytest.raises(abi.CfdError) as e:
        runtime.Boundary(ctx, g, c.bc)
    assert e.value.status == abi.EUNSUPPORTED


def test_singular_box_gather_path_matches_oracle(ctx, oracle_mod):
    from cfd_gb300 import cases, runtime
    c = cases.singular_box(shape=(9, 7, 7), seed=3)
    s = runtime.Solver(ctx, c)
    assert s.info().path == "gather"
    s.set_flow(c.arrays["flow"])
    s.step(c.dt, 2)
    flow = s.get_flow()
    s.close()
    a = c.copy().arrays
    oracle_mod.rk3_steps_bc(a, c.g_node, c.sd_node, c.params, c.dt, 2, c.bc)
    assert rel_l2(flow[1:], a["flow"][1:]) <= TOL


def _singular_channel():
    from cfd_gb300 import cases
    return cases.with_singular_nodes(cases.channel(ni=16, nj=12, nk=8), seed=4)


def test_singular_channel_lattice_fp64_matches_oracle(ctx, oracle_mod):
    from cfd_gb300 import runtime
    c = _singular_channel()
    s = runtime.Solver(ctx, c)
    assert s.info().path == "structured"
    s.set_flow(c.arrays["flow"])
    s.step(c.dt, 3)
    flow = s.get_flow()
    s.close()
    a = c.copy().arrays
    oracle_mod.rk3_steps_bc(a, c.g_node, c.sd_node, c.params, c.dt, 3, c.bc)
    assert np.isfinite(a["flow"][1:]).all()
    assert rel_l2(flow[1:], a["flow"][1:]) <= TOL


@pytest.mark.parametrize("precision", [1, 2])
def test_singular_channel_reduced_forms_within_budget(ctx, precision):
    from cfd_gb300 import layout, runtime
    c = _singular_channel()
    out = {}
    for prec in (0, precision):
        s = runtime.Solver(ctx, c, precision=prec)
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 3)
        out[prec] = s.get_flow()[1:c.sd_node + 1]
        s.close()
    cols = [layout.FLOW[k] for k in ("rho", "u", "v", "w", "p")]
    assert np.isfinite(out[precision]).all()
    assert rel_l2(out[precision][:, cols], out[0][:, cols]) <= 1e-6
