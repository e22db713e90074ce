"""The allocation-free stage entry point (cfd_lattice_stage_static).

It exists for callers that cannot allocate device memory while they step a
solution, so it keeps its intermediates in a library-owned static device
array instead.  Its results must equal those of the resident solver's
structured path (cfd_solver_stage) on the three stages of a step called in
a row, and its state slots those of the oracle, within the FP64 tolerance
of the other tests.  This file is collected last so that a run
that stops at the first failure has run every other test already."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _static_stage(ctx, dev, shape, j, dt, params):
    from cfd_gb300 import abi, runtime
    pr = runtime.to_params(params)
    ni, nj, nk = shape
    return ctx.lib.cfd_lattice_stage_static(None, ni, nj, nk, j, dt, C.byref(pr), dev["det"], dev["deter"],
                                            dev["metric"], dev["U0"], dev["U1"], dev["U2"], dev["flow"], dev["L"])


def test_static_stage_matches_solver_stage(ctx, oracle_mod):
    """Three calls in a row (stages 0, 1 and 2, the last advancing U0): L and
    FLOW after each against the resident solver, and the three state slots
    after the step against the oracle."""
    from cfd_gb300 import abi, cases, runtime
    c = cases.taylor_green(n=20, shape=(20, 18, 16))
    assert c.sd_node <= abi.STATIC_MAX_NODES
    # reference: the resident solver (allocating) entry points
    s = runtime.Solver(ctx, c)
    assert s.info().path == "structured"
    s.set_flow(c.arrays["flow"])
    # buffers for the allocation-free entry point (allocated here by the test,
    # not by the entry point)
    dev = ctx.upload_case(c.arrays, names=["det", "deter", "metric", "flow", "U0", "U1", "U2", "L"])
    own = slice(1, c.sd_node + 1)
    for j in (0, 1, 2):                   # calls in a row
        L_ref = s.stage(j, c.dt)
        flow_ref = s.get_flow()
        st = _static_stage(ctx, dev, c.shape, j, c.dt, c.params)
        assert st == abi.OK, abi.STATUS_NAMES.get(st, st)
        L_new = ctx.download(dev, "L", np.zeros((c.g_node + 1, 5)))
        flow_new = ctx.download(dev, "flow", c.arrays["flow"])
        assert rel_l2(L_new[own], L_ref[own]) <= TOL, f"stage {j} L"
        assert rel_l2(flow_new[own], flow_ref[own]) <= TOL, f"stage {j} FLOW"
    s.close()
    a = {k: v.copy() for k, v in c.arrays.items()}
    for j in range(3):
        oracle_mod.stage(a, c.g_node, c.sd_node, c.params, j, c.dt)
    for k in ("U0", "U1", "U2"):
        got = ctx.download(dev, k, c.arrays[k])
        assert rel_l2(got[own], a[k][own]) <= TOL, k
    for p in dev.values():
        ctx.free(p)


def test_static_stage_rejects_oversize_lattice(ctx):
    from cfd_gb300 import abi, cases
    c = cases.isentropic_vortex(n=4)
    dev = ctx.upload_case(c.arrays, names=["det", "deter", "metric", "flow", "U0", "U1", "U2", "L"])
    n = abi.STATIC_MAX_NODES
    st = _static_stage(ctx, dev, (n + 1, 1, 1), 0, c.dt, c.params)
    assert st == abi.EINVAL
    for p in dev.values():
        ctx.free(p)
