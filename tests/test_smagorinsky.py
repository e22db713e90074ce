"""Smagorinsky SGS model (les = 2, C_s = params.smagorinsky_cs), the LES
model the Taylor-Green LES workload names; the reference implements only the mixed-time-scale
model (Viscous.cl:490-558), so parity for les = 2 is pinned to the oracle's
restatement of this builder addition, not to the reference.

CPU: with C_s = 0 the model adds exactly nothing (bit-identical to les = 0),
and with C_s > 0 it removes kinetic energy.  GPU: the FP64 lattice path and
the drop-in entry points match the oracle (relative L2 <= 1e-12), C_s = 0
equals les = 0 bit for bit on the device, and the mixed form stays within
1e-6 of the FP64 form."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

from helpers import copy_arrays, rel_l2


def _tgv(les, cs, n=12, shape=(12, 10, 8)):
    from cfd_gb300 import cases
    c = cases.taylor_green(n=n, shape=shape)
    c.params = dataclasses.replace(c.params, les=les, smagorinsky_cs=cs)
    return c


def _oracle_run(oracle_mod, c, stages):
    a = copy_arrays(c.arrays)
    L = None
    for j in range(stages):
        L = oracle_mod.stage(a, c.g_node, c.sd_node, c.params, j % 3, c.dt, want_L=True)
    return a, L


def test_zero_cs_adds_nothing(oracle_mod):
    c0, c2 = _tgv(0, 0.0), _tgv(2, 0.0)
    a0, L0 = _oracle_run(oracle_mod, c0, 3)
    a2, L2 = _oracle_run(oracle_mod, c2, 3)
    for k in ("flow", "U0", "U1", "U2", "Fv", "Ev", "Gv"):
        assert np.array_equal(a0[k], a2[k]), k
    assert np.array_equal(L0, L2)


def test_smagorinsky_dissipates_kinetic_energy(oracle_mod):
    from cfd_gb300 import layout as L
    own = slice(1, None)
    ke = {}
    for les, cs in ((0, 0.0), (2, 0.1)):
        c = _tgv(les, cs, n=16, shape=(16, 16, 16))
        c.params = dataclasses.replace(c.params, reynolds=1e5)   # the model, not molecular viscosity, dominates
        a, _ = _oracle_run(oracle_mod, c, 6)
        f = a["flow"][own]
        rho, u, v, w = (f[:, L.FLOW[k]] for k in ("rho", "u", "v", "w"))
        ke[les] = float(np.sum(0.5 * rho * (u * u + v * v + w * w) * a["det"][own]))
    assert ke[2] < ke[0]


@pytest.mark.gpu
def test_fp64_paths_match_oracle(ctx, oracle_mod):
    from cfd_gb300 import runtime
    c = _tgv(2, 0.1, n=14, shape=(14, 12, 10))
    want, _ = _oracle_run(oracle_mod, c, 6)
    s = runtime.Solver(ctx, c)
    assert s.info().path == "structured"
    s.set_flow(c.arrays["flow"])
    s.step(c.dt, 2)
    got = s.get_flow()
    s.close()
    assert rel_l2(got[1:], want["flow"][1:]) <= 1e-12
    dev = ctx.upload_case(copy_arrays(c.arrays))
    for j in range(6):
        ctx.stage(dev, c.g_node, c.sd_node, c.params, j % 3, c.dt)
    got = ctx.download(dev, "flow", c.arrays["flow"])
    for p in dev.values():
        ctx.free(p)
    assert rel_l2(got[1:], want["flow"][1:]) <= 1e-12


@pytest.mark.gpu
def test_zero_cs_equals_no_les_on_device(ctx):
    from cfd_gb300 import runtime
    out = []
    for les in (0, 2):
        c = _tgv(les, 0.0, n=14, shape=(14, 12, 10))
        s = runtime.Solver(ctx, c)
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 2)
        out.append(s.get_flow())
        s.close()
    assert np.array_equal(out[0].view(np.uint64), out[1].view(np.uint64))


@pytest.mark.gpu
def test_mixed_form_within_tolerance(ctx):
    from cfd_gb300 import runtime
    c = _tgv(2, 0.1, n=16, shape=(16, 16, 16))
    res = []
    for prec in (0, 1):
        s = runtime.Solver(ctx, c, precision=prec)
        s.set_flow(c.arrays["flow"])
        s.step(c.dt, 5)
        res.append(s.get_u0())
        s.close()
    assert rel_l2(res[1][1:], res[0][1:]) <= 1e-6
