"""Generates the golden vectors under tests/golden/ from the reference's own
sources (U_Q.cl, Viscous.cl, Weno.cl and the boundary routine
Flow_Initialisation.cpp, compiled as host C++ by oracle/build_ref.sh).  Run
in a checkout that has the reference sources:

    python tests/golden/make_golden.py

Each .npz holds the inputs of a small case (reference layout, rows 0..g_node)
and the buffers the reference kernels wrote during the three RK stages of one
step (U_Q -> Viscous -> Weno(j), j passed per stage): after stage 0 every
buffer (Q, ROE_AVER, F, E, G, Fv, Ev, Gv, U0, U1, U2, FLOW); after stages 1
and 2 the advanced state (the U that Weno wrote, and FLOW).  For the ghost-box
case a mask marks the rows whose values the reference defines (outputs that
depend on its uninitialised derivative branches are excluded), computed with
the restatement's poison mode.
"""
from __future__ import annotations

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from cfd_gb300 import cases  # noqa: E402

import oracle  # noqa: E402

OUT_KEYS = ("Q", "roe", "F", "E", "G", "Fv", "Ev", "Gv", "U0", "U1", "U2", "flow")
IN_KEYS = ("grid", "det", "deter", "metric", "flow")


def golden_cases():
    vortex = cases.isentropic_vortex(n=8, length=10.0 * 8 / 64 * 4)  # D = 0.625
    tgv_ref = cases.taylor_green(n=6)
    p = tgv_ref.params
    p.mach, p.reynolds, p.prandtl, p.t_inf = 1.5, 500.0, 0.72, 273.0   # the reference's own constants
    tgv = cases.taylor_green(n=6)                                        # Mach 0.1, Re 1600 (substituted copy)
    box = cases.ghost_box(shape=(6, 5, 5), seed=3)
    return {"vortex8": vortex, "tgv6_refconst": tgv_ref, "tgv6": tgv, "ghostbox": box}


def stage_keys(j):
    """Stage 0 keeps every buffer the kernels write; later stages keep the
    advanced state (the U written by Weno and FLOW)."""
    return OUT_KEYS if j == 0 else (("U1", "U2", "U0")[j], "flow")


def run(case, stages=3):
    a = {k: v.copy() for k, v in case.arrays.items()}
    res = {}
    for j in range(stages):
        oracle.ref_stage(a, case.g_node, case.sd_node, case.params, j, case.dt)
        for k in stage_keys(j):
            res[f"s{j}_{k}"] = a[k].copy()
    return res


def poison_mask(case, stages=3):
    a = {k: v.copy() for k, v in case.arrays.items()}
    oracle.set_poison(True)
    masks = {}
    try:
        for j in range(stages):
            oracle.stage(a, case.g_node, case.sd_node, case.params, j, case.dt)
            for k in stage_keys(j):
                masks[f"s{j}_{k}"] = np.isfinite(a[k]).reshape(a[k].shape[0], -1).all(axis=1)
    finally:
        oracle.set_poison(False)
    return masks


BC_MACH = 0.8


def make_bc_golden():
    """bc_ghostbox.npz: the reference's boundary routine intialise()
    (Flow_Initialisation.cpp:23-1394) on a ghost box whose boundary rows are
    split over the outlet, inlet, boundary and wall lists (face, edge and
    corner codes), from a seeded random FLOW, with initial = 1 and 0."""
    box = cases.ghost_box(shape=(5, 4, 4), seed=3, bc=True)
    rng = np.random.default_rng(20261203)
    flow = box.arrays["flow"].copy()
    flow[1:] = rng.uniform(0.5, 1.5, flow[1:].shape)
    payload = {"in_grid": box.arrays["grid"], "in_flow": flow, "sd_node": np.array(box.sd_node),
               "mach": np.array(BC_MACH)}
    for t in ("outlet", "inlet", "boundary", "wall"):
        payload[f"list_{t}"] = getattr(box.bc, t)
    for initial in (1, 0):
        a = {"grid": box.arrays["grid"].copy(), "flow": flow.copy()}
        oracle.ref_boundary_fill(a, box.bc, BC_MACH, initial, box.sd_node)
        payload[f"out_flow_initial{initial}"] = a["flow"]
    np.savez_compressed(HERE / "bc_ghostbox.npz", **payload)
    print("bc_ghostbox ->", (HERE / "bc_ghostbox.npz").stat().st_size, "bytes")


def make_bc_singular_golden():
    """bc_singular.npz: the reference's intialise() with its singular-node
    wall branches (Flow_Initialisation.cpp:1194-1392: codes 29/30, ID 10,
    codes 33..52) on cases.singular_box, from a seeded random FLOW, with
    initial = 1 and 0.  The table and the relabelled grid are stored with
    the lists; the tip rows are not part of intialise and are left out."""
    box = cases.singular_box(shape=(8, 6, 8), seed=5)
    rng = np.random.default_rng(20261204)
    flow = box.arrays["flow"].copy()
    flow[1:] = rng.integers(50, 151, flow[1:].shape) / 100.0   # few distinct inputs: a small fixture
    grid = box.arrays["grid"].copy()
    for k in ("x", "y", "z"):
        grid[k] = 0.0   # the routine reads only the neighbour slots, ID and loc
    payload = {"in_grid": grid, "in_flow": flow, "sd_node": np.array(box.sd_node),
               "mach": np.array(BC_MACH), "singular": box.bc.singular}
    for t in ("outlet", "inlet", "boundary", "wall"):
        payload[f"list_{t}"] = getattr(box.bc, t)
    bc = cases.BoundaryLists(box.bc.outlet, box.bc.inlet, box.bc.boundary, box.bc.wall, singular=box.bc.singular)
    for initial in (1, 0):
        a = {"grid": grid.copy(), "flow": flow.copy()}
        oracle.ref_boundary_fill(a, bc, BC_MACH, initial, box.sd_node)
        payload[f"out_flow_initial{initial}"] = a["flow"]
    np.savez_compressed(HERE / "bc_singular.npz", **payload)
    print("bc_singular ->", (HERE / "bc_singular.npz").stat().st_size, "bytes")


def main(only=None):
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference build missing: run oracle/build_ref.sh in a checkout with the reference")
    if only in (None, "bc"):
        make_bc_golden()
    if only in (None, "bc", "bc_singular"):
        make_bc_singular_golden()
    if only in ("bc", "bc_singular"):
        return
    for name, case in golden_cases().items():
        stages = 1 if name == "ghostbox" else 3
        res = run(case, stages)
        payload = {f"in_{k}": case.arrays[k] for k in IN_KEYS}
        payload.update(res)
        p = case.params
        payload["meta"] = np.array([case.g_node, case.sd_node, stages], dtype=np.int64)
        payload["params"] = np.array([p.mach, p.reynolds, p.prandtl, p.t_inf, p.weno_eps, p.viscous, p.les, case.dt])
        payload["shape"] = np.array(case.shape, dtype=np.int64)
        if name == "ghostbox":
            for k, m in poison_mask(case, stages).items():
                payload[f"mask_{k}"] = m
        np.savez_compressed(HERE / f"{name}.npz", **payload)
        print(name, "rows", case.g_node + 1, "->", (HERE / f"{name}.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    # python tests/golden/make_golden.py [bc|bc_singular]   (only the boundary-routine fixtures / the singular one)
    main(sys.argv[1] if len(sys.argv) > 1 else None)
