"""Benchmark of the RHS path: cell-updates/s (nodes x full SSP-RK3 steps / s).

Workload (default): Taylor-Green vortex on a 128^3 periodic grid with
sinusoidally perturbed node positions (curvilinear metrics), Re 1600,
Mach 0.1, Pr 0.72, reference mixed-time-scale LES, synthetic inputs generated
in-process.  One "step" = one full SSP-RK3 step (three stages of U_Q ->
Viscous -> Weno) over the whole grid.

Arms:
  --impl gb300      (default) the CUDA library.  ``value``: FP64 form, state
                    resident in HBM, CUDA events on the launching stream;
                    ``e2e``: the same metric through the drop-in entry points
                    (cfd_uq / cfd_viscous / cfd_weno per stage, the calls a
                    reference host binds) with FLOW copied from / to pinned
                    host memory every step (``e2e_resident``: the same through
                    the resident solver API); ``split`` and ``mixed``: the two
                    reduced-precision forms (FP64 state/RK/metric products +
                    FP32 flux physics; everything FP32 with a hi+lo state),
                    each with its relative L2 error against the FP64 form on
                    the same run; then the Taylor-Green diagnostics, the
                    batched, serving, NACA0012 and shocked legs.
  --impl reference  the reference algorithm on the host cores (the CPU
                    restatement in oracle/, its timed build, all threads),
                    same workload and config.

Multi-GPU: the path does not exchange data between instances; N ranks run
N independent replicas (weak scaling), timed between barriers, max over
ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

METRIC = "cell-updates/s FP64 vs mixed at <=1e-6 rel L2 vs FP64; p50/p99 solve latency"
UNIT = "cell-updates/s"

# Algorithmic (compulsory) bytes of an ideal fused face-based FP64 SSP-RK3
# step per cell: 5 state reads + 3 state writes of 40 B, plus 22 doubles of
# geometry per stage (node metrics 9, det 1, three face metrics 3x3, three
# face dets 3), x3 stages.
ALGO_BYTES_PER_CELL_UPDATE = 5 * 40 + 3 * 40 + 3 * 22 * 8          # 848
# Per-launch compulsory bytes per node of each structured kernel (every
# input and output element once).
KERNEL_BYTES_PER_NODE = {
    "prep": (5 + 9 + 1 + 5 + 5 + 15 + 2) * 8,          # prims, metrics, det -> Q, U_j, F/E/G, sqrt(rho), H
    "viscous": (5 + 9 + 1 + 4 + 15 + 1) * 8,           # U_j, metrics, det, prims -> Fv/Ev/Gv, mu
    "mu_only": (5 + 1) * 8,
    "face_i": (5 + 3 + 2 + 3 + 1 + 5 + 5) * 8,         # Q, u/v/w, sqrt(rho)/H, face metric, face det, F -> Fh
    "face_j": (5 + 3 + 2 + 3 + 1 + 5 + 5) * 8,
    "face_k": (5 + 3 + 2 + 3 + 1 + 5 + 5) * 8,
    "update": (15 + 15 + 10 + 1 + 5 + 8) * 8,          # Fh, Fv/Ev/Gv, two U, det -> U, 8 FLOW fields
}
# FP64 operations per face of the FP64 face kernels, from ncu's FP64
# instruction counters on the 64^3 Taylor-Green case (per face: 818 DFMA,
# 784 DMUL, 575 DADD; FMA = 2), and the DRAM bytes the same capture measured
# per face (dram__bytes_read.sum + dram__bytes_write.sum over 262,144 faces;
# scaled by the face count of a launch for other sizes).
FP64_FLOP_PER_NODE = {"face_i": 2995, "face_j": 2995, "face_k": 2995}
DRAM_BYTES_PER_NODE = {"face_i": 153, "face_j": 155, "face_k": 155}


# The precision forms (cfd_precision_t) and how each one's arithmetic reads.
FP64, MIXED, SPLIT = 0, 1, 2
FORM_NAMES = {FP64: "fp64", MIXED: "mixed", SPLIT: "split"}
FORM_DTYPES = {
    FP64: "f64",
    MIXED: "f32 throughout: f32 fluxes and WENO, state and RK3 as f32 hi+lo pairs, f32 metrics and det",
    SPLIT: "f64 state, RK3, Q and face-flux metric/Jacobian products + f32 characteristic WENO, LLF speed, "
           "viscous fluxes",
}


def parse_args(argv=None):
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    p.add_argument("--config", choices=("tgv128", "tgv64", "vortex64"), default="tgv128")
    p.add_argument("--les", choices=("mts", "smagorinsky"), default="mts",
                   help="SGS model of the TGV workloads: the reference's mixed time scale (parity) or "
                        "Smagorinsky C_s = 0.1 (the model the Taylor-Green LES workload names)")
    p.add_argument("--cpu-steps", type=int, default=1, help="full steps timed for the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-mixed", action="store_true", help="skip the two reduced-precision forms")
    p.add_argument("--dropin-steps", type=int, default=0,
                   help="steps timed through the drop-in entry points (0 = --steps)")
    p.add_argument("--batch-count", type=int, default=64, help="instances of the batched workload (0 = skip)")
    p.add_argument("--batch-steps", type=int, default=20)
    p.add_argument("--batch-forms", default="fp64,mixed,split", help="forms of the batched leg")
    p.add_argument("--batch-tile", type=int, default=0, help="tile size of the batched leg (0 = tuned)")
    p.add_argument("--serve-requests", type=int, default=100,
                   help="requests of the serving workload at its 50/s rate (0 = skip the serving leg)")
    p.add_argument("--serve-forms", default="split,mixed", help="forms served at the workload's rate")
    p.add_argument("--serve-sub-requests", type=int, default=64,
                   help="requests of the stream at a rate below capacity (0 = skip)")
    p.add_argument("--serve-sub-load", type=float, default=0.75,
                   help="offered load of that stream as a fraction of the measured capacity")
    p.add_argument("--serve-acc-requests", type=int, default=100,
                   help="requests of the reduced stream served in FP64 and the reduced forms for the "
                        "per-request error (0 = skip)")
    p.add_argument("--serve-fill", type=int, default=0,
                   help="lattice nodes per batch step of the least_work policy (0 = the library default)")
    p.add_argument("--diag-steps", type=int, default=200,
                   help="steps of the kinetic-energy/enstrophy comparison on the main case (0 = skip)")
    p.add_argument("--naca-steps", type=int, default=500,
                   help="steps of the NACA0012 O-grid case, FP64 vs the reduced forms with the boundary "
                        "routine (0 = skip)")
    p.add_argument("--naca-grid", default="512,128,32", help="NACA0012 O-grid nodes around,normal,span")
    p.add_argument("--shock-steps", type=int, default=300,
                   help="steps of the shocked curvilinear case, FP64 vs the reduced forms (0 = skip)")
    return p.parse_args(argv)


def make_case(config: str, les: str = "mts"):
    """The workload and its config: only keys that define the work, so that
    both arms report the same config."""
    import dataclasses
    from cfd_gb300 import cases
    if config in ("tgv128", "tgv64"):
        n = 128 if config == "tgv128" else 64
        c = cases.taylor_green(n=n)
        cfg = {"workload": f"taylor_green_{n}^3_curvilinear_les", "grid": [n, n, n], "re": 1600, "mach": 0.1,
               "les": les}
        if les == "smagorinsky":   # the Taylor-Green LES workload's model (C_s = 0.1); the reference implements MTS only
            c.params = dataclasses.replace(c.params, les=2, smagorinsky_cs=0.1)
            cfg["smagorinsky_cs"] = 0.1
        return c, cfg
    # the 64^3 vortex workload specifies WENO eps = 1e-6 (the reference's constant, 1e-7, is the parity tests' value)
    return cases.isentropic_vortex(n=64, weno_eps=1e-6), {"workload": "isentropic_vortex_64^3_periodic_inviscid",
                                                          "grid": [64, 64, 64], "weno_eps": 1e-6}


# ------------------------------------------------------------ distributed --

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world: int, backend: str):
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend=backend)


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def aggregate(seconds: float, units: float, world: int, device=None):
    """Whole-job throughput: units summed over ranks / max time over ranks."""
    if world == 1:
        return units / seconds, seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()) / float(t.item()), float(t.item())


# ----------------------------------------------------------------- clocks --

class ClockSampler:
    """nvidia-smi samples of SM clock, power and throttle reasons while the
    timed region runs."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]
        return False

    def summary(self):
        if not getattr(self, "lines", None):
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU legs ---

def cpu_oracle_rate(case, nsteps: int, threads: int | None = None):
    """Times the timed build of the CPU restatement of the reference algorithm
    (oracle/) on the host cores: nsteps full SSP-RK3 steps of the whole case.
    Returns (cell-updates/s, threads, seconds, compiler flags)."""
    import oracle
    oracle.build()
    L = oracle.timed_lib()
    if threads:
        L.oracle_set_threads(int(threads))
    cores = L.oracle_get_threads()
    a = {k: v.copy() for k, v in case.arrays.items()}
    t0 = time.perf_counter()
    oracle.rk3_steps(a, case.g_node, case.sd_node, case.params, case.dt, nsteps, timed=True)
    dt = time.perf_counter() - t0
    return case.sd_node * nsteps / dt, cores, dt, oracle.timed_build_flags()


def cpu_sample_text(steps: int, workload: str, secs: float, cores: int, flags: str) -> str:
    return (f"{steps} full SSP-RK3 step(s) of the whole {workload} grid ({secs:.1f} s on {cores} threads); "
            f"the reference's kernel arithmetic through its C restatement (bit-exact against the reference "
            f"sources in its parity build), timed build: gcc {flags}; the reference's own OpenCL/MPI build "
            f"cannot run on this host (no OpenCL ICD, no MPI)")


def reference_arm(args):
    world, rank, local = dist_env()
    if rank != 0:
        return 0
    case, cfg = make_case(args.config, args.les)
    import oracle
    oracle.build()
    L = oracle.timed_lib()
    cores = L.oracle_get_threads()
    a = {k: v.copy() for k, v in case.arrays.items()}
    for _ in range(args.warmup):
        oracle.rk3_steps(a, case.g_node, case.sd_node, case.params, case.dt, 1, timed=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.rk3_steps(a, case.g_node, case.sd_node, case.params, case.dt, 1, timed=True)
    secs = time.perf_counter() - t0
    value = case.sd_node * args.steps / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "run": {"parallelism": f"host cores (OpenMP, {cores} threads)", "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": cpu_sample_text(args.steps, cfg["workload"], secs, cores,
                                                   oracle.timed_build_flags())},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------- GPU arm ----

def rel_l2(a, b) -> float:
    import numpy as np
    den = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def gpu_arm(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    dist_init(world, "nccl")
    torch.cuda.set_device(local)
    __graft_entry__.load_package()
    from cfd_gb300 import runtime

    case, cfg = make_case(args.config, args.les)
    N = case.sd_node
    ctx = runtime.Context(local)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    peaks = load_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0

    def time_resident(precision: int, steps: int, warmup: int):
        s = runtime.Solver(ctx, case, precision=precision)
        assert s.info().path == "structured"
        s.set_flow(case.arrays["flow"])
        s.step(case.dt, warmup)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier(world)
        torch.cuda.synchronize()
        launches0 = ctx.launch_count
        with ClockSampler(local) as clk:
            with torch.cuda.stream(stream):
                e0.record(stream)
            s.step(case.dt, steps)
            with torch.cuda.stream(stream):
                e1.record(stream)
            torch.cuda.synchronize()
        barrier(world)
        secs = e0.elapsed_time(e1) / 1e3
        return s, secs, ctx.launch_count - launches0, clk.summary()

    # --- FP64 form, resident ---
    s64, secs64, launches64, clocks = time_resident(FP64, args.steps, args.warmup)
    value, tmax = aggregate(secs64, N * args.steps, world, device=f"cuda:{local}")
    prof = [s64.profile_stage(j, case.dt) for j in range(3)]   # advances 1 step (3 stages) after timing
    u64 = s64.get_u0()

    # --- reduced-precision forms, resident, same number of steps from the same state ---
    reduced = {}
    if not args.no_mixed:
        for prec in (SPLIT, MIXED):
            sm, secsm, launchesm, clocks_m = time_resident(prec, args.steps, args.warmup)
            vm, _ = aggregate(secsm, N * args.steps, world, device=f"cuda:{local}")
            prof_m = [sm.profile_stage(j, case.dt) for j in range(3)]
            um = sm.get_u0()
            reduced[FORM_NAMES[prec]] = {
                "value": vm, "unit": UNIT, "ms_per_step": 1e3 * secsm / args.steps, "speedup_vs_fp64": vm / value,
                "rel_l2_vs_fp64": rel_l2(um[1:], u64[1:]), "steps_compared": args.warmup + args.steps + 1,
                "dtype": FORM_DTYPES[prec], "gpu_launches": launchesm, "clocks": clocks_m,
                "step_algorithmic_hbm_frac": ALGO_BYTES_PER_CELL_UPDATE * vm / world / 1e9 / hbm_peak,
                "face_tiles_tuned": list(sm.info().face_tiles),
                "kernels_ms_per_stage": _kernel_table(prof_m)}
            sm.close()

    # --- end to end through the public API with host buffers ---
    host_in = torch.empty((case.g_node + 1, 9), dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty((case.g_node + 1, 9), dtype=torch.float64, pin_memory=True).numpy()
    host_in[...] = case.arrays["flow"]
    se = runtime.Solver(ctx, case)
    for _ in range(min(args.warmup, 2)):
        se.set_flow(host_in)
        se.step(case.dt, 1)
        se.get_flow(host_out)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        se.set_flow(host_in)
        se.step(case.dt, 1)
        se.get_flow(host_out)
        host_in, host_out = host_out, host_in
    e2e_secs = time.perf_counter() - t0
    barrier(world)
    e2e_value, _ = aggregate(e2e_secs, N * args.steps, world, device=f"cuda:{local}")
    se.close()

    # --- roofline of the dominant kernel ---
    table = _kernel_table(prof)
    dom = max(table, key=lambda k: table[k])
    dom_bytes = KERNEL_BYTES_PER_NODE.get(dom, 0) * N
    achieved = dom_bytes / (table[dom] * 1e-3) / 1e9
    fp64_peak = ctx.probe_flops(True)
    fp32_peak = ctx.probe_flops(False)
    fp64_roof = None
    if dom in FP64_FLOP_PER_NODE:
        f = FP64_FLOP_PER_NODE[dom] * N / (table[dom] * 1e-3)
        fp64_roof = {"kernel": dom, "achieved": f / 1e12, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                     "frac": f / fp64_peak, "peak_source": "FP64 FMA probe of this run",
                     "note": "DMUL/DADD count one FLOP but take a full FP64 issue slot"}
    traffic = DRAM_BYTES_PER_NODE[dom] * N if dom in DRAM_BYTES_PER_NODE else None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tmax / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "run": {"parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                "l2": "inputs larger than L2 (resident working set %.2f GB)" % (s64.info().device_bytes / 1e9),
                "path": "structured face-based, exact FP64 evaluation order",
                "fp64_face_blocks_tuned": list(s64.info().face_blocks)},
        "gpu_launches": launches64,
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(host_in.nbytes),
                "d2h_bytes_per_step": int(host_out.nbytes)},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic, "peak_source": peak_src,
                     "note": "FP64-pipe bound; see roofline_fp64"},
        "roofline_fp64": fp64_roof,
        "step_algorithmic_gbs": ALGO_BYTES_PER_CELL_UPDATE * value / world / 1e9,
        "peaks_probed": {"fp64_tflops": fp64_peak / 1e12, "fp32_tflops": fp32_peak / 1e12},
        "kernels_ms_per_stage": table,
    }
    line.update(reduced)
    if "split" in reduced:
        line["reduced_precision_claim"] = {
            "form": "split",
            "why": "the split form is the specified one: f64 for the conserved state, the RK3 accumulation and "
                   "the metric/Jacobian terms; f32 for projection, WENO, LLF and viscous fluxes",
            "speedup_vs_fp64": reduced["split"]["speedup_vs_fp64"],
            "rel_l2_vs_fp64": reduced["split"]["rel_l2_vs_fp64"]}
    s64.close()

    # headline e2e: the reference-facing drop-in entry points with host FLOW
    dropin = bench_dropin(ctx, torch, stream, case, args, world, device=f"cuda:{local}")
    line["dropin"] = dropin
    line["e2e_resident"] = dict(line["e2e"], api="cfd_solver_set_flow / cfd_solver_step / cfd_solver_get_flow")
    line["e2e"] = dict(dropin["e2e"], api="cfd_uq / cfd_viscous / cfd_weno per stage, FLOW written and read "
                                          "back every step (pinned host memory)")
    if args.diag_steps > 0 and args.config.startswith("tgv"):
        line["tgv_diagnostics"] = bench_diagnostics(ctx, case, args)
    if args.batch_count > 0:
        line["batched"] = bench_batched(ctx, torch, stream, args)
    if args.serve_requests > 0:
        line["serving"] = bench_serving(ctx, args)
    if args.naca_steps > 0:
        line["naca0012"] = bench_naca(ctx, torch, stream, args)
    if args.shock_steps > 0:
        line["shock"] = bench_shock(ctx, torch, stream, args)

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, cores, secs, flags = cpu_oracle_rate(case, args.cpu_steps)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": cpu_sample_text(args.cpu_steps, cfg["workload"], secs, cores, flags)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def load_peaks() -> dict:
    """Measured peaks of this GPU type (MEASURED_PEAKS.json: HBM copy GB/s, bf16)."""
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        return {}


def batched_cases(count: int, seed: int = 20261203):
    """Batched workload: `count` isentropic-vortex instances with lattice edge
    log-uniform in [32, 96], vortex strength uniform in [2, 6] and advection
    speed uniform in [0.2, 0.8] (seeded)."""
    import numpy as np
    from cfd_gb300 import cases
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(32), math.log(96)))))
        beta, u_inf = float(rng.uniform(2.0, 6.0)), float(rng.uniform(0.2, 0.8))
        out.append(cases.isentropic_vortex(n=n, beta=beta, u_inf=u_inf))
    return out


def bench_batched(ctx, torch, stream, args):
    """One persistent launch per RK stage over all instances; each form
    (tuned tiles); the reduced forms' error against FP64 after the same
    number of steps."""
    import numpy as np
    from cfd_gb300 import runtime
    t0 = time.perf_counter()
    cs = batched_cases(args.batch_count)
    gen_s = time.perf_counter() - t0
    nodes = sum(c.sd_node for c in cs)
    out = {"instances": len(cs), "nodes_total": nodes, "case_generation_s": gen_s,
           "workload": "isentropic vortices, edge log-uniform [32, 96], beta U[2,6], u_inf U[0.2,0.8], seed 20261203"}

    def timed(b, steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        b.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    forms = [f.strip() for f in args.batch_forms.split(",")]
    fp64_steps = max(1, args.batch_steps // 5)
    ref_steps = 1 + fp64_steps
    u_ref = None
    for prec in (FP64, SPLIT, MIXED):
        key = FORM_NAMES[prec]
        if key not in forms:
            continue
        steps = fp64_steps if prec == FP64 else args.batch_steps
        b = runtime.Batch(ctx, prec)
        slots = [b.add(c) for c in cs]
        if args.batch_tile:
            b.set_tiling(args.batch_tile)
        elif prec != FP64:
            b.tune(1)
        b.step(1)
        secs = timed(b, steps)
        info = b.info()
        out[key] = {"value": nodes * steps / secs, "unit": UNIT, "ms_per_step": 1e3 * secs / steps, "steps": steps,
                    "dtype": FORM_DTYPES[prec], "tile_nodes": info.tile_nodes, "face_tiles": info.face_tiles,
                    "blocks": info.blocks, "cuda_graph": info.graph, "device_gb": info.device_bytes / 1e9}
        if prec == FP64:
            u_ref = [b.get_u0(s)[1:] for s in slots]
        b.close()
    for prec in (SPLIT, MIXED):
        key = FORM_NAMES[prec]
        if u_ref is None or key not in out:
            continue
        # the reduced form after the same number of steps as the FP64 reference
        b = runtime.Batch(ctx, prec)
        slots = [b.add(c) for c in cs]
        b.step(ref_steps)
        num = sum(float(np.sum((b.get_u0(s)[1:] - u) ** 2)) for s, u in zip(slots, u_ref))
        den = sum(float(np.sum(u ** 2)) for u in u_ref)
        b.close()
        out[key]["rel_l2_vs_fp64"] = math.sqrt(num / den)
        out[key]["speedup_vs_fp64"] = out[key]["value"] / out["fp64"]["value"]
    return out


def bench_diagnostics(ctx, case, args):
    """Kinetic energy and enstrophy of the main case over `diag_steps` steps,
    the reduced forms against the FP64 form (which matches the oracle to
    1e-12)."""
    import numpy as np
    from cfd_gb300 import diagnostics, runtime
    every = max(1, args.diag_steps // 4)
    hist = {}
    for prec in (FP64, SPLIT, MIXED):
        s = runtime.Solver(ctx, case, precision=prec)
        s.set_flow(case.arrays["flow"])
        h = [diagnostics.kinetic_energy_enstrophy(case.arrays["flow"], case.arrays["metric"], case.arrays["det"],
                                                  case.shape)]
        done = 0
        while done < args.diag_steps:
            k = min(every, args.diag_steps - done)
            s.step(case.dt, k)
            done += k
            h.append(diagnostics.kinetic_energy_enstrophy(s.get_flow(), case.arrays["metric"], case.arrays["det"],
                                                          case.shape))
        s.close()
        hist[prec] = np.array(h)
    out = {"steps": args.diag_steps, "samples_every": every,
           "kinetic_energy_fp64": hist[FP64][:, 0].tolist(), "enstrophy_fp64": hist[FP64][:, 1].tolist()}
    for prec in (SPLIT, MIXED):
        err = np.abs(hist[prec] - hist[FP64]) / np.abs(hist[FP64])
        out[f"kinetic_energy_max_rel_err_{FORM_NAMES[prec]}"] = float(err[:, 0].max())
        out[f"enstrophy_max_rel_err_{FORM_NAMES[prec]}"] = float(err[:, 1].max())
    return out


def bench_naca(ctx, torch, stream, args):
    """NACA0012 O-grid (Mach 0.8, AoA 1.25 deg, Re 5e5, MTS LES), no-slip wall
    and inlet/outlet far field filled by the reference's boundary routine
    after every stage.  Each form from the same start (the free stream after
    one boundary fill); relative L2 and Linf of density and pressure of the
    reduced forms against FP64."""
    import numpy as np
    from cfd_gb300 import layout, runtime
    from cfd_gb300 import cases
    ni, nj, nk = (int(x) for x in args.naca_grid.split(","))
    t0 = time.perf_counter()
    case = cases.naca0012(ni=ni, nj=nj, nk=nk)
    gen_s = time.perf_counter() - t0
    # the reference fills the boundaries once before its time loop
    bnd = runtime.Boundary(ctx, case.arrays["grid"], case.bc)
    dev = ctx.alloc(case.arrays["flow"].nbytes)
    ctx.write(dev, case.arrays["flow"])
    bnd.fill(dev, case.params.mach, 1, case.sd_node)
    flow0 = np.empty_like(case.arrays["flow"])
    ctx.read(flow0, dev)
    ctx.free(dev)
    bnd.close()
    N = case.sd_node
    steps = args.naca_steps
    out = {"workload": f"naca0012_ogrid_{ni}x{nj}x{nk}_m0.8_aoa1.25_re5e5_les", "grid": [ni, nj, nk],
           "nodes_owned": N, "nodes_with_ghosts": case.g_node, "steps": steps, "dt": case.dt,
           "case_generation_s": gen_s,
           "boundary_lists": {t: int(len(getattr(case.bc, t))) for t in ("outlet", "inlet", "boundary", "wall")}}
    res = {}
    for prec in (FP64, SPLIT, MIXED):
        s = runtime.Solver(ctx, case, precision=prec)
        assert s.info().path == "structured"
        s.set_flow(flow0)
        s.step(case.dt, 1)        # untimed: the first stage runs the FP64 face tuner
        s.set_flow(flow0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        s.step(case.dt, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        secs = e0.elapsed_time(e1) / 1e3
        res[prec] = s.get_flow()[1:N + 1]
        prof = [s.profile_stage(j, case.dt) for j in range(3)]   # one more step, per-kernel times
        mb = list(s.info().face_blocks)
        s.close()
        out[FORM_NAMES[prec]] = {"value": N * steps / secs, "unit": UNIT, "ms_per_step": 1e3 * secs / steps,
                                 "dtype": FORM_DTYPES[prec], "kernels_ms_per_stage": _kernel_table(prof)}
        if prec == FP64:
            out["fp64"]["face_blocks_tuned"] = mb
    f = layout.FLOW
    for prec in (SPLIT, MIXED):
        key = FORM_NAMES[prec]
        for name in ("rho", "p"):
            a, b = res[prec][:, f[name]], res[FP64][:, f[name]]
            out[key][f"{name}_rel_l2_vs_fp64"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
            out[key][f"{name}_rel_linf_vs_fp64"] = float(np.abs(a - b).max() / np.abs(b).max())
        out[key]["speedup_vs_fp64"] = out[key]["value"] / out["fp64"]["value"]
    out["finite"] = bool(all(np.isfinite(r).all() for r in res.values()))
    return out


def _stream_offered(reqs) -> float:
    """Cell-updates/s the sampled stream offers: its work over its arrival span."""
    span = max(r.arrival for r in reqs) - min(r.arrival for r in reqs)
    return sum(r.n ** 3 * r.steps for r in reqs) / span if span > 0 else float("inf")


def _serve_summary(r, offered=None) -> dict:
    out = {"policy": r["policy"], "completed": r["requests"], "cell_updates_per_s": r["cell_updates_per_s"],
           "latency_p50_s": r["latency_p50_s"], "latency_p99_s": r["latency_p99_s"],
           "latency_mean_s": r["latency_mean_s"], "latency_max_s": r["latency_max_s"],
           "makespan_s": r["makespan_s"], "batch_steps": r["batch_steps"], "time_in_s": r["time_in_s"]}
    if offered is not None:
        out["offered_over_delivered"] = offered / r["cell_updates_per_s"] if r["cell_updates_per_s"] else None
    return out


def bench_serving(ctx, args):
    """Continuous batching of seeded Poisson request streams (vortex or
    Taylor-Green 50:50, edge log-uniform, step count uniform):
    * the workload's stream (50 req/s, edges [32, 160], steps [50, 400]) in
      each reduced form: at that rate the offered work is well above what one
      GPU delivers, so its latencies are a queue draining;
    * the same distribution at a rate below the measured capacity
      (serve_sub_load x capacity / mean request work), where latency is the
      steady-state service time; p99 of the first and second halves of the
      requests shows whether it stays bounded;
    * a reduced stream (edges [24, 48], steps [20, 60]) served in FP64 and in
      the reduced forms, with every request's relative L2 against its FP64
      result (density, velocity, pressure)."""
    import numpy as np
    from cfd_gb300 import layout, serving
    fill = args.serve_fill or serving.FILL_NODES
    rate, n_range, s_range = 50.0, (32, 160), (50, 400)
    e_work = serving.mean_request_work(n_range, s_range)
    out = {"workload": "Poisson(50/s) vortex/TGV 50:50, edge log-uniform [32,160], steps U[50,400], seed 20261203",
           "policy": "least_work", "fill_nodes": fill, "mean_request_cell_updates": e_work,
           "offered_cell_updates_per_s": rate * e_work}
    forms = [f.strip() for f in args.serve_forms.split(",") if f.strip()]
    name_to_prec = {v: k for k, v in FORM_NAMES.items()}
    reqs = serving.poisson_requests(args.serve_requests, rate=rate, n_range=n_range, steps_range=s_range)
    t0 = time.perf_counter()
    cache = serving.make_cases(reqs)
    out["case_generation_s"] = time.perf_counter() - t0
    out["requests"] = len(reqs)
    out["offered_in_stream_cell_updates_per_s"] = _stream_offered(reqs)
    capacity = {}
    for key in forms:
        srv = serving.Server(ctx, precision=name_to_prec[key], tune=True, fill_nodes=fill)
        r = srv.run(reqs, case_cache=cache)
        srv.close()
        out[key] = _serve_summary(r, out["offered_in_stream_cell_updates_per_s"])
        out[key]["dtype"] = FORM_DTYPES[name_to_prec[key]]
        # the highest mean arrival rate the form can serve: delivered capacity over the mean request work
        out[key]["saturation_rate_per_s"] = r["cell_updates_per_s"] / e_work
        out[key]["overloaded"] = rate > out[key]["saturation_rate_per_s"]
        capacity[key] = r["cell_updates_per_s"]
    if args.serve_sub_requests > 0 and forms:
        key = forms[0]
        sub_rate = args.serve_sub_load * capacity[key] / e_work
        reqs2 = serving.poisson_requests(args.serve_sub_requests, rate=sub_rate, n_range=n_range,
                                         steps_range=s_range, seed=20261204)
        cache2 = serving.make_cases(reqs2)
        srv = serving.Server(ctx, precision=name_to_prec[key], tune=True, fill_nodes=fill)
        r = srv.run(reqs2, case_cache=cache2)
        srv.close()
        done = sorted(r["completed"], key=lambda c: c.arrival)
        half = len(done) // 2
        lat = [np.array([c.latency for c in part]) for part in (done[:half], done[half:])]
        sub = _serve_summary(r, _stream_offered(reqs2))
        sub.update({"form": key, "arrival_rate_per_s": sub_rate, "load_fraction_of_capacity": args.serve_sub_load,
                    "offered_cell_updates_per_s": sub_rate * e_work,
                    "offered_in_stream_cell_updates_per_s": _stream_offered(reqs2),
                    "latency_p99_first_half_s": float(np.percentile(lat[0], 99)) if len(lat[0]) else None,
                    "latency_p99_second_half_s": float(np.percentile(lat[1], 99)) if len(lat[1]) else None,
                    "mean_service_s_at_capacity": e_work / capacity[key],
                    "workload": "the same distribution, seed 20261204"})
        out["below_capacity"] = sub
    if args.serve_acc_requests > 0:
        acc_n, acc_s = (24, 48), (20, 60)
        reqs3 = serving.poisson_requests(args.serve_acc_requests, rate=rate, n_range=acc_n, steps_range=acc_s,
                                         seed=20261205)
        cache3 = serving.make_cases(reqs3)
        results = {}
        acc = {"workload": f"Poisson(50/s) vortex/TGV 50:50, edge log-uniform [{acc_n[0]},{acc_n[1]}], "
                           f"steps U[{acc_s[0]},{acc_s[1]}], seed 20261205",
               "requests": len(reqs3), "offered_cell_updates_per_s": rate * serving.mean_request_work(acc_n, acc_s)}
        for prec in (FP64, SPLIT, MIXED):
            srv = serving.Server(ctx, precision=prec, tune=True, fill_nodes=fill, keep_results=True)
            r = srv.run(reqs3, case_cache=cache3)
            srv.close()
            results[prec] = {c.rid: c.flow for c in r["completed"]}
            acc[FORM_NAMES[prec]] = _serve_summary(r, acc["offered_cell_updates_per_s"])
        cols = [layout.FLOW[k] for k in ("rho", "u", "v", "w", "p")]
        for prec in (SPLIT, MIXED):
            errs = []
            for rid, f64 in results[FP64].items():
                got = results[prec][rid]
                errs.append(rel_l2(got[1:, cols], f64[1:, cols]))
            errs = np.array(errs)
            acc[FORM_NAMES[prec]].update({"requests_compared": int(len(errs)),
                                          "max_rel_l2_vs_fp64": float(errs.max()),
                                          "median_rel_l2_vs_fp64": float(np.median(errs))})
        out["accuracy_stream"] = acc
    return out


def bench_shock(ctx, torch, stream, args):
    """The shocked curvilinear case: a high-pressure slab (cases.shock_slab,
    256 x 64 x 64 nodes of the perturbed periodic lattice, Mach 0.8,
    Re 5e5 MTS LES, pressure ratio 10) drifting at 1.5 times the sound
    speed, for `shock_steps` steps in each form from the same start.  The
    shock is located in each form (largest pressure jump between
    i-neighbours, averaged over j and k); density and pressure of the reduced
    forms against FP64, relative L2 and Linf."""
    import numpy as np
    from cfd_gb300 import cases, layout, runtime
    shape = (256, 64, 64)
    t0 = time.perf_counter()
    case = cases.shock_slab(shape=shape)
    gen_s = time.perf_counter() - t0
    N, steps = case.sd_node, args.shock_steps
    ni, nj, nk = shape

    def front(flow):
        p = flow[1:, layout.FLOW["p"]].reshape(nk, nj, ni).mean(axis=(0, 1))
        jump = np.abs(np.roll(p, -1) - p)
        i = int(np.argmax(jump))
        a, b = p[i], p[(i + 1) % ni]
        w0, w1 = p[(i - 2) % ni], p[(i + 3) % ni]   # across the few cells WENO spreads the shock over
        return {"i_plus_half": i, "pressure_ratio_one_cell": float(max(a, b) / min(a, b)),
                "pressure_ratio_across_6_nodes": float(max(w0, w1) / min(w0, w1)),
                "max_jump_over_p_inf": float(jump[i] * 1.4 * case.params.mach ** 2)}

    out = {"workload": "shock_slab_256x64x64_perturbed_periodic_m0.8_re5e5_les_pratio10", "grid": list(shape),
           "steps": steps, "dt": case.dt, "case_generation_s": gen_s}
    res = {}
    for prec in (FP64, SPLIT, MIXED):
        s = runtime.Solver(ctx, case, precision=prec)
        s.set_flow(case.arrays["flow"])
        s.step(case.dt, 1)        # untimed: the first stage runs the FP64 face tuner
        s.set_flow(case.arrays["flow"])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        s.step(case.dt, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        secs = e0.elapsed_time(e1) / 1e3
        res[prec] = s.get_flow()
        mb = list(s.info().face_blocks)
        s.close()
        out[FORM_NAMES[prec]] = {"value": N * steps / secs, "unit": UNIT, "ms_per_step": 1e3 * secs / steps,
                                 "dtype": FORM_DTYPES[prec], "shock": front(res[prec])}
        if prec == FP64:
            out["fp64"]["face_blocks_tuned"] = mb
    f = layout.FLOW
    for prec in (SPLIT, MIXED):
        key = FORM_NAMES[prec]
        for name in ("rho", "p"):
            a, b = res[prec][1:, f[name]], res[FP64][1:, f[name]]
            out[key][f"{name}_rel_l2_vs_fp64"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
            out[key][f"{name}_rel_linf_vs_fp64"] = float(np.abs(a - b).max() / np.abs(b).max())
        out[key]["speedup_vs_fp64"] = out[key]["value"] / out["fp64"]["value"]
    out["finite"] = bool(all(np.isfinite(r[1:]).all() for r in res.values()))
    return out


def bench_dropin(ctx, torch, stream, case, args, world: int = 1, device=None):
    """The FP64 step through the three drop-in entry points on the
    reference's AoS buffers (what a reference host loop binds): U_Q ->
    Viscous -> Weno per stage.  Device-resident rate, and end to end with
    FLOW written from and read back to pinned host memory every step."""
    import numpy as np
    steps = args.dropin_steps if args.dropin_steps > 0 else args.steps
    N = case.sd_node
    dev = ctx.upload_case(case.arrays)
    flow0 = case.arrays["flow"]

    def run_step():
        for j in range(3):
            ctx.stage(dev, case.g_node, case.sd_node, case.params, j, case.dt)

    for _ in range(2):
        run_step()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launch_count
    with torch.cuda.stream(stream):
        e0.record(stream)
    for _ in range(steps):
        run_step()
    with torch.cuda.stream(stream):
        e1.record(stream)
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1e3
    launches = ctx.launch_count - launches0
    host_in = torch.empty(flow0.shape, dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty(flow0.shape, dtype=torch.float64, pin_memory=True).numpy()
    host_in[...] = flow0
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.write(dev["flow"], host_in)
        run_step()
        ctx.read(host_out, dev["flow"])
        host_in, host_out = host_out, host_in
    e2e_secs = time.perf_counter() - t0
    barrier(world)
    for p in dev.values():
        ctx.free(p)
    value, tmax = aggregate(secs, N * steps, world, device=device)
    e2e_value, _ = aggregate(e2e_secs, N * steps, world, device=device)
    return {"value": value, "unit": UNIT, "ms_per_step": 1e3 * tmax / steps, "steps": steps,
            "gpu_launches": launches,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(host_in.nbytes),
                    "d2h_bytes_per_step": int(host_out.nbytes)},
            "path": "cfd_uq / cfd_viscous / cfd_weno on the reference AoS buffers (neighbour-table gathers)"}


def _kernel_table(prof) -> dict:
    """Mean device ms per stage of each kernel name over the three stages."""
    acc = {}
    for stage in prof:
        for name, ms in stage:
            acc.setdefault(name, []).append(ms)
    return {k: sum(v) / len(v) for k, v in acc.items()}


def main(argv=None):
    args = parse_args(argv)
    __graft_entry__.load_package()
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
