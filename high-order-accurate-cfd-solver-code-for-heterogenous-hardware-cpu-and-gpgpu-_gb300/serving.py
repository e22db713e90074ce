"""Serving loop: continuous batching of independent solves on one GPU.

Requests (an initial-value problem on a periodic lattice plus a number of
SSP-RK3 steps) arrive over time.  The loop keeps every admitted solve's
state resident in one batch (``runtime.Batch``: one persistent launch per RK
stage over all instances) and, between steps:

* admits queued requests in arrival order while their device-memory
  footprint fits the batch budget (``cfd_batch_instance_bytes``);
* picks the admitted solves that advance in this step (``policy``) and
  queues one step of them (``Batch.step_async``: the host admits and
  schedules the next step while the device runs this one);
* retires the solves that reached their step count (their FLOW is read back
  as the result) and frees their memory for the queue.

Requests that arrive while others run join at the next step boundary, so
their work overlaps on the device with the solves already in flight.  The
reference has no serving layer; this is the builder's request loop around the
RHS path.  Latency = completion time - arrival time.

Policies:

* ``"all"``: every admitted solve advances every step.  Each solve then
  finishes after its own step count of batch steps, but every batch step
  costs the whole batch, so a small solve waits on the large ones.
* ``"least_work"`` (default): the solves with the least remaining work
  (nodes x remaining steps; arrival order breaks ties) advance, as many as
  it takes to reach ``fill_nodes`` lattice nodes per step, enough to keep the
  GPU busy; the others stay resident, held (``Batch.set_hold``).  This is
  shortest-remaining-work-first with a minimum batch size: the device does
  the same total work, and small solves finish first.  Solves that have
  not advanced for ``max_hold_s`` seconds go first, the longest wait first
  (aging), so a sustained stream of small requests cannot postpone a large
  one indefinitely.

Checkpoint/resume: with ``checkpoint_dir`` every solve keeps the reference's
restart pair (files.py) under ``<dir>/req_<rid>/``, written every
``checkpoint_every`` batch steps and at completion; a request admitted again
(after the loop stopped, e.g. ``max_batch_steps``) starts from its newest
complete restart with the remaining steps.  Restarting from FLOW at a step
boundary is exact for the FP64 form (every stage's U_Q rebuilds U from FLOW).
"""
from __future__ import annotations

import concurrent.futures as cf
import dataclasses
import math
import pathlib
import time

import numpy as np

from . import cases, files, runtime


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds from the start of the run
    kind: str               # "vortex" or "tgv"
    n: int                  # lattice edge (n^3 nodes)
    steps: int
    seed: int


@dataclasses.dataclass
class Completed:
    rid: int
    arrival: float
    admitted: float
    finished: float
    nodes: int
    steps: int
    flow: np.ndarray | None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def poisson_requests(count: int, rate: float = 50.0, n_range=(32, 160), steps_range=(50, 400),
                     seed: int = 20261203) -> list:
    """Seeded request stream: Poisson arrivals of mean rate `rate` per second,
    50/50 vortex/Taylor-Green, lattice edge log-uniform in n_range, step count
    uniform in steps_range."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for r in range(count):
        t += rng.exponential(1.0 / rate)
        kind = "vortex" if rng.random() < 0.5 else "tgv"
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        out.append(Request(r, t, kind, n, steps, int(rng.integers(0, 2**31 - 1))))
    return out


def mean_request_work(n_range=(32, 160), steps_range=(50, 400), samples: int = 400000, seed: int = 1) -> float:
    """Mean cell-updates (nodes x steps) of one request of the stream that
    poisson_requests draws with these ranges: the mean of n^3 over the
    rounded log-uniform edge (sampled) times the mean step count."""
    rng = np.random.default_rng(seed)
    n = np.round(np.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1]), samples)))
    return float(np.mean(n ** 3)) * 0.5 * (steps_range[0] + steps_range[1])


def make_cases(requests, workers: int = 0) -> dict:
    """rid -> case of every request, generated on a pool of host threads
    (the generators spend their time in numpy, which releases the GIL).
    Taylor-Green cases of one edge are identical, so each edge is made once."""
    import os
    workers = workers or min(16, os.cpu_count() or 1)
    tgv_edges = sorted({r.n for r in requests if r.kind == "tgv"})
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        tgv = dict(zip(tgv_edges, ex.map(lambda n: cases.taylor_green(n=n), tgv_edges)))
        vort = [r for r in requests if r.kind != "tgv"]
        made = dict(zip((r.rid for r in vort), ex.map(make_case, vort)))
    for r in requests:
        if r.kind == "tgv":
            made[r.rid] = tgv[r.n]
    return made


def least_work_first(entries, fill_nodes: int, max_hold_s: float = math.inf) -> set:
    """Slots that advance under the "least_work" policy.  entries: iterable
    of (slot, nodes, remaining steps, arrival[, seconds since its last
    step]).  Takes the slots that waited longer than max_hold_s first, the
    longest wait first, then the others in order of nodes x remaining steps
    (then arrival), until their nodes reach fill_nodes; at least one slot
    when there is any."""
    def key(e):
        waited = e[4] if len(e) > 4 else 0.0
        if waited > max_hold_s:
            return (0, -waited, e[0])
        return (1, e[1] * e[2], e[3], e[0])

    chosen, nodes = set(), 0
    for slot, n, left, arrival, *_ in sorted(entries, key=key):
        if chosen and nodes >= fill_nodes:
            break
        chosen.add(slot)
        nodes += n
    return chosen


def make_case(req: Request):
    rng = np.random.default_rng(req.seed)
    if req.kind == "vortex":
        return cases.isentropic_vortex(n=req.n, beta=float(rng.uniform(2.0, 6.0)), u_inf=float(rng.uniform(0.2, 0.8)))
    return cases.taylor_green(n=req.n)


# Lattice nodes per batch step under "least_work".  The batched mixed
# stage kernel runs at 1.0e9 cell-updates/s from 2.6e5 nodes on and at
# 1.06e9 from 1e6 (one GB300); a smaller step finishes small solves sooner.
# On the 24-request Poisson stream 2^19, 2^20 and 2^21 nodes gave the same
# throughput (1.12e9) and latency p50 0.56, 0.71 and 1.09 s.
FILL_NODES = 1 << 19


class Server:
    """Continuous-batching request loop over one ``runtime.Batch``."""

    def __init__(self, ctx, precision: int = 1, capacity_bytes: int = 0, keep_results: bool = False,
                 tune: bool = False, policy: str = "least_work", fill_nodes: int = FILL_NODES,
                 stage_workers: int = 1, max_hold_s: float = 5.0, steps_per_call: int = 8):
        if policy not in ("all", "least_work"):
            raise ValueError(f"unknown policy {policy!r}")
        self.batch = runtime.Batch(ctx, precision, capacity_bytes)
        self.precision = precision
        self.policy = policy
        self.fill_nodes = int(fill_nodes)
        self.stage_workers = int(stage_workers)
        self.max_hold_s = float(max_hold_s)
        self.steps_per_call = max(1, int(steps_per_call))
        self.keep_results = keep_results
        self.tune = tune
        self.info0 = self.batch.info()

    def close(self):
        self.batch.close()

    def run(self, requests: list, case_cache: dict | None = None, clock=time.perf_counter,
            checkpoint_dir=None, checkpoint_every: int = 0, max_batch_steps: int | None = None) -> dict:
        """Serves `requests` (sorted by arrival) in real time; returns the
        completed solves and summary statistics.  max_batch_steps stops the
        loop early (the unfinished solves are reported as `pending`)."""
        case_cache = {} if case_cache is None else case_cache
        queue = list(sorted(requests, key=lambda r: r.arrival))
        active = {}              # slot -> [request, remaining steps, admitted time, case, next restart number,
        #                                   time of its last step]
        held = set()             # slots the batch currently leaves out of its steps
        done = []

        def ckpt_dir(req):
            d = pathlib.Path(checkpoint_dir) / f"req_{req.rid}"
            d.mkdir(parents=True, exist_ok=True)
            return d

        def checkpoint(slot):
            req, left, _, case, num, _ = active[slot]
            files.write_restart(ckpt_dir(req), self.batch.get_flow(slot), case.sd_node, req.steps - left, num)
            active[slot][4] = 3 - num
        budget = self.info0.capacity_bytes
        spent = {"admit": 0.0, "step": 0.0, "sync": 0.0, "retire": 0.0}   # wall time inside the batch calls

        def prepare(req):
            """Host half of an admission: the case, its restart and the
            staged instance (runs on the worker thread)."""
            c = case_cache.get(req.rid) or make_case(req)
            left, num, flow = req.steps, 1, None
            if checkpoint_dir is not None:
                got = files.read_restart(ckpt_dir(req), c.sd_node)
                if got is not None:
                    values, it, num = got
                    flow = files.restart_flow(c.arrays["flow"], values, c.params.mach)
                    left = req.steps - it
            return c, left, num, flow, runtime.Batch.stage(c, flow=flow)

        pool = cf.ThreadPoolExecutor(max_workers=self.stage_workers) if self.stage_workers > 0 else None
        prepared = {}            # rid -> future of prepare(req)

        def prepare_arrived(now, lookahead=2):
            for req in queue[:lookahead]:
                if req.arrival > now:
                    break
                if req.rid not in prepared:
                    prepared[req.rid] = pool.submit(prepare, req)

        try:
            return self._loop(queue, active, held, done, prepare, prepare_arrived, prepared, pool, budget, spent,
                              clock, checkpoint_dir, checkpoint_every, max_batch_steps, checkpoint)
        finally:
            if pool is not None:
                pool.shutdown(wait=True, cancel_futures=True)

    def _loop(self, queue, active, held, done, prepare, prepare_arrived, prepared, pool, budget, spent, clock,
              checkpoint_dir, checkpoint_every, max_batch_steps, checkpoint):
        t0 = clock()
        steps_run = 0
        tuned = not self.tune
        while queue or active:
            now = clock() - t0
            # admission: arrived requests in order while their footprint fits;
            # their host half runs on the worker while the device steps
            used = self.batch.info().device_bytes
            if pool is not None:
                prepare_arrived(now)
            while queue and queue[0].arrival <= now:
                req = queue[0]
                need = runtime.Batch.instance_bytes(self.precision, req.n ** 3)
                if used + need > budget:
                    if not active:
                        raise RuntimeError(f"request {req.rid} ({req.n}^3) exceeds the device budget")
                    break
                if pool is None:
                    job = prepare(req)
                else:
                    if req.rid not in prepared:
                        prepared[req.rid] = pool.submit(prepare, req)
                    fut = prepared[req.rid]
                    if not fut.done() and active:
                        break                  # keep stepping; admit it when it is ready
                    job = fut.result()
                    del prepared[req.rid]
                c, left, num, flow, staged = job
                ta = clock()
                slot = self.batch.add_staged(staged)
                spent["admit"] += clock() - ta
                used += need
                active[slot] = [req, left, clock() - t0, c, num, clock() - t0]
                queue.pop(0)
                if left <= 0:       # finished before the stop: report it again
                    self.batch.remove(slot)
                    active.pop(slot)
                    done.append(Completed(req.rid, req.arrival, clock() - t0, clock() - t0, req.n ** 3, req.steps,
                                          flow if self.keep_results else None))
            if not active:
                if not queue:
                    break
                time.sleep(max(0.0, min(queue[0].arrival - (clock() - t0), 0.05)))
                continue
            if max_batch_steps is not None and steps_run >= max_batch_steps:
                break
            if self.policy == "all":
                run = set(active)
            else:
                now = clock() - t0
                run = least_work_first(((s, a[0].n ** 3, a[1], a[0].arrival, now - a[5]) for s, a in active.items()),
                                       self.fill_nodes, self.max_hold_s)
            for s in active:
                if (s in held) == (s in run):
                    self.batch.set_hold(s, s not in run)
                    held.symmetric_difference_update({s})
            ts = clock()
            if not tuned and len(run) > 1:
                self.batch.tune(1)
                tuned = True
            # several steps per call while nothing can change the schedule: no
            # request left to arrive, no solve of the step finishing before
            # its last step, no checkpoint or stop in between
            k = 1
            if not queue and checkpoint_dir is None and max_batch_steps is None:
                k = max(1, min(self.steps_per_call, min(active[s][1] for s in run)))
            self.batch.step_async(k)
            spent["step"] += clock() - ts
            steps_run += k
            finished = [s for s in run if active[s][1] == k]
            t_step = clock() - t0
            for s in run:
                active[s][1] -= k
                active[s][5] = t_step
            if finished or checkpoint_dir is not None:
                ts = clock()
                self.batch.sync()          # results are read after the step has run
                spent["sync"] += clock() - ts
            if checkpoint_dir is not None:
                for s in active:
                    if s in finished or (checkpoint_every and steps_run % checkpoint_every == 0):
                        checkpoint(s)
            for s in finished:
                req, _, adm, _, _, _ = active.pop(s)
                tr = clock()
                flow = self.batch.get_flow(s) if self.keep_results else None
                self.batch.remove(s)
                spent["retire"] += clock() - tr
                held.discard(s)
                done.append(Completed(req.rid, req.arrival, adm, clock() - t0, req.n ** 3, req.steps, flow))
        self.batch.sync()
        pending = [a[0].rid for a in active.values()] + [r.rid for r in queue]
        for s in list(active):          # a stop keeps the progress of the solves in flight
            if checkpoint_dir is not None:
                checkpoint(s)
            self.batch.remove(s)
        makespan = clock() - t0
        lat = np.array([c.latency for c in done])
        work = float(sum(c.nodes * c.steps for c in done))
        return {
            "completed": done,
            "requests": len(done),
            "makespan_s": makespan,
            "batch_steps": steps_run,
            "cell_updates": work,
            "cell_updates_per_s": work / makespan if makespan > 0 else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "latency_max_s": float(lat.max()) if len(lat) else None,
            "latency_mean_s": float(lat.mean()) if len(lat) else None,
            "policy": self.policy,
            "time_in_s": spent,
            "pending": pending,
        }
