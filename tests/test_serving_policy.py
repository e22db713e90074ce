"""Scheduling of the serving loop on the host: the "least_work" policy picks
the solves with the least remaining work up to a node budget, held solves do
not advance, and every solve still gets exactly its own step count.  The
batch is a stand-in that counts steps per slot and advances a simulated
clock by the nodes it steps (no GPU)."""
from __future__ import annotations

import types

import numpy as np
import pytest


def test_least_work_first_orders_by_remaining_work(pkg):
    from cfd_gb300.serving import least_work_first
    # (slot, nodes, remaining steps, arrival)
    e = [(0, 1000, 10, 0.0), (1, 10, 50, 0.1), (2, 100, 3, 0.2), (3, 500, 1, 0.3)]
    # remaining work: slot 0 10,000, slot 1 500, slot 2 300, slot 3 500
    assert least_work_first(e, 1) == {2}                  # slot 2's 100 nodes already reach the budget
    assert least_work_first(e, 0) == {2}                  # at least one slot
    assert least_work_first(e, 101) == {2, 1}             # 300, then 500 (tie with slot 3, earlier arrival)
    assert least_work_first(e, 111) == {2, 1, 3}
    assert least_work_first(e, 10 ** 9) == {0, 1, 2, 3}
    assert least_work_first([], 5) == set()


class FakeBatch:
    """runtime.Batch stand-in: FLOW of a slot = the steps it was advanced."""
    sim = None

    def __init__(self, ctx, precision, capacity_bytes):
        self.slots, self.hold, self.next = {}, {}, 0
        self.capacity = capacity_bytes or 10 ** 12
        self.rate = 1e9                                   # simulated nodes x steps per second

    @staticmethod
    def instance_bytes(precision, nodes):
        return 100 * nodes

    def info(self):
        used = sum(100 * n for n, _ in self.slots.values())
        return types.SimpleNamespace(capacity_bytes=self.capacity, device_bytes=used)

    @staticmethod
    def stage(case, flow=None):
        return case

    def add_staged(self, staged):
        return self.add(staged)

    def add(self, case, flow=None):
        s = min(set(range(len(self.slots) + 1)) - set(self.slots))
        self.slots[s] = (case.nodes, 0)
        self.hold[s] = False
        return s

    def set_hold(self, slot, hold):
        assert slot in self.slots
        self.hold[slot] = bool(hold)

    def tune(self, steps):
        pass

    def step(self, n=1):
        nodes = 0
        for s, (nn, k) in list(self.slots.items()):
            if not self.hold[s]:
                self.slots[s] = (nn, k + n)
                nodes += nn
        FakeBatch.sim[0] += n * (nodes / self.rate + 1e-5)

    def step_async(self, n=1):
        self.step(n)

    def sync(self):
        pass

    def get_flow(self, slot):
        return np.array([float(self.slots[slot][1])])

    def remove(self, slot):
        del self.slots[slot]
        del self.hold[slot]

    def close(self):
        pass


def _serve(monkeypatch, reqs, policy, fill, workers=0):
    from cfd_gb300 import serving
    FakeBatch.sim = [0.0]
    monkeypatch.setattr(serving.runtime, "Batch", FakeBatch)
    monkeypatch.setattr(serving.time, "sleep", lambda s: FakeBatch.sim.__setitem__(0, FakeBatch.sim[0] + s))
    cache = {r.rid: types.SimpleNamespace(nodes=r.n ** 3) for r in reqs}
    srv = serving.Server(None, precision=1, keep_results=True, policy=policy, fill_nodes=fill,
                         stage_workers=workers)
    return srv.run(reqs, case_cache=cache, clock=lambda: FakeBatch.sim[0])


@pytest.mark.parametrize("policy,fill,workers", [("all", 0, 0), ("least_work", 1, 0), ("least_work", 300_000, 0),
                                                 ("least_work", 300_000, 1), ("all", 0, 2)])
def test_every_solve_gets_its_steps(pkg, monkeypatch, policy, fill, workers):
    """Also with the host half of admission on worker threads, where a
    request joins once its staging is done."""
    from cfd_gb300 import serving
    reqs = serving.poisson_requests(30, rate=50.0, n_range=(16, 96), steps_range=(5, 60), seed=3)
    out = _serve(monkeypatch, reqs, policy, fill, workers)
    assert out["requests"] == len(reqs) and out["pending"] == []
    assert out["policy"] == policy
    for c in out["completed"]:
        req = next(r for r in reqs if r.rid == c.rid)
        assert c.flow[0] == req.steps, (policy, c.rid)
        assert c.finished >= c.admitted >= req.arrival


def test_least_work_lowers_mean_latency(pkg, monkeypatch):
    """Same simulated device rate: small solves no longer wait on the large
    ones, so the mean latency drops, and the makespan stays close."""
    from cfd_gb300 import serving
    reqs = serving.poisson_requests(24, rate=50.0, n_range=(32, 160), steps_range=(50, 400), seed=20261203)
    lock = _serve(monkeypatch, reqs, "all", 0)
    srpt = _serve(monkeypatch, reqs, "least_work", 1 << 22)
    assert srpt["latency_mean_s"] < 0.6 * lock["latency_mean_s"]
    assert srpt["latency_p50_s"] < lock["latency_p50_s"]
    assert srpt["makespan_s"] < 1.05 * lock["makespan_s"]


def test_longest_waiting_slot_goes_first(pkg):
    from cfd_gb300.serving import least_work_first
    # (slot, nodes, remaining steps, arrival, seconds since its last step)
    e = [(0, 1000, 10, 0.0, 9.0), (1, 10, 50, 0.1, 6.0), (2, 100, 3, 0.2, 0.0)]
    assert least_work_first(e, 1) == {2}                   # no bound on the wait
    assert least_work_first(e, 1, max_hold_s=5.0) == {0}   # waited longest, despite the most work
    assert least_work_first(e, 1001, max_hold_s=5.0) == {0, 1}
    assert least_work_first(e, 1011, max_hold_s=5.0) == {0, 1, 2}


def test_aging_bounds_the_wait_of_a_large_solve(pkg, monkeypatch):
    """A large solve among an overload of small ones: without aging it runs
    after every small solve of the stream; with a short max_hold_s it takes
    its turn among the longest-waiting solves and finishes well before the
    stream is drained."""
    from cfd_gb300 import serving

    def stream():
        reqs = [serving.Request(0, 0.0, "vortex", 96, 60, 1)]
        # small solves (2.6 ms of simulated device time each) arriving every 1 ms: an overload
        reqs += [serving.Request(r, 0.001 * r, "vortex", 40, 40, 1) for r in range(1, 600)]
        return reqs

    def finish_of_large(max_hold):
        FakeBatch.sim = [0.0]
        monkeypatch.setattr(serving.runtime, "Batch", FakeBatch)
        monkeypatch.setattr(serving.time, "sleep", lambda s: FakeBatch.sim.__setitem__(0, FakeBatch.sim[0] + s))
        reqs = stream()
        cache = {r.rid: types.SimpleNamespace(nodes=r.n ** 3) for r in reqs}
        srv = serving.Server(None, precision=1, keep_results=True, policy="least_work", fill_nodes=1,
                             stage_workers=0, max_hold_s=max_hold)
        out = srv.run(reqs, case_cache=cache, clock=lambda: FakeBatch.sim[0])
        assert all(c.flow[0] == next(r for r in reqs if r.rid == c.rid).steps for c in out["completed"])
        big = next(c for c in out["completed"] if c.rid == 0)
        return big.finished, out["makespan_s"]

    late, makespan = finish_of_large(1e9)
    early, _ = finish_of_large(0.005)              # one step at least every ~5 ms
    assert late > 0.9 * makespan                    # starved until the stream drained
    assert early < 0.8 * late


def test_unknown_policy_is_rejected(pkg):
    from cfd_gb300 import serving
    with pytest.raises(ValueError):
        serving.Server(None, policy="round_robin")
