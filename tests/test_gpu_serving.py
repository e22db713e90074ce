"""Serving loop (continuous batching): requests join the resident batch as
they arrive and memory allows; every result must equal the same solve run
alone (bitwise), and the loop reports latency percentiles."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_requests():
    from cfd_gb300 import serving
    reqs = serving.poisson_requests(7, rate=400.0, n_range=(8, 14), steps_range=(2, 6), seed=7)
    return reqs


@pytest.mark.parametrize("precision", [1, 0])
def test_served_results_equal_alone(ctx, precision):
    from cfd_gb300 import runtime, serving
    reqs = small_requests()
    cache = {r.rid: serving.make_case(r) for r in reqs}
    # a budget that holds only some of the requests at once: the rest queue
    per = max(runtime.Batch.instance_bytes(precision, r.n ** 3) for r in reqs)
    srv = serving.Server(ctx, precision=precision, capacity_bytes=int(3.5 * per), keep_results=True)
    out = srv.run(reqs, case_cache=cache)
    srv.close()
    assert out["requests"] == len(reqs)
    assert out["latency_p99_s"] >= out["latency_p50_s"] > 0
    for c in out["completed"]:
        req = next(r for r in reqs if r.rid == c.rid)
        alone = runtime.Batch(ctx, precision)
        s = alone.add(cache[c.rid])
        alone.step(req.steps)
        assert np.array_equal(alone.get_flow(s), c.flow), c.rid
        alone.close()


def test_checkpoint_and_resume_equal_uninterrupted(ctx, tmp_path):
    """FP64 serving stopped after a few batch steps (every solve in flight
    checkpointed to its restart pair), then resumed by a new loop from the
    restart files: every result equals the uninterrupted solve bit for bit
    (restart values carry 17 digits, and the FP64 stage rebuilds U from
    FLOW)."""
    from cfd_gb300 import files, runtime, serving
    reqs = serving.poisson_requests(5, rate=1000.0, n_range=(8, 12), steps_range=(6, 10), seed=11)
    cache = {r.rid: serving.make_case(r) for r in reqs}
    srv = serving.Server(ctx, precision=0, keep_results=True)
    first = srv.run(reqs, case_cache=cache, checkpoint_dir=tmp_path, checkpoint_every=2, max_batch_steps=4)
    srv.close()
    assert first["pending"]                                    # stopped with work left
    some = [r for r in reqs if (tmp_path / f"req_{r.rid}").exists()]
    assert some and files.read_restart(tmp_path / f"req_{some[0].rid}", cache[some[0].rid].sd_node) is not None
    left = [r for r in reqs if r.rid in first["pending"]]
    srv = serving.Server(ctx, precision=0, keep_results=True)
    second = srv.run(left, case_cache=cache, checkpoint_dir=tmp_path, checkpoint_every=2)
    srv.close()
    assert second["pending"] == [] and second["requests"] == len(left)
    results = {c.rid: c.flow for c in first["completed"] + second["completed"]}
    assert set(results) == {r.rid for r in reqs}
    for r in reqs:
        alone = runtime.Batch(ctx, 0)
        s = alone.add(cache[r.rid])
        alone.step(r.steps)
        assert np.array_equal(alone.get_flow(s)[1:], results[r.rid][1:]), r.rid
        alone.close()
