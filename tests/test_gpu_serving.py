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
