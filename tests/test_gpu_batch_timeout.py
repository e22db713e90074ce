"""The batched kernel's bounded grid-barrier wait, made to expire.

With a deadline of 0 ns, every block that reaches the barrier before the
last one gives up at once (after at most a few hundred ns of polling),
sets the timeout flag and skips the rest of the stage; the last block
completes the barrier and finishes its own tiles.  Nothing spins and no
access leaves its buffers, so the context stays usable.  The test checks
that the step reports CFD_ETIMEOUT once, that the interrupted instances are
refused until restored, and that after cfd_batch_set_flow the batch steps
normally and matches a batch built from the same states.
(The reference ends the process on any kernel failure, Solver.cpp:378-381.)
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cases_for_timeout():
    from cfd_gb300 import cases
    return [cases.isentropic_vortex(n=24), cases.taylor_green(n=20),
            cases.isentropic_vortex(n=20, beta=3.0, u_inf=0.3, shape=(20, 24, 16))]


@pytest.mark.parametrize("precision", [0, 1])
def test_barrier_timeout_reports_once_and_recovers(ctx, precision):
    from cfd_gb300 import abi, runtime
    cs = cases_for_timeout()
    b = runtime.Batch(ctx, precision)
    slots = [b.add(c) for c in cs]
    b.step(1)
    assert b.info().blocks > 1
    saved = [b.get_flow(s) for s in slots]

    b.set_wait_limit(0)
    with pytest.raises(abi.CfdError) as e:
        b.step(1)
    assert e.value.status == abi.ETIMEOUT
    assert all(b.slot_status(s) == abi.ETIMEOUT for s in slots)

    # the deadline back at its default: the interrupted instances are refused
    b.set_wait_limit(-1)
    with pytest.raises(abi.CfdError) as e:
        b.step(1)
    assert e.value.status == abi.ETIMEOUT

    for s, f in zip(slots, saved):
        b.set_flow(s, f)
    assert all(b.slot_status(s) == abi.OK for s in slots)
    b.step(2)                      # no latched timeout

    ref = runtime.Batch(ctx, precision)
    rs = [ref.add(c, flow=f) for c, f in zip(cs, saved)]
    ref.step(2)
    for s, r in zip(slots, rs):
        assert np.array_equal(b.get_flow(s), ref.get_flow(r))
        assert np.array_equal(b.get_u0(s), ref.get_u0(r))
    ref.close()
    b.close()


def test_held_instance_survives_a_timeout(ctx):
    """An instance held out of the timed-out step keeps its state and steps
    afterwards without a restore."""
    from cfd_gb300 import abi, runtime
    cs = cases_for_timeout()
    b = runtime.Batch(ctx, 1)
    slots = [b.add(c) for c in cs]
    b.set_hold(slots[0], True)
    before = b.get_flow(slots[0])
    b.set_wait_limit(0)
    with pytest.raises(abi.CfdError):
        b.step(1)
    assert b.slot_status(slots[0]) == abi.OK
    assert np.array_equal(b.get_flow(slots[0]), before)
    b.set_wait_limit(-1)
    for s in slots[1:]:
        b.remove(s)
    b.set_hold(slots[0], False)
    b.step(1)
    b.close()
