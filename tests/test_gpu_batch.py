"""Batched lattices (cfd_batch_*): one persistent launch per RK stage over
instances of different sizes.  Each instance must give the same result in a
mix as alone (bitwise: the per-node arithmetic does not depend on the batch),
FP64 instances must match the oracle (relative L2 <= 1e-12), and mixed
instances the FP64 form (<= 1e-6)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import copy_arrays, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def mix_cases():
    from cfd_gb300 import cases
    return [
        cases.isentropic_vortex(n=12, shape=(12, 10, 8)),
        cases.taylor_green(n=10, shape=(10, 12, 9)),
        cases.isentropic_vortex(n=9, beta=3.0, u_inf=0.3, shape=(9, 9, 11)),
        cases.taylor_green(n=8, shape=(8, 8, 8), amp=0.03),
    ]


@pytest.mark.parametrize("precision", [0, 1])
def test_mix_equals_alone_bitwise(ctx, precision):
    from cfd_gb300 import runtime
    cs = mix_cases()
    mix = runtime.Batch(ctx, precision)
    slots = [mix.add(c) for c in cs]
    info = mix.info()
    assert info.n_active == len(cs) and info.nodes_total == sum(c.sd_node for c in cs)
    mix.step(3)
    for c, s in zip(cs, slots):
        alone = runtime.Batch(ctx, precision)
        a = alone.add(c)
        alone.step(3)
        assert np.array_equal(alone.get_flow(a), mix.get_flow(s))
        assert np.array_equal(alone.get_u0(a), mix.get_u0(s))
        alone.close()
    mix.close()


def test_fp64_batch_matches_oracle_and_solver(ctx, oracle_mod):
    from cfd_gb300 import runtime
    cs = mix_cases()
    b = runtime.Batch(ctx, 0)
    slots = [b.add(c) for c in cs]
    b.step(4)
    for c, s in zip(cs, slots):
        a = copy_arrays(c.arrays)
        oracle_mod.rk3_steps(a, c.g_node, c.sd_node, c.params, c.dt, 4)
        own = slice(1, c.sd_node + 1)
        got = b.get_flow(s)
        assert rel_l2(got[own], a["flow"][own]) <= TOL
        sv = runtime.Solver(ctx, c)
        sv.set_flow(c.arrays["flow"])
        sv.step(c.dt, 4)
        assert np.array_equal(sv.get_flow()[own], got[own])   # same per-node arithmetic
        sv.close()
    b.close()


def test_mixed_batch_error_budget(ctx):
    from cfd_gb300 import runtime
    cs = mix_cases()
    res = []
    for prec in (0, 1):
        b = runtime.Batch(ctx, prec)
        slots = [b.add(c) for c in cs]
        b.step(6)
        res.append([b.get_u0(s)[1:] for s in slots])
        b.close()
    for u64, um in zip(*res):
        assert rel_l2(um, u64) <= 1e-6


def test_add_remove_between_steps_and_slot_reuse(ctx):
    from cfd_gb300 import runtime
    cs = mix_cases()
    b = runtime.Batch(ctx, 1)
    s0 = b.add(cs[0])
    s1 = b.add(cs[1])
    b.step(2)
    b.remove(s0)
    s2 = b.add(cs[2])
    assert s2 == s0                      # freed slot reused
    b.step(1)
    # instance 1 stepped 3 times in a changing batch == alone 3 steps
    alone = runtime.Batch(ctx, 1)
    a = alone.add(cs[1])
    alone.step(3)
    assert np.array_equal(alone.get_flow(a), b.get_flow(s1))
    # instance 2 stepped once after joining == alone 1 step
    alone2 = runtime.Batch(ctx, 1)
    a2 = alone2.add(cs[2])
    alone2.step(1)
    assert np.array_equal(alone2.get_flow(a2), b.get_flow(s2))
    for x in (b, alone, alone2):
        x.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_held_instance_does_not_advance(ctx, precision):
    """cfd_batch_set_hold: a held instance keeps its state through steps of
    the others and, released, continues as if it had never paused."""
    from cfd_gb300 import runtime
    cs = mix_cases()
    b = runtime.Batch(ctx, precision)
    s = [b.add(c) for c in cs[:3]]
    b.step(1)
    before = b.get_flow(s[1])
    b.set_hold(s[1], True)
    b.set_hold(s[1], True)               # idempotent
    assert b.info().n_held == 1
    b.step(2)
    assert np.array_equal(b.get_flow(s[1]), before)
    b.set_hold(s[0], True)
    b.set_hold(s[2], True)
    b.step(1)                            # everything held: nothing moves
    assert np.array_equal(b.get_flow(s[1]), before)
    for x in s:
        b.set_hold(x, False)
    assert b.info().n_held == 0
    b.step(1)
    got = {x: b.get_flow(x) for x in s}
    for x, c, n in zip(s, cs[:3], (4, 2, 4)):
        alone = runtime.Batch(ctx, precision)
        a = alone.add(c)
        alone.step(n)
        assert np.array_equal(alone.get_flow(a), got[x]), x
        alone.close()
    with pytest.raises(Exception):
        b.set_hold(99, True)
    b.close()


def test_staged_add_equals_add(ctx):
    """cfd_batch_stage on a worker thread + cfd_batch_add_staged give the
    instance cfd_batch_add gives; a table the batch cannot take fails at
    cfd_batch_add_staged with the same status; an unused staged instance is
    freed."""
    import concurrent.futures as cf
    from cfd_gb300 import abi, cases, runtime
    cs = mix_cases()
    with cf.ThreadPoolExecutor(max_workers=2) as pool:
        staged = list(pool.map(runtime.Batch.stage, cs[:2]))
    a = runtime.Batch(ctx, 1)
    s = [a.add_staged(st) for st in staged]
    with pytest.raises(ValueError):
        a.add_staged(staged[0])                      # consumed
    a.step(2)
    b = runtime.Batch(ctx, 1)
    t = [b.add(c) for c in cs[:2]]
    b.step(2)
    for x, y in zip(s, t):
        assert np.array_equal(a.get_flow(x), b.get_flow(y))
    bad = runtime.Batch.stage(cases.ghost_box(shape=(6, 6, 6)))
    with pytest.raises(abi.CfdError) as e:
        a.add_staged(bad)
    assert e.value.status == abi.EUNSUPPORTED
    unused = runtime.Batch.stage(cs[3])
    del unused
    a.close()
    b.close()


def test_async_steps_equal_steps_and_report_at_sync(ctx):
    """cfd_batch_step_async queues the same steps as cfd_batch_step (the
    same bits), also across holds, removals and additions between calls;
    a non-finite instance is reported by the next cfd_batch_sync."""
    from cfd_gb300 import abi, runtime
    cs = mix_cases()
    a = runtime.Batch(ctx, 1)
    s = [a.add(c) for c in cs[:3]]
    for _ in range(3):
        a.step_async(1)
    a.set_hold(s[0], True)
    a.step_async(2)
    a.remove(s[2])
    s3 = a.add(cs[3])
    a.step_async(1)
    a.sync()
    b = runtime.Batch(ctx, 1)
    t = [b.add(c) for c in cs[:3]]
    b.step(3)
    b.set_hold(t[0], True)
    b.step(2)
    b.remove(t[2])
    t3 = b.add(cs[3])
    b.step(1)
    for x, y in ((s[0], t[0]), (s[1], t[1]), (s3, t3)):
        assert np.array_equal(a.get_flow(x), b.get_flow(y))
    a.close()
    b.close()
    bad = copy_arrays(cs[1].arrays)["flow"]
    bad[7, 5] = np.nan
    c = runtime.Batch(ctx, 0)
    c.add(cs[0])
    c.add(cs[1], flow=bad)
    c.step_async(1)
    c.step_async(1)
    with pytest.raises(abi.CfdError) as e:
        c.sync()
    assert e.value.status == abi.ENONFINITE
    c.close()


def test_empty_batch_steps_and_info(ctx):
    """Steps of a batch with no instance (or only held ones) do nothing and
    succeed, in both forms and both step calls."""
    from cfd_gb300 import runtime
    for prec in (0, 1):
        b = runtime.Batch(ctx, prec)
        b.step(2)
        b.step_async(1)
        b.sync()
        assert b.info().n_active == 0 and b.info().nodes_total == 0
        s = b.add(mix_cases()[0])
        flow = b.get_flow(s)
        b.set_hold(s, True)
        b.step(1)
        assert np.array_equal(b.get_flow(s), flow)
        b.remove(s)
        b.step(1)
        b.close()


@pytest.mark.parametrize("tile", [32, 64, 256])
def test_every_tile_size_gives_the_same_bits(ctx, tile):
    """The batched kernel takes phase-A items from a shared counter, in an
    order that depends on timing; every item writes only its own faces, so
    the results do not depend on the tile size or on which block took what."""
    from cfd_gb300 import runtime
    cs = mix_cases()
    out = []
    for t in (128, tile):
        b = runtime.Batch(ctx, 1)
        b.set_tiling(t, 0, use_graph=False)
        ss = [b.add(c) for c in cs]
        b.step(3)
        out.append([b.get_flow(s_) for s_ in ss])
        b.close()
    for a, c in zip(*out):
        assert np.array_equal(a, c)


def test_tuning_and_graph_do_not_change_results(ctx):
    from cfd_gb300 import runtime
    cs = mix_cases()
    ref = runtime.Batch(ctx, 1)
    ref.set_tiling(128, 0, use_graph=False)
    rs = [ref.add(c) for c in cs]
    ref.step(2)
    tuned = runtime.Batch(ctx, 1)
    ts = [tuned.add(c) for c in cs]
    tuned.tune(1)                        # trials run on the live batch, state restored
    tuned.step(2)
    assert tuned.info().tile_nodes in (32, 64, 128, 256)
    for r, t in zip(rs, ts):
        assert np.array_equal(ref.get_flow(r), tuned.get_flow(t))
    ref.close()
    tuned.close()


def test_admission_budget_and_unsupported_geometry(ctx):
    from cfd_gb300 import abi, cases, runtime
    c = cases.isentropic_vortex(n=10)
    need = runtime.Batch.instance_bytes(0, c.sd_node)
    b = runtime.Batch(ctx, 0, capacity_bytes=int(1.5 * need))
    b.add(c)
    with pytest.raises(abi.CfdError) as e:
        b.add(c)
    assert e.value.status == abi.ENOMEM
    with pytest.raises(abi.CfdError) as e:
        b.add(cases.ghost_box(shape=(6, 6, 6)))
    assert e.value.status == abi.EUNSUPPORTED
    b.close()


def test_nonfinite_instance_is_isolated(ctx):
    """A poisoned instance reports CFD_ENONFINITE for its own slot; the other
    instances of the batch advance exactly as they would alone."""
    from cfd_gb300 import abi, runtime
    cs = mix_cases()
    bad = copy_arrays(cs[1].arrays)["flow"]
    bad[7, 5] = np.nan
    b = runtime.Batch(ctx, 0)
    s_good = b.add(cs[0])
    s_bad = b.add(cs[1], flow=bad)
    with pytest.raises(abi.CfdError) as e:
        b.step(1)
    assert e.value.status == abi.ENONFINITE
    assert b.slot_status(s_bad) == abi.ENONFINITE
    assert b.slot_status(s_good) == abi.OK
    alone = runtime.Batch(ctx, 0)
    a = alone.add(cs[0])
    alone.step(1)
    assert np.array_equal(alone.get_flow(a), b.get_flow(s_good))
    b.close()
    alone.close()


@pytest.mark.parametrize("precision", [1, 2])
def test_face_tiles_equal_node_tiles_bitwise(ctx, precision):
    """Phase A on shared-memory face tiles (CFD_BATCH_FACE_TILES) evaluates
    the same arithmetic as the 1-D tiles: the same bits."""
    from cfd_gb300 import abi, runtime
    cs = mix_cases()
    out = []
    for tiling in (128, abi.BATCH_FACE_TILES):
        b = runtime.Batch(ctx, precision)
        slots = [b.add(c) for c in cs]
        b.set_tiling(tiling)
        assert b.info().face_tiles == (tiling == abi.BATCH_FACE_TILES)
        b.step(3)
        out.append([b.get_u0(s) for s in slots])
        b.close()
    for a, t in zip(*out):
        assert np.array_equal(a, t)


def test_face_tiles_refused_for_fp64(ctx):
    from cfd_gb300 import abi, runtime
    b = runtime.Batch(ctx, 0)
    with pytest.raises(abi.CfdError) as e:
        b.set_tiling(abi.BATCH_FACE_TILES)
    assert e.value.status == abi.EINVAL
    b.close()
