"""The batch schedule and its autotuner (cpgpu_batch_create_tuned), on a GB300.

A schedule (parts stepped concurrently, solver-chain workers per SM, the
island size that takes the warp-per-island solver) must never change a
result: every schedule steps every world exactly as it does alone.  The
autotuner times candidate schedules on trial steps, restores the state after
each, and keeps the fastest; the batch it returns starts from the worlds'
state, and a later plain batch with the same world-size histogram reuses the
choice.
"""
import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu


def _worlds(n, seed=3):
    rng = np.random.default_rng(seed)
    pool = scenes.HullPool(seed, size=32)
    return [scenes.batched_world(rng, pool, 8, 200) for _ in range(n)]


def _build(scs):
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    return ws


@pytest.mark.parametrize("stagger", [1, 0])
def test_schedules_give_identical_results(monkeypatch, stagger):
    """Parts stepped with staggered first halves (the default) or fully
    concurrently, graduated shares, per-part chain workers: the same bits."""
    scs = _worlds(600)
    ref = None
    monkeypatch.setenv("CPGPU_BATCH_STAGGER", str(stagger))
    for parts, share, second, per_sm, mid in ((1, 100, 0, 0, -1), (2, 20, 0, 2, -1), (3, 30, 0, 1, -1),
                                              (3, 5, 20, 3, 0), (4, 3, 12, 2, 4)):
        monkeypatch.setenv("CPGPU_BATCH_PARTS", str(parts))
        monkeypatch.setenv("CPGPU_BATCH_FIRST_SHARE", str(share))
        monkeypatch.setenv("CPGPU_BATCH_SECOND_SHARE", str(second))
        monkeypatch.setenv("CPGPU_PGS_REST_PER_SM", str(per_sm))
        monkeypatch.setenv("CPGPU_PGS_MID_PER_SM", str(mid))
        b = cg.Batch(_build(scs))
        sch = b.schedule()
        assert sch["parts"] == parts and sch["second_share_pct"] == (second if parts > 2 else 0)
        b.step(25)
        st = [b.state(i) for i in range(0, 600, 37)]
        b.close()
        if ref is None:
            ref = st
        else:
            for x, y in zip(st, ref):
                for k in x:
                    assert np.array_equal(x[k], y[k]), (parts, k)


def test_autotuned_batch_starts_from_the_worlds_and_matches_the_default():
    scs = _worlds(600, seed=4)
    plain = cg.Batch(_build(scs))
    tuned = cg.Batch(_build(scs))
    plain.step(15)
    tuned.step(15)
    tuned.tune(2)   # from the state after 15 steps; the trial steps are undone
    sch = tuned.schedule()
    assert sch["tuned"] and sch["tuned_ms_per_step"] > 0 and sch["default_ms_per_step"] > 0
    assert sch["tuned_ms_per_step"] <= sch["default_ms_per_step"] * 1.0001
    assert sch["big_island_rows"] in (32, 48, 96)
    plain.step(20)
    tuned.step(20)
    for i in range(0, 600, 23):
        a, b = plain.state(i), tuned.state(i)
        for k in a:
            assert np.array_equal(a[k], b[k]), k
    # a later plain batch with the same histogram takes the cached choice
    again = cg.Batch(_build(scs))
    s2 = again.schedule()
    assert s2["tuned"] and s2["parts"] == sch["parts"] and s2["big_island_rows"] == sch["big_island_rows"]


def test_tuning_leaves_the_worlds_alone_and_refuses_changed_ones():
    scs = _worlds(40, seed=5)
    ws = _build(scs)
    before = [w.state() for w in ws]
    b = cg.Batch(ws)
    b.step(10)
    b.tune(1)
    for w, s0 in zip(ws, before):         # the worlds' own state is untouched
        s1 = w.state()
        for k in s0:
            assert np.array_equal(s0[k], s1[k]), k
    ws[3].set_velocity(ws[3].n_bodies, (0.0, 1.0, 0.0))   # a world changed after the batch was made
    with pytest.raises(cg.CPGPUError):
        b.tune(1)
    b.close()
    # worlds dropped while a batch made from them lives stay valid for it
    b2 = cg.Batch(_build(scs))
    b2.step(5)
    b2.tune(1)
    b2.step(2)
    b2.close()


def test_timeline_marks_are_ordered_per_part(monkeypatch):
    """cpgpu_batch_timeline: per part, the stage marks of a step in order,
    and the timed steps advance the batch as plain steps do."""
    monkeypatch.setenv("CPGPU_BATCH_PARTS", "3")
    monkeypatch.setenv("CPGPU_BATCH_FIRST_SHARE", "10")
    monkeypatch.setenv("CPGPU_BATCH_SECOND_SHARE", "30")
    b = cg.Batch(_build(_worlds(300, seed=6)))
    b.step(10)
    tl = b.timeline(3)
    assert tl.shape == (3, 10)   # 7 + 3 marks of one substep
    assert np.all(np.diff(tl, axis=1) >= -1e-3)
    # the timed steps advanced the batch like plain steps
    ref = cg.Batch(_build(_worlds(300, seed=6)))
    ref.step(13)
    for i in range(0, 300, 17):
        a, c = b.state(i), ref.state(i)
        for k in a:
            assert np.array_equal(a[k], c[k]), k
