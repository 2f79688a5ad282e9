"""Continuous-batching server (cpgpu_server_*) and world cloning, on a GB300.

The serving contract: requests that arrive while others run are admitted as
memory frees up and stepped together with them, and each request's result is
the same alone and in the mix.  The tolerance is exact equality: a batch steps
each world exactly as it steps alone, and re-forming the batch moves the state
through the host without rounding (FP32 values stored as FP64 and back).
"""
import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu

KEYS = ("com", "quat", "vel", "ang_vel")


def _templates(seed, n, nmin=8, nmax=60):
    rng = np.random.default_rng(seed)
    pool = scenes.HullPool(seed, size=8)
    out = []
    for _ in range(n):
        w = cg.world()
        scenes.apply(scenes.batched_world(rng, pool, nmin, nmax), w)
        out.append(w)
    return out


def test_clone_steps_like_original():
    t = _templates(3, 1)[0]
    t.step(20)
    c = cg.clone(t)
    t.step(30)
    c.step(30)
    a, b = t.state(), c.state()
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k


def test_served_results_equal_alone():
    temps = _templates(7, 4)
    ks = [25, 40, 17, 33]
    alone = []
    for t, k in zip(temps, ks):
        w = cg.clone(t)
        w.step(k)
        alone.append(w.state())
    srv = cg.Server(budget_bytes=8 << 30, epoch_steps=4)
    reqs = [cg.clone(t) for t in temps]
    toks = [srv.submit(reqs[0], ks[0])]
    srv.advance(7)                              # request 0 runs alone
    toks.append(srv.submit(reqs[1], ks[1]))     # arrives mid-flight
    toks.append(srv.submit(reqs[2], ks[2]))
    srv.advance(9)
    toks.append(srv.submit(reqs[3], ks[3]))
    done = set(srv.poll())
    for _ in range(200):
        running, waiting = srv.advance(50)
        done |= set(srv.poll())
        if running == 0 and waiting == 0:
            break
    assert done == set(toks)
    st = srv.stats()
    assert st["reforms"] >= 3
    # every request advanced exactly its own step count (the plate is fixed)
    assert st["body_steps"] == sum(k * (r.state()["com"].shape[0] - 1) for r, k in zip(reqs, ks))
    for i, (r, a) in enumerate(zip(reqs, alone)):
        s = r.state()
        for k in KEYS:
            assert np.array_equal(s[k], a[k]), (i, k)


def test_budget_admission_queues_requests():
    """A budget that fits one request at a time: the others wait, are admitted
    as earlier ones complete, and still produce their stand-alone results."""
    temps = _templates(11, 3, 20, 40)
    ks = [12, 9, 15]
    alone = []
    for t, k in zip(temps, ks):
        w = cg.clone(t)
        w.step(k)
        alone.append(w.state())
    srv = cg.Server(budget_bytes=1, epoch_steps=2)   # always admits one at a time
    reqs = [cg.clone(t) for t in temps]
    for r, k in zip(reqs, ks):
        srv.submit(r, k)
    running, waiting = srv.advance(1)
    assert running == 1 and waiting == 2
    for _ in range(100):
        running, waiting = srv.advance(20)
        if running == 0 and waiting == 0:
            break
    assert len(srv.poll()) == 3
    for i, (r, a) in enumerate(zip(reqs, alone)):
        s = r.state()
        for k in KEYS:
            assert np.array_equal(s[k], a[k]), (i, k)


def test_size_lanes_exact_and_small_first():
    """Requests of three world sizes (one per server lane: < 128, < 512 and
    >= 512 dynamic bodies) submitted together with the same step count: each
    result equals its stand-alone run bit for bit, and the small request is
    done no later than the large one (its lane steps at its own pace)."""
    rng = np.random.default_rng(31)
    pool = scenes.HullPool(5, size=8)
    sizes = [(30, 60), (200, 300), (560, 700)]
    temps = []
    for lo, hi in sizes:
        sc = None
        while sc is None or not sc.name.startswith("pyramid"):
            sc = scenes.batched_world(rng, pool, lo, hi)
        w = cg.world()
        scenes.apply(sc, w)
        temps.append(w)
    k = 40
    alone = []
    for t in temps:
        w = cg.clone(t)
        w.step(k)
        alone.append(w.state())
    srv = cg.Server(budget_bytes=8 << 30, epoch_steps=4)
    reqs = [cg.clone(t) for t in temps]
    toks = [srv.submit(r, k) for r in reqs]
    order = []
    for _ in range(1000):
        running, waiting = srv.advance(5)
        order += srv.poll()
        if running == 0 and waiting == 0:
            break
    assert sorted(order) == sorted(toks)
    assert order.index(toks[0]) <= order.index(toks[2])
    for i, (r, a) in enumerate(zip(reqs, alone)):
        s = r.state()
        for key in KEYS:
            assert np.array_equal(s[key], a[key]), (i, key)
