"""Sleeping on the device against the CPU restatement (pinned bit for bit to
the reference on the same scene), on a GB300.

Three box stacks and a ball settle on the plate with sleeping enabled: their
islands fall asleep (zero velocity, no solve, no integration), a velocity set
on a sleeping box wakes its stack at step 150, the ball dropped onto a stack
at step 300 wakes it through the contact, and the boxes fall asleep again.
The device's sleeping sets (RigidBody::getAsleep) and settled positions
differ from the restatement's no more than those of an FP32-state control
(the restatement with the state rounded to FP32 after every step) do.
"""
import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu


def _r32(st):
    return {k: np.asarray(v, np.float32).astype(np.float64) for k, v in st.items()}


def _run(w, ball, x, steps=500, record=None, round32=False):
    asleep = []
    for s in range(steps):
        if s == 150:
            w.set_velocity(3, (0.5, 0.0, 0.0))
        if s == 300:
            w.set_position(ball, (x, 4.5, 0.1))
            w.set_velocity(ball, (0.0, -3.0, 0.0))
        w.step(1)
        if round32:
            w.set_state(**_r32(w.state()))
        asleep.append(tuple(int(x) for x in w.asleep()))
        if record is not None and s in record:
            record[s] = w.state()["com"].copy()
    return asleep


@pytest.mark.parametrize("seed", [0, 2])
def test_sleep_events_follow_the_restatement(oracle_mod, seed):
    """The device's sleeping sets and settled positions differ from the FP64
    restatement's no more than an FP32-state control's do (the restatement
    with every body's state rounded to FP32 after each step): settling stacks
    cross the sleep thresholds a few steps apart, and a ball dropped on a
    stack settles differently, with or without FP32 arithmetic."""
    sc, ball, x = scenes.sleep_stacks(seed)
    g = cg.world()
    scenes.apply(sc, g)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    q = oracle_mod.port_world()
    scenes.apply(sc, q)
    keys = (149, 299)
    rg, rp, rq = ({k: None for k in keys} for _ in range(3))
    ag = _run(g, ball, x, record=rg)
    ap = _run(p, ball, x, record=rp)
    aq = _run(q, ball, x, record=rq, round32=True)
    n = len(ag[0])
    # every dynamic body (all but the plate) asleep before each waking action
    assert sum(ag[149]) == n - 1 and sum(ag[299]) == n - 1, (sum(ag[149]), sum(ag[299]))
    # the actions wake bodies on the device too
    assert sum(ag[151]) < n - 1 and min(sum(a) for a in ag[300:330]) < n - 3
    # sleeping sets: the device differs from the restatement on no more steps
    # than the FP32-state control does (a few steps at each threshold crossing)
    differ = [s for s in range(500) if ag[s] != ap[s]]
    differ_ctl = [s for s in range(500) if aq[s] != ap[s]]
    assert len(differ) <= max(10, 2 * len(differ_ctl)), (differ, differ_ctl)
    # the settling before the drop: the same events within a few steps
    assert len([s for s in differ if s < 300]) <= 10, differ
    # settled stacks agree in position like the control (one FP32 realisation
    # each: within 3x the control's distance)
    for s in keys:
        dev, ctl = np.abs(rg[s] - rp[s]).max(), np.abs(rq[s] - rp[s]).max()
        assert dev <= max(2e-3, 3 * ctl), (s, dev, ctl)


def test_sleeping_worlds_batched_equal_alone():
    scs = [scenes.sleep_stacks(seed)[0] for seed in (0, 1, 2, 3)]
    alone = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        w.step(160)
        alone.append(w.state())
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    b = cg.Batch(ws)
    b.step(160)
    for i, st in enumerate(alone):
        got = b.state(i)
        for k in st:
            assert np.array_equal(got[k], st[k]), (i, k)


def test_box_vs_ground_with_the_reference_defaults():
    """CollisionTests.h:77-165 (Box vs Ground) with sleeping enabled, as the
    reference's defaults have it: the box comes to rest asleep (exactly zero
    velocity) at y = 0.5 +- 0.1 with vertical contact normals."""
    w = cg.world()
    w.set_params(step_time=1.0 / 60.0, sleeping=True)
    w.add_box((-50.0, -0.5, -50.0), 100.0, 0.5, 100.0, None, scenes.FIXED)
    box = w.add_box((0.0, 5.0, 0.0), 1.0, 1.0, 1.0, None, scenes.DYNAMIC)
    w.step(300)
    st, c = w.state(), w.contacts()
    assert np.all(st["vel"][box - 1] == 0) and np.all(st["ang_vel"][box - 1] == 0)
    assert abs(st["com"][box - 1, 1] - 0.5) < 0.1
    assert len(c["b1"]) > 0 and (np.abs(c["n_local_b1"][:, 1]) >= 0.9999).all()
