"""Sleeping on the device against the CPU restatement (pinned bit for bit to
the reference on the same scene), on a GB300.

Three box stacks and a ball settle on the plate with sleeping enabled: their
islands fall asleep (zero velocity, no solve, no integration), a velocity set
on a sleeping box wakes its stack at step 150, the ball dropped onto a stack
at step 300 wakes it through the contact, and the boxes fall asleep again.
The device follows the restatement's sleep events step for step (the set of
sleeping bodies, RigidBody::getAsleep) except where a sleep test sits at its
threshold, and its settled positions agree within
FP32 tolerance.
"""
import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu


def _run(w, ball, x, steps=500, record=None):
    asleep = []
    for s in range(steps):
        if s == 150:
            w.set_velocity(3, (0.5, 0.0, 0.0))
        if s == 300:
            w.set_position(ball, (x, 4.5, 0.1))
            w.set_velocity(ball, (0.0, -3.0, 0.0))
        w.step(1)
        asleep.append(tuple(int(x) for x in w.asleep()))
        if record is not None and s in record:
            record[s] = w.state()["com"].copy()
    return asleep


@pytest.mark.parametrize("seed", [0, 2])
def test_sleep_events_follow_the_restatement(oracle_mod, seed):
    sc, ball, x = scenes.sleep_stacks(seed)
    g = cg.world()
    scenes.apply(sc, g)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    rg, rp = {149: None, 299: None, 499: None}, {149: None, 299: None, 499: None}
    ag = _run(g, ball, x, record=rg)
    ap = _run(p, ball, x, record=rp)
    n = len(ag[0])
    # every dynamic body (all but the plate) asleep before each waking action
    assert sum(ag[149]) == n - 1 and sum(ag[299]) == n - 1, (sum(ag[149]), sum(ag[299]))
    # the actions wake bodies on the device too
    assert sum(ag[151]) < n - 1 and min(sum(a) for a in ag[300:330]) < n - 3
    # the same sleeping set as the restatement on all but a few steps
    differ = [s for s in range(500) if ag[s] != ap[s]]
    assert len(differ) <= 10, differ
    # settled stacks agree in position
    for s in (149, 299):
        assert np.abs(rg[s] - rp[s]).max() <= 2e-3, (s, np.abs(rg[s] - rp[s]).max())


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
