"""Distance, weld, slider and sliding-hinge joints, cone and twist limits,
motors, pistons and springs on the device, against the CPU restatement (pinned bit for bit to the
reference on the same scenes), on a GB300.

Per-step parity: the device's bodies, contacts and joint state (impulses,
tangent bases, twist angles and limit flags) after k steps are imported into
the restatement, both advance one step (4 substeps) and the results are
compared with the FP32-vs-FP64 tolerances of the ball-socket/hinge chains.
Trajectories: both step the scene from scratch for 40 steps (swinging and
sliding, before the first ground contacts) and agree within 1e-3 m.

The limit scenes here use a small correction strength (60): the reference's
limit rows correct with the raw strength times the error, unscaled by the
step, so at the default 15,000 a limit passed by a few degrees throws the
chain (the restatement's pinning tests keep the default); and a limit
reached exactly at a step boundary activates a step earlier or later in FP32
than in FP64, which the default strength turns into metres within a step.
"""
import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu

SCENES = {
    "distance": lambda: scenes.distance_chain(False),
    "distance_ball": lambda: scenes.distance_chain(True),
    "weld": lambda: scenes.weld_cantilever(False),
    "weld_hinge": lambda: scenes.weld_cantilever(True),
    "slider": lambda: scenes.slider_chain(("slider",) * 4),
    "sliding_hinge": lambda: scenes.slider_chain(("sliding_hinge",) * 4),
    "slider_mixed": lambda: scenes.slider_chain(("slider", "hinge", "sliding_hinge", "slider")),
    "spring": lambda: scenes.spring_chain(False),
    "spring_ball": lambda: scenes.spring_chain(True),
    "cone": lambda: scenes.cone_chain(1, rot_strength=60.0),
    "cone_no_block_solve": lambda: scenes.cone_chain(0, rot_strength=60.0),
    "twist": lambda: scenes.twist_chain(rot_strength=60.0),
    "motor_torque": lambda: scenes.motor_chain(1, False),
    "motor_velocity": lambda: scenes.motor_chain(2, True),
    "motor_position": lambda: scenes.motor_chain(3, True),
    "piston_force": lambda: scenes.piston_chain(1, True),
    "piston_velocity": lambda: scenes.piston_chain(2, True),
    "piston_position": lambda: scenes.piston_chain(3, False),
}


def _scene(name):
    return SCENES[name]()


def _step_both(sc, k, oracle_mod):
    g = cg.world()
    scenes.apply(sc, g)
    g.step(k)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    if k > 0:
        p.set_state(**g.state())
        p.set_contacts(g.contacts())
        p.set_joint_state(g.joint_state())
    g.step(1)
    p.step(1)
    return g, p


def _stick_slip_bodies(cg_, cp_):
    """Bodies with a contact that slips (static_ready false: its friction was
    clamped to the cone in the last pass) in either engine.  Such a contact
    switches between the static and the kinetic coefficient from substep to
    substep; FP32 and FP64 can take the switch in different substeps."""
    out = set()
    for c in (cg_, cp_):
        for i in range(len(c["b1"])):
            if not int(c["static_ready"][i]):
                out.update((int(c["b1"][i]), int(c["b2"][i])))
    return out


def test_every_joint_kind_is_accepted_on_the_device():
    for name in SCENES:
        w = cg.world()
        scenes.apply(_scene(name), w)   # raises on CPGPU_ERR_UNSUPPORTED
        w.step(1)


@pytest.mark.parametrize("k", [0, 40, 120])
@pytest.mark.parametrize("name", sorted(SCENES))
def test_joint_kind_single_step_parity(oracle_mod, name, k):
    sc = _scene(name)
    g, p = _step_both(sc, k, oracle_mod)
    assert np.array_equal(g.pairs(), p.pairs())
    sg, sp = g.state(), p.state()
    dv = np.linalg.norm(sg["vel"] - sp["vel"], axis=1)
    dw = np.linalg.norm(sg["ang_vel"] - sp["ang_vel"], axis=1)
    vm = np.linalg.norm(sp["vel"], axis=1)
    wm = np.linalg.norm(sp["ang_vel"], axis=1)
    dx = np.abs(sg["com"] - sp["com"]).max()
    stats = f"dv max {dv.max():.2e} dw max {dw.max():.2e} dx {dx:.2e}"
    # a contact at the edge of its friction cone (the stick/slip switch
    # between the static and kinetic coefficients, taken in different
    # substeps in FP32 and FP64) moves its bodies by up to (mu_s - mu_k) N / m;
    # bodies with a slipping contact get a looser bound
    slip = _stick_slip_bodies(g.contacts(), p.contacts())
    tight = np.array([i + 1 not in slip for i in range(len(dv))])
    # FP32 rows through 4 substeps of 10 velocity sweeps and the block solve
    assert np.all((dv <= 2e-3 + 2e-3 * vm) | ~tight), stats   # m/s
    assert np.all((dw <= 5e-3 + 2e-3 * wm) | ~tight), stats   # rad/s
    assert np.all(dv <= 2e-2 + 2e-3 * vm), stats
    assert dx <= 1e-4, stats                        # m
    jg, jp = g.joint_state(), p.joint_state()
    if len(jp["impulse"]):
        scale = np.abs(jp["impulse"]).max() + 1.0
        assert np.abs(jg["impulse"] - jp["impulse"]).max() <= 1e-2 * scale, stats
        # limits and pistons: the same reached flags (0 / 1); motors: the
        # relative angular velocity; twist and motor angles and slide
        # positions within FP32 rounding
        assert np.allclose(jg["aux"][:, 1], jp["aux"][:, 1], rtol=1e-3, atol=1e-4), (jg["aux"], jp["aux"])
        assert np.abs(jg["aux"][:, 0] - jp["aux"][:, 0]).max() <= 1e-4


@pytest.mark.parametrize("name", sorted(SCENES))
def test_joint_kind_trajectory(oracle_mod, name):
    sc = _scene(name)
    g = cg.world()
    scenes.apply(sc, g)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    for k in range(4):
        g.step(10)
        p.step(10)
        err = np.abs(g.state()["com"] - p.state()["com"]).max()
        assert err <= 1e-3, (10 * (k + 1), err)


def test_cone_and_twist_limits_hold_on_the_device():
    """The limits engage on the device: with them the swung chain's joints stay
    within a few degrees of their cone (25 degrees), without them they swing
    past it."""
    def max_angle(sc, steps=240):
        w = cg.world()
        scenes.apply(sc, w)
        worst = 0.0
        for _ in range(steps // 10):
            w.step(10)
            q = w.state()["quat"]
            for i in range(2, len(q)):
                def down(qq):
                    r, x, y, z = qq
                    # body's -y axis in world space
                    return -np.array([2 * x * y - 2 * r * z, r * r - x * x + y * y - z * z, 2 * y * z + 2 * r * x])
                a, b = down(q[i - 1]) if i > 2 else np.array([0.0, -1.0, 0.0]), down(q[i])
                worst = max(worst, float(np.degrees(np.arccos(np.clip(np.dot(a, b), -1, 1)))))
        return worst
    limited = max_angle(scenes.cone_chain(1))
    sc = scenes.cone_chain(1)
    sc.ops = [op for op in sc.ops if op[0] != "cone_limit"]
    free = max_angle(sc)
    assert limited <= 25.0 + 5.0, limited
    assert free > 35.0, free


def test_springs_do_not_stop_collisions_joints_do():
    """A pair joined only by a spring still collides; the same pair joined by a
    weld does not (addSpring adds no collision exception)."""
    m = scenes.PILE_MATERIAL
    for joint, expect_contacts in (("spring", True), ("weld", False)):
        sc = scenes.Scene("overlap", scenes.JOINT_PARAMS)
        a = sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, m, scenes.DYNAMIC)
        b = sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, m, scenes.DYNAMIC, (0.9, 0.0, 0.0))
        if joint == "spring":
            sc.spring(a, b, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0, 10.0)
        else:
            sc.weld(a, b, (0.45, 0.0, 0.0), (-0.45, 0.0, 0.0))
        w = cg.world()
        scenes.apply(sc, w)
        w.step(1)
        assert len(w.pairs()) == 1
        assert (len(w.contacts()["b1"]) > 0) == expect_contacts, joint


def test_joint_kinds_batched_equal_alone():
    scs = [_scene(n) for n in sorted(SCENES)]
    singles = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        w.step(30)
        singles.append(w.state())
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    b = cg.Batch(ws)
    b.step(30)
    for i, st in enumerate(singles):
        got = b.state(i)
        for k in st:
            assert np.array_equal(got[k], st[k]), (sorted(SCENES)[i], k)


def test_motor_and_piston_positions_follow_the_restatement(oracle_mod):
    """getMotorAngularPosition / getPistonPosition on the device match the
    restatement's along 60 steps from the same scene, and the powered joints
    reach their targets."""
    for sc, getter in ((scenes.motor_chain(3, True), "motor_position"), (scenes.piston_chain(3, False), "piston_position")):
        g = cg.world()
        scenes.apply(sc, g)
        p = oracle_mod.port_world()
        scenes.apply(sc, p)
        ids_g, ids_p = g.constraint_ids[1::2], p.constraint_ids[1::2]
        assert ids_g == ids_p                      # the reference's constraint-id numbering on both
        for _ in range(6):
            g.step(10)
            p.step(10)
            pg = np.array([getattr(g, getter)(c) for c in ids_g])
            pp = np.array([getattr(p, getter)(c) for c in ids_p])
            assert np.abs(pg - pp).max() <= 2e-3, (sc.name, pg, pp)
