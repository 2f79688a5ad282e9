"""The oracle is pinned: the CPU restatement of the contact path (oracle/cport)
reproduces the reference engine (compiled from its own sources) bit for bit,
and the reference's own scenario checks hold for both.  CPU only."""
import ctypes

import numpy as np
import pytest

from constraintphysics_gb300 import scenes


def _states_equal(a, b):
    return all(np.array_equal(a[k], b[k]) for k in a)


def test_restatement_bitwise_on_hull_pile(oracle_mod):
    # 27 random hulls dropped on the plate: impacts, stacking, contact churn
    r, p = oracle_mod.twin_worlds(scenes.hull_drop(seed=1, n_side=3))
    for s in range(160):
        r.step(1)
        p.step(1)
        if s % 20 == 19:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
            assert np.array_equal(r.pairs(), p.pairs()), f"pair set differs at step {s}"
    cr, cp = r.contacts(), p.contacts()
    assert len(cr["b1"]) > 40
    for k in ("b1", "b2", "magic_b", "live", "memory_life", "normal_impulse", "friction_impulse", "pen_depth"):
        assert np.array_equal(cr[k], cp[k]), k


def test_restatement_bitwise_on_batched_worlds(oracle_mod):
    rng = np.random.default_rng(11)
    pool = scenes.HullPool(3, size=8)
    for _ in range(3):
        sc = scenes.batched_world(rng, pool, nmin=10, nmax=60)
        r, p = oracle_mod.twin_worlds(sc)
        r.step(90)
        p.step(90)
        assert _states_equal(r.state(), p.state()), sc.name
        assert len(r.contacts()["b1"]) == len(p.contacts()["b1"])


def test_restatement_bitwise_on_mixed_drop(oracle_mod):
    # boxes, spheres, cylinders and hulls: every primitive pair kind occurs
    sc = scenes.mixed_drop(seed=2, n_side=4, n_layers=3)
    kinds = [op[0] for op in sc.ops if op[0] in ("hull", "box", "sphere", "cylinder")]
    r, p = oracle_mod.twin_worlds(sc)
    seen = set()
    for s in range(200):
        r.step(1)
        p.step(1)
        c = r.contacts()
        for a, b in zip(c["b1"].tolist(), c["b2"].tolist()):
            seen.add(tuple(sorted((kinds[a - 1].replace("box", "hull"), kinds[b - 1].replace("box", "hull")))))
        if s % 25 == 24:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
            assert np.array_equal(r.pairs(), p.pairs()), f"pair set differs at step {s}"
    cr, cp = r.contacts(), p.contacts()
    for k in ("b1", "b2", "magic_b", "live", "memory_life", "normal_impulse", "friction_impulse", "pen_depth"):
        assert np.array_equal(cr[k], cp[k]), k
    assert {("cylinder", "hull"), ("hull", "sphere"), ("cylinder", "cylinder"), ("cylinder", "sphere"),
            ("sphere", "sphere")} <= seen, seen


def test_mass_properties_agree(oracle_mod):
    sc = scenes.hull_drop(seed=4, n_side=2)
    r, p = oracle_mod.ref_world(), oracle_mod.port_world()
    scenes.apply(sc, r)
    scenes.apply(sc, p)
    get_r = oracle_mod.ref_abi()._lib.cpref_get_mass_properties
    get_p = oracle_mod.port_abi()._lib.cport_get_mass_properties
    for f in (get_r, get_p):
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    for bid in range(1, sc.n_bodies + 1):
        out = []
        for f, w in ((get_r, r), (get_p, p)):
            m, c, t = np.zeros(1), np.zeros(3), np.zeros(9)
            assert f(w.h, bid, m.ctypes.data, c.ctypes.data, t.ctypes.data) == 0
            out.append((m, c, t))
        (mr, cr, tr), (mp, cp, tp) = out
        assert abs(mr[0] - mp[0]) <= 1e-12 * mr[0]
        assert np.abs(cr - cp).max() <= 1e-12 * (1 + np.abs(cr).max())
        assert np.abs(tr - tp).max() <= 1e-10 * np.abs(tr).max()


def _box_vs_ground(w, sleeping):
    w.set_params(step_time=1.0 / 60.0, sleeping=sleeping)
    w.add_box((-50.0, -0.5, -50.0), 100.0, 0.5, 100.0, None, scenes.FIXED)
    box = w.add_box((0.0, 5.0, 0.0), 1.0, 1.0, 1.0, None, scenes.DYNAMIC)
    saw_contact = False
    for _ in range(300):
        w.step(1)
        c = w.contacts()
        # contacts re-detected this step had their life reset to 6 and
        # decremented once at the end of the step
        live = c["memory_life"] == 5
        if live.any():
            saw_contact = True
            # ground is body 1 (fixed, identity orientation): local normal = world normal
            assert (np.abs(c["n_local_b1"][live][:, 1]) >= 0.9999).all()
    st = w.state()
    return saw_contact, st["com"][box - 1], np.linalg.norm(st["vel"][box - 1]), np.linalg.norm(st["ang_vel"][box - 1])


def test_box_vs_ground_reference_defaults(oracle_mod):
    """Demo/src/Demos/Tests/CollisionTests.h:77-165 (Box vs Ground), headless,
    on the reference engine with its defaults (sleeping on): a 1 m box dropped
    from y=5 on a fixed 100 x 0.5 x 100 plate at 60 Hz rests with |v|, |w| <
    1e-5 at y = 0.5 +- 0.1 with vertical manifold normals."""
    saw, com, v, w = _box_vs_ground(oracle_mod.ref_world(), sleeping=True)
    assert saw and v < 1e-5 and w < 1e-5 and abs(com[1] - 0.5) < 0.1


@pytest.mark.parametrize("which", ["ref", "port"])
def test_box_vs_ground_sleeping_disabled(oracle_mod, which):
    """Same scenario with sleeping disabled (the configuration the device path
    implements): the box still rests at y = 0.5 +- 0.1 with vertical normals;
    without sleep the solver leaves ~5e-4 m/s of residual motion, so the
    velocity bound is 1e-3."""
    w = oracle_mod.ref_world() if which == "ref" else oracle_mod.port_world()
    saw, com, v, av = _box_vs_ground(w, sleeping=False)
    assert saw and v < 1e-3 and av < 1e-3 and abs(com[1] - 0.5) < 0.1


def test_tree_pair_set_equals_brute_force(oracle_mod):
    """The reference's AABB-tree candidate pairs are exactly the pairs whose
    AABBs overlap (inclusive compare) -- the brute-force check of
    PhysicsEngine.cpp:117-154, done on the pair set instead of its size."""
    w = oracle_mod.ref_world()
    scenes.apply(scenes.hull_drop(seed=2, n_side=4), w)
    checked = 0
    for s in range(120):
        aabb = w.aabbs()
        w.step(1)
        lo, hi = aabb[:, :3], aabb[:, 3:]
        ov = ~((hi[:, None, :] < lo[None, :, :]) | (lo[:, None, :] > hi[None, :, :])).any(axis=2)
        i, j = np.nonzero(np.triu(ov, 1))
        brute = np.stack([i + 1, j + 1], axis=1).astype(np.uint32)
        assert np.array_equal(brute, w.pairs()), f"step {s}"
        checked += len(brute)
    assert checked > 1000


def test_golden_fixture(oracle_mod):
    """The restatement reproduces the committed reference outputs
    (tests/golden/make_golden.py, generated from the reference engine)."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "hull_drop_3_seed1.npz")
    g = np.load(path)
    sc = scenes.hull_drop(seed=1, n_side=3)
    r, p = oracle_mod.twin_worlds(sc)
    p.step(int(g["steps"]))
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.allclose(st[k], g[k], rtol=0, atol=1e-9), k
    c = p.contacts()
    assert np.array_equal(c["magic_b"], g["magic_b"])
    assert np.allclose(c["normal_impulse"], g["normal_impulse"], rtol=0, atol=1e-9)


def test_golden_fixture_mixed(oracle_mod):
    """Spheres, cylinders, boxes and hulls: the restatement, started from the
    reference's mass properties stored in the fixture, reproduces the
    reference's state and contacts after 150 steps (no reference library
    needed)."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "mixed_drop_4x4x2_seed1.npz")
    g = np.load(path)
    sc = scenes.mixed_drop(seed=1, n_side=4, n_layers=2)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    put = oracle_mod.port_abi()._lib.cport_body_set_mass_properties
    put.restype = ctypes.c_int
    put.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    for i in range(sc.n_bodies):
        c = np.ascontiguousarray(g["com_geom"][i])
        t = np.ascontiguousarray(g["tensor"][i])
        assert put(p.h, i + 1, float(g["mass"][i]), c.ctypes.data, t.ctypes.data) == 0
    # orientations set by the scene after creation: replay them on the moved bodies
    for op in sc.ops:
        if op[0] == "orient":
            p.set_orientation(op[1], op[2])
    p.step(int(g["steps"]))
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.array_equal(st[k], g[k]), k
    c = p.contacts()
    assert np.array_equal(c["magic_b"], g["magic_b"])
    assert np.array_equal(c["normal_impulse"], g["normal_impulse"])


def test_restatement_bitwise_on_chains(oracle_mod):
    """Articulated chains (ball-sockets and hinges, holonomic block solve,
    fixed spheres in the swing volume): bit-identical to the reference."""
    rng = np.random.default_rng(3)
    for _ in range(2):
        sc = scenes.chain_world(rng, 12, 24, n_spheres=30)
        r, p = oracle_mod.twin_worlds(sc)
        for s in range(120):
            r.step(1)
            p.step(1)
        assert _states_equal(r.state(), p.state()), sc.name
        cr, cp = r.contacts(), p.contacts()
        for k in ("b1", "b2", "magic_b", "normal_impulse"):
            assert np.array_equal(cr[k], cp[k]), k


def _holonomic_check(oracle_mod, world):
    f = oracle_mod.port_abi()._lib.cport_holonomic_check
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 4
    n, d, e = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    assert f(world.h, ctypes.byref(n), ctypes.byref(d), ctypes.byref(e)) == 0
    return n.value, d.value, e.value


def test_heavy_chain_known_answer(oracle_mod):
    """HolonomicBlockSolvingTests.h:8-91 ("High mass Ratio Chain"): over 30 s
    the ball stays within 65 m of the fixture; the restatement matches the
    reference bit for bit at every check; the block factorisation passes the
    reference's verifyInverse bound (HolonomicBlockSolver.cpp:545-583)."""
    r, p = oracle_mod.twin_worlds(scenes.heavy_chain())
    worst = 0.0
    for s in range(30):
        r.step(60)
        p.step(60)
        sr, sp = r.state(), p.state()
        assert _states_equal(sr, sp), f"differs after {60 * (s + 1)} steps"
        worst = max(worst, float(np.linalg.norm(sp["com"][-1])))
        assert worst <= 65.0, worst
    n, deg, err = _holonomic_check(oracle_mod, p)
    assert n == 1 and deg == 36 * 3
    assert err < 1e-5, err


def test_golden_fixture_chain(oracle_mod):
    """Ball-sockets, hinges and the holonomic block solve: the restatement,
    started from the reference's mass properties stored in the fixture,
    reproduces the reference's state after 200 steps bit for bit (no
    reference library needed)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "chain_seed5.npz"))
    sc = scenes.chain_world(np.random.default_rng(5), 10, 14, n_spheres=20)
    p = oracle_mod.port_world_with_mass(sc, g["mass"], g["com_geom"], g["tensor"])
    p.step(int(g["steps"]))
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.array_equal(st[k], g[k]), k


def test_restatement_bitwise_on_terrain(oracle_mod):
    """Boxes, spheres, cylinders and hulls on a value-noise triangle-mesh
    terrain (mesh tree candidates, triangle SAT with Gauss-region validity,
    manifold merging): bit-identical to the reference."""
    sc = scenes.terrain_drop(seed=1, n_grid=24, n_side=4, n_layers=2)
    r, p = oracle_mod.twin_worlds(sc)
    for s in range(150):
        r.step(1)
        p.step(1)
        if s % 30 == 29:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
    cr, cp = r.contacts(), p.contacts()
    assert np.sum(cr["b1"] == 1) > 20   # contacts with the terrain (body 1)
    for k in ("b1", "b2", "magic_b", "normal_impulse", "pen_depth"):
        assert np.array_equal(cr[k], cp[k]), k
    # the triangle id half of the contact-pair id (the other half is the
    # reference's process-global primitive counter, equal within an edge)
    assert np.array_equal(_tri_ids(cr), _tri_ids(cp))


def _tri_ids(c):
    return np.where(c["b1"] == 1, c["magic_c"] & 0xFFFFFFFF, 0)


def test_golden_fixture_terrain(oracle_mod):
    """The terrain scene against the committed reference outputs (no
    reference library needed)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "terrain_drop_seed2.npz"))
    sc = scenes.terrain_drop(seed=2, n_grid=16, n_side=3, n_layers=2)
    p = oracle_mod.port_world_with_mass(sc, g["mass"], g["com_geom"], g["tensor"])
    p.step(int(g["steps"]))
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.array_equal(st[k], g[k]), k
    c = p.contacts()
    assert np.array_equal(_tri_ids(c), np.where(c["b1"] == 1, g["magic_c"] & 0xFFFFFFFF, 0))
    assert np.array_equal(c["magic_b"], g["magic_b"])


@pytest.mark.parametrize("terrain", [False, True])
def test_restatement_bitwise_on_capsules(oracle_mod, terrain):
    """Capsules with every other primitive, on the plate or on a terrain
    mesh (SAT_PolyCapsule, detectSphereCapsule, detectCapsuleCapsule,
    detectCapsuleCylinder, SAT_CapsuleTriangle): bit-identical to the
    reference, and every capsule pair kind occurs."""
    sc = scenes.capsule_drop(seed=3, n_side=4, n_layers=2, terrain=terrain)
    kinds = [op[0] for op in sc.ops if op[0] in ("hull", "box", "sphere", "cylinder", "capsule", "mesh")]
    r, p = oracle_mod.twin_worlds(sc)
    seen = set()
    for s in range(150):
        r.step(1)
        p.step(1)
        c = r.contacts()
        for a, b in zip(c["b1"].tolist(), c["b2"].tolist()):
            seen.add(tuple(sorted((kinds[a - 1].replace("box", "hull"), kinds[b - 1].replace("box", "hull")))))
        if s % 25 == 24:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
    cr, cp = r.contacts(), p.contacts()
    for k in ("b1", "b2", "magic_b", "normal_impulse", "pen_depth"):
        assert np.array_equal(cr[k], cp[k]), k
    want = {("capsule", "capsule"), ("capsule", "hull"), ("capsule", "sphere"), ("capsule", "cylinder")}
    if terrain:
        want.add(("capsule", "mesh"))
    else:
        assert ("capsule", "hull") in seen   # the plate
    assert want <= seen, seen


def test_capsule_mass_properties_agree(oracle_mod):
    """Capsule mass properties (RigidBody.cpp:570-600: the mass is the volume,
    the density scales only the tensor) restated within rounding."""
    sc = scenes.Scene("capsules", dict(step_time=1.0 / 60.0))
    dense = dict(scenes.PILE_MATERIAL, density=2.5)
    for i, (r_, h_) in enumerate(((0.3, 0.8), (0.5, 0.0), (0.25, 1.7))):
        sc.capsule((float(i), -h_ / 2, 0.0), r_, h_, dense, scenes.DYNAMIC, (3.0 * i, 2.0, 0.0))
    r, p = oracle_mod.ref_world(), oracle_mod.port_world()
    scenes.apply(sc, r)
    scenes.apply(sc, p)
    get_r = oracle_mod.ref_abi()._lib.cpref_get_mass_properties
    get_p = oracle_mod.port_abi()._lib.cport_get_mass_properties
    for f in (get_r, get_p):
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    for bid in range(1, sc.n_bodies + 1):
        out = []
        for f, w in ((get_r, r), (get_p, p)):
            m, c, t = np.zeros(1), np.zeros(3), np.zeros(9)
            assert f(w.h, bid, m.ctypes.data, c.ctypes.data, t.ctypes.data) == 0
            out.append((m, c, t))
        (mr, cr, tr), (mp, cp, tp) = out
        assert abs(mr[0] - mp[0]) <= 1e-12 * mr[0]
        assert np.abs(cr - cp).max() <= 1e-12 * (1 + np.abs(cr).max())
        assert np.abs(tr - tp).max() <= 1e-10 * np.abs(tr).max()


def test_golden_fixture_capsules(oracle_mod):
    """Capsules on the terrain against the committed reference outputs (no
    reference library needed)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "capsule_terrain_seed5.npz"))
    sc = scenes.capsule_drop(seed=5, n_side=3, n_layers=2, terrain=True, n_grid=16)
    p = oracle_mod.port_world_with_mass(sc, g["mass"], g["com_geom"], g["tensor"])
    p.step(int(g["steps"]))
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.array_equal(st[k], g[k]), k
    c = p.contacts()
    assert np.array_equal(c["b1"], g["b1"]) and np.array_equal(c["b2"], g["b2"])
    assert np.array_equal(_tri_ids(c), np.where(c["b1"] == 1, g["magic_c"] & 0xFFFFFFFF, 0))
    assert np.array_equal(c["magic_b"], g["magic_b"])


def test_restatement_bitwise_with_kinematic_bodies(oracle_mod):
    """Kinematic bodies (infinite mass, moved by their own velocity, no
    gyroscopic term; islands stop at them as at fixed bodies): a sliding
    pusher and a spinning cylinder among dynamic bodies, bit-identical to the
    reference for 240 steps."""
    sc = scenes.kinematic_push(seed=1)
    r, p = oracle_mod.twin_worlds(sc)
    for s in range(240):
        r.step(1)
        p.step(1)
        if s % 40 == 39:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
    st = r.state()
    assert abs(st["com"][1, 0] - (-4.0 + 240 / 60.0)) < 1e-9   # the pusher moved 1 m/s x 4 s
    assert np.array_equal(st["ang_vel"][2], [0.0, 1.5, 0.0])
    cr, cp = r.contacts(), p.contacts()
    assert ((cr["b1"] == 2) | (cr["b2"] == 2)).any()            # the pusher touches the boxes
    for k in ("b1", "b2", "magic_b", "normal_impulse", "pen_depth"):
        assert np.array_equal(cr[k], cp[k]), k


def test_golden_fixture_kinematic(oracle_mod):
    """The kinematic scene against the committed reference outputs (no
    reference library needed)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "kinematic_push_seed1.npz"))
    sc = scenes.kinematic_push(seed=1)
    p = oracle_mod.port_world_with_mass(sc, g["mass"], g["com_geom"], g["tensor"])
    p.step(int(g["steps"]))
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.array_equal(st[k], g[k]), k
    c = p.contacts()
    for k in ("b1", "b2", "magic_b", "normal_impulse"):
        assert np.array_equal(c[k], g[k]), k


def _ray_batch(seed, n):
    rng = np.random.default_rng(seed)
    o = rng.uniform([-8, 2, -8], [8, 12, 8], size=(n, 3))
    d = rng.uniform([-6, -1, -6], [6, 4, 6], size=(n, 3)) - o
    return o, d / np.linalg.norm(d, axis=1, keepdims=True)


def test_raycast_restatement_matches_reference(oracle_mod):
    """raycastFirstIntersection: the restatement gives the reference's hit
    body, point, normal and distance bit for bit on 2,000 rays through a
    settled scene of every primitive kind on a terrain mesh (the reference's
    broadphase tree refreshed to the current AABBs first), also with bodies
    on the ignore list."""
    sc = scenes.capsule_drop(seed=3, n_side=4, n_layers=2, terrain=True)
    r, p = oracle_mod.twin_worlds(sc)
    r.step(90)
    p.step(90)
    o, d = _ray_batch(0, 2000)
    for ignore in ((), (1, 5, 9)):
        hr, hp = r.raycast(o, d, ignore), p.raycast(o, d, ignore)
        for k in ("body", "pos", "normal", "dist"):
            assert np.array_equal(hr[k], hp[k]), k
        assert (hr["body"] > 0).sum() > 150
        assert not np.isin(hr["body"], ignore).any()
    kinds = [op[0] for op in sc.ops if op[0] in ("hull", "box", "sphere", "cylinder", "capsule", "mesh")]
    hit = r.raycast(o, d)["body"]
    assert {kinds[b - 1] for b in hit[hit > 0]} >= {"box", "sphere", "cylinder", "capsule", "hull", "mesh"}


def _sleep_scene(seed):
    return scenes.sleep_stacks(seed)


@pytest.mark.parametrize("seed", [0, 2])
def test_restatement_bitwise_with_sleeping(oracle_mod, seed):
    """Sleeping enabled (PhysicsEngine.cpp:65-87, 174, 1113-1136, 1221-1290,
    1536-1613; Contact::isExpired): three box stacks and a ball settle and
    fall asleep, a velocity set on a sleeping box wakes it, the ball is then
    dropped onto a sleeping stack and wakes it, and the boxes fall asleep
    again; bit-identical to the reference over 500 steps."""
    sc, ball, x = _sleep_scene(seed)
    r, p = oracle_mod.twin_worlds(sc)
    saw_all_asleep = saw_wake = False
    for s in range(500):
        if s == 150:
            for w in (r, p):
                w.set_velocity(3, (0.5, 0.0, 0.0))
        if s == 300:
            for w in (r, p):
                w.set_position(ball, (x, 4.5, 0.1))
                w.set_velocity(ball, (0.0, -3.0, 0.0))
        r.step(1)
        p.step(1)
        st = r.state()
        assert _states_equal(st, p.state()), f"state differs at step {s}"
        asleep = r.asleep()
        assert np.array_equal(asleep, p.asleep()), f"sleeping set differs at step {s}"
        if s == 149:
            saw_all_asleep = asleep[1:].all()                # every body but the plate
        if 300 < s < 330 and (asleep[1:-1] == 0).sum() >= 2:
            saw_wake = True                                  # the impact woke boxes of the stack
    assert saw_all_asleep and saw_wake
    assert r.asleep().sum() >= 4   # most boxes asleep again


@pytest.mark.parametrize("seed,terrain", [(0, False), (1, False), (2, True)])
def test_restatement_bitwise_with_union_bodies(oracle_mod, seed, terrain):
    """Multi-primitive bodies (ConvexUnionGeometry::merge; per-primitive
    AABBs and materials, primitive pairs tested one by one and their
    manifolds merged per body pair, PhysicsEngine.cpp:182-219): box L-shapes,
    dumbbells, tables on cylinder legs and hull-sphere pairs among boxes,
    bit-identical to the reference over 240 steps, contacts included; ray
    queries through them too."""
    sc = scenes.union_drop(seed=seed, n=10, terrain=terrain)
    r, p = oracle_mod.twin_worlds(sc)
    for s in range(240):
        r.step(1)
        p.step(1)
        if s % 40 == 39:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
    cr, cp = r.contacts(), p.contacts()
    assert len(cr["b1"]) > 20
    for k in ("b1", "b2", "magic_b", "normal_impulse", "pen_depth"):
        assert np.array_equal(cr[k], cp[k]), k
    o, d = _ray_batch(seed + 7, 1000)
    hr, hp = r.raycast(o, d), p.raycast(o, d)
    for k in ("body", "pos", "normal", "dist"):
        assert np.array_equal(hr[k], hp[k]), k
    assert (hr["body"] > 1).sum() > 10


def test_union_mass_properties_agree(oracle_mod):
    """Mass properties of multi-primitive bodies summed over the primitives
    (RigidBody.cpp:427-640) agree with the reference's to rounding."""
    sc = scenes.union_drop(seed=3, n=10)
    r, p = oracle_mod.ref_world(), oracle_mod.port_world()
    scenes.apply(sc, r)
    scenes.apply(sc, p)
    get_r = oracle_mod.ref_abi()._lib.cpref_get_mass_properties
    get_p = oracle_mod.port_abi()._lib.cport_get_mass_properties
    for f in (get_r, get_p):
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    for bid in range(2, sc.n_bodies + 1):
        out = []
        for f, w in ((get_r, r), (get_p, p)):
            m, c, t = np.zeros(1), np.zeros(3), np.zeros(9)
            assert f(w.h, bid, m.ctypes.data, c.ctypes.data, t.ctypes.data) == 0
            out.append((m, c, t))
        (mr, cr, tr), (mp, cp, tp) = out
        assert abs(mr[0] - mp[0]) <= 1e-12 * mr[0], bid
        assert np.abs(cr - cp).max() <= 1e-12 * (1 + np.abs(cr).max()), bid
        assert np.abs(tr - tp).max() <= 1e-10 * np.abs(tr).max(), bid


def test_golden_fixture_unions(oracle_mod):
    """Multi-primitive bodies on the terrain against the committed reference
    outputs (no reference library needed)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "union_terrain_seed2.npz"))
    sc = scenes.union_drop(seed=2, n=10, terrain=True)
    p = oracle_mod.port_world_with_mass(sc, g["mass"], g["com_geom"], g["tensor"])
    p.step(int(g["steps"]))
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.array_equal(st[k], g[k]), k
    c = p.contacts()
    for k in ("b1", "b2", "magic_b", "normal_impulse"):
        assert np.array_equal(c[k], g[k]), k


@pytest.mark.parametrize("mixed", [False, True])
def test_restatement_bitwise_with_distance_joints(oracle_mod, mixed):
    """Distance constraints (PhysicsEngine::addDistanceConstraint,
    DistanceConstraint rows, ConstraintSolver.cpp:348-377): a hanging chain of
    spheres linked by distance joints, or by alternating distance and
    ball-socket joints (one holonomic system, solved by the block LDL), hit by
    a box; bit-identical to the reference over 300 steps."""
    sc = scenes.distance_chain(mixed)
    r, p = oracle_mod.twin_worlds(sc)
    for s in range(300):
        r.step(1)
        p.step(1)
        if s % 50 == 49:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
    st = r.state()
    assert st["com"][2:8, 1].min() < 7.0   # the chain swung down


@pytest.mark.parametrize("mixed", [False, True])
def test_restatement_bitwise_with_weld_joints(oracle_mod, mixed):
    """Weld constraints (PhysicsEngine::addWeldConstraint, WeldConstraint
    rows, ConstraintSolver.cpp:861-899): a cantilever of boxes welded to a
    fixed post, one link turned so the orientation correction acts, or with
    every other weld a hinge (one holonomic system of 6- and 5-dof blocks),
    hit by a falling box; bit-identical to the reference over 300 steps."""
    sc = scenes.weld_cantilever(mixed)
    r, p = oracle_mod.twin_worlds(sc)
    for s in range(300):
        r.step(1)
        p.step(1)
        if s % 50 == 49:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
    st = r.state()
    assert st["com"][7, 1] < 5.0   # the dropped box came down


@pytest.mark.parametrize("kinds", [("slider",) * 4, ("sliding_hinge",) * 4,
                                   ("slider", "sliding_hinge", "hinge", "slider")])
def test_restatement_bitwise_with_slider_joints(oracle_mod, kinds):
    """Slider and sliding-hinge constraints (PhysicsEngine::addSliderConstraint
    / addSlidingHingeConstraint; SliderConstraint, ConstraintSolver.cpp:611-696,
    SlidingHingeConstraint, :781-852): a chain of boxes hung from a fixed post
    on tilted slide axes, one link turned, alone or mixed with a hinge in one
    holonomic system, hit by a falling box; bit-identical to the reference over
    300 steps."""
    sc = scenes.slider_chain(kinds)
    r, p = oracle_mod.twin_worlds(sc)
    start = r.state()["com"][2:6].copy()
    for s in range(300):
        r.step(1)
        p.step(1)
        if s % 50 == 49:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
    moved = np.linalg.norm(r.state()["com"][2:6] - start, axis=1)
    assert moved.max() > 0.3   # the links slid


@pytest.mark.parametrize("with_joints", [False, True])
def test_restatement_bitwise_with_springs(oracle_mod, with_joints):
    """Springs (PhysicsEngine::addSpring, the impulse pass of
    PhysicsEngine.cpp:1313-1356): boxes hung from a fixed post on damped
    springs (two sharing a body, one at its creation length), bouncing on the
    ground and off each other, or sharing bodies with ball-socket joints;
    bit-identical to the reference over 300 steps."""
    sc = scenes.spring_chain(with_joints)
    r, p = oracle_mod.twin_worlds(sc)
    start = r.state()["com"][2:6].copy()
    for s in range(300):
        r.step(1)
        p.step(1)
        if s % 50 == 49:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"
    assert np.linalg.norm(r.state()["com"][2:6] - start, axis=1).max() > 0.2   # the springs moved the boxes


@pytest.mark.parametrize("holo", [0, 1])
def test_restatement_bitwise_with_cone_limits(oracle_mod, holo):
    """Cone limits (PhysicsEngine::addConeLimitConstraint; ConeLimitConstraint,
    ConstraintSolver.cpp:410-436, an inequality row that exists only while the
    limit is reached): a ball-socket chain swung sideways with a 25-degree cone
    on each joint, with and without the holonomic block solve (the cone rows
    stay out of the holonomic system); bit-identical to the reference over 300
    steps, and the limits do engage."""
    sc = scenes.cone_chain(holo)
    r, p = oracle_mod.twin_worlds(sc)
    for s in range(300):
        r.step(1)
        p.step(1)
        if s % 50 == 49:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"


def test_restatement_bitwise_with_twist_limits(oracle_mod):
    """Twist limits (PhysicsEngine::addTwistLimitConstraint; TwistLimit's
    unwrapped angle, PersistentConstraint.cpp:115-131, and the one-sided
    TwistLimitConstraint row, ConstraintSolver.cpp:439-466) beside cone limits
    on a ball-socket chain spun about its axis; bit-identical to the
    reference over 300 steps, and the twist limit does engage."""
    sc = scenes.twist_chain()
    r, p = oracle_mod.twin_worlds(sc)
    for s in range(300):
        r.step(1)
        p.step(1)
        if s % 50 == 49:
            assert _states_equal(r.state(), p.state()), f"state differs at step {s}"


def _state_chain():
    M = scenes.PILE_MATERIAL
    sc = scenes.Scene("state_chain", dict(step_time=1.0 / 60.0, substeps=4, pgs=(10, 1, 1), sleeping=False))
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, scenes.FIXED)
    prev = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, scenes.FIXED, (0.0, 4.0, 0.0))
    for i, kind in enumerate(("hinge", "ball", "weld", "hinge", "ball")):
        b = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, scenes.DYNAMIC, (0.6 * (i + 1), 4.0, 0.0))
        if kind == "hinge":
            sc.hinge(prev, b, (0.3, 0, 0), (-0.3, 0, 0), (0, 0, 1), (0, 0, 1))
        elif kind == "ball":
            sc.ball_socket(prev, b, (0.3, 0, 0), (-0.3, 0, 0))
            sc.cone_limit(prev, b, (1.0, 0.0, 0.0), (1.0, 0.0, 0.0), 15.0 * np.pi / 180.0)
            sc.twist_limit(prev, b, (1.0, 0.0, 0.0), (1.0, 0.0, 0.0), -0.2, 0.2)
        else:
            sc.weld(prev, b, (0.3, 0, 0), (-0.3, 0, 0))
        prev = b
    sc.ang_velocity(prev, (6.0, 2.0, 0.0))
    return sc


def test_restatement_joint_state_layout(oracle_mod):
    """The restatement's joint-state export and import use the C ABI's layout
    (6 impulses per joint, 2 auxiliary values for limits): a round trip
    through a second world reproduces the state, for hinges, ball sockets, a
    weld (all 6 impulses), cone and twist limits (angle and reached flag)."""
    sc = _state_chain()
    a, b = oracle_mod.port_world(), oracle_mod.port_world()
    scenes.apply(sc, a)
    scenes.apply(sc, b)
    a.step(20)
    ja = a.joint_state()
    assert ja["impulse"].shape == (9, 6) and ja["aux"].shape == (9, 2)
    kinds = ["hinge", "ball", "cone", "twist", "weld", "hinge", "ball", "cone", "twist"]
    weld = kinds.index("weld")
    assert np.abs(ja["impulse"][weld, 5]) > 0                                  # the weld's sixth row
    ball = kinds.index("ball")
    assert np.all(ja["impulse"][ball, 3:] == 0) and np.abs(ja["impulse"][ball, :2]).min() > 0   # 3 rows
    twist = [i for i, k in enumerate(kinds) if k == "twist"]
    assert np.abs(ja["aux"][twist, 0]).max() > 0                               # twist angles tracked
    b.set_joint_state(ja)
    jb = b.joint_state()
    for k in ja:
        assert np.array_equal(ja[k], jb[k]), k


def test_restatement_checkpoint_restore_steps_like_the_uninterrupted_run(oracle_mod):
    """A world restored from a checkpoint (bodies, contacts and joint state,
    limits included) steps exactly like the run that was never interrupted."""
    sc = _state_chain()
    a = oracle_mod.port_world()
    scenes.apply(sc, a)
    a.step(25)
    b = oracle_mod.port_world()
    scenes.apply(sc, b)
    b.set_state(**a.state())
    b.set_contacts(a.contacts())
    b.set_joint_state(a.joint_state())
    for _ in range(4):
        a.step(10)
        b.step(10)
        sa, sb = a.state(), b.state()
        for k in sa:
            assert np.array_equal(sa[k], sb[k]), k
    ja, jb = a.joint_state(), b.joint_state()
    for k in ja:
        assert np.array_equal(ja[k], jb[k]), k

POWERED = [("motor", m, lim) for m in (1, 2, 3) for lim in (False, True) if not (m == 1 and lim)] + \
          [("piston", m, lim) for m in (1, 2, 3) for lim in (False, True)]


def _powered_scene(kind, mode, limits):
    return scenes.motor_chain(mode, limits) if kind == "motor" else scenes.piston_chain(mode, limits)


@pytest.mark.parametrize("kind,mode,limits", POWERED)
def test_restatement_bitwise_with_motors_and_pistons(oracle_mod, kind, mode, limits):
    """Motors on hinges and pistons on sliders (PhysicsEngine.cpp:725-852;
    Motor / Piston, PersistentConstraint.cpp:5-200, 300-328; MotorConstraint,
    PistonConstraint, SlideLimitConstraint, ConstraintSolver.cpp:555-775) in
    constant, target-velocity and target-position modes, with and without
    limits, switched off and to another mode mid-run: bit-identical to the
    reference, angles and slide positions included.  (A constant torque
    driving a hinge past a limit on the side it pushes from makes the
    reference's target velocity infinite and its state NaN; that case is
    left out.)"""
    sc = _powered_scene(kind, mode, limits)
    r, p = oracle_mod.twin_worlds(sc)
    ids = r.constraint_ids[1::2]            # hinge / slider, then its motor / piston
    getter = "motor_position" if kind == "motor" else "piston_position"
    setter = "set_motor" if kind == "motor" else "set_piston"
    for s in range(160):
        if s == 60:
            for w in (r, p):
                getattr(w, setter)(ids[0], 0)                       # off
                getattr(w, setter)(ids[1], 2, 50.0, -0.4)           # target velocity
        if s == 110:
            for w in (r, p):
                getattr(w, setter)(ids[2], 3, 60.0, 0.2)            # target position
        r.step(1)
        p.step(1)
        sr, sp = r.state(), p.state()
        assert _states_equal(sr, sp), f"state differs at step {s}"
        pr = [getattr(r, getter)(c) for c in ids]
        pp = [getattr(p, getter)(c) for c in ids]
        assert pr == pp, (s, pr, pp)
    assert np.abs(np.array(pr)).max() > 1e-3     # the joints moved


def test_restatement_checkpoint_restore_with_motors_and_pistons(oracle_mod):
    """Joint state of motors (angle, previous relative velocity) and pistons
    (slide position, past-limit flag; two slots each) restores exactly."""
    for sc in (scenes.motor_chain(3, True), scenes.piston_chain(2, True)):
        a = oracle_mod.port_world()
        scenes.apply(sc, a)
        a.step(30)
        b = oracle_mod.port_world()
        scenes.apply(sc, b)
        b.set_state(**a.state())
        b.set_contacts(a.contacts())
        b.set_joint_state(a.joint_state())
        for _ in range(3):
            a.step(10)
            b.step(10)
            sa, sb = a.state(), b.state()
            for k in sa:
                assert np.array_equal(sa[k], sb[k]), (sc.name, k)


def _golden_scenes():
    """The joint-kinds fixture's scene table, from the script that made it."""
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.joint_scenes()


@pytest.mark.parametrize("name", ["distance", "weld", "slider", "cone", "twist", "spring", "motor_pos", "motor_vel",
                                  "piston_vel", "piston_pos"])
def test_golden_fixture_joint_kinds(oracle_mod, name):
    """Distance, weld, slider / sliding-hinge, cone- and twist-limit joints,
    springs, motors and pistons against the committed reference outputs (no
    reference library needed): the restatement, started from the reference's
    mass properties, gives the reference's states after 200 steps bit for
    bit, and the motors' angles and pistons' slide positions."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "joint_kinds.npz"))
    sc, steps = _golden_scenes()[name]
    assert int(g[f"{name}_steps"]) == steps
    p = oracle_mod.port_world_with_mass(sc, g[f"{name}_mass"], g[f"{name}_com_geom"], g[f"{name}_tensor"])
    p.step(steps)
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.array_equal(st[k], g[f"{name}_{k}"]), k
    if f"{name}_positions" in g.files:
        get = p.motor_position if name.startswith("motor") else p.piston_position
        got = np.array([get(cid) for cid in p.constraint_ids[1::2]])
        assert np.array_equal(got, g[f"{name}_positions"])


def test_golden_fixture_sleeping(oracle_mod):
    """Sleeping against the committed reference outputs: three box stacks and
    a ball settle and fall asleep; after 400 steps the restatement's states
    and sleeping bodies are the reference's, bit for bit."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "sleep_stacks_seed0.npz"))
    sc, _, _ = scenes.sleep_stacks(0)
    p = oracle_mod.port_world_with_mass(sc, g["mass"], g["com_geom"], g["tensor"])
    p.step(int(g["steps"]))
    st = p.state()
    for k in ("com", "quat", "vel", "ang_vel"):
        assert np.array_equal(st[k], g[k]), k
    assert g["asleep"].sum() >= 9   # the stacks sleep
    assert np.array_equal(p.asleep(), g["asleep"])


def test_golden_fixture_rays(oracle_mod):
    """raycastFirstIntersection against the committed reference outputs (no
    reference library needed): 2,000 rays through a settled scene of every
    primitive kind on a terrain and through bodies of several primitives,
    with and without an ignore list; hit body, point, normal and distance
    bit for bit."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "rays.npz"))
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(__file__), "golden",
                                                                             "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    o, d = g["origins"], g["dirs"]
    for name, (sc, steps, ignores) in mod.ray_scenes().items():
        p = oracle_mod.port_world_with_mass(sc, g[f"{name}_mass"], g[f"{name}_com_geom"], g[f"{name}_tensor"])
        p.step(steps)
        for i, ig in enumerate(ignores):
            h = p.raycast(o, d, ig)
            for k in ("body", "pos", "normal", "dist"):
                assert np.array_equal(h[k], g[f"{name}_{i}_{k}"]), (name, i, k)
            assert (h["body"] > 0).sum() > 100
