"""Device path against the oracle, on a GB300.

Per-step parity: the device state (bodies and the persistent contact graph)
after k steps is imported into the CPU restatement, both advance one step from
that identical input, and the results are compared.  Tolerances are FP32-vs-FP64
ones, written at each assertion; at exact ties of the separating-axis choice
(face-on-face stacking) the two sides may pick different but equivalent
features, so contact-id equality is asserted only where no such tie exists.
"""
import os

import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu


def _step_both(sc, k, oracle_mod):
    g = cg.world()
    scenes.apply(sc, g)
    g.step(k)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    p.set_state(**g.state())
    p.set_contacts(g.contacts())
    aabb = g.aabbs()
    g.step(1)
    p.step(1)
    return g, p, aabb


def _fresh(c):
    m = c["memory_life"] == 5   # detected in the last step
    return set(zip(c["b1"][m].tolist(), c["b2"][m].tolist(), c["magic_b"][m].tolist()))


def _fresh_points(c):
    m = c["memory_life"] == 5
    return {(int(c["b1"][i]), int(c["b2"][i]), int(c["magic_b"][i])): c["p_local_b1"][i] for i in np.nonzero(m)[0]}


def _match(cg_, cp_, tol=2e-4):
    """Last-step contacts paired by MagicID, or else by position within `tol`
    on the same body pair: at a parallel-face near-tie FP32 and FP64 may take
    the other face as the reference and clip out the same points with other
    ids.  Returns (by id, by position, unmatched restatement, unmatched device)."""
    G, P = _fresh_points(cg_), _fresh_points(cp_)
    by_id = [k for k in P if k in G]
    rest = [k for k in G if k not in P]
    used, miss = set(), []
    for k in (k for k in P if k not in G):
        near = [j for j in rest if j[:2] == k[:2] and j not in used and np.abs(G[j] - P[k]).max() <= tol]
        if near:
            used.add(near[0])
        else:
            miss.append(k)
    return by_id, len(used), miss, [j for j in rest if j not in used]


def _on_segment(c, key, tol=1e-4):
    """Whether restatement contact `key` lies on the segment between two other
    points of its manifold.  A hull face with a vertex on the line of its
    neighbours makes two nearly parallel clipping edges; FP64 keeps that vertex
    as a contact point, FP32 clipping may drop it, and the manifold's support
    polygon is the same either way."""
    P = _fresh_points(c)
    x = P[key]
    others = [v for k, v in P.items() if k[:2] == key[:2] and k != key]
    for i in range(len(others)):
        for j in range(i + 1, len(others)):
            a, b = others[i], others[j]
            d = b - a
            t = float(np.dot(x - a, d) / max(np.dot(d, d), 1e-30))
            if 0.0 < t < 1.0 and np.linalg.norm(a + t * d - x) <= tol:
                return True
    return False


def test_smoke():
    import __graft_entry__
    __graft_entry__.smoke()


@pytest.mark.parametrize("k", [40, 80, 120])
def test_single_step_parity_hull_pile(oracle_mod, k):
    g, p, aabb = _step_both(scenes.hull_drop(seed=1, n_side=3), k, oracle_mod)
    # pair set: bit-exact, and exactly the overlaps of the device's own AABBs
    assert np.array_equal(g.pairs(), p.pairs())
    lo, hi = aabb[:, :3], aabb[:, 3:]
    ov = ~((hi[:, None, :] < lo[None, :, :]) | (lo[:, None, :] > hi[None, :, :])).any(axis=2)
    i, j = np.nonzero(np.triu(ov, 1))
    assert np.array_equal(np.stack([i + 1, j + 1], 1).astype(np.uint32), g.pairs())
    # contact features (MagicIDs) identical, up to the parallel-face near-tie
    by_id, by_pos, miss_p, miss_g = _match(g.contacts(), p.contacts())
    assert not miss_g, miss_g
    assert all(_on_segment(p.contacts(), k) for k in miss_p), miss_p
    sg, sp = g.state(), p.state()
    # a contact matched by position has a new MagicID in the restatement, which
    # therefore solves it without the warm-start impulse the device keeps
    dv, dw, dx = (1e-4, 1e-4, 1e-5) if by_pos == 0 else (1e-2, 5e-2, 2e-4)
    stats = f"ties {by_pos} of {len(by_id) + by_pos}"
    assert np.abs(sg["vel"] - sp["vel"]).max() <= dv, stats          # m/s, FP32 vs FP64
    assert np.abs(sg["ang_vel"] - sp["ang_vel"]).max() <= dw, stats  # rad/s
    assert np.abs(sg["com"] - sp["com"]).max() <= dx, stats          # m


def test_single_step_parity_1000_hulls(oracle_mod):
    g, p, _ = _step_both(scenes.hull_drop(seed=0, n_side=10), 60, oracle_mod)
    assert np.array_equal(g.pairs(), p.pairs())
    fg, fp = _fresh(g.contacts()), _fresh(p.contacts())
    assert len(fg ^ fp) <= 0.05 * len(fp)
    sg, sp = g.state(), p.state()
    dv = np.linalg.norm(sg["vel"] - sp["vel"], axis=1)
    vm = np.linalg.norm(sp["vel"], axis=1)
    assert np.mean(dv <= 1e-4 + 1e-3 * vm) >= 0.99
    assert np.median(dv) <= 1e-5


def test_single_step_parity_pyramid(oracle_mod):
    rng = np.random.default_rng(7)
    pool = scenes.HullPool(0, size=8)
    sc = None
    while sc is None or not sc.name.startswith("pyramid"):
        sc = scenes.batched_world(rng, pool, 30, 120)
    g, p, _ = _step_both(sc, 60, oracle_mod)
    assert np.array_equal(g.pairs(), p.pairs())
    sg, sp = g.state(), p.state()
    # stacked boxes touch face-on-face: the separating-axis choice is an exact
    # tie that FP32 and FP64 break differently (equivalent contact features),
    # so per-body velocities agree to 1e-3 m/s in the median and to 1e-2 m/s
    # for the bodies whose contact features flipped
    dv = np.linalg.norm(sg["vel"] - sp["vel"], axis=1)
    stats = f"median {np.median(dv):.2e} max {dv.max():.2e} frac<=1e-4 {np.mean(dv <= 1e-4):.2f}"
    assert np.median(dv) <= 1e-3, stats
    assert dv.max() <= 1e-2, stats
    assert np.abs(sg["com"] - sp["com"]).max() <= 2e-4


def test_box_vs_ground_device():
    """CollisionTests.h:77-165 (Box vs Ground) with sleeping disabled: the box
    rests at y = 0.5 +- 0.1 with vertical normals."""
    w = cg.world()
    w.set_params(step_time=1.0 / 60.0, sleeping=False)
    w.add_box((-50.0, -0.5, -50.0), 100.0, 0.5, 100.0, None, scenes.FIXED)
    box = w.add_box((0.0, 5.0, 0.0), 1.0, 1.0, 1.0, None, scenes.DYNAMIC)
    w.step(300)
    st, c = w.state(), w.contacts()
    fresh = c["memory_life"] == 5
    assert fresh.any() and (np.abs(c["n_local_b1"][fresh][:, 1]) >= 0.9999).all()
    # FP32 leaves ~2e-3 m/s of residual motion at rest (FP64: ~5e-4)
    assert np.linalg.norm(st["vel"][box - 1]) < 5e-3
    assert abs(st["com"][box - 1, 1] - 0.5) < 0.1


def test_trajectory_drift_box_drop(oracle_mod):
    """A tilted box dropped on the plate, 300 steps, device vs reference engine:
    positions agree to 1e-3 m until the box comes to rest; at rest both settle
    inside the 0.05 m penetration slop, so the final heights agree to 1e-2 m."""
    sc = scenes.Scene("box", dict(step_time=1 / 60, sleeping=False))
    sc.box((-50, -2, -50), 100, 2, 100, None, scenes.FIXED)
    b = sc.box((-0.5, 3, -0.5), 1, 1, 1, None, scenes.DYNAMIC)
    sc.orient(b, scenes.random_quat(np.random.default_rng(3)))
    g = cg.world()
    scenes.apply(sc, g)
    r = oracle_mod.ref_world()
    scenes.apply(sc, r)
    for s in range(300):
        g.step(1)
        r.step(1)
        if s == 100:
            assert np.abs(g.state()["com"] - r.state()["com"]).max() <= 1e-3
    assert np.abs(g.state()["com"] - r.state()["com"]).max() <= 1e-2


def test_batch_equals_single_worlds():
    rng = np.random.default_rng(5)
    pool = scenes.HullPool(1, size=8)
    scs = [scenes.batched_world(rng, pool, 8, 60) for _ in range(3)]
    singles = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        w.step(50)
        singles.append(w.state())
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    b = cg.Batch(ws)
    b.step(50)
    for i, st in enumerate(singles):
        bs = b.state(i)
        for k in ("com", "quat", "vel", "ang_vel"):
            assert np.array_equal(bs[k], st[k]), (i, k)


def test_batch_state_roundtrip_is_exact():
    rng = np.random.default_rng(9)
    pool = scenes.HullPool(2, size=8)
    scs = [scenes.batched_world(rng, pool, 8, 60) for _ in range(2)]
    outs = []
    for roundtrip in (False, True):
        ws = []
        for sc in scs:
            w = cg.world()
            scenes.apply(sc, w)
            ws.append(w)
        b = cg.Batch(ws)
        for _ in range(40):
            if roundtrip:
                b.write_state(b.read_state())
            b.step(1)
        outs.append([b.state(i) for i in range(len(scs))])
    for a, c in zip(*outs):
        for k in a:
            assert np.array_equal(a[k], c[k]), k


def _worlds(scs):
    out = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        out.append(w)
    return out


def test_partitioned_batch_equals_single_worlds(monkeypatch):
    """A batch of 12 worlds of mixed sizes is split into parts stepped on
    their own streams; every world still steps exactly as it does alone, and
    the host-layout state rows follow the batch's world order."""
    rng = np.random.default_rng(21)
    pool = scenes.HullPool(3, size=8)
    scs = [scenes.batched_world(rng, pool, 8, 120) for _ in range(12)]
    monkeypatch.setenv("CPGPU_BATCH_PARTS", "4")
    singles = []
    for w in _worlds(scs):
        w.step(40)
        singles.append(w.state())
    b = cg.Batch(_worlds(scs))
    b.step(40)
    rows = b.read_state()
    r0 = 0
    for i, st in enumerate(singles):
        bs = b.state(i)
        for k in ("com", "quat", "vel", "ang_vel"):
            assert np.array_equal(bs[k], st[k]), (i, k)
        n = len(st["com"])
        assert np.array_equal(rows[r0:r0 + n, 0:3].astype(np.float64), st["com"]), i
        assert np.array_equal(rows[r0:r0 + n, 4:8].astype(np.float64), st["quat"]), i
        r0 += n
    assert r0 == b.n_bodies


def test_partitioned_state_roundtrip_is_exact(monkeypatch):
    monkeypatch.setenv("CPGPU_BATCH_PARTS", "3")
    rng = np.random.default_rng(22)
    pool = scenes.HullPool(4, size=8)
    scs = [scenes.batched_world(rng, pool, 8, 60) for _ in range(9)]
    outs = []
    for roundtrip in (False, True):
        b = cg.Batch(_worlds(scs))
        for _ in range(30):
            if roundtrip:
                b.write_state(b.read_state())
            b.step(1)
        outs.append([b.state(i) for i in range(len(scs))])
    for a, c in zip(*outs):
        for k in a:
            assert np.array_equal(a[k], c[k]), k


def test_capacity_overflow_is_reported(monkeypatch):
    """A pair buffer that is too small makes step() return CPGPU_ERR_CAPACITY
    (the kernels clamp their writes); the world stays usable for queries."""
    monkeypatch.setenv("CPGPU_CAPACITY_FLOOR", "16")
    monkeypatch.setenv("CPGPU_PAIRS_PER_BODY", "0")
    w = cg.world()
    scenes.apply(scenes.hull_drop(seed=1, n_side=3), w)
    with pytest.raises(cg.CPGPUError, match="status -3"):
        w.step(120)
    assert np.isfinite(w.state()["com"]).all()


def test_default_partition_of_large_worlds_equals_single(monkeypatch):
    """512 worlds, four of 500 bodies and the rest of 8-16: the default
    partition puts the large worlds in a part of their own, whose kernels use
    more dynamic shared memory (island graph, solver Δv) than the part built
    after it.  Every world still steps exactly as it does alone."""
    monkeypatch.delenv("CPGPU_BATCH_PARTS", raising=False)
    monkeypatch.delenv("CPGPU_BATCH_FIRST_SHARE", raising=False)
    rng = np.random.default_rng(33)
    pool = scenes.HullPool(4, size=8)
    scs = [scenes.batched_world(rng, pool, 500, 501) for _ in range(4)]
    scs += [scenes.batched_world(rng, pool, 8, 16) for _ in range(508)]
    order = rng.permutation(len(scs))
    scs = [scs[i] for i in order]
    check = [int(np.where(order == k)[0][0]) for k in range(4)] + [0, 1, 2, 511]
    b = cg.Batch(_worlds(scs))
    b.step(20)
    for i in check:
        w = _worlds([scs[i]])[0]
        w.step(20)
        st, bs = w.state(), b.state(i)
        for k in ("com", "quat", "vel", "ang_vel"):
            assert np.array_equal(bs[k], st[k]), (i, k)


def test_large_world_pair_set_is_the_brute_force_set():
    """A world above the tiled pair pass's size (3,001 bodies: spheres and
    boxes scattered so that many AABBs overlap, and a plate under them): the
    pair list is exactly the sorted set of overlapping AABB pairs
    of the device's own AABBs, as in small worlds."""
    rng = np.random.default_rng(11)
    sc = scenes.Scene("scatter_3001", dict(step_time=1.0 / 60.0, sleeping=False, gravity=(0.0, 0.0, 0.0)))
    sc.box((-30.0, -1.0, -30.0), 60.0, 1.0, 60.0, scenes.PILE_MATERIAL, scenes.FIXED)
    for k in range(3000):
        pos = tuple(rng.uniform(-25.0, 25.0, 3) * np.array([1.0, 0.2, 1.0]) + np.array([0.0, 5.0, 0.0]))
        if k % 3:
            sc.sphere((0, 0, 0), float(rng.uniform(0.2, 0.6)), scenes.PILE_MATERIAL, scenes.DYNAMIC, pos)
        else:
            sc.box((-0.4, -0.4, -0.4), 0.8, 0.8, 0.8, scenes.PILE_MATERIAL, scenes.DYNAMIC, pos)
    w = cg.world()
    scenes.apply(sc, w)
    w.step(1)
    aabb = w.aabbs()
    w.step(1)
    lo, hi = aabb[:, :3], aabb[:, 3:]
    ov = ~((hi[:, None, :] < lo[None, :, :]) | (lo[:, None, :] > hi[None, :, :])).any(axis=2)
    i, j = np.nonzero(np.triu(ov, 1))
    want = np.stack([i + 1, j + 1], 1).astype(np.uint32)
    got = w.pairs()
    assert len(want) > 100
    assert np.array_equal(got, want)
