"""Bodies of several primitives (ConvexUnionGeometry) on the device, against
the CPU restatement (pinned bit for bit to the reference on the same scenes:
tests/test_oracle.py::test_restatement_bitwise_with_union_bodies), on a GB300.

Box L-shapes, dumbbells (a capsule and two spheres), tables (a box top on
four cylinder legs) and hull-sphere pairs among boxes, on a plate and on a
terrain mesh: each primitive pair whose AABBs overlap is tested by its own
detector, the pair's manifolds merged and culled as for mesh pairs
(PhysicsEngine.cpp:182-295), each contact taking the touching primitives'
materials; per-primitive AABBs for the pair and ray queries.

Per-step parity as in test_gpu_capsules: the device state after k steps is
imported into the restatement and both step once; contacts pair by MagicID
(feature ids and the primitive pair) or position.
"""
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
    if k > 0:
        p.set_state(**g.state())
        p.set_contacts(g.contacts())
    g.step(1)
    p.step(1)
    return g, p


def _fresh(c):
    m = c["memory_life"] == 5
    return {(int(c["b1"][i]), int(c["b2"][i]), int(c["magic_c"][i]), int(c["magic_b"][i])): i for i in np.nonzero(m)[0]}


def _match(cg_, cp_, tol=2e-4):
    G, P = _fresh(cg_), _fresh(cp_)
    by_id = [k for k in P if k in G]
    rest_g = [k for k in G if k not in P]
    used, unmatched = set(), []
    for k in (k for k in P if k not in G):
        near = [j for j in rest_g if j[:2] == k[:2] and j not in used and
                np.abs(cg_["p_local_b1"][G[j]] - cp_["p_local_b1"][P[k]]).max() <= tol]
        if near:
            used.add(near[0])
        else:
            unmatched.append(k)
    return by_id, len(used), unmatched, [j for j in rest_g if j not in used]


@pytest.mark.parametrize("seed,terrain,k", [(0, False, 0), (0, False, 60), (0, False, 160), (1, False, 120), (1, False, 220),
                                            (2, True, 80), (2, True, 140), (2, True, 200)])
def test_union_single_step_parity(oracle_mod, seed, terrain, k):
    sc = scenes.union_drop(seed=seed, n=10, terrain=terrain)
    g, p = _step_both(sc, k, oracle_mod)
    assert np.array_equal(g.pairs(), p.pairs())
    cg_, cp_ = g.contacts(), p.contacts()
    by_id, by_pos, miss_p, miss_g = _match(cg_, cp_)
    n = len(by_id) + by_pos + len(miss_p)
    if k > 0:
        assert n >= 3   # bodies land from step ~40 on; 15-35 contacts by step 100
    assert len(miss_p) + len(miss_g) <= max(2, 0.05 * n), (len(by_id), by_pos, miss_p, miss_g)
    # the paired contacts' depths and normals
    G, P = _fresh(cg_), _fresh(cp_)
    for key in by_id:
        assert abs(cg_["pen_depth"][G[key]] - cp_["pen_depth"][P[key]]) <= 2e-4, key
        assert np.abs(cg_["n_local_b1"][G[key]] - cp_["n_local_b1"][P[key]]).max() <= 1e-4, key
    sg, sp = g.state(), p.state()
    dv = np.linalg.norm(sg["vel"] - sp["vel"], axis=1)
    vm = np.linalg.norm(sp["vel"], axis=1)
    stats = f"median {np.median(dv):.2e} max {dv.max():.2e} ties {by_pos} contacts {n}"
    assert np.median(dv) <= 1e-5, stats                                   # m/s
    assert np.mean(dv <= 1e-4 + 1e-3 * vm) >= 0.9, stats
    assert np.abs(sg["com"] - sp["com"]).max() <= 1e-3, stats            # m


def test_union_trajectory_before_contact(oracle_mod):
    """From scratch, 30 steps of free fall and first impacts: positions
    within 1e-4 m of the restatement's."""
    sc = scenes.union_drop(seed=1, n=10)
    g = cg.world()
    scenes.apply(sc, g)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    for _ in range(3):
        g.step(10)
        p.step(10)
        assert np.abs(g.state()["com"] - p.state()["com"]).max() <= 1e-4


def test_union_worlds_batched_equal_alone():
    scs = [scenes.union_drop(seed=s, n=10, terrain=(s == 2)) for s in (0, 1, 2)]
    alone = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        w.step(90)
        alone.append(w.state())
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    b = cg.Batch(ws)
    b.step(90)
    for i, st in enumerate(alone):
        got = b.state(i)
        for k in st:
            assert np.array_equal(got[k], st[k]), (i, k)


def test_union_raycast(oracle_mod):
    """Rays through settled union bodies: each primitive behind its own AABB
    (RigidBody.cpp:185-200); the same body as the restatement for >= 99 % of
    rays, distances within 1e-4 relative."""
    sc = scenes.union_drop(seed=0, n=10)
    g = cg.world()
    scenes.apply(sc, g)
    g.step(90)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    p.set_state(**g.state())
    rng = np.random.default_rng(3)
    o = rng.uniform([-8, 2, -8], [8, 12, 8], size=(2000, 3))
    d = rng.uniform([-6, -1, -6], [6, 4, 6], size=(2000, 3)) - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    hg, hp = g.raycast(o, d), p.raycast(o, d)
    same = hg["body"] == hp["body"]
    assert same.mean() >= 0.99
    hit = same & (hp["body"] > 0)
    assert hit.sum() > 50
    assert np.all(np.abs(hg["dist"][hit] - hp["dist"][hit]) <= 1e-4 * np.maximum(1.0, hp["dist"][hit]))
