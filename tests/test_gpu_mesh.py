"""Static triangle meshes on the device path against the oracle, on a GB300.

Same method as test_gpu_primitives: the device state and contact graph after
k steps are imported into the CPU restatement, both advance one step, and the
results are compared (FP32 device vs FP64 restatement; tolerances written at
each assertion).  A contact with a mesh is identified by its MagicID: the
feature pair (magic_b) and the triangle id carried in the cID (magic_c).

The single-body scenes cover each triangle detector (hull, sphere and
cylinder against a face, an edge and a vertex region), the mesh as the first
or the second body of the pair (flipped manifolds), Gauss-region validity on
a ridge, and the merging of coplanar triangle manifolds followed by the cull.
"""
import math

import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu

MAT = scenes.PILE_MATERIAL
D, F = scenes.DYNAMIC, scenes.FIXED


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


def _fresh_points(c):
    """Contacts detected in the last step keyed by (b1, b2, cID, feature id)."""
    m = c["memory_life"] == 5
    out = {}
    for i in np.nonzero(m)[0]:
        key = (int(c["b1"][i]), int(c["b2"][i]), int(c["magic_c"][i]), int(c["magic_b"][i]))
        out[key] = (c["p_local_b1"][i], c["n_local_b1"][i], float(c["pen_depth"][i]))
    return out


def _match(cg_, cp_, tol=2e-4):
    """Pairs the last step's contacts by MagicID, or else by position within
    `tol` on the same body pair and triangle (the clipping near-tie of a face
    inside a larger face: a vertex on a clipping edge up to rounding comes out
    as the vertex or as an intersection point at the same place).  Returns
    (matched by id, matched by position, unmatched restatement contacts,
    unmatched device contacts)."""
    G, P = _fresh_points(cg_), _fresh_points(cp_)
    by_id = [k for k in P if k in G]
    rest_g = [k for k in G if k not in P]
    used, unmatched = set(), []
    for k in (k for k in P if k not in G):
        near = [j for j in rest_g if j[:3] == k[:3] and j not in used and np.abs(G[j][0] - P[k][0]).max() <= tol]
        if near:
            used.add(near[0])
        else:
            unmatched.append(k)
    return by_id, len(used), unmatched, [j for j in rest_g if j not in used]


def _quat(axis, deg):
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    h = math.radians(deg) / 2
    return (math.cos(h), *(a * math.sin(h)))


def _flat(sc, n=8, spacing=1.0):
    pts, tris = scenes.grid_mesh(np.zeros((n + 1, n + 1)), spacing, (-n * spacing / 2, 0.0, -n * spacing / 2))
    return sc.mesh(pts, tris, MAT)


def _tent(sc):
    """A 4 x 4 grid with a raised centre vertex (a convex peak) and a valley
    row (concave edges)."""
    h = np.zeros((5, 5))
    h[2, 2] = 0.6
    h[:, 4] = 0.4
    pts, tris = scenes.grid_mesh(h, 1.0, (-2.0, 0.0, -2.0))
    return sc.mesh(pts, tris, MAT)


def _scene(name):
    return scenes.Scene(name, scenes.DROP_PARAMS)


def case_sphere_on_face():
    sc = _scene("sphere_on_face")
    _flat(sc)
    sc.sphere((0.0, 0.0, 0.0), 0.5, MAT, D, (0.31, 0.49, 0.17))
    return sc


def case_sphere_on_peak():
    sc = _scene("sphere_on_peak")
    _tent(sc)
    sc.sphere((0.0, 0.0, 0.0), 0.4, MAT, D, (0.05, 0.99, 0.02))
    return sc


def case_sphere_on_ridge_side():
    sc = _scene("sphere_ridge_side")
    _tent(sc)
    sc.sphere((0.0, 0.0, 0.0), 0.3, MAT, D, (0.6, 0.5875, 0.45))
    return sc


def case_sphere_before_mesh():
    # the sphere has the lower id: the manifold is not flipped
    sc = _scene("sphere_first")
    sc.sphere((0.0, 0.0, 0.0), 0.5, MAT, D, (0.31, 0.49, 0.17))
    _flat(sc)
    return sc


def case_box_on_peak():
    sc = _scene("box_on_peak")
    _tent(sc)
    b = sc.box((-0.4, -0.4, -0.4), 0.8, 0.8, 0.8, MAT, D, (0.1, 1.05, 0.05))
    sc.orient(b, _quat((1, 2, 3), 25))
    return sc


def case_box_tilted_edge():
    # a box resting on one edge across a face (rotated off the grid axes so the
    # cull's extremes are unique)
    sc = _scene("box_edge")
    _flat(sc)
    b = sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, MAT, D, (0.2, 0.69, 0.3))
    sc.orient(b, _quat((0.3, 0.0, 1.0), 40))
    return sc


def case_cylinder_tilted():
    sc = _scene("cylinder_tilted")
    _flat(sc)
    b = sc.cylinder((0.0, -0.5, 0.0), 0.4, 1.0, MAT, D, (0.23, 0.62, 0.11))
    sc.orient(b, _quat((0, 0, 1), 30))
    return sc


def case_cylinder_on_peak():
    sc = _scene("cylinder_on_peak")
    _tent(sc)
    b = sc.cylinder((0.0, -0.4, 0.0), 0.3, 0.8, MAT, D, (0.05, 1.06, 0.1))
    sc.orient(b, _quat((1, 0, 1), 35))
    return sc


def case_hull_on_tent():
    sc = _scene("hull_on_tent")
    _tent(sc)
    rng = np.random.default_rng(3)
    pts, faces = scenes.random_hull(rng, 12, 20)
    b = sc.hull(pts, faces, MAT, D, (0.7, 0.6, -0.4))
    sc.orient(b, scenes.random_quat(rng))
    return sc


# one clear minimum-penetration axis and no face lying inside another face
UNIQUE = [case_sphere_on_face, case_sphere_on_peak, case_sphere_on_ridge_side, case_sphere_before_mesh,
          case_box_on_peak, case_box_tilted_edge, case_cylinder_tilted, case_cylinder_on_peak, case_hull_on_tent]
# a sphere balanced on the peak or rolling down the slope bounces: its
# contacts come and go from step to step, so it is compared on the first step
FIRST_STEP_ONLY = {case_sphere_on_peak, case_sphere_on_ridge_side}
UNIQUE_RUNS = [(c, k) for c in UNIQUE for k in ([0] if c in FIRST_STEP_ONLY else [0, 20])]


def case_box_flat():
    # a box face across several coplanar triangles: one manifold per triangle,
    # merged into one and culled to 4 points
    sc = _scene("box_flat")
    _flat(sc)
    b = sc.box((-0.6, -0.5, -0.6), 1.2, 1.0, 1.2, MAT, D, (0.13, 0.49, 0.21))
    sc.orient(b, _quat((0, 1, 0), 17))
    return sc


def case_cylinder_upright():
    sc = _scene("cylinder_upright")
    _flat(sc)
    b = sc.cylinder((0.0, 0.0, 0.0), 0.5, 1.0, MAT, D, (0.21, -0.01, 0.33))
    sc.orient(b, _quat((0, 1, 0), 11))
    return sc


def case_cylinder_lying():
    # the barrel line inside one triangle (a line across three or more
    # coplanar triangles merges into collinear points, where the cull's
    # directions across the line tie exactly)
    sc = _scene("cylinder_lying")
    _flat(sc)
    b = sc.cylinder((0.0, -0.25, 0.0), 0.25, 0.5, MAT, D, (0.3, 0.24, 0.7))
    sc.orient(b, _quat((1, 0, 0.3), 90))
    return sc


FACE = [case_box_flat, case_cylinder_upright, case_cylinder_lying]


def _cases_run(g, p):
    assert np.array_equal(g.pairs(), p.pairs())
    return g.contacts(), p.contacts()


@pytest.mark.parametrize("case,k", UNIQUE_RUNS, ids=[f"{c.__name__[5:]}-{k}" for c, k in UNIQUE_RUNS])
def test_mesh_pair_parity(oracle_mod, case, k):
    g, p = _step_both(case(), k, oracle_mod)
    cg_, cp_ = _cases_run(g, p)
    pg, pp = _fresh_points(cg_), _fresh_points(cp_)
    assert len(pp) > 0
    assert set(pg) == set(pp), (sorted(pg), sorted(pp))     # MagicIDs (feature + triangle) identical
    for key, (x, n, pen) in pp.items():
        xg, ng, peng = pg[key]
        assert np.abs(xg - x).max() <= 2e-4, (key, xg, x)    # m, local contact point on body 1
        assert np.abs(ng - n).max() <= 1e-4, (key, ng, n)    # local normal
        assert abs(peng - pen) <= 2e-4, (key, peng, pen)     # m
    sg, sp = g.state(), p.state()
    assert np.abs(sg["vel"] - sp["vel"]).max() <= 1e-4        # m/s
    assert np.abs(sg["ang_vel"] - sp["ang_vel"]).max() <= 1e-3  # rad/s
    assert np.abs(sg["com"] - sp["com"]).max() <= 1e-5        # m


@pytest.mark.parametrize("case", FACE, ids=lambda f: f.__name__[5:])
@pytest.mark.parametrize("k", [0, 20])
def test_mesh_face_contact_parity(oracle_mod, case, k):
    """Face-on-face contacts on the mesh: every contact has its counterpart by
    MagicID or, at the clipping near-tie, by position."""
    g, p = _step_both(case(), k, oracle_mod)
    cg_, cp_ = _cases_run(g, p)
    by_id, by_pos, miss_p, miss_g = _match(cg_, cp_)
    assert len(by_id) + by_pos > 0
    assert not miss_p and not miss_g, (miss_p, miss_g)
    pg, pp = _fresh_points(cg_), _fresh_points(cp_)
    for key in by_id:
        assert np.abs(pg[key][0] - pp[key][0]).max() <= 2e-4, key   # m
        assert np.abs(pg[key][1] - pp[key][1]).max() <= 1e-3, key   # normal
    sg, sp = g.state(), p.state()
    stats = (f"dv {np.abs(sg['vel'] - sp['vel']).max():.2e} dw {np.abs(sg['ang_vel'] - sp['ang_vel']).max():.2e} "
             f"ties {by_pos}")
    dv_max, dw_max, dx_max = (5e-4, 5e-3, 1e-5) if by_pos == 0 else (1e-2, 5e-2, 2e-4)
    assert np.abs(sg["vel"] - sp["vel"]).max() <= dv_max, stats        # m/s
    assert np.abs(sg["ang_vel"] - sp["ang_vel"]).max() <= dw_max, stats  # rad/s
    assert np.abs(sg["com"] - sp["com"]).max() <= dx_max, stats         # m


def test_mesh_pairs_ignored():
    """Two overlapping meshes produce a candidate pair and no contact
    (fixed-fixed pairs and mesh-mesh pairs are not collided)."""
    sc = _scene("two_meshes")
    _flat(sc)
    _tent(sc)
    sc.sphere((0.0, 0.0, 0.0), 0.3, MAT, D, (3.0, 0.29, 3.0))
    w = cg.world()
    scenes.apply(sc, w)
    w.step(2)
    c = w.contacts()
    assert not np.any((c["b1"] == 1) & (c["b2"] == 2))
    assert np.any(c["b2"] == 3)


def _islands(c, n_bodies, fixed):
    parent = list(range(n_bodies + 1))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x
    for a, b, life in zip(c["b1"].tolist(), c["b2"].tolist(), c["memory_life"].tolist()):
        if life == 5 and a not in fixed and b not in fixed:
            parent[find(a)] = find(b)
    return np.array([find(i) for i in range(n_bodies + 1)])


@pytest.mark.parametrize("k", [100, 140, 200])
def test_terrain_single_step_parity(oracle_mod, k):
    g, p = _step_both(scenes.terrain_drop(seed=1, n_grid=24, n_side=4, n_layers=2), k, oracle_mod)
    assert np.array_equal(g.pairs(), p.pairs())
    cg_, cp_ = g.contacts(), p.contacts()
    by_id, by_pos, miss_p, miss_g = _match(cg_, cp_)
    n = len(by_id) + by_pos + len(miss_p)
    assert n > 0
    assert np.sum(cp_["b1"] == 1) > 0   # terrain contacts
    assert len(miss_p) + len(miss_g) <= 0.05 * n, (len(by_id), by_pos, miss_p, miss_g)
    sg, sp = g.state(), p.state()
    dv = np.linalg.norm(sg["vel"] - sp["vel"], axis=1)
    vm = np.linalg.norm(sp["vel"], axis=1)
    isl = _islands(cp_, len(dv), fixed={1})
    PG, PP = _fresh_points(cg_), _fresh_points(cp_)
    tie_bodies = {b for key in [k_ for k_ in PP if k_ not in PG] for b in key[:2]}
    tie_isl = {isl[b] for b in tie_bodies if b != 1}
    clean = np.array([isl[i + 1] not in tie_isl for i in range(len(dv))])
    stats = (f"clean {clean.sum()} median {np.median(dv[clean]):.2e} max {dv[clean].max():.2e}; "
             f"tie {(~clean).sum()} max {dv[~clean].max() if (~clean).any() else 0:.2e}")
    assert clean.sum() >= len(dv) // 2, stats
    assert np.mean(dv[clean] <= 1e-4 + 1e-3 * vm[clean]) >= 0.95, stats
    assert np.median(dv[clean]) <= 1e-5, stats
    assert dv.max() <= 0.1, stats   # m/s, warm-start loss at a near-tie


def test_terrain_drops_trajectory(oracle_mod):
    """Separate bodies of each kind dropped on the tent mesh and a flat mesh
    region: after 120 steps the device and the restatement agree within
    2e-3 m."""
    sc = _scene("terrain_drops")
    _tent(sc)
    sc.sphere((0.0, 0.0, 0.0), 0.4, MAT, D, (0.3, 2.0, 0.2))
    b = sc.cylinder((0.0, -0.4, 0.0), 0.3, 0.8, MAT, D, (-1.2, 2.0, 1.1))
    sc.orient(b, _quat((1, 0, 1), 35))
    b = sc.box((-0.3, -0.3, -0.3), 0.6, 0.6, 0.6, MAT, D, (1.2, 2.0, -1.1))
    sc.orient(b, _quat((1, 2, 3), 25))
    g = cg.world()
    scenes.apply(sc, g)
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    g.step(120)
    p.step(120)
    err = np.abs(g.state()["com"] - p.state()["com"]).max()
    assert err <= 2e-3, err


def test_terrain_batch_equals_single_worlds():
    """Terrain worlds batched together (their meshes deduplicated in the shape
    pool) step exactly as they do alone."""
    scs = [scenes.terrain_drop(seed=s, n_grid=16, n_side=3, n_layers=1) for s in range(3)]
    singles = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        w.step(60)
        singles.append(w.state())
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    b = cg.Batch(ws)
    b.step(60)
    for i, st in enumerate(singles):
        bs = b.state(i)
        for k in ("com", "quat", "vel", "ang_vel"):
            assert np.array_equal(bs[k], st[k]), (i, k)


def test_terrain_20k_bodies_full_size(oracle_mod):
    """The single large world at full size: 20,000 mixed bodies (40 % boxes,
    20 % spheres, 20 % cylinders, 20 % hulls) dropped on a 256 x 256 value-noise
    heightfield (131,072 triangles, amplitude 8 m), 20 PGS iterations.  After
    150 device steps (every body landed or landing) the state is imported into
    the restatement and both step once: the pair set is identical, contacts
    match as on the small terrain, and bodies in tie-free islands agree to
    FP32 bounds; no body has passed below the terrain."""
    import time
    sc = scenes.terrain_drop(seed=3, n_grid=256, n_side=50, n_layers=8)
    g = cg.world()
    t0 = time.time()
    scenes.apply(sc, g)
    g.step(150)
    dev_s = time.time() - t0
    p = oracle_mod.port_world()
    scenes.apply(sc, p)
    p.set_state(**g.state())
    p.set_contacts(g.contacts())
    g.step(1)
    p.step(1)
    assert np.array_equal(g.pairs(), p.pairs())
    cg_, cp_ = g.contacts(), p.contacts()
    by_id, by_pos, miss_p, miss_g = _match(cg_, cp_)
    n = len(by_id) + by_pos + len(miss_p)
    assert np.sum(cp_["b1"] == 1) > 5000, "terrain contacts"
    assert len(miss_p) + len(miss_g) <= 0.05 * n, (len(by_id), by_pos, len(miss_p), len(miss_g))
    sg, sp = g.state(), p.state()
    dv = np.linalg.norm(sg["vel"] - sp["vel"], axis=1)
    vm = np.linalg.norm(sp["vel"], axis=1)
    isl = _islands(cp_, len(dv), fixed={1})
    PG, PP = _fresh_points(cg_), _fresh_points(cp_)
    tie_bodies = {b for key in [k_ for k_ in PP if k_ not in PG] for b in key[:2]}
    tie_isl = {isl[b] for b in tie_bodies if b != 1}
    clean = np.array([isl[i + 1] not in tie_isl for i in range(len(dv))])
    stats = (f"bodies {len(dv)} clean {clean.sum()} median {np.median(dv[clean]):.2e} max {dv[clean].max():.2e}; "
             f"tie max {dv[~clean].max() if (~clean).any() else 0:.2e}; 151 device steps incl. setup {dev_s:.1f} s")
    assert clean.sum() >= len(dv) // 2, stats
    assert np.mean(dv[clean] <= 1e-4 + 1e-3 * vm[clean]) >= 0.95, stats
    assert np.median(dv[clean]) <= 1e-5, stats
    # nothing fell through: every dynamic body's centre is above the lowest terrain point
    assert np.all(sg["com"][1:, 1] > -8.0 - 1.0), stats
    print(stats)
