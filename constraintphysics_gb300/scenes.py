"""Seeded synthetic scenes for the contact-path workloads.

The reference ships no benchmark scenes beyond its profiling demo
(Demo/src/Demos/PerformanceProfilingScenes.h:218-262: a fixed 500x2x500 base
plate, sleeping disabled, dt 1/60, bodies created through createRigidBody).
These generators build the same kind of scenes with seeded numpy RNGs; a scene
is a list of operations that `apply()` replays on any World (device path or
oracle), so every backend receives bit-identical inputs.

Workloads:
  hull_drop      1,000 convex hulls (8-32 random points on the unit sphere,
                 scale U[0.5,1.5] m, density 1000) on a 10x10x10 grid with 0.1 m
                 jitter and random orientations, dropped on the static plate;
                 friction 0.5, restitution 0, dt 1/60, 10 PGS iterations, one
                 substep.
  mixed_drop     mixed bodies (40% boxes with sides U[0.5,1.5] m, 20% spheres
                 r U[0.3,0.8], 20% cylinders r U[0.3,0.6] h U[0.5,1.5], 20%
                 random hulls of 12-32 points) on a jittered grid with random
                 orientations, dropped on the static plate; 20 PGS iterations.
  chain_world    one articulated chain: L unit boxes (L in [lmin, lmax]) with
                 link masses log-uniform in [0.1, 100] kg, pinned to a fixed box
                 by a ball-socket and joined alternately by ball-sockets and
                 hinges with random axes, starting horizontal and swinging
                 through fixed spheres (r U[0.5,1.5]) placed in its swing
                 volume; engine defaults (8 substeps, PGS (4,1,1)).
  terrain_drop   mixed bodies as in mixed_drop falling onto a fixed triangle-
                 mesh terrain: an n x n heightfield at 1 m spacing triangulated
                 as generateGridMeshInput does (Geometry.cpp:589-611), heights
                 summed from 4 octaves of seeded value noise (periods 32, 16, 8,
                 4 m, amplitudes halving) scaled to 8 m; 20 PGS iterations.
  batched_world  one world of the 4,096-world batch: floor(exp(U[ln 8, ln 512]))
                 bodies, either a box pyramid (base 4-16) or a hull pile built as
                 in hull_drop, each world with its own plate.
"""
import math

import numpy as np

DYNAMIC, FIXED, KINEMATIC = 0, 1, 2

PILE_MATERIAL = {"density": 1000.0, "restitution": 0.0, "kinetic_friction": 0.5, "static_friction": 0.5}

# engine settings shared by the hull_drop and batched workloads
DROP_PARAMS = dict(step_time=1.0 / 60.0, substeps=1, pgs=(10, 1, 1), sleeping=False)


def unit_sphere_points(rng, n):
    g = rng.normal(size=(n, 3))
    return g / np.linalg.norm(g, axis=1, keepdims=True)


def convex_hull(points):
    """Vertices and triangular faces of the convex hull of `points`."""
    from scipy.spatial import ConvexHull
    h = ConvexHull(points)
    verts = np.asarray(h.vertices)
    remap = -np.ones(len(points), dtype=np.int64)
    remap[verts] = np.arange(len(verts))
    faces = [[int(remap[i]) for i in s] for s in h.simplices]
    return np.ascontiguousarray(points[verts]), faces


def random_quat(rng):
    q = rng.normal(size=4)
    return q / np.linalg.norm(q)


def random_hull(rng, nmin=8, nmax=32):
    n = int(rng.integers(nmin, nmax + 1))
    pts = unit_sphere_points(rng, n) * rng.uniform(0.5, 1.5)
    return convex_hull(pts)


class Scene:
    """Replayable list of world-building operations."""

    def __init__(self, name, params):
        self.name = name
        self.params = dict(params)
        self.ops = []
        self.n_bodies = 0
        self.n_constraints = 0

    def _body(self, op):
        self.ops.append(op)
        self.n_bodies += 1
        return self.n_bodies  # ids start at 1

    def _constraint(self, op):
        """Joints and springs: the handle is the scene's constraint index
        (apply() maps it to the world's constraint id)."""
        self.ops.append(op)
        self.n_constraints += 1
        return self.n_constraints - 1

    def hull(self, points, faces, material, movement, pos):
        return self._body(("hull", points, faces, material, movement, tuple(pos)))

    def box(self, corner, dx, dy, dz, material, movement, pos=(0, 0, 0)):
        return self._body(("box", tuple(corner), dx, dy, dz, material, movement, tuple(pos)))

    def sphere(self, center, r, material, movement, pos=(0, 0, 0)):
        return self._body(("sphere", tuple(center), r, material, movement, tuple(pos)))

    def cylinder(self, base, r, h, material, movement, pos=(0, 0, 0)):
        return self._body(("cylinder", tuple(base), r, h, material, movement, tuple(pos)))

    def union(self, prims, movement, pos=(0, 0, 0)):
        """A multi-primitive body (see World.add_union for the primitive tuples)."""
        return self._body(("union", tuple(prims), movement, tuple(pos)))

    def capsule(self, bot, r, h, material, movement, pos=(0, 0, 0)):
        return self._body(("capsule", tuple(bot), r, h, material, movement, tuple(pos)))

    def mesh(self, points, tris, material):
        return self._body(("mesh", np.asarray(points, dtype=np.float64), np.asarray(tris, dtype=np.int32), material))

    def mass(self, bid, m):
        self.ops.append(("mass", bid, float(m)))

    def ball_socket(self, b1, b2, a1, a2, strength=15000.0):
        return self._constraint(("ball", b1, b2, tuple(a1), tuple(a2), float(strength)))

    def distance(self, b1, b2, a1, a2, target=-1.0, strength=15000.0):
        return self._constraint(("distance", b1, b2, tuple(a1), tuple(a2), float(target), float(strength)))

    def weld(self, b1, b2, a1, a2, pos_strength=15000.0, rot_strength=15000.0):
        return self._constraint(("weld", b1, b2, tuple(a1), tuple(a2), float(pos_strength), float(rot_strength)))

    def twist_limit(self, b1, b2, ax1, ax2, min_angle, max_angle, rot_strength=15000.0):
        return self._constraint(("twist_limit", b1, b2, tuple(ax1), tuple(ax2), float(min_angle), float(max_angle),
                         float(rot_strength)))

    def cone_limit(self, b1, b2, ax1, ax2, max_angle, rot_strength=15000.0):
        return self._constraint(("cone_limit", b1, b2, tuple(ax1), tuple(ax2), float(max_angle), float(rot_strength)))

    def spring(self, b1, b2, a1, a2, damping, stiffness, resting_length=-1.0):
        return self._constraint(("spring", b1, b2, tuple(a1), tuple(a2), float(damping), float(stiffness),
                         float(resting_length)))

    def slider(self, b1, b2, a1, a2, ax1, ax2, pos_strength=15000.0, rot_strength=15000.0):
        return self._constraint(("slider", b1, b2, tuple(a1), tuple(a2), tuple(ax1), tuple(ax2), float(pos_strength),
                         float(rot_strength)))

    def sliding_hinge(self, b1, b2, a1, a2, ax1, ax2, pos_strength=15000.0, rot_strength=15000.0):
        return self._constraint(("sliding_hinge", b1, b2, tuple(a1), tuple(a2), tuple(ax1), tuple(ax2), float(pos_strength),
                         float(rot_strength)))

    def hinge(self, b1, b2, a1, a2, ax1, ax2, pos_strength=15000.0, rot_strength=15000.0):
        return self._constraint(("hinge", b1, b2, tuple(a1), tuple(a2), tuple(ax1), tuple(ax2), float(pos_strength),
                         float(rot_strength)))

    def motor(self, base, min_angle=-np.inf, max_angle=np.inf):
        """A motor on the hinge or sliding hinge with handle `base`."""
        return self._constraint(("motor", base, float(min_angle), float(max_angle)))

    def piston(self, base, min_pos=-np.inf, max_pos=np.inf):
        """A piston on the slider or sliding hinge with handle `base`."""
        return self._constraint(("piston", base, float(min_pos), float(max_pos)))

    def set_motor(self, handle, mode, max_torque=0.0, target=0.0):
        self.ops.append(("set_motor", handle, int(mode), float(max_torque), float(target)))

    def set_piston(self, handle, mode, max_force=0.0, target=0.0):
        self.ops.append(("set_piston", handle, int(mode), float(max_force), float(target)))

    def orient(self, bid, q):
        self.ops.append(("orient", bid, tuple(q)))

    def velocity(self, bid, v):
        self.ops.append(("vel", bid, tuple(v)))

    def ang_velocity(self, bid, w):
        self.ops.append(("angvel", bid, tuple(w)))

    def movements(self):
        """Movement type of each body, in id order."""
        slot = {"hull": 4, "box": 6, "sphere": 4, "cylinder": 5, "capsule": 5, "union": 2}
        return [FIXED if op[0] == "mesh" else op[slot[op[0]]] for op in self.ops if op[0] in slot or op[0] == "mesh"]


def apply(scene, world):
    """Replay `scene` on a World; returns the list of created body ids.  The
    world's ids of the scene's joints and springs (in handle order) are left
    in `world.constraint_ids`."""
    world.set_params(**scene.params)
    ids = []
    cids = []
    for op in scene.ops:
        kind = op[0]
        if kind == "hull":
            ids.append(world.add_hull(op[1], op[2], op[3], op[4], op[5]))
        elif kind == "box":
            ids.append(world.add_box(op[1], op[2], op[3], op[4], op[5], op[6], op[7]))
        elif kind == "sphere":
            ids.append(world.add_sphere(op[1], op[2], op[3], op[4], op[5]))
        elif kind == "cylinder":
            ids.append(world.add_cylinder(op[1], op[2], op[3], op[4], op[5], op[6]))
        elif kind == "capsule":
            ids.append(world.add_capsule(op[1], op[2], op[3], op[4], op[5], op[6]))
        elif kind == "union":
            ids.append(world.add_union(list(op[1]), op[2], op[3]))
        elif kind == "mesh":
            ids.append(world.add_mesh(op[1], op[2], op[3], True))
        elif kind == "orient":
            world.set_orientation(op[1], op[2])
        elif kind == "vel":
            world.set_velocity(op[1], op[2])
        elif kind == "angvel":
            world.set_ang_velocity(op[1], op[2])
        elif kind == "mass":
            world.set_mass(op[1], op[2])
        elif kind == "distance":
            cids.append(world.add_distance(op[1], op[2], op[3], op[4], op[5], op[6]))
        elif kind in ("slider", "sliding_hinge", "spring", "cone_limit", "twist_limit"):
            cids.append(getattr(world, "add_" + kind)(*op[1:]))
        elif kind == "weld":
            cids.append(world.add_weld(op[1], op[2], op[3], op[4], op[5], op[6]))
        elif kind == "ball":
            cids.append(world.add_ball_socket(op[1], op[2], op[3], op[4], op[5]))
        elif kind == "hinge":
            cids.append(world.add_hinge(op[1], op[2], op[3], op[4], op[5], op[6], op[7], op[8]))
        elif kind == "motor":
            cids.append(world.add_motor(cids[op[1]], op[2], op[3]))
        elif kind == "piston":
            cids.append(world.add_piston(cids[op[1]], op[2], op[3]))
        elif kind == "set_motor":
            world.set_motor(cids[op[1]], op[2], op[3], op[4])
        elif kind == "set_piston":
            world.set_piston(cids[op[1]], op[2], op[3], op[4])
        else:
            raise ValueError(kind)
    world.constraint_ids = cids
    return ids


def _plate(scene, material=PILE_MATERIAL):
    # PerformanceProfilingScenes.h:233-237: box((-s/2, -2, -s/2), s, 2, s), FIXED
    s = 500.0
    return scene.box((-s / 2, -2.0, -s / 2), s, 2.0, s, material, FIXED)


def hull_drop(seed=0, n_side=10, spacing=3.2, jitter=0.1, base_y=2.0):
    """1,000 random hulls (n_side^3) dropped on the static plate."""
    rng = np.random.default_rng(seed)
    sc = Scene(f"hull_drop_{n_side}^3_seed{seed}", DROP_PARAMS)
    _plate(sc)
    off = (n_side - 1) * spacing / 2.0
    for i in range(n_side):
        for j in range(n_side):
            for k in range(n_side):
                pts, faces = random_hull(rng)
                pos = np.array([i * spacing - off, base_y + j * spacing, k * spacing - off])
                pos += rng.uniform(-jitter, jitter, size=3)
                bid = sc.hull(pts, faces, PILE_MATERIAL, DYNAMIC, pos)
                sc.orient(bid, random_quat(rng))
    return sc


MIXED_PARAMS = dict(step_time=1.0 / 60.0, substeps=1, pgs=(20, 1, 1), sleeping=False)


def mixed_drop(seed=0, n_side=6, spacing=3.2, jitter=0.1, base_y=2.0, n_layers=None):
    """Mixed boxes, spheres, cylinders and hulls (n_side^2 x n_layers) dropped
    on the static plate."""
    rng = np.random.default_rng(seed)
    n_layers = n_side if n_layers is None else n_layers
    sc = Scene(f"mixed_drop_{n_side}x{n_side}x{n_layers}_seed{seed}", MIXED_PARAMS)
    _plate(sc)
    off = (n_side - 1) * spacing / 2.0
    for j in range(n_layers):
        for i in range(n_side):
            for k in range(n_side):
                pos = np.array([i * spacing - off, base_y + j * spacing, k * spacing - off])
                pos += rng.uniform(-jitter, jitter, size=3)
                u = rng.random()
                if u < 0.4:
                    d = rng.uniform(0.5, 1.5, size=3)
                    bid = sc.box((-d[0] / 2, -d[1] / 2, -d[2] / 2), d[0], d[1], d[2], PILE_MATERIAL, DYNAMIC, pos)
                elif u < 0.6:
                    bid = sc.sphere((0.0, 0.0, 0.0), rng.uniform(0.3, 0.8), PILE_MATERIAL, DYNAMIC, pos)
                elif u < 0.8:
                    r, h = rng.uniform(0.3, 0.6), rng.uniform(0.5, 1.5)
                    bid = sc.cylinder((0.0, -h / 2, 0.0), r, h, PILE_MATERIAL, DYNAMIC, pos)
                else:
                    pts, faces = random_hull(rng, 12, 32)
                    bid = sc.hull(pts, faces, PILE_MATERIAL, DYNAMIC, pos)
                sc.orient(bid, random_quat(rng))
    return sc


CHAIN_PARAMS = dict(step_time=1.0 / 60.0, substeps=8, pgs=(4, 1, 1), sleeping=False)


def chain_world(rng, lmin=16, lmax=64, n_spheres=50, pitch=1.1):
    """One articulated chain (see the module docstring)."""
    n = int(rng.integers(lmin, lmax + 1))
    sc = Scene(f"chain_{n}", CHAIN_PARAMS)
    anchor = sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, PILE_MATERIAL, FIXED)
    links = []
    for i in range(n):
        b = sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, PILE_MATERIAL, DYNAMIC, ((i + 1) * pitch, 0.0, 0.0))
        sc.mass(b, float(math.exp(rng.uniform(math.log(0.1), math.log(100.0)))))
        links.append(b)
    prev = anchor
    for i, b in enumerate(links):
        # the joint sits halfway between the two bodies' centres; anchors are
        # given in each body's own model coordinates
        x = (i + 0.5) * pitch
        a_prev = (x - (i * pitch if i > 0 else 0.0), 0.0, 0.0)
        a_this = (x - (i + 1) * pitch, 0.0, 0.0)
        if i % 2 == 0:
            sc.ball_socket(prev, b, a_prev, a_this)
        else:
            axis = unit_sphere_points(rng, 1)[0]
            sc.hinge(prev, b, a_prev, a_this, tuple(axis), tuple(axis))
        prev = b
    reach = (n + 1) * pitch
    placed = 0
    while placed < n_spheres:
        r = rng.uniform(0.5, 1.5)
        c = np.array([rng.uniform(-reach, reach), rng.uniform(-reach, -1.0), rng.uniform(-2.0, 2.0)])
        if c[1] + r > -0.8:   # clear of the chain's starting line
            continue
        sc.sphere(tuple(c), r, PILE_MATERIAL, FIXED)
        placed += 1
    return sc


def heavy_chain():
    """The reference's "High mass Ratio Chain" scenario
    (Demo/src/Demos/Tests/HolonomicBlockSolvingTests.h:8-91): 35 links of
    0.31 x 1 x 0.31 (density 2) hanging from a fixed box by ball-sockets, a
    radius-7 ball (density 2) on the end moving at 25 m/s; 24 substeps, PGS
    (1, 1, 1).  The reference requires the ball to stay within 65 m of the
    fixture for 30 s.  Sleeping is disabled here (the reference scenario leaves
    it on; a swinging chain does not sleep)."""
    sc = Scene("heavy_chain", dict(step_time=1.0 / 60.0, substeps=24, pgs=(1, 1, 1), sleeping=False))
    default = {"density": 1.0, "restitution": 0.3, "kinetic_friction": 0.6, "static_friction": 1.1}
    heavy = dict(default, density=2.0)
    w, h = 0.31, 1.0
    anchor = sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, default, FIXED)
    prev = anchor
    for i in range(35):
        pos = (0.0, -i * h, 0.0)
        link = sc.box((-w / 2.0, -i * h, -w / 2.0), w, -h, w, heavy, DYNAMIC)
        sc.ball_socket(prev, link, pos, pos)
        prev = link
    final = (0.0, -35 * h, 0.0)
    ball = sc.sphere((0.0, -35 * h - 7.0, 0.0), 7.0, heavy, DYNAMIC)
    sc.velocity(ball, (25.0, 0.0, 0.0))
    sc.ball_socket(ball, prev, final, final)
    return sc


def value_noise(rng, n, periods=(32, 16, 8, 4), amplitude=8.0):
    """(n+1) x (n+1) heights: octaves of lattice value noise (uniform lattice
    values, smoothstep interpolation), weights halving per octave, the sum
    scaled so its largest magnitude is `amplitude`."""
    xs = np.arange(n + 1, dtype=np.float64)
    total = np.zeros((n + 1, n + 1))
    for k, per in enumerate(periods):
        m = int(np.ceil(n / per)) + 2
        lat = rng.uniform(-1.0, 1.0, size=(m, m))
        f = xs / per
        i0 = np.floor(f).astype(int)
        t = f - i0
        t = t * t * (3 - 2 * t)
        a = lat[i0][:, i0]
        b = lat[i0 + 1][:, i0]
        c = lat[i0][:, i0 + 1]
        d = lat[i0 + 1][:, i0 + 1]
        ti, tj = t[:, None], t[None, :]
        total += 0.5 ** k * (a * (1 - ti) * (1 - tj) + b * ti * (1 - tj) + c * (1 - ti) * tj + d * ti * tj)
    return total * (amplitude / max(np.abs(total).max(), 1e-12))


def grid_mesh(heights, spacing=1.0, origin=(0.0, 0.0, 0.0)):
    """Points and triangles of an n x n grid, indexed and wound as
    generateGridMeshInput (Geometry.cpp:589-611) does; point (i, j) sits at
    origin + (spacing i, height, spacing j)."""
    n = heights.shape[0] - 1
    pts = np.zeros(((n + 1) * (n + 1), 3))
    for j in range(n + 1):
        for i in range(n + 1):
            pts[i + (n + 1) * j] = (origin[0] + spacing * i, origin[1] + heights[i, j], origin[2] + spacing * j)
    tris = np.zeros((2 * n * n, 3), dtype=np.int64)
    for j in range(1, n + 1):
        for i in range(1, n + 1):
            tile = i - 1 + n * (j - 1)
            i1 = i - 1 + (n + 1) * (j - 1)
            i2 = i + (n + 1) * (j - 1)
            i3 = i + (n + 1) * j
            i4 = i - 1 + (n + 1) * j
            tris[2 * tile] = (i3, i2, i1)
            tris[2 * tile + 1] = (i4, i3, i1)
    return pts, tris


def terrain_drop(seed=0, n_grid=32, n_side=6, n_layers=2, spacing=3.2, clearance=3.0):
    """Mixed bodies (see mixed_drop) dropped on a value-noise terrain mesh."""
    rng = np.random.default_rng(seed)
    h = value_noise(rng, n_grid)
    pts, tris = grid_mesh(h, 1.0, (-n_grid / 2.0, 0.0, -n_grid / 2.0))
    sc = Scene(f"terrain_drop_{n_grid}_{n_side}x{n_side}x{n_layers}_seed{seed}", MIXED_PARAMS)
    sc.mesh(pts, tris, PILE_MATERIAL)
    top = float(h.max()) + clearance
    off = (n_side - 1) * spacing / 2.0
    for j in range(n_layers):
        for i in range(n_side):
            for k in range(n_side):
                pos = np.array([i * spacing - off, top + j * spacing, k * spacing - off])
                pos += rng.uniform(-0.1, 0.1, size=3)
                u = rng.random()
                if u < 0.4:
                    d = rng.uniform(0.5, 1.5, size=3)
                    bid = sc.box((-d[0] / 2, -d[1] / 2, -d[2] / 2), d[0], d[1], d[2], PILE_MATERIAL, DYNAMIC, pos)
                elif u < 0.6:
                    bid = sc.sphere((0.0, 0.0, 0.0), rng.uniform(0.3, 0.8), PILE_MATERIAL, DYNAMIC, pos)
                elif u < 0.8:
                    r, hh = rng.uniform(0.3, 0.6), rng.uniform(0.5, 1.5)
                    bid = sc.cylinder((0.0, -hh / 2, 0.0), r, hh, PILE_MATERIAL, DYNAMIC, pos)
                else:
                    p_, f_ = random_hull(rng, 12, 32)
                    bid = sc.hull(p_, f_, PILE_MATERIAL, DYNAMIC, pos)
                sc.orient(bid, random_quat(rng))
    return sc


def capsule_drop(seed=0, n_side=4, n_layers=2, terrain=False, n_grid=16, spacing=3.2):
    """Capsules (about half the bodies, r U[0.25,0.5], drum height
    U[0.3,1.2]) mixed with boxes, spheres, cylinders and hulls, dropped on the
    plate or on a value-noise terrain mesh: every capsule pair kind occurs."""
    rng = np.random.default_rng(seed)
    sc = Scene(f"capsule_drop_{'terrain' if terrain else 'plate'}_{n_side}x{n_side}x{n_layers}_seed{seed}", MIXED_PARAMS)
    if terrain:
        hts = value_noise(rng, n_grid)
        pts, tris = grid_mesh(hts, 1.0, (-n_grid / 2.0, 0.0, -n_grid / 2.0))
        sc.mesh(pts, tris, PILE_MATERIAL)
        base = float(hts.max()) + 3.0
    else:
        _plate(sc)
        base = 2.0
    off = (n_side - 1) * spacing / 2.0
    for j in range(n_layers):
        for i in range(n_side):
            for k in range(n_side):
                pos = np.array([i * spacing - off, base + j * spacing, k * spacing - off])
                pos += rng.uniform(-0.1, 0.1, size=3)
                u = rng.random()
                if u < 0.5:
                    r, hh = rng.uniform(0.25, 0.5), rng.uniform(0.3, 1.2)
                    bid = sc.capsule((0.0, -hh / 2, 0.0), r, hh, PILE_MATERIAL, DYNAMIC, pos)
                elif u < 0.625:
                    d = rng.uniform(0.5, 1.5, size=3)
                    bid = sc.box((-d[0] / 2, -d[1] / 2, -d[2] / 2), d[0], d[1], d[2], PILE_MATERIAL, DYNAMIC, pos)
                elif u < 0.75:
                    bid = sc.sphere((0.0, 0.0, 0.0), rng.uniform(0.3, 0.8), PILE_MATERIAL, DYNAMIC, pos)
                elif u < 0.875:
                    r, hh = rng.uniform(0.3, 0.6), rng.uniform(0.5, 1.5)
                    bid = sc.cylinder((0.0, -hh / 2, 0.0), r, hh, PILE_MATERIAL, DYNAMIC, pos)
                else:
                    p_, f_ = random_hull(rng, 12, 32)
                    bid = sc.hull(p_, f_, PILE_MATERIAL, DYNAMIC, pos)
                sc.orient(bid, random_quat(rng))
    return sc


def kinematic_push(seed=0):
    """Kinematic bodies (RigidBody::KINEMATIC: infinite mass, moved by their
    own velocity) among dynamic ones: a long box sliding at 1 m/s into a row
    of stacked boxes, and a wide cylinder spinning about +y at 1.5 rad/s
    under a sphere and a capsule."""
    rng = np.random.default_rng(seed)
    sc = Scene(f"kinematic_push_seed{seed}", DROP_PARAMS)
    sc.box((-20.0, -1.0, -20.0), 40.0, 1.0, 40.0, PILE_MATERIAL, FIXED)
    pusher = sc.box((-0.5, -0.5, -2.0), 1.0, 1.0, 4.0, PILE_MATERIAL, KINEMATIC, (-4.0, 0.5, 0.0))
    sc.velocity(pusher, (1.0, 0.0, 0.0))
    spin = sc.cylinder((0.0, -0.25, 0.0), 2.0, 0.5, PILE_MATERIAL, KINEMATIC, (5.0, 0.25, 0.0))
    sc.ang_velocity(spin, (0.0, 1.5, 0.0))
    for i in range(6):
        pos = np.array([-1.0 + 0.9 * (i % 3), 0.4 + 0.85 * (i // 3), 0.3 * (i % 2)]) + rng.uniform(-0.02, 0.02, 3)
        sc.box((-0.4, -0.4, -0.4), 0.8, 0.8, 0.8, PILE_MATERIAL, DYNAMIC, pos)
    sc.sphere((0.0, 0.0, 0.0), 0.4, PILE_MATERIAL, DYNAMIC, (5.5, 1.0, 0.5))
    sc.capsule((0.0, -0.4, 0.0), 0.25, 0.8, PILE_MATERIAL, DYNAMIC, (4.2, 1.2, -0.6))
    return sc


def union_drop(seed=0, n=8, terrain=False):
    """Multi-primitive bodies (ConvexUnionGeometry::merge): L-shapes of two
    boxes, dumbbells (a capsule and two spheres), small tables (a box top on
    four cylinder legs) and hull-sphere pairs, dropped with single boxes on
    the plate or on a 16 x 16 value-noise terrain mesh."""
    rng = np.random.default_rng(seed)
    sc = Scene(f"union_drop_{n}_{'terrain' if terrain else 'plate'}_seed{seed}", MIXED_PARAMS)
    if terrain:
        hts = value_noise(rng, 16)
        pts, tris = grid_mesh(hts, 1.0, (-8.0, 0.0, -8.0))
        sc.mesh(pts, tris, PILE_MATERIAL)
    else:
        _plate(sc)
    lift = float(hts.max()) + 1.0 if terrain else 0.0
    m = PILE_MATERIAL
    for i in range(n):
        pos = np.array([(i % 4) * 3.2 - 4.8, 2.0 + lift + 2.5 * (i // 4), (i % 3) * 1.5 - 1.5]) + rng.uniform(-0.1, 0.1, 3)
        kind = i % 5
        if kind == 0:
            prims = [("box", (-0.5, -0.25, -0.25), 1.0, 0.5, 0.5, m), ("box", (0.25, 0.25, -0.25), 0.5, 1.0, 0.5, m)]
        elif kind == 1:
            prims = [("capsule", (0.0, -0.6, 0.0), 0.15, 1.2, m), ("sphere", (0.0, 0.75, 0.0), 0.35, m),
                     ("sphere", (0.0, -0.75, 0.0), 0.35, m)]
        elif kind == 2:
            prims = [("box", (-0.8, 0.4, -0.6), 1.6, 0.2, 1.2, m)]
            prims += [("cylinder", (x, -0.4, z), 0.1, 0.8, m) for x in (-0.65, 0.65) for z in (-0.45, 0.45)]
        elif kind == 3:
            pts, faces = random_hull(rng, 10, 20)
            prims = [("hull", pts * 0.8, faces, m), ("sphere", (0.0, 0.9, 0.0), 0.4, m)]
        else:
            d = rng.uniform(0.6, 1.2, size=3)
            sc.box((-d[0] / 2, -d[1] / 2, -d[2] / 2), d[0], d[1], d[2], m, DYNAMIC, pos)
            continue
        bid = sc.union(prims, DYNAMIC, pos)
        sc.orient(bid, random_quat(rng))
    return sc


class HullPool:
    """A pool of unit-scale random hulls reused (with a per-body scale) by the
    batched workload, so that generating 10^5 hulls does not need 10^5 Qhull
    runs."""

    def __init__(self, seed, size=512, nmin=8, nmax=32):
        rng = np.random.default_rng(seed + 7919)
        self.shapes = []
        for _ in range(size):
            n = int(rng.integers(nmin, nmax + 1))
            self.shapes.append(convex_hull(unit_sphere_points(rng, n)))

    def draw(self, rng):
        pts, faces = self.shapes[int(rng.integers(len(self.shapes)))]
        return pts * rng.uniform(0.5, 1.5), faces


# Vertical placement of the pyramid boxes: the lowest layer starts PYR_LIFT
# above the plate and the layers PYR_PITCH apart (box height 1 m).  The values
# keep every first touch away from a step boundary: a body falling from rest
# under g = 6 m/s^2 with dt = 1/60 s covers 0.00167, 0.005, 0.01, ... m after
# 1, 2, 3, ... steps, so a gap of exactly 0.005 m (the earlier 0.005 m lift
# and 1.01 m pitch) made every layer touch down with zero depth at step 2,
# and whether the contact exists that step was decided by rounding (in FP64
# as much as in FP32), shifting whole pyramids by one step of fall.
PYR_LIFT = 0.0043
PYR_PITCH = 1.0087


def batched_world(rng, pool, nmin=8, nmax=512, gap=0.05):
    """One world of the batched workload (log-uniform body count)."""
    n = int(math.floor(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
    kind = "pyramid" if rng.random() < 0.5 else "pile"
    sc = Scene(f"{kind}_{n}", DROP_PARAMS)
    _plate(sc)
    if kind == "pyramid":
        base = int(rng.integers(4, 17))
        pitch = 1.0 + gap
        placed, pyr = 0, 0
        while placed < n:  # extra pyramids go beside the first when n exceeds one
            shift = pyr * (base * pitch + 4.0)
            for layer in range(base):
                side = base - layer
                off = (side - 1) * pitch / 2.0
                for x in range(side):
                    for z in range(side):
                        if placed >= n:
                            break
                        corner = (x * pitch - off + shift, layer * PYR_PITCH + PYR_LIFT, z * pitch - off)
                        sc.box((0.0, 0.0, 0.0), 1.0, 1.0, 1.0, PILE_MATERIAL, DYNAMIC, corner)
                        placed += 1
            pyr += 1
    else:
        side = max(1, int(math.ceil(n ** (1.0 / 3.0))))
        spacing = 3.2
        off = (side - 1) * spacing / 2.0
        placed = 0
        j = 0
        while placed < n:
            for i in range(side):
                for k in range(side):
                    if placed >= n:
                        break
                    pts, faces = pool.draw(rng)
                    pos = np.array([i * spacing - off, 2.0 + j * spacing, k * spacing - off])
                    pos += rng.uniform(-0.1, 0.1, size=3)
                    bid = sc.hull(pts, faces, PILE_MATERIAL, DYNAMIC, pos)
                    sc.orient(bid, random_quat(rng))
                    placed += 1
            j += 1
    return sc


def batched_worlds(seed=0, n_worlds=4096, nmin=8, nmax=512):
    rng = np.random.default_rng(seed)
    pool = HullPool(seed)
    return [batched_world(rng, pool, nmin, nmax) for _ in range(n_worlds)]


# ---- joint scenes: one kind of joint (or spring) each, engine settings of 4
# substeps and PGS (10, 1, holo); used by the restatement's pinning tests and
# the device's parity tests
JOINT_PARAMS = dict(step_time=1.0 / 60.0, substeps=4, pgs=(10, 1, 1), sleeping=False)
_TURN_Z10 = (0.9961946980917455, 0.0, 0.0, 0.08715574274765817)   # 10 degrees about z


def distance_chain(mixed=False):
    """A hanging chain of spheres linked by distance joints (or alternating
    distance and ball-socket joints: one holonomic system), hit by a box."""
    M = PILE_MATERIAL
    sc = Scene("distance_chain", JOINT_PARAMS)
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, FIXED)
    prev = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, FIXED, (0.0, 8.0, 0.0))
    for i in range(6):
        b = sc.sphere((0, 0, 0), 0.25, M, DYNAMIC, (0.9 * (i + 1), 8.0, 0.0))
        if mixed and i % 2 == 1:
            sc.ball_socket(prev, b, (0.45, 0, 0), (-0.45, 0, 0))
        else:
            sc.distance(prev, b, (0.25, 0, 0), (-0.25, 0, 0))
        prev = b
    # dropped from 0.513 m: a free fall covers g dt^2 n (n + 1) / 2 in n
    # steps, and 0.5 m (n = 24) would touch down exactly at a step boundary
    sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, M, DYNAMIC, (2.0, 1.013, 0.3))
    return sc


def weld_cantilever(mixed=False):
    """A cantilever of boxes welded to a fixed post, one link turned so the
    orientation correction acts (or every other weld a hinge: one holonomic
    system of 6- and 5-dof blocks), hit by a falling box."""
    M = PILE_MATERIAL
    sc = Scene("weld_cantilever", JOINT_PARAMS)
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, FIXED)
    prev = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, FIXED, (0.0, 4.0, 0.0))
    for i in range(5):
        b = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, DYNAMIC, (0.6 * (i + 1), 4.0, 0.0))
        if i == 2:
            sc.orient(b, _TURN_Z10)
        if mixed and i % 2 == 1:
            sc.hinge(prev, b, (0.3, 0, 0), (-0.3, 0, 0), (0, 0, 1), (0, 0, 1))
        else:
            sc.weld(prev, b, (0.3, 0, 0), (-0.3, 0, 0))
        prev = b
    sc.box((-0.3, -0.3, -0.3), 0.6, 0.6, 0.6, M, DYNAMIC, (2.4, 6.0, 0.1))
    return sc


def slider_chain(kinds=("slider",) * 4):
    """Boxes hung from a fixed post by slider / sliding-hinge (/ hinge) joints
    on tilted axes, one link turned, hit by a falling box."""
    M = PILE_MATERIAL
    sc = Scene("slider_chain", JOINT_PARAMS)
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, FIXED)
    prev = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, FIXED, (0.0, 4.0, 0.0))
    axes = [(1.0, -0.4, 0.2), (0.3, -1.0, 0.0), (1.0, 0.2, -0.5), (0.0, -1.0, 0.4)]
    for i, kind in enumerate(kinds):
        b = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, DYNAMIC, (0.6 * (i + 1), 4.0, 0.0))
        if i == 1:
            sc.orient(b, _TURN_Z10)
        getattr(sc, kind)(prev, b, (0.3, 0, 0), (-0.3, 0, 0), axes[i], axes[i])
        prev = b
    sc.box((-0.3, -0.3, -0.3), 0.6, 0.6, 0.6, M, DYNAMIC, (1.8, 6.0, 0.1))
    return sc


def motor_chain(mode=1, limits=False):
    """Boxes hung from a fixed post by hinges on horizontal axes, each hinge
    driven by a motor: mode 1 constant torque, 2 target velocity, 3 target
    position (modes of World.set_motor); with `limits` the motors also limit
    the hinge angle to [-0.6, 0.9] rad."""
    M = PILE_MATERIAL
    sc = Scene(f"motor_chain_{mode}{'_lim' if limits else ''}", JOINT_PARAMS)
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, FIXED)
    prev = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, FIXED, (0.0, 4.0, 0.0))
    axes = [(0.0, 0.0, 1.0), (0.0, 0.3, 1.0), (0.2, 0.0, 1.0)]
    for i in range(3):
        b = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, DYNAMIC, (0.7 * (i + 1), 4.0, 0.0))
        h = sc.hinge(prev, b, (0.35, 0, 0), (-0.35, 0, 0), axes[i], axes[i])
        m = sc.motor(h, -0.6, 0.9) if limits else sc.motor(h)
        if mode == 1:
            sc.set_motor(m, 1, 40.0 - 15.0 * i)
        elif mode == 2:
            sc.set_motor(m, 2, 60.0, 1.5 - 1.0 * i)
        else:
            sc.set_motor(m, 3, 80.0, 0.5 + 0.3 * i)
        prev = b
    return sc


def piston_chain(mode=2, limits=True):
    """Boxes on slider joints along tilted axes from a fixed post, each slider
    driven by a piston: mode 1 constant force, 2 target velocity, 3 target
    position; with `limits` the slide is limited to [-0.2, 0.5] m."""
    M = PILE_MATERIAL
    sc = Scene(f"piston_chain_{mode}{'_lim' if limits else ''}", JOINT_PARAMS)
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, FIXED)
    prev = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, FIXED, (0.0, 4.0, 0.0))
    axes = [(1.0, -0.4, 0.2), (1.0, 0.3, 0.0), (1.0, 0.0, -0.3)]
    for i in range(3):
        b = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, DYNAMIC, (0.6 * (i + 1), 4.0, 0.0))
        s = sc.slider(prev, b, (0.3, 0, 0), (-0.3, 0, 0), axes[i], axes[i])
        p = sc.piston(s, -0.2, 0.5) if limits else sc.piston(s)
        if mode == 1:
            sc.set_piston(p, 1, 30.0 - 25.0 * i)
        elif mode == 2:
            sc.set_piston(p, 2, 80.0, 0.6 - 0.5 * i)
        else:
            sc.set_piston(p, 3, 80.0, 0.3 - 0.2 * i)
        prev = b
    return sc


def large_mixed_world(seed=0, n_stacks=600, n_chains=40):
    """One world of ~2,400 bodies: stacks of three boxes, ball-socket chains of
    eight boxes hung from fixed posts and spheres dropped between them, all
    apart from each other (many islands), with sleeping enabled."""
    M = PILE_MATERIAL
    sc = Scene(f"large_mixed_{seed}", dict(step_time=1.0 / 60.0, substeps=2, pgs=(10, 1, 1), sleeping=True))
    rng = np.random.default_rng(seed)
    sc.box((-200.0, -1.0, -200.0), 400.0, 1.0, 400.0, M, FIXED)
    side = int(np.ceil(np.sqrt(n_stacks + n_chains)))
    cells = [(3.0 * (k % side) - 1.5 * side, 3.0 * (k // side) - 1.5 * side) for k in range(n_stacks + n_chains)]
    rng.shuffle(cells)
    for k in range(n_stacks):
        x, z = cells[k]
        for j in range(3):
            sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, M, DYNAMIC, (x, 0.6 + 1.05 * j, z + 0.1 * rng.uniform()))
        if k % 3 == 0:
            sc.sphere((0, 0, 0), 0.3, M, DYNAMIC, (x + 1.2, 0.5 + 2.0 * rng.uniform(), z))
    for k in range(n_chains):
        x, z = cells[n_stacks + k]
        prev = sc.box((-0.2, -0.2, -0.2), 0.4, 0.4, 0.4, M, FIXED, (x, 9.0, z))
        for i in range(8):
            b = sc.box((-0.2, -0.2, -0.2), 0.4, 0.4, 0.4, M, DYNAMIC, (x + 0.5 * (i + 1), 9.0, z))
            sc.ball_socket(prev, b, (0.25, 0, 0), (-0.25, 0, 0))
            prev = b
    return sc


def spring_chain(with_joints=False):
    """Boxes hung from a fixed post on damped springs (two sharing a body, one
    at its creation length), bouncing on the ground and off each other, or
    sharing bodies with a ball-socket joint."""
    M = PILE_MATERIAL
    sc = Scene("spring_chain", JOINT_PARAMS)
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, FIXED)
    post = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, FIXED, (0.0, 4.0, 0.0))
    prev = post
    for i in range(4):
        b = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, DYNAMIC, (0.4 * (i + 1), 3.2 - 0.7 * i, 0.1 * i))
        if with_joints and i == 2:
            sc.ball_socket(prev, b, (0.2, -0.35, 0.05), (-0.2, 0.35, -0.05))
        else:
            sc.spring(prev, b, (0.1, -0.25, 0.0), (0.0, 0.25, 0.1), 2.0 + i, 300.0 + 100.0 * i, 0.6 if i % 2 else -1.0)
        prev = b
    sc.spring(post, prev, (0.25, 0.0, 0.0), (0.0, 0.0, 0.25), 5.0, 80.0, 1.0)
    return sc


def cone_chain(holo=1, rot_strength=15000.0):
    """A ball-socket chain swung sideways with a 25-degree cone limit on each
    joint (holo = 0: without the holonomic block solve).  The limit rows'
    position correction is the raw strength times the error (not scaled by
    the step), so the default strength corrects violently once a limit is
    passed; a small strength keeps the motion smooth."""
    M = PILE_MATERIAL
    sc = Scene("cone_chain", dict(JOINT_PARAMS, pgs=(10, 1, holo)))
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, FIXED)
    prev = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, FIXED, (0.0, 6.0, 0.0))
    for i in range(4):
        b = sc.box((-0.15, -0.4, -0.15), 0.3, 0.8, 0.3, M, DYNAMIC, (0.0, 5.2 - 1.0 * i, 0.0))
        sc.ball_socket(prev, b, (0.0, -0.5 if i else -0.25, 0.0), (0.0, 0.5, 0.0))
        sc.cone_limit(prev, b, (0.0, -1.0, 0.0), (0.0, -1.0, 0.0), 25.0 * math.pi / 180.0, rot_strength)
        prev = b
    sc.velocity(prev, (6.0, 0.0, 2.0))
    return sc


def twist_chain(rot_strength=15000.0):
    """Twist limits beside cone limits on a ball-socket chain spun about its
    axis (strength: as for cone_chain)."""
    M = PILE_MATERIAL
    sc = Scene("twist_chain", JOINT_PARAMS)
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, M, FIXED)
    prev = sc.box((-0.25, -0.25, -0.25), 0.5, 0.5, 0.5, M, FIXED, (0.0, 6.0, 0.0))
    for i in range(3):
        b = sc.box((-0.3, -0.4, -0.1), 0.6, 0.8, 0.2, M, DYNAMIC, (0.0, 5.2 - 1.0 * i, 0.0))
        sc.ball_socket(prev, b, (0.0, -0.5 if i else -0.25, 0.0), (0.0, 0.5, 0.0))
        sc.cone_limit(prev, b, (0.0, -1.0, 0.0), (0.0, -1.0, 0.0), 20.0 * math.pi / 180.0, rot_strength)
        sc.twist_limit(prev, b, (0.0, -1.0, 0.0), (0.0, -1.0, 0.0), -0.3, 0.5, rot_strength)
        prev = b
    sc.ang_velocity(prev, (0.5, 9.0, 0.0))
    sc.velocity(prev, (2.0, 0.0, 0.0))
    return sc


def sleep_stacks(seed=0):
    """Three stacks of three boxes and a ball on the plate with sleeping
    enabled (dt 1/60, 1 substep, PGS (10,1,1)).  Returns the scene, the ball's
    id and an x position above the middle stack (for dropping the ball)."""
    params = dict(step_time=1.0 / 60.0, substeps=1, pgs=(10, 1, 1), sleeping=True)
    sc = Scene(f"sleepers_{seed}", params)
    sc.box((-10.0, -1.0, -10.0), 20.0, 1.0, 20.0, PILE_MATERIAL, FIXED)
    rng = np.random.default_rng(seed)
    for i in range(3):
        for j in range(3):
            sc.box((-0.5, -0.5, -0.5), 1.0, 1.0, 1.0, PILE_MATERIAL, DYNAMIC, (3.0 * i - 3, 0.6 + 1.05 * j, 0.1 * rng.uniform()))
    ball = sc.sphere((0, 0, 0), 0.5, PILE_MATERIAL, DYNAMIC, (8.0, 2.0, 0.0))
    return sc, ball, 3.0 + 0.2 * rng.uniform()
