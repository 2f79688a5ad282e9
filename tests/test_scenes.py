"""Seeded synthetic scenes are deterministic and well formed.  CPU only."""
import numpy as np

from constraintphysics_gb300 import scenes


def test_hull_drop_is_deterministic():
    a, b = scenes.hull_drop(seed=5, n_side=3), scenes.hull_drop(seed=5, n_side=3)
    assert a.n_bodies == b.n_bodies == 28
    for x, y in zip(a.ops, b.ops):
        assert x[0] == y[0]
        if x[0] == "hull":
            assert np.array_equal(x[1], y[1]) and x[2] == y[2] and x[5] == y[5]


def test_random_hulls_are_closed_convex_polyhedra():
    rng = np.random.default_rng(0)
    for _ in range(50):
        pts, faces = scenes.random_hull(rng)
        v, f = len(pts), len(faces)
        edges = {tuple(sorted((t[i], t[(i + 1) % 3]))) for t in faces for i in range(3)}
        assert v - len(edges) + f == 2          # Euler characteristic of a sphere
        assert 8 <= v <= 32
        assert np.allclose(np.linalg.norm(pts, axis=1).std(), 0, atol=1e-12)  # one scale per hull
        c = pts.mean(axis=0)
        for t in faces:                           # every face plane has all points on one side
            n = np.cross(pts[t[1]] - pts[t[0]], pts[t[2]] - pts[t[0]])
            s = (pts - pts[t[0]]) @ n
            assert (s <= 1e-9).all() or (s >= -1e-9).all()
        assert np.isfinite(c).all()


def test_batched_worlds_body_counts():
    ws = scenes.batched_worlds(seed=0, n_worlds=200)
    counts = np.array([w.n_bodies - 1 for w in ws])    # minus the plate
    assert counts.min() >= 8 and counts.max() <= 512
    # log-uniform in [8, 512]: median near sqrt(8 * 512) = 64
    assert 40 < np.median(counts) < 100
    kinds = {w.name.split("_")[0] for w in ws}
    assert kinds == {"pyramid", "pile"}
