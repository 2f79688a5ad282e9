"""Worlds above the size at which the pair pass runs over tiles and the
islands are searched per connected component in parallel (2,048 bodies), on
a GB300.

  * a ~2,400-body world of box stacks, ball-socket chains and spheres with
    sleeping enabled steps bit-identically with the component-parallel
    island search and with the serial one (CPGPU_ISLANDS_SERIAL=1): the same
    islands, row order, sleeping and joint rows;
  * its pair list is the sorted set of overlapping AABB pairs.
(The 20,000-body terrain at full size is tests/test_gpu_mesh.py's.)
"""
import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu


def _run(sc, steps, monkeypatch=None, serial=False):
    if monkeypatch is not None:
        if serial:
            monkeypatch.setenv("CPGPU_ISLANDS_SERIAL", "1")
        else:
            monkeypatch.delenv("CPGPU_ISLANDS_SERIAL", raising=False)
    w = cg.world()
    scenes.apply(sc, w)
    out = []
    for s in range(steps):
        w.step(1)
        if s % 25 == 24:
            out.append((w.state(), w.asleep(), w.joint_state()["impulse"].copy()))
    return w, out


def test_parallel_islands_equal_the_serial_search(monkeypatch):
    sc = scenes.large_mixed_world(0)
    assert sc.n_bodies > 2048
    _, par = _run(sc, 150, monkeypatch, serial=False)
    _, ser = _run(sc, 150, monkeypatch, serial=True)
    slept = False
    for (sa, aa, ja), (sb, ab, jb) in zip(par, ser):
        for k in sa:
            assert np.array_equal(sa[k], sb[k]), k
        assert np.array_equal(aa, ab)
        assert np.array_equal(ja, jb)
        slept |= bool(aa.sum() > 100)
    assert slept                                   # stacks fell asleep on the way


def test_large_world_pairs_are_the_overlaps():
    sc = scenes.large_mixed_world(1)
    w = cg.world()
    scenes.apply(sc, w)
    w.step(30)
    aabb = w.aabbs()
    w.step(1)
    lo, hi = aabb[:, :3], aabb[:, 3:]
    ov = ~((hi[:, None, :] < lo[None, :, :]) | (lo[:, None, :] > hi[None, :, :])).any(axis=2)
    i, j = np.nonzero(np.triu(ov, 1))
    assert np.array_equal(w.pairs(), np.stack([i + 1, j + 1], 1).astype(np.uint32))
