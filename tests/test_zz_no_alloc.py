"""cpgpu_pairs_noalloc: candidate pairs for callers that cannot allocate device
memory (code inside another framework's memory pool, allocation-free real-time
loops, plugins given only pre-allocated buffers).  The caller owns every
buffer; the call's only scratch is a fixed device array inside the library.

Checked through the C ABI against the existing entry point: the pairs a world
step generated (cpgpu_get_pairs) for the AABBs it started from
(cpgpu_get_aabbs), on two calls in a row with different inputs.  Pair sets
are compared exactly, as in the other pair tests.  The device buffers here
come from PyTorch, standing in for the caller's own pool.
"""
import ctypes

import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    fn = cg.lib()._lib.cpgpu_pairs_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def test_pairs_noalloc_matches_world_pairs_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fn = _noalloc_fn()
    w = cg.world()
    scenes.apply(scenes.hull_drop(seed=2, n_side=4), w)
    stream = torch.cuda.current_stream()
    cap = 4096
    pairs_dev = torch.zeros(2 * cap, dtype=torch.int32, device="cuda")
    count_dev = torch.zeros(1, dtype=torch.int32, device="cuda")
    done = 0
    for k in (70, 110):                      # two calls, different inputs
        w.step(k - done)
        done = k
        aabbs = w.aabbs()                    # the AABBs the next step's broadphase uses
        w.step(1)
        done += 1
        expected = w.pairs()
        assert len(expected) > 0
        aabb_dev = torch.tensor(aabbs.astype(np.float32), device="cuda")
        pairs_dev.fill_(-1)
        rc = fn(aabb_dev.data_ptr(), aabbs.shape[0], pairs_dev.data_ptr(), cap, count_dev.data_ptr(),
                stream.cuda_stream)
        assert rc == 0, cg.lib().last_error()
        torch.cuda.synchronize()
        n = int(count_dev.item())
        got = pairs_dev[: 2 * n].cpu().numpy().view(np.uint32).reshape(-1, 2)
        assert n == len(expected)
        assert np.array_equal(got, expected)


def test_pairs_noalloc_rejects_too_many_bodies():
    fn = _noalloc_fn()
    dummy = ctypes.c_int()
    rc = fn(ctypes.c_void_p(16), 65537, ctypes.c_void_p(16), 1, ctypes.addressof(dummy), None)
    assert rc == -1
    assert b"65536" in cg.lib().last_error()


def _brute_pairs(aabbs):
    """Every overlapping pair (i < j, 1-based) under the inclusive test, by a
    sweep over the boxes sorted by their lower x (numpy, FP32 compares as on
    the device): in that order box k overlaps a later box k' in x exactly when
    lo_x[k'] <= hi_x[k], and the y and z tests filter those candidates."""
    a = aabbs.astype(np.float32)
    order = np.argsort(a[:, 0], kind="stable")
    s = a[order]
    end = np.searchsorted(s[:, 0], s[:, 3], side="right")
    out = []
    for k0 in range(0, len(s), 2048):
        k = np.arange(k0, min(k0 + 2048, len(s)))
        cnt = np.maximum(end[k] - k - 1, 0)
        kk = np.repeat(k, cnt)
        kp = kk + 1 + (np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt))
        lo1, hi1, lo2, hi2 = s[kk, :3], s[kk, 3:], s[kp, :3], s[kp, 3:]
        ok = ~((hi1 < lo2) | (lo1 > hi2)).any(axis=1)
        i, j = order[kk[ok]], order[kp[ok]]
        out.append(np.stack([np.minimum(i, j), np.maximum(i, j)], 1))
    p = np.concatenate(out) if out else np.zeros((0, 2), dtype=np.int64)
    p = p[np.lexsort((p[:, 1], p[:, 0]))]
    return (p + 1).astype(np.uint32)


def _random_aabbs(rng, n, extent):
    c = rng.uniform(0.0, extent, size=(n, 3))
    h = rng.uniform(0.05, 0.6, size=(n, 3))
    return np.concatenate([c - h, c + h], axis=1).astype(np.float32)


@pytest.mark.parametrize("n", [3000, 65536])
def test_pairs_noalloc_many_chunks_and_truncation(n):
    """Several scan chunks (1,024 bodies each, up to the 65,536 maximum) against
    a brute-force pair list, then a second call whose capacity is below the
    pair count: the count is the full total and exactly the first `cap` pairs
    are written (the rest of the buffer untouched)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fn = _noalloc_fn()
    rng = np.random.default_rng(n)
    aabbs = _random_aabbs(rng, n, extent=(n * 2.0) ** (1.0 / 3.0) * 1.6)
    expected = _brute_pairs(aabbs)
    assert len(expected) > n // 10
    stream = torch.cuda.current_stream()
    aabb_dev = torch.tensor(aabbs, device="cuda")
    count_dev = torch.zeros(1, dtype=torch.int32, device="cuda")
    cap = len(expected) + 16
    pairs_dev = torch.full((2 * cap,), -1, dtype=torch.int32, device="cuda")
    rc = fn(aabb_dev.data_ptr(), n, pairs_dev.data_ptr(), cap, count_dev.data_ptr(), stream.cuda_stream)
    assert rc == 0, cg.lib().last_error()
    torch.cuda.synchronize()
    assert int(count_dev.item()) == len(expected)
    got = pairs_dev[: 2 * len(expected)].cpu().numpy().view(np.uint32).reshape(-1, 2)
    assert np.array_equal(got, expected)
    # truncation: cap below the count
    small = len(expected) // 3
    pairs_dev.fill_(-1)
    rc = fn(aabb_dev.data_ptr(), n, pairs_dev.data_ptr(), small, count_dev.data_ptr(), stream.cuda_stream)
    assert rc == 0, cg.lib().last_error()
    torch.cuda.synchronize()
    assert int(count_dev.item()) == len(expected)
    host = pairs_dev.cpu().numpy()
    assert np.array_equal(host[: 2 * small].view(np.uint32).reshape(-1, 2), expected[:small])
    assert (host[2 * small:] == -1).all()
