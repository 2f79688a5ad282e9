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
