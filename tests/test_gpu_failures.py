"""Failure detection of the device path, exercised without any GPU fault.

  * non-finite state: a NaN velocity written from the host through the C ABI
    (cpgpu_set_body_state) must make the next step return CPGPU_ERR_NAN;
  * bounded waits: with CPGPU_WAIT_LIMIT=0 every mbarrier wait of the
    narrowphase and large-island solver kernels gives up at once (the copies
    it waited for are still drained with the normal bound before the warp
    leaves its shared memory), and the step must return CPGPU_ERR_TIMEOUT;
  * in both cases the CUDA context stays usable: a new world steps afterwards
    and matches a world that never failed, bit for bit.
"""
import os

import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu

ERR_NAN, ERR_TIMEOUT = -4, -7


def _pyramid():
    rng = np.random.default_rng(5)
    pool = scenes.HullPool(0, size=8)
    sc = None
    while sc is None or not sc.name.startswith("pyramid"):
        sc = scenes.batched_world(rng, pool, 60, 120)
    return sc


def _resting_state(sc, steps=60):
    w = cg.world()
    scenes.apply(sc, w)
    w.step(steps)
    return w.state(), w.contacts()


def _status(excinfo):
    return int(str(excinfo.value).split("status ")[1].split(":")[0])


def _fresh_world_still_matches(sc):
    a = cg.world()
    scenes.apply(sc, a)
    a.step(10)
    b = cg.world()
    scenes.apply(sc, b)
    b.step(10)
    sa, sb = a.state(), b.state()
    assert all(np.array_equal(sa[k], sb[k]) for k in sa)
    assert np.isfinite(sa["com"]).all()


def test_nan_velocity_is_reported():
    sc = _pyramid()
    w = cg.world()
    scenes.apply(sc, w)
    w.step(30)
    st = w.state()
    st["vel"][3] = [np.nan, 0.0, 0.0]
    w.set_state(**st)
    with pytest.raises(cg.CPGPUError) as e:
        w.step(1)
    assert _status(e) == ERR_NAN, str(e.value)
    assert "non-finite" in str(e.value)
    _fresh_world_still_matches(sc)


def test_bounded_waits_give_up_with_timeout(monkeypatch):
    sc = _pyramid()
    state, contacts = _resting_state(sc)
    monkeypatch.setenv("CPGPU_WAIT_LIMIT", "0")
    w = cg.world()
    scenes.apply(sc, w)
    w.set_state(**state)
    w.set_contacts(contacts)
    with pytest.raises(cg.CPGPUError) as e:
        w.step(1)
    assert _status(e) == ERR_TIMEOUT, str(e.value)
    assert "bounded-wait-timeout" in str(e.value)
    monkeypatch.delenv("CPGPU_WAIT_LIMIT")
    _fresh_world_still_matches(sc)
