"""Accuracy of the device path over 300 steps against the reference engine
(positions within 1e-3 m after 300 steps), on worlds of the batched workload
(4,096 worlds of 8-512 bodies, seed 0).

Box pyramids settle into resting stacks: the device (FP32) stays within
1e-3 m of the reference (FP64) for at least 90 % of the bodies, as close as
the FP64 restatement itself does.  Hull piles are chaotic: bodies tumble
off each other and rounding-level differences grow to metres within 300
steps, for the FP64 restatement as much as for the device.  There the device
is held to the drift of a control that makes the smallest perturbation any
FP32 implementation makes: the restatement in FP64 with its state rounded to
FP32 after every step.
"""
import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu

# worlds of scenes.batched_worlds(seed=0): box pyramids of 113, 151, 100, 289
# and 13 boxes; hull piles of 8, 33, 17 and 16 hulls
PYRAMIDS = [0, 644, 1340, 1979, 3407]
PILES = [1, 1388, 2114, 3402]
STEPS = 300


@pytest.fixture(scope="module")
def workload():
    return scenes.batched_worlds(seed=0, n_worlds=max(PYRAMIDS + PILES) + 1)


def _f32(st):
    return {k: np.asarray(v, np.float32).astype(np.float64) for k, v in st.items()}


def _drift(oracle_mod, sc, controls=("fp64",)):
    dyn = np.array([m == scenes.DYNAMIC for m in sc.movements()])
    g = cg.world()
    scenes.apply(sc, g)
    g.step(STEPS)
    r = oracle_mod.ref_world()
    scenes.apply(sc, r)
    r.step(STEPS)
    rc = r.state()["com"][dyn]
    out = {"device": np.linalg.norm(g.state()["com"][dyn] - rc, axis=1)}
    if "fp64" in controls:
        p = oracle_mod.port_world()
        scenes.apply(sc, p)
        p.step(STEPS)
        out["fp64"] = np.linalg.norm(p.state()["com"][dyn] - rc, axis=1)
    if "fp32_state" in controls:
        q = oracle_mod.port_world()
        scenes.apply(sc, q)
        for _ in range(STEPS):
            q.set_state(**_f32(q.state()))
            q.step(1)
        out["fp32_state"] = np.linalg.norm(q.state()["com"][dyn] - rc, axis=1)
    return out


def test_resting_pyramids_within_1mm_of_the_reference(oracle_mod, workload):
    dev, ctl = [], []
    for i in PYRAMIDS:
        sc = workload[i]
        assert sc.name.startswith("pyramid")
        d = _drift(oracle_mod, sc)
        dev.append(d["device"])
        ctl.append(d["fp64"])
    dev, ctl = np.concatenate(dev), np.concatenate(ctl)
    stats = (f"device median {np.median(dev):.2e} m, within 1e-3 m {np.mean(dev <= 1e-3):.3f}; "
             f"FP64 restatement median {np.median(ctl):.2e} m, within {np.mean(ctl <= 1e-3):.3f}")
    # measured on a GB300: device 0.958 within 1e-3 m (median 1e-5 m); FP64
    # restatement 0.955
    assert np.mean(dev <= 1e-3) >= 0.90, stats
    assert np.mean(dev <= 1e-3) >= np.mean(ctl <= 1e-3) - 0.03, stats
    assert np.median(dev) <= 3e-4, stats


def test_chaotic_piles_drift_like_an_fp32_state_control(oracle_mod, workload):
    dev, ctl64, ctl32 = [], [], []
    for i in PILES:
        sc = workload[i]
        assert sc.name.startswith("pile")
        d = _drift(oracle_mod, sc, controls=("fp64", "fp32_state"))
        dev.append(d["device"])
        ctl64.append(d["fp64"])
        ctl32.append(d["fp32_state"])
    dev, ctl64, ctl32 = np.concatenate(dev), np.concatenate(ctl64), np.concatenate(ctl32)
    stats = (f"median drift: device {np.median(dev):.2e} m, FP32-state control {np.median(ctl32):.2e} m, "
             f"FP64 restatement {np.median(ctl64):.2e} m")
    # stated factors: the device's median drift is at most twice the FP32-state
    # control's and five times the FP64 restatement's
    assert np.median(dev) <= 2.0 * np.median(ctl32), stats
    assert np.median(dev) <= 5.0 * np.median(ctl64), stats
