"""FP64 momentum / energy audit of the device path (cpgpu_*_audit), on a GB300.

The audit sums, per world and in FP64, momentum, angular momentum about the
origin, kinetic and potential energy over the dynamic bodies after every step.
Checked three ways: against the same sums taken here in numpy (FP64) over the
device's own state with the reference's mass properties; against the CPU
restatement stepping the same scene; and batched worlds against the same
worlds audited alone (bit for bit).
"""
import ctypes

import numpy as np
import pytest

import constraintphysics_gb300 as cg
from constraintphysics_gb300 import scenes

pytestmark = pytest.mark.gpu


def _rot(q):
    r, i, j, k = q
    return np.array([[r * r + i * i - j * j - k * k, 2 * i * j - 2 * r * k, 2 * i * k + 2 * r * j],
                     [2 * i * j + 2 * r * k, r * r - i * i + j * j - k * k, 2 * j * k - 2 * r * i],
                     [2 * i * k - 2 * r * j, 2 * j * k + 2 * r * i, r * r - i * i - j * j + k * k]])


def _mass_props(oracle_mod, sc):
    """Mass and reference-frame tensor of every body, from the reference engine."""
    mass, _, tensor, _ = oracle_mod.capture_mass_properties(sc)
    return mass, tensor.reshape(-1, 3, 3)


def _audit_numpy(state, mass, tensor, movements, g):
    p = np.zeros(3); L = np.zeros(3); ke = 0.0; pe = 0.0
    for i, mv in enumerate(movements):
        if mv != scenes.DYNAMIC:
            continue
        m = mass[i]
        x, v, w = state["com"][i], state["vel"][i], state["ang_vel"][i]
        R = _rot(state["quat"][i])
        Iw = R @ tensor[i] @ R.T
        p += m * v
        L += m * np.cross(x, v) + Iw @ w
        ke += 0.5 * m * v @ v + 0.5 * w @ Iw @ w
        pe -= m * np.dot(g, x)
    return p, L, ke, pe


def _spinning_free_fall():
    sc = scenes.Scene("audit_free_fall", dict(step_time=1.0 / 60.0, sleeping=False))
    mat = scenes.PILE_MATERIAL
    rng = np.random.default_rng(3)
    for k in range(6):
        pos = (3.0 * k, 10.0 + k, -2.0 * k)
        if k % 3 == 0:
            b = sc.box((-0.5, -0.3, -0.7), 1.0, 0.6, 1.4, mat, scenes.DYNAMIC, pos)
        elif k % 3 == 1:
            b = sc.cylinder((0.0, -0.5, 0.0), 0.4, 1.0, mat, scenes.DYNAMIC, pos)
        else:
            pts, faces = scenes.random_hull(rng)
            b = sc.hull(pts, faces, mat, scenes.DYNAMIC, pos)
        sc.orient(b, scenes.random_quat(rng))
        sc.velocity(b, tuple(rng.uniform(-2, 2, 3)))
        sc.ang_velocity(b, tuple(rng.uniform(-4, 4, 3)))
    return sc


def test_audit_matches_fp64_sums_of_device_state(oracle_mod):
    sc = _spinning_free_fall()
    mass, tensor = _mass_props(oracle_mod, sc)
    w = cg.world()
    scenes.apply(sc, w)
    cg.set_audit(w, True)
    w.step(25)
    a = cg.read_audit(w)
    assert a["steps"] == 25
    p, L, ke, pe = _audit_numpy(w.state(), mass, tensor, sc.movements(), np.array([0.0, -6.0, 0.0]))
    # the device's masses and tensors are FP32 copies of the reference's:
    # sums agree to FP32 rounding of the inputs (1e-6 relative)
    assert np.allclose(a["momentum"], p, rtol=1e-6, atol=1e-6 * np.abs(p).max())
    assert np.allclose(a["angular_momentum"], L, rtol=1e-6, atol=1e-6 * np.abs(L).max())
    assert a["kinetic"] == pytest.approx(ke, rel=1e-6)
    assert a["potential"] == pytest.approx(pe, rel=1e-6)
    # free fall: the momentum grows by M g dt per step exactly (up to FP32 velocity rounding)
    m_tot = mass.sum()
    w0 = cg.world()
    scenes.apply(sc, w0)
    v0 = w0.state()["vel"]
    p0 = (mass[:, None] * v0).sum(axis=0)
    expect = p0 + m_tot * np.array([0.0, -6.0, 0.0]) * 25 / 60.0
    assert np.allclose(a["momentum"], expect, rtol=1e-5, atol=1e-5 * np.abs(expect).max())


def test_audit_against_restatement_on_a_pile(oracle_mod):
    sc = scenes.hull_drop(seed=2, n_side=3)
    mass, tensor = _mass_props(oracle_mod, sc)
    w = cg.world()
    scenes.apply(sc, w)
    cg.set_audit(w, True)
    p_ = oracle_mod.port_world()
    scenes.apply(sc, p_)
    g = np.array([0.0, -6.0, 0.0])
    for k in (10, 30):
        w.step(k - (10 if k == 30 else 0))
        p_.step(k - (10 if k == 30 else 0))
        a = cg.read_audit(w)
        p, L, ke, pe = _audit_numpy(p_.state(), mass, tensor, sc.movements(), g)
        # FP32 trajectory against the FP64 restatement over a few dozen steps
        # of falling and first impacts: 1e-4 relative
        assert np.abs(a["momentum"] - p).max() <= 1e-4 * np.abs(p).max()
        assert np.abs(a["angular_momentum"] - L).max() <= 1e-4 * np.abs(L).max()
        assert a["kinetic"] == pytest.approx(ke, rel=1e-4)
        assert a["potential"] == pytest.approx(pe, rel=1e-4)
    assert a["steps"] == 30
    assert np.isfinite(a["max_step_gain"])


def test_batch_audit_equals_worlds_audited_alone():
    rng = np.random.default_rng(11)
    pool = scenes.HullPool(2, size=16)
    scs = [scenes.batched_world(rng, pool, 8, 60) for _ in range(5)]
    alone = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        cg.set_audit(w, True)
        w.step(20)
        a = cg.read_audit(w)
        alone.append(np.concatenate([a["momentum"], a["angular_momentum"],
                                     [a["kinetic"], a["potential"], a["max_step_gain"], a["steps"]]]))
    ws = []
    for sc in scs:
        w = cg.world()
        scenes.apply(sc, w)
        ws.append(w)
    b = cg.Batch(ws)
    b.set_audit(True)
    b.step(20)
    got = b.read_audit()
    assert np.array_equal(got, np.array(alone))
    b.set_audit(False)
    with pytest.raises(cg.CPGPUError):
        b.read_audit()
