"""Generate the golden fixtures from the reference engine itself.

Runs the reference (oracle/_ref/libcpref.so, built from the reference's own
sources) on seeded scenes and stores the resulting states and contacts.
Usage: python tests/golden/make_golden.py [fixture function ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from constraintphysics_gb300 import scenes  # noqa: E402


def mass_properties(world, n):
    """The reference's mass, centre of mass (geometry frame) and inertia tensor
    of bodies 1..n."""
    import ctypes
    g = oracle.ref_abi()._lib.cpref_get_mass_properties
    g.restype = ctypes.c_int
    g.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    mass, com, tensor = np.zeros(n), np.zeros((n, 3)), np.zeros((n, 9))
    for i in range(n):
        m = np.zeros(1)
        c = np.zeros(3)
        t = np.zeros(9)
        assert g(world.h, i + 1, m.ctypes.data, c.ctypes.data, t.ctypes.data) == 0
        mass[i], com[i], tensor[i] = m[0], c, t
    return mass, com, tensor


def mixed():
    """Boxes, spheres, cylinders and hulls (scenes.mixed_drop, 4x4x2, seed 1)
    after 150 reference steps, with the reference's mass properties so the
    restatement can start from the same bodies without the reference."""
    steps = 150
    sc = scenes.mixed_drop(seed=1, n_side=4, n_layers=2)
    w = oracle.ref_world()
    scenes.apply(sc, w)
    mass, com, tensor = mass_properties(w, sc.n_bodies)
    w.step(steps)
    st = w.state()
    c = w.contacts()
    np.savez_compressed(os.path.join(HERE, "mixed_drop_4x4x2_seed1.npz"), steps=steps, mass=mass, com_geom=com,
                        tensor=tensor, com=st["com"], quat=st["quat"], vel=st["vel"], ang_vel=st["ang_vel"],
                        magic_b=c["magic_b"], b1=c["b1"], b2=c["b2"], normal_impulse=c["normal_impulse"],
                        pen_depth=c["pen_depth"])


def chain():
    """One articulated chain (scenes.chain_world, rng seed 5, 10-14 links, 20
    spheres) after 200 reference steps, with the reference's mass properties
    as created (before the scene's setMass calls)."""
    steps = 200
    sc = scenes.chain_world(np.random.default_rng(5), 10, 14, n_spheres=20)
    mass, com, tensor, w = oracle.capture_mass_properties(sc)
    w.step(steps)
    st = w.state()
    np.savez_compressed(os.path.join(HERE, "chain_seed5.npz"), steps=steps, mass=mass, com_geom=com, tensor=tensor,
                        com=st["com"], quat=st["quat"], vel=st["vel"], ang_vel=st["ang_vel"])


def terrain():
    """Mixed bodies on a 16 x 16 value-noise terrain mesh (scenes.terrain_drop,
    seed 2) after 150 reference steps, with creation-time mass properties."""
    steps = 150
    sc = scenes.terrain_drop(seed=2, n_grid=16, n_side=3, n_layers=2)
    mass, com, tensor, w = oracle.capture_mass_properties(sc)
    w.step(steps)
    st = w.state()
    c = w.contacts()
    np.savez_compressed(os.path.join(HERE, "terrain_drop_seed2.npz"), steps=steps, mass=mass, com_geom=com, tensor=tensor,
                        com=st["com"], quat=st["quat"], vel=st["vel"], ang_vel=st["ang_vel"], magic_c=c["magic_c"],
                        magic_b=c["magic_b"])


def capsules():
    """Capsules with boxes, spheres, cylinders and hulls on a 16 x 16
    value-noise terrain (scenes.capsule_drop, seed 5, 3x3x2) after 150
    reference steps, with creation-time mass properties."""
    steps = 150
    sc = scenes.capsule_drop(seed=5, n_side=3, n_layers=2, terrain=True, n_grid=16)
    mass, com, tensor, w = oracle.capture_mass_properties(sc)
    w.step(steps)
    st = w.state()
    c = w.contacts()
    np.savez_compressed(os.path.join(HERE, "capsule_terrain_seed5.npz"), steps=steps, mass=mass, com_geom=com,
                        tensor=tensor, com=st["com"], quat=st["quat"], vel=st["vel"], ang_vel=st["ang_vel"],
                        magic_c=c["magic_c"], magic_b=c["magic_b"], b1=c["b1"], b2=c["b2"])


def kinematic():
    """A kinematic pusher and spinner among dynamic bodies
    (scenes.kinematic_push, seed 1) after 240 reference steps, with
    creation-time mass properties."""
    steps = 240
    sc = scenes.kinematic_push(seed=1)
    mass, com, tensor, w = oracle.capture_mass_properties(sc)
    w.step(steps)
    st = w.state()
    c = w.contacts()
    np.savez_compressed(os.path.join(HERE, "kinematic_push_seed1.npz"), steps=steps, mass=mass, com_geom=com,
                        tensor=tensor, com=st["com"], quat=st["quat"], vel=st["vel"], ang_vel=st["ang_vel"],
                        magic_b=c["magic_b"], b1=c["b1"], b2=c["b2"], normal_impulse=c["normal_impulse"])


def unions():
    """Multi-primitive bodies on a terrain (scenes.union_drop, seed 2, 10
    bodies) after 240 reference steps, with creation-time mass properties."""
    steps = 240
    sc = scenes.union_drop(seed=2, n=10, terrain=True)
    mass, com, tensor, w = oracle.capture_mass_properties(sc)
    w.step(steps)
    st = w.state()
    c = w.contacts()
    np.savez_compressed(os.path.join(HERE, "union_terrain_seed2.npz"), steps=steps, mass=mass, com_geom=com,
                        tensor=tensor, com=st["com"], quat=st["quat"], vel=st["vel"], ang_vel=st["ang_vel"],
                        magic_b=c["magic_b"], b1=c["b1"], b2=c["b2"], normal_impulse=c["normal_impulse"])


# joint scenes of the joint-kinds fixture: name -> (scene, steps)
def joint_scenes():
    return {
        "distance": (scenes.distance_chain(True), 200),
        "weld": (scenes.weld_cantilever(True), 200),
        "slider": (scenes.slider_chain(("slider", "sliding_hinge", "slider", "sliding_hinge")), 200),
        "cone": (scenes.cone_chain(), 200),
        "twist": (scenes.twist_chain(), 200),
        "spring": (scenes.spring_chain(True), 200),
        "motor_pos": (scenes.motor_chain(3, True), 200),
        "motor_vel": (scenes.motor_chain(2, False), 200),
        "piston_vel": (scenes.piston_chain(2, True), 200),
        "piston_pos": (scenes.piston_chain(3, True), 200),
    }


def joint_kinds():
    """Distance, weld, slider / sliding-hinge, cone- and twist-limit chains,
    springs sharing bodies with ball-sockets, motors and pistons in their
    powered modes (with and without limits): each scene after 200 reference
    steps, with creation-time mass properties, states, and the motors'
    angles / pistons' slide positions."""
    out = {}
    for name, (sc, steps) in joint_scenes().items():
        mass, com, tensor, w = oracle.capture_mass_properties(sc)
        w.step(steps)
        st = w.state()
        out[f"{name}_steps"] = steps
        for k, v in (("mass", mass), ("com_geom", com), ("tensor", tensor), ("com", st["com"]), ("quat", st["quat"]),
                     ("vel", st["vel"]), ("ang_vel", st["ang_vel"])):
            out[f"{name}_{k}"] = v
        if name.startswith("motor") or name.startswith("piston"):
            get = w.motor_position if name.startswith("motor") else w.piston_position
            out[f"{name}_positions"] = np.array([get(cid) for cid in w.constraint_ids[1::2]])
    np.savez_compressed(os.path.join(HERE, "joint_kinds.npz"), **out)


def sleeping():
    """Three box stacks and a ball with sleeping enabled (scenes.sleep_stacks,
    seed 0) after 400 reference steps: states and which bodies sleep, with
    creation-time mass properties."""
    steps = 400
    sc, _, _ = scenes.sleep_stacks(0)
    mass, com, tensor, w = oracle.capture_mass_properties(sc)
    w.step(steps)
    st = w.state()
    np.savez_compressed(os.path.join(HERE, "sleep_stacks_seed0.npz"), steps=steps, mass=mass, com_geom=com,
                        tensor=tensor, com=st["com"], quat=st["quat"], vel=st["vel"], ang_vel=st["ang_vel"],
                        asleep=w.asleep())


# ray fixture scenes: name -> (scene, steps, ignore lists)
def ray_scenes():
    return {
        "capsules": (scenes.capsule_drop(seed=3, n_side=4, n_layers=2, terrain=True), 90, ((), (1, 5, 9))),
        "unions": (scenes.union_drop(seed=0, n=10), 90, ((), (2, 4))),
    }


def ray_batch(seed, n):
    """n rays from above the scenes towards them (unit directions)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform([-8, 2, -8], [8, 12, 8], size=(n, 3))
    d = rng.uniform([-6, -1, -6], [6, 4, 6], size=(n, 3)) - o
    return o, d / np.linalg.norm(d, axis=1, keepdims=True)


def rays():
    """raycastFirstIntersection on 2,000 rays through settled scenes (every
    primitive kind on a terrain; bodies of several primitives), with and
    without an ignore list, after 90 reference steps, with creation-time mass
    properties."""
    out = {}
    o, d = ray_batch(0, 2000)
    out["origins"], out["dirs"] = o, d
    for name, (sc, steps, ignores) in ray_scenes().items():
        mass, com, tensor, w = oracle.capture_mass_properties(sc)
        w.step(steps)
        out[f"{name}_mass"], out[f"{name}_com_geom"], out[f"{name}_tensor"] = mass, com, tensor
        for i, ig in enumerate(ignores):
            h = w.raycast(o, d, ig)
            for k in ("body", "pos", "normal", "dist"):
                out[f"{name}_{i}_{k}"] = h[k]
    np.savez_compressed(os.path.join(HERE, "rays.npz"), **out)


def main(names=()):
    if names:
        for n in names:
            globals()[n]()
        return
    rays()
    joint_kinds()
    sleeping()
    unions()
    kinematic()
    capsules()
    terrain()
    chain()
    mixed()
    steps = 120
    w = oracle.ref_world()
    scenes.apply(scenes.hull_drop(seed=1, n_side=3), w)
    w.step(steps)
    st = w.state()
    c = w.contacts()
    np.savez_compressed(os.path.join(HERE, "hull_drop_3_seed1.npz"), steps=steps, com=st["com"], quat=st["quat"],
                        vel=st["vel"], ang_vel=st["ang_vel"], magic_b=c["magic_b"], b1=c["b1"], b2=c["b2"],
                        normal_impulse=c["normal_impulse"], pen_depth=c["pen_depth"])


if __name__ == "__main__":
    main(sys.argv[1:])
