"""ctypes signature table of the C ABI declared in include/cpgpu.h.

`bind(lib, prefix)` attaches argument/return types to every entry point of one
shared library whose functions carry `prefix` (``cpgpu_`` for the product,
``cpref_``/``cport_`` for the oracle libraries, which export the same set).
Pointers are passed as raw addresses (numpy ``arr.ctypes.data``) so that no
copies are made at the boundary.
"""
import ctypes as C

P = C.c_void_p
I = C.c_int
U32 = C.c_uint32
D = C.c_double

# name -> (restype, argtypes); every function returns an int status unless noted
SIGNATURES = {
    "world_create": (I, [P]),
    "world_destroy": (I, [P]),
    "set_step_time": (I, [P, D]),
    "set_gravity": (I, [P, D, D, D]),
    "set_substep_count": (I, [P, I]),
    "set_pgs_iterations": (I, [P, I, I, I]),
    "set_sleeping_enabled": (I, [P, I]),
    "set_warm_start_disabled": (I, [P, I]),
    "set_global_cfm": (I, [P, D]),
    "set_angle_vel_update_tick_count": (I, [P, I]),
    "set_internal_gyro_forces_disabled": (I, [P, I]),
    "body_hull": (I, [P, P, I, P, P, I, P, I, P, P]),
    "body_box": (I, [P, P, D, D, D, P, I, P, P]),
    "body_sphere": (I, [P, P, D, P, I, P, P]),
    "body_cylinder": (I, [P, P, D, D, P, I, P, P]),
    "body_capsule": (I, [P, P, D, D, P, I, P, P]),
    "raycast": (I, [P, P, P, I, P, I, P, P, P, P]),
    "body_union": (I, [P, P, I, I, P, P]),
    "body_mesh": (I, [P, P, I, P, I, P, I, P]),
    "body_set_velocity": (I, [P, U32, P]),
    "body_set_ang_velocity": (I, [P, U32, P]),
    "body_set_orientation": (I, [P, U32, P]),
    "body_set_position": (I, [P, U32, P]),
    "body_set_mass": (I, [P, U32, D]),
    "add_ball_socket": (I, [P, U32, U32, P, P, D, P]),
    "add_motor": (I, [P, U32, D, D, P]),
    "add_piston": (I, [P, U32, D, D, P]),
    "set_motor": (I, [P, U32, I, D, D]),
    "set_piston": (I, [P, U32, I, D, D]),
    "get_motor_position": (I, [P, U32, P]),
    "get_piston_position": (I, [P, U32, P]),
    "add_distance": (I, [P, U32, U32, P, P, D, D, P]),
    "add_weld": (I, [P, U32, U32, P, P, D, D, P]),
    "add_spring": (I, [P, U32, U32, P, P, D, D, D, P]),
    "add_cone_limit": (I, [P, U32, U32, P, P, D, D, P]),
    "add_twist_limit": (I, [P, U32, U32, P, P, D, D, D, P]),
    "add_slider": (I, [P, U32, U32, P, P, P, P, D, D, P]),
    "add_sliding_hinge": (I, [P, U32, U32, P, P, P, P, D, D, P]),
    "add_hinge": (I, [P, U32, U32, P, P, P, P, D, D, P]),
    "step": (I, [P, I]),
    "num_bodies": (I, [P, P]),
    "get_body_state": (I, [P, P, P, P, P]),
    "get_asleep": (I, [P, P]),
    "set_body_state": (I, [P, P, P, P, P]),
    "get_aabbs": (I, [P, P]),
    "get_pairs": (I, [P, P, I, P]),
    "get_contacts": (I, [P, P, I, P]),
    "set_contacts": (I, [P, P, I]),
    "get_joint_state": (I, [P, P, P, P, P, P]),
    "set_joint_state": (I, [P, P, P, P, P, I]),
    "batch_create": (I, [P, I, P]),
    "batch_destroy": (I, [P]),
    "batch_step": (I, [P, I]),
    "batch_get_body_state": (I, [P, I, P, P, P, P]),
    "batch_info": (I, [P, P, P, P]),
    "last_error": (C.c_char_p, []),
}


class Contact(C.Structure):
    """Mirror of struct cpgpu_contact (include/cpgpu.h)."""
    _fields_ = [
        ("b1", C.c_uint32), ("b2", C.c_uint32), ("live", C.c_uint32), ("memory_life", C.c_int32),
        ("magic_c", C.c_uint64), ("magic_b", C.c_uint64),
        ("p_local_b1", C.c_double * 3), ("p_local_b2", C.c_double * 3), ("n_local_b1", C.c_double * 3),
        ("pen_depth", C.c_double), ("bounce", C.c_double), ("friction_coeff", C.c_double),
        ("normal_impulse", C.c_double), ("friction_impulse", C.c_double * 2),
        ("friction_u", C.c_double * 3), ("friction_w", C.c_double * 3),
        ("static_ready", C.c_uint32), ("pad_", C.c_uint32),
    ]


class Material(C.Structure):
    """Mirror of struct cpgpu_material (include/cpgpu.h)."""
    _fields_ = [("density", C.c_double), ("restitution", C.c_double),
                ("kinetic_friction", C.c_double), ("static_friction", C.c_double)]


class Primitive(C.Structure):
    """Mirror of struct cpgpu_primitive (include/cpgpu.h)."""
    _fields_ = [("kind", C.c_int), ("p", C.c_double * 3), ("a", C.c_double), ("b", C.c_double), ("c", C.c_double),
                ("points", C.c_void_p), ("n_points", C.c_int), ("face_offsets", C.c_void_p),
                ("face_indices", C.c_void_p), ("n_faces", C.c_int), ("mat", Material)]


PRIM_KINDS = {"hull": 0, "box": 1, "sphere": 2, "cylinder": 3, "capsule": 4}


def bind(lib, prefix, optional=()):
    """Attach signatures for every SIGNATURES entry that `lib` exports.

    Missing symbols raise unless their short name is listed in `optional`.
    Returns a namespace object whose attributes are the bound functions keyed
    by short name (without prefix)."""
    ns = type("ABI", (), {})()
    for short, (res, args) in SIGNATURES.items():
        name = prefix + short
        try:
            fn = getattr(lib, name)
        except AttributeError:
            if short in optional:
                continue
            raise
        fn.restype = res
        fn.argtypes = args
        setattr(ns, short, fn)
    return ns
