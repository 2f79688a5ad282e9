"""Python handle over one world of any library exporting the cpgpu C ABI.

The product library (libcpgpu.so) and the oracle libraries export the same
function set (include/cpgpu.h), so this one class drives all of them; tests use
it to run identical scenes through the device path and the oracles.
"""
import ctypes as C

import numpy as np

from ._abi import Contact, Material


class CPGPUError(RuntimeError):
    pass


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


class World:
    """One PhysicsEngine instance behind a cpgpu-style C ABI."""

    def __init__(self, abi):
        self.abi = abi
        h = C.c_void_p()
        self._check(abi.world_create(C.byref(h)))
        self.h = h
        self.n_bodies = 0

    # -- error handling ----------------------------------------------------
    def _check(self, rc):
        if rc != 0:
            msg = self.abi.last_error() if hasattr(self.abi, "last_error") else b""
            raise CPGPUError(f"status {rc}: {msg.decode(errors='replace') if msg else ''}")
        return rc

    def close(self):
        if self.h is not None and self.h.value:
            self.abi.world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters (PhysicsEngine setters) -----------------------------------
    def set_params(self, step_time=None, gravity=None, substeps=None, pgs=None,
                   sleeping=None, warm_start_disabled=None, cfm=None,
                   angle_vel_ticks=None, gyro_disabled=None):
        a, h = self.abi, self.h
        if step_time is not None:
            self._check(a.set_step_time(h, float(step_time)))
        if gravity is not None:
            self._check(a.set_gravity(h, *map(float, gravity)))
        if substeps is not None:
            self._check(a.set_substep_count(h, int(substeps)))
        if pgs is not None:
            self._check(a.set_pgs_iterations(h, *map(int, pgs)))
        if sleeping is not None:
            self._check(a.set_sleeping_enabled(h, int(bool(sleeping))))
        if warm_start_disabled is not None:
            self._check(a.set_warm_start_disabled(h, int(bool(warm_start_disabled))))
        if cfm is not None:
            self._check(a.set_global_cfm(h, float(cfm)))
        if angle_vel_ticks is not None:
            self._check(a.set_angle_vel_update_tick_count(h, int(angle_vel_ticks)))
        if gyro_disabled is not None:
            self._check(a.set_internal_gyro_forces_disabled(h, int(bool(gyro_disabled))))

    # -- bodies -----------------------------------------------------------------
    @staticmethod
    def _mat(m):
        m = m or {}
        return Material(m.get("density", 1.0), m.get("restitution", 0.3),
                        m.get("kinetic_friction", 0.6), m.get("static_friction", 1.1))

    def _new_id(self, rc, out):
        self._check(rc)
        self.n_bodies += 1
        return out.value

    def add_hull(self, points, faces, material=None, movement=0, pos=(0, 0, 0)):
        pts = _f64(points)
        offs = np.zeros(len(faces) + 1, dtype=np.int32)
        offs[1:] = np.cumsum([len(f) for f in faces])
        idx = np.ascontiguousarray(np.concatenate([np.asarray(f, dtype=np.int32) for f in faces]))
        pos = _f64(pos, 3)
        mat = self._mat(material)
        out = C.c_uint32()
        rc = self.abi.body_hull(self.h, _ptr(pts), pts.size // 3, _ptr(offs), _ptr(idx), len(faces),
                                C.addressof(mat), int(movement), _ptr(pos), C.addressof(out))
        return self._new_id(rc, out)

    def add_box(self, corner, dx, dy, dz, material=None, movement=0, pos=(0, 0, 0)):
        corner = _f64(corner, 3)
        pos = _f64(pos, 3)
        mat = self._mat(material)
        out = C.c_uint32()
        rc = self.abi.body_box(self.h, _ptr(corner), float(dx), float(dy), float(dz),
                               C.addressof(mat), int(movement), _ptr(pos), C.addressof(out))
        return self._new_id(rc, out)

    def add_sphere(self, center, radius, material=None, movement=0, pos=(0, 0, 0)):
        center = _f64(center, 3)
        pos = _f64(pos, 3)
        mat = self._mat(material)
        out = C.c_uint32()
        rc = self.abi.body_sphere(self.h, _ptr(center), float(radius), C.addressof(mat), int(movement),
                                  _ptr(pos), C.addressof(out))
        return self._new_id(rc, out)

    def add_cylinder(self, base, radius, height, material=None, movement=0, pos=(0, 0, 0)):
        base = _f64(base, 3)
        pos = _f64(pos, 3)
        mat = self._mat(material)
        out = C.c_uint32()
        rc = self.abi.body_cylinder(self.h, _ptr(base), float(radius), float(height), C.addressof(mat),
                                    int(movement), _ptr(pos), C.addressof(out))
        return self._new_id(rc, out)

    def add_capsule(self, bot, radius, drum_height, material=None, movement=0, pos=(0, 0, 0)):
        """ConvexUnionGeometry::capsule: `bot` is the centre of the bottom cap
        sphere, `drum_height` the distance between the cap-sphere centres."""
        bot = _f64(bot, 3)
        pos = _f64(pos, 3)
        mat = self._mat(material)
        out = C.c_uint32()
        rc = self.abi.body_capsule(self.h, _ptr(bot), float(radius), float(drum_height), C.addressof(mat),
                                   int(movement), _ptr(pos), C.addressof(out))
        return self._new_id(rc, out)

    def add_union(self, prims, movement=0, pos=(0, 0, 0)):
        """ConvexUnionGeometry::merge of primitives, each a tuple:
        ("box", corner, dx, dy, dz, material), ("sphere", centre, r, material),
        ("cylinder", base, r, h, material), ("capsule", bot, r, h, material) or
        ("hull", points, faces, material)."""
        from ._abi import Primitive, PRIM_KINDS
        arr = (Primitive * len(prims))()
        keep = []
        for q, pr in zip(arr, prims):
            kind = pr[0]
            q.kind = PRIM_KINDS[kind]
            if kind == "hull":
                pts = _f64(pr[1])
                offs = np.zeros(len(pr[2]) + 1, dtype=np.int32)
                for i, f in enumerate(pr[2]):
                    offs[i + 1] = offs[i] + len(f)
                idx = np.ascontiguousarray([v for f in pr[2] for v in f], dtype=np.int32)
                keep += [pts, offs, idx]
                q.points, q.n_points = pts.ctypes.data, pts.size // 3
                q.face_offsets, q.face_indices, q.n_faces = offs.ctypes.data, idx.ctypes.data, len(pr[2])
                q.mat = self._mat(pr[3])
            else:
                q.p[:] = [float(x) for x in pr[1]]
                vals = [float(x) for x in pr[2:-1]] + [0.0] * 3
                q.a, q.b, q.c = vals[:3]
                q.mat = self._mat(pr[-1])
        pos = _f64(pos, 3)
        out = C.c_uint32()
        rc = self.abi.body_union(self.h, C.addressof(arr), len(prims), int(movement), _ptr(pos), C.addressof(out))
        return self._new_id(rc, out)

    def raycast(self, origins, dirs, ignore=()):
        """raycastFirstIntersection for each row of `origins` / `dirs` (unit
        directions): dict of body (0: no hit), pos, normal, dist (-1: no hit)."""
        o = _f64(origins).reshape(-1, 3)
        d = _f64(dirs).reshape(-1, 3)
        n = len(o)
        ig = np.ascontiguousarray(list(ignore) or [0], dtype=np.uint32)
        body = np.zeros(n, dtype=np.uint32)
        pos, nrm, dist = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
        self._check(self.abi.raycast(self.h, _ptr(o), _ptr(d), n, ig.ctypes.data, len(list(ignore)), body.ctypes.data,
                                     _ptr(pos), _ptr(nrm), _ptr(dist)))
        return {"body": body, "pos": pos, "normal": nrm, "dist": dist}

    def add_mesh(self, points, tris, material=None, fixed=True):
        pts = _f64(points)
        tr = np.ascontiguousarray(tris, dtype=np.int32)
        mat = self._mat(material)
        out = C.c_uint32()
        rc = self.abi.body_mesh(self.h, _ptr(pts), pts.size // 3, _ptr(tr), tr.size // 3,
                                C.addressof(mat), int(bool(fixed)), C.addressof(out))
        return self._new_id(rc, out)

    def set_velocity(self, bid, v):
        v = _f64(v, 3)
        self._check(self.abi.body_set_velocity(self.h, int(bid), _ptr(v)))

    def set_ang_velocity(self, bid, v):
        v = _f64(v, 3)
        self._check(self.abi.body_set_ang_velocity(self.h, int(bid), _ptr(v)))

    def set_orientation(self, bid, q):
        q = _f64(q, 4)
        self._check(self.abi.body_set_orientation(self.h, int(bid), _ptr(q)))

    def set_position(self, bid, p):
        p = _f64(p, 3)
        self._check(self.abi.body_set_position(self.h, int(bid), _ptr(p)))

    def set_mass(self, bid, m):
        self._check(self.abi.body_set_mass(self.h, int(bid), float(m)))

    def add_ball_socket(self, b1, b2, a1, a2, strength=15000.0):
        a1, a2 = _f64(a1, 3), _f64(a2, 3)
        out = C.c_uint32()
        self._check(self.abi.add_ball_socket(self.h, int(b1), int(b2), _ptr(a1), _ptr(a2),
                                             float(strength), C.addressof(out)))
        return out.value

    def add_distance(self, b1, b2, a1, a2, target=-1.0, strength=15000.0):
        a1, a2 = _f64(a1, 3), _f64(a2, 3)
        out = C.c_uint32()
        self._check(self.abi.add_distance(self.h, int(b1), int(b2), _ptr(a1), _ptr(a2), float(target),
                                          float(strength), C.addressof(out)))
        return out.value

    def add_weld(self, b1, b2, a1, a2, pos_strength=15000.0, rot_strength=15000.0):
        a1, a2 = _f64(a1, 3), _f64(a2, 3)
        out = C.c_uint32()
        self._check(self.abi.add_weld(self.h, int(b1), int(b2), _ptr(a1), _ptr(a2), float(pos_strength),
                                      float(rot_strength), C.addressof(out)))
        return out.value

    def add_twist_limit(self, b1, b2, ax1, ax2, min_angle, max_angle, rot_strength=15000.0):
        ax1, ax2 = _f64(ax1, 3), _f64(ax2, 3)
        out = C.c_uint32()
        self._check(self.abi.add_twist_limit(self.h, int(b1), int(b2), _ptr(ax1), _ptr(ax2), float(min_angle),
                                             float(max_angle), float(rot_strength), C.addressof(out)))
        return out.value

    def add_cone_limit(self, b1, b2, ax1, ax2, max_angle, rot_strength=15000.0):
        ax1, ax2 = _f64(ax1, 3), _f64(ax2, 3)
        out = C.c_uint32()
        self._check(self.abi.add_cone_limit(self.h, int(b1), int(b2), _ptr(ax1), _ptr(ax2), float(max_angle),
                                            float(rot_strength), C.addressof(out)))
        return out.value

    def add_spring(self, b1, b2, a1, a2, damping, stiffness, resting_length=-1.0):
        a1, a2 = _f64(a1, 3), _f64(a2, 3)
        out = C.c_uint32()
        self._check(self.abi.add_spring(self.h, int(b1), int(b2), _ptr(a1), _ptr(a2), float(damping),
                                        float(stiffness), float(resting_length), C.addressof(out)))
        return out.value

    def add_slider(self, b1, b2, a1, a2, ax1, ax2, pos_strength=15000.0, rot_strength=15000.0):
        return self._axis_joint(self.abi.add_slider, b1, b2, a1, a2, ax1, ax2, pos_strength, rot_strength)

    def add_sliding_hinge(self, b1, b2, a1, a2, ax1, ax2, pos_strength=15000.0, rot_strength=15000.0):
        return self._axis_joint(self.abi.add_sliding_hinge, b1, b2, a1, a2, ax1, ax2, pos_strength, rot_strength)

    def _axis_joint(self, fn, b1, b2, a1, a2, ax1, ax2, pos_strength, rot_strength):
        a1, a2, ax1, ax2 = (_f64(x, 3) for x in (a1, a2, ax1, ax2))
        out = C.c_uint32()
        self._check(fn(self.h, int(b1), int(b2), _ptr(a1), _ptr(a2), _ptr(ax1), _ptr(ax2), float(pos_strength),
                       float(rot_strength), C.addressof(out)))
        return out.value

    def add_hinge(self, b1, b2, a1, a2, ax1, ax2, pos_strength=15000.0, rot_strength=15000.0):
        a1, a2, ax1, ax2 = (_f64(x, 3) for x in (a1, a2, ax1, ax2))
        out = C.c_uint32()
        self._check(self.abi.add_hinge(self.h, int(b1), int(b2), _ptr(a1), _ptr(a2), _ptr(ax1), _ptr(ax2),
                                       float(pos_strength), float(rot_strength), C.addressof(out)))
        return out.value

    def add_motor(self, base_id, min_angle=-np.inf, max_angle=np.inf):
        """PhysicsEngine::addMotorConstraint on a hinge or sliding hinge id."""
        out = C.c_uint32()
        self._check(self.abi.add_motor(self.h, int(base_id), float(min_angle), float(max_angle), C.addressof(out)))
        return out.value

    def add_piston(self, base_id, min_pos=-np.inf, max_pos=np.inf):
        """PhysicsEngine::addPistonConstraint on a slider or sliding hinge id."""
        out = C.c_uint32()
        self._check(self.abi.add_piston(self.h, int(base_id), float(min_pos), float(max_pos), C.addressof(out)))
        return out.value

    # powered modes of set_motor / set_piston
    OFF, CONSTANT, TARGET_VELOCITY, TARGET_POSITION = 0, 1, 2, 3

    def set_motor(self, cid, mode, max_torque=0.0, target=0.0):
        """setMotorOff / ConstantTorque / TargetVelocity / TargetPosition."""
        self._check(self.abi.set_motor(self.h, int(cid), int(mode), float(max_torque), float(target)))

    def set_piston(self, cid, mode, max_force=0.0, target=0.0):
        """setPistonOff / ConstantForce / TargetVelocity / TargetPosition."""
        self._check(self.abi.set_piston(self.h, int(cid), int(mode), float(max_force), float(target)))

    def motor_position(self, cid):
        out = C.c_double()
        self._check(self.abi.get_motor_position(self.h, int(cid), C.addressof(out)))
        return out.value

    def piston_position(self, cid):
        out = C.c_double()
        self._check(self.abi.get_piston_position(self.h, int(cid), C.addressof(out)))
        return out.value

    # -- stepping and state -------------------------------------------------------
    def step(self, n=1):
        self._check(self.abi.step(self.h, int(n)))

    def state(self):
        n = C.c_int()
        self._check(self.abi.num_bodies(self.h, C.addressof(n)))
        n = n.value
        com = np.zeros((n, 3)); quat = np.zeros((n, 4)); vel = np.zeros((n, 3)); ang = np.zeros((n, 3))
        self._check(self.abi.get_body_state(self.h, _ptr(com), _ptr(quat), _ptr(vel), _ptr(ang)))
        return {"com": com, "quat": quat, "vel": vel, "ang_vel": ang}

    def asleep(self):
        """Per body, 1 when asleep (RigidBody::getAsleep), as int32."""
        n = C.c_int()
        self._check(self.abi.num_bodies(self.h, C.addressof(n)))
        out = np.zeros(n.value, dtype=np.int32)
        self._check(self.abi.get_asleep(self.h, _ptr(out)))
        return out

    def set_state(self, com=None, quat=None, vel=None, ang_vel=None):
        arrs = [None if a is None else _f64(a) for a in (com, quat, vel, ang_vel)]
        self._check(self.abi.set_body_state(self.h, *[_ptr(a) for a in arrs]))

    def aabbs(self):
        out = np.zeros((self.n_bodies, 6))
        self._check(self.abi.get_aabbs(self.h, _ptr(out)))
        return out

    def pairs(self):
        n = C.c_int()
        self._check(self.abi.get_pairs(self.h, None, 0, C.addressof(n)))
        out = np.zeros((max(n.value, 1), 2), dtype=np.uint32)
        self._check(self.abi.get_pairs(self.h, _ptr(out), n.value, C.addressof(n)))
        return out[: n.value]

    def contacts(self):
        n = C.c_int()
        self._check(self.abi.get_contacts(self.h, None, 0, C.addressof(n)))
        arr = (Contact * max(n.value, 1))()
        self._check(self.abi.get_contacts(self.h, C.addressof(arr), n.value, C.addressof(n)))
        return contacts_to_numpy(arr, n.value)

    def joint_state(self):
        """Warm-start state of the joints in creation order: impulses (n x 6),
        tangent bases u, w (n x 3), and aux (n x 2: a twist limit's angle, and
        1 when a cone or twist limit was reached at the last rebuild)."""
        n = C.c_int()
        self._check(self.abi.get_joint_state(self.h, None, None, None, None, C.addressof(n)))
        imp, u, w = np.zeros((n.value, 6)), np.zeros((n.value, 3)), np.zeros((n.value, 3))
        aux = np.zeros((n.value, 2))
        self._check(self.abi.get_joint_state(self.h, _ptr(imp), _ptr(u), _ptr(w), _ptr(aux), C.addressof(n)))
        return {"impulse": imp, "u": u, "w": w, "aux": aux}

    def set_joint_state(self, st):
        imp = np.ascontiguousarray(st["impulse"], dtype=np.float64)
        u = np.ascontiguousarray(st["u"], dtype=np.float64)
        w = np.ascontiguousarray(st["w"], dtype=np.float64)
        aux = np.ascontiguousarray(st["aux"], dtype=np.float64) if "aux" in st else None
        self._check(self.abi.set_joint_state(self.h, _ptr(imp), _ptr(u), _ptr(w), _ptr(aux), int(imp.shape[0])))

    def set_contacts(self, cts):
        arr = numpy_to_contacts(cts)
        self._check(self.abi.set_contacts(self.h, C.addressof(arr), len(cts["b1"])))


_CONTACT_FIELDS = [f[0] for f in Contact._fields_ if f[0] != "pad_"]


def contacts_to_numpy(arr, n):
    out = {}
    for name in _CONTACT_FIELDS:
        vals = [getattr(arr[i], name) for i in range(n)]
        if vals and isinstance(vals[0], C.Array):
            out[name] = np.array([list(v) for v in vals], dtype=np.float64).reshape(n, -1)
        else:
            out[name] = np.array(vals)
    return out


def numpy_to_contacts(cts):
    n = len(cts["b1"])
    arr = (Contact * max(n, 1))()
    for i in range(n):
        c = arr[i]
        for name in _CONTACT_FIELDS:
            v = cts[name][i]
            f = getattr(c, name)
            if isinstance(f, C.Array):
                for k in range(len(f)):
                    f[k] = float(v[k])
            else:
                setattr(c, name, type(f)(v) if not isinstance(f, float) else float(v))
    return arr
