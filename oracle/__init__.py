"""Oracle libraries for parity tests and the CPU baseline (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the product (constraintphysics_gb300) never does.

  ref()   the reference engine itself (phyz::PhysicsEngine) compiled from the
          staged copy of its sources, behind the cpref_ C ABI (ref_capi.cpp)
  port()  the CPU restatement of the contact path (cport/), behind cport_

Both export the function set of include/cpgpu.h and are driven through
constraintphysics_gb300.world.World.
"""
import ctypes
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")

if REPO not in sys.path:
    sys.path.insert(0, REPO)

from constraintphysics_gb300._abi import bind  # noqa: E402
from constraintphysics_gb300.world import World  # noqa: E402

_LIBS = {}


def build(jobs=None, reference_root=None):
    """Stage the reference sources (from `reference_root`, else from
    $CONSTRAINTPHYSICS_REFERENCE, when that checkout is present) and build both
    oracle libraries with make.  Without a checkout the sources staged earlier
    (baseline/_ref/src, which travels with the working tree) are built."""
    from oracle import stage_ref
    staged = os.path.join(REPO, "baseline", "_ref", "src")
    root = reference_root or stage_ref.reference_root()
    if root and os.path.isdir(root):
        stage_ref.stage(root)
    jobs = jobs or max(1, os.cpu_count() or 1)
    targets = ["port"] + (["ref"] if os.path.isdir(staged) else [])
    subprocess.run(["make", "-s", f"-j{jobs}", *targets], cwd=HERE, check=True)


def _load(name, prefix):
    if name not in _LIBS:
        path = os.path.join(OUT, name)
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built (run oracle.build())")
        lib = ctypes.CDLL(path)
        _LIBS[name] = bind(lib, prefix, optional=("set_body_state", "set_contacts", "get_joint_state",
                                                  "set_joint_state", "batch_create",
                                                  "batch_destroy", "batch_step", "batch_get_body_state",
                                                  "batch_info"))
        _LIBS[name]._lib = lib
    return _LIBS[name]


def ref_abi():
    return _load("libcpref.so", "cpref_")


def port_abi():
    return _load("libcport.so", "cport_")


def ref_available():
    return os.path.exists(os.path.join(OUT, "libcpref.so"))


def ref_world():
    return World(ref_abi())


def port_world():
    return World(port_abi())


def _mass_hooks():
    ref = ref_abi()._lib
    port = port_abi()._lib
    g = ref.cpref_get_mass_properties
    g.restype = ctypes.c_int
    g.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    s = port.cport_body_set_mass_properties
    s.restype = ctypes.c_int
    s.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    return g, s


def twin_worlds(scene):
    """The reference engine and the restatement built from the same scene,
    with the reference's mass properties imported into the restatement right
    after each body is created, so both start from bit-identical bodies."""
    import numpy as np
    from constraintphysics_gb300 import scenes as sc_mod
    get, put = _mass_hooks()
    r = ref_world()
    p = port_world()
    r.set_params(**scene.params)
    p.set_params(**scene.params)

    class _Twin:
        def __getattr__(self, name):
            fr, fp = getattr(r, name), getattr(p, name)

            def both(*a, **k):
                out = fr(*a, **k)
                fp(*a, **k)
                if name in ("add_hull", "add_box", "add_sphere", "add_cylinder", "add_capsule", "add_union"):
                    m = np.zeros(1); c = np.zeros(3); t = np.zeros(9)
                    assert get(r.h, out, m.ctypes.data, c.ctypes.data, t.ctypes.data) == 0
                    assert put(p.h, out, float(m[0]), c.ctypes.data, t.ctypes.data) == 0
                return out
            return both

        def set_params(self, **k):
            pass

    twin = _Twin()
    sc_mod.apply(scene, twin)
    r.constraint_ids = p.constraint_ids = twin.constraint_ids   # the same numbering on both
    return r, p


_CREATE = ("add_hull", "add_box", "add_sphere", "add_cylinder", "add_capsule", "add_union", "add_mesh")


class _Hooked:
    """Forwards world calls; runs `after(body_id, kind)` right after each body
    is created (before any later operation of the scene touches it)."""

    def __init__(self, world, after):
        self._w, self._after = world, after

    def __getattr__(self, name):
        f = getattr(self._w, name)

        def call(*a, **k):
            out = f(*a, **k)
            if name in _CREATE:
                self._after(out, name)
            return out
        return call


def capture_mass_properties(scene):
    """The reference's mass properties of every body of `scene`, read right
    after the body is created (mass, centre of mass in the geometry frame,
    3x3 tensor), with the reference world the scene was applied to."""
    import numpy as np
    from constraintphysics_gb300 import scenes as sc_mod
    get, _ = _mass_hooks()
    r = ref_world()
    r.set_params(**scene.params)
    rows = []

    def after(bid, kind):
        m, c, t = np.zeros(1), np.zeros(3), np.zeros(9)
        if kind != "add_mesh":   # meshes have no mass properties
            assert get(r.h, bid, m.ctypes.data, c.ctypes.data, t.ctypes.data) == 0
        rows.append((m[0], c, t))
    hooked = _Hooked(r, after)
    sc_mod.apply(scene, hooked)
    r.constraint_ids = getattr(hooked, "constraint_ids", [])   # apply() leaves them on the wrapper
    mass = np.array([x[0] for x in rows])
    return mass, np.array([x[1] for x in rows]), np.array([x[2] for x in rows]), r


def port_world_with_mass(scene, mass, com, tensor):
    """The restatement built from `scene`, each body's mass properties replaced
    by the given ones right after it is created."""
    import numpy as np
    from constraintphysics_gb300 import scenes as sc_mod
    _, put = _mass_hooks()
    p = port_world()
    p.set_params(**scene.params)

    def after(bid, kind):
        if kind == "add_mesh":
            return
        i = bid - 1
        c = np.ascontiguousarray(com[i], dtype=np.float64)
        t = np.ascontiguousarray(tensor[i], dtype=np.float64)
        assert put(p.h, bid, float(mass[i]), c.ctypes.data, t.ctypes.data) == 0
    hooked = _Hooked(p, after)
    sc_mod.apply(scene, hooked)
    p.constraint_ids = getattr(hooked, "constraint_ids", [])
    return p
