"""GB300 per-step contact path of the ConstraintPhysics rigid-body engine.

The compute lives in libcpgpu.so (hand-written sm_103a CUDA behind the C ABI
of include/cpgpu.h, built in-tree by constraintphysics_gb300.build).  This
package only loads that library and wraps it for Python callers:

  world()            a new PhysicsEngine-like world (constraintphysics_gb300.world.World)
  Batch(worlds)      independent worlds packed into one device batch
  Server(budget)     continuous-batching rollout server (requests = world + K steps)
  clone(world)       a copy of a world that steps exactly as the original

There is no CPU fallback: if the library is missing or no CUDA device is
present, the calls raise.
"""
import ctypes
import os

import numpy as np

from ._abi import bind
from .world import CPGPUError, World

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcpgpu.so")
_ABI = None


def lib():
    """The bound product library (raises if it was not built)."""
    global _ABI
    if _ABI is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built: run constraintphysics_gb300.build.build()")
        handle = ctypes.CDLL(LIB_PATH)
        abi = bind(handle, "cpgpu_")
        extra = {
            "batch_step_timed": [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p],
            "batch_read_state": [ctypes.c_void_p, ctypes.c_void_p],
            "batch_write_state": [ctypes.c_void_p, ctypes.c_void_p],
            "batch_profile": [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
            "batch_timeline": [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                               ctypes.c_void_p],
            "batch_launches_per_step": [ctypes.c_void_p, ctypes.c_void_p],
            "world_clone": [ctypes.c_void_p, ctypes.c_void_p],
            "server_create": [ctypes.c_int64, ctypes.c_int, ctypes.c_void_p],
            "server_destroy": [ctypes.c_void_p],
            "server_submit": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p],
            "server_advance": [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
            "server_poll": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p],
            "server_stats": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.c_void_p],
            "batch_create_tuned": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
            "batch_tune": [ctypes.c_void_p, ctypes.c_int],
            "batch_schedule": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
            "world_set_audit": [ctypes.c_void_p, ctypes.c_int],
            "world_read_audit": [ctypes.c_void_p, ctypes.c_void_p],
            "batch_set_audit": [ctypes.c_void_p, ctypes.c_int],
            "batch_read_audit": [ctypes.c_void_p, ctypes.c_void_p],
        }
        for short, args in extra.items():
            fn = getattr(handle, "cpgpu_" + short)
            fn.restype = ctypes.c_int
            fn.argtypes = args
            setattr(abi, short, fn)
        abi._lib = handle
        _ABI = abi
    return _ABI


def world():
    return World(lib())


AUDIT_FIELDS = ("px", "py", "pz", "Lx", "Ly", "Lz", "kinetic", "potential", "max_step_gain", "steps")


def _audit_dict(v):
    return {"momentum": v[0:3].copy(), "angular_momentum": v[3:6].copy(), "kinetic": float(v[6]),
            "potential": float(v[7]), "max_step_gain": float(v[8]), "steps": int(v[9])}


def set_audit(w, enabled=True):
    """Enable (or disable) the per-step FP64 momentum / energy audit of world
    `w` (cpgpu_world_set_audit)."""
    abi = lib()
    rc = abi.world_set_audit(w.h, 1 if enabled else 0)
    if rc != 0:
        raise CPGPUError(f"status {rc}: {abi.last_error().decode(errors='replace')}")


def read_audit(w):
    """The audit values of world `w` after its last step (cpgpu_world_read_audit)."""
    abi = lib()
    v = np.zeros(len(AUDIT_FIELDS))
    rc = abi.world_read_audit(w.h, v.ctypes.data)
    if rc != 0:
        raise CPGPUError(f"status {rc}: {abi.last_error().decode(errors='replace')}")
    return _audit_dict(v)


def _addr(buf):
    if hasattr(buf, "data_ptr"):          # torch tensor (e.g. pinned host memory)
        return buf.data_ptr()
    return buf.ctypes.data


class Batch:
    """Independent worlds advanced together by one launch sequence per step."""

    def __init__(self, worlds, tune_steps=0):
        """Pack `worlds`; with tune_steps > 0 the schedule is chosen by timing
        that many trial steps per candidate (cpgpu_batch_create_tuned)."""
        self.abi = lib()
        arr = (ctypes.c_void_p * len(worlds))(*[w.h.value for w in worlds])
        h = ctypes.c_void_p()
        if tune_steps > 0:
            self._check(self.abi.batch_create_tuned(arr, len(worlds), int(tune_steps), ctypes.byref(h)))
        else:
            self._check(self.abi.batch_create(arr, len(worlds), ctypes.byref(h)))
        self.h = h
        self.sizes = [w.n_bodies for w in worlds]

    def tune(self, trial_steps=3):
        """Re-choose the schedule by timing from the current state
        (cpgpu_batch_tune); the state is unchanged."""
        self._check(self.abi.batch_tune(self.h, int(trial_steps)))

    def schedule(self):
        """The batch's schedule (cpgpu_batch_schedule)."""
        sched = (ctypes.c_int * 6)()
        times = (ctypes.c_double * 2)()
        self._check(self.abi.batch_schedule(self.h, ctypes.addressof(sched), ctypes.addressof(times)))
        return {"parts": sched[0], "first_share_pct": sched[1], "rest_chain_workers_per_sm": sched[2],
                "big_island_rows": sched[3], "tuned": bool(sched[4]), "second_share_pct": sched[5],
                "tuned_ms_per_step": times[0] if times[0] >= 0 else None,
                "default_ms_per_step": times[1] if times[1] >= 0 else None}

    def _check(self, rc):
        if rc != 0:
            raise CPGPUError(f"status {rc}: {self.abi.last_error().decode(errors='replace')}")

    def step(self, n=1):
        self._check(self.abi.batch_step(self.h, int(n)))

    def step_timed(self, n=1):
        ms = ctypes.c_double()
        self._check(self.abi.batch_step_timed(self.h, int(n), ctypes.addressof(ms)))
        return ms.value

    def state(self, wi):
        n = self.sizes[wi]
        com = np.zeros((n, 3)); quat = np.zeros((n, 4)); vel = np.zeros((n, 3)); ang = np.zeros((n, 3))
        self._check(self.abi.batch_get_body_state(self.h, int(wi), com.ctypes.data, quat.ctypes.data,
                                                  vel.ctypes.data, ang.ctypes.data))
        return {"com": com, "quat": quat, "vel": vel, "ang_vel": ang}

    STAGES = ("gravity", "pairs", "narrowphase", "merge", "islands", "rows", "pgs", "integrate", "geometry")

    @property
    def n_bodies(self):
        return int(sum(self.sizes))

    def read_state(self, out=None):
        """All bodies' state, 16 floats per body (see cpgpu_batch_read_state).
        `out` may be any writable float32 buffer with 16 * n_bodies entries
        (e.g. pinned host memory); its address is passed to the library."""
        if out is None:
            out = np.empty((self.n_bodies, 16), dtype=np.float32)
        self._check(self.abi.batch_read_state(self.h, _addr(out)))
        return out

    def write_state(self, buf):
        self._check(self.abi.batch_write_state(self.h, _addr(buf)))

    def profile(self, n=1):
        ms = np.zeros(len(self.STAGES))
        counts = np.zeros(3, dtype=np.int64)
        self._check(self.abi.batch_profile(self.h, int(n), ms.ctypes.data, counts.ctypes.data))
        return dict(zip(self.STAGES, ms.tolist())), {"pairs": int(counts[0]), "contacts": int(counts[1]),
                                                      "islands": int(counts[2])}

    def timeline(self, n=1):
        """Per part, the mean ms from the step's start to each stage mark
        (cpgpu_batch_timeline): array (parts, 7 + 3 * substeps)."""
        np_, nm = ctypes.c_int(), ctypes.c_int()
        self._check(self.abi.batch_timeline(self.h, 0, None, 0, ctypes.addressof(np_), ctypes.addressof(nm)))
        out = np.zeros((np_.value, nm.value))
        self._check(self.abi.batch_timeline(self.h, int(n), out.ctypes.data, out.size, ctypes.addressof(np_),
                                            ctypes.addressof(nm)))
        return out

    def set_audit(self, enabled=True):
        """Per-step FP64 momentum / energy audit of every world (cpgpu_batch_set_audit)."""
        self._check(self.abi.batch_set_audit(self.h, 1 if enabled else 0))

    def read_audit(self):
        """Audit values per world, (n_worlds, 10) FP64 in batch order."""
        v = np.zeros((len(self.sizes), len(AUDIT_FIELDS)))
        self._check(self.abi.batch_read_audit(self.h, v.ctypes.data))
        return v

    def launches_per_step(self):
        n = ctypes.c_int()
        self._check(self.abi.batch_launches_per_step(self.h, ctypes.addressof(n)))
        return n.value

    def info(self):
        nb, nw, nc = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._check(self.abi.batch_info(self.h, ctypes.addressof(nb), ctypes.addressof(nw), ctypes.addressof(nc)))
        return {"bodies": nb.value, "worlds": nw.value, "contacts": nc.value}

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.abi.batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def clone(w):
    """A copy of world `w` (cpgpu_world_clone)."""
    abi = lib()
    h = ctypes.c_void_p()
    rc = abi.world_clone(w.h, ctypes.addressof(h))
    if rc != 0:
        raise CPGPUError(f"status {rc}: {abi.last_error().decode(errors='replace')}")
    c = World.__new__(World)
    c.abi = abi
    c.h = h
    c.n_bodies = getattr(w, "n_bodies", 0)
    return c


class Server:
    """Continuous-batching rollout server (cpgpu_server_*): submit(world, K)
    returns a token; advance(n) runs up to n batch steps, admitting waiting
    requests under the device-memory budget and re-forming the batch as
    requests complete; poll() returns the tokens completed since the last
    call, whose worlds then hold their final state."""

    def __init__(self, budget_bytes, epoch_steps=10):
        self.abi = lib()
        self.h = ctypes.c_void_p()
        self._check(self.abi.server_create(int(budget_bytes), int(epoch_steps), ctypes.addressof(self.h)))
        self._worlds = {}

    def _check(self, rc):
        if rc != 0:
            raise CPGPUError(f"status {rc}: {self.abi.last_error().decode(errors='replace')}")

    def submit(self, w, steps):
        tok = ctypes.c_uint64()
        self._check(self.abi.server_submit(self.h, w.h, int(steps), ctypes.addressof(tok)))
        self._worlds[tok.value] = w   # keep the world alive while it is served
        return tok.value

    def advance(self, max_steps):
        r, q = ctypes.c_int(), ctypes.c_int()
        self._check(self.abi.server_advance(self.h, int(max_steps), ctypes.addressof(r), ctypes.addressof(q)))
        return r.value, q.value

    def poll(self):
        out = []
        buf = (ctypes.c_uint64 * 4096)()
        n = ctypes.c_int()
        while True:
            self._check(self.abi.server_poll(self.h, ctypes.addressof(buf), 4096, ctypes.addressof(n)))
            out.extend(buf[i] for i in range(n.value))
            if n.value < 4096:
                break
        for t in out:
            self._worlds.pop(t, None)
        return out

    def stats(self):
        bs, rf, ms, db, rb = (ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64())
        self._check(self.abi.server_stats(self.h, ctypes.addressof(bs), ctypes.addressof(rf), ctypes.addressof(ms),
                                          ctypes.addressof(db), ctypes.addressof(rb)))
        return {"body_steps": bs.value, "reforms": rf.value, "reform_ms": ms.value, "device_bytes": db.value,
                "running_bodies": rb.value}

    def close(self):
        if self.h:
            self.abi.server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
