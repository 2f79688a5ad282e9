"""Stage the reference engine's sources for the oracle build.

Test infrastructure only.  Copies the reference engine's C++ sources
(ConstraintPhysics/src and Math/src) from the read-only reference checkout into
baseline/_ref/src (git-ignored: never committed, but it travels with the
working tree so a machine without the checkout can rebuild the oracle), writes
the Linux build shim, and applies documented fixes:

  * the narrowphase reads a constraint-graph node's edge list without holding
    the node mutexes (ConstraintPhysics/src/PhysicsEngine.cpp:197-210) while
    other workers insert edges under those mutexes (:285-287, :1984-1995).  With
    worker threads on Linux this crashes; the staged copy takes both node
    mutexes (in the same id order the engine already uses) around that read.
    Single-threaded results are unchanged (the lock only serialises).

  * RigidBody never initialises `no_collision` and `sleep_disabled`
    (RigidBody.h:89,122 are plain `bool` members that the constructors at
    RigidBody.cpp:13-39,41-58 leave unset), so whether a body collides at all
    depends on heap contents.  The staged copy gives both the value the API
    implies (false: setNoCollision / setSleepDisabled turn them on).

  * the static-mesh constructor (RigidBody.cpp:41-58) never sets `com_type`
    (RigidBody.h:80; the convex constructor sets PHYSICALLY_BASED), so
    getCOM() of a mesh body returns either its com or the (-1, -1, -1) of an
    invalid tracked point, depending on heap contents.  The dynamics do not
    depend on it (a mesh body is fixed: the offset cancels between a
    contact's stored local point and its rebuild, and every Jacobian term of a
    body with zero inverse mass vanishes); the reported state does.  The
    staged copy initialises it to PHYSICALLY_BASED.

The shim makes the MSVC-only code compile with g++:
  * a forced-include header that pulls in the C headers MSVC includes
    transitively, drops the libc M_PI macro (CollisionDetect.h:20 defines its
    own constant) and brings std::abs/std::isnan into the global namespace (with
    libstdc++ an unqualified abs(double) would otherwise bind to abs(int));
  * a header named `Vector` (RigidBody.h:9 includes <Vector>).

Usage: python oracle/stage_ref.py [reference_root]
The reference root is the argument, else the environment variable
CONSTRAINTPHYSICS_REFERENCE, else DEFAULT_REFERENCE_ROOT when it exists.
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
DEST = os.path.join(REPO, "baseline", "_ref")

SHIM_PRE = """// forced-include shim for building the reference engine with g++ (generated)
#include <cstdint>
#include <cmath>
#include <climits>
#include <cstring>
#include <cassert>
#include <limits>
#include <algorithm>
#undef M_PI
using std::isnan;
using std::abs;
"""

RACE_ANCHOR = "SharedConstraintsEdge* e = lock_first->getEdgeToMightBeNull(lock_second);"
RACE_FIX = (
    "lock_first->mutex.lock(); lock_second->mutex.lock(); "
    "SharedConstraintsEdge* e = lock_first->getEdgeToMightBeNull(lock_second); "
    "if (e != nullptr) { surface1id = e->cached_surfaceid1; surface2id = e->cached_surfaceid2; } "
    "else { surface1id = -1; surface2id = -1; } "
    "lock_first->mutex.unlock(); lock_second->mutex.unlock(); "
    "e = nullptr;"
)


def stage(ref_root):
    src_engine = os.path.join(ref_root, "ConstraintPhysics", "src")
    src_math = os.path.join(ref_root, "Math", "src")
    if not (os.path.isdir(src_engine) and os.path.isdir(src_math)):
        raise SystemExit(f"reference sources not found under {ref_root}")
    out_src = os.path.join(DEST, "src")
    if os.path.isdir(out_src):
        shutil.rmtree(out_src)
    for sub, srcdir in (("ConstraintPhysics/src", src_engine), ("Math/src", src_math)):
        d = os.path.join(out_src, sub)
        os.makedirs(d, exist_ok=True)
        for name in sorted(os.listdir(srcdir)):
            if name.endswith((".h", ".cpp")):
                shutil.copy2(os.path.join(srcdir, name), os.path.join(d, name))
                os.chmod(os.path.join(d, name), 0o644)
    pe = os.path.join(out_src, "ConstraintPhysics/src/PhysicsEngine.cpp")
    text = open(pe, encoding="utf-8", errors="surrogateescape").read()
    if text.count(RACE_ANCHOR) != 1:
        raise SystemExit("race-fix anchor not found exactly once in PhysicsEngine.cpp")
    # After the fix `e` is nulled, so the original if/else that follows
    # re-assigns the same ids only when e != nullptr; keep ids from the locked read.
    text = text.replace(RACE_ANCHOR, RACE_FIX)
    old_tail = ("if (e != nullptr) {\n\t\t\t\t\t\t\t\t\tsurface1id = e->cached_surfaceid1;\n"
                "\t\t\t\t\t\t\t\t\tsurface2id = e->cached_surfaceid2;\n\t\t\t\t\t\t\t\t}\n"
                "\t\t\t\t\t\t\t\telse {\n\t\t\t\t\t\t\t\t\tsurface1id = -1;\n"
                "\t\t\t\t\t\t\t\t\tsurface2id = -1;\n\t\t\t\t\t\t\t\t}")
    if text.count(old_tail) != 1:
        raise SystemExit("race-fix tail not found exactly once in PhysicsEngine.cpp")
    text = text.replace(old_tail, "")
    open(pe, "w", encoding="utf-8", errors="surrogateescape").write(text)
    rb = os.path.join(out_src, "ConstraintPhysics/src/RigidBody.h")
    text = open(rb, encoding="utf-8", errors="surrogateescape").read()
    for member in ("bool no_collision;", "bool sleep_disabled;"):
        if text.count(member) != 1:
            raise SystemExit(f"anchor {member!r} not found exactly once in RigidBody.h")
        text = text.replace(member, member[:-1] + " = false;")
    member = "CenterOfMassType com_type;"
    if text.count(member) != 1:
        raise SystemExit(f"anchor {member!r} not found exactly once in RigidBody.h")
    text = text.replace(member, "CenterOfMassType com_type = PHYSICALLY_BASED;")
    open(rb, "w", encoding="utf-8", errors="surrogateescape").write(text)
    shim = os.path.join(DEST, "shim")
    os.makedirs(shim, exist_ok=True)
    open(os.path.join(shim, "pre.h"), "w").write(SHIM_PRE)
    open(os.path.join(shim, "Vector"), "w").write("#include <vector>\n")
    with open(os.path.join(DEST, "STAGED_FROM"), "w") as f:
        f.write(os.path.abspath(ref_root) + "\n")
    return out_src


# where this build's read-only reference checkout lives when
# CONSTRAINTPHYSICS_REFERENCE does not say otherwise
DEFAULT_REFERENCE_ROOT = "/root/reference"


def reference_root():
    """The reference checkout to stage from: $CONSTRAINTPHYSICS_REFERENCE, else
    the default checkout location; None when neither is a directory (a
    machine that only has the staged copy)."""
    for root in (os.environ.get("CONSTRAINTPHYSICS_REFERENCE"), DEFAULT_REFERENCE_ROOT):
        if root and os.path.isdir(root):
            return root
    return None


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else reference_root()
    if not root:
        raise SystemExit("usage: stage_ref.py REFERENCE_ROOT (or set CONSTRAINTPHYSICS_REFERENCE)")
    print(stage(root))
