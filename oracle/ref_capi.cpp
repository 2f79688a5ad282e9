// ref_capi.cpp — test infrastructure: exposes the reference engine itself
// (phyz::PhysicsEngine, built from the staged reference sources) through the
// same C function set as include/cpgpu.h, with the prefix cpref_.  Tests and the
// CPU-baseline leg of bench.py load it to produce reference outputs on the same
// inputs as the device path.  Nothing in the product links or loads this file.
//
// Engine internals (the constraint graph and the broadphase tree) are reached
// through the friend declaration `friend class DebugDemo;`
// (ConstraintPhysics/src/PhysicsEngine.h:158).
#include <vector>
#include <set>
#include <map>
#include <functional>
#include <unordered_map>
#include <mutex>
#include <thread>
#include <atomic>
#include <algorithm>
#include <string>
#include <cstdint>
#include <cstring>
#include <cassert>
#include <chrono>
#include <cinttypes>
#include <cmath>
#include <condition_variable>
#include <stack>
#include <sstream>
#include <iostream>
#include <limits>

// RigidBody keeps its mass properties private and befriends only
// PhysicsEngine; this test harness reads them directly.  The standard headers
// above are included first so the access override only touches the engine's.
#define private public
#include "PhysicsEngine.h"
#include "Geometry.h"
#undef private

// odr-use of the in-class constant needs one out-of-line definition
// (HolonomicBlockSolver.h:35, used by reference at HolonomicBlockSolver.cpp:105).
const int phyz::HolonomicSystem::BLOCK_EMPTY;

extern "C" {
#include "../include/cpgpu.h"
}

namespace {
struct RefWorld {
    phyz::PhysicsEngine engine;
    std::vector<phyz::RigidBody*> bodies;   // index = id - 1
    std::vector<uint32_t> last_pairs;       // flattened (lo, hi)
    std::unordered_map<uint32_t, phyz::ConstraintID> cids;   // returned id -> the engine's ConstraintID
};

thread_local std::string g_err;

int fail(const char* msg) { g_err = msg; return CPGPU_ERR_INVALID_ARG; }

phyz::Material to_mat(const cpgpu_material* m) {
    phyz::Material out = phyz::Material::default_material();
    if (m) {
        out.density = m->density;
        out.restitution = m->restitution;
        out.kinetic_friction_coeff = m->kinetic_friction;
        out.static_friction_coeff = m->static_friction;
    }
    return out;
}

mthz::Vec3 v3(const double* p) { return p ? mthz::Vec3(p[0], p[1], p[2]) : mthz::Vec3(); }

int finish_body(RefWorld* w, phyz::RigidBody* r, uint32_t* out_id) {
    w->bodies.push_back(r);
    if (out_id) *out_id = r->getID();
    return CPGPU_OK;
}

phyz::RigidBody* body(RefWorld* w, uint32_t id) {
    if (id == 0 || id > w->bodies.size()) return nullptr;
    return w->bodies[id - 1];
}
}  // namespace

// Friend of phyz::PhysicsEngine (PhysicsEngine.h:158; the unqualified friend
// declaration names phyz::DebugDemo): reads private state.
namespace phyz {
class DebugDemo {
public:
    static void candidate_pairs(phyz::PhysicsEngine& e, std::vector<uint32_t>& out) {
        // Same tree update as PhysicsEngine::timeStep (PhysicsEngine.cpp:103-105);
        // a second update with unchanged bounds inside timeStep does not alter
        // the tree, so the step that follows is unaffected.
        for (phyz::RigidBody* b : e.bodies) {
            e.aabb_tree.update(b, b->getMovementType() != phyz::RigidBody::DYNAMIC, b->getID(), b->getAABB());
        }
        std::vector<phyz::Pair<phyz::RigidBody*>> pairs = e.aabb_tree.getAllCollisionCandidates();
        std::vector<std::pair<uint32_t, uint32_t>> ps;
        for (auto& p : pairs) {
            uint32_t a = p.t1->getID(), b = p.t2->getID();
            ps.push_back({std::min(a, b), std::max(a, b)});
        }
        std::sort(ps.begin(), ps.end());
        out.clear();
        for (auto& p : ps) { out.push_back(p.first); out.push_back(p.second); }
    }

    static int contacts(phyz::PhysicsEngine& e, cpgpu_contact* out, int cap, int* n) {
        using Edge = phyz::PhysicsEngine::SharedConstraintsEdge;
        std::set<Edge*> seen;
        std::vector<std::pair<std::pair<uint32_t, uint32_t>, Edge*>> edges;
        for (auto& kv : e.constraint_graph_nodes) {
            for (Edge* ed : kv.second->constraints) {
                if (seen.insert(ed).second) {
                    uint32_t a = ed->n1->b->getID(), b = ed->n2->b->getID();
                    edges.push_back({{std::min(a, b), std::max(a, b)}, ed});
                }
            }
        }
        std::sort(edges.begin(), edges.end(),
                  [](const auto& x, const auto& y) { return x.first < y.first; });
        int count = 0;
        for (auto& pe : edges) {
            for (phyz::PersistentConstraint* pc : pe.second->constraints) {
                if (pc->getId().getType() != phyz::ConstraintID::CONTACT) continue;
                phyz::Contact* c = static_cast<phyz::Contact*>(pc);
                if (count < cap && out) {
                    cpgpu_contact& o = out[count];
                    std::memset(&o, 0, sizeof(o));
                    o.b1 = c->b1->getID();
                    o.b2 = c->b2->getID();
                    o.live = c->is_live_contact ? 1u : 0u;
                    o.memory_life = c->memory_life;
                    o.magic_c = c->magic.cID;
                    o.magic_b = c->magic.bID;
                    const mthz::Vec3* vs[3] = {&c->contact_pos_local_b1, &c->contact_pos_local_b2, &c->normal_local_b1};
                    double* ds[3] = {o.p_local_b1, o.p_local_b2, o.n_local_b1};
                    for (int k = 0; k < 3; k++) { ds[k][0] = vs[k]->x; ds[k][1] = vs[k]->y; ds[k][2] = vs[k]->z; }
                    o.pen_depth = c->pen_depth;
                    o.bounce = c->bounce;
                    o.friction_coeff = c->friction_coeff;
                    o.normal_impulse = c->contact.impulse.v[0];
                    o.friction_impulse[0] = c->friction.impulse.v[0];
                    o.friction_impulse[1] = c->friction.impulse.v[1];
                    o.friction_u[0] = c->friction.u.x; o.friction_u[1] = c->friction.u.y; o.friction_u[2] = c->friction.u.z;
                    o.friction_w[0] = c->friction.w.x; o.friction_w[1] = c->friction.w.y; o.friction_w[2] = c->friction.w.z;
                    o.static_ready = c->friction.getStaticReady() ? 1u : 0u;
                }
                count++;
            }
        }
        *n = count;
        return CPGPU_OK;
    }
};
}  // namespace phyz

extern "C" {

const char* cpref_last_error(void) { return g_err.c_str(); }

int cpref_world_create(cpgpu_world** out) {
    if (!out) return fail("null out");
    *out = reinterpret_cast<cpgpu_world*>(new RefWorld());
    return CPGPU_OK;
}
int cpref_world_destroy(cpgpu_world* w) { delete reinterpret_cast<RefWorld*>(w); return CPGPU_OK; }

#define RW reinterpret_cast<RefWorld*>(w)
int cpref_set_step_time(cpgpu_world* w, double dt) { RW->engine.setStep_time(dt); return CPGPU_OK; }
int cpref_set_gravity(cpgpu_world* w, double x, double y, double z) { RW->engine.setGravity(mthz::Vec3(x, y, z)); return CPGPU_OK; }
int cpref_set_substep_count(cpgpu_world* w, int s) { RW->engine.setSubstepCount(s); return CPGPU_OK; }
int cpref_set_pgs_iterations(cpgpu_world* w, int v, int p, int h) { RW->engine.setPGSIterations(v, p, h); return CPGPU_OK; }
int cpref_set_sleeping_enabled(cpgpu_world* w, int e) { RW->engine.setSleepingEnabled(e != 0); return CPGPU_OK; }
int cpref_set_warm_start_disabled(cpgpu_world* w, int d) { RW->engine.setWarmStartDisabled(d != 0); return CPGPU_OK; }
int cpref_set_global_cfm(cpgpu_world* w, double c) { RW->engine.setGlobalConstraintForceMixing(c); return CPGPU_OK; }
int cpref_set_angle_vel_update_tick_count(cpgpu_world* w, int n) { RW->engine.setAngleVelUpdateTickCount(n); return CPGPU_OK; }
int cpref_set_internal_gyro_forces_disabled(cpgpu_world* w, int d) { RW->engine.setInternalGyroscopicForcesDisabled(d != 0); return CPGPU_OK; }
// PhysicsEngine::enableMultithreading (PhysicsEngine.cpp:15-20); CPU baseline only.
int cpref_enable_multithreading(cpgpu_world* w, int n) {
    if (n >= 1) RW->engine.enableMultithreading(n); else RW->engine.disableMultithreading();
    return CPGPU_OK;
}

int cpref_body_hull(cpgpu_world* w, const double* points, int n_points, const int* face_offsets,
                    const int* face_indices, int n_faces, const cpgpu_material* mat, int movement,
                    const double pos[3], uint32_t* out_id) {
    if (n_points < 4 || n_faces < 4) return fail("hull needs >= 4 points and faces");
    std::vector<mthz::Vec3> pts(n_points);
    for (int i = 0; i < n_points; i++) pts[i] = mthz::Vec3(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
    std::vector<std::vector<uint32_t>> faces(n_faces);
    for (int f = 0; f < n_faces; f++)
        for (int k = face_offsets[f]; k < face_offsets[f + 1]; k++) faces[f].push_back((uint32_t)face_indices[k]);
    phyz::Polyhedron poly(pts, faces);
    phyz::ConvexUnionGeometry g(phyz::ConvexPrimitive((const phyz::ConvexGeometry&)poly, to_mat(mat)));
    phyz::RigidBody* r = RW->engine.createRigidBody(g, (phyz::RigidBody::MovementType)movement, v3(pos));
    return finish_body(RW, r, out_id);
}

int cpref_body_box(cpgpu_world* w, const double corner[3], double dx, double dy, double dz,
                   const cpgpu_material* mat, int movement, const double pos[3], uint32_t* out_id) {
    phyz::ConvexUnionGeometry g = phyz::ConvexUnionGeometry::box(v3(corner), dx, dy, dz, to_mat(mat));
    phyz::RigidBody* r = RW->engine.createRigidBody(g, (phyz::RigidBody::MovementType)movement, v3(pos));
    return finish_body(RW, r, out_id);
}

int cpref_body_sphere(cpgpu_world* w, const double center[3], double radius, const cpgpu_material* mat,
                      int movement, const double pos[3], uint32_t* out_id) {
    phyz::ConvexUnionGeometry g = phyz::ConvexUnionGeometry::sphere(v3(center), radius, to_mat(mat));
    phyz::RigidBody* r = RW->engine.createRigidBody(g, (phyz::RigidBody::MovementType)movement, v3(pos));
    return finish_body(RW, r, out_id);
}

int cpref_body_cylinder(cpgpu_world* w, const double base[3], double radius, double height,
                        const cpgpu_material* mat, int movement, const double pos[3], uint32_t* out_id) {
    phyz::ConvexUnionGeometry g = phyz::ConvexUnionGeometry::cylinder(v3(base), radius, height, to_mat(mat));
    phyz::RigidBody* r = RW->engine.createRigidBody(g, (phyz::RigidBody::MovementType)movement, v3(pos));
    return finish_body(RW, r, out_id);
}

int cpref_body_capsule(cpgpu_world* w, const double bot[3], double radius, double drum_height,
                       const cpgpu_material* mat, int movement, const double pos[3], uint32_t* out_id) {
    phyz::ConvexUnionGeometry g = phyz::ConvexUnionGeometry::capsule(v3(bot), radius, drum_height, to_mat(mat));
    phyz::RigidBody* r = RW->engine.createRigidBody(g, (phyz::RigidBody::MovementType)movement, v3(pos));
    return finish_body(RW, r, out_id);
}

// ConvexUnionGeometry::merge of the primitives in order (Geometry.cpp:540-550)
int cpref_body_union(cpgpu_world* w, const cpgpu_primitive* prims, int n, int movement, const double pos[3],
                     uint32_t* out_id) {
    if (!prims || n < 1) return fail("a union needs >= 1 primitive");
    phyz::ConvexUnionGeometry g;
    for (int i = 0; i < n; i++) {
        const cpgpu_primitive& q = prims[i];
        phyz::Material m = to_mat(&q.mat);
        phyz::ConvexUnionGeometry gi;
        switch (q.kind) {
        case CPGPU_PRIM_HULL: {
            std::vector<mthz::Vec3> pts(q.n_points);
            for (int k = 0; k < q.n_points; k++) pts[k] = mthz::Vec3(q.points[3 * k], q.points[3 * k + 1], q.points[3 * k + 2]);
            std::vector<std::vector<uint32_t>> faces(q.n_faces);
            for (int f = 0; f < q.n_faces; f++)
                for (int k = q.face_offsets[f]; k < q.face_offsets[f + 1]; k++) faces[f].push_back((uint32_t)q.face_indices[k]);
            phyz::Polyhedron poly(pts, faces);
            gi = phyz::ConvexUnionGeometry(phyz::ConvexPrimitive((const phyz::ConvexGeometry&)poly, m));
            break;
        }
        case CPGPU_PRIM_BOX: gi = phyz::ConvexUnionGeometry::box(v3(q.p), q.a, q.b, q.c, m); break;
        case CPGPU_PRIM_SPHERE: gi = phyz::ConvexUnionGeometry::sphere(v3(q.p), q.a, m); break;
        case CPGPU_PRIM_CYLINDER: gi = phyz::ConvexUnionGeometry::cylinder(v3(q.p), q.a, q.b, m); break;
        case CPGPU_PRIM_CAPSULE: gi = phyz::ConvexUnionGeometry::capsule(v3(q.p), q.a, q.b, m); break;
        default: return fail("bad primitive kind");
        }
        g = i == 0 ? gi : phyz::ConvexUnionGeometry::merge(g, gi);
    }
    phyz::RigidBody* r = RW->engine.createRigidBody(g, (phyz::RigidBody::MovementType)movement, v3(pos));
    return finish_body(RW, r, out_id);
}

int cpref_body_mesh(cpgpu_world* w, const double* points, int n_points, const int* tris, int n_tris,
                    const cpgpu_material* mat, int fixed, uint32_t* out_id) {
    phyz::MeshInput in;
    in.points.resize(n_points);
    for (int i = 0; i < n_points; i++) in.points[i] = mthz::Vec3(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
    phyz::Material m = to_mat(mat);
    for (int t = 0; t < n_tris; t++)
        in.triangle_indices.push_back(phyz::TriIndices{(uint32_t)tris[3 * t], (uint32_t)tris[3 * t + 1], (uint32_t)tris[3 * t + 2], m});
    phyz::StaticMeshGeometry g(in);
    phyz::RigidBody* r = RW->engine.createRigidBody(g, fixed != 0);
    return finish_body(RW, r, out_id);
}

int cpref_body_set_velocity(cpgpu_world* w, uint32_t id, const double v[3]) {
    phyz::RigidBody* r = body(RW, id); if (!r) return fail("bad body id");
    r->setVel(v3(v)); return CPGPU_OK;
}
int cpref_body_set_ang_velocity(cpgpu_world* w, uint32_t id, const double v[3]) {
    phyz::RigidBody* r = body(RW, id); if (!r) return fail("bad body id");
    r->setAngVel(v3(v)); return CPGPU_OK;
}
int cpref_body_set_orientation(cpgpu_world* w, uint32_t id, const double q[4]) {
    phyz::RigidBody* r = body(RW, id); if (!r) return fail("bad body id");
    r->setOrientation(mthz::Quaternion(q[0], q[1], q[2], q[3])); return CPGPU_OK;
}
int cpref_body_set_position(cpgpu_world* w, uint32_t id, const double p[3]) {
    phyz::RigidBody* r = body(RW, id); if (!r) return fail("bad body id");
    r->setToPosition(v3(p)); return CPGPU_OK;
}
int cpref_body_set_mass(cpgpu_world* w, uint32_t id, double m) {
    phyz::RigidBody* r = body(RW, id); if (!r) return fail("bad body id");
    r->setMass(m); return CPGPU_OK;
}

int cpref_add_ball_socket(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                          double strength, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addBallSocketConstraint(r1, r2, v3(a1), v3(a2), strength);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_distance(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                       double target, double strength, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addDistanceConstraint(r1, r2, v3(a1), v3(a2), target, strength);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_weld(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double ps,
                   double rs, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addWeldConstraint(r1, r2, v3(a1), v3(a2), ps, rs);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_twist_limit(cpgpu_world* w, uint32_t b1, uint32_t b2, const double ax1[3], const double ax2[3],
                          double min_angle, double max_angle, double rs, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addTwistLimitConstraint(r1, r2, v3(ax1), v3(ax2), min_angle, max_angle, rs);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_cone_limit(cpgpu_world* w, uint32_t b1, uint32_t b2, const double ax1[3], const double ax2[3],
                         double max_angle, double rs, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addConeLimitConstraint(r1, r2, v3(ax1), v3(ax2), max_angle, rs);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_spring(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                     double damping, double stiffness, double rest, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addSpring(r1, r2, v3(a1), v3(a2), damping, stiffness, rest);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_slider(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                     const double ax1[3], const double ax2[3], double ps, double rs, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addSliderConstraint(r1, r2, v3(a1), v3(a2), v3(ax1), v3(ax2), ps, rs);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_sliding_hinge(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                            const double ax1[3], const double ax2[3], double ps, double rs, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addSlidingHingeConstraint(r1, r2, v3(a1), v3(a2), v3(ax1), v3(ax2), ps, rs);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_hinge(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                    const double ax1[3], const double ax2[3], double ps, double rs, uint32_t* out_id) {
    phyz::RigidBody* r1 = body(RW, b1); phyz::RigidBody* r2 = body(RW, b2);
    if (!r1 || !r2) return fail("bad body id");
    phyz::ConstraintID id = RW->engine.addHingeConstraint(r1, r2, v3(a1), v3(a2), v3(ax1), v3(ax2), ps, rs);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}

// PhysicsEngine::addMotorConstraint / addPistonConstraint and the powered
// constraints' setters and getters
int cpref_add_motor(cpgpu_world* w, uint32_t base, double min_angle, double max_angle, uint32_t* out_id) {
    auto it = RW->cids.find(base);
    if (it == RW->cids.end()) return fail("bad constraint id");
    phyz::ConstraintID id = RW->engine.addMotorConstraint(it->second, min_angle, max_angle);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_add_piston(cpgpu_world* w, uint32_t base, double min_pos, double max_pos, uint32_t* out_id) {
    auto it = RW->cids.find(base);
    if (it == RW->cids.end()) return fail("bad constraint id");
    phyz::ConstraintID id = RW->engine.addPistonConstraint(it->second, min_pos, max_pos);
    RW->cids[id.getID()] = id;
    if (out_id) *out_id = id.getID();
    return CPGPU_OK;
}
int cpref_set_motor(cpgpu_world* w, uint32_t cid, int mode, double max_torque, double target) {
    auto it = RW->cids.find(cid);
    if (it == RW->cids.end()) return fail("bad constraint id");
    switch (mode) {
        case 0: RW->engine.setMotorOff(it->second); break;
        case 1: RW->engine.setMotorConstantTorque(it->second, max_torque); break;
        case 2: RW->engine.setMotorTargetVelocity(it->second, max_torque, target); break;
        case 3: RW->engine.setMotorTargetPosition(it->second, max_torque, target); break;
        default: return fail("bad mode");
    }
    return CPGPU_OK;
}
int cpref_set_piston(cpgpu_world* w, uint32_t cid, int mode, double max_force, double target) {
    auto it = RW->cids.find(cid);
    if (it == RW->cids.end()) return fail("bad constraint id");
    switch (mode) {
        case 0: RW->engine.setPistonOff(it->second); break;
        case 1: RW->engine.setPistonConstantForce(it->second, max_force); break;
        case 2: RW->engine.setPistonTargetVelocity(it->second, max_force, target); break;
        case 3: RW->engine.setPistonTargetPosition(it->second, max_force, target); break;
        default: return fail("bad mode");
    }
    return CPGPU_OK;
}
int cpref_get_motor_position(cpgpu_world* w, uint32_t cid, double* out) {
    auto it = RW->cids.find(cid);
    if (it == RW->cids.end()) return fail("bad constraint id");
    *out = RW->engine.getMotorAngularPosition(it->second);
    return CPGPU_OK;
}
int cpref_get_piston_position(cpgpu_world* w, uint32_t cid, double* out) {
    auto it = RW->cids.find(cid);
    if (it == RW->cids.end()) return fail("bad constraint id");
    *out = RW->engine.getPistonPosition(it->second);
    return CPGPU_OK;
}

int cpref_step(cpgpu_world* w, int n_steps) {
    for (int i = 0; i < n_steps; i++) {
        phyz::DebugDemo::candidate_pairs(RW->engine, RW->last_pairs);
        RW->engine.timeStep();
    }
    return CPGPU_OK;
}
// Step without recording the candidate pairs (used for timing).
int cpref_step_untraced(cpgpu_world* w, int n_steps) {
    for (int i = 0; i < n_steps; i++) RW->engine.timeStep();
    return CPGPU_OK;
}

int cpref_num_bodies(cpgpu_world* w, int* n) { *n = (int)RW->bodies.size(); return CPGPU_OK; }

// raycastFirstIntersection per ray, after refreshing the broadphase tree's
// leaves to the bodies' current AABBs (the same update timeStep makes first,
// PhysicsEngine.cpp:103-105; without it the leaves hold the AABBs of the
// start of the last step)
int cpref_raycast(cpgpu_world* w, const double* origins, const double* dirs, int n_rays, const uint32_t* ignore,
                  int n_ignore, uint32_t* hit_body, double* hit_pos, double* hit_normal, double* hit_dist) {
    std::vector<uint32_t> tmp;
    phyz::DebugDemo::candidate_pairs(RW->engine, tmp);
    std::vector<phyz::RigidBody*> ig;
    for (int k = 0; k < n_ignore; k++)
        if (phyz::RigidBody* r = body(RW, ignore[k])) ig.push_back(r);
    for (int k = 0; k < n_rays; k++) {
        phyz::RayHitInfo h = RW->engine.raycastFirstIntersection(v3(origins + 3 * k), v3(dirs + 3 * k), ig);
        if (hit_body) hit_body[k] = h.did_hit ? h.hit_object->getID() : 0;
        const double p[3] = {h.hit_position.x, h.hit_position.y, h.hit_position.z};
        const double n[3] = {h.surface_normal.x, h.surface_normal.y, h.surface_normal.z};
        for (int i = 0; i < 3; i++) {
            if (hit_pos) hit_pos[3 * k + i] = h.did_hit ? p[i] : 0;
            if (hit_normal) hit_normal[3 * k + i] = h.did_hit ? n[i] : 0;
        }
        if (hit_dist) hit_dist[k] = h.did_hit ? h.hit_distance : -1;
    }
    return CPGPU_OK;
}

int cpref_get_body_state(cpgpu_world* w, double* com, double* quat, double* vel, double* ang_vel) {
    for (size_t i = 0; i < RW->bodies.size(); i++) {
        phyz::RigidBody* r = RW->bodies[i];
        mthz::Vec3 c = r->getCOM(); mthz::Quaternion q = r->getOrientation();
        mthz::Vec3 v = r->getVel(); mthz::Vec3 a = r->getAngVel();
        if (com) { com[3 * i] = c.x; com[3 * i + 1] = c.y; com[3 * i + 2] = c.z; }
        if (quat) { quat[4 * i] = q.r; quat[4 * i + 1] = q.i; quat[4 * i + 2] = q.j; quat[4 * i + 3] = q.k; }
        if (vel) { vel[3 * i] = v.x; vel[3 * i + 1] = v.y; vel[3 * i + 2] = v.z; }
        if (ang_vel) { ang_vel[3 * i] = a.x; ang_vel[3 * i + 1] = a.y; ang_vel[3 * i + 2] = a.z; }
    }
    return CPGPU_OK;
}

int cpref_get_asleep(cpgpu_world* w, int* flags) {
    for (size_t i = 0; i < RW->bodies.size(); i++) flags[i] = RW->bodies[i]->getAsleep() ? 1 : 0;
    return CPGPU_OK;
}

int cpref_get_aabbs(cpgpu_world* w, double* out) {
    for (size_t i = 0; i < RW->bodies.size(); i++) {
        phyz::AABB a = RW->bodies[i]->getAABB();
        double* o = out + 6 * i;
        o[0] = a.min.x; o[1] = a.min.y; o[2] = a.min.z; o[3] = a.max.x; o[4] = a.max.y; o[5] = a.max.z;
    }
    return CPGPU_OK;
}

int cpref_get_pairs(cpgpu_world* w, uint32_t* pairs, int cap, int* n) {
    int np = (int)(RW->last_pairs.size() / 2);
    *n = np;
    for (int i = 0; i < np && i < cap; i++) { pairs[2 * i] = RW->last_pairs[2 * i]; pairs[2 * i + 1] = RW->last_pairs[2 * i + 1]; }
    return CPGPU_OK;
}

// Mass properties of body `id` as computed by the reference at creation:
// mass, centre of mass in the geometry's own frame (minus the local origin,
// RigidBody.cpp:32) and the COM-frame inertia tensor (row-major).
int cpref_get_mass_properties(cpgpu_world* w, uint32_t id, double* mass, double* com_geom, double* tensor) {
    phyz::RigidBody* r = body(RW, id); if (!r) return fail("bad body id");
    *mass = r->mass;
    com_geom[0] = -r->local_coord_origin.x; com_geom[1] = -r->local_coord_origin.y; com_geom[2] = -r->local_coord_origin.z;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) tensor[3 * i + j] = r->reference_tensor.v[i][j];
    return CPGPU_OK;
}

int cpref_get_contacts(cpgpu_world* w, cpgpu_contact* out, int cap, int* n) {
    return phyz::DebugDemo::contacts(RW->engine, out, cap, n);
}
#undef RW

}  // extern "C"
