// cpgpu_engine.hpp — header-only C++ facade over the cpgpu C ABI with the
// method names of the reference's phyz::PhysicsEngine
// (ConstraintPhysics/src/PhysicsEngine.h:60-161), so scene code written for
// the reference compiles against the device path with a namespace change.
//
// Differences a caller sees:
//   * bodies are addressed by id (RigidBody handles wrap the id);
//   * errors that the reference reports with assert() throw cpgpu::Error;
//   * on the device: convex hulls, boxes, spheres, cylinders, capsules and
//     fixed static triangle meshes; ball-socket, hinge, distance, weld,
//     slider and sliding-hinge joints, cone and twist limits, motors,
//     pistons and springs; sleeping; bodies of several primitives
//     (ConvexUnionGeometry::merge).
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "cpgpu.h"

namespace cpgpu {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != CPGPU_OK) throw Error(rc, std::string("cpgpu: ") + cpgpu_last_error());
}

struct Vec3 {
    double x = 0, y = 0, z = 0;
    Vec3() {}
    Vec3(double a, double b, double c) : x(a), y(b), z(c) {}
    const double* data() const { return &x; }
};
struct Quaternion {
    double r = 1, i = 0, j = 0, k = 0;
    Quaternion() {}
    Quaternion(double a, double b, double c, double d) : r(a), i(b), j(c), k(d) {}
};

enum MovementType { DYNAMIC = CPGPU_DYNAMIC, FIXED = CPGPU_FIXED, KINEMATIC = CPGPU_KINEMATIC };

// Material (ConvexPrimitive.h:17-34)
struct Material {
    double density = 1.0, restitution = 0.3, kinetic_friction_coeff = 0.6, static_friction_coeff = 1.1;
    static Material default_material() { return Material(); }
    static Material modified_density(double d) { Material m; m.density = d; return m; }
    cpgpu_material c() const { return cpgpu_material{density, restitution, kinetic_friction_coeff, static_friction_coeff}; }
};

// One convex primitive of a ConvexUnionGeometry (ConvexPrimitive.h:36-60)
struct ConvexPrimitive {
    enum Kind { HULL, BOX, SPHERE, CYLINDER, CAPSULE } kind = HULL;
    std::vector<Vec3> points;
    std::vector<std::vector<int>> faces;
    Vec3 corner;                 // box corner, sphere centre, cylinder base, capsule bottom-sphere centre
    double dx = 0, dy = 0, dz = 0;
    double radius = 0, height = 0;   // sphere / cylinder / capsule (capsule: drum height)
    Material material;
};

// ConvexUnionGeometry (Geometry.h:9-47): a list of convex primitives that one
// rigid body is made of
struct ConvexUnionGeometry {
    std::vector<ConvexPrimitive> polyhedra;

    static ConvexUnionGeometry of(const ConvexPrimitive& c) {
        ConvexUnionGeometry g;
        g.polyhedra.push_back(c);
        return g;
    }
    static ConvexUnionGeometry sphere(Vec3 center, double radius, Material m = Material::default_material()) {
        ConvexPrimitive c;
        c.kind = ConvexPrimitive::SPHERE; c.corner = center; c.radius = radius; c.material = m;
        return of(c);
    }
    static ConvexUnionGeometry cylinder(Vec3 pos, double radius, double height, Material m = Material::default_material()) {
        ConvexPrimitive c;
        c.kind = ConvexPrimitive::CYLINDER; c.corner = pos; c.radius = radius; c.height = height; c.material = m;
        return of(c);
    }
    static ConvexUnionGeometry capsule(Vec3 bot_sphere_center, double radius, double drum_height,
                                       Material m = Material::default_material()) {
        ConvexPrimitive c;
        c.kind = ConvexPrimitive::CAPSULE; c.corner = bot_sphere_center; c.radius = radius; c.height = drum_height;
        c.material = m;
        return of(c);
    }
    static ConvexUnionGeometry box(Vec3 pos, double dx, double dy, double dz, Material m = Material::default_material()) {
        ConvexPrimitive c;
        c.kind = ConvexPrimitive::BOX; c.corner = pos; c.dx = dx; c.dy = dy; c.dz = dz; c.material = m;
        return of(c);
    }
    static ConvexUnionGeometry polyhedron(const std::vector<Vec3>& pts, const std::vector<std::vector<int>>& faces,
                                          Material m = Material::default_material()) {
        ConvexPrimitive c;
        c.kind = ConvexPrimitive::HULL; c.points = pts; c.faces = faces; c.material = m;
        return of(c);
    }
    // ConvexUnionGeometry::merge (Geometry.cpp:540-550): g1's primitives, then g2's
    static ConvexUnionGeometry merge(const ConvexUnionGeometry& g1, const ConvexUnionGeometry& g2) {
        ConvexUnionGeometry g = g1;
        g.polyhedra.insert(g.polyhedra.end(), g2.polyhedra.begin(), g2.polyhedra.end());
        return g;
    }
    ConvexUnionGeometry getNewMaterial(Material m) const {
        ConvexUnionGeometry g = *this;
        for (ConvexPrimitive& c : g.polyhedra) c.material = m;
        return g;
    }
    ConvexUnionGeometry getTranslated(Vec3 v) const {
        ConvexUnionGeometry g = *this;
        for (ConvexPrimitive& c : g.polyhedra) {
            c.corner = Vec3(c.corner.x + v.x, c.corner.y + v.y, c.corner.z + v.z);
            for (Vec3& p : c.points) p = Vec3(p.x + v.x, p.y + v.y, p.z + v.z);
        }
        return g;
    }
};

class PhysicsEngine;

// Handle with the RigidBody getters/setters used by scene code (RigidBody.h:25-68)
class RigidBody {
public:
    RigidBody(PhysicsEngine* e, uint32_t id) : e_(e), id_(id) {}
    uint32_t getID() const { return id_; }
    Vec3 getCOM() const;
    Quaternion getOrientation() const;
    Vec3 getVel() const;
    Vec3 getAngVel() const;
    void setVel(Vec3 v);
    void setAngVel(Vec3 w);
    void setOrientation(Quaternion q);
    void setToPosition(const Vec3& p);
    void setMass(double m);
private:
    PhysicsEngine* e_;
    uint32_t id_;
};

struct ConstraintID { uint32_t id; };

// RayHitInfo (PhysicsEngine.h:40-46)
struct RayHitInfo {
    bool did_hit = false;
    RigidBody* hit_object = nullptr;
    Vec3 hit_position, surface_normal;
    double hit_distance = -1;
};

class PhysicsEngine {
public:
    PhysicsEngine() { check(cpgpu_world_create(&w_)); }
    ~PhysicsEngine() { if (w_) cpgpu_world_destroy(w_); for (RigidBody* b : owned_) delete b; }
    PhysicsEngine(const PhysicsEngine&) = delete;
    PhysicsEngine& operator=(const PhysicsEngine&) = delete;

    void timeStep() { check(cpgpu_step(w_, 1)); }
    void timeSteps(int n) { check(cpgpu_step(w_, n)); }

    RigidBody* createRigidBody(const ConvexUnionGeometry& g, MovementType movement = DYNAMIC, Vec3 position = Vec3()) {
        const size_t n = g.polyhedra.size();
        if (n == 0) throw Error(CPGPU_ERR_INVALID_ARG, "cpgpu: createRigidBody of an empty ConvexUnionGeometry");
        // storage the primitive descriptors point into, alive until the call returns
        std::vector<std::vector<double>> pts(n);
        std::vector<std::vector<int>> offs(n), idx(n);
        std::vector<cpgpu_primitive> prims(n);
        for (size_t i = 0; i < n; i++) {
            const ConvexPrimitive& c = g.polyhedra[i];
            cpgpu_primitive& q = prims[i];
            q = cpgpu_primitive{};
            q.mat = c.material.c();
            q.p[0] = c.corner.x; q.p[1] = c.corner.y; q.p[2] = c.corner.z;
            switch (c.kind) {
            case ConvexPrimitive::BOX: q.kind = CPGPU_PRIM_BOX; q.a = c.dx; q.b = c.dy; q.c = c.dz; break;
            case ConvexPrimitive::SPHERE: q.kind = CPGPU_PRIM_SPHERE; q.a = c.radius; break;
            case ConvexPrimitive::CYLINDER: q.kind = CPGPU_PRIM_CYLINDER; q.a = c.radius; q.b = c.height; break;
            case ConvexPrimitive::CAPSULE: q.kind = CPGPU_PRIM_CAPSULE; q.a = c.radius; q.b = c.height; break;
            default:
                for (const Vec3& p : c.points) { pts[i].push_back(p.x); pts[i].push_back(p.y); pts[i].push_back(p.z); }
                offs[i].push_back(0);
                for (const auto& f : c.faces) {
                    idx[i].insert(idx[i].end(), f.begin(), f.end());
                    offs[i].push_back((int)idx[i].size());
                }
                q.kind = CPGPU_PRIM_HULL;
                q.points = pts[i].data(); q.n_points = (int)c.points.size();
                q.face_offsets = offs[i].data(); q.face_indices = idx[i].data(); q.n_faces = (int)c.faces.size();
            }
        }
        uint32_t id = 0;
        check(cpgpu_body_union(w_, prims.data(), (int)n, movement, position.data(), &id));
        RigidBody* b = new RigidBody(this, id);
        owned_.push_back(b);
        return b;
    }

    // createRigidBody(StaticMeshGeometry(MeshInput{triangle_indices, points}), FIXED)
    // (PhysicsEngine.cpp:498-512): triangles (three point indices each) in world coordinates
    RigidBody* createStaticMesh(const std::vector<Vec3>& points, const std::vector<std::array<int, 3>>& tris,
                                Material mat = Material::default_material()) {
        std::vector<double> pts;
        for (const Vec3& p : points) { pts.push_back(p.x); pts.push_back(p.y); pts.push_back(p.z); }
        std::vector<int> idx;
        for (const auto& t : tris) idx.insert(idx.end(), t.begin(), t.end());
        cpgpu_material m = mat.c();
        uint32_t id = 0;
        check(cpgpu_body_mesh(w_, pts.data(), (int)points.size(), idx.data(), (int)tris.size(), &m, 1, &id));
        RigidBody* b = new RigidBody(this, id);
        owned_.push_back(b);
        return b;
    }

    // PhysicsEngine::raycastFirstIntersection (PhysicsEngine.cpp:582-609)
    RayHitInfo raycastFirstIntersection(Vec3 ray_origin, Vec3 ray_dir, const std::vector<RigidBody*>& ignore_list = {}) const {
        std::vector<uint32_t> ig;
        for (RigidBody* b : ignore_list) ig.push_back(b->getID());
        uint32_t id = 0;
        double p[3], n[3], t = -1;
        check(cpgpu_raycast(w_, ray_origin.data(), ray_dir.data(), 1, ig.data(), (int)ig.size(), &id, p, n, &t));
        RayHitInfo h;
        if (id == 0) return h;
        h.did_hit = true;
        h.hit_object = id <= owned_.size() ? owned_[id - 1] : nullptr;
        h.hit_position = Vec3(p[0], p[1], p[2]);
        h.surface_normal = Vec3(n[0], n[1], n[2]);
        h.hit_distance = t;
        return h;
    }

    ConstraintID addBallSocketConstraint(RigidBody* b1, RigidBody* b2, Vec3 p1, Vec3 p2, double strength = 15000) {
        uint32_t id = 0;
        check(cpgpu_add_ball_socket(w_, b1->getID(), b2->getID(), p1.data(), p2.data(), strength, &id));
        return ConstraintID{id};
    }
    // addDistanceConstraint / addWeldConstraint / addSliderConstraint /
    // addSlidingHingeConstraint / addConeLimitConstraint /
    // addTwistLimitConstraint / addSpring (PhysicsEngine.cpp:623-998)
    ConstraintID addDistanceConstraint(RigidBody* b1, RigidBody* b2, Vec3 p1, Vec3 p2, double target = -1,
                                       double strength = 15000) {
        uint32_t id = 0;
        check(cpgpu_add_distance(w_, b1->getID(), b2->getID(), p1.data(), p2.data(), target, strength, &id));
        return ConstraintID{id};
    }
    ConstraintID addWeldConstraint(RigidBody* b1, RigidBody* b2, Vec3 p1, Vec3 p2, double pos_strength = 15000,
                                   double rot_strength = 15000) {
        uint32_t id = 0;
        check(cpgpu_add_weld(w_, b1->getID(), b2->getID(), p1.data(), p2.data(), pos_strength, rot_strength, &id));
        return ConstraintID{id};
    }
    ConstraintID addTwistLimitConstraint(RigidBody* b1, RigidBody* b2, Vec3 d1, Vec3 d2, double min_angle,
                                         double max_angle, double rot_strength = 15000) {
        uint32_t id = 0;
        check(cpgpu_add_twist_limit(w_, b1->getID(), b2->getID(), d1.data(), d2.data(), min_angle, max_angle,
                                    rot_strength, &id));
        return ConstraintID{id};
    }
    ConstraintID addConeLimitConstraint(RigidBody* b1, RigidBody* b2, Vec3 d1, Vec3 d2, double max_angle,
                                        double rot_strength = 15000) {
        uint32_t id = 0;
        check(cpgpu_add_cone_limit(w_, b1->getID(), b2->getID(), d1.data(), d2.data(), max_angle, rot_strength, &id));
        return ConstraintID{id};
    }
    ConstraintID addSpring(RigidBody* b1, RigidBody* b2, Vec3 p1, Vec3 p2, double damping, double stiffness,
                           double resting_length = -1) {
        uint32_t id = 0;
        check(cpgpu_add_spring(w_, b1->getID(), b2->getID(), p1.data(), p2.data(), damping, stiffness,
                               resting_length, &id));
        return ConstraintID{id};
    }
    ConstraintID addSliderConstraint(RigidBody* b1, RigidBody* b2, Vec3 p1, Vec3 p2, Vec3 a1, Vec3 a2,
                                     double pos_strength = 15000, double rot_strength = 15000) {
        uint32_t id = 0;
        check(cpgpu_add_slider(w_, b1->getID(), b2->getID(), p1.data(), p2.data(), a1.data(), a2.data(), pos_strength,
                               rot_strength, &id));
        return ConstraintID{id};
    }
    ConstraintID addSlidingHingeConstraint(RigidBody* b1, RigidBody* b2, Vec3 p1, Vec3 p2, Vec3 a1, Vec3 a2,
                                           double pos_strength = 15000, double rot_strength = 15000) {
        uint32_t id = 0;
        check(cpgpu_add_sliding_hinge(w_, b1->getID(), b2->getID(), p1.data(), p2.data(), a1.data(), a2.data(),
                                      pos_strength, rot_strength, &id));
        return ConstraintID{id};
    }
    ConstraintID addHingeConstraint(RigidBody* b1, RigidBody* b2, Vec3 p1, Vec3 p2, Vec3 a1, Vec3 a2,
                                    double pos_strength = 15000, double rot_strength = 15000) {
        uint32_t id = 0;
        check(cpgpu_add_hinge(w_, b1->getID(), b2->getID(), p1.data(), p2.data(), a1.data(), a2.data(), pos_strength,
                              rot_strength, &id));
        return ConstraintID{id};
    }
    // addMotorConstraint / addPistonConstraint (PhysicsEngine.cpp:725-852)
    // and the powered constraints' setters and getters (:1800-1930)
    ConstraintID addMotorConstraint(ConstraintID base, double min_angle = -INFINITY, double max_angle = INFINITY) {
        uint32_t id = 0;
        check(cpgpu_add_motor(w_, base.id, min_angle, max_angle, &id));
        return ConstraintID{id};
    }
    ConstraintID addPistonConstraint(ConstraintID base, double negative_slide_limit = -INFINITY,
                                     double positive_slide_limit = INFINITY) {
        uint32_t id = 0;
        check(cpgpu_add_piston(w_, base.id, negative_slide_limit, positive_slide_limit, &id));
        return ConstraintID{id};
    }
    void setMotorOff(ConstraintID id) { check(cpgpu_set_motor(w_, id.id, 0, 0, 0)); }
    void setMotorConstantTorque(ConstraintID id, double torque) { check(cpgpu_set_motor(w_, id.id, 1, torque, 0)); }
    void setMotorTargetVelocity(ConstraintID id, double max_torque, double v) { check(cpgpu_set_motor(w_, id.id, 2, max_torque, v)); }
    void setMotorTargetPosition(ConstraintID id, double max_torque, double a) { check(cpgpu_set_motor(w_, id.id, 3, max_torque, a)); }
    void setPistonOff(ConstraintID id) { check(cpgpu_set_piston(w_, id.id, 0, 0, 0)); }
    void setPistonConstantForce(ConstraintID id, double force) { check(cpgpu_set_piston(w_, id.id, 1, force, 0)); }
    void setPistonTargetVelocity(ConstraintID id, double max_force, double v) { check(cpgpu_set_piston(w_, id.id, 2, max_force, v)); }
    void setPistonTargetPosition(ConstraintID id, double max_force, double x) { check(cpgpu_set_piston(w_, id.id, 3, max_force, x)); }
    double getMotorAngularPosition(ConstraintID id) {
        double out = 0;
        check(cpgpu_get_motor_position(w_, id.id, &out));
        return out;
    }
    double getPistonPosition(ConstraintID id) {
        double out = 0;
        check(cpgpu_get_piston_position(w_, id.id, &out));
        return out;
    }

    void setStep_time(double d) { check(cpgpu_set_step_time(w_, d)); }
    void setGravity(const Vec3& g) { check(cpgpu_set_gravity(w_, g.x, g.y, g.z)); }
    void setSubstepCount(int c) { check(cpgpu_set_substep_count(w_, c)); }
    void setPGSIterations(int v, int p, int h = 1) { check(cpgpu_set_pgs_iterations(w_, v, p, h)); }
    void setSleepingEnabled(bool s) { check(cpgpu_set_sleeping_enabled(w_, s ? 1 : 0)); }
    void setWarmStartDisabled(bool b) { check(cpgpu_set_warm_start_disabled(w_, b ? 1 : 0)); }
    void setGlobalConstraintForceMixing(double c) { check(cpgpu_set_global_cfm(w_, c)); }
    void setAngleVelUpdateTickCount(int n) { check(cpgpu_set_angle_vel_update_tick_count(w_, n)); }
    void setInternalGyroscopicForcesDisabled(bool b) { check(cpgpu_set_internal_gyro_forces_disabled(w_, b ? 1 : 0)); }
    uint32_t getNumBodies() { int n = 0; check(cpgpu_num_bodies(w_, &n)); return (uint32_t)n; }

    cpgpu_world* handle() { return w_; }

    // per-body state of body `id` (all bodies are fetched; cache when iterating)
    void bodyState(uint32_t id, double* com, double* quat, double* vel, double* ang) {
        int n = (int)getNumBodies();
        std::vector<double> c(3 * n), q(4 * n), v(3 * n), a(3 * n);
        check(cpgpu_get_body_state(w_, c.data(), q.data(), v.data(), a.data()));
        size_t i = id - 1;
        if (com) for (int k = 0; k < 3; k++) com[k] = c[3 * i + k];
        if (quat) for (int k = 0; k < 4; k++) quat[k] = q[4 * i + k];
        if (vel) for (int k = 0; k < 3; k++) vel[k] = v[3 * i + k];
        if (ang) for (int k = 0; k < 3; k++) ang[k] = a[3 * i + k];
    }

private:
    cpgpu_world* w_ = nullptr;
    std::vector<RigidBody*> owned_;
};

inline Vec3 RigidBody::getCOM() const { double c[3]; e_->bodyState(id_, c, nullptr, nullptr, nullptr); return Vec3(c[0], c[1], c[2]); }
inline Quaternion RigidBody::getOrientation() const {
    double q[4]; e_->bodyState(id_, nullptr, q, nullptr, nullptr); return Quaternion(q[0], q[1], q[2], q[3]);
}
inline Vec3 RigidBody::getVel() const { double v[3]; e_->bodyState(id_, nullptr, nullptr, v, nullptr); return Vec3(v[0], v[1], v[2]); }
inline Vec3 RigidBody::getAngVel() const { double a[3]; e_->bodyState(id_, nullptr, nullptr, nullptr, a); return Vec3(a[0], a[1], a[2]); }
inline void RigidBody::setVel(Vec3 v) { check(cpgpu_body_set_velocity(e_->handle(), id_, v.data())); }
inline void RigidBody::setAngVel(Vec3 w) { check(cpgpu_body_set_ang_velocity(e_->handle(), id_, w.data())); }
inline void RigidBody::setOrientation(Quaternion q) { double d[4] = {q.r, q.i, q.j, q.k}; check(cpgpu_body_set_orientation(e_->handle(), id_, d)); }
inline void RigidBody::setToPosition(const Vec3& p) { check(cpgpu_body_set_position(e_->handle(), id_, p.data())); }
inline void RigidBody::setMass(double m) { check(cpgpu_body_set_mass(e_->handle(), id_, m)); }

}  // namespace cpgpu
