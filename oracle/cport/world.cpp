// world.cpp — per-step pipeline of the CPU restatement (test infrastructure;
// see cport.h): broadphase, narrowphase, contact persistence, islands, row
// rebuild, PGS and integration, plus the cport_ C ABI.
#include "cport.h"

#include <set>
#include <string>

extern "C" {
#include "cpgpu.h"
}

namespace cport {

// ------------------------------------------------------------ bodies ----
static AABB boxUnion(const AABB& a, const AABB& b);
static AABB genAABB(const Hull& h) {
    const double inf = std::numeric_limits<double>::infinity();
    AABB a{V3(inf, inf, inf), V3(-inf, -inf, -inf)};
    for (const V3& p : h.pts) {
        a.mn.x = std::min<double>(a.mn.x, p.x); a.mn.y = std::min<double>(a.mn.y, p.y); a.mn.z = std::min<double>(a.mn.z, p.z);
        a.mx.x = std::max<double>(a.mx.x, p.x); a.mx.y = std::max<double>(a.mx.y, p.y); a.mx.z = std::max<double>(a.mx.z, p.z);
    }
    return a;
}

// Sphere::gen_AABB (ConvexPrimitive.cpp:439-443)
static AABB genAABB(const SphereG& s) {
    return AABB{s.c - V3(s.r, s.r, s.r), s.c + V3(s.r, s.r, s.r)};
}

// Capsule::gen_AABB (ConvexPrimitive.cpp:390-401)
static AABB genAABB(const CapG& c) {
    V3 v = c.axis * c.h / 2.0;
    double dx = std::abs(v.x) + c.r, dy = std::abs(v.y) + c.r, dz = std::abs(v.z) + c.r;
    return AABB{V3(c.c.x - dx, c.c.y - dy, c.c.z - dz), V3(c.c.x + dx, c.c.y + dy, c.c.z + dz)};
}

// Cylinder::gen_AABB (ConvexPrimitive.cpp:289-298): the two cap 8-gons,
// interleaved top/bottom as the reference collects them
static AABB genAABB(const CylG& c) {
    const double inf = std::numeric_limits<double>::infinity();
    AABB a{V3(inf, inf, inf), V3(-inf, -inf, -inf)};
    for (size_t i = 0; i < c.top.size(); i++) {
        for (const V3& p : {c.top[i], c.bot[i]}) {
            a.mn.x = std::min<double>(a.mn.x, p.x); a.mn.y = std::min<double>(a.mn.y, p.y); a.mn.z = std::min<double>(a.mn.z, p.z);
            a.mx.x = std::max<double>(a.mx.x, p.x); a.mx.y = std::max<double>(a.mx.y, p.y); a.mx.z = std::max<double>(a.mx.z, p.z);
        }
    }
    return a;
}

// Cylinder::recomputeFromReference (ConvexPrimitive.cpp:272-287): the bottom
// cap is re-derived from the top one
static void cylFromReference(CylG& out, const CylG& ref, const M3& rot, const V3& trans) {
    out.c = rot * ref.c + trans;
    out.axis = rot * ref.axis;
    for (size_t i = 0; i < out.gv.size(); i++) out.gv[i] = rot * ref.gv[i];
    for (size_t i = 0; i < out.top.size(); i++) {
        out.top[i] = rot * ref.top[i] + trans;
        out.bot[i] = out.top[i] - out.h * out.axis;
    }
}

// RigidBody::updateGeometry (RigidBody.cpp:281-312) for a single primitive
// one primitive's world geometry from its reference geometry at (rot, com)
// (the primitives' recomputeFromReference, ConvexPrimitive.cpp:272-287,
// 383-388, 433-437, 715-729) and its AABB
static void partWorld(Body* g, const M3& rot, const V3& com) {
    if (g->kind == K_SPHERE) {
        g->sph.c = com + rot * g->sph_ref.c;
        g->aabb = genAABB(g->sph);
    } else if (g->kind == K_CYLINDER) {
        cylFromReference(g->cyl, g->cyl_ref, rot, com);
        g->aabb = genAABB(g->cyl);
    } else if (g->kind == K_CAPSULE) {
        g->cap.c = com + rot * g->cap_ref.c;
        g->cap.axis = rot * g->cap_ref.axis;
        g->aabb = genAABB(g->cap);
    } else {
        for (size_t i = 0; i < g->shape.pts.size(); i++) g->shape.pts[i] = com + rot * g->ref_shape.pts[i];
        g->shape.interior = com + rot * g->ref_shape.interior;
        for (size_t i = 0; i < g->shape.gv.size(); i++) g->shape.gv[i] = rot * g->ref_shape.gv[i];
        g->aabb = genAABB(g->shape);
    }
}

void Body::updateGeometry() {
    if (kind == K_MESH) return;   // fixed meshes stay in world coordinates
    q = q.normalize();
    M3 rot = q.rotMatrix();
    if (kind == K_UNION) {   // every primitive, then AABB::combine of theirs
        for (size_t i = 0; i < parts.size(); i++) {
            partWorld(parts[i].get(), rot, com);
            aabb = i == 0 ? parts[i]->aabb : boxUnion(aabb, parts[i]->aabb);
        }
        return;
    }
    if (kind == K_SPHERE) {
        sph.c = com + rot * sph_ref.c;            // Sphere::recomputeFromReference (ConvexPrimitive.cpp:433-437)
        aabb = genAABB(sph);
        return;
    }
    if (kind == K_CYLINDER) {
        cylFromReference(cyl, cyl_ref, rot, com);
        aabb = genAABB(cyl);
        return;
    }
    if (kind == K_CAPSULE) {
        cap.c = com + rot * cap_ref.c;            // Capsule::recomputeFromReference (ConvexPrimitive.cpp:383-388)
        cap.axis = rot * cap_ref.axis;
        aabb = genAABB(cap);
        return;
    }
    for (size_t i = 0; i < shape.pts.size(); i++) shape.pts[i] = com + rot * ref_shape.pts[i];
    shape.interior = com + rot * ref_shape.interior;
    for (size_t i = 0; i < shape.gv.size(); i++) shape.gv[i] = rot * ref_shape.gv[i];
    aabb = genAABB(shape);
}

// RigidBody::updateInertiaTensor (RigidBody.cpp:270-279)
void Body::updateInertiaTensor() {
    q = q.normalize();
    M3 rot = q.rotMatrix();
    M3 rc = q.conj().rotMatrix();
    tensor = rot * ref_tensor * rc;
    inv_tensor = rot * ref_inv_tensor * rc;
}

// RigidBody::rotateWhileApplyingGyroAccel (RigidBody.cpp:207-255): implicit
// gyroscopic update, n_itr sub-steps of two Newton iterations each
void Body::rotateWithGyro(double dt, int n_itr, bool gyro_disabled) {
    const double CUT = 0.00000000001;
    if (ang_vel.mag2() == 0) return;
    if (gyro_disabled) {
        Q rot = Q::axisAngle(ang_vel.mag() * dt, ang_vel.normalize());
        q = rot * q;
        return;
    }
    M3 it = tensor;
    Q iq = q;
    V3 iw = ang_vel;
    for (int i = 0; i < n_itr; i++) {
        V3 w = iw;
        double ts = dt / n_itr;
        for (int k = 0; k < 2; k++) {
            V3 f = ts * w.cross(it * w) - it * (iw - w);
            M3 jac = it + ts * (M3::crossMat(w) * it - M3::crossMat(it * w));
            if (std::abs(jac.det()) > CUT) w -= jac.inverse() * f;
        }
        iw = w;
        iq = Q::axisAngle(ts * iw.mag(), iw) * iq;
        if (i + 1 < n_itr) {
            M3 rot = iq.rotMatrix();
            M3 rc = iq.conj().rotMatrix();
            it = rot * ref_tensor * rc;
        }
    }
    q = iq;
    ang_vel = iw;
}

// RigidBody::RigidBody + PhysicsEngine::createRigidBody (RigidBody.cpp:13-39,
// PhysicsEngine.cpp:486-496)
Body* World::addHull(const std::vector<V3>& pts, const std::vector<std::vector<int>>& faces, const Material& m,
                     int movement, V3 pos) {
    auto b = std::make_unique<Body>();
    b->id = (uint32_t)bodies.size() + 1;
    b->movement = movement;
    b->mat = m;
    b->src_shape.build(pts, faces);
    b->create_pos = pos;
    double mass;
    V3 com;
    M3 tensor;
    massProperties(b->src_shape, m.density, &com, &tensor, &mass);
    Body* raw = b.get();
    bodies.push_back(std::move(b));
    placeBody(raw, mass, com, tensor);
    nodes[raw->id] = raw;
    adj[raw];
    return raw;
}

// recenterTensor (RigidBody.cpp:406-425): parallel-axis shift of an inertia
// tensor to a new centre of rotation
static M3 recenterTensor(double mass, const M3& t, V3 new_c, V3 old_origin, V3 true_com) {
    M3 o = t;
    V3 d = new_c - old_origin;
    V3 c = true_com - old_origin;
    o.m[0][0] += mass * (d.y * d.y + d.z * d.z - 2 * d.y * c.y - 2 * d.z * c.z);
    o.m[0][1] += mass * (d.x * c.y + d.y * c.x - d.x * d.y);
    o.m[0][2] += mass * (d.x * c.z + d.z * c.x - d.x * d.z);
    o.m[1][1] += mass * (d.x * d.x + d.z * d.z - 2 * d.x * c.x - 2 * d.z * c.z);
    o.m[1][2] += mass * (d.y * c.z + d.z * c.y - d.y * d.z);
    o.m[2][2] += mass * (d.x * d.x + d.y * d.y - 2 * d.x * c.x - 2 * d.y * c.y);
    o.m[1][0] = o.m[0][1];
    o.m[2][0] = o.m[0][2];
    o.m[2][1] = o.m[1][2];
    return o;
}

// calculateMassProperties (RigidBody.cpp:427-640), SPHERE and CYLINDER cases
// for a body of one primitive with the default height axis
static void primitiveMass(const Body& b, double* mass, V3* com, M3* tensor) {
    double m;
    V3 c;
    M3 local;
    if (b.kind == K_SPHERE) {
        double r = b.sph_src.r;
        m = (4.0 / 3.0) * PI_TRUNC * r * r * r * b.mat.density;
        c = b.sph_src.c;
        double k = 2.0 / 5.0 * m * r * r;
        local = k * M3::iden();
    } else if (b.kind == K_CAPSULE) {
        // RigidBody.cpp:570-600 (the mass is the volume: the density scales
        // only the tensor there); the height axis is +y, no rotation
        double h = b.cap_src.h, r = b.cap_src.r;
        double r3 = r * r * r, r4 = r3 * r, r5 = r4 * r;
        double d = b.mat.density;
        m = (4.0 / 3.0) * PI_TRUNC * r * r * r + PI_TRUNC * r * r * h;
        c = b.cap_src.c;
        local.m[0][0] = d * PI_TRUNC * ((8.0 / 15.0) * r5 + (1.0 / 3.0) * r3 * h * h + 0.75 * r4 * h + (1.0 / 12.0) * r * r * h * h * h);
        local.m[1][1] = d * PI_TRUNC * ((8.0 / 15.0) * r5 + 0.5 * h * r4);
        local.m[2][2] = local.m[0][0];
    } else {
        double h = b.cyl_src.h, r = b.cyl_src.r;
        m = PI_TRUNC * r * r * h * b.mat.density;
        c = b.cyl_src.c;
        local.m[0][0] = m * (h * h / 12 + r * r / 4);
        local.m[1][1] = m * r * r / 2;
        local.m[2][2] = local.m[0][0];
    }
    M3 t = M3() + recenterTensor(m, local, V3(0, 0, 0), c, c);
    V3 csum = V3(0, 0, 0) + m * c;
    double msum = 0 + m;
    *com = csum / msum;
    *mass = msum;
    *tensor = recenterTensor(msum, t, *com, V3(0, 0, 0), *com);
}

Body* World::addSphere(V3 center, double r, const Material& m, int movement, V3 pos) {
    auto b = std::make_unique<Body>();
    b->kind = K_SPHERE;
    b->movement = movement;
    b->mat = m;
    b->sph_src.c = center;
    b->sph_src.r = r;
    b->create_pos = pos;
    double mass; V3 com; M3 tensor;
    primitiveMass(*b, &mass, &com, &tensor);
    return finishBody(std::move(b), mass, com, tensor);
}

// ConvexUnionGeometry::cylinder (Geometry.cpp:47-49): the base point is the
// centre of the bottom cap
Body* World::addCylinder(V3 base, double r, double h, const Material& m, int movement, V3 pos) {
    auto b = std::make_unique<Body>();
    b->kind = K_CYLINDER;
    b->movement = movement;
    b->mat = m;
    b->cyl_src = makeCylinder(base + V3(0, h / 2.0, 0), r, h);
    b->create_pos = pos;
    double mass; V3 com; M3 tensor;
    primitiveMass(*b, &mass, &com, &tensor);
    return finishBody(std::move(b), mass, com, tensor);
}

// ConvexUnionGeometry::capsule (Geometry.cpp:43-45): `bot` is the centre of
// the bottom cap sphere, the height axis +y
Body* World::addCapsule(V3 bot, double r, double h, const Material& m, int movement, V3 pos) {
    auto b = std::make_unique<Body>();
    b->kind = K_CAPSULE;
    b->movement = movement;
    b->mat = m;
    b->cap_src.c = bot + V3(0, h / 2.0, 0);
    b->cap_src.axis = V3(0, 1, 0);
    b->cap_src.r = r;
    b->cap_src.h = h;
    b->create_pos = pos;
    double mass; V3 com; M3 tensor;
    primitiveMass(*b, &mass, &com, &tensor);
    return finishBody(std::move(b), mass, com, tensor);
}

// createRigidBody(ConvexUnionGeometry of several primitives) (RigidBody.cpp:
// 13-39, 427-640): mass, centre of mass and tensor summed over the primitives
// in order (hulls by the tetrahedral decomposition, to rounding)
Body* World::addUnion(std::vector<std::unique_ptr<Body>> parts, int movement, V3 pos) {
    auto b = std::make_unique<Body>();
    b->kind = K_UNION;
    b->movement = movement;
    b->mat = parts.front()->mat;
    b->create_pos = pos;
    const uint32_t id = (uint32_t)bodies.size() + 1;
    double msum = 0;
    V3 csum;
    M3 tsum;
    for (size_t i = 0; i < parts.size(); i++) {
        Body* g = parts[i].get();
        g->id = (id << 8) | (uint32_t)i;
        g->movement = movement;
        double m;
        V3 c;
        M3 t;
        if (g->kind == K_HULL) {
            massProperties(g->src_shape, g->mat.density, &c, &t, &m);
            t = recenterTensor(m, t, V3(0, 0, 0), c, c);
        } else {
            primitiveMass(*g, &m, &c, &t);
            t = recenterTensor(m, t, V3(0, 0, 0), c, c);
        }
        tsum = tsum + t;
        csum = csum + m * c;
        msum = msum + m;
    }
    V3 com = csum / msum;
    M3 tensor = recenterTensor(msum, tsum, com, V3(0, 0, 0), com);
    b->parts = std::move(parts);
    return finishBody(std::move(b), msum, com, tensor);
}

Body* World::finishBody(std::unique_ptr<Body> b, double mass, const V3& com, const M3& tensor) {
    b->id = (uint32_t)bodies.size() + 1;
    Body* raw = b.get();
    bodies.push_back(std::move(b));
    placeBody(raw, mass, com, tensor);
    nodes[raw->id] = raw;
    adj[raw];
    return raw;
}

// The part of the RigidBody constructor that follows the mass properties
// (RigidBody.cpp:19-36): recentre the reference geometry on the COM, track the
// geometry origin and move it to the creation position.
void World::placeBody(Body* b, double mass, const V3& com_geom, const M3& tensor) {
    b->mass = mass;
    b->com = com_geom;
    b->ref_tensor = tensor;
    b->ref_inv_tensor = b->ref_tensor.inverse();
    b->tensor = b->ref_tensor;
    b->inv_tensor = b->ref_inv_tensor;
    b->q = Q();
    M3 I = M3::iden();
    V3 mc = -b->com;
    if (b->kind == K_UNION) {
        // each primitive's reference geometry recentred on the body's COM
        // (RigidBody.cpp:23-25)
        for (auto& g : b->parts) {
            g->sph_ref = g->sph_src;
            g->sph_ref.c = mc + I * g->sph_src.c;
            g->cyl_ref = g->cyl_src;
            if (g->kind == K_CYLINDER) cylFromReference(g->cyl_ref, g->cyl_src, I, mc);
            g->cap_ref = g->cap_src;
            g->cap_ref.c = mc + I * g->cap_src.c;
            g->cap_ref.axis = I * g->cap_src.axis;
            g->ref_shape = g->src_shape;
            for (V3& pt : g->ref_shape.pts) pt = mc + I * pt;
            g->ref_shape.interior = mc + I * g->ref_shape.interior;
            for (V3& gv : g->ref_shape.gv) gv = I * gv;
            g->sph = g->sph_src;
            g->cyl = g->cyl_src;
            g->cap = g->cap_src;
            g->shape = g->src_shape;
        }
    } else if (b->kind == K_SPHERE) {
        b->sph_ref = b->sph_src;
        b->sph_ref.c = mc + I * b->sph_src.c;
        b->sph = b->sph_src;
        b->aabb = genAABB(b->sph);
    } else if (b->kind == K_CYLINDER) {
        b->cyl_ref = b->cyl_src;
        cylFromReference(b->cyl_ref, b->cyl_src, I, mc);
        b->cyl = b->cyl_src;
        b->aabb = genAABB(b->cyl);
    } else if (b->kind == K_CAPSULE) {
        b->cap_ref = b->cap_src;
        b->cap_ref.c = mc + I * b->cap_src.c;
        b->cap_ref.axis = I * b->cap_src.axis;
        b->cap = b->cap_src;
        b->aabb = genAABB(b->cap);
    } else {
        b->ref_shape = b->src_shape;
        for (V3& p : b->ref_shape.pts) p = mc + I * p;
        b->ref_shape.interior = mc + I * b->ref_shape.interior;
        for (V3& g : b->ref_shape.gv) g = I * g;
        b->shape = b->src_shape;
        b->aabb = genAABB(b->shape);
    }
    b->local_origin = -b->com;
    b->track_p.assign(1, b->local_origin + V3(0, 0, 0));
    V3 t = b->create_pos - b->trackedP(0);
    b->com += t;
    b->updateGeometry();
}

// ------------------------------------------------------------ meshes ----
static AABB boxUnion(const AABB& a, const AABB& b) {   // AABB::combine
    AABB o;
    o.mn.x = std::min<double>(a.mn.x, b.mn.x); o.mn.y = std::min<double>(a.mn.y, b.mn.y); o.mn.z = std::min<double>(a.mn.z, b.mn.z);
    o.mx.x = std::max<double>(a.mx.x, b.mx.x); o.mx.y = std::max<double>(a.mx.y, b.mx.y); o.mx.z = std::max<double>(a.mx.z, b.mx.z);
    return o;
}
// AABB::surfaceArea (AABB.h:112-118), as written there: 2 dx dy + dy dz + dz dx
static double boxCost(const AABB& a) {
    double dx = a.mx.x - a.mn.x, dy = a.mx.y - a.mn.y, dz = a.mx.z - a.mn.z;
    return 2 * (dx * dy) + (dy * dz) + (dz * dx);
}

// AABBTree::add (AABB_Tree.h:39-105): best sibling by branch-and-bound on the
// inherited cost, new parent, ancestors refitted and rebalanced by rotations
void MeshTree::add(int obj, const AABB& b) {
    Node leaf;
    leaf.leaf = true; leaf.obj = obj; leaf.true_box = b; leaf.box = b; leaf.cost = boxCost(b);
    const int nl = (int)nodes.size();
    nodes.push_back(leaf);
    if (root < 0) { root = nl; return; }
    int best = -1;
    double best_cost = std::numeric_limits<double>::infinity();
    std::vector<std::pair<int, double>> cand{{root, 0.0}};
    while (!cand.empty()) {
        auto c = cand.back();
        cand.pop_back();
        if (c.second >= best_cost) continue;
        AABB cb = boxUnion(nodes[nl].box, nodes[c.first].box);
        double direct = boxCost(cb);
        double cost = c.second + direct;
        if (cost < best_cost) { best = c.first; best_cost = cost; }
        if (!nodes[c.first].leaf) {
            double inherited = c.second + direct - nodes[c.first].cost;
            cand.push_back({nodes[c.first].left, inherited});
            cand.push_back({nodes[c.first].right, inherited});
        }
    }
    Node par;
    const int np = (int)nodes.size();
    nodes.push_back(par);
    if (best == root) root = np;
    else {
        int op = nodes[best].parent;
        if (nodes[op].left == best) nodes[op].left = np; else nodes[op].right = np;
        nodes[np].parent = op;
    }
    nodes[np].left = best; nodes[best].parent = np;
    nodes[np].right = nl; nodes[nl].parent = np;
    // haveAncestorsRecalculateAABB
    for (int cur = nodes[nl].parent; cur >= 0; cur = nodes[cur].parent) {
        nodes[cur].box = boxUnion(nodes[nodes[cur].left].box, nodes[nodes[cur].right].box);
        nodes[cur].cost = boxCost(nodes[cur].box);
    }
    // rebalanceAncestors (AABB_Tree.h:373-421)
    auto swapNodes = [&](int n1, int n2) {
        int p1 = nodes[n1].parent, p2n = nodes[n2].parent;
        if (nodes[p1].left == n1) nodes[p1].left = n2; else nodes[p1].right = n2;
        if (nodes[p2n].left == n2) nodes[p2n].left = n1; else nodes[p2n].right = n1;
        nodes[n1].parent = p2n;
        nodes[n2].parent = p1;
    };
    int cur = nodes[nl].parent;
    while (cur >= 0 && nodes[cur].parent >= 0) {
        int pp = nodes[cur].parent;
        int sib = nodes[pp].left == cur ? nodes[pp].right : nodes[pp].left;
        if (sib >= 0) {
            AABB sl_box = boxUnion(nodes[nodes[cur].right].box, nodes[sib].box);
            AABB sr_box = boxUnion(nodes[nodes[cur].left].box, nodes[sib].box);
            double sl = boxCost(sl_box), sr = boxCost(sr_box), cl, cr;
            AABB cl_box, cr_box;
            if (nodes[sib].leaf) {
                cl = std::numeric_limits<double>::infinity();
                cr = std::numeric_limits<double>::infinity();
            } else {
                cl_box = boxUnion(nodes[nodes[sib].right].box, nodes[cur].box);
                cr_box = boxUnion(nodes[nodes[sib].left].box, nodes[cur].box);
                cl = boxCost(cl_box);
                cr = boxCost(cr_box);
            }
            double clc = cl - nodes[sib].cost, crc = cr - nodes[sib].cost;
            double slc = sl - nodes[cur].cost, src = sr - nodes[cur].cost;
            double mn = std::min<double>(clc, std::min<double>(crc, std::min<double>(slc, src)));
            if (mn >= 0) {
            } else if (mn == clc) {
                swapNodes(cur, nodes[sib].left);
                nodes[sib].box = cl_box; nodes[sib].cost = cl;
            } else if (mn == crc) {
                swapNodes(cur, nodes[sib].right);
                nodes[sib].box = cr_box; nodes[sib].cost = cr;
            } else if (mn == slc) {
                swapNodes(sib, nodes[cur].left);
                nodes[cur].box = sl_box; nodes[cur].cost = sl;
            } else {
                swapNodes(sib, nodes[cur].right);
                nodes[cur].box = sr_box; nodes[cur].cost = sr;
            }
        }
        cur = nodes[cur].parent;
    }
}

// getCollisionCandidatesWith (AABB_Tree.h:226-246): LIFO traversal, leaves
// tested on their true boxes
std::vector<int> MeshTree::candidates(const AABB& target) const {
    std::vector<int> out;
    if (root < 0) return out;
    std::vector<int> st{root};
    while (!st.empty()) {
        int n = st.back();
        st.pop_back();
        const Node& x = nodes[n];
        if (x.leaf) {
            if (AABB::overlap(x.true_box, target)) out.push_back(x.obj);
        } else if (AABB::overlap(x.box, target)) {
            st.push_back(x.left);
            st.push_back(x.right);
        }
    }
    return out;
}

// StaticMeshGeometry::StaticMeshGeometry (Geometry.cpp:675-820): face normals,
// neighbours across shared edges, ids (faces 0.., vertices n_faces + i, edges
// after), outward edge directions, Gauss regions with concave-neighbour count;
// then RigidBody(StaticMeshGeometry) (RigidBody.cpp:41-58) as a fixed body
Body* World::addMesh(const std::vector<V3>& pts, const std::vector<std::array<int, 3>>& tri_idx, const Material& m) {
    struct E { int p1, p2, opp, id = -1; uint64_t key; };
    struct TN { int p[3]; int nb[3]; E e[3]; V3 normal; };
    auto mkE = [](int a, int b, int o) {
        E e; e.p1 = a; e.p2 = b; e.opp = o;
        unsigned mx = (unsigned)std::max(a, b), mn = (unsigned)std::min(a, b);
        e.key = (((uint64_t)mx << 32) & 0xFFFFFFFF00000000ull) + mn;
        return e;
    };
    std::vector<TN> g;
    for (auto& t : tri_idx) {
        V3 v1 = pts[t[1]] - pts[t[0]], v2 = pts[t[2]] - pts[t[0]];
        TN n;
        n.p[0] = t[0]; n.p[1] = t[1]; n.p[2] = t[2];
        n.nb[0] = n.nb[1] = n.nb[2] = -1;
        n.e[0] = mkE(t[0], t[1], t[2]); n.e[1] = mkE(t[1], t[2], t[0]); n.e[2] = mkE(t[2], t[0], t[1]);
        n.normal = v1.cross(v2).normalize();
        g.push_back(n);
    }
    std::unordered_map<uint64_t, unsigned> efm;
    for (int i = 0; i < (int)g.size(); i++)
        for (int j = 0; j < 3; j++) {
            const E& e = g[i].e[j];
            auto q = efm.find(e.key);
            if (q != efm.end()) {
                g[i].nb[j] = (int)q->second;
                for (int k = 0; k < 3; k++)
                    if (g[q->second].e[k].key == e.key) g[q->second].nb[k] = i;
                efm.erase(q);
            } else {
                efm[e.key] = (unsigned)i;
            }
        }
    auto b = std::make_unique<Body>();
    b->kind = K_MESH;
    b->movement = FIXED;
    b->mat = m;
    int next_tri = 0, voff = (int)tri_idx.size(), next_edge = (int)(tri_idx.size() + pts.size());
    for (TN& t : g) {
        MeshTri tri;
        tri.concave = 0;
        tri.normal = t.normal;
        for (int i = 0; i < 3; i++) { tri.v[i] = pts[t.p[i]]; tri.vid[i] = t.p[i] + voff; }
        tri.id = next_tri++;
        for (int i = 0; i < 3; i++) {
            tri.ep1[i] = tri.v[i];
            tri.ep2[i] = tri.v[(i + 1) % 3];
            tri.out[i] = (tri.ep2[i] - tri.ep1[i]).cross(tri.normal).normalize();
            if (t.e[i].id == -1) t.e[i].id = next_edge++;
            tri.eid[i] = t.e[i].id;
            if (t.nb[i] == -1) {
                tri.gauss.push_back(tri.out[i]);
            } else {
                E comp{};
                for (int j = 0; j < 3; j++) {
                    const E& ne = g[t.nb[i]].e[j];
                    if (t.e[i].p1 == ne.p2 && t.e[i].p2 == ne.p1) comp = ne;
                }
                V3 tip = pts[t.e[i].opp], ntip = pts[comp.opp];
                const double EPS = 0.00001;
                bool concave = (ntip - tip).normalize().dot(t.normal) >= -EPS;
                if (concave) {
                    tri.concave++;
                    if (tri.concave <= 1) tri.gauss.push_back(tri.normal);
                } else {
                    tri.gauss.push_back(g[t.nb[i]].normal);
                }
            }
        }
        AABB a;
        a.mn = V3(std::numeric_limits<double>::infinity(), std::numeric_limits<double>::infinity(), std::numeric_limits<double>::infinity());
        a.mx = V3(-std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity());
        for (int i = 0; i < 3; i++) {
            a.mn.x = std::min<double>(a.mn.x, tri.v[i].x); a.mn.y = std::min<double>(a.mn.y, tri.v[i].y); a.mn.z = std::min<double>(a.mn.z, tri.v[i].z);
            a.mx.x = std::max<double>(a.mx.x, tri.v[i].x); a.mx.y = std::max<double>(a.mx.y, tri.v[i].y); a.mx.z = std::max<double>(a.mx.z, tri.v[i].z);
        }
        tri.aabb = a;
        b->tris.push_back(tri);
    }
    for (int i = 0; i < (int)b->tris.size(); i++) b->tree.add(i, b->tris[i].aabb);
    AABB box = b->tris[0].aabb;
    for (size_t i = 1; i < b->tris.size(); i++) box = boxUnion(box, b->tris[i].aabb);
    b->aabb = box;
    b->mass = std::numeric_limits<double>::quiet_NaN();
    b->track_p.assign(1, V3());
    b->id = (uint32_t)bodies.size() + 1;
    Body* raw = b.get();
    bodies.push_back(std::move(b));
    nodes[raw->id] = raw;
    adj[raw];
    return raw;
}

// --------------------------------------------------------- constraint graph ----
Edge* World::edgeBetween(Body* a, Body* b) {
    for (Edge* e : adj[a]) if (e->other(a) == b) return e;
    return nullptr;
}

// ConstraintGraphNode::getOrCreateEdgeTo / insertNewEdge
// (PhysicsEngine.cpp:1958-1995): node edge lists stay sorted by other id
Edge* World::getOrCreateEdge(Body* a, Body* b) {
    if (Edge* e = edgeBetween(a, b)) return e;
    auto e = std::make_unique<Edge>();
    e->n1 = a;
    e->n2 = b;
    Edge* raw = e.get();
    edges.push_back(std::move(e));
    for (Body* n : {a, b}) {
        std::vector<Edge*>& l = adj[n];
        uint32_t oid = raw->other(n)->id;
        size_t i = 0;
        while (i < l.size() && !(oid < l[i]->other(n)->id)) i++;
        l.insert(l.begin() + i, raw);
    }
    return raw;
}

void World::deleteEdge(Edge* e) {
    for (Body* n : {e->n1, e->n2}) {
        std::vector<Edge*>& l = adj[n];
        l.erase(std::remove(l.begin(), l.end(), e), l.end());
    }
    for (size_t i = 0; i < edges.size(); i++)
        if (edges[i].get() == e) { edges.erase(edges.begin() + i); break; }
}

// PhysicsEngine::addContact (PhysicsEngine.cpp:1062-1111): warm-start match by
// MagicID, otherwise append a new contact
void World::addContact(Body* b1, Body* b2, const ManifoldPoint& mp, const V3& n) {
    Edge* e = getOrCreateEdge(b1, b2);
    M3 i1 = b1->q.conj().rotMatrix();
    M3 i2 = b2->q.conj().rotMatrix();
    V3 nl = i1 * n;
    V3 p1 = i1 * (mp.pos - b1->com);
    V3 p2 = i2 * (mp.pos - b2->com);
    for (auto& c : e->contacts) {
        if (c->magic_b == mp.magic_b && c->magic_c == mp.magic_c) {
            c->friction_coeff = c->static_ready ? mp.stat : mp.kinetic;
            c->pen = mp.pen;
            c->n_local = nl;
            c->p1_local = p1;
            c->p2_local = p2;
            c->life = p.contact_life;
            c->live = true;
            return;
        }
    }
    auto c = std::make_unique<Contact>();
    c->b1 = b1; c->b2 = b2;
    c->p1_local = p1; c->p2_local = p2; c->n_local = nl;
    c->pen = mp.pen;
    c->bounce = mp.restitution;
    c->hardness = p.hardness;
    c->friction_coeff = mp.kinetic;
    c->cutoff = p.cutoff_vel;
    c->magic_c = mp.magic_c;
    c->magic_b = mp.magic_b;
    c->life = p.contact_life;
    c->live = true;
    e->contacts.push_back(std::move(c));
}

// ------------------------------------------------------------- rows ----
static Mat<6, 6> invMassMat(const Body* b) {
    Mat<6, 6> o;
    double im = b->invMass();
    M3 it = b->invTensor();
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) { o.v[i][j] = (i == j ? 1.0 : 0.0) * im; o.v[3 + i][3 + j] = it.m[i][j]; }
    return o;
}

template <int N>
static Mat<N, N> withCFM(Mat<N, N> m, double cfm) {
    for (int i = 0; i < N; i++) m.v[i][i] *= (1 + cfm);
    return m;
}

// Contact::updateSolverConstraints (PersistentConstraint.cpp:201-215) with the
// ContactConstraint and FrictionConstraint constructors
// (ConstraintSolver.cpp:240-261, 277-329)
static void rebuildContact(Contact* c, const Params& p, double dt) {
    Body* a = c->b1;
    Body* b = c->b2;
    V3 pa = a->q.rotate(c->p1_local) + a->com;
    V3 pb = b->q.rotate(c->p2_local) + b->com;
    V3 n = a->q.rotate(c->n_local);
    double depth = (pb - pa).dot(n) + c->pen;
    Vec<1> wn = p.warm_start_disabled ? Vec<1>() : scale(1.0, c->normal.impulse);
    Vec<2> wf = p.warm_start_disabled ? Vec<2>() : scale(1.0, c->friction.impulse);
    double pcc = std::min<double>(c->hardness * dt, 1.0 / dt);
    V3 rA = pa - a->com, rB = pa - b->com;
    Mat<6, 6> ma = invMassMat(a), mb = invMassMat(b);

    Row<1>& r = c->normal;
    r = Row<1>();
    r.a = a; r.b = b;
    Mat<1, 3> nd; nd.v[0][0] = n.x; nd.v[0][1] = n.y; nd.v[0][2] = n.z;
    put(r.ja, -nd, 0, 0);
    put(r.ja, nd * skew(rA), 0, 3);
    put(r.jb, nd, 0, 0);
    put(r.jb, (-nd) * skew(rB), 0, 3);
    r.ita = ma * r.ja.T();
    r.itb = mb * r.jb.T();
    Mat<1, 1> itv = r.ja * r.ita + r.jb * r.itb;
    r.minv = inverse(withCFM(itv, p.cfm));
    r.ptarget.v[0] = std::max<double>(0.0, depth - 0.05) * pcc;
    r.impulse = wn;

    Row<2>& f = c->friction;
    V3 su = c->fu, sw = c->fw;
    f = Row<2>();
    f.a = a; f.b = b;
    V3 u, w;
    n.perpBasis(&u, &w);
    f.impulse.v[0] = u.dot(su) * wf.v[0] + u.dot(sw) * wf.v[1];
    f.impulse.v[1] = w.dot(su) * wf.v[0] + w.dot(sw) * wf.v[1];
    Mat<1, 3> ud, wd;
    ud.v[0][0] = u.x; ud.v[0][1] = u.y; ud.v[0][2] = u.z;
    wd.v[0][0] = w.x; wd.v[0][1] = w.y; wd.v[0][2] = w.z;
    put(f.ja, ud, 0, 0);
    put(f.ja, (-ud) * skew(rA), 0, 3);
    put(f.jb, -ud, 0, 0);
    put(f.jb, ud * skew(rB), 0, 3);
    put(f.ja, wd, 1, 0);
    put(f.ja, (-wd) * skew(rA), 1, 3);
    put(f.jb, -wd, 1, 0);
    put(f.jb, wd * skew(rB), 1, 3);
    f.ita = ma * f.ja.T();
    f.itb = mb * f.jb.T();
    Mat<2, 2> fv = f.ja * f.ita + f.jb * f.itb;
    f.minv = inverse(withCFM(fv, p.cfm));
    c->fu = u;
    c->fw = w;
    c->static_ready = false;
    c->friction_built = true;
}

static Vec<6> velAng(const V3& v, const V3& w) { Vec<6> o; o.v[0] = v.x; o.v[1] = v.y; o.v[2] = v.z; o.v[3] = w.x; o.v[4] = w.y; o.v[5] = w.z; return o; }

// PGSConstraintStep (ConstraintSolver.cpp:12-40): Gauss-Seidel update with the
// projection applied to the accumulated impulse
template <int N, class Proj>
static void pgsStep(Row<N>& r, bool pseudo, Proj proj) {
    Vec<6>* va = pseudo ? &r.da->pv : &r.da->v;
    Vec<6>* vb = pseudo ? &r.db->pv : &r.db->v;
    Vec<N>* acc = pseudo ? &r.pimpulse : &r.impulse;
    Vec<N> target = pseudo ? r.ptarget : r.target;
    Vec<N> cur = r.value(*va, *vb);
    Vec<N> delta = target - cur;
    Vec<N> nw = *acc + mul(r.minv, delta);
    Vec<N> diff = proj(nw) - *acc;
    if (!diff.isZero()) {
        r.applyImpulse(diff, va, vb);
        *acc += diff;
    }
}

// PGS_solve (ConstraintSolver.cpp:80-213) for the contact rows of one island
static void pgsSolve(World& world, std::vector<RowRef>& rows, int n_vel, int n_pos, const std::vector<HoloSys*>& blocks,
                     int n_holo, double lin_err_threshold) {
    std::unordered_map<Body*, std::unique_ptr<DV>> dv;
    auto slot = [&](Body* b) { auto& s = dv[b]; if (!s) s = std::make_unique<DV>(); return s.get(); };
    for (RowRef& rr : rows) {
        if (rr.kind == 0) { rr.c->normal.da = slot(rr.c->b1); rr.c->normal.db = slot(rr.c->b2); }
        else if (rr.kind == 1) { rr.c->friction.da = slot(rr.c->b1); rr.c->friction.db = slot(rr.c->b2); }
        else { rr.j->row.da = slot(rr.j->b1); rr.j->row.db = slot(rr.j->b2); }
    }
    for (RowRef& rr : rows) {
        Contact* c = rr.c;
        if (rr.kind == 2) {
            jrowTarget(rr.j->row);
        } else if (rr.kind == 0) {
            Row<1>& r = c->normal;
            double cur = r.value(velAng(r.a->getVel(), r.a->getAngVel()), velAng(r.b->getVel(), r.b->getAngVel())).v[0];
            r.target.v[0] = (cur < -c->cutoff) ? -(1 + c->bounce) * cur : -cur;
        } else {
            Row<2>& r = c->friction;
            r.target = -r.value(velAng(r.a->getVel(), r.a->getAngVel()), velAng(r.b->getVel(), r.b->getAngVel()));
        }
    }
    for (RowRef& rr : rows) {
        if (rr.kind == 0) { Row<1>& r = rr.c->normal; if (!r.impulse.isZero()) r.applyImpulse(r.impulse, &r.da->v, &r.db->v); }
        else if (rr.kind == 1) { Row<2>& r = rr.c->friction; if (!r.impulse.isZero()) r.applyImpulse(r.impulse, &r.da->v, &r.db->v); }
        else jrowWarm(rr.j->row);
    }
    auto projN = [](const Vec<1>& x) { Vec<1> o; o.v[0] = std::max<double>(x.v[0], 0); return o; };
    for (int it = 0; it < n_vel; it++) {
        for (RowRef& rr : rows) {
            Contact* c = rr.c;
            if (rr.kind == 2) jrowStep(rr.j->row, false);
            else if (rr.kind == 0) pgsStep(c->normal, false, projN);
            else {
                pgsStep(c->friction, false, [c](const Vec<2>& x) {
                    double mx = c->friction_coeff * std::min<double>(std::numeric_limits<double>::infinity(), c->normal.impulse.v[0]);
                    double mag = std::sqrt(x.v[0] * x.v[0] + x.v[1] * x.v[1]);
                    if (mag > mx) {
                        c->static_ready = false;
                        double r = mx / mag;
                        Vec<2> o; o.v[0] = x.v[0] * r; o.v[1] = x.v[1] * r;
                        return o;
                    }
                    c->static_ready = true;
                    return x;
                });
            }
        }
    }
    for (int it = 0; it < n_pos; it++)
        for (RowRef& rr : rows) {
            if (rr.kind == 0) pgsStep(rr.c->normal, true, projN);
            else if (rr.kind == 2 && rr.j->row.pos) jrowStep(rr.j->row, true);   // needsPosCorrect
        }
    // direct solve of the holonomic systems after the sweeps
    // (ConstraintSolver.cpp:160-190); the holonomic impulse is carried into the
    // next warm start scaled by 0
    if (n_holo > 0 && !blocks.empty()) {
        for (int it = 0; it < n_holo; it++)
            for (HoloSys* h : blocks) {
                h->computeAndApply(false, -1.0);
                h->computeAndApply(true, lin_err_threshold);
            }
        const float scale = 0.0f;
        for (RowRef& rr : rows) {
            if (rr.kind != 2 || !rr.j->row.in_holo) continue;
            JRow& r = rr.j->row;
            for (int i = 0; i < r.n; i++) r.impulse[i] += scale * r.holo[i];
        }
    }
    // the island's velocity changes (ConstraintSolver.cpp:201-211), in the
    // velocity-change map's iteration order
    for (auto& kv : dv) {
        const DV& d = *kv.second;
        world.applyVelocityChange(kv.first, V3(d.v.v[0], d.v.v[1], d.v.v[2]), V3(d.v.v[3], d.v.v[4], d.v.v[5]),
                                  V3(d.pv.v[0], d.pv.v[1], d.pv.v[2]), V3(d.pv.v[3], d.pv.v[4], d.pv.v[5]));
    }
}

// PhysicsEngine::applyVelocityChange (PhysicsEngine.cpp:1113-1136): a sleeping
// body whose new velocity exceeds a quarter of the sleep velocity wakes its
// island, otherwise it stays at rest.  (The reference visits the island's
// bodies in the order of an unordered_map keyed by body address, so when one
// sleeping body of an island wakes it and another would have been zeroed,
// the outcome depends on that order; this restatement's order is its own.)
void World::applyVelocityChange(Body* b, const V3& dv, const V3& dw, const V3& dpv, const V3& dpw) {
    if (b->movement == FIXED || b->movement == KINEMATIC) return;
    b->vel += dv;
    b->ang_vel += dw;
    b->pvel += dpv;
    b->pang_vel += dpw;
    const double wake_vel = 0.25 * p.vel_sleep_coeff * p.g.mag();
    if (b->getAsleep() && (b->vel.mag() > wake_vel || b->ang_vel.mag() > wake_vel)) {
        wakeupIsland(b);
    } else if (b->getAsleep()) {
        b->vel = V3();
        b->ang_vel = V3();
    }
}

// PhysicsEngine::bodySleepy (PhysicsEngine.cpp:1221-1254): average velocity,
// angular velocity and accelerations over the recorded history below the
// thresholds (at least half the sleep delay recorded)
bool World::bodySleepy(const Body* r) const {
    const int n = (int)r->history.size();
    if (n == 0 || 2 * n < (p.sleep_delay / p.dt)) return false;
    V3 av, aw;
    for (const auto& s : r->history) { av += s.first; aw += s.second; }
    av /= n;
    aw /= n;
    V3 acc = (r->history.back().first - r->history.front().first) / (p.dt * (n - 1));
    V3 aacc = (r->history.back().second - r->history.front().second) / (p.dt * (n - 1));
    const double vel_eps = p.vel_sleep_coeff * p.g.mag();
    const double accel_eps = p.accel_sleep_coeff * p.g.mag();
    const double ang_accel_eps = p.accel_sleep_coeff * 2.5;
    return av.mag() <= vel_eps && aw.mag() <= p.ang_vel_eps && acc.mag() <= accel_eps && aacc.mag() <= ang_accel_eps;
}

// PhysicsEngine::readyToSleep (PhysicsEngine.cpp:1256-1258)
bool World::readyToSleep(const Body* b) const {
    return b->movement != KINEMATIC && (b->sleep_ready >= p.sleep_delay || b->movement == FIXED);
}

// PhysicsEngine::wakeupIsland / bfsVisitAll (PhysicsEngine.cpp:1263-1290):
// every dynamic body reachable through dynamic bodies wakes
void World::wakeupIsland(Body* foothold) {
    std::set<Body*> visited;
    std::vector<Body*> stack{foothold};
    while (!stack.empty()) {
        Body* cur = stack.back();
        stack.pop_back();
        if (!visited.insert(cur).second) continue;
        if (cur->movement == DYNAMIC) cur->wake();
        for (Edge* e : adj[cur]) {
            Body* o = e->other(cur);
            if (o->movement == DYNAMIC && !visited.count(o)) stack.push_back(o);
        }
    }
}

// detectCollision (CollisionDetect.cpp:57-150): primitive-type dispatch; the
// pairs the detectors take the other way round are flipped back so that the
// normal points away from b1
static Manifold collide(const Body* b1, const Body* b2) {
    int k1 = b1->kind, k2 = b2->kind;
    uint32_t i1 = b1->id, i2 = b2->id;
    const Material &m1 = b1->mat, &m2 = b2->mat;
    if (k1 == K_HULL) {
        if (k2 == K_HULL) return satPolyPoly(b1->shape, i1, m1, b2->shape, i2, m2);
        if (k2 == K_SPHERE) return satPolySphere(b1->shape, i1, m1, b2->sph, i2, m2);
        if (k2 == K_CAPSULE) return satPolyCapsule(b1->shape, i1, m1, b2->cap, i2, m2);
        return satPolyCylinder(b1->shape, i1, m1, b2->cyl, i2, m2);
    }
    if (k1 == K_SPHERE) {
        if (k2 == K_HULL) return flipped(satPolySphere(b2->shape, i2, m2, b1->sph, i1, m1));
        if (k2 == K_SPHERE) return sphereSphere(b1->sph, i1, m1, b2->sph, i2, m2);
        if (k2 == K_CAPSULE) return sphereCapsule(b1->sph, i1, m1, b2->cap, i2, m2);
        return sphereCylinder(b1->sph, i1, m1, b2->cyl, i2, m2);
    }
    if (k1 == K_CAPSULE) {
        if (k2 == K_HULL) return flipped(satPolyCapsule(b2->shape, i2, m2, b1->cap, i1, m1));
        if (k2 == K_SPHERE) return flipped(sphereCapsule(b2->sph, i2, m2, b1->cap, i1, m1));
        if (k2 == K_CAPSULE) return capsuleCapsule(b1->cap, i1, m1, b2->cap, i2, m2);
        return capsuleCylinder(b1->cap, i1, m1, b2->cyl, i2, m2);
    }
    if (k2 == K_HULL) return flipped(satPolyCylinder(b2->shape, i2, m2, b1->cyl, i1, m1));
    if (k2 == K_SPHERE) return flipped(sphereCylinder(b2->sph, i2, m2, b1->cyl, i1, m1));
    if (k2 == K_CAPSULE) return flipped(capsuleCylinder(b2->cap, i2, m2, b1->cyl, i1, m1));
    return cylinderCylinder(b1->cyl, i1, m1, b2->cyl, i2, m2);
}

// -------------------------------------------------------------- step ----
// RigidBody::applyImpulse (RigidBody.cpp:60-67)
static void applyImpulseAt(Body* b, V3 impulse, V3 pos) {
    V3 torque = (pos - b->com).cross(impulse);
    b->vel += b->invMass() * impulse;
    b->ang_vel += b->invTensor() * torque;
    b->alertWaking();
}

// The spring pass of maintainConstraintGraphApplyPoweredConstraints
// (PhysicsEngine.cpp:1309-1356): every edge once, in node order then edge
// order; a stiffness impulse along the attachment direction, then a damping
// impulse capped so it does not reverse the relative velocity
void World::applySprings(double dt) {
    std::set<Edge*> seen;
    for (auto& kv : nodes) {
        for (Edge* e : adj[kv.second]) {
            if (!seen.insert(e).second) continue;
            for (Spring* sp : e->springs) {
                Body* a = sp->b1; Body* b = sp->b2;
                V3 pa = a->trackedP(sp->k1), pb = b->trackedP(sp->k2);
                V3 diff = pb - pa;
                double distance = diff.mag();
                V3 dir = distance != 0 ? (pb - pa).normalize() : V3(0, -1, 0);
                double expand = sp->stiffness * (distance - sp->rest);
                applyImpulseAt(a, dir * expand * dt, pa);
                applyImpulseAt(b, -dir * expand * dt, pb);
                V3 rA = pa - a->com, rB = pb - b->com;
                V3 rdA = a->invTensor() * dir.cross(rA);
                V3 rdB = b->invTensor() * dir.cross(rB);
                double sens = 1.0 / (a->invMass() + b->invMass() + rA.cross(rdA).dot(dir) + rB.cross(rdB).dot(dir));
                // getVelOfPoint (RigidBody.cpp:153-155), with the reference's
                // crossed attachment points
                double velocity = (b->vel + b->ang_vel.cross(pa - b->com)).dot(dir) -
                                  (a->vel + a->ang_vel.cross(pb - a->com)).dot(dir);
                double dampen = sp->damping * velocity;
                double max_dampen = velocity * sens / dt;
                if (velocity > 0 && dampen > max_dampen) dampen = max_dampen;
                else if (velocity < 0 && dampen < max_dampen) dampen = max_dampen;
                applyImpulseAt(a, dir * dampen * dt, pa);
                applyImpulseAt(b, -dir * dampen * dt, pb);
            }
        }
    }
}

// PhysicsEngine::addSpring (PhysicsEngine.cpp:974-998): no collision filter,
// rest length < 0 means the attachment points' current distance
Spring* World::addSpring(Body* b1, Body* b2, V3 p1, V3 p2, double damping, double stiffness, double rest) {
    auto sp = std::make_unique<Spring>();
    sp->seq = constraint_seq++;
    sp->b1 = b1; sp->b2 = b2;
    b1->track_p.push_back(b1->local_origin + p1);
    sp->k1 = (int)b1->track_p.size() - 1;
    b2->track_p.push_back(b2->local_origin + p2);
    sp->k2 = (int)b2->track_p.size() - 1;
    if (rest < 0) rest = (b1->trackedP(sp->k1) - b2->trackedP(sp->k2)).mag();
    sp->stiffness = stiffness; sp->damping = damping; sp->rest = rest;
    getOrCreateEdge(b1, b2)->springs.push_back(sp.get());
    springs.push_back(std::move(sp));
    return springs.back().get();
}

void World::step() {
    // waking actions, sleep bookkeeping and gravity once per step
    // (PhysicsEngine.cpp:65-87; RigidBody::recordMovementState, RigidBody.cpp:347-352)
    for (auto& bp : bodies) {
        Body* b = bp.get();
        if (b->waking) wakeupIsland(b);
        b->waking = false;
        if (b->movement == DYNAMIC && !b->getAsleep()) {
            const int len = static_cast<int>(p.sleep_delay / p.dt);
            b->history.push_back({b->vel, b->ang_vel});
            while ((int)b->history.size() > len) b->history.erase(b->history.begin());
            if (bodySleepy(b)) {
                b->sleep_ready += p.dt;
            } else {
                b->non_sleepy++;
                if (b->non_sleepy >= p.non_sleepy_threshold) {
                    b->sleep_ready = 0.0;
                    b->non_sleepy = 0;
                }
            }
            b->vel += p.g * p.dt;
        }
    }

    // broadphase: every pair whose true AABBs overlap (AABB_Tree.h:153-224)
    last_pairs.clear();
    for (size_t i = 0; i < bodies.size(); i++)
        for (size_t j = i + 1; j < bodies.size(); j++)
            if (AABB::overlap(bodies[i]->aabb, bodies[j]->aabb)) last_pairs.push_back({bodies[i]->id, bodies[j]->id});

    // narrowphase + contact persistence (PhysicsEngine.cpp:167-326)
    for (auto& pr : last_pairs) {
        Body* b1 = bodies[pr.first - 1].get();
        Body* b2 = bodies[pr.second - 1].get();
        // at least one dynamic and one awake body (PhysicsEngine.cpp:174)
        if (!(b1->movement == DYNAMIC || b2->movement == DYNAMIC) || !(!b1->getAsleep() || !b2->getAsleep())) continue;
        if (b1->no_collide.count(b2)) continue;   // collisionAllowed (PhysicsEngine.cpp:570-572)
        if (b1->kind == K_MESH && b2->kind == K_MESH) continue;
        std::vector<Manifold> mans;
        // a body's primitives: itself, or the parts of a union
        auto prims = [](Body* b) {
            std::vector<Body*> v;
            if (b->kind == K_UNION) for (auto& g : b->parts) v.push_back(g.get());
            else v.push_back(b);
            return v;
        };
        if (b2->kind == K_MESH) {
            for (Body* g : prims(b1))
                for (Manifold& x : meshCollide(g, b2)) mans.push_back(x);
        } else if (b1->kind == K_MESH) {
            for (Body* g : prims(b2))
                for (Manifold& x : meshCollide(g, b1)) mans.push_back(flipped(x));
        } else {
            // primitive pairs, skipping those whose AABBs miss unless both
            // bodies have one primitive (PhysicsEngine.cpp:182-219)
            const std::vector<Body*> p1 = prims(b1), p2 = prims(b2);
            const bool single = p1.size() == 1 && p2.size() == 1;
            for (Body* g1 : p1)
                for (Body* g2 : p2) {
                    if (!single && !AABB::overlap(g1->aabb, g2->aabb)) continue;
                    Manifold man = collide(g1, g2);
                    if (man.max_pen > 0) mans.push_back(man);
                }
        }
        // manifolds with normals within 1 degree merge (PhysicsEngine.cpp:257-295)
        std::vector<char> merged(mans.size(), 0);
        for (size_t i = 0; i < mans.size(); i++) {
            if (merged[i]) continue;
            for (size_t j = i + 1; j < mans.size(); j++) {
                if (merged[j]) continue;
                double v = mans[i].normal.dot(mans[j].normal);
                if (1 - v < cosTol()) { mans[i] = mergeManifold(mans[i], mans[j]); merged[j] = 1; }
            }
            Manifold m = cullManifold(mans[i], 4);
            getOrCreateEdge(b1, b2);
            for (const ManifoldPoint& mp : m.pts) addContact(b1, b2, mp, m.normal);
        }
    }

    // holonomic systems of new joints (PhysicsEngine.cpp:360-362)
    const bool holo = p.pgs_holo > 0;
    if (holo) maintainHolonomicSystems();

    // islands in constraint_graph_nodes iteration order (PhysicsEngine.cpp:1536-1613)
    std::vector<std::vector<RowRef>> islands;
    std::vector<std::vector<HoloSys*>> island_blocks;
    std::set<Body*> visited;
    for (auto& kv : nodes) {
        Body* n = kv.second;
        if (n->movement != DYNAMIC || visited.count(n)) continue;
        std::vector<RowRef> rows;
        std::vector<HoloSys*> blocks;
        std::vector<Body*> island_bodies;
        bool all_ready = true;
        std::vector<Body*> stack{n};
        while (!stack.empty()) {
            Body* cur = stack.back();
            stack.pop_back();
            if (!visited.insert(cur).second) continue;
            if (cur->movement == DYNAMIC) {
                island_bodies.push_back(cur);
                bool kinematic_contact = false;
                for (Edge* e : adj[cur]) {
                    Body* o = e->other(cur);
                    if (o->movement == KINEMATIC) kinematic_contact = true;
                    // a sleeping body's edges to sleeping or fixed bodies carry no rows
                    if ((cur->getAsleep() && (o->getAsleep() || o->movement == FIXED)) || visited.count(o)) continue;
                    if (holo && e->h && std::find(blocks.begin(), blocks.end(), e->h) == blocks.end()) blocks.push_back(e->h);
                    // addSolverConstraints: limits only while reached, motors and
                    // pistons only while powered or past a limit
                    for (Joint* j : e->joints)
                        if (j->listed()) rows.push_back({2, nullptr, j});
                    for (auto& c : e->contacts)
                        if (c->live) { rows.push_back({0, c.get()}); rows.push_back({1, c.get()}); }
                }
                if (kinematic_contact || !readyToSleep(cur)) all_ready = false;
            }
            for (Edge* e : adj[cur]) {
                Body* o = e->other(cur);
                if (o->movement == DYNAMIC && !visited.count(o)) stack.push_back(o);
            }
        }
        // an island whose bodies are all ready sleeps instead of being solved
        if (p.sleeping && all_ready) {
            for (Body* b : island_bodies) b->sleep();
        } else if (!rows.empty()) {
            islands.push_back(std::move(rows));
            island_blocks.push_back(std::move(blocks));
        }
    }

    // substeps (PhysicsEngine.cpp:368-420)
    double dts = p.dt / p.substeps;
    for (int s = 0; s < p.substeps; s++) {
        bool first = s == 0, last = s == p.substeps - 1;
        if (!springs.empty()) applySprings(dts);
        std::vector<Edge*> dead;
        for (auto& e : edges) {
            // holonomic rows were rebuilt (and factorised) at the end of the
            // previous step for the first substep (PhysicsEngine.cpp:1397-1404)
            const bool in_holo = e->h != nullptr;
            for (Joint* j : e->joints)
                if (!(first && in_holo && holo && j->holonomic())) j->rebuild(p, dts, in_holo);
            for (auto& c : e->contacts) {
                bool skip = !c->live;
                if (last) { c->life--; c->live = false; }
                if (skip) continue;
                rebuildContact(c.get(), p, dts);
            }
            if (first) {
                auto& v = e->contacts;
                // Contact::isExpired (PersistentConstraint.h:74): a contact of a
                // sleeping body does not expire
                v.erase(std::remove_if(v.begin(), v.end(),
                                       [](const std::unique_ptr<Contact>& c) {
                                           return !c->b1->getAsleep() && !c->b2->getAsleep() && c->life < 0;
                                       }),
                        v.end());
                if (v.empty() && e->joints.empty() && e->springs.empty()) dead.push_back(e.get());
            }
        }
        for (Edge* e : dead) deleteEdge(e);
        for (size_t k = 0; k < islands.size(); k++)
            pgsSolve(*this, islands[k], p.pgs_vel, p.pgs_pos, island_blocks[k], first ? p.pgs_holo : 0, p.lin_err_threshold);
        for (auto& bp : bodies) {
            Body* b = bp.get();
            if (b->movement == FIXED || b->getAsleep()) continue;
            b->prev_com = b->com;
            b->prev_q = b->q;
            b->com += (b->vel + b->pvel) * dts;
            if (b->ang_vel.mag2() != 0) {
                bool no_gyro = p.gyro_disabled || b->movement == KINEMATIC;
                b->rotateWithGyro(dts, p.angle_ticks, no_gyro);
                V3 pr = b->pang_vel;
                b->q = Q::axisAngle(dts * pr.mag(), pr) * b->q;
            }
            b->pvel = V3();
            b->pang_vel = V3();
            b->updateInertiaTensor();
        }
    }
    for (auto& bp : bodies) {
        Body* b = bp.get();
        if (b->movement == FIXED || b->getAsleep()) continue;
        if (b->com != b->prev_com || b->q != b->prev_q) b->updateGeometry();
    }
    if (holo) updateHolonomicInverses();
}

}  // namespace cport

// ================================================================ C ABI ====
using namespace cport;

namespace {
thread_local std::string g_err;
int fail(const char* m, int code = CPGPU_ERR_INVALID_ARG) { g_err = m; return code; }
World* W(cpgpu_world* w) { return reinterpret_cast<World*>(w); }
Body* B(cpgpu_world* w, uint32_t id) {
    World* x = W(w);
    if (id == 0 || id > x->bodies.size()) return nullptr;
    return x->bodies[id - 1].get();
}
Material mat(const cpgpu_material* m) {
    Material o;
    if (m) { o.density = m->density; o.restitution = m->restitution; o.kinetic = m->kinetic_friction; o.stat = m->static_friction; }
    return o;
}
V3 v3(const double* p) { return p ? V3(p[0], p[1], p[2]) : V3(); }
void cutoff(World* w) { w->p.cutoff_vel = 2 * w->p.g.mag() * w->p.dt; }  // PhysicsEngine.h:203
}  // namespace

extern "C" {

const char* cport_last_error(void) { return g_err.c_str(); }
int cport_world_create(cpgpu_world** out) {
    World* w = new World();
    w->p.sleeping = false;  // as the device path: sleeping off unless enabled
    *out = reinterpret_cast<cpgpu_world*>(w);
    return CPGPU_OK;
}
int cport_world_destroy(cpgpu_world* w) { delete W(w); return CPGPU_OK; }
int cport_set_step_time(cpgpu_world* w, double dt) { W(w)->p.dt = dt; cutoff(W(w)); return CPGPU_OK; }
int cport_set_gravity(cpgpu_world* w, double x, double y, double z) { W(w)->p.g = V3(x, y, z); cutoff(W(w)); return CPGPU_OK; }
int cport_set_substep_count(cpgpu_world* w, int s) { if (s < 1) return fail("substeps < 1"); W(w)->p.substeps = s; return CPGPU_OK; }
int cport_set_pgs_iterations(cpgpu_world* w, int v, int p, int h) { W(w)->p.pgs_vel = v; W(w)->p.pgs_pos = p; W(w)->p.pgs_holo = h; return CPGPU_OK; }
int cport_set_sleeping_enabled(cpgpu_world* w, int e) {
    W(w)->p.sleeping = e != 0;
    return CPGPU_OK;
}
int cport_set_warm_start_disabled(cpgpu_world* w, int d) { W(w)->p.warm_start_disabled = d != 0; return CPGPU_OK; }
int cport_set_global_cfm(cpgpu_world* w, double c) { W(w)->p.cfm = c; return CPGPU_OK; }
int cport_set_angle_vel_update_tick_count(cpgpu_world* w, int n) { W(w)->p.angle_ticks = n; return CPGPU_OK; }
int cport_set_internal_gyro_forces_disabled(cpgpu_world* w, int d) { W(w)->p.gyro_disabled = d != 0; return CPGPU_OK; }

int cport_body_hull(cpgpu_world* w, const double* points, int n_points, const int* face_offsets, const int* face_indices,
                    int n_faces, const cpgpu_material* m, int movement, const double pos[3], uint32_t* out_id) {
    if (n_points < 4 || n_faces < 4) return fail("hull needs >= 4 points and faces");
    std::vector<V3> pts(n_points);
    for (int i = 0; i < n_points; i++) pts[i] = V3(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
    std::vector<std::vector<int>> faces(n_faces);
    for (int f = 0; f < n_faces; f++)
        for (int k = face_offsets[f]; k < face_offsets[f + 1]; k++) faces[f].push_back(face_indices[k]);
    Body* b = W(w)->addHull(pts, faces, mat(m), movement, v3(pos));
    if (out_id) *out_id = b->id;
    return CPGPU_OK;
}
// ConvexUnionGeometry::box (Geometry.cpp:14-37)
int cport_body_box(cpgpu_world* w, const double c[3], double dx, double dy, double dz, const cpgpu_material* m,
                   int movement, const double pos[3], uint32_t* out_id) {
    V3 p = v3(c);
    std::vector<V3> pts = {V3(p.x, p.y, p.z), V3(p.x + dx, p.y, p.z), V3(p.x + dx, p.y + dy, p.z), V3(p.x, p.y + dy, p.z),
                           V3(p.x, p.y, p.z + dz), V3(p.x + dx, p.y, p.z + dz), V3(p.x + dx, p.y + dy, p.z + dz), V3(p.x, p.y + dy, p.z + dz)};
    std::vector<std::vector<int>> faces = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
    Body* b = W(w)->addHull(pts, faces, mat(m), movement, v3(pos));
    if (out_id) *out_id = b->id;
    return CPGPU_OK;
}
// ConvexUnionGeometry::sphere (Geometry.cpp:39-41)
int cport_body_sphere(cpgpu_world* w, const double center[3], double radius, const cpgpu_material* m, int movement,
                      const double pos[3], uint32_t* out_id) {
    if (!(radius > 0)) return fail("sphere radius must be > 0");
    Body* b = W(w)->addSphere(v3(center), radius, mat(m), movement, v3(pos));
    if (out_id) *out_id = b->id;
    return CPGPU_OK;
}
// ConvexUnionGeometry::cylinder (Geometry.cpp:47-49)
int cport_body_cylinder(cpgpu_world* w, const double base[3], double radius, double height, const cpgpu_material* m,
                        int movement, const double pos[3], uint32_t* out_id) {
    if (!(radius > 0) || !(height > 0)) return fail("cylinder radius and height must be > 0");
    Body* b = W(w)->addCylinder(v3(base), radius, height, mat(m), movement, v3(pos));
    if (out_id) *out_id = b->id;
    return CPGPU_OK;
}
// ConvexUnionGeometry::capsule (Geometry.cpp:43-45)
int cport_body_capsule(cpgpu_world* w, const double bot[3], double radius, double drum_height, const cpgpu_material* m,
                       int movement, const double pos[3], uint32_t* out_id) {
    if (!(radius > 0) || !(drum_height >= 0)) return fail("capsule radius must be > 0 and drum height >= 0");
    Body* b = W(w)->addCapsule(v3(bot), radius, drum_height, mat(m), movement, v3(pos));
    if (out_id) *out_id = b->id;
    return CPGPU_OK;
}
// createRigidBody(ConvexUnionGeometry::merge of the primitives in order)
int cport_body_union(cpgpu_world* w, const cpgpu_primitive* prims, int n, int movement, const double pos[3],
                     uint32_t* out_id) {
    if (!prims || n < 1 || n > 255) return fail("a union needs 1 to 255 primitives");
    std::vector<std::unique_ptr<Body>> parts;
    for (int i = 0; i < n; i++) {
        const cpgpu_primitive& q = prims[i];
        auto g = std::make_unique<Body>();
        g->mat = mat(&q.mat);
        switch (q.kind) {
        case CPGPU_PRIM_HULL: {
            if (q.n_points < 4 || q.n_faces < 4) return fail("hull needs >= 4 points and faces");
            std::vector<V3> pts(q.n_points);
            for (int k = 0; k < q.n_points; k++) pts[k] = V3(q.points[3 * k], q.points[3 * k + 1], q.points[3 * k + 2]);
            std::vector<std::vector<int>> faces(q.n_faces);
            for (int f = 0; f < q.n_faces; f++)
                for (int k = q.face_offsets[f]; k < q.face_offsets[f + 1]; k++) faces[f].push_back(q.face_indices[k]);
            g->kind = K_HULL;
            g->src_shape.build(pts, faces);
            break;
        }
        case CPGPU_PRIM_BOX: {
            // ConvexUnionGeometry::box (Geometry.cpp:14-37)
            const V3 c = v3(q.p);
            const double dx = q.a, dy = q.b, dz = q.c;
            std::vector<V3> pts = {c, c + V3(dx, 0, 0), c + V3(dx, dy, 0), c + V3(0, dy, 0),
                                   c + V3(0, 0, dz), c + V3(dx, 0, dz), c + V3(dx, dy, dz), c + V3(0, dy, dz)};
            std::vector<std::vector<int>> faces = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
            g->kind = K_HULL;
            g->src_shape.build(pts, faces);
            break;
        }
        case CPGPU_PRIM_SPHERE:
            g->kind = K_SPHERE;
            g->sph_src.c = v3(q.p);
            g->sph_src.r = q.a;
            break;
        case CPGPU_PRIM_CYLINDER:
            g->kind = K_CYLINDER;
            g->cyl_src = makeCylinder(v3(q.p) + V3(0, q.b / 2.0, 0), q.a, q.b);
            break;
        case CPGPU_PRIM_CAPSULE:
            g->kind = K_CAPSULE;
            g->cap_src.c = v3(q.p) + V3(0, q.b / 2.0, 0);
            g->cap_src.axis = V3(0, 1, 0);
            g->cap_src.r = q.a;
            g->cap_src.h = q.b;
            break;
        default: return fail("bad primitive kind");
        }
        parts.push_back(std::move(g));
    }
    Body* b = W(w)->addUnion(std::move(parts), movement, v3(pos));
    if (out_id) *out_id = b->id;
    return CPGPU_OK;
}
// createRigidBody(StaticMeshGeometry(MeshInput), fixed) (PhysicsEngine.cpp:498-512)
int cport_body_mesh(cpgpu_world* w, const double* points, int n_points, const int* tris, int n_tris, const cpgpu_material* m,
                    int fixed, uint32_t* out_id) {
    if (!fixed) return fail("kinematic meshes are not implemented in the restatement", CPGPU_ERR_UNSUPPORTED);
    if (n_points < 3 || n_tris < 1) return fail("mesh needs >= 3 points and >= 1 triangle");
    std::vector<V3> pts(n_points);
    for (int i = 0; i < n_points; i++) pts[i] = V3(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
    std::vector<std::array<int, 3>> t(n_tris);
    for (int i = 0; i < n_tris; i++) {
        for (int k = 0; k < 3; k++) {
            int x = tris[3 * i + k];
            if (x < 0 || x >= n_points) return fail("mesh index out of range");
            t[i][k] = x;
        }
    }
    Body* b = W(w)->addMesh(pts, t, mat(m));
    if (out_id) *out_id = b->id;
    return CPGPU_OK;
}
int cport_body_set_velocity(cpgpu_world* w, uint32_t id, const double v[3]) {
    Body* b = B(w, id); if (!b) return fail("bad id"); b->vel = v3(v); b->alertWaking(); return CPGPU_OK;
}
int cport_body_set_ang_velocity(cpgpu_world* w, uint32_t id, const double v[3]) {
    Body* b = B(w, id); if (!b) return fail("bad id"); b->ang_vel = v3(v); b->alertWaking(); return CPGPU_OK;
}
// RigidBody::setOrientation (RigidBody.cpp:103-107): the world inertia tensor is
// left as it was until the next integration
int cport_body_set_orientation(cpgpu_world* w, uint32_t id, const double q[4]) {
    Body* b = B(w, id); if (!b) return fail("bad id");
    b->q = Q(q[0], q[1], q[2], q[3]);
    b->updateGeometry();
    b->alertWaking();
    return CPGPU_OK;
}
int cport_body_set_position(cpgpu_world* w, uint32_t id, const double p[3]) {
    Body* b = B(w, id); if (!b) return fail("bad id");
    b->com += v3(p) - b->trackedP(0);
    b->updateGeometry();
    b->alertWaking();
    return CPGPU_OK;
}
// RigidBody::setMass (RigidBody.cpp:80-89)
int cport_body_set_mass(cpgpu_world* w, uint32_t id, double m) {
    Body* b = B(w, id); if (!b) return fail("bad id");
    double r = m / b->mass;
    b->ref_tensor *= r; b->ref_inv_tensor /= r; b->tensor *= r; b->inv_tensor /= r;
    b->mass = m;
    return CPGPU_OK;
}
// PhysicsEngine::addBallSocketConstraint (PhysicsEngine.cpp:664-687)
int cport_add_ball_socket(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double strength,
                          uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addJoint(3, x, y, v3(a1), v3(a2), V3(), V3(), strength, 0);
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addDistanceConstraint (PhysicsEngine.cpp:623-660)
int cport_add_distance(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double target,
                       double strength, uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addJoint(1, x, y, v3(a1), v3(a2), V3(), V3(), strength, 0, target);
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addWeldConstraint (PhysicsEngine.cpp:896-915)
int cport_add_weld(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double ps,
                   double rs, uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addJoint(6, x, y, v3(a1), v3(a2), V3(), V3(), ps, rs);
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addTwistLimitConstraint (PhysicsEngine.cpp:952-972)
int cport_add_twist_limit(cpgpu_world* w, uint32_t b1, uint32_t b2, const double ax1[3], const double ax2[3],
                          double min_angle, double max_angle, double rs, uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addTwist(x, y, v3(ax1), v3(ax2), min_angle, max_angle, rs);
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addConeLimitConstraint (PhysicsEngine.cpp:926-946)
int cport_add_cone_limit(cpgpu_world* w, uint32_t b1, uint32_t b2, const double ax1[3], const double ax2[3],
                         double max_angle, double rs, uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addCone(x, y, v3(ax1), v3(ax2), max_angle, rs);
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addSpring (PhysicsEngine.cpp:974-998)
int cport_add_spring(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double damping,
                     double stiffness, double rest, uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addSpring(x, y, v3(a1), v3(a2), damping, stiffness, rest);
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addSliderConstraint (PhysicsEngine.cpp:773-806)
int cport_add_slider(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                     const double ax1[3], const double ax2[3], double ps, double rs, uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addJoint(5, x, y, v3(a1), v3(a2), v3(ax1), v3(ax2), ps, rs)->slider = true;
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addSlidingHingeConstraint (PhysicsEngine.cpp:860-890)
int cport_add_sliding_hinge(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                            const double ax1[3], const double ax2[3], double ps, double rs, uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addJoint(4, x, y, v3(a1), v3(a2), v3(ax1), v3(ax2), ps, rs);
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addHingeConstraint (PhysicsEngine.cpp:693-723)
int cport_add_hinge(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], const double ax1[3],
                    const double ax2[3], double ps, double rs, uint32_t* out_id) {
    Body* x = B(w, b1); Body* y = B(w, b2);
    if (!x || !y || x == y) return fail("bad body id");
    W(w)->addJoint(5, x, y, v3(a1), v3(a2), v3(ax1), v3(ax2), ps, rs);
    if (out_id) *out_id = (uint32_t)(W(w)->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addMotorConstraint (PhysicsEngine.cpp:725-763): on a hinge or
// a sliding hinge
int cport_add_motor(cpgpu_world* w, uint32_t base, double min_angle, double max_angle, uint32_t* out_id) {
    World* x = W(w);
    Joint* b = x->jointById(base);
    if (!b) return fail("bad constraint id");
    const bool hinge = b->n == 5 && !b->slider && !b->powered() && !b->cone && !b->twist;
    if (!hinge && b->n != 4) return fail("a motor needs a hinge or a sliding hinge");
    x->addMotor(b, min_angle, max_angle);
    if (out_id) *out_id = (uint32_t)(x->constraint_seq - 1);
    return CPGPU_OK;
}
// PhysicsEngine::addPistonConstraint (PhysicsEngine.cpp:808-852): on a slider
// or a sliding hinge; the id names the powered joint (its slide limit is the
// joint before it)
int cport_add_piston(cpgpu_world* w, uint32_t base, double min_pos, double max_pos, uint32_t* out_id) {
    World* x = W(w);
    Joint* b = x->jointById(base);
    if (!b) return fail("bad constraint id");
    if (!(b->n == 5 && b->slider) && b->n != 4) return fail("a piston needs a slider or a sliding hinge");
    x->addPiston(b, min_pos, max_pos);
    if (out_id) *out_id = (uint32_t)(x->constraint_seq - 1);
    return CPGPU_OK;
}
// setMotorOff / setMotorConstantTorque / setMotorTargetVelocity /
// setMotorTargetPosition (PhysicsEngine.cpp:1857-1912) and the piston's
// (:1800-1855): mode 0 off, 1 constant torque (force) = max, 2 target velocity,
// 3 target position; each sets the fields the reference's setter sets and
// alerts both bodies
static int setPowered(cpgpu_world* w, uint32_t id, bool motor, int mode, double max, double target) {
    World* x = W(w);
    Joint* j = x->jointById(id);
    if (!j) return fail("bad constraint id");
    if (motor ? !j->motor : !j->piston) return fail(motor ? "not a motor" : "not a piston");
    if (mode < 0 || mode > 3) return fail("bad mode");
    j->mode = mode;
    if (mode >= 1) j->power_max = max;
    if (mode == 2) j->target_vel = target;
    if (mode == 3) j->target_pos = target;
    j->b1->alertWaking();
    j->b2->alertWaking();
    return CPGPU_OK;
}
int cport_set_motor(cpgpu_world* w, uint32_t id, int mode, double max_torque, double target) {
    return setPowered(w, id, true, mode, max_torque, target);
}
int cport_set_piston(cpgpu_world* w, uint32_t id, int mode, double max_force, double target) {
    return setPowered(w, id, false, mode, max_force, target);
}
// getMotorAngularPosition / getPistonPosition (PhysicsEngine.cpp:1914-1930)
int cport_get_motor_position(cpgpu_world* w, uint32_t id, double* out) {
    Joint* j = W(w)->jointById(id);
    if (!j || !j->motor) return fail("not a motor");
    *out = j->position;
    return CPGPU_OK;
}
int cport_get_piston_position(cpgpu_world* w, uint32_t id, double* out) {
    Joint* j = W(w)->jointById(id);
    if (!j || !j->piston) return fail("not a piston");
    *out = j->position;
    return CPGPU_OK;
}
// Test hook: replace the mass properties computed at creation by given ones
// (the reference's, so that both engines start from bit-identical bodies).
// Valid right after the body was created.
int cport_body_set_mass_properties(cpgpu_world* w, uint32_t id, double mass, const double* com_geom, const double* tensor) {
    Body* b = B(w, id); if (!b) return fail("bad id");
    M3 t;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) t.m[i][j] = tensor[3 * i + j];
    W(w)->placeBody(b, mass, v3(com_geom), t);
    return CPGPU_OK;
}
// Mass properties computed by the restatement (same layout as cpref_get_mass_properties).
int cport_get_mass_properties(cpgpu_world* w, uint32_t id, double* mass, double* com_geom, double* tensor) {
    Body* b = B(w, id); if (!b) return fail("bad id");
    *mass = b->mass;
    com_geom[0] = -b->local_origin.x; com_geom[1] = -b->local_origin.y; com_geom[2] = -b->local_origin.z;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) tensor[3 * i + j] = b->ref_tensor.m[i][j];
    return CPGPU_OK;
}
// Joint warm-start state (same layout as cpgpu_get/set_joint_state): the
// row impulse (kStateDof per joint), the tangent basis u, w, and for limits
// the twist angle and whether the limit was reached at the last rebuild
int cport_get_joint_state(cpgpu_world* w, double* impulse, double* u, double* wv, double* aux, int* n) {
    World* x = W(w);
    *n = (int)x->joints.size();
    for (size_t j = 0; j < x->joints.size(); j++) {
        const Joint& J = *x->joints[j];
        for (int k = 0; k < kStateDof; k++) if (impulse) impulse[kStateDof * j + k] = k < J.row.n ? J.row.impulse[k] : 0.0;
        if (u) { u[3 * j] = J.u.x; u[3 * j + 1] = J.u.y; u[3 * j + 2] = J.u.z; }
        if (wv) { wv[3 * j] = J.w.x; wv[3 * j + 1] = J.w.y; wv[3 * j + 2] = J.w.z; }
        if (aux) {
            aux[2 * j] = J.powered() ? J.position : J.cur_angle;
            aux[2 * j + 1] = J.motor ? J.prev_vel
                             : (J.slide_limit || J.piston) ? (J.exceeded ? 1.0 : 0.0)
                             : ((J.cone || J.twist) && !J.inactive) ? 1.0 : 0.0;
        }
    }
    return CPGPU_OK;
}
// Import: the impulses become the warm start of every joint's next rebuild
// (the rebuild of the first substep for rows inside a holonomic system, which
// the restatement otherwise takes from the end of the previous step, is
// redone here from the current poses with the imported impulses).
int cport_set_joint_state(cpgpu_world* w, const double* impulse, const double* u, const double* wv, const double* aux,
                          int n) {
    World* x = W(w);
    if (n != (int)x->joints.size()) return fail("joint count mismatch");
    for (int j = 0; j < n; j++) {
        Joint& J = *x->joints[j];
        for (int k = 0; k < std::min(J.row.n, kStateDof); k++) if (impulse) J.row.impulse[k] = impulse[kStateDof * j + k];
        if (u) J.u = V3(u[3 * j], u[3 * j + 1], u[3 * j + 2]);
        if (wv) J.w = V3(wv[3 * j], wv[3 * j + 1], wv[3 * j + 2]);
        if (aux) {
            if (J.powered()) J.position = aux[2 * j];
            else J.cur_angle = aux[2 * j];
            if (J.cone || J.twist) J.inactive = aux[2 * j + 1] == 0.0;
            if (J.motor) J.prev_vel = aux[2 * j + 1];
            if (J.slide_limit || J.piston) J.exceeded = aux[2 * j + 1] != 0.0;
        }
    }
    if (x->p.pgs_holo > 0) {
        // the rows inside holonomic systems are rebuilt (and factorised) from
        // the current poses, as the end of the exporting world's last step
        // did; that rebuild re-projects the warm impulses onto the tangent
        // basis of the same poses, which the exported impulses and bases
        // already are, so the imported values are put back unchanged.  A world
        // that has not stepped yet forms its systems first (its first step
        // would otherwise form them and rebuild their rows once more).
        x->maintainHolonomicSystems();
        x->updateHolonomicInverses();
        for (int j = 0; j < n; j++) {
            Joint& J = *x->joints[j];
            for (int k = 0; k < std::min(J.row.n, kStateDof); k++) if (impulse) J.row.impulse[k] = impulse[kStateDof * j + k];
            if (u) J.u = V3(u[3 * j], u[3 * j + 1], u[3 * j + 2]);
            if (wv) J.w = V3(wv[3 * j], wv[3 * j + 1], wv[3 * j + 2]);
        }
    }
    return CPGPU_OK;
}
// Test hook: number of holonomic systems and the largest verifyInverse error
// over them (factorisations as left by the last step).
int cport_holonomic_check(cpgpu_world* w, int* n_systems, int* max_degree, double* max_err) {
    World* x = W(w);
    *n_systems = (int)x->systems.size();
    *max_degree = 0;
    *max_err = 0;
    for (auto& h : x->systems) {
        *max_degree = std::max(*max_degree, h->degree);
        *max_err = std::max(*max_err, h->inverseError(x->p.cfm));
    }
    return CPGPU_OK;
}
int cport_step(cpgpu_world* w, int n) { for (int i = 0; i < n; i++) W(w)->step(); return CPGPU_OK; }
int cport_num_bodies(cpgpu_world* w, int* n) { *n = (int)W(w)->bodies.size(); return CPGPU_OK; }
// ---- ray queries (PhysicsEngine::raycastFirstIntersection,
// PhysicsEngine.cpp:582-609) against the bodies' current geometry: every
// body whose current AABB the ray crosses (the reference filters with its
// broadphase tree, whose leaves hold the AABBs of the start of the last step)
// is tested with its primitive's ray test; the nearest hit wins (strictly
// nearer replaces, in body order).
namespace {
struct RayHit { bool hit = false; V3 p, n; double t = 0; };

// AABB::rayIntersectsAABB (AABB.h:143-172)
bool rayAABB(const AABB& b, const V3& o, const V3& d) {
    double t_min = -std::numeric_limits<double>::infinity(), t_max = std::numeric_limits<double>::infinity();
    const double eps = 0.00000000001;
    for (int i = 0; i < 3; i++) {
        const double oi = o[i], di = d[i], lo = b.mn[i], hi = b.mx[i];
        if (std::abs(di) < eps) {
            if (oi < lo || oi > hi) return false;
        } else {
            double t0 = (lo - oi) / di, t1 = (hi - oi) / di;
            if (t0 > t1) std::swap(t0, t1);
            t_min = std::max<double>(t0, t_min);
            t_max = std::min<double>(t1, t_max);
            if (t_max < 0 || t_max < t_min) return false;
        }
    }
    return true;
}

// the smaller non-negative root of a t^2 + b t + c (both ray tests below).
// As in the reference, a ray parallel to a cylinder axis (a = b = 0) passes
// the double-root test with t = NaN and is reported as a hit at NaN.
bool rayRoot(double a, double b, double c, double* t) {
    double radical = b * b - 4 * a * c;
    if (radical < 0) return false;
    if (radical == 0) {
        *t = -0.5 * b / a;
        return !(*t < 0);
    }
    double t1 = (-b + std::sqrt(radical)) / (2 * a), t2 = (-b - std::sqrt(radical)) / (2 * a);
    if (t1 < 0 && t2 < 0) return false;
    *t = t1 < 0 ? t2 : t2 < 0 ? t1 : std::min<double>(t1, t2);
    return true;
}

// testRayAgainstSphere (ConvexPrimitive.cpp:170-202)
RayHit raySphere(const V3& o, const V3& d, const V3& c, double r) {
    V3 rel = o - c;
    double t;
    if (!rayRoot(d.mag2(), 2 * rel.dot(d), rel.mag2() - r * r, &t)) return {};
    V3 hp = o + t * d;
    return RayHit{true, hp, (hp - c).normalize(), t};
}

// testRayAgainstCylinderSide (ConvexPrimitive.cpp:113-168)
RayHit rayCylSide(const V3& o, const V3& d, const V3& c, double r, double h, const V3& ax) {
    V3 u = d - ax * ax.dot(d);
    V3 w = o - c - ax * (ax.dot(o) - ax.dot(c));
    double a = u.x * u.x + u.y * u.y + u.z * u.z;
    double b = 2 * (u.x * w.x + u.y * w.y + u.z * w.z);
    double cc = w.x * w.x + w.y * w.y + w.z * w.z - r * r;
    double t;
    if (!rayRoot(a, b, cc, &t)) return {};
    V3 hp = o + t * d;
    double x = (hp - c).dot(ax);
    if (std::abs(x) > h / 2.0) return {};
    return RayHit{true, hp, ((hp - c) - ax * x).normalize(), t};
}

// checkDiskIntersection (ConvexPrimitive.cpp:300-306)
RayHit rayDisk(const V3& o, const V3& d, const V3& c, const V3& n, double r) {
    double t = n.dot(c - o) / n.dot(d);
    V3 ip = o + t * d;
    if (t < 0 || (ip - c).mag2() > r * r) return {};
    return RayHit{true, ip, n, t};
}

void nearer(RayHit* out, const RayHit& h) {
    if (h.hit && (!out->hit || h.t < out->t)) *out = h;
}

// Polyhedron::testRayIntersection (ConvexPrimitive.cpp:731-758): the first
// face, in surface order, whose plane the ray enters from outside at a point
// inside the face
RayHit rayHull(const Hull& h, const V3& o, const V3& d) {
    for (size_t f = 0; f < h.faces.size(); f++) {
        const std::vector<int>& s = h.faces[f];
        V3 sp = h.pts[s[0]];
        V3 n = h.faceNormal((int)f);
        const double eps = 0.0001;
        if (d.dot(n) > -eps || (o - sp).dot(n) < 0) continue;
        double t = n.dot(sp - o) / n.dot(d);
        V3 ip = o + t * d;
        bool inside = true;
        for (size_t i = 0; i < s.size() && inside; i++) {
            V3 e1 = h.pts[s[i]], e2 = h.pts[s[i + 1 == s.size() ? 0 : i + 1]];
            if ((e2 - e1).cross(n).dot(ip - e1) > 0) inside = false;
        }
        if (inside) return RayHit{true, ip, n, t};
    }
    return {};
}

// StaticMeshGeometry::testRayIntersection (Geometry.cpp:867-897): triangles
// whose AABB the ray crosses, nearest plane hit inside the triangle (a later
// triangle at an equal distance replaces)
RayHit rayMesh(const Body* m, const V3& o, const V3& d) {
    RayHit best;
    for (const MeshTri& tri : m->tris) {
        if (!rayAABB(tri.aabb, o, d)) continue;
        if (std::abs(tri.normal.dot(d)) < 0.0000000001) continue;
        double t = -(o - tri.v[1]).dot(tri.normal) / d.dot(tri.normal);
        if (t < 0 || (best.hit && best.t < t)) continue;
        V3 hp = o + t * d;
        if ((hp - tri.ep1[0]).dot(tri.out[0]) > 0 || (hp - tri.ep1[1]).dot(tri.out[1]) > 0 ||
            (hp - tri.ep1[2]).dot(tri.out[2]) > 0)
            continue;
        best = RayHit{true, hp, tri.normal, t};
    }
    return best;
}

// RigidBody::checkRayIntersection (RigidBody.cpp:185-204) and the
// primitives' testRayIntersection (ConvexPrimitive.cpp:205-212, 308-318,
// 403-411, 445-447)
RayHit rayBody(const Body* b, const V3& o, const V3& d) {
    if (b->kind == K_UNION) {   // each primitive behind its own AABB (RigidBody.cpp:188-197)
        RayHit out;
        for (const auto& g : b->parts) {
            if (b->parts.size() != 1 && !rayAABB(g->aabb, o, d)) continue;
            nearer(&out, rayBody(g.get(), o, d));
        }
        return out;
    }
    switch (b->kind) {
    case K_MESH: return rayMesh(b, o, d);
    case K_SPHERE: return raySphere(o, d, b->sph.c, b->sph.r);
    case K_CYLINDER: {
        const CylG& c = b->cyl;
        RayHit out = rayCylSide(o, d, c.c, c.r, c.h, c.axis);
        double sgn = c.axis.dot(d) < 0 ? 1.0 : -1.0;
        nearer(&out, rayDisk(o, d, c.c + sgn * c.axis * (c.h / 2.0), c.axis, c.r));
        return out;
    }
    case K_CAPSULE: {
        const CapG& c = b->cap;
        RayHit out = rayCylSide(o, d, c.c, c.r, c.h, c.axis);
        nearer(&out, raySphere(o, d, c.c + c.axis * (c.h / 2.0), c.r));
        nearer(&out, raySphere(o, d, c.c - c.axis * (c.h / 2.0), c.r));
        return out;
    }
    default: return rayHull(b->shape, o, d);
    }
}
}  // namespace

int cport_raycast(cpgpu_world* w, const double* origins, const double* dirs, int n_rays, const uint32_t* ignore,
                  int n_ignore, uint32_t* hit_body, double* hit_pos, double* hit_normal, double* hit_dist) {
    if (n_rays < 0 || (n_rays > 0 && (!origins || !dirs)) || n_ignore < 0 || (n_ignore > 0 && !ignore))
        return fail("bad ray arguments");
    World* wd = W(w);
    std::set<uint32_t> skip(ignore, ignore + n_ignore);
    for (int k = 0; k < n_rays; k++) {
        V3 o = v3(origins + 3 * k), d = v3(dirs + 3 * k);
        RayHit best;
        uint32_t id = 0;
        for (const auto& b : wd->bodies) {
            if (skip.count(b->id) || !rayAABB(b->aabb, o, d)) continue;
            RayHit h = rayBody(b.get(), o, d);
            if (h.hit && (!best.hit || h.t < best.t)) { best = h; id = b->id; }
        }
        if (hit_body) hit_body[k] = id;
        for (int i = 0; i < 3; i++) {
            if (hit_pos) hit_pos[3 * k + i] = best.hit ? best.p[i] : 0;
            if (hit_normal) hit_normal[3 * k + i] = best.hit ? best.n[i] : 0;
        }
        if (hit_dist) hit_dist[k] = best.hit ? best.t : -1;
    }
    return CPGPU_OK;
}

int cport_get_body_state(cpgpu_world* w, double* com, double* quat, double* vel, double* ang) {
    World* x = W(w);
    for (size_t i = 0; i < x->bodies.size(); i++) {
        const Body* b = x->bodies[i].get();
        V3 v = b->getVel(), a = b->getAngVel();
        if (com) { com[3 * i] = b->com.x; com[3 * i + 1] = b->com.y; com[3 * i + 2] = b->com.z; }
        if (quat) { quat[4 * i] = b->q.r; quat[4 * i + 1] = b->q.i; quat[4 * i + 2] = b->q.j; quat[4 * i + 3] = b->q.k; }
        if (vel) { vel[3 * i] = v.x; vel[3 * i + 1] = v.y; vel[3 * i + 2] = v.z; }
        if (ang) { ang[3 * i] = a.x; ang[3 * i + 1] = a.y; ang[3 * i + 2] = a.z; }
    }
    return CPGPU_OK;
}
int cport_get_asleep(cpgpu_world* w, int* flags) {
    World* x = W(w);
    for (size_t i = 0; i < x->bodies.size(); i++) flags[i] = x->bodies[i]->getAsleep() ? 1 : 0;
    return CPGPU_OK;
}
// State import: poses and velocities, then the derived tensors and geometry
// are recomputed from the new poses.
int cport_set_body_state(cpgpu_world* w, const double* com, const double* quat, const double* vel, const double* ang) {
    World* x = W(w);
    for (size_t i = 0; i < x->bodies.size(); i++) {
        Body* b = x->bodies[i].get();
        if (com) b->com = V3(com[3 * i], com[3 * i + 1], com[3 * i + 2]);
        if (quat) b->q = Q(quat[4 * i], quat[4 * i + 1], quat[4 * i + 2], quat[4 * i + 3]);
        if (vel) b->vel = V3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        if (ang) b->ang_vel = V3(ang[3 * i], ang[3 * i + 1], ang[3 * i + 2]);
        if (b->movement != FIXED) b->updateInertiaTensor();
        b->updateGeometry();
    }
    return CPGPU_OK;
}
int cport_get_aabbs(cpgpu_world* w, double* out) {
    World* x = W(w);
    for (size_t i = 0; i < x->bodies.size(); i++) {
        const AABB& a = x->bodies[i]->aabb;
        double* o = out + 6 * i;
        o[0] = a.mn.x; o[1] = a.mn.y; o[2] = a.mn.z; o[3] = a.mx.x; o[4] = a.mx.y; o[5] = a.mx.z;
    }
    return CPGPU_OK;
}
int cport_get_pairs(cpgpu_world* w, uint32_t* pairs, int cap, int* n) {
    World* x = W(w);
    *n = (int)x->last_pairs.size();
    for (int i = 0; i < *n && i < cap; i++) { pairs[2 * i] = x->last_pairs[i].first; pairs[2 * i + 1] = x->last_pairs[i].second; }
    return CPGPU_OK;
}
int cport_get_contacts(cpgpu_world* w, cpgpu_contact* out, int cap, int* n) {
    World* x = W(w);
    std::vector<std::pair<std::pair<uint32_t, uint32_t>, Edge*>> es;
    for (auto& e : x->edges) {
        uint32_t a = e->n1->id, b = e->n2->id;
        es.push_back({{std::min(a, b), std::max(a, b)}, e.get()});
    }
    std::sort(es.begin(), es.end(), [](const auto& p, const auto& q) { return p.first < q.first; });
    int k = 0;
    for (auto& pe : es) {
        for (auto& c : pe.second->contacts) {
            if (out && k < cap) {
                cpgpu_contact& o = out[k];
                std::memset(&o, 0, sizeof(o));
                o.b1 = c->b1->id; o.b2 = c->b2->id;
                o.live = c->live; o.memory_life = c->life;
                o.magic_c = c->magic_c; o.magic_b = c->magic_b;
                const V3* vs[3] = {&c->p1_local, &c->p2_local, &c->n_local};
                double* ds[3] = {o.p_local_b1, o.p_local_b2, o.n_local_b1};
                for (int t = 0; t < 3; t++) { ds[t][0] = vs[t]->x; ds[t][1] = vs[t]->y; ds[t][2] = vs[t]->z; }
                o.pen_depth = c->pen; o.bounce = c->bounce; o.friction_coeff = c->friction_coeff;
                o.normal_impulse = c->normal.impulse.v[0];
                o.friction_impulse[0] = c->friction.impulse.v[0]; o.friction_impulse[1] = c->friction.impulse.v[1];
                o.friction_u[0] = c->fu.x; o.friction_u[1] = c->fu.y; o.friction_u[2] = c->fu.z;
                o.friction_w[0] = c->fw.x; o.friction_w[1] = c->fw.y; o.friction_w[2] = c->fw.z;
                o.static_ready = c->static_ready;
            }
            k++;
        }
    }
    *n = k;
    return CPGPU_OK;
}
// State import of the persistent contact graph (same layout and order as
// cport_get_contacts); edges without contacts are dropped.
int cport_set_contacts(cpgpu_world* w, const cpgpu_contact* in, int n) {
    World* x = W(w);
    // contacts are replaced; edges that carry joints stay (with their joints)
    std::vector<Edge*> all;
    for (auto& e : x->edges) {
        e->contacts.clear();
        if (e->joints.empty() && e->springs.empty()) all.push_back(e.get());
    }
    for (Edge* e : all) x->deleteEdge(e);
    for (int k = 0; k < n; k++) {
        const cpgpu_contact& r = in[k];
        Body* b1 = B(w, r.b1);
        Body* b2 = B(w, r.b2);
        if (!b1 || !b2 || r.b1 >= r.b2) return fail("bad contact body ids");
        Edge* e = x->getOrCreateEdge(b1, b2);
        auto c = std::make_unique<Contact>();
        c->b1 = b1; c->b2 = b2;
        c->p1_local = v3(r.p_local_b1); c->p2_local = v3(r.p_local_b2); c->n_local = v3(r.n_local_b1);
        c->pen = r.pen_depth; c->bounce = r.bounce; c->hardness = x->p.hardness; c->friction_coeff = r.friction_coeff;
        c->cutoff = x->p.cutoff_vel;
        c->magic_c = r.magic_c; c->magic_b = r.magic_b;
        c->life = r.memory_life; c->live = r.live != 0;
        c->normal.impulse.v[0] = r.normal_impulse;
        c->friction.impulse.v[0] = r.friction_impulse[0]; c->friction.impulse.v[1] = r.friction_impulse[1];
        c->fu = v3(r.friction_u); c->fw = v3(r.friction_w);
        c->static_ready = r.static_ready != 0;
        e->contacts.push_back(std::move(c));
    }
    return CPGPU_OK;
}

}  // extern "C"
