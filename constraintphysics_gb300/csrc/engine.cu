// engine.cu — host side of the device path: worlds, batches, upload/download,
// the per-step launch sequence (captured in CUDA graphs) and the C ABI of
// include/cpgpu.h.
//
// A cpgpu_world mirrors one phyz::PhysicsEngine (PhysicsEngine.h:60-161): the
// host keeps its bodies, shapes and parameters; the dynamic state lives on the
// device once the world has stepped.  Mutations between steps pull the state
// back, change the host mirror and re-upload on the next step.  A batch packs
// many worlds into one set of segmented device arrays.
#include <algorithm>
#include <thread>
#include <array>
#include <cmath>
#include <chrono>
#include <deque>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "hull.hpp"
#include "kernels.cuh"

extern "C" {
#include "../../include/cpgpu.h"
}

namespace cpgpu {

thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

void set_last_error(const char* msg) { g_err = msg; }

#define CK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) throw CudaFail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct CudaFail {
    std::string msg;
    explicit CudaFail(std::string m) : msg(std::move(m)) {}
};
struct ApiFail {
    int code;
    std::string msg;
};

// ---------------------------------------------------------------- host mirror ----
struct Quat { double r = 1, i = 0, j = 0, k = 0; };

static D3 qrot(const Quat& q, const D3& v) {
    double r = q.r, i = q.i, j = q.j, k = q.k;
    return D3(v.x * (r * r + i * i - j * j - k * k) + v.y * (2 * i * j - 2 * r * k) + v.z * (2 * i * k + 2 * r * j),
              v.x * (2 * i * j + 2 * r * k) + v.y * (r * r - i * i + j * j - k * k) + v.z * (2 * j * k - 2 * r * i),
              v.x * (2 * i * k - 2 * r * j) + v.y * (2 * j * k + 2 * r * i) + v.z * (r * r - i * i - j * j + k * k));
}
static Quat qnorm(const Quat& q) {
    double m = std::sqrt(q.r * q.r + q.i * q.i + q.j * q.j + q.k * q.k);
    return Quat{q.r / m, q.i / m, q.j / m, q.k / m};
}

static void inv3(const double a[9], double o[9]) {
    double A = a[0], B = a[1], C = a[2], D = a[3], E = a[4], F = a[5], G = a[6], H = a[7], I = a[8];
    double dt = A * (E * I - F * H) - B * (D * I - F * G) + C * (D * H - E * G);
    o[0] = (E * I - F * H) / dt; o[1] = (C * H - B * I) / dt; o[2] = (B * F - C * E) / dt;
    o[3] = (F * G - D * I) / dt; o[4] = (A * I - C * G) / dt; o[5] = (C * D - A * F) / dt;
    o[6] = (D * H - E * G) / dt; o[7] = (B * G - A * H) / dt; o[8] = (A * E - B * D) / dt;
}

struct Shape {
    std::vector<uint8_t> blob;   // 16-byte multiple
    int hot = 0;                 // bytes staged to shared memory
};

struct Body {
    int shape = 0;
    int movement = CPGPU_DYNAMIC;
    double mass = 0;
    D3 com, vel, angv;
    Quat q;
    double iref[9], iinv_ref[9], iw[9], iinv[9];
    D3 local_origin;             // tracked geometry origin (RigidBody.cpp:32-33)
    double rest = 0.3, kin = 0.6, sta = 1.1;
    // sleep state (RigidBody.h: asleep, sleep_ready_counter as a count of
    // sleepy steps, non_sleepy_tick_count, recievedWakingAction, history):
    // hist holds hist_n (velocity, angular velocity) records, oldest first
    int asleep = 0, waking = 0, ready_cnt = 0, non_sleepy = 0, hist_n = 0;
    std::vector<float> hist;
    // a body of several primitives (ConvexUnionGeometry): their shapes, in
    // order, and materials (restitution, kinetic, static); empty for a body of one
    std::vector<int> prims;
    std::vector<std::array<double, 3>> prim_mat;
    // pose given through the API since the last read-back from a device: its
    // orientation is renormalised on upload (a read-back pose was normalised
    // by the step that produced it, and normalising it again could change
    // its last bits, so a batch re-packed from read-back state continues
    // exactly)
    int fresh = 1;
    // RigidBody::alertWaking (RigidBody.cpp:318-324)
    void alert_waking() { waking = 1; ready_cnt = 0; non_sleepy = 0; hist_n = 0; hist.clear(); }
};

struct Params {
    double dt = 1.0 / 90;
    D3 g = D3(0, -6, 0);
    int substeps = 8, pgs_vel = 4, pgs_pos = 1, pgs_holo = 1;
    double cfm = 0.0000025;
    int contact_life = 6;
    double hardness = 1000;
    int angle_ticks = 4;
    bool gyro_disabled = false, warm_disabled = false;
    double cutoff = 0;           // 2|g|dt, set by setStep_time / setGravity
    bool sleeping = false;       // the device path starts with sleeping disabled
    // sleep parameters (PhysicsEngine.h:219-224)
    double sleep_delay = 0.5, vel_sleep_coeff = 0.1, ang_vel_eps = 0.1, accel_sleep_coeff = 0.044;
    int non_sleepy_threshold = 3;
};

struct Batch;

// A joint (PersistentConstraint.h:90-420) in the host mirror
struct HJoint {
    int b1 = 0, b2 = 0;          // body indices (0-based) in the world
    int kind = JK_BALL;          // JointKind
    int n = 3;                   // dofs of its row
    int seq = 0;                 // creation order among the world's joints and springs
    D3 p1, p2;                   // anchors: tracked points relative to the COM, body frame
    D3 ax1, ax2;                 // axes / directions, body space
    double ph = 15000, rh = 15000;
    double target = 0;           // distance: the attachment points' distance
    double min_angle = 0, max_angle = 0;   // limits
    D3 ul, wl;                   // twist: body 1's u and w axes (body space)
    float impulse[kJMax] = {};   // warm-start impulse carried between uploads
    float u[3] = {}, w[3] = {};  // hinge / slider basis of the last rebuild
    float angle = 0;             // twist: current angle (unwrapped); motor: angular position; slide limit / piston: slide position
    int active = 0;              // limits: reached at the last rebuild
    // motor (PersistentConstraint.h:253-275) / piston (:217-251): the powered
    // mode (0 off, 1 constant torque or force, 2 target velocity, 3 target
    // position) and its settings; limits in min_angle / max_angle (motor
    // angles, slide positions); a motor's body 1 reference axes in ul / wl and
    // body 2's comparison axis in ax2
    int mode = 0;
    double pmax = 0, tvel = 0, tpos = 0;
    float aux = 0;               // motor: relative angular velocity of the last rebuild; slide limit / piston: past a limit
    // listed in the next island (addSolverConstraints)
    int listed() const {
        if (kind == JK_MOTOR) return ((mode != 0 && pmax != 0) || angle < min_angle || angle > max_angle) ? 1 : 0;
        if (kind == JK_SLIDE_LIMIT) return aux != 0.f ? 1 : 0;
        if (kind == JK_PISTON) return (mode != 0 && pmax != 0) ? 1 : 0;
        return active;
    }
};

// A spring (PhysicsEngine::addSpring, PhysicsEngine.cpp:974-998)
struct HSpring {
    int b1 = 0, b2 = 0;
    int seq = 0;
    D3 p1, p2;                   // tracked points relative to the COM, body frame
    double damping = 0, stiffness = 0, rest = 0;
};

struct World {
    Params p;
    std::vector<Shape> shapes;
    std::vector<Body> bodies;
    std::vector<HJoint> joints;
    std::vector<HSpring> springs;
    int constraint_seq = 0;                        // joints and springs created so far
    std::unordered_map<unsigned int, int> nodes;   // same insert sequence as constraint_graph_nodes
    std::vector<cpgpu_contact> contacts;           // host copy of the contact graph
    std::vector<uint32_t> last_pairs;
    std::unique_ptr<Batch> dev;
    bool dev_valid = false;
    bool audit = false;                            // FP64 audit requested (cpgpu_world_set_audit)
    uint64_t version = 0;                          // API mutations so far (a batch checks it before re-packing)
};

// A world's description and host state without its device copy: the
// autotuner's private copies.  The node map is copied, not re-inserted, so
// its iteration order (island and system order) is the source's.
static void copy_world(const World& s, World& c) {
    c.p = s.p;
    c.shapes = s.shapes;
    c.bodies = s.bodies;
    c.joints = s.joints;
    c.springs = s.springs;
    c.constraint_seq = s.constraint_seq;
    c.nodes = s.nodes;
    c.contacts = s.contacts;
    c.last_pairs = s.last_pairs;
    c.audit = s.audit;
}

// ---------------------------------------------------------------- shape packing ----
static void put16(std::vector<uint8_t>& b) { while (b.size() % 16) b.push_back(0); }
template <class T>
static void put(std::vector<uint8_t>& b, const T& v) {
    size_t o = b.size();
    b.resize(o + sizeof(T));
    std::memcpy(b.data() + o, &v, sizeof(T));
}

// Packs a prepared hull (reference frame = centred on `com`) into the blob the
// kernels read.  Hot sections first (header, vertices, normals, cache, arcs).
static Shape pack_hull(const HullPrep& h, const D3& com) {
    if ((int)h.pts.size() > kMaxHullVerts || (int)h.faces.size() > kMaxHullFaces || (int)h.edges.size() > kMaxHullEdges ||
        (int)h.arcs.size() > kMaxHullEdges)
        throw ApiFail{CPGPU_ERR_UNSUPPORTED, "hull too large (limit 255 vertices / faces / edges)"};
    HullHeader H;
    std::memset(&H, 0, sizeof(H));
    H.nv = (uint16_t)h.pts.size();
    H.nf = (uint16_t)h.faces.size();
    H.ne = (uint16_t)h.edges.size();
    H.na = (uint16_t)h.arcs.size();
    std::vector<uint8_t> b(sizeof(HullHeader));
    double rad = 0;
    for (const D3& p : h.pts) {
        D3 q = p - com;
        rad = std::max(rad, q.mag());
        put(b, make_float4((float)q.x, (float)q.y, (float)q.z, 0.f));
    }
    H.off_norm = (uint16_t)b.size();
    for (size_t f = 0; f < h.faces.size(); f++)
        put(b, make_float4((float)h.gn[f].x, (float)h.gn[f].y, (float)h.gn[f].z, h.redundant[f] ? 1.f : 0.f));
    H.off_cache = (uint16_t)b.size();
    for (size_t f = 0; f < h.faces.size(); f++) {
        // recentred extrema (CollisionDetect.cpp:622-625): shift by the change of
        // the reference point's projection between construction frame and COM frame
        const D3& n = h.gn[f];
        double shift = n.dot(h.pts[h.ref_idx[f]] - com) - h.ref_val[f];
        float4 c;
        c.x = (float)(h.cmax[f] + shift);
        c.y = (float)(h.cmin[f] + shift);
        int mx = h.cmax_id[f], mn = h.cmin_id[f];
        std::memcpy(&c.z, &mx, 4);
        std::memcpy(&c.w, &mn, 4);
        put(b, c);
    }
    H.off_arc = (uint16_t)b.size();
    for (auto& a : h.arcs) { b.push_back((uint8_t)a.first); b.push_back((uint8_t)a.second); }
    put16(b);
    H.off_fofs = (uint16_t)b.size();  // end of the hot part
    {
        uint16_t o = 0;
        for (auto& f : h.faces) { put(b, o); o = (uint16_t)(o + f.size()); }
        put(b, o);
        H.nfi = o;
        put16(b);
        H.off_fidx = (uint16_t)b.size();
        for (auto& f : h.faces) for (int v : f) b.push_back((uint8_t)v);
        put16(b);
    }
    H.off_edge = (uint16_t)b.size();
    for (auto& e : h.edges) { b.push_back((uint8_t)e.first); b.push_back((uint8_t)e.second); }
    put16(b);
    auto csr = [&](const std::vector<std::vector<int>>& lists, uint16_t* off_ofs, uint16_t* off_idx) {
        *off_ofs = (uint16_t)b.size();
        uint16_t o = 0;
        for (auto& l : lists) { put(b, o); o = (uint16_t)(o + l.size()); }
        put(b, o);
        put16(b);
        *off_idx = (uint16_t)b.size();
        for (auto& l : lists) for (int x : l) b.push_back((uint8_t)x);
        put16(b);
    };
    csr(h.vfaces, &H.off_vfofs, &H.off_vfidx);
    csr(h.vedges, &H.off_veofs, &H.off_veidx);
    if (b.size() > (size_t)kMaxHullBlob) throw ApiFail{CPGPU_ERR_UNSUPPORTED, "hull blob too large"};
    H.size16 = (uint16_t)(b.size() / 16);
    H.kind = 0;
    H.radius = (float)rad;
    std::memcpy(b.data(), &H, sizeof(H));
    Shape s;
    s.blob = std::move(b);
    s.hot = H.off_fofs;
    return s;
}

// Sphere / cylinder blobs (layout.h), geometry given in the reference frame.
static Shape pack_prim(uint32_t kind, const std::vector<float4>& body, float bound) {
    HullHeader H;
    std::memset(&H, 0, sizeof(H));
    std::vector<uint8_t> b(sizeof(HullHeader));
    for (const float4& v : body) put(b, v);
    H.size16 = (uint16_t)(b.size() / 16);
    H.off_fofs = (uint16_t)b.size();   // the whole blob is staged
    H.kind = kind;
    H.radius = bound;
    std::memcpy(b.data(), &H, sizeof(H));
    Shape s;
    s.blob = std::move(b);
    s.hot = H.off_fofs;
    return s;
}

static float4 f4(const D3& v, double w) { return make_float4((float)v.x, (float)v.y, (float)v.z, (float)w); }

// Sphere at `cref` (reference frame) of radius r
static Shape pack_sphere(const D3& cref, double r) {
    return pack_prim(SHAPE_SPHERE, {f4(cref, r)}, (float)(cref.mag() + r));
}

// Cylinder (ConvexPrimitive.cpp:222-256, default height axis (0,1,0)) centred at
// `cref` in the reference frame: Gauss vertices of the two caps and the
// 12-vertex ring, and the 8-gon cap approximations of radius r / cos(pi/8).
// PI is the reference's truncated 3.1415926535 (Math/src/Quaternion.h:4).
static Shape pack_cylinder(const D3& cref, double r, double h) {
    const double pi = 3.1415926535;
    std::vector<float4> v;
    v.push_back(f4(cref, r));
    v.push_back(make_float4(0.f, 1.f, 0.f, (float)h));
    v.push_back(make_float4(0.f, 1.f, 0.f, 0.f));
    v.push_back(make_float4(0.f, -1.f, 0.f, 0.f));
    for (int i = 0; i < kCylRing; i++) {
        double th = i * (2 * pi / kCylRing);
        v.push_back(make_float4((float)std::sin(th), 0.f, (float)std::cos(th), 0.f));
    }
    double er = r / std::cos(pi / kCylCap);
    for (int side = 0; side < 2; side++)
        for (int i = 0; i < kCylCap; i++) {
            double th = i * (2 * pi / kCylCap);
            double y = side == 0 ? h / 2.0 : -h / 2.0;
            v.push_back(f4(cref + D3(er * std::sin(th), y, er * std::cos(th)), 0));
        }
    return pack_prim(SHAPE_CYLINDER, v, (float)(cref.mag() + std::sqrt(er * er + h * h / 4)));
}

// Capsule (ConvexPrimitive.cpp:357-360, height axis (0,1,0)) centred at `cref`
// in the reference frame: radius r, drum height h
static Shape pack_capsule(const D3& cref, double r, double h) {
    return pack_prim(SHAPE_CAPSULE, {f4(cref, r), make_float4(0.f, 1.f, 0.f, (float)h)}, (float)(cref.mag() + h / 2 + r));
}

// ---------------------------------------------------------------- static meshes ----
// StaticMeshGeometry (Geometry.cpp:675-820) prepared on the host: face normals,
// neighbours across shared edges, ids (faces from 0, edges after the
// vertices), outward edge directions, Gauss regions with the concave-neighbour
// count; and the AABB tree the reference's copy constructor builds
// (Geometry.cpp:660-666: AABBTree::add per face in order, surface-area cost,
// no margin, AABB_Tree.h:39-105, 373-421), whose traversal order decides the
// order of a body's triangle candidates and so its contacts.
struct MBox { D3 lo, hi; };
static MBox mbox_union(const MBox& a, const MBox& b) {
    return MBox{D3(std::min(a.lo.x, b.lo.x), std::min(a.lo.y, b.lo.y), std::min(a.lo.z, b.lo.z)),
                D3(std::max(a.hi.x, b.hi.x), std::max(a.hi.y, b.hi.y), std::max(a.hi.z, b.hi.z))};
}
// AABB::surfaceArea as written in AABB.h:112-118 (2 dx dy + dy dz + dz dx)
static double mbox_cost(const MBox& a) {
    double dx = a.hi.x - a.lo.x, dy = a.hi.y - a.lo.y, dz = a.hi.z - a.lo.z;
    return 2 * (dx * dy) + (dy * dz) + (dz * dx);
}

struct MTree {
    struct Node { int parent = -1, left = -1, right = -1, obj = -1; bool leaf = false; MBox box; double cost = 0; };
    std::vector<Node> n;
    int root = -1;
    void add(int obj, const MBox& b) {
        Node leaf;
        leaf.leaf = true; leaf.obj = obj; leaf.box = b; leaf.cost = mbox_cost(b);
        const int nl = (int)n.size();
        n.push_back(leaf);
        if (root < 0) { root = nl; return; }
        int best = -1;
        double best_cost = std::numeric_limits<double>::infinity();
        std::vector<std::pair<int, double>> cand{{root, 0.0}};
        while (!cand.empty()) {
            auto c = cand.back();
            cand.pop_back();
            if (c.second >= best_cost) continue;
            double direct = mbox_cost(mbox_union(n[nl].box, n[c.first].box));
            double cost = c.second + direct;
            if (cost < best_cost) { best = c.first; best_cost = cost; }
            if (!n[c.first].leaf) {
                double inh = c.second + direct - n[c.first].cost;
                cand.push_back({n[c.first].left, inh});
                cand.push_back({n[c.first].right, inh});
            }
        }
        const int np = (int)n.size();
        n.push_back(Node());
        if (best == root) root = np;
        else {
            int op = n[best].parent;
            if (n[op].left == best) n[op].left = np; else n[op].right = np;
            n[np].parent = op;
        }
        n[np].left = best; n[best].parent = np;
        n[np].right = nl; n[nl].parent = np;
        for (int cur = n[nl].parent; cur >= 0; cur = n[cur].parent) {
            n[cur].box = mbox_union(n[n[cur].left].box, n[n[cur].right].box);
            n[cur].cost = mbox_cost(n[cur].box);
        }
        auto swp = [&](int a, int b) {
            int pa = n[a].parent, pb = n[b].parent;
            if (n[pa].left == a) n[pa].left = b; else n[pa].right = b;
            if (n[pb].left == b) n[pb].left = a; else n[pb].right = a;
            n[a].parent = pb;
            n[b].parent = pa;
        };
        for (int cur = n[nl].parent; cur >= 0 && n[cur].parent >= 0; cur = n[cur].parent) {
            const int pp = n[cur].parent;
            const int sib = n[pp].left == cur ? n[pp].right : n[pp].left;
            MBox slb = mbox_union(n[n[cur].right].box, n[sib].box), srb = mbox_union(n[n[cur].left].box, n[sib].box), clb, crb;
            double sl = mbox_cost(slb), sr = mbox_cost(srb), cl, cr;
            if (n[sib].leaf) { cl = cr = std::numeric_limits<double>::infinity(); }
            else {
                clb = mbox_union(n[n[sib].right].box, n[cur].box);
                crb = mbox_union(n[n[sib].left].box, n[cur].box);
                cl = mbox_cost(clb);
                cr = mbox_cost(crb);
            }
            double clc = cl - n[sib].cost, crc = cr - n[sib].cost, slc = sl - n[cur].cost, src = sr - n[cur].cost;
            double mn = std::min(clc, std::min(crc, std::min(slc, src)));
            if (mn >= 0) continue;
            if (mn == clc) { swp(cur, n[sib].left); n[sib].box = clb; n[sib].cost = cl; }
            else if (mn == crc) { swp(cur, n[sib].right); n[sib].box = crb; n[sib].cost = cr; }
            else if (mn == slc) { swp(sib, n[cur].left); n[cur].box = slb; n[cur].cost = sl; }
            else { swp(sib, n[cur].right); n[cur].box = srb; n[cur].cost = sr; }
        }
    }
};

static float4 f4b(const D3& v, int bits) {
    float4 o = make_float4((float)v.x, (float)v.y, (float)v.z, 0.f);
    std::memcpy(&o.w, &bits, 4);
    return o;
}

static Shape pack_mesh(const std::vector<D3>& pts, const std::vector<std::array<int, 3>>& tris, D3* lo_out, D3* hi_out) {
    struct E { int p1, p2, opp, id = -1; uint64_t key; };
    struct TN { int p[3]; int nb[3]; E e[3]; D3 normal; };
    auto mkE = [](int a, int b, int o) {
        E e; e.p1 = a; e.p2 = b; e.opp = o;
        uint64_t mx = (uint32_t)std::max(a, b), mn = (uint32_t)std::min(a, b);
        e.key = ((mx << 32) & 0xFFFFFFFF00000000ull) + mn;
        return e;
    };
    std::vector<TN> g(tris.size());
    for (size_t i = 0; i < tris.size(); i++) {
        const auto& t = tris[i];
        TN& x = g[i];
        for (int k = 0; k < 3; k++) { x.p[k] = t[k]; x.nb[k] = -1; }
        x.e[0] = mkE(t[0], t[1], t[2]); x.e[1] = mkE(t[1], t[2], t[0]); x.e[2] = mkE(t[2], t[0], t[1]);
        x.normal = (pts[t[1]] - pts[t[0]]).cross(pts[t[2]] - pts[t[0]]).normalize();
    }
    std::unordered_map<uint64_t, unsigned> efm;
    for (size_t i = 0; i < g.size(); i++)
        for (int j = 0; j < 3; j++) {
            auto q = efm.find(g[i].e[j].key);
            if (q != efm.end()) {
                g[i].nb[j] = (int)q->second;
                for (int k = 0; k < 3; k++)
                    if (g[q->second].e[k].key == g[i].e[j].key) g[q->second].nb[k] = (int)i;
                efm.erase(q);
            } else {
                efm[g[i].e[j].key] = (unsigned)i;
            }
        }
    std::vector<float4> tri_data;
    std::vector<MBox> boxes;
    int next_edge = (int)(tris.size() + pts.size());
    for (size_t ti = 0; ti < g.size(); ti++) {
        TN& t = g[ti];
        D3 v[3] = {pts[t.p[0]], pts[t.p[1]], pts[t.p[2]]};
        D3 out[3];
        int eid[3];
        std::vector<D3> gauss;
        int concave = 0;
        for (int i = 0; i < 3; i++) {
            out[i] = (v[(i + 1) % 3] - v[i]).cross(t.normal).normalize();
            if (t.e[i].id == -1) t.e[i].id = next_edge++;
            eid[i] = t.e[i].id;
            if (t.nb[i] == -1) { gauss.push_back(out[i]); continue; }
            E comp{};
            for (int j = 0; j < 3; j++) {
                const E& ne = g[t.nb[i]].e[j];
                if (t.e[i].p1 == ne.p2 && t.e[i].p2 == ne.p1) comp = ne;
            }
            bool conc = (pts[comp.opp] - pts[t.e[i].opp]).normalize().dot(t.normal) >= -0.00001;
            if (conc) { concave++; if (concave <= 1) gauss.push_back(t.normal); }
            else gauss.push_back(g[t.nb[i]].normal);
        }
        MBox b{D3(std::min(v[0].x, std::min(v[1].x, v[2].x)), std::min(v[0].y, std::min(v[1].y, v[2].y)), std::min(v[0].z, std::min(v[1].z, v[2].z))),
               D3(std::max(v[0].x, std::max(v[1].x, v[2].x)), std::max(v[0].y, std::max(v[1].y, v[2].y)), std::max(v[0].z, std::max(v[1].z, v[2].z)))};
        boxes.push_back(b);
        tri_data.push_back(f4b(t.normal, concave));
        for (int i = 0; i < 3; i++) tri_data.push_back(f4b(v[i], 0));
        for (int i = 0; i < 3; i++) tri_data.push_back(f4b(out[i], 0));
        for (int i = 0; i < 3; i++) tri_data.push_back(f4b(i < (int)gauss.size() ? gauss[i] : D3(), i == 0 ? (int)gauss.size() : 0));
        float4 ids;
        int idv[4] = {eid[0], eid[1], eid[2], (int)ti};
        std::memcpy(&ids, idv, 16);
        tri_data.push_back(ids);
        tri_data.push_back(f4b(b.lo, 0));
        tri_data.push_back(f4b(b.hi, 0));
    }
    MTree tree;
    for (int i = 0; i < (int)boxes.size(); i++) tree.add(i, boxes[i]);
    // flatten with the root first (indices remapped)
    std::vector<int> order, remap(tree.n.size(), -1);
    std::vector<int> st{tree.root};
    while (!st.empty()) {
        int x = st.back();
        st.pop_back();
        remap[x] = (int)order.size();
        order.push_back(x);
        if (!tree.n[x].leaf) { st.push_back(tree.n[x].right); st.push_back(tree.n[x].left); }
    }
    HullHeader H;
    std::memset(&H, 0, sizeof(H));
    H.kind = SHAPE_MESH;
    H.pad[0] = (uint32_t)tris.size();
    H.pad[1] = (uint32_t)order.size();
    std::vector<uint8_t> blob(sizeof(HullHeader));
    MBox all = boxes[0];
    for (size_t i = 1; i < boxes.size(); i++) all = mbox_union(all, boxes[i]);
    put(blob, f4b(all.lo, 0));
    put(blob, f4b(all.hi, 0));
    for (int x : order) {
        const MTree::Node& nd = tree.n[x];
        // node boxes rounded outwards so FP32 traversal never drops a candidate
        // the FP64 test keeps; leaves carry the triangle's own box (in the
        // triangle record) for the final test
        auto down = [](double v) { float f = (float)v; return (double)f > v ? std::nextafter(f, -INFINITY) : f; };
        auto up = [](double v) { float f = (float)v; return (double)f < v ? std::nextafter(f, INFINITY) : f; };
        float4 lo = make_float4(down(nd.box.lo.x), down(nd.box.lo.y), down(nd.box.lo.z), 0.f);
        float4 hi = make_float4(up(nd.box.hi.x), up(nd.box.hi.y), up(nd.box.hi.z), 0.f);
        int l = nd.leaf ? -1 : remap[nd.left];
        int r = nd.leaf ? nd.obj : remap[nd.right];
        std::memcpy(&lo.w, &l, 4);
        std::memcpy(&hi.w, &r, 4);
        put(blob, lo);
        put(blob, hi);
    }
    for (const float4& f : tri_data) put(blob, f);
    std::memcpy(blob.data(), &H, sizeof(H));
    *lo_out = all.lo;
    *hi_out = all.hi;
    Shape sh;
    sh.blob = std::move(blob);
    sh.hot = 0;   // read from global memory, never staged
    return sh;
}

// ---------------------------------------------------------------- device batch ----
struct Arena {
    uint8_t* base = nullptr;
    size_t size = 0, used = 0;
    template <class T>
    T* take(size_t n) {
        used = (used + 255) & ~size_t(255);
        T* p = reinterpret_cast<T*>(base + used);
        used += sizeof(T) * std::max<size_t>(n, 1);
        return p;
    }
};

struct Batch {
    int n_worlds = 0, n_bodies = 0;
    int substeps = 1;
    int n_sms = 0;
    int slot_bytes = 0;
    bool prims = false;                // the batch holds spheres or cylinders
    bool meshes = false;               // the batch holds static triangle meshes
    bool unions = false;               // the batch holds bodies of several primitives
    bool joints = false;               // the batch holds joints (or springs: joint edges)
    bool springs = false;              // the batch holds springs
    bool tiles = false;                // the batch holds worlds above kTileWorld bodies (tiled pair pass)
    bool systems = false;              // ... and holonomic systems
    cudaStream_t st = nullptr;
    cudaStream_t side = nullptr;       // concurrent branch (small-island PGS)
    cudaEvent_t fork = nullptr, join = nullptr;
    int dv_cap = 64;                   // island bodies whose Δv fits in shared memory
    int pgs_blocks = 0;                // k_pgs_big grid: one resident chain per block
    int isl_smem = 0;                  // k_islands dynamic shared memory
    uint8_t* mem = nullptr;
    size_t bytes = 0;                  // device arena size
    Dev d[2];                  // d[p]: old = buffer p, new = buffer 1-p
    int parity = 0;
    // per parity, the step as two graphs: up to the PGS schedule, and the rest
    cudaGraphExec_t graph_pre[2] = {nullptr, nullptr}, graph_rest[2] = {nullptr, nullptr};
    cudaEvent_t pre_done = nullptr;    // recorded after each step's first graph
    std::vector<int> world_start;
    std::vector<int> world_jstart;     // joint ranges of the worlds
    std::vector<uint8_t> movement;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double* audit = nullptr;           // FP64 audit values (kAuditValues per world), null when disabled

    void drop_graphs() {
        for (auto* gs : {graph_pre, graph_rest})
            for (int p = 0; p < 2; p++) if (gs[p]) { cudaGraphExecDestroy(gs[p]); gs[p] = nullptr; }
    }
    ~Batch() {
        drop_graphs();
        if (pre_done) cudaEventDestroy(pre_done);
        if (audit) cudaFree(audit);
        if (snap) cudaFree(snap);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (mem) cudaFree(mem);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (side) cudaStreamDestroy(side);
        if (st) cudaStreamDestroy(st);
    }

    const Dev& cur() const { return d[parity]; }      // old buffers hold the current graph

    // stage markers: when `marks` is set an event is recorded after each stage
    std::vector<cudaEvent_t>* marks = nullptr;
    void mark(int stage) {
        if (marks) CK(cudaEventRecord((*marks)[stage], st));
    }
    // a step in two halves: gravity to the PGS schedule (the work every
    // island's solver chain waits for), then the substeps and geometry
    void launch_pre(const Dev& x) {
        Launch L{n_sms, st};
        mark(0);
        launch_step_begin(x, L);   mark(1);
        launch_pairs(x, L);        mark(2);
        launch_narrowphase(x, slot_bytes, n_sms, prims, st); mark(3);   // + mesh pairs
        launch_merge(x, L);        mark(4);
        launch_islands(x, isl_smem, L);
        launch_pgs_schedule(x, L); mark(5);
    }
    void launch_step(const Dev& x) {
        launch_pre(x);
        launch_rest(x);
    }
    void launch_rest(const Dev& x) {
        Launch L{n_sms, st};
        for (int s = 0; s < substeps; s++) {
            launch_springs(x, L);                          // impulses before the rows read the velocities
            launch_rows(x, s == 0, s == substeps - 1, L);
            launch_joint_rows(x, s == 0, L);               mark(6 + 3 * s);
            launch_pgs(x, dv_cap, pgs_blocks, side, fork, join, L);
            launch_pgs_joint(x, s == 0, L);                mark(7 + 3 * s);
            launch_integrate(x, s == substeps - 1, L);     mark(8 + 3 * s);
        }
        launch_geometry(x, 0, L);  mark(6 + 3 * substeps);
        launch_audit(x, L);
    }
    // kernels per step: gravity 1, pairs 2 + scan 3 + clamp 1, narrowphase 2
    // (+1 with spheres / cylinders, +1 with meshes), merge 6 + 3 scans, islands 2 + scan 3,
    // schedule 3, 5 per substep (rows, small + grouped + large PGS, integrate), geometry 1
    // (+2 per substep and 1 factorisation with joints)
    int launches_per_step() const {
        return 1 + 6 + 2 + (prims ? 1 : 0) + ((meshes || unions) ? 1 : 0) + (6 + 9) + (2 + 3) + 3 + 5 * substeps + 1 + (joints ? 2 * substeps : 0) +
               (systems ? 1 : 0) + (audit ? 1 : 0) + (springs ? substeps : 0) + (tiles ? 3 : 0);
    }

    // solver schedule: chain workers per SM of k_pgs_big (0 = as many as fit)
    // and the big-island row threshold; the step graphs are rebuilt
    int pgs_per_sm = 0;
    void set_schedule(int per_sm, int big_rows) {
        CK(cudaStreamSynchronize(st));
        pgs_per_sm = per_sm;
        const int fit = pgs_big_blocks_per_sm(dv_cap);
        pgs_blocks = n_sms * (per_sm > 0 ? std::min(per_sm, fit) : fit);
        d[0].big_rows = d[1].big_rows = big_rows;
        drop_graphs();
        build_graphs();
    }
    // whole device state (one arena) copied aside and back, so that trial
    // steps leave no trace (the autotuner's timing runs)
    uint8_t* snap = nullptr;
    int snap_parity = 0;
    void snapshot() {
        if (!snap) CK(cudaMalloc(&snap, bytes));
        CK(cudaMemcpyAsync(snap, mem, bytes, cudaMemcpyDeviceToDevice, st));
        CK(cudaStreamSynchronize(st));
        snap_parity = parity;
    }
    void restore(bool release) {
        CK(cudaMemcpyAsync(mem, snap, bytes, cudaMemcpyDeviceToDevice, st));
        CK(cudaStreamSynchronize(st));
        parity = snap_parity;
        if (release) { CK(cudaFree(snap)); snap = nullptr; }
    }

    // FP64 audit on or off: the values restart (zeroed) when it is enabled,
    // and the step graphs are rebuilt with or without the audit kernel
    void set_audit(bool on) {
        if (on == (audit != nullptr)) return;
        CK(cudaStreamSynchronize(st));
        if (on) {
            CK(cudaMalloc(&audit, sizeof(double) * kAuditValues * std::max(n_worlds, 1)));
            CK(cudaMemset(audit, 0, sizeof(double) * kAuditValues * std::max(n_worlds, 1)));
        } else {
            CK(cudaFree(audit));
            audit = nullptr;
        }
        d[0].audit = d[1].audit = audit;
        drop_graphs();
        build_graphs();
    }
    void read_audit(double* out) {
        if (!audit) throw ApiFail{CPGPU_ERR_INVALID_ARG, "the audit is not enabled"};
        CK(cudaMemcpyAsync(out, audit, sizeof(double) * kAuditValues * n_worlds, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }

    void build_graphs() {
        if (!pre_done) CK(cudaEventCreateWithFlags(&pre_done, cudaEventDisableTiming));
        for (int p = 0; p < 2; p++)
            for (int half = 0; half < 2; half++) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                if (half == 0) launch_pre(d[p]);
                else launch_rest(d[p]);
                CK(cudaStreamEndCapture(st, &g));
                CK(cudaGraphInstantiate(half == 0 ? &graph_pre[p] : &graph_rest[p], g, 0));
                cudaGraphDestroy(g);
            }
    }

    // one step from the graphs; `after` (may be null): the step's first half
    // waits for that event (another part's first half of the same step)
    void step_one(cudaEvent_t after) {
        if (after) CK(cudaStreamWaitEvent(st, after, 0));
        CK(cudaGraphLaunch(graph_pre[parity], st));
        CK(cudaEventRecord(pre_done, st));
        CK(cudaGraphLaunch(graph_rest[parity], st));
        parity ^= 1;
    }
    void step(int n) {
        for (int i = 0; i < n; i++) step_one(nullptr);
    }

    int check_status() {
        int s = 0;
        CK(cudaMemcpyAsync(&s, d[0].status, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (s == 0) return CPGPU_OK;
        std::string m = "device status";
        if (s & ST_PAIR_OVERFLOW) m += " pair-capacity-overflow";
        if (s & ST_EDGE_OVERFLOW) m += " edge-capacity-overflow";
        if (s & ST_CONTACT_OVERFLOW) m += " contact-capacity-overflow";
        if (s & ST_CLIP_OVERFLOW) m += " clip-overflow";
        if (s & ST_STACK_OVERFLOW) m += " island-stack-overflow";
        if (s & ST_MESH_OVERFLOW) m += " mesh-pair-overflow";
        if (s & ST_NAN) m += " non-finite-state";
        if (s & ST_TIMEOUT) m += " bounded-wait-timeout";
        int code = (s & ST_NAN) ? CPGPU_ERR_NAN : (s & ST_TIMEOUT) ? CPGPU_ERR_TIMEOUT : CPGPU_ERR_CAPACITY;
        throw ApiFail{code, m};
    }
};

static int env_int(const char* name, int dflt) {
    const char* v = std::getenv(name);
    return v ? std::atoi(v) : dflt;
}

static std::vector<int> map_iteration_order(const World& w) {
    // constraint_graph_nodes iteration order (PhysicsEngine.h:230); ids are 1-based
    std::vector<int> order;
    order.reserve(w.nodes.size());
    for (const auto& kv : w.nodes) order.push_back(kv.second);
    return order;
}

// ---------------------------------------------------------------- holonomic systems ----
// A world's joint edges (one per body pair joined by joints or springs, the
// joints in insertion order) and its holonomic systems, found as
// PhysicsEngine::maintainHolonomicSystems (PhysicsEngine.cpp:1292-1306,
// 1466-1532, 1745-1777) finds them on the first step: nodes in node-map order,
// each node's edges by the other body's id, a scan from every edge holding a
// holonomic joint and not yet in a system, collecting the edges with
// holonomic joints connected to it through dynamic bodies.  Cone and twist
// limits are not holonomic (PersistentConstraint.h:168, 208) and springs are
// no constraint rows: their edges connect islands but join no system.
struct HSystem {
    std::vector<int> cons;       // joint indices (world-local) in elimination order
    std::vector<int> vpos, table;
    int degree = 0, cap = 0;
    bool fp64 = false;
};

struct JointGraph {
    std::vector<std::pair<int, int>> edge_pair;       // (lower body, higher body)
    std::vector<std::vector<int>> edge_joints;        // world-local joint indices, creation order
    std::vector<int> edge_first;                      // body the edge was created from (its first constraint's b1)
    std::vector<int> edge_sys;
    std::vector<HSystem> systems;
};

static bool holonomic_kind(int k) { return !jk_conditional(k); }

// HolonomicSystem::HolonomicSystem (HolonomicBlockSolver.cpp:11-132): greedy
// minimum-fill elimination order over constraints that share a body, and the
// lower-triangle block table of the factor
static HSystem order_system(const World& w, const std::vector<int>& og) {
    HSystem H;
    const int n = (int)og.size();
    std::vector<char> edge((size_t)n * n, 0), empty((size_t)n * n, 1);
    auto E = [&](int i, int j) -> char& { return edge[(size_t)i + (size_t)j * n]; };
    auto shares = [&](int x, int y) {
        const HJoint &a = w.joints[og[x]], &b = w.joints[og[y]];
        return a.b1 == b.b1 || a.b1 == b.b2 || a.b2 == b.b1 || a.b2 == b.b2;
    };
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            if (shares(i, j)) { empty[(size_t)i * n + j] = empty[(size_t)j * n + i] = 0; E(i, j) = E(j, i) = 1; }
    std::vector<int> remaining(n), order;
    for (int i = 0; i < n; i++) remaining[i] = i;
    while (!remaining.empty()) {
        int best_i = -1, best = INT32_MAX;
        std::vector<int> best_nb;
        for (int i = 0; i < (int)remaining.size(); i++) {
            std::vector<int> nb;
            for (int j = 0; j < n; j++)
                if (j != remaining[i] && E(remaining[i], j)) nb.push_back(j);
            int un = 0;
            for (size_t a = 0; a < nb.size(); a++)
                for (size_t b = a + 1; b < nb.size(); b++) un += !E(nb[a], nb[b]);
            if (un < best) { best = un; best_i = i; best_nb = nb; if (un == 0) break; }
        }
        const int x = remaining[best_i];
        order.push_back(x);
        remaining.erase(remaining.begin() + best_i);
        for (int j = 0; j < n; j++) E(x, j) = E(j, x) = 0;
        for (size_t a = 0; a < best_nb.size(); a++)
            for (size_t b = a + 1; b < best_nb.size(); b++) {
                const int p = best_nb[a], q = best_nb[b];
                empty[(size_t)p * n + q] = empty[(size_t)q * n + p] = 0;
                E(p, q) = E(q, p) = 1;
            }
    }
    for (int xi : order) H.cons.push_back(og[xi]);
    for (int col = 0; col < n; col++) {
        H.vpos.push_back(H.degree);
        H.degree += w.joints[H.cons[col]].n;
        for (int row = col; row < n; row++) {
            if (empty[(size_t)order[row] * n + order[col]]) H.table.push_back(-1);
            else { H.table.push_back(H.cap); H.cap += w.joints[H.cons[row]].n * w.joints[H.cons[col]].n; }
        }
    }
    double mmin = 1e300, mmax = 0;
    for (int j : H.cons)
        for (int b : {w.joints[j].b1, w.joints[j].b2})
            if (w.bodies[b].movement == CPGPU_DYNAMIC) { mmin = std::min(mmin, w.bodies[b].mass); mmax = std::max(mmax, w.bodies[b].mass); }
    H.fp64 = mmax > 100.0 * mmin;   // FP64 factorisation for mass ratios above 100
    return H;
}

static JointGraph joint_graph(const World& w, const std::vector<int>& map_order) {
    JointGraph G;
    std::map<std::pair<int, int>, int> idx;
    // joints and springs in creation order: an edge is created by the first
    // constraint between its bodies
    std::vector<std::pair<int, int>> items;   // (seq, joint index or -(spring index + 1))
    for (int j = 0; j < (int)w.joints.size(); j++) items.push_back({w.joints[j].seq, j});
    for (int k = 0; k < (int)w.springs.size(); k++) items.push_back({w.springs[k].seq, -(k + 1)});
    std::sort(items.begin(), items.end());
    for (const auto& it0 : items) {
        const int b1 = it0.second >= 0 ? w.joints[it0.second].b1 : w.springs[-it0.second - 1].b1;
        const int b2 = it0.second >= 0 ? w.joints[it0.second].b2 : w.springs[-it0.second - 1].b2;
        std::pair<int, int> k(std::min(b1, b2), std::max(b1, b2));
        auto it = idx.find(k);
        if (it == idx.end()) {
            it = idx.emplace(k, (int)G.edge_pair.size()).first;
            G.edge_pair.push_back(k);
            G.edge_joints.emplace_back();
            G.edge_first.push_back(b1);
        }
        if (it0.second >= 0) G.edge_joints[it->second].push_back(it0.second);
    }
    const int ne = (int)G.edge_pair.size();
    G.edge_sys.assign(ne, -1);
    if (ne == 0 || w.p.pgs_holo <= 0) return G;
    std::vector<char> holo(ne, 0);
    for (int e = 0; e < ne; e++)
        for (int j : G.edge_joints[e]) holo[e] |= holonomic_kind(w.joints[j].kind);
    const int nb = (int)w.bodies.size();
    std::vector<std::vector<int>> adj(nb);
    for (int e = 0; e < ne; e++) { adj[G.edge_pair[e].first].push_back(e); adj[G.edge_pair[e].second].push_back(e); }
    for (int b = 0; b < nb; b++)
        std::sort(adj[b].begin(), adj[b].end(), [&](int x, int y) {
            auto other = [&](int e) { return G.edge_pair[e].first == b ? G.edge_pair[e].second : G.edge_pair[e].first; };
            return other(x) < other(y);
        });
    std::vector<char> scanned(ne, 0);
    for (int node : map_order)
        for (int e0 : adj[node]) {
            if (scanned[e0] || !holo[e0]) continue;
            scanned[e0] = 1;
            // getAllEdgesConnectedHolonomically: DFS with a LIFO stack
            std::vector<char> vis(ne, 0);
            std::vector<int> stack{e0}, conn;
            while (!stack.empty()) {
                int v = stack.back();
                stack.pop_back();
                if (vis[v]) continue;
                vis[v] = 1;
                conn.push_back(v);
                // the first body's edges, then the second's (n1 is the body
                // the edge was created from)
                std::vector<int> nbr;
                const int first = G.edge_first[v];
                const int second = first == G.edge_pair[v].first ? G.edge_pair[v].second : G.edge_pair[v].first;
                for (int end : {first, second})
                    if (w.bodies[end].movement == CPGPU_DYNAMIC) nbr.insert(nbr.end(), adj[end].begin(), adj[end].end());
                for (int x : nbr) if (!vis[x] && holo[x]) stack.push_back(x);
            }
            for (int x : conn) scanned[x] = 1;
            if (conn.size() <= 1) continue;
            std::vector<int> og;
            for (int x : conn)
                for (int j : G.edge_joints[x])
                    if (holonomic_kind(w.joints[j].kind)) og.push_back(j);
            const int sid = (int)G.systems.size();
            for (int x : conn) G.edge_sys[x] = sid;
            G.systems.push_back(order_system(w, og));
        }
    return G;
}

static bool is_mesh(const World& w, uint32_t id) {
    const Shape& sh = w.shapes[w.bodies[id - 1].shape];
    return reinterpret_cast<const HullHeader*>(sh.blob.data())->kind == SHAPE_MESH;
}

// The cID of a contact's MagicID (CollisionDetect.cpp: the primitives' ids,
// first body low): a primitive's id is its body's id for a body of one, and
// (body id << 8 | index) for the primitives of a body of several (the ids are
// process-global counters in the reference; only their equality matters);
// for a mesh pair the mesh's half is the triangle id.  The device keeps the
// part of a contact's cID that the pair does not fix in the contact's
// triangle field: the triangle id (| the convex body's primitive << 24), or
// (primitive of body 1 << 8 | of body 2) for a pair with a body of several.
static bool is_union_body(const World& w, uint32_t id) { return w.bodies[id - 1].prims.size() > 1; }
static uint32_t prim_id(const World& w, uint32_t id, int k) { return is_union_body(w, id) ? ((id << 8) | (uint32_t)k) : id; }
static uint64_t contact_cid(const World& w, uint32_t b1, uint32_t b2, int tri) {
    if (is_mesh(w, b1)) return (uint32_t)(tri & 0xffffff) | ((uint64_t)prim_id(w, b2, (tri >> 24) & 0xff) << 32);
    if (is_mesh(w, b2)) return prim_id(w, b1, (tri >> 24) & 0xff) | ((uint64_t)(uint32_t)(tri & 0xffffff) << 32);
    return ((uint64_t)prim_id(w, b2, tri & 0xff) << 32) | prim_id(w, b1, (tri >> 8) & 0xff);
}
static int contact_tri(const World& w, uint32_t b1, uint32_t b2, uint64_t cid) {
    if (is_mesh(w, b1)) return (int)(uint32_t)(cid & 0xffffff) | (is_union_body(w, b2) ? (int)(((cid >> 32) & 0xff) << 24) : 0);
    if (is_mesh(w, b2)) return (int)(uint32_t)((cid >> 32) & 0xffffff) | (is_union_body(w, b1) ? (int)((cid & 0xff) << 24) : 0);
    const int i = is_union_body(w, b1) ? (int)(cid & 0xff) : 0;
    const int j = is_union_body(w, b2) ? (int)((cid >> 32) & 0xff) : 0;
    return (i << 8) | j;
}

// `rank` >= 0: the batch is part `rank` of a batch cut into parts, and its
// streams take the device's greatest priority lowered by `rank` (a graph
// launched into a stream runs at that stream's priority), so the block
// scheduler serves the part holding the largest worlds first and their
// serial solver chains start as early as the step allows.  Priorities order
// the work, never its results.
static std::unique_ptr<Batch> build_batch(const std::vector<World*>& worlds, int pgs_per_sm = 0, int rank = -1) {
    auto B = std::make_unique<Batch>();
    B->n_worlds = (int)worlds.size();
    B->substeps = worlds.empty() ? 1 : worlds[0]->p.substeps;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&B->n_sms, cudaDevAttrMultiProcessorCount, dev));
    int prio_least = 0, prio_greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    const int prio = rank < 0 ? prio_least : std::min(prio_least, prio_greatest + rank);
    CK(cudaStreamCreateWithPriority(&B->st, cudaStreamNonBlocking, prio));
    CK(cudaStreamCreateWithPriority(&B->side, cudaStreamNonBlocking, prio));
    CK(cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&B->join, cudaEventDisableTiming));
    CK(cudaEventCreate(&B->ev0));
    CK(cudaEventCreate(&B->ev1));

    // ---- host packing
    std::vector<int> wstart{0};
    int N = 0, n_contacts = 0;
    for (World* w : worlds) {
        if (w->p.substeps != B->substeps) throw ApiFail{CPGPU_ERR_INVALID_ARG, "worlds of a batch must use the same substep count"};
        N += (int)w->bodies.size();
        wstart.push_back(N);
        n_contacts += (int)w->contacts.size();
    }
    B->n_bodies = N;
    B->world_start = wstart;
    // large worlds' pair pass: tasks over (i tile, j tile >= i tile) blocks
    std::vector<int4> tile_task;
    std::vector<int> tile_base(worlds.size(), -1);
    size_t tile_cells = 0;
    for (size_t k = 0; k < worlds.size(); k++) {
        const int n = wstart[k + 1] - wstart[k];
        if (n <= kTileWorld) continue;
        const int T = (n + kTile - 1) / kTile;
        tile_base[k] = (int)tile_cells;
        tile_cells += (size_t)n * T;
        for (int it = 0; it < T; it++)
            for (int jt = it; jt < T; jt++) tile_task.push_back(make_int4((int)k, it, jt, T));
    }
    B->tiles = !tile_task.empty();
    {
        int max_world = 0;
        for (size_t k = 0; k + 1 < wstart.size(); k++) max_world = std::max(max_world, wstart[k + 1] - wstart[k]);
        // islands of more bodies keep their Δv in global memory (the same
        // arithmetic); CPGPU_PGS_DV_CAP lowers the cap, so that a batch of a
        // few very large worlds does not hold every chain worker's shared area
        // at the largest world's size
        const int dv_max = std::max(32, std::min(kPgsDvCapMax, env_int("CPGPU_PGS_DV_CAP", kPgsDvCapMax)));
        B->dv_cap = std::min(dv_max, std::max(64, max_world));
        B->isl_smem = islands_smem_bytes(max_world);
    }
    std::vector<uint8_t> pool;
    std::map<std::string, int> dedupe;
    std::vector<int> shape_off(N);
    std::vector<float4> pos(N), rot(N), vel(N), angv(N), zero4(N, make_float4(0.f, 0.f, 0.f, 0.f)), mat(N);
    // sleep state: kept on the device when a world has sleeping enabled or a
    // body is asleep; the velocity records as a ring of hist_cap entries
    bool has_sleep = false;
    int hist_cap = 1;
    for (const World* w : worlds) {
        bool any_asleep = false;
        for (const Body& b : w->bodies) any_asleep |= b.asleep != 0;
        has_sleep |= w->p.sleeping || any_asleep;
        hist_cap = std::max(hist_cap, (int)(w->p.sleep_delay / w->p.dt));
    }
    std::vector<int> s_asleep, s_waking, s_ready, s_nons, s_hn;
    std::vector<float> s_hist;
    if (has_sleep) {
        s_asleep.assign(N, 0); s_waking.assign(N, 0); s_ready.assign(N, 0); s_nons.assign(N, 0); s_hn.assign(N, 0);
        s_hist.assign((size_t)N * hist_cap * 6, 0.f);
    }
    std::vector<float> iref(9 * (size_t)N), iinv_ref(9 * (size_t)N), iw(9 * (size_t)N), iinv(9 * (size_t)N);
    std::vector<int> world_of(N), map_order(N);
    std::vector<uint8_t> movement(N);
    std::vector<int> fresh(N, 1);
    std::vector<int> prim_start(N, -1), prim_count(N, 1), prim_shape;
    std::vector<float4> prim_mat;
    std::vector<WorldParams> wp(worlds.size());
    int max_hot = 16;
    for (size_t wi = 0; wi < worlds.size(); wi++) {
        World& w = *worlds[wi];
        std::vector<int> shape_pool_off(w.shapes.size());
        for (size_t s = 0; s < w.shapes.size(); s++) {
            const Shape& sh = w.shapes[s];
            std::string key(reinterpret_cast<const char*>(sh.blob.data()), sh.blob.size());
            auto it = dedupe.find(key);
            if (it == dedupe.end()) {
                int off = (int)pool.size();
                pool.insert(pool.end(), sh.blob.begin(), sh.blob.end());
                dedupe.emplace(std::move(key), off);
                shape_pool_off[s] = off;
            } else {
                shape_pool_off[s] = it->second;
            }
            max_hot = std::max(max_hot, (sh.hot + 15) & ~15);
            const uint32_t kind = reinterpret_cast<const HullHeader*>(sh.blob.data())->kind;
            if (kind == SHAPE_SPHERE || kind == SHAPE_CYLINDER || kind == SHAPE_CAPSULE) B->prims = true;
            if (kind == SHAPE_MESH) B->meshes = true;
        }
        const int base = wstart[wi];
        for (size_t i = 0; i < w.bodies.size(); i++) {
            const Body& b = w.bodies[i];
            int g = base + (int)i;
            shape_off[g] = shape_pool_off[b.shape];
            if (b.prims.size() > 1) {
                B->unions = true;
                prim_start[g] = (int)prim_shape.size();
                prim_count[g] = (int)b.prims.size();
                for (size_t k = 0; k < b.prims.size(); k++) {
                    prim_shape.push_back(shape_pool_off[b.prims[k]]);
                    prim_mat.push_back(make_float4((float)b.prim_mat[k][0], (float)b.prim_mat[k][1], (float)b.prim_mat[k][2], 0.f));
                }
            }
            bool dyn = b.movement == CPGPU_DYNAMIC;
            pos[g] = make_float4((float)b.com.x, (float)b.com.y, (float)b.com.z, dyn ? (float)(1.0 / b.mass) : 0.f);
            rot[g] = make_float4((float)b.q.r, (float)b.q.i, (float)b.q.j, (float)b.q.k);
            vel[g] = b.movement == CPGPU_FIXED ? zero4[0] : make_float4((float)b.vel.x, (float)b.vel.y, (float)b.vel.z, 0.f);
            angv[g] = b.movement == CPGPU_FIXED ? zero4[0] : make_float4((float)b.angv.x, (float)b.angv.y, (float)b.angv.z, 0.f);
            mat[g] = make_float4((float)b.rest, (float)b.kin, (float)b.sta, 0.f);
            for (int k = 0; k < 9; k++) {
                iref[9 * (size_t)g + k] = (float)b.iref[k];
                iinv_ref[9 * (size_t)g + k] = (float)b.iinv_ref[k];
                iw[9 * (size_t)g + k] = (float)b.iw[k];
                iinv[9 * (size_t)g + k] = dyn ? (float)b.iinv[k] : 0.f;
            }
            world_of[g] = (int)wi;
            movement[g] = (uint8_t)b.movement;
            fresh[g] = b.fresh;
            if (has_sleep) {
                s_asleep[g] = b.asleep; s_waking[g] = b.waking; s_ready[g] = b.ready_cnt; s_nons[g] = b.non_sleepy;
                // the newest records that fit this world's history length, oldest first
                const int len = std::max(1, (int)(w.p.sleep_delay / w.p.dt));
                const int keep = std::min(b.hist_n, len), skip = b.hist_n - keep;
                s_hn[g] = keep;
                for (int q = 0; q < keep; q++)
                    for (int k = 0; k < 6; k++) s_hist[((size_t)g * hist_cap + q) * 6 + k] = b.hist[6 * (skip + q) + k];
            }
        }
        std::vector<int> order = map_iteration_order(w);
        for (size_t k = 0; k < order.size(); k++) map_order[base + k] = base + order[k];
        WorldParams& P = wp[wi];
        std::memset(&P, 0, sizeof(P));
        P.dt = (float)w.p.dt;
        P.dt_sub = (float)(w.p.dt / w.p.substeps);
        P.gx = (float)w.p.g.x; P.gy = (float)w.p.g.y; P.gz = (float)w.p.g.z;
        P.cfm = (float)w.p.cfm;
        P.cutoff_vel = (float)w.p.cutoff;
        P.hardness = (float)w.p.hardness;
        P.contact_life = w.p.contact_life;
        P.angle_ticks = w.p.angle_ticks;
        P.gyro_disabled = w.p.gyro_disabled;
        P.warm_disabled = w.p.warm_disabled;
        P.pgs_vel = w.p.pgs_vel;
        P.pgs_pos = w.p.pgs_pos;
        P.pgs_holo = w.p.pgs_holo;
        {
            // the reference's thresholds (PhysicsEngine.cpp:1221-1258) and its
            // FP64 step arithmetic turned into step counts
            const double gm = w.p.g.mag(), span = w.p.sleep_delay / w.p.dt;
            P.sleeping = w.p.sleeping ? 1 : 0;
            P.hist_len = std::max(1, (int)span);
            int hm = 1;
            while (2.0 * hm < span) hm++;
            P.hist_min = hm;
            double acc = 0.0;
            int rs = 0;
            while (!(acc >= w.p.sleep_delay) && rs < (1 << 28)) { acc += w.p.dt; rs++; }
            P.ready_steps = rs;
            P.non_sleepy_threshold = w.p.non_sleepy_threshold;
            P.vel_eps = (float)(w.p.vel_sleep_coeff * gm);
            P.ang_vel_eps = (float)w.p.ang_vel_eps;
            P.accel_eps = (float)(w.p.accel_sleep_coeff * gm);
            P.ang_accel_eps = (float)(w.p.accel_sleep_coeff * 2.5);
            P.wake_vel = (float)(0.25 * w.p.vel_sleep_coeff * gm);
        }
    }
    B->movement = movement;
    B->slot_bytes = 2 * max_hot;
    if (pool.empty()) pool.resize(16);

    // ---- contacts of the worlds (sorted by (b1, b2) within each world)
    std::vector<uint64_t> ekey;
    std::vector<int> ecstart, eccount;
    std::vector<uint64_t> cmag;
    std::vector<float4> cp1, cp2, cn, cimp, cfu, cfw;
    std::vector<int> cstate, cedge, ctri;
    for (size_t wi = 0; wi < worlds.size(); wi++) {
        const int base = wstart[wi];
        for (const cpgpu_contact& c : worlds[wi]->contacts) {
            ctri.push_back(contact_tri(*worlds[wi], c.b1, c.b2, c.magic_c));
            uint64_t key = ((uint64_t)(base + c.b1 - 1) << 32) | (uint32_t)(base + c.b2 - 1);
            if (ekey.empty() || ekey.back() != key) {
                ekey.push_back(key);
                ecstart.push_back((int)cmag.size());
                eccount.push_back(0);
            }
            eccount.back()++;
            cmag.push_back(c.magic_b);
            cp1.push_back(make_float4((float)c.p_local_b1[0], (float)c.p_local_b1[1], (float)c.p_local_b1[2], (float)c.pen_depth));
            cp2.push_back(make_float4((float)c.p_local_b2[0], (float)c.p_local_b2[1], (float)c.p_local_b2[2], (float)c.bounce));
            cn.push_back(make_float4((float)c.n_local_b1[0], (float)c.n_local_b1[1], (float)c.n_local_b1[2], (float)c.friction_coeff));
            cimp.push_back(make_float4((float)c.normal_impulse, (float)c.friction_impulse[0], (float)c.friction_impulse[1], 0.f));
            cfu.push_back(make_float4((float)c.friction_u[0], (float)c.friction_u[1], (float)c.friction_u[2], 0.f));
            cfw.push_back(make_float4((float)c.friction_w[0], (float)c.friction_w[1], (float)c.friction_w[2], 0.f));
            cstate.push_back(cs_make(c.memory_life, c.live != 0, c.static_ready != 0, false));
            cedge.push_back((int)ekey.size() - 1);
        }
    }

    // ---- joints, joint edges, springs and holonomic systems of the worlds
    std::vector<int> j_b1, j_b2, j_n, j_kind, j_active;
    std::vector<float4> j_p1, j_p2, j_ax1, j_ax2, j_u, j_w, j_par, j_ul, j_wl;
    std::vector<float2> j_hard;
    std::vector<float> j_imp, j_angle, j_aux;
    std::vector<float4> j_power;
    std::vector<uint64_t> je_key;
    std::vector<int> je_jstart, je_jcount, je_jlist, je_sys, je_wstart{0}, je_wjstart{0}, hs_wstart{0};
    std::vector<int> hs_cstart{0}, hs_cons, hs_vpos, hs_degree, hs_tstart{0}, hs_table, hs_bstart, hs_cap, hs_fp64, hs_wk;
    std::vector<int> hs_lbase, hs_lstart, hs_lrow, hs_lloc;   // per-column lists of the nonzero blocks below the diagonal
    std::vector<int> sp_b1, sp_b2, sp_wstart{0};
    std::vector<float4> sp_p1, sp_p2, sp_par;
    size_t pool32_n = 0, pool64_n = 0, work_n = 0;
    auto f4d = [](const D3& v) { return make_float4((float)v.x, (float)v.y, (float)v.z, 0.f); };
    for (size_t wi = 0; wi < worlds.size(); wi++) {
        const World& w = *worlds[wi];
        const int base = wstart[wi], jbase = (int)j_b1.size();
        for (const HJoint& j : w.joints) {
            j_b1.push_back(base + j.b1); j_b2.push_back(base + j.b2); j_n.push_back(j.n); j_kind.push_back(j.kind);
            j_p1.push_back(f4d(j.p1)); j_p2.push_back(f4d(j.p2));
            j_ax1.push_back(f4d(j.ax1)); j_ax2.push_back(f4d(j.ax2));
            j_u.push_back(make_float4(j.u[0], j.u[1], j.u[2], 0.f));
            j_w.push_back(make_float4(j.w[0], j.w[1], j.w[2], 0.f));
            j_hard.push_back(make_float2((float)j.ph, (float)j.rh));
            const double par_x = j.kind == JK_DISTANCE ? j.target : j.max_angle;
            j_par.push_back(make_float4((float)par_x, (float)j.min_angle, 0.f, 0.f));
            j_ul.push_back(f4d(j.ul)); j_wl.push_back(f4d(j.wl));
            j_angle.push_back(j.angle);
            j_active.push_back(j.listed());
            j_aux.push_back(j.aux);
            j_power.push_back(make_float4((float)j.mode, (float)j.pmax, (float)j.tvel, (float)j.tpos));
            for (int k = 0; k < kJMax; k++) j_imp.push_back(j.impulse[k]);
        }
        if (!w.joints.empty() || !w.springs.empty()) {
            std::vector<int> order = map_iteration_order(w);
            JointGraph G = joint_graph(w, order);
            std::vector<int> eorder(G.edge_pair.size());
            for (size_t e = 0; e < eorder.size(); e++) eorder[e] = (int)e;
            std::sort(eorder.begin(), eorder.end(), [&](int x, int y) { return G.edge_pair[x] < G.edge_pair[y]; });
            const int sbase = (int)hs_degree.size();
            for (int e : eorder) {
                je_key.push_back(((uint64_t)(base + G.edge_pair[e].first) << 32) | (uint32_t)(base + G.edge_pair[e].second));
                // the edge's joints (creation order) through an index list; a
                // spring-only edge has none: it connects islands without rows
                // and does not stop the pair from colliding
                je_jstart.push_back((int)je_jlist.size());
                je_jcount.push_back((int)G.edge_joints[e].size());
                for (int j : G.edge_joints[e]) je_jlist.push_back(jbase + j);
                je_sys.push_back(G.edge_sys[e] >= 0 ? sbase + G.edge_sys[e] : -1);
            }
            // springs in the order the reference applies them: nodes in
            // node-map order, each node's edges by the other body's id, each
            // edge once, an edge's springs in creation order
            if (!w.springs.empty()) {
                const int nb = (int)w.bodies.size();
                std::vector<std::vector<int>> sadj(nb);
                for (int e = 0; e < (int)G.edge_pair.size(); e++) {
                    sadj[G.edge_pair[e].first].push_back(e);
                    sadj[G.edge_pair[e].second].push_back(e);
                }
                std::map<std::pair<int, int>, std::vector<int>> by_pair;
                for (int k = 0; k < (int)w.springs.size(); k++)
                    by_pair[{std::min(w.springs[k].b1, w.springs[k].b2), std::max(w.springs[k].b1, w.springs[k].b2)}].push_back(k);
                std::vector<char> seen(G.edge_pair.size(), 0);
                for (int node : order) {
                    std::vector<int> es = sadj[node];
                    std::sort(es.begin(), es.end(), [&](int x, int y) {
                        auto other = [&](int e) { return G.edge_pair[e].first == node ? G.edge_pair[e].second : G.edge_pair[e].first; };
                        return other(x) < other(y);
                    });
                    for (int e : es) {
                        if (seen[e]) continue;
                        seen[e] = 1;
                        auto it = by_pair.find(G.edge_pair[e]);
                        if (it == by_pair.end()) continue;
                        for (int k : it->second) {
                            const HSpring& sp = w.springs[k];
                            sp_b1.push_back(base + sp.b1); sp_b2.push_back(base + sp.b2);
                            sp_p1.push_back(f4d(sp.p1)); sp_p2.push_back(f4d(sp.p2));
                            sp_par.push_back(make_float4((float)sp.damping, (float)sp.stiffness, (float)sp.rest, 0.f));
                        }
                    }
                }
            }
            for (const HSystem& H : G.systems) {
                for (int j : H.cons) hs_cons.push_back(jbase + j);
                hs_vpos.insert(hs_vpos.end(), H.vpos.begin(), H.vpos.end());
                hs_cstart.push_back((int)hs_cons.size());
                hs_degree.push_back(H.degree);
                hs_table.insert(hs_table.end(), H.table.begin(), H.table.end());
                hs_tstart.push_back((int)hs_table.size());
                {
                    const int nc = (int)H.cons.size();
                    hs_lbase.push_back((int)hs_lstart.size());
                    for (int col = 0; col < nc; col++) {
                        hs_lstart.push_back((int)hs_lrow.size());
                        const int base = col * nc - (col * (col - 1)) / 2;   // column col starts at its diagonal
                        for (int row = col + 1; row < nc; row++) {
                            const int l = H.table[base + (row - col)];
                            if (l >= 0) { hs_lrow.push_back(row); hs_lloc.push_back(l); }
                        }
                    }
                    hs_lstart.push_back((int)hs_lrow.size());
                }
                hs_cap.push_back(H.cap);
                hs_fp64.push_back(H.fp64 ? 1 : 0);
                const size_t need = (size_t)H.cap + 6 * (size_t)H.degree;
                if (H.fp64) { hs_bstart.push_back((int)pool64_n); pool64_n += need; }
                else { hs_bstart.push_back((int)pool32_n); pool32_n += (need + 3) & ~size_t(3); }
                hs_wk.push_back((int)work_n);
                work_n += 2 * (size_t)H.degree;
            }
        }
        je_wstart.push_back((int)je_key.size());
        je_wjstart.push_back((int)j_b1.size());
        hs_wstart.push_back((int)hs_degree.size());
        sp_wstart.push_back((int)sp_b1.size());
    }
    const int n_joints = (int)j_b1.size(), n_je = (int)je_key.size(), n_sys = (int)hs_degree.size();
    const int n_springs = (int)sp_b1.size();
    B->world_jstart = je_wjstart;
    B->joints = n_je > 0;
    B->springs = n_springs > 0;
    B->systems = n_sys > 0;

    // ---- capacities and device allocation
    // capacities per body, with floors; both can be overridden by the environment
    const int floor_ = env_int("CPGPU_CAPACITY_FLOOR", 1 << 14);
    // polls of each bounded device wait; lowering it makes the waits give up
    // (ST_TIMEOUT, CPGPU_ERR_TIMEOUT) without any fault, for failure tests
    const long long wait_limit = std::max(0, env_int("CPGPU_WAIT_LIMIT", (int)std::min<long long>(kDefaultWaitLimit, 1 << 30)));
    const int cap_pairs = std::max(floor_, env_int("CPGPU_PAIRS_PER_BODY", 24) * N);
    const int cap_edges = cap_pairs;
    const int cap_contacts = std::max(std::max(2 * floor_, 2 * (int)cmag.size()), env_int("CPGPU_CONTACTS_PER_BODY", 24) * N);
    const bool mstore = B->meshes || B->unions;   // pairs through the mesh store
    const int cap_mesh = mstore ? std::max(4096, env_int("CPGPU_MESH_POINTS_PER_BODY", 32) * N) : 0;
    const int mesh_warps = mstore ? mesh_scratch_warps(B->n_sms) : 0;
    const int scan_tmp = std::max(cap_pairs, cap_contacts) / 1024 + 64;
    Dev x;
    EdgeStore es[2];
    ContactStore cs[2];
    int* counts = nullptr;
    WorldParams* d_wp = nullptr;
    int *d_wstart = nullptr, *d_map = nullptr, *d_shape = nullptr, *d_world = nullptr;
    float *d_iref = nullptr, *d_iinv_ref = nullptr;
    uint8_t *d_mov = nullptr, *d_pool = nullptr;
    float4* d_mat = nullptr;
    // the same carving runs twice: once to measure, once on the allocation
    auto carve = [&](Arena& A) {
        std::memset(&x, 0, sizeof(x));
        x.n_worlds = (int)worlds.size();
        x.n_bodies = N;
        x.cap_pairs = cap_pairs; x.cap_edges = cap_edges; x.cap_contacts = cap_contacts;
        d_wp = A.take<WorldParams>(worlds.size());
        d_wstart = A.take<int>(wstart.size());
        d_map = A.take<int>(N);
        x.wparams = d_wp; x.world_start = d_wstart; x.map_order = d_map;
        x.pos = A.take<float4>(N); x.rot = A.take<float4>(N); x.vel = A.take<float4>(N); x.angv = A.take<float4>(N);
        x.pvel = A.take<float4>(N); x.pangv = A.take<float4>(N);
        x.iinv = A.take<float>(9 * (size_t)N); x.iw = A.take<float>(9 * (size_t)N);
        d_iref = A.take<float>(9 * (size_t)N);
        d_iinv_ref = A.take<float>(9 * (size_t)N);
        x.iref = d_iref; x.iinv_ref = d_iinv_ref;
        d_shape = A.take<int>(N); d_world = A.take<int>(N);
        d_mov = A.take<uint8_t>(N);
        d_mat = A.take<float4>(N);
        x.shape = d_shape; x.world = d_world; x.movement = d_mov; x.material = d_mat;
        x.aabb_lo = A.take<float4>(N); x.aabb_hi = A.take<float4>(N);
        x.moved = A.take<int>(N);
        if (has_sleep) {
            x.has_sleep = 1;
            x.hist_cap = hist_cap;
            x.asleep = A.take<int>(N); x.waking = A.take<int>(N); x.ready_cnt = A.take<int>(N);
            x.non_sleepy = A.take<int>(N); x.hist_n = A.take<int>(N); x.hist_head = A.take<int>(N);
            x.hist = A.take<float>((size_t)N * hist_cap * 6);
        }
        d_pool = A.take<uint8_t>(pool.size());
        x.shapes = d_pool;
        x.pair_count = A.take<int>(N);
        x.n_tile_tasks = (int)tile_task.size();
        x.tile_task = A.take<int4>(tile_task.size());
        x.tile_base = A.take<int>(worlds.size());
        x.tile_cnt = A.take<int>(tile_cells);
        // CPGPU_ISLANDS_SERIAL=1: large worlds take the serial search too (a
        // test compares the two)
        if (!tile_task.empty() && !env_int("CPGPU_ISLANDS_SERIAL", 0)) {
            x.comp = A.take<int>((size_t)kCompArrays * N);
            x.sys_mark = A.take<int>(std::max<size_t>(hs_degree.size(), 1));
        }
        x.pair_a = A.take<int>(cap_pairs); x.pair_b = A.take<int>(cap_pairs);
        x.mf_n = A.take<float4>(cap_pairs); x.mf_cnt = A.take<int>(cap_pairs);
        x.mf_pt = A.take<float4>(4 * (size_t)cap_pairs); x.mf_magic = A.take<uint64_t>(4 * (size_t)cap_pairs);
        x.mf_feat = A.take<int2>(cap_pairs);
        for (int k = 0; k < 2; k++) {
            es[k].key = A.take<uint64_t>(cap_edges); es[k].cstart = A.take<int>(cap_edges); es[k].ccount = A.take<int>(cap_edges);
            cs[k].magic = A.take<uint64_t>(cap_contacts);
            cs[k].p1 = A.take<float4>(cap_contacts); cs[k].p2 = A.take<float4>(cap_contacts); cs[k].n = A.take<float4>(cap_contacts);
            cs[k].imp = A.take<float4>(cap_contacts); cs[k].fu = A.take<float4>(cap_contacts); cs[k].fw = A.take<float4>(cap_contacts);
            cs[k].state = A.take<int>(cap_contacts); cs[k].edge = A.take<int>(cap_contacts);
            cs[k].tri = A.take<int>(cap_contacts);
        }
        counts = A.take<int>(64);   // n_pairs, n_edges[2], n_contacts[2], n_islands, status, .., cnt[16..]
        x.n_pairs = counts + 0;
        x.surv = A.take<int>(cap_edges); x.surv_scan = A.take<int>(cap_edges);
        x.unm = A.take<int>(cap_pairs); x.unm_scan = A.take<int>(cap_pairs); x.pair_edge = A.take<int>(cap_pairs);
        x.edge_src = A.take<int>(cap_edges); x.edge_pair = A.take<int>(cap_edges); x.edge_cnt = A.take<int>(cap_edges);
        x.edge_live = A.take<int>(cap_edges); x.edge_row = A.take<int>(cap_edges);
        x.scan_tmp = A.take<int>(scan_tmp);
        x.adj_ofs = A.take<int>(N); x.adj_cursor = A.take<int>(N);
        x.adj_list = A.take<int>(2 * (2 * ((size_t)cap_edges + n_je) + N));
        x.visited = A.take<int>(N);
        x.stack = A.take<int>(2 * ((size_t)cap_edges + n_je) + N);
        x.isl_count_w = A.take<int>(worlds.size()); x.isl_scan = A.take<int>(worlds.size());
        x.isl_row_start = A.take<int>(N); x.isl_row_count = A.take<int>(N); x.isl_body_start = A.take<int>(N);
        x.isl_body_count = A.take<int>(N); x.isl_world = A.take<int>(N);
        x.g_isl_row_start = A.take<int>(N); x.g_isl_row_count = A.take<int>(N); x.g_isl_body_start = A.take<int>(N);
        x.g_isl_body_count = A.take<int>(N); x.g_isl_world = A.take<int>(N);
        x.n_islands = counts + 5;
        x.isl_bodies = A.take<int>(N);
        x.row_contact = A.take<int>((size_t)cap_contacts + n_joints); x.row_of_contact = A.take<int>(cap_contacts);
        x.rows = A.take<RowBlock>((size_t)cap_contacts + n_joints);
        x.dv = A.take<float4>(4 * (size_t)N);
        x.stage = A.take<float4>(4 * (size_t)N);
        x.big_list = A.take<int>(N);
        x.small_list = A.take<int>(N);
        x.sched = A.take<int>(kSchedInts);
        x.status = counts + 6;
        x.cnt = counts + 16;
        if (mstore) {
            x.has_mesh = B->meshes ? 1 : 0;
            x.cap_mesh_pts = cap_mesh;
            x.mesh_warps = mesh_warps;
            x.mf_ofs = A.take<int>(cap_pairs);
            x.mm_pt = A.take<float4>(cap_mesh); x.mm_n = A.take<float4>(cap_mesh);
            x.mm_magic = A.take<uint64_t>(cap_mesh); x.mm_tri = A.take<int>(cap_mesh);
            x.mm_count = counts + 8;
            x.msc = A.take<MeshScratch>(mesh_warps);
        }
        if (B->unions) {
            x.has_union = 1;
            x.prim_start = A.take<int>(N);
            x.prim_count = A.take<int>(N);
            x.prim_shape = A.take<int>(prim_shape.size());
            x.prim_mat = A.take<float4>(prim_mat.size());
            x.prim_lo = A.take<float4>(prim_shape.size());
            x.prim_hi = A.take<float4>(prim_shape.size());
        }
        x.n_joints = n_joints;
        x.n_joint_edges = n_je;
        x.lin_err_threshold = 15.0f;   // excessive_linear_error_torque_threshold (PhysicsEngine.h:217)
        x.wait_limit = wait_limit;
        x.big_rows = kDefaultBigRows;
        if (n_springs > 0) {
            SpringStore& S = x.sp;
            S.n = n_springs;
            S.b1 = A.take<int>(n_springs); S.b2 = A.take<int>(n_springs);
            S.p1 = A.take<float4>(n_springs); S.p2 = A.take<float4>(n_springs); S.par = A.take<float4>(n_springs);
            S.world_start = A.take<int>(worlds.size() + 1);
        }
        if (n_je > 0) {
            // joint edges (joints or springs): the joint store is allocated
            // even when only springs are present
            JointStore& J = x.jt;
            int* ib1 = A.take<int>(n_joints); int* ib2 = A.take<int>(n_joints); int* in = A.take<int>(n_joints);
            J.b1 = ib1; J.b2 = ib2; J.n = in;
            J.kind = A.take<int>(n_joints);
            J.p1 = A.take<float4>(n_joints); J.p2 = A.take<float4>(n_joints);
            J.ax1 = A.take<float4>(n_joints); J.ax2 = A.take<float4>(n_joints);
            J.hard = A.take<float2>(n_joints);
            J.par = A.take<float4>(n_joints); J.ul = A.take<float4>(n_joints); J.wl = A.take<float4>(n_joints);
            J.impulse = A.take<float>(kJMax * (size_t)n_joints);
            J.u = A.take<float4>(n_joints); J.w = A.take<float4>(n_joints);
            J.angle = A.take<float>(n_joints); J.active = A.take<int>(n_joints);
            J.aux = A.take<float>(n_joints); J.power = A.take<float4>(n_joints);
            J.rows = A.take<JointRow>(n_joints);
            JointEdgeStore& E = x.je;
            E.key = A.take<uint64_t>(n_je); E.jstart = A.take<int>(n_je); E.jcount = A.take<int>(n_je);
            E.jlist = A.take<int>(je_jlist.size());
            E.sys = A.take<int>(n_je);
            E.world_start = A.take<int>(worlds.size() + 1); E.world_jstart = A.take<int>(worlds.size() + 1);
            HoloStore& H = x.hs;
            H.n = n_sys;
            H.cstart = A.take<int>(n_sys + 1); H.cons = A.take<int>(hs_cons.size()); H.vpos = A.take<int>(hs_vpos.size());
            H.degree = A.take<int>(n_sys); H.tstart = A.take<int>(n_sys + 1); H.table = A.take<int>(hs_table.size());
            H.lbase = A.take<int>(n_sys); H.lstart = A.take<int>(hs_lstart.size());
            H.lrow = A.take<int>(hs_lrow.size()); H.lloc = A.take<int>(hs_lloc.size());
            H.bstart = A.take<int>(n_sys); H.cap = A.take<int>(n_sys); H.fp64 = A.take<int>(n_sys);
            H.wstart = A.take<int>(n_sys);
            H.pool32 = A.take<float>(pool32_n); H.pool64 = A.take<double>(pool64_n); H.work = A.take<double>(work_n);
            H.isl = nullptr;
            x.hs_world_start = A.take<int>(worlds.size() + 1);
            x.isl_flags = A.take<int>(N); x.g_isl_flags = A.take<int>(N);
            x.isl_sys_start = A.take<int>(N); x.isl_sys_count = A.take<int>(N);
            x.g_isl_sys_start = A.take<int>(N); x.g_isl_sys_count = A.take<int>(N);
            x.isl_sys = A.take<int>(n_sys);
            x.joint_list = A.take<int>(N);
            x.dv_err = A.take<float4>(4 * (size_t)N);
        }
    };
    Arena measure{nullptr, 0, 0};
    carve(measure);
    const size_t bytes = measure.used + 256;
    B->bytes = bytes;
    CK(cudaMalloc(&B->mem, bytes));
    Arena A{B->mem, bytes, 0};
    carve(A);

    // ---- upload
    auto up = [&](void* dst, const void* src, size_t n) { if (n) CK(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, B->st)); };
    CK(cudaMemsetAsync(counts, 0, 64 * sizeof(int), B->st));
    up(d_wp, wp.data(), wp.size() * sizeof(WorldParams));
    up(d_wstart, wstart.data(), wstart.size() * sizeof(int));
    up(d_map, map_order.data(), N * sizeof(int));
    up(x.pos, pos.data(), N * sizeof(float4)); up(x.rot, rot.data(), N * sizeof(float4));
    up(x.vel, vel.data(), N * sizeof(float4)); up(x.angv, angv.data(), N * sizeof(float4));
    up(x.pvel, zero4.data(), N * sizeof(float4)); up(x.pangv, zero4.data(), N * sizeof(float4));
    up(x.iinv, iinv.data(), iinv.size() * 4); up(x.iw, iw.data(), iw.size() * 4);
    up(d_iref, iref.data(), iref.size() * 4); up(d_iinv_ref, iinv_ref.data(), iinv_ref.size() * 4);
    up(d_shape, shape_off.data(), N * 4); up(d_world, world_of.data(), N * 4);
    up(d_mov, movement.data(), N); up(d_mat, mat.data(), N * sizeof(float4));
    up(d_pool, pool.data(), pool.size());
    up(x.moved, fresh.data(), N * 4);   // the first geometry pass renormalises these orientations
    up((void*)x.tile_task, tile_task.data(), tile_task.size() * sizeof(int4));
    if (B->unions) {
        up((void*)x.prim_start, prim_start.data(), N * 4); up((void*)x.prim_count, prim_count.data(), N * 4);
        up((void*)x.prim_shape, prim_shape.data(), prim_shape.size() * 4);
        up((void*)x.prim_mat, prim_mat.data(), prim_mat.size() * 16);
    }
    up((void*)x.tile_base, tile_base.data(), tile_base.size() * 4);
    if (has_sleep) {
        up(x.asleep, s_asleep.data(), N * 4); up(x.waking, s_waking.data(), N * 4); up(x.ready_cnt, s_ready.data(), N * 4);
        up(x.non_sleepy, s_nons.data(), N * 4); up(x.hist_n, s_hn.data(), N * 4);
        CK(cudaMemsetAsync(x.hist_head, 0, N * sizeof(int), B->st));
        up(x.hist, s_hist.data(), s_hist.size() * 4);
    }
    const int ne = (int)ekey.size(), nc = (int)cmag.size();
    up(es[0].key, ekey.data(), ne * 8); up(es[0].cstart, ecstart.data(), ne * 4); up(es[0].ccount, eccount.data(), ne * 4);
    up(cs[0].magic, cmag.data(), nc * 8);
    up(cs[0].p1, cp1.data(), nc * 16); up(cs[0].p2, cp2.data(), nc * 16); up(cs[0].n, cn.data(), nc * 16);
    up(cs[0].imp, cimp.data(), nc * 16); up(cs[0].fu, cfu.data(), nc * 16); up(cs[0].fw, cfw.data(), nc * 16);
    up(cs[0].state, cstate.data(), nc * 4); up(cs[0].edge, cedge.data(), nc * 4);
    up(cs[0].tri, ctri.data(), nc * 4);
    int host_counts[5] = {0, ne, 0, nc, 0};   // n_pairs, n_edges[0], n_edges[1], n_contacts[0], n_contacts[1]
    up(counts, host_counts, sizeof(host_counts));
    if (n_springs > 0) {
        const SpringStore& S = x.sp;
        up((void*)S.b1, sp_b1.data(), n_springs * 4); up((void*)S.b2, sp_b2.data(), n_springs * 4);
        up((void*)S.p1, sp_p1.data(), n_springs * 16); up((void*)S.p2, sp_p2.data(), n_springs * 16);
        up((void*)S.par, sp_par.data(), n_springs * 16);
        up((void*)S.world_start, sp_wstart.data(), sp_wstart.size() * 4);
    }
    if (n_je > 0) {
        const JointStore& J = x.jt;
        up((void*)J.b1, j_b1.data(), n_joints * 4); up((void*)J.b2, j_b2.data(), n_joints * 4); up((void*)J.n, j_n.data(), n_joints * 4);
        up((void*)J.kind, j_kind.data(), n_joints * 4);
        up((void*)J.p1, j_p1.data(), n_joints * 16); up((void*)J.p2, j_p2.data(), n_joints * 16);
        up((void*)J.ax1, j_ax1.data(), n_joints * 16); up((void*)J.ax2, j_ax2.data(), n_joints * 16);
        up((void*)J.hard, j_hard.data(), n_joints * 8);
        up((void*)J.par, j_par.data(), n_joints * 16); up((void*)J.ul, j_ul.data(), n_joints * 16); up((void*)J.wl, j_wl.data(), n_joints * 16);
        up(J.impulse, j_imp.data(), j_imp.size() * 4);
        up(J.u, j_u.data(), n_joints * 16); up(J.w, j_w.data(), n_joints * 16);
        up(J.angle, j_angle.data(), n_joints * 4); up(J.active, j_active.data(), n_joints * 4);
        up(J.aux, j_aux.data(), n_joints * 4); up((void*)J.power, j_power.data(), n_joints * 16);
        if (n_joints > 0) CK(cudaMemsetAsync(J.rows, 0, sizeof(JointRow) * (size_t)n_joints, B->st));
        const JointEdgeStore& E = x.je;
        up((void*)E.key, je_key.data(), n_je * 8); up((void*)E.jstart, je_jstart.data(), n_je * 4);
        up((void*)E.jcount, je_jcount.data(), n_je * 4); up((void*)E.sys, je_sys.data(), n_je * 4);
        up((void*)E.jlist, je_jlist.data(), je_jlist.size() * 4);
        up((void*)E.world_start, je_wstart.data(), je_wstart.size() * 4);
        up((void*)E.world_jstart, je_wjstart.data(), je_wjstart.size() * 4);
        const HoloStore& H = x.hs;
        up((void*)H.cstart, hs_cstart.data(), hs_cstart.size() * 4); up((void*)H.cons, hs_cons.data(), hs_cons.size() * 4);
        up((void*)H.vpos, hs_vpos.data(), hs_vpos.size() * 4); up((void*)H.degree, hs_degree.data(), hs_degree.size() * 4);
        up((void*)H.tstart, hs_tstart.data(), hs_tstart.size() * 4); up((void*)H.table, hs_table.data(), hs_table.size() * 4);
        up((void*)H.lbase, hs_lbase.data(), hs_lbase.size() * 4); up((void*)H.lstart, hs_lstart.data(), hs_lstart.size() * 4);
        up((void*)H.lrow, hs_lrow.data(), hs_lrow.size() * 4); up((void*)H.lloc, hs_lloc.data(), hs_lloc.size() * 4);
        up((void*)H.bstart, hs_bstart.data(), hs_bstart.size() * 4); up((void*)H.cap, hs_cap.data(), hs_cap.size() * 4);
        up((void*)H.fp64, hs_fp64.data(), hs_fp64.size() * 4); up((void*)H.wstart, hs_wk.data(), hs_wk.size() * 4);
        up((void*)x.hs_world_start, hs_wstart.data(), hs_wstart.size() * 4);
    }
    for (int p = 0; p < 2; p++) {
        Dev y = x;
        y.e_old = es[p]; y.e_new = es[1 - p];
        y.c_old = cs[p]; y.c_new = cs[1 - p];
        y.n_edges_old = counts + 1 + p; y.n_edges_new = counts + 1 + (1 - p);
        y.n_contacts_old = counts + 3 + p; y.n_contacts_new = counts + 3 + (1 - p);
        B->d[p] = y;
    }
    B->parity = 0;
    Launch L{B->n_sms, B->st};
    launch_geometry(B->d[0], 2, L);
    prepare_kernels();
    prepare_pgs(B->dv_cap);
    B->pgs_per_sm = pgs_per_sm;
    B->pgs_blocks = B->n_sms * (pgs_per_sm > 0 ? std::min(pgs_per_sm, pgs_big_blocks_per_sm(B->dv_cap)) : pgs_big_blocks_per_sm(B->dv_cap));
    CK(cudaStreamSynchronize(B->st));
    CK(cudaGetLastError());
    B->build_graphs();
    return B;
}

// ---------------------------------------------------------------- world helpers ----
// Pull the device state of the batch's worlds into their host mirrors: poses,
// velocities, world inertia tensors, joint warm starts, the persistent contact
// graph (dead contacts dropped, as the next merge would) and the last pair
// list.  All arrays are read once and split per world.
// The sleep state of one world's bodies (global range [g0, g0 + nb)) into
// their host mirrors, the velocity records turned oldest first
static void download_sleep(const Batch& B, int g0, World& w) {
    const Dev& x = B.cur();
    if (!x.has_sleep) return;
    const int nb = (int)w.bodies.size(), cap = x.hist_cap;
    std::vector<int> a(nb), wk(nb), rd(nb), ns(nb), hn(nb), hh(nb);
    std::vector<float> h((size_t)nb * cap * 6);
    CK(cudaMemcpyAsync(a.data(), x.asleep + g0, nb * 4, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(wk.data(), x.waking + g0, nb * 4, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(rd.data(), x.ready_cnt + g0, nb * 4, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(ns.data(), x.non_sleepy + g0, nb * 4, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(hn.data(), x.hist_n + g0, nb * 4, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(hh.data(), x.hist_head + g0, nb * 4, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(h.data(), x.hist + (size_t)g0 * cap * 6, h.size() * 4, cudaMemcpyDeviceToHost, B.st));
    CK(cudaStreamSynchronize(B.st));
    const int len = std::max(1, (int)(w.p.sleep_delay / w.p.dt));
    for (int i = 0; i < nb; i++) {
        Body& b = w.bodies[i];
        b.asleep = a[i]; b.waking = wk[i]; b.ready_cnt = rd[i]; b.non_sleepy = ns[i]; b.hist_n = hn[i];
        b.hist.assign(6 * (size_t)hn[i], 0.f);
        for (int q = 0; q < hn[i]; q++) {
            const int slot = (hh[i] + q) % len;
            for (int k = 0; k < 6; k++) b.hist[6 * q + k] = h[((size_t)i * cap + slot) * 6 + k];
        }
    }
}

static void download_worlds(Batch& B, const std::vector<World*>& ws) {
    const Dev& x = B.cur();
    const int N = B.n_bodies;
    std::vector<float4> pos(N), rot(N), vel(N), angv(N);
    std::vector<float> iw(9 * (size_t)N), iinv(9 * (size_t)N);
    CK(cudaMemcpyAsync(pos.data(), x.pos, N * 16, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(rot.data(), x.rot, N * 16, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(vel.data(), x.vel, N * 16, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(angv.data(), x.angv, N * 16, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(iw.data(), x.iw, iw.size() * 4, cudaMemcpyDeviceToHost, B.st));
    CK(cudaMemcpyAsync(iinv.data(), x.iinv, iinv.size() * 4, cudaMemcpyDeviceToHost, B.st));
    int counts[6];
    CK(cudaMemcpyAsync(counts, x.n_pairs, sizeof(counts), cudaMemcpyDeviceToHost, B.st));
    const int nj = x.n_joints;
    std::vector<float> jimp((size_t)kJMax * nj), jang(nj), jaux(nj);
    std::vector<float4> ju(nj), jw(nj);
    std::vector<int> jact(nj);
    if (nj > 0) {
        CK(cudaMemcpyAsync(jimp.data(), x.jt.impulse, jimp.size() * 4, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(ju.data(), x.jt.u, nj * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(jw.data(), x.jt.w, nj * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(jang.data(), x.jt.angle, nj * 4, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(jact.data(), x.jt.active, nj * 4, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(jaux.data(), x.jt.aux, nj * 4, cudaMemcpyDeviceToHost, B.st));
    }
    CK(cudaStreamSynchronize(B.st));
    // contact graph (current = the old buffers of the next step)
    const int ne = *(&counts[1] + B.parity), nc = *(&counts[3] + B.parity);
    std::vector<uint64_t> key(ne), mag(nc);
    std::vector<int> cstart(ne), ccount(ne), state(nc), tri(nc);
    std::vector<float4> p1(nc), p2(nc), n(nc), imp(nc), fu(nc), fw(nc);
    const EdgeStore& E = x.e_old;
    const ContactStore& C = x.c_old;
    if (ne) {
        CK(cudaMemcpyAsync(key.data(), E.key, ne * 8, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(cstart.data(), E.cstart, ne * 4, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(ccount.data(), E.ccount, ne * 4, cudaMemcpyDeviceToHost, B.st));
    }
    if (nc) {
        CK(cudaMemcpyAsync(mag.data(), C.magic, nc * 8, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(p1.data(), C.p1, nc * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(p2.data(), C.p2, nc * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(n.data(), C.n, nc * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(imp.data(), C.imp, nc * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(fu.data(), C.fu, nc * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(fw.data(), C.fw, nc * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(state.data(), C.state, nc * 4, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(tri.data(), C.tri, nc * 4, cudaMemcpyDeviceToHost, B.st));
    }
    int np = counts[0];
    std::vector<int> pa(np), pb(np);
    if (np) {
        CK(cudaMemcpyAsync(pa.data(), x.pair_a, np * 4, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(pb.data(), x.pair_b, np * 4, cudaMemcpyDeviceToHost, B.st));
    }
    CK(cudaStreamSynchronize(B.st));
    int e_cursor = 0, p_cursor = 0;
    for (size_t wi = 0; wi < ws.size(); wi++) {
        World& w = *ws[wi];
        const int s0 = B.world_start[wi], s1 = B.world_start[wi + 1];
        for (int i = s0; i < s1; i++) {
            Body& b = w.bodies[i - s0];
            b.com = D3(pos[i].x, pos[i].y, pos[i].z);
            b.q = Quat{rot[i].x, rot[i].y, rot[i].z, rot[i].w};
            b.fresh = 0;
            if (b.movement != CPGPU_FIXED) {
                b.vel = D3(vel[i].x, vel[i].y, vel[i].z);
                b.angv = D3(angv[i].x, angv[i].y, angv[i].z);
            }
            if (b.movement == CPGPU_DYNAMIC)
                for (int k = 0; k < 9; k++) { b.iw[k] = iw[9 * (size_t)i + k]; b.iinv[k] = iinv[9 * (size_t)i + k]; }
        }
        if (nj > 0) {
            const int j0 = B.world_jstart[wi];
            for (size_t j = 0; j < w.joints.size(); j++) {
                const size_t g = (size_t)j0 + j;
                for (int k = 0; k < kJMax; k++) w.joints[j].impulse[k] = jimp[kJMax * g + k];
                w.joints[j].angle = jang[g];
                w.joints[j].active = jact[g];
                w.joints[j].aux = jaux[g];
                w.joints[j].u[0] = ju[g].x; w.joints[j].u[1] = ju[g].y; w.joints[j].u[2] = ju[g].z;
                w.joints[j].w[0] = jw[g].x; w.joints[j].w[1] = jw[g].y; w.joints[j].w[2] = jw[g].z;
            }
        }
        w.contacts.clear();
        for (; e_cursor < ne && (int)(key[e_cursor] >> 32) < s1; e_cursor++) {
            const int e = e_cursor;
            uint32_t b1 = (uint32_t)((key[e] >> 32) - s0) + 1, b2 = (uint32_t)((key[e] & 0xffffffffu) - s0) + 1;
            for (int k = cstart[e]; k < cstart[e] + ccount[e]; k++) {
                if (cs_dead(state[k])) continue;
                cpgpu_contact c;
                std::memset(&c, 0, sizeof(c));
                c.b1 = b1; c.b2 = b2;
                c.live = cs_live(state[k]);
                c.memory_life = cs_life(state[k]);
                c.magic_c = contact_cid(w, b1, b2, tri[k]);
                c.magic_b = mag[k];
                c.p_local_b1[0] = p1[k].x; c.p_local_b1[1] = p1[k].y; c.p_local_b1[2] = p1[k].z;
                c.p_local_b2[0] = p2[k].x; c.p_local_b2[1] = p2[k].y; c.p_local_b2[2] = p2[k].z;
                c.n_local_b1[0] = n[k].x; c.n_local_b1[1] = n[k].y; c.n_local_b1[2] = n[k].z;
                c.pen_depth = p1[k].w; c.bounce = p2[k].w; c.friction_coeff = n[k].w;
                c.normal_impulse = imp[k].x; c.friction_impulse[0] = imp[k].y; c.friction_impulse[1] = imp[k].z;
                c.friction_u[0] = fu[k].x; c.friction_u[1] = fu[k].y; c.friction_u[2] = fu[k].z;
                c.friction_w[0] = fw[k].x; c.friction_w[1] = fw[k].y; c.friction_w[2] = fw[k].z;
                c.static_ready = cs_static(state[k]);
                w.contacts.push_back(c);
            }
        }
        download_sleep(B, s0, w);
        w.last_pairs.clear();
        for (; p_cursor < np && pa[p_cursor] < s1; p_cursor++) {
            w.last_pairs.push_back((uint32_t)(pa[p_cursor] - s0) + 1);
            w.last_pairs.push_back((uint32_t)(pb[p_cursor] - s0) + 1);
        }
    }
}

// The state of some of the batch's worlds (indices `widx`) into their host
// mirrors, reading only their ranges: bodies, joints, and their contacts via
// the per-world edge / contact ranges of the current graph.
static void download_subset(Batch& B, const std::vector<int>& widx, const std::vector<World*>& ws) {
    const Dev& x = B.cur();
    const int n = (int)widx.size();
    if (n == 0) return;
    int* dwi = nullptr;
    CK(cudaMallocAsync((void**)&dwi, sizeof(int) * 5 * (size_t)n, B.st));
    int* dout = dwi + n;
    CK(cudaMemcpyAsync(dwi, widx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, B.st));
    launch_world_ranges(x, dwi, n, dout, B.st);
    std::vector<int> rg(4 * (size_t)n);
    CK(cudaMemcpyAsync(rg.data(), dout, sizeof(int) * 4 * (size_t)n, cudaMemcpyDeviceToHost, B.st));
    CK(cudaFreeAsync(dwi, B.st));
    CK(cudaStreamSynchronize(B.st));
    struct Buf {
        std::vector<float4> pos, rot, vel, angv;
        std::vector<float> iw, iinv, jimp, jang, jaux;
        std::vector<float4> ju, jw;
        std::vector<int> jact;
        std::vector<uint64_t> key, mag;
        std::vector<int> cstart, ccount, state, tri;
        std::vector<float4> p1, p2, nrm, imp, fu, fw;
    };
    std::vector<Buf> bufs(n);
    auto get = [&](void* dst, const void* src, size_t bytes) {
        if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, B.st));
    };
    for (int i = 0; i < n; i++) {
        const int w = widx[i], s0 = B.world_start[w], nb = B.world_start[w + 1] - s0;
        Buf& b = bufs[i];
        b.pos.resize(nb); b.rot.resize(nb); b.vel.resize(nb); b.angv.resize(nb);
        b.iw.resize(9 * (size_t)nb); b.iinv.resize(9 * (size_t)nb);
        get(b.pos.data(), x.pos + s0, nb * 16); get(b.rot.data(), x.rot + s0, nb * 16);
        get(b.vel.data(), x.vel + s0, nb * 16); get(b.angv.data(), x.angv + s0, nb * 16);
        get(b.iw.data(), x.iw + 9 * (size_t)s0, 36 * (size_t)nb); get(b.iinv.data(), x.iinv + 9 * (size_t)s0, 36 * (size_t)nb);
        if (x.n_joints > 0) {
            const int j0 = B.world_jstart[w], nj = B.world_jstart[w + 1] - j0;
            b.jimp.resize((size_t)kJMax * nj); b.ju.resize(nj); b.jw.resize(nj); b.jang.resize(nj); b.jact.resize(nj);
            b.jaux.resize(nj);
            get(b.jimp.data(), x.jt.impulse + (size_t)kJMax * j0, (size_t)kJMax * nj * 4);
            get(b.ju.data(), x.jt.u + j0, nj * 16); get(b.jw.data(), x.jt.w + j0, nj * 16);
            get(b.jang.data(), x.jt.angle + j0, nj * 4); get(b.jact.data(), x.jt.active + j0, nj * 4);
            get(b.jaux.data(), x.jt.aux + j0, nj * 4);
        }
        const int e0 = rg[4 * i], e1 = rg[4 * i + 1], c0 = rg[4 * i + 2], c1 = rg[4 * i + 3];
        const int ne = e1 - e0, nc = c1 - c0;
        b.key.resize(ne); b.cstart.resize(ne); b.ccount.resize(ne);
        get(b.key.data(), x.e_old.key + e0, ne * 8); get(b.cstart.data(), x.e_old.cstart + e0, ne * 4);
        get(b.ccount.data(), x.e_old.ccount + e0, ne * 4);
        b.mag.resize(nc); b.state.resize(nc); b.tri.resize(nc);
        get(b.tri.data(), x.c_old.tri + c0, nc * 4);
        b.p1.resize(nc); b.p2.resize(nc); b.nrm.resize(nc); b.imp.resize(nc); b.fu.resize(nc); b.fw.resize(nc);
        get(b.mag.data(), x.c_old.magic + c0, nc * 8); get(b.state.data(), x.c_old.state + c0, nc * 4);
        get(b.p1.data(), x.c_old.p1 + c0, nc * 16); get(b.p2.data(), x.c_old.p2 + c0, nc * 16);
        get(b.nrm.data(), x.c_old.n + c0, nc * 16); get(b.imp.data(), x.c_old.imp + c0, nc * 16);
        get(b.fu.data(), x.c_old.fu + c0, nc * 16); get(b.fw.data(), x.c_old.fw + c0, nc * 16);
        for (int& c : b.cstart) c -= c0;
    }
    CK(cudaStreamSynchronize(B.st));
    for (int i = 0; i < n; i++) {
        World& w = *ws[i];
        const Buf& b = bufs[i];
        const int s0 = B.world_start[widx[i]];
        for (size_t k = 0; k < w.bodies.size(); k++) {
            Body& bd = w.bodies[k];
            bd.com = D3(b.pos[k].x, b.pos[k].y, b.pos[k].z);
            bd.q = Quat{b.rot[k].x, b.rot[k].y, b.rot[k].z, b.rot[k].w};
            bd.fresh = 0;
            if (bd.movement != CPGPU_FIXED) {
                bd.vel = D3(b.vel[k].x, b.vel[k].y, b.vel[k].z);
                bd.angv = D3(b.angv[k].x, b.angv[k].y, b.angv[k].z);
            }
            if (bd.movement == CPGPU_DYNAMIC)
                for (int q = 0; q < 9; q++) { bd.iw[q] = b.iw[9 * k + q]; bd.iinv[q] = b.iinv[9 * k + q]; }
        }
        for (size_t j = 0; j < b.ju.size() && j < w.joints.size(); j++) {
            for (int k = 0; k < kJMax; k++) w.joints[j].impulse[k] = b.jimp[kJMax * j + k];
            w.joints[j].angle = b.jang[j];
            w.joints[j].active = b.jact[j];
            w.joints[j].aux = b.jaux[j];
            w.joints[j].u[0] = b.ju[j].x; w.joints[j].u[1] = b.ju[j].y; w.joints[j].u[2] = b.ju[j].z;
            w.joints[j].w[0] = b.jw[j].x; w.joints[j].w[1] = b.jw[j].y; w.joints[j].w[2] = b.jw[j].z;
        }
        w.contacts.clear();
        for (size_t e = 0; e < b.key.size(); e++) {
            uint32_t b1 = (uint32_t)((b.key[e] >> 32) - s0) + 1, b2 = (uint32_t)((b.key[e] & 0xffffffffu) - s0) + 1;
            for (int k = b.cstart[e]; k < b.cstart[e] + b.ccount[e]; k++) {
                if (cs_dead(b.state[k])) continue;
                cpgpu_contact c;
                std::memset(&c, 0, sizeof(c));
                c.b1 = b1; c.b2 = b2;
                c.live = cs_live(b.state[k]);
                c.memory_life = cs_life(b.state[k]);
                c.magic_c = contact_cid(w, b1, b2, b.tri[k]);
                c.magic_b = b.mag[k];
                c.p_local_b1[0] = b.p1[k].x; c.p_local_b1[1] = b.p1[k].y; c.p_local_b1[2] = b.p1[k].z;
                c.p_local_b2[0] = b.p2[k].x; c.p_local_b2[1] = b.p2[k].y; c.p_local_b2[2] = b.p2[k].z;
                c.n_local_b1[0] = b.nrm[k].x; c.n_local_b1[1] = b.nrm[k].y; c.n_local_b1[2] = b.nrm[k].z;
                c.pen_depth = b.p1[k].w; c.bounce = b.p2[k].w; c.friction_coeff = b.nrm[k].w;
                c.normal_impulse = b.imp[k].x; c.friction_impulse[0] = b.imp[k].y; c.friction_impulse[1] = b.imp[k].z;
                c.friction_u[0] = b.fu[k].x; c.friction_u[1] = b.fu[k].y; c.friction_u[2] = b.fu[k].z;
                c.friction_w[0] = b.fw[k].x; c.friction_w[1] = b.fw[k].y; c.friction_w[2] = b.fw[k].z;
                c.static_ready = cs_static(b.state[k]);
                w.contacts.push_back(c);
            }
        }
        w.last_pairs.clear();
        download_sleep(B, s0, w);
    }
}

static void download_state(World& w) {
    if (!w.dev || !w.dev_valid) return;
    std::vector<World*> one{&w};
    download_worlds(*w.dev, one);
}

// Pull device state into the host mirror and mark the device copy stale, so the
// next step re-uploads the (mutated) world.
static void begin_mutation(World& w) {
    if (w.dev && w.dev_valid) download_state(w);
    w.dev_valid = false;
    w.version++;
}

static void update_cutoff(World& w) { w.p.cutoff = 2 * w.p.g.mag() * w.p.dt; }

static Body& body_ref(World& w, uint32_t id) {
    if (id == 0 || id > w.bodies.size()) throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad body id"};
    return w.bodies[id - 1];
}

static uint32_t add_hull(World& w, const std::vector<D3>& pts, const std::vector<std::vector<int>>& faces,
                         const cpgpu_material* m, int movement, const double* pos) {
    if (movement < 0 || movement > 2) throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad movement type"};
    HullPrep h;
    if (pts.size() < 4 || faces.size() < 4 || !h.build(pts, faces)) throw ApiFail{CPGPU_ERR_INVALID_ARG, "invalid hull"};
    Body b;
    double density = m ? m->density : 1.0;
    double t[3][3];
    hullMassProperties(h, density, &b.com, t, &b.mass);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) b.iref[3 * i + j] = t[i][j];
    inv3(b.iref, b.iinv_ref);
    std::memcpy(b.iw, b.iref, sizeof(b.iw));
    std::memcpy(b.iinv, b.iinv_ref, sizeof(b.iinv));
    Shape s = pack_hull(h, b.com);
    b.local_origin = -b.com;
    // setToPosition: translate so the geometry origin lands on pos
    D3 p = pos ? D3(pos[0], pos[1], pos[2]) : D3();
    D3 tracked = b.com + qrot(b.q, b.local_origin);
    b.com = b.com + (p - tracked);
    b.movement = movement;
    if (m) { b.rest = m->restitution; b.kin = m->kinetic_friction; b.sta = m->static_friction; }
    begin_mutation(w);
    b.shape = (int)w.shapes.size();
    w.shapes.push_back(std::move(s));
    w.bodies.push_back(b);
    uint32_t id = (uint32_t)w.bodies.size();
    w.nodes[id] = (int)id - 1;
    return id;
}

// calculateMassProperties (RigidBody.cpp:427-640), SPHERE, CYLINDER and
// CAPSULE cases for a one-primitive body with the default height axis: mass,
// centre of mass and the inertia tensor about it.  For a capsule the
// reference's mass is the volume (the density scales only the tensor,
// RigidBody.cpp:577-585); kept.
static void prim_mass(uint32_t kind, const D3& c, double r, double h, double density, double* mass, double t[9]) {
    const double pi = 3.1415926535;
    double m, d0, d1;
    if (kind == SHAPE_SPHERE) {
        m = (4.0 / 3.0) * pi * r * r * r * density;
        d0 = d1 = 2.0 / 5.0 * m * r * r;
    } else if (kind == SHAPE_CAPSULE) {
        const double r3 = r * r * r, r4 = r3 * r, r5 = r4 * r;
        m = (4.0 / 3.0) * pi * r * r * r + pi * r * r * h;
        d0 = density * pi * ((8.0 / 15.0) * r5 + (1.0 / 3.0) * r3 * h * h + 0.75 * r4 * h + (1.0 / 12.0) * r * r * h * h * h);
        d1 = density * pi * ((8.0 / 15.0) * r5 + 0.5 * h * r4);
    } else {
        m = pi * r * r * h * density;
        d0 = m * (h * h / 12 + r * r / 4);
        d1 = m * r * r / 2;
    }
    (void)c;   // one primitive: its centre is the centre of mass, the parallel-axis terms cancel
    *mass = m;
    for (int k = 0; k < 9; k++) t[k] = 0;
    t[0] = d0; t[4] = d1; t[8] = d0;
}

static uint32_t add_prim(World& w, uint32_t kind, const D3& center, double r, double h, const cpgpu_material* m,
                         int movement, const double* pos) {
    if (movement < 0 || movement > 2) throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad movement type"};
    if (!(r > 0) || (kind == SHAPE_CYLINDER && !(h > 0)) || (kind == SHAPE_CAPSULE && !(h >= 0)))
        throw ApiFail{CPGPU_ERR_INVALID_ARG, "radius must be > 0, cylinder height > 0, capsule drum height >= 0"};
    Body b;
    double density = m ? m->density : 1.0;
    prim_mass(kind, center, r, h, density, &b.mass, b.iref);
    b.com = center;
    inv3(b.iref, b.iinv_ref);
    std::memcpy(b.iw, b.iref, sizeof(b.iw));
    std::memcpy(b.iinv, b.iinv_ref, sizeof(b.iinv));
    Shape s = kind == SHAPE_SPHERE ? pack_sphere(D3(), r) : kind == SHAPE_CAPSULE ? pack_capsule(D3(), r, h) : pack_cylinder(D3(), r, h);
    b.local_origin = -b.com;
    D3 p = pos ? D3(pos[0], pos[1], pos[2]) : D3();
    D3 tracked = b.com + qrot(b.q, b.local_origin);
    b.com = b.com + (p - tracked);
    b.movement = movement;
    if (m) { b.rest = m->restitution; b.kin = m->kinetic_friction; b.sta = m->static_friction; }
    begin_mutation(w);
    b.shape = (int)w.shapes.size();
    w.shapes.push_back(std::move(s));
    w.bodies.push_back(b);
    uint32_t id = (uint32_t)w.bodies.size();
    w.nodes[id] = (int)id - 1;
    return id;
}

static void ensure_device(World& w) {
    if (w.dev && w.dev_valid) return;
    w.dev.reset();
    std::vector<World*> one{&w};
    w.dev = build_batch(one);
    w.dev_valid = true;
}

}  // namespace cpgpu

// ================================================================== C ABI ====
using namespace cpgpu;

// A batch's schedule: how its worlds are cut into parts that step
// concurrently (each on its own streams with its own graphs), how many solver
// chains per SM the later parts may run, and the island size from which an
// island takes the warp-per-island solver.  Every world steps exactly as it
// does alone under any schedule (the parts never interact; both island
// solvers give identical results), so the schedule only changes the time.
namespace cpgpu {
struct Schedule {
    int parts = 1;          // batch parts
    int first_share = 100;  // percent of the bodies in the first part (the largest worlds)
    int rest_per_sm = 0;    // chain workers per SM of the later parts (0 = as many as fit)
    int big_rows = kDefaultBigRows;
    int second_share = 0;   // three or more parts: percent of the bodies in the second part (0: the rest split evenly)
    int mid_per_sm = -1;    // three or more parts: chain workers per SM of the second part (-1: rest_per_sm)
};
}  // namespace cpgpu

// A world handle.  Batches pin the worlds they were made from (the
// autotuner re-packs from them): cpgpu_world_destroy of a pinned world only
// marks it, and the last batch holding it frees it.
struct cpgpu_world {
    World w;
    int batch_refs = 0;
    bool dropped = false;
};
// A batch of worlds, split by world size into parts that step concurrently,
// each on its own streams with its own graphs.  A step is bounded by the
// longest serial Gauss-Seidel chain of its largest island; with the largest
// worlds in a part of their own, the other parts' narrowphase and solves run
// beside that chain instead of after it.  Worlds never interact, so every
// world steps exactly as it does alone, whatever its part.
struct cpgpu_batch {
    std::vector<std::unique_ptr<Batch>> parts;
    std::vector<int> part_of, local_of;   // per world: its part and index within it
    std::vector<int> row0;                // per world: first row in the batch's body order
    int64_t n_bodies = 0;
    float4* stage = nullptr;              // host-layout rows of all bodies (4 float4 each)
    std::vector<int*> rows;               // per part: batch row of each of its bodies
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr;
    std::vector<cudaEvent_t> done;        // per part
    Schedule sched;                       // the schedule the batch was built for
    bool stagger = true;                  // step_parts: the parts' first halves in order (CPGPU_BATCH_STAGGER=0: concurrent)
    bool tuned = false;                   // chosen by the autotuner (now or from its cache)
    double tuned_ms = -1, default_ms = -1;   // per step, measured when tuned here
    std::vector<World*> worlds;           // the worlds, in batch order (their host mirrors)
    std::vector<cpgpu_world*> pins;       // the handles pinned by this batch (API-made batches)
    std::vector<uint64_t> versions;       // the worlds' mutation counts when the batch was made
    void pin(cpgpu_world* const* ws, int n) {
        for (int i = 0; i < n; i++) {
            ws[i]->batch_refs++;
            pins.push_back(ws[i]);
            versions.push_back(ws[i]->w.version);
        }
    }
    void release() {
        for (int* r : rows) if (r) cudaFree(r);
        if (stage) cudaFree(stage);
        for (cudaEvent_t e : done) cudaEventDestroy(e);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (fork) cudaEventDestroy(fork);
        rows.clear(); done.clear();
        stage = nullptr; ev0 = ev1 = fork = nullptr;
        parts.clear();
    }
    ~cpgpu_batch() {
        release();
        for (cpgpu_world* w : pins)
            if (--w->batch_refs == 0 && w->dropped) delete w;
    }
    // take over another batch object's device resources (this one's are freed)
    void adopt(cpgpu_batch& o) {
        release();
        parts = std::move(o.parts);
        part_of = std::move(o.part_of); local_of = std::move(o.local_of); row0 = std::move(o.row0);
        n_bodies = o.n_bodies;
        stage = o.stage; o.stage = nullptr;
        rows = std::move(o.rows); o.rows.clear();
        ev0 = o.ev0; ev1 = o.ev1; fork = o.fork; o.ev0 = o.ev1 = o.fork = nullptr;
        done = std::move(o.done); o.done.clear();
        sched = o.sched;   // the worlds, pins and versions stay this batch's
        stagger = o.stagger;
    }
    Batch& part(int p) { return *parts[p]; }
    cudaStream_t st0() { return parts[0]->st; }
    // n steps of every part from the graphs.  Over several steps
    // (staggered, the default) part p's first half of each step (gravity to
    // the PGS schedule) waits for part p-1's, so the parts holding the
    // largest worlds reach their serial solver chains without the other
    // parts' pair, narrowphase and island kernels competing for the SMs; the
    // chains and second halves overlap freely, and the parts drift apart
    // over the steps.  A single step, which the caller waits for, runs the
    // parts fully concurrently: its end is the last part's, which the stagger
    // would delay.  Worlds never interact: the order changes no result.
    void step_parts(int n) {
        if (parts.size() > 1 && stagger && n > 1)
            for (int i = 0; i < n; i++)
                for (size_t p = 0; p < parts.size(); p++) parts[p]->step_one(p > 0 ? parts[p - 1]->pre_done : nullptr);
        else
            for (auto& p : parts) p->step(n);   // graph launches only: the parts run concurrently
    }
    // every part's stream waits for what part 0's stream has issued so far
    void fan_out() {
        CK(cudaEventRecord(fork, st0()));
        for (size_t p = 1; p < parts.size(); p++) CK(cudaStreamWaitEvent(parts[p]->st, fork, 0));
    }
    // part 0's stream waits for what every part has issued so far
    void fan_in() {
        for (size_t p = 1; p < parts.size(); p++) {
            CK(cudaEventRecord(done[p], parts[p]->st));
            CK(cudaStreamWaitEvent(st0(), done[p], 0));
        }
    }
};

template <class F>
static int guarded(F&& f) {
    try {
        return f();
    } catch (const ApiFail& e) {
        return fail(e.code, e.msg);
    } catch (const CudaFail& e) {
        return fail(CPGPU_ERR_CUDA, e.msg);
    } catch (const std::bad_alloc&) {
        return fail(CPGPU_ERR_CUDA, "host allocation failed");
    } catch (...) {
        return fail(CPGPU_ERR_INVALID_ARG, "unexpected error");
    }
}

#define W_OR_FAIL(w) if (!(w)) return fail(CPGPU_ERR_INVALID_ARG, "null world")

extern "C" {

const char* cpgpu_last_error(void) { return g_err.c_str(); }

int cpgpu_world_create(cpgpu_world** out) {
    return guarded([&] {
        if (!out) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null out"};
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw ApiFail{CPGPU_ERR_NO_DEVICE, "no CUDA device"};
        *out = new cpgpu_world();
        return CPGPU_OK;
    });
}
int cpgpu_world_destroy(cpgpu_world* w) {
    if (w && w->batch_refs > 0) {
        w->dropped = true;   // freed with the last batch made from it
        return CPGPU_OK;
    }
    delete w;
    return CPGPU_OK;
}

#define SETTER(name, ...)                                                           \
    int name {                                                                      \
        W_OR_FAIL(w);                                                               \
        return guarded([&] { begin_mutation(w->w); __VA_ARGS__; return CPGPU_OK; }); \
    }
SETTER(cpgpu_set_step_time(cpgpu_world* w, double dt), {
    if (!(dt > 0)) throw ApiFail{CPGPU_ERR_INVALID_ARG, "step time must be positive"};
    w->w.p.dt = dt; update_cutoff(w->w); })
SETTER(cpgpu_set_gravity(cpgpu_world* w, double x, double y, double z), { w->w.p.g = D3(x, y, z); update_cutoff(w->w); })
SETTER(cpgpu_set_substep_count(cpgpu_world* w, int s), {
    if (s < 1) throw ApiFail{CPGPU_ERR_INVALID_ARG, "substeps < 1"};
    w->w.p.substeps = s; })
SETTER(cpgpu_set_pgs_iterations(cpgpu_world* w, int v, int p, int h), {
    if (v < 0 || p < 0 || h < 0) throw ApiFail{CPGPU_ERR_INVALID_ARG, "negative iteration count"};
    w->w.p.pgs_vel = v; w->w.p.pgs_pos = p; w->w.p.pgs_holo = h; })
// (bodies already asleep stay asleep until woken, as in the reference)
SETTER(cpgpu_set_sleeping_enabled(cpgpu_world* w, int e), { w->w.p.sleeping = e != 0; })
SETTER(cpgpu_set_warm_start_disabled(cpgpu_world* w, int d), { w->w.p.warm_disabled = d != 0; })
SETTER(cpgpu_set_global_cfm(cpgpu_world* w, double c), { w->w.p.cfm = c; })
SETTER(cpgpu_set_angle_vel_update_tick_count(cpgpu_world* w, int n), {
    if (n < 0) throw ApiFail{CPGPU_ERR_INVALID_ARG, "negative tick count"};
    w->w.p.angle_ticks = n; })
SETTER(cpgpu_set_internal_gyro_forces_disabled(cpgpu_world* w, int d), { w->w.p.gyro_disabled = d != 0; })

int cpgpu_body_hull(cpgpu_world* w, const double* points, int n_points, const int* face_offsets, const int* face_indices,
                    int n_faces, const cpgpu_material* m, int movement, const double pos[3], uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!points || !face_offsets || !face_indices || n_points < 4 || n_faces < 4)
            throw ApiFail{CPGPU_ERR_INVALID_ARG, "hull needs >= 4 points and faces"};
        std::vector<D3> pts(n_points);
        for (int i = 0; i < n_points; i++) pts[i] = D3(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
        std::vector<std::vector<int>> faces(n_faces);
        for (int f = 0; f < n_faces; f++)
            for (int k = face_offsets[f]; k < face_offsets[f + 1]; k++) faces[f].push_back(face_indices[k]);
        uint32_t id = add_hull(w->w, pts, faces, m, movement, pos);
        if (out_id) *out_id = id;
        return CPGPU_OK;
    });
}

int cpgpu_body_box(cpgpu_world* w, const double c[3], double dx, double dy, double dz, const cpgpu_material* m,
                   int movement, const double pos[3], uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!c) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null corner"};
        // ConvexUnionGeometry::box (Geometry.cpp:14-37): same points and faces
        D3 p(c[0], c[1], c[2]);
        std::vector<D3> pts = {D3(p.x, p.y, p.z), D3(p.x + dx, p.y, p.z), D3(p.x + dx, p.y + dy, p.z), D3(p.x, p.y + dy, p.z),
                               D3(p.x, p.y, p.z + dz), D3(p.x + dx, p.y, p.z + dz), D3(p.x + dx, p.y + dy, p.z + dz), D3(p.x, p.y + dy, p.z + dz)};
        std::vector<std::vector<int>> faces = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
        uint32_t id = add_hull(w->w, pts, faces, m, movement, pos);
        if (out_id) *out_id = id;
        return CPGPU_OK;
    });
}

int cpgpu_body_sphere(cpgpu_world* w, const double center[3], double radius, const cpgpu_material* m, int movement,
                      const double pos[3], uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!center) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null center"};
        uint32_t id = add_prim(w->w, SHAPE_SPHERE, D3(center[0], center[1], center[2]), radius, 0, m, movement, pos);
        if (out_id) *out_id = id;
        return CPGPU_OK;
    });
}
// ConvexUnionGeometry::cylinder (Geometry.cpp:47-49): `base` is the centre of
// the bottom cap, the height axis is +y
int cpgpu_body_cylinder(cpgpu_world* w, const double base[3], double radius, double height, const cpgpu_material* m,
                        int movement, const double pos[3], uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!base) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null base"};
        D3 c(base[0], base[1] + height / 2.0, base[2]);
        uint32_t id = add_prim(w->w, SHAPE_CYLINDER, c, radius, height, m, movement, pos);
        if (out_id) *out_id = id;
        return CPGPU_OK;
    });
}
// ConvexUnionGeometry::capsule (Geometry.cpp:43-45): `bot` is the centre of the
// bottom cap sphere, the height axis is +y
int cpgpu_body_capsule(cpgpu_world* w, const double bot[3], double radius, double drum_height, const cpgpu_material* m,
                       int movement, const double pos[3], uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!bot) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null bot"};
        D3 c(bot[0], bot[1] + drum_height / 2.0, bot[2]);
        uint32_t id = add_prim(w->w, SHAPE_CAPSULE, c, radius, drum_height, m, movement, pos);
        if (out_id) *out_id = id;
        return CPGPU_OK;
    });
}
// recenterTensor (RigidBody.cpp:406-425): the parallel-axis shift of an
// inertia tensor from one reference point to another
static void recenter_tensor(double m, const double* t, D3 new_c, D3 old_origin, D3 true_com, double* o) {
    for (int k = 0; k < 9; k++) o[k] = t[k];
    const D3 d = new_c - old_origin, c = true_com - old_origin;
    o[0] += m * (d.y * d.y + d.z * d.z - 2 * d.y * c.y - 2 * d.z * c.z);
    o[1] += m * (d.x * c.y + d.y * c.x - d.x * d.y);
    o[2] += m * (d.x * c.z + d.z * c.x - d.x * d.z);
    o[4] += m * (d.x * d.x + d.z * d.z - 2 * d.x * c.x - 2 * d.z * c.z);
    o[5] += m * (d.y * c.z + d.z * c.y - d.y * d.z);
    o[8] += m * (d.x * d.x + d.y * d.y - 2 * d.x * c.x - 2 * d.y * c.y);
    o[3] = o[1];
    o[6] = o[2];
    o[7] = o[5];
}

// createRigidBody(ConvexUnionGeometry) (Geometry.cpp:540-550, RigidBody.cpp:
// 13-39, 427-640): one primitive is the single-primitive calls; several make
// a body whose mass, centre of mass and tensor are summed over the
// primitives in order (each primitive's tensor moved to the origin, the sum
// to the common centre of mass), each primitive packed about that centre
// with its own material
int cpgpu_body_union(cpgpu_world* w, const cpgpu_primitive* prims, int n, int movement, const double pos[3],
                     uint32_t* out_id) {
    W_OR_FAIL(w);
    if (!prims || n < 1) return fail(CPGPU_ERR_INVALID_ARG, "a union needs >= 1 primitive");
    if (n == 1) {
        const cpgpu_primitive& q = prims[0];
        switch (q.kind) {
        case CPGPU_PRIM_HULL:
            return cpgpu_body_hull(w, q.points, q.n_points, q.face_offsets, q.face_indices, q.n_faces, &q.mat, movement, pos, out_id);
        case CPGPU_PRIM_BOX: return cpgpu_body_box(w, q.p, q.a, q.b, q.c, &q.mat, movement, pos, out_id);
        case CPGPU_PRIM_SPHERE: return cpgpu_body_sphere(w, q.p, q.a, &q.mat, movement, pos, out_id);
        case CPGPU_PRIM_CYLINDER: return cpgpu_body_cylinder(w, q.p, q.a, q.b, &q.mat, movement, pos, out_id);
        case CPGPU_PRIM_CAPSULE: return cpgpu_body_capsule(w, q.p, q.a, q.b, &q.mat, movement, pos, out_id);
        default: return fail(CPGPU_ERR_INVALID_ARG, "bad primitive kind");
        }
    }
    return guarded([&] {
        if (n > 255) throw ApiFail{CPGPU_ERR_INVALID_ARG, "a union holds at most 255 primitives"};
        if (movement < 0 || movement > 2) throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad movement type"};
        struct Part { uint32_t kind; HullPrep h; D3 center; double r = 0, hh = 0, m = 0; D3 c; double t[9]; };
        std::vector<Part> parts(n);
        double msum = 0, tsum[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        D3 csum;
        for (int i = 0; i < n; i++) {
            const cpgpu_primitive& q = prims[i];
            Part& P = parts[i];
            const double density = q.mat.density;
            if (q.kind == CPGPU_PRIM_HULL || q.kind == CPGPU_PRIM_BOX) {
                std::vector<D3> pts;
                std::vector<std::vector<int>> faces;
                if (q.kind == CPGPU_PRIM_BOX) {
                    // ConvexUnionGeometry::box (Geometry.cpp:14-37)
                    const D3 p(q.p[0], q.p[1], q.p[2]);
                    const double dx = q.a, dy = q.b, dz = q.c;
                    pts = {D3(p.x, p.y, p.z), D3(p.x + dx, p.y, p.z), D3(p.x + dx, p.y + dy, p.z), D3(p.x, p.y + dy, p.z),
                           D3(p.x, p.y, p.z + dz), D3(p.x + dx, p.y, p.z + dz), D3(p.x + dx, p.y + dy, p.z + dz), D3(p.x, p.y + dy, p.z + dz)};
                    faces = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
                } else {
                    if (!q.points || !q.face_offsets || !q.face_indices || q.n_points < 4 || q.n_faces < 4)
                        throw ApiFail{CPGPU_ERR_INVALID_ARG, "hull needs >= 4 points and faces"};
                    for (int k = 0; k < q.n_points; k++) pts.push_back(D3(q.points[3 * k], q.points[3 * k + 1], q.points[3 * k + 2]));
                    faces.resize(q.n_faces);
                    for (int f = 0; f < q.n_faces; f++)
                        for (int k = q.face_offsets[f]; k < q.face_offsets[f + 1]; k++) faces[f].push_back(q.face_indices[k]);
                }
                if (!P.h.build(pts, faces)) throw ApiFail{CPGPU_ERR_INVALID_ARG, "invalid hull"};
                P.kind = SHAPE_HULL;
                double t[3][3];
                hullMassProperties(P.h, density, &P.c, t, &P.m);
                for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) P.t[3 * a + b] = t[a][b];
            } else {
                P.r = q.a;
                if (q.kind == CPGPU_PRIM_SPHERE) { P.kind = SHAPE_SPHERE; P.center = D3(q.p[0], q.p[1], q.p[2]); }
                else if (q.kind == CPGPU_PRIM_CYLINDER) { P.kind = SHAPE_CYLINDER; P.hh = q.b; P.center = D3(q.p[0], q.p[1] + q.b / 2.0, q.p[2]); }
                else if (q.kind == CPGPU_PRIM_CAPSULE) { P.kind = SHAPE_CAPSULE; P.hh = q.b; P.center = D3(q.p[0], q.p[1] + q.b / 2.0, q.p[2]); }
                else throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad primitive kind"};
                if (!(P.r > 0) || (P.kind == SHAPE_CYLINDER && !(P.hh > 0)) || (P.kind == SHAPE_CAPSULE && !(P.hh >= 0)))
                    throw ApiFail{CPGPU_ERR_INVALID_ARG, "radius must be > 0, cylinder height > 0, capsule drum height >= 0"};
                prim_mass(P.kind, P.center, P.r, P.hh, density, &P.m, P.t);
                P.c = P.center;
            }
            double t0[9];
            recenter_tensor(P.m, P.t, D3(), P.c, P.c, t0);
            for (int k = 0; k < 9; k++) tsum[k] = tsum[k] + t0[k];
            csum = csum + P.c * P.m;
            msum = msum + P.m;
        }
        const D3 com = csum / msum;
        Body b;
        b.mass = msum;
        recenter_tensor(msum, tsum, com, D3(), com, b.iref);
        inv3(b.iref, b.iinv_ref);
        std::memcpy(b.iw, b.iref, sizeof(b.iw));
        std::memcpy(b.iinv, b.iinv_ref, sizeof(b.iinv));
        b.com = com;
        b.local_origin = -b.com;
        D3 p = pos ? D3(pos[0], pos[1], pos[2]) : D3();
        D3 tracked = b.com + qrot(b.q, b.local_origin);
        b.com = b.com + (p - tracked);
        b.movement = movement;
        b.rest = prims[0].mat.restitution; b.kin = prims[0].mat.kinetic_friction; b.sta = prims[0].mat.static_friction;
        begin_mutation(w->w);
        for (int i = 0; i < n; i++) {
            const Part& P = parts[i];
            Shape sh = P.kind == SHAPE_HULL ? pack_hull(P.h, com)
                       : P.kind == SHAPE_SPHERE ? pack_sphere(P.center - com, P.r)
                       : P.kind == SHAPE_CAPSULE ? pack_capsule(P.center - com, P.r, P.hh)
                                                 : pack_cylinder(P.center - com, P.r, P.hh);
            b.prims.push_back((int)w->w.shapes.size());
            w->w.shapes.push_back(std::move(sh));
            b.prim_mat.push_back({prims[i].mat.restitution, prims[i].mat.kinetic_friction, prims[i].mat.static_friction});
        }
        b.shape = b.prims[0];
        w->w.bodies.push_back(b);
        uint32_t id = (uint32_t)w->w.bodies.size();
        w->w.nodes[id] = (int)id - 1;
        if (out_id) *out_id = id;
        return CPGPU_OK;
    });
}
// createRigidBody(StaticMeshGeometry(MeshInput{tris, points}), fixed)
// (PhysicsEngine.cpp:498-512, RigidBody.cpp:41-58): a fixed body at the
// origin whose triangles are in world coordinates
int cpgpu_body_mesh(cpgpu_world* w, const double* points, int n_points, const int* tris, int n_tris, const cpgpu_material* m,
                    int fixed, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!fixed) throw ApiFail{CPGPU_ERR_UNSUPPORTED, "kinematic meshes are not implemented on the device path"};
        if (!points || !tris || n_points < 3 || n_tris < 1) throw ApiFail{CPGPU_ERR_INVALID_ARG, "mesh needs >= 3 points and >= 1 triangle"};
        // a contact carries the triangle id in 24 bits (a union primitive's index above it)
        if (n_tris >= (1 << 24)) throw ApiFail{CPGPU_ERR_INVALID_ARG, "a mesh holds fewer than 16,777,216 triangles"};
        std::vector<D3> pts(n_points);
        for (int i = 0; i < n_points; i++) pts[i] = D3(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
        std::vector<std::array<int, 3>> t(n_tris);
        for (int i = 0; i < n_tris; i++)
            for (int k = 0; k < 3; k++) {
                int x = tris[3 * i + k];
                if (x < 0 || x >= n_points) throw ApiFail{CPGPU_ERR_INVALID_ARG, "mesh index out of range"};
                t[i][k] = x;
            }
        D3 lo, hi;
        Shape sh = pack_mesh(pts, t, &lo, &hi);
        Body b;
        b.movement = CPGPU_FIXED;
        b.mass = std::numeric_limits<double>::quiet_NaN();
        for (int k = 0; k < 9; k++) { b.iref[k] = 0; b.iinv_ref[k] = 0; b.iw[k] = 0; b.iinv[k] = 0; }
        b.local_origin = D3();
        if (m) { b.rest = m->restitution; b.kin = m->kinetic_friction; b.sta = m->static_friction; }
        begin_mutation(w->w);
        b.shape = (int)w->w.shapes.size();
        w->w.shapes.push_back(std::move(sh));
        w->w.bodies.push_back(b);
        uint32_t id = (uint32_t)w->w.bodies.size();
        w->w.nodes[id] = (int)id - 1;
        if (out_id) *out_id = id;
        return CPGPU_OK;
    });
}

int cpgpu_body_set_velocity(cpgpu_world* w, uint32_t id, const double v[3]) {
    W_OR_FAIL(w);
    return guarded([&] {
        begin_mutation(w->w);
        Body& b = body_ref(w->w, id);
        b.vel = D3(v[0], v[1], v[2]);
        b.alert_waking();
        return CPGPU_OK;
    });
}
int cpgpu_body_set_ang_velocity(cpgpu_world* w, uint32_t id, const double v[3]) {
    W_OR_FAIL(w);
    return guarded([&] {
        begin_mutation(w->w);
        Body& b = body_ref(w->w, id);
        b.angv = D3(v[0], v[1], v[2]);
        b.alert_waking();
        return CPGPU_OK;
    });
}
// RigidBody::setOrientation (RigidBody.cpp:103-107): the orientation is set and
// normalised by updateGeometry; the world inertia tensor keeps its value until
// the next integration updates it.
int cpgpu_body_set_orientation(cpgpu_world* w, uint32_t id, const double q[4]) {
    W_OR_FAIL(w);
    return guarded([&] {
        begin_mutation(w->w);
        Body& b = body_ref(w->w, id);
        b.q = qnorm(Quat{q[0], q[1], q[2], q[3]});
        b.fresh = 1;
        b.alert_waking();
        return CPGPU_OK;
    });
}
int cpgpu_body_set_position(cpgpu_world* w, uint32_t id, const double p[3]) {
    W_OR_FAIL(w);
    return guarded([&] {
        begin_mutation(w->w);
        Body& b = body_ref(w->w, id);
        D3 tracked = b.com + qrot(b.q, b.local_origin);
        b.com = b.com + (D3(p[0], p[1], p[2]) - tracked);
        b.q = qnorm(b.q);
        b.fresh = 1;
        b.alert_waking();
        return CPGPU_OK;
    });
}
int cpgpu_body_set_mass(cpgpu_world* w, uint32_t id, double mass) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!(mass > 0)) throw ApiFail{CPGPU_ERR_INVALID_ARG, "mass must be positive"};
        begin_mutation(w->w);
        Body& b = body_ref(w->w, id);
        double r = mass / b.mass;
        for (int k = 0; k < 9; k++) { b.iref[k] *= r; b.iinv_ref[k] /= r; b.iw[k] *= r; b.iinv[k] /= r; }
        b.mass = mass;
        return CPGPU_OK;
    });
}

// PhysicsEngine::add*Constraint (PhysicsEngine.cpp:623-972): anchors in each
// body's model coordinates become tracked points (RigidBody::trackPoint,
// RigidBody.cpp:134-137); hinge, slider and sliding-hinge axes are
// normalised (cone and twist directions are taken as given); the two bodies
// stop colliding with each other.
static HJoint& add_joint(World& w, int kind, int n, uint32_t b1, uint32_t b2, const double* a1, const double* a2,
                         const double* ax1, const double* ax2, double ph, double rh) {
    const bool need_anchor = !jk_limit(kind);
    const bool need_axis = kind == JK_HINGE || kind == JK_SLIDER || kind == JK_SLIDING_HINGE || jk_limit(kind);
    if ((need_anchor && (!a1 || !a2)) || (need_axis && (!ax1 || !ax2))) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null anchor or axis"};
    if (b1 == b2) throw ApiFail{CPGPU_ERR_INVALID_ARG, "a joint needs two different bodies"};
    Body& x = body_ref(w, b1);
    Body& y = body_ref(w, b2);
    begin_mutation(w);
    HJoint j;
    j.b1 = (int)b1 - 1; j.b2 = (int)b2 - 1; j.n = n; j.kind = kind;
    j.seq = w.constraint_seq++;
    if (need_anchor) {
        j.p1 = x.local_origin + D3(a1[0], a1[1], a1[2]);
        j.p2 = y.local_origin + D3(a2[0], a2[1], a2[2]);
    }
    if (need_axis) {
        j.ax1 = D3(ax1[0], ax1[1], ax1[2]);
        j.ax2 = D3(ax2[0], ax2[1], ax2[2]);
        if (!jk_limit(kind)) { j.ax1 = j.ax1.normalize(); j.ax2 = j.ax2.normalize(); }
    }
    j.ph = ph; j.rh = rh;
    w.joints.push_back(j);
    return w.joints.back();
}

// the id of the constraint just created: PhysicsEngine::nextConstraintID
// order over joints and springs, from 0 (PhysicsEngine.h:301)
static uint32_t joint_id(const World& w) { return (uint32_t)(w.constraint_seq - 1); }

int cpgpu_add_ball_socket(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double strength,
                          uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        add_joint(w->w, JK_BALL, 3, b1, b2, a1, a2, nullptr, nullptr, strength, 0);
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}
int cpgpu_add_distance(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double target,
                       double strength, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        HJoint& j = add_joint(w->w, JK_DISTANCE, 1, b1, b2, a1, a2, nullptr, nullptr, strength, 0);
        // -1: the attachment points' distance now (PhysicsEngine.cpp:630-635)
        if (target == -1) {
            const Body &x = w->w.bodies[j.b1], &y = w->w.bodies[j.b2];
            target = ((x.com + qrot(x.q, j.p1)) - (y.com + qrot(y.q, j.p2))).mag();
        }
        j.target = target;
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}
int cpgpu_add_weld(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double ps, double rs,
                   uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        add_joint(w->w, JK_WELD, 6, b1, b2, a1, a2, nullptr, nullptr, ps, rs);
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}
int cpgpu_add_twist_limit(cpgpu_world* w, uint32_t b1, uint32_t b2, const double ax1[3], const double ax2[3], double min_angle,
                          double max_angle, double rs, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        HJoint& j = add_joint(w->w, JK_TWIST, 1, b1, b2, nullptr, nullptr, ax1, ax2, 0, rs);
        j.min_angle = min_angle;
        j.max_angle = max_angle;
        // TwistLimit constructor (PersistentConstraint.h:177-184): body 1's
        // perpendicular basis of its twist axis, w first
        j.ax1.basis(&j.wl, &j.ul);
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}
int cpgpu_add_cone_limit(cpgpu_world* w, uint32_t b1, uint32_t b2, const double ax1[3], const double ax2[3], double max_angle,
                         double rs, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        HJoint& j = add_joint(w->w, JK_CONE, 1, b1, b2, nullptr, nullptr, ax1, ax2, 0, rs);
        j.max_angle = max_angle;
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}
int cpgpu_add_spring(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], double damping,
                     double stiffness, double rest, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!a1 || !a2) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null anchor"};
        if (b1 == b2) throw ApiFail{CPGPU_ERR_INVALID_ARG, "a spring needs two different bodies"};
        Body& x = body_ref(w->w, b1);
        Body& y = body_ref(w->w, b2);
        begin_mutation(w->w);
        HSpring sp;
        sp.b1 = (int)b1 - 1; sp.b2 = (int)b2 - 1;
        sp.seq = w->w.constraint_seq++;
        sp.p1 = x.local_origin + D3(a1[0], a1[1], a1[2]);
        sp.p2 = y.local_origin + D3(a2[0], a2[1], a2[2]);
        // a negative resting length: the attachment points' distance now
        if (rest < 0) rest = ((x.com + qrot(x.q, sp.p1)) - (y.com + qrot(y.q, sp.p2))).mag();
        sp.damping = damping; sp.stiffness = stiffness; sp.rest = rest;
        w->w.springs.push_back(sp);
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}
int cpgpu_add_slider(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], const double ax1[3],
                     const double ax2[3], double ps, double rs, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        add_joint(w->w, JK_SLIDER, 5, b1, b2, a1, a2, ax1, ax2, ps, rs);
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}
int cpgpu_add_sliding_hinge(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3],
                            const double ax1[3], const double ax2[3], double ps, double rs, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        add_joint(w->w, JK_SLIDING_HINGE, 4, b1, b2, a1, a2, ax1, ax2, ps, rs);
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}
int cpgpu_add_hinge(cpgpu_world* w, uint32_t b1, uint32_t b2, const double a1[3], const double a2[3], const double ax1[3],
                    const double ax2[3], double ps, double rs, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        add_joint(w->w, JK_HINGE, 5, b1, b2, a1, a2, ax1, ax2, ps, rs);
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}

// The joint a constraint id names (ids count joints and springs in creation
// order from 0; a piston's two joints share its id, the powered one last)
static HJoint* joint_by_id(World& w, uint32_t id) {
    HJoint* found = nullptr;
    for (HJoint& j : w.joints)
        if ((uint32_t)j.seq == id) found = &j;
    return found;
}

// PhysicsEngine::addMotorConstraint (PhysicsEngine.cpp:725-763) and the Motor
// constructor (PersistentConstraint.cpp:5-24): on a hinge's or sliding
// hinge's axes and rotation strength, in the base's edge; the reference
// frame (body 1's perpendicular basis of its axis, body 2's first
// perpendicular axis) fixed at creation, the angle measured from it
int cpgpu_add_motor(cpgpu_world* w, uint32_t base, double min_angle, double max_angle, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        HJoint* b = joint_by_id(w->w, base);
        if (!b || (b->kind != JK_HINGE && b->kind != JK_SLIDING_HINGE))
            throw ApiFail{CPGPU_ERR_INVALID_ARG, "a motor needs a hinge or a sliding hinge"};
        const HJoint base_j = *b;
        begin_mutation(w->w);
        HJoint j;
        j.b1 = base_j.b1; j.b2 = base_j.b2; j.kind = JK_MOTOR; j.n = 1;
        j.seq = w->w.constraint_seq++;
        j.ax1 = base_j.ax1;
        j.rh = base_j.rh;
        j.min_angle = min_angle; j.max_angle = max_angle;
        D3 u2, tmp;
        base_j.ax1.basis(&j.ul, &j.wl);
        base_j.ax2.basis(&u2, &tmp);
        j.ax2 = u2;
        // Motor::calculatePosition from zero with no velocity: the angle of
        // body 2's comparison axis in body 1's frame now
        const Body &x = w->w.bodies[j.b1], &y = w->w.bodies[j.b2];
        const D3 axis = qrot(x.q, j.ax1), ref_u = qrot(x.q, j.ul), ref_w = qrot(x.q, j.wl), cmp = qrot(y.q, j.ax2);
        double pos = 0;
        if (!(std::fabs(cmp.dot(axis)) > 0.999)) {
            const D3 cn = (cmp - axis * axis.dot(cmp)).normalize();
            const double kPi = 3.1415926535;
            double rel = 2 * kPi - std::acos(std::min(1.0, std::max(-1.0, cn.dot(ref_u))));
            if (cn.dot(ref_w) < 0) rel = 2 * kPi - rel;
            double closest = INFINITY;
            for (double c : {rel - 2 * kPi, rel, rel + 2 * kPi})
                if (std::fabs(c) < std::fabs(closest)) closest = c;
            pos = closest;
        }
        j.angle = (float)pos;
        w->w.joints.push_back(j);
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}

// PhysicsEngine::addPistonConstraint (PhysicsEngine.cpp:808-852) and the
// Piston constructor (PersistentConstraint.cpp:134-143): on a slider's or
// sliding hinge's tracked points, body 1 axis and position strength, in the
// base's edge, as two joints (its slide limit, then the powered row) under
// one id.  The position before the first step is measured between the two
// tracked points (the reference's constructor reads body 2's point key on
// body 1; every rebuild measures it between the bodies)
int cpgpu_add_piston(cpgpu_world* w, uint32_t base, double min_pos, double max_pos, uint32_t* out_id) {
    W_OR_FAIL(w);
    return guarded([&] {
        HJoint* b = joint_by_id(w->w, base);
        if (!b || (b->kind != JK_SLIDER && b->kind != JK_SLIDING_HINGE))
            throw ApiFail{CPGPU_ERR_INVALID_ARG, "a piston needs a slider or a sliding hinge"};
        const HJoint base_j = *b;
        begin_mutation(w->w);
        const int seq = w->w.constraint_seq++;
        const Body &x = w->w.bodies[base_j.b1], &y = w->w.bodies[base_j.b2];
        const D3 axis = qrot(x.q, base_j.ax1);
        const double pos = (y.com + qrot(y.q, base_j.p2)).dot(axis) - (x.com + qrot(x.q, base_j.p1)).dot(axis);
        for (int kind : {JK_SLIDE_LIMIT, JK_PISTON}) {
            HJoint j;
            j.b1 = base_j.b1; j.b2 = base_j.b2; j.kind = kind; j.n = 1;
            j.seq = seq;
            j.p1 = base_j.p1; j.p2 = base_j.p2;
            j.ax1 = base_j.ax1;
            j.ph = base_j.ph;
            j.min_angle = min_pos; j.max_angle = max_pos;
            j.angle = (float)pos;
            w->w.joints.push_back(j);
        }
        if (out_id) *out_id = joint_id(w->w);
        return CPGPU_OK;
    });
}

// setMotorOff / setMotorConstantTorque / setMotorTargetVelocity /
// setMotorTargetPosition (PhysicsEngine.cpp:1857-1912) and the piston's
// setters (:1800-1855): each sets the fields the reference's setter sets and
// alerts both bodies
static int set_powered(cpgpu_world* w, uint32_t id, int kind, int mode, double max, double target) {
    W_OR_FAIL(w);
    return guarded([&] {
        HJoint* j = joint_by_id(w->w, id);
        if (!j || j->kind != kind) throw ApiFail{CPGPU_ERR_INVALID_ARG, kind == JK_MOTOR ? "not a motor" : "not a piston"};
        if (mode < 0 || mode > 3) throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad mode"};
        begin_mutation(w->w);
        j = joint_by_id(w->w, id);
        j->mode = mode;
        if (mode >= 1) j->pmax = max;
        if (mode == 2) j->tvel = target;
        if (mode == 3) j->tpos = target;
        w->w.bodies[j->b1].alert_waking();
        w->w.bodies[j->b2].alert_waking();
        return CPGPU_OK;
    });
}
int cpgpu_set_motor(cpgpu_world* w, uint32_t id, int mode, double max_torque, double target) {
    return set_powered(w, id, JK_MOTOR, mode, max_torque, target);
}
int cpgpu_set_piston(cpgpu_world* w, uint32_t id, int mode, double max_force, double target) {
    return set_powered(w, id, JK_PISTON, mode, max_force, target);
}
// getMotorAngularPosition / getPistonPosition (PhysicsEngine.cpp:1914-1930)
static int get_powered(cpgpu_world* w, uint32_t id, int kind, double* out) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!out) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null output"};
        if (w->w.dev && w->w.dev_valid) download_state(w->w);
        HJoint* j = joint_by_id(w->w, id);
        if (!j || j->kind != kind) throw ApiFail{CPGPU_ERR_INVALID_ARG, kind == JK_MOTOR ? "not a motor" : "not a piston"};
        *out = j->angle;
        return CPGPU_OK;
    });
}
int cpgpu_get_motor_position(cpgpu_world* w, uint32_t id, double* out) { return get_powered(w, id, JK_MOTOR, out); }
int cpgpu_get_piston_position(cpgpu_world* w, uint32_t id, double* out) { return get_powered(w, id, JK_PISTON, out); }

int cpgpu_step(cpgpu_world* w, int n_steps) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (n_steps < 0) throw ApiFail{CPGPU_ERR_INVALID_ARG, "negative step count"};
        if (w->w.bodies.empty()) return CPGPU_OK;
        ensure_device(w->w);
        w->w.dev->set_audit(w->w.audit);
        w->w.dev->step(n_steps);
        return w->w.dev->check_status();
    });
}

int cpgpu_world_set_audit(cpgpu_world* w, int enabled) {
    W_OR_FAIL(w);
    return guarded([&] {
        w->w.audit = enabled != 0;
        if (w->w.dev && w->w.dev_valid) w->w.dev->set_audit(w->w.audit);
        return CPGPU_OK;
    });
}

int cpgpu_world_read_audit(cpgpu_world* w, double* out) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!out) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null output"};
        if (!w->w.audit) throw ApiFail{CPGPU_ERR_INVALID_ARG, "the audit is not enabled"};
        if (!(w->w.dev && w->w.dev_valid)) {
            // not stepped since the audit was enabled (or since a rebuild)
            for (int k = 0; k < kAuditValues; k++) out[k] = 0.0;
            return CPGPU_OK;
        }
        w->w.dev->set_audit(true);
        w->w.dev->read_audit(out);
        return CPGPU_OK;
    });
}

// PhysicsEngine::raycastFirstIntersection (PhysicsEngine.cpp:582-609), one
// device thread per ray against the world's current geometry
int cpgpu_raycast(cpgpu_world* w, const double* origins, const double* dirs, int n_rays, const uint32_t* ignore,
                  int n_ignore, uint32_t* hit_body, double* hit_pos, double* hit_normal, double* hit_dist) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (n_rays < 0 || n_ignore < 0 || (n_rays > 0 && (!origins || !dirs)) || (n_ignore > 0 && !ignore))
            throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad ray arguments"};
        std::vector<float> out(8 * (size_t)n_rays, 0.f);
        for (int k = 0; k < n_rays; k++) out[8 * (size_t)k + 7] = -1.f;
        if (n_rays > 0 && !w->w.bodies.empty()) {
            ensure_device(w->w);
            Batch& B = *w->w.dev;
            std::vector<float> rays(6 * (size_t)n_rays);
            for (size_t i = 0; i < 3 * (size_t)n_rays; i++) {
                const size_t k = i / 3, c = i % 3;
                rays[6 * k + c] = (float)origins[i];
                rays[6 * k + 3 + c] = (float)dirs[i];
            }
            float *d_rays = nullptr, *d_out = nullptr;
            uint32_t* d_ig = nullptr;
            CK(cudaMalloc(&d_rays, sizeof(float) * rays.size()));
            CK(cudaMalloc(&d_out, sizeof(float) * out.size()));
            CK(cudaMalloc(&d_ig, sizeof(uint32_t) * std::max(n_ignore, 1)));
            CK(cudaMemcpyAsync(d_rays, rays.data(), sizeof(float) * rays.size(), cudaMemcpyHostToDevice, B.st));
            if (n_ignore > 0) CK(cudaMemcpyAsync(d_ig, ignore, sizeof(uint32_t) * n_ignore, cudaMemcpyHostToDevice, B.st));
            launch_raycast(B.cur(), 0, (int)w->w.bodies.size(), d_rays, n_rays, d_ig, n_ignore, d_out, B.st);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(out.data(), d_out, sizeof(float) * out.size(), cudaMemcpyDeviceToHost, B.st));
            CK(cudaStreamSynchronize(B.st));
            cudaFree(d_rays);
            cudaFree(d_out);
            cudaFree(d_ig);
        }
        for (int k = 0; k < n_rays; k++) {
            const float* r = &out[8 * (size_t)k];
            uint32_t id;
            std::memcpy(&id, &r[0], 4);
            if (hit_body) hit_body[k] = id;
            for (int c = 0; c < 3; c++) {
                if (hit_pos) hit_pos[3 * k + c] = r[1 + c];
                if (hit_normal) hit_normal[3 * k + c] = r[4 + c];
            }
            if (hit_dist) hit_dist[k] = r[7];
        }
        return CPGPU_OK;
    });
}

int cpgpu_num_bodies(cpgpu_world* w, int* n) {
    W_OR_FAIL(w);
    *n = (int)w->w.bodies.size();
    return CPGPU_OK;
}

int cpgpu_get_body_state(cpgpu_world* w, double* com, double* quat, double* vel, double* ang) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (w->w.dev && w->w.dev_valid) download_state(w->w);
        for (size_t i = 0; i < w->w.bodies.size(); i++) {
            const Body& b = w->w.bodies[i];
            D3 v = b.movement == CPGPU_FIXED ? D3() : b.vel, a = b.movement == CPGPU_FIXED ? D3() : b.angv;
            if (com) { com[3 * i] = b.com.x; com[3 * i + 1] = b.com.y; com[3 * i + 2] = b.com.z; }
            if (quat) { quat[4 * i] = b.q.r; quat[4 * i + 1] = b.q.i; quat[4 * i + 2] = b.q.j; quat[4 * i + 3] = b.q.k; }
            if (vel) { vel[3 * i] = v.x; vel[3 * i + 1] = v.y; vel[3 * i + 2] = v.z; }
            if (ang) { ang[3 * i] = a.x; ang[3 * i + 1] = a.y; ang[3 * i + 2] = a.z; }
        }
        return CPGPU_OK;
    });
}

int cpgpu_get_asleep(cpgpu_world* w, int* flags) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!flags) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null output"};
        if (w->w.dev && w->w.dev_valid) download_state(w->w);
        for (size_t i = 0; i < w->w.bodies.size(); i++) {
            const Body& b = w->w.bodies[i];
            flags[i] = (b.asleep && b.movement == CPGPU_DYNAMIC) ? 1 : 0;
        }
        return CPGPU_OK;
    });
}

// Checkpoint restore of the dynamic state: poses and velocities are replaced
// and the world inertia tensors recomputed from the new orientations.
int cpgpu_set_body_state(cpgpu_world* w, const double* com, const double* quat, const double* vel, const double* ang) {
    W_OR_FAIL(w);
    return guarded([&] {
        begin_mutation(w->w);
        for (size_t i = 0; i < w->w.bodies.size(); i++) {
            Body& b = w->w.bodies[i];
            if (com) b.com = D3(com[3 * i], com[3 * i + 1], com[3 * i + 2]);
            if (quat) b.q = qnorm(Quat{quat[4 * i], quat[4 * i + 1], quat[4 * i + 2], quat[4 * i + 3]});
            if (com || quat) b.fresh = 1;
            if (vel) b.vel = D3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
            if (ang) b.angv = D3(ang[3 * i], ang[3 * i + 1], ang[3 * i + 2]);
            if (b.movement == CPGPU_DYNAMIC) {
                // I_world = R I_ref R^T (RigidBody::updateInertiaTensor)
                double R[9];
                const Quat& q = b.q;
                double r = q.r, ii = q.i, j = q.j, k = q.k;
                R[0] = r * r + ii * ii - j * j - k * k; R[1] = 2 * ii * j - 2 * r * k; R[2] = 2 * ii * k + 2 * r * j;
                R[3] = 2 * ii * j + 2 * r * k; R[4] = r * r - ii * ii + j * j - k * k; R[5] = 2 * j * k - 2 * r * ii;
                R[6] = 2 * ii * k - 2 * r * j; R[7] = 2 * j * k + 2 * r * ii; R[8] = r * r - ii * ii - j * j + k * k;
                for (int which = 0; which < 2; which++) {
                    const double* I = which ? b.iinv_ref : b.iref;
                    double* out = which ? b.iinv : b.iw;
                    double T[9];
                    for (int a = 0; a < 3; a++) for (int c = 0; c < 3; c++) { double s = 0; for (int m = 0; m < 3; m++) s += R[3 * a + m] * I[3 * m + c]; T[3 * a + c] = s; }
                    for (int a = 0; a < 3; a++) for (int c = 0; c < 3; c++) { double s = 0; for (int m = 0; m < 3; m++) s += T[3 * a + m] * R[3 * c + m]; out[3 * a + c] = s; }
                }
            }
        }
        return CPGPU_OK;
    });
}

int cpgpu_get_aabbs(cpgpu_world* w, double* out) {
    W_OR_FAIL(w);
    return guarded([&] {
        ensure_device(w->w);
        Batch& B = *w->w.dev;
        int N = B.n_bodies;
        std::vector<float4> lo(N), hi(N);
        CK(cudaMemcpyAsync(lo.data(), B.cur().aabb_lo, N * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(hi.data(), B.cur().aabb_hi, N * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaStreamSynchronize(B.st));
        for (int i = 0; i < N; i++) {
            double* o = out + 6 * i;
            o[0] = lo[i].x; o[1] = lo[i].y; o[2] = lo[i].z; o[3] = hi[i].x; o[4] = hi[i].y; o[5] = hi[i].z;
        }
        return CPGPU_OK;
    });
}

int cpgpu_get_pairs(cpgpu_world* w, uint32_t* pairs, int cap, int* n) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (w->w.dev && w->w.dev_valid) download_state(w->w);
        int np = (int)(w->w.last_pairs.size() / 2);
        *n = np;
        for (int i = 0; i < np && i < cap; i++) { pairs[2 * i] = w->w.last_pairs[2 * i]; pairs[2 * i + 1] = w->w.last_pairs[2 * i + 1]; }
        return CPGPU_OK;
    });
}

int cpgpu_get_contacts(cpgpu_world* w, cpgpu_contact* out, int cap, int* n) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (w->w.dev && w->w.dev_valid) download_state(w->w);
        *n = (int)w->w.contacts.size();
        if (out) for (int i = 0; i < *n && i < cap; i++) out[i] = w->w.contacts[i];
        return CPGPU_OK;
    });
}

int cpgpu_set_contacts(cpgpu_world* w, const cpgpu_contact* in, int n) {
    W_OR_FAIL(w);
    return guarded([&] {
        begin_mutation(w->w);
        std::vector<cpgpu_contact> cs(in, in + n);
        for (const cpgpu_contact& c : cs)
            if (c.b1 == 0 || c.b2 == 0 || c.b1 >= c.b2 || c.b2 > w->w.bodies.size())
                throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad contact body ids"};
        std::stable_sort(cs.begin(), cs.end(), [](const cpgpu_contact& a, const cpgpu_contact& b) {
            return a.b1 != b.b1 ? a.b1 < b.b1 : a.b2 < b.b2;
        });
        w->w.contacts = cs;
        return CPGPU_OK;
    });
}

int cpgpu_get_joint_state(cpgpu_world* w, double* impulse, double* u, double* wv, double* aux, int* n) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (!n) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null count"};
        if (w->w.dev && w->w.dev_valid) download_state(w->w);
        *n = (int)w->w.joints.size();
        for (size_t j = 0; j < w->w.joints.size(); j++) {
            const HJoint& x = w->w.joints[j];
            for (int k = 0; k < kJMax; k++) if (impulse) impulse[kJMax * j + k] = x.impulse[k];
            for (int k = 0; k < 3; k++) { if (u) u[3 * j + k] = x.u[k]; if (wv) wv[3 * j + k] = x.w[k]; }
            if (aux) { aux[2 * j] = x.angle; aux[2 * j + 1] = jk_powered(x.kind) ? (double)x.aux : (double)x.active; }
        }
        return CPGPU_OK;
    });
}

int cpgpu_set_joint_state(cpgpu_world* w, const double* impulse, const double* u, const double* wv, const double* aux, int n) {
    W_OR_FAIL(w);
    return guarded([&] {
        if (n != (int)w->w.joints.size()) throw ApiFail{CPGPU_ERR_INVALID_ARG, "joint count mismatch"};
        begin_mutation(w->w);
        for (int j = 0; j < n; j++) {
            HJoint& x = w->w.joints[j];
            for (int k = 0; k < kJMax; k++) if (impulse) x.impulse[k] = (float)impulse[kJMax * j + k];
            for (int k = 0; k < 3; k++) { if (u) x.u[k] = (float)u[3 * j + k]; if (wv) x.w[k] = (float)wv[3 * j + k]; }
            if (aux) {
                x.angle = (float)aux[2 * j];
                if (jk_powered(x.kind)) x.aux = (float)aux[2 * j + 1];
                else x.active = aux[2 * j + 1] != 0.0 ? 1 : 0;
            }
        }
        return CPGPU_OK;
    });
}

// ---------------------------------------------------------------- batch schedule ----

// The hand-set schedule: a large batch of very unequal worlds (at least 512
// worlds, the largest at least 4 times the median) gets two parts, the
// largest worlds holding 20 % of the bodies and the rest, the later part at
// most 2 chain workers per SM (the parts' solver kernels share the SMs'
// shared memory; measured on 4,096 worlds of 8-512 bodies: 23.7 -> 21.3 ms
// per step with the parts, 21.5 -> 20.3 ms with the cap); otherwise one
// part.  CPGPU_BATCH_PARTS, CPGPU_BATCH_FIRST_SHARE (percent),
// CPGPU_BATCH_SECOND_SHARE (percent, three or more parts),
// CPGPU_PGS_REST_PER_SM, CPGPU_PGS_MID_PER_SM (the second part's chain
// workers per SM, three or more parts) and CPGPU_PGS_BIG_ROWS (the island
// rows from which an island takes the warp-per-island solver) override it.
static std::vector<int> size_order(const std::vector<World*>& ws) {
    std::vector<int> order(ws.size());
    for (size_t i = 0; i < ws.size(); i++) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ws[a]->bodies.size() > ws[b]->bodies.size(); });
    return order;
}

static Schedule default_schedule(const std::vector<World*>& ws) {
    const int n = (int)ws.size();
    const std::vector<int> order = size_order(ws);
    const bool skewed = n >= 512 && ws[order[0]]->bodies.size() >= 4 * ws[order[n / 2]]->bodies.size();
    Schedule S;
    S.parts = std::max(1, std::min(env_int("CPGPU_BATCH_PARTS", skewed ? 2 : 1), n));
    const int first_dflt = (skewed && S.parts == 2) ? 20 : 100 / S.parts;
    S.first_share = S.parts > 1 ? std::max(1, std::min(99, env_int("CPGPU_BATCH_FIRST_SHARE", first_dflt))) : 100;
    S.rest_per_sm = S.parts > 1 ? env_int("CPGPU_PGS_REST_PER_SM", 2) : 0;
    S.big_rows = std::max(1, env_int("CPGPU_PGS_BIG_ROWS", kDefaultBigRows));
    if (S.parts > 2) {
        S.second_share = std::max(0, std::min(99 - S.first_share, env_int("CPGPU_BATCH_SECOND_SHARE", 0)));
        S.mid_per_sm = env_int("CPGPU_PGS_MID_PER_SM", -1);
    }
    return S;
}

// Worlds sorted by body count (largest first) and cut into S.parts runs:
// the first holds S.first_share percent of the bodies, the others split the
// rest evenly.
static std::vector<std::vector<int>> batch_partition(const std::vector<World*>& ws, const Schedule& S) {
    const int n = (int)ws.size();
    const std::vector<int> order = size_order(ws);
    const int P = std::max(1, std::min(S.parts, n));
    int64_t total = 0;
    for (World* w : ws) total += (int64_t)w->bodies.size();
    const int first = S.first_share;
    const int second = P > 2 ? S.second_share : 0;
    auto bound = [&](int q) {
        if (P == 1) return total;
        if (second > 0 && q >= 1)   // the first two parts by their shares, the later ones split the rest
            return total * ((first + second) * (P - 2) + (100 - first - second) * (q - 1)) / (100 * (P - 2));
        return total * (first * (P - 1) + (100 - first) * q) / (100 * (P - 1));
    };
    std::vector<std::vector<int>> parts(P);
    int64_t acc = 0;
    int p = 0;
    for (int k = 0; k < n; k++) {
        const int left = n - k;
        // move on once this part holds its share, keeping one world for each later part
        if (p + 1 < P && !parts[p].empty() && (acc >= bound(p) || left <= P - 1 - p)) p++;
        parts[p].push_back(order[k]);
        acc += (int64_t)ws[order[k]]->bodies.size();
    }
    for (auto& q : parts) std::sort(q.begin(), q.end());   // batch order within a part
    parts.erase(std::remove_if(parts.begin(), parts.end(), [](const std::vector<int>& q) { return q.empty(); }), parts.end());
    return parts;
}

// Autotuner cache: schedules chosen by timing, keyed on the batch's
// world-size histogram (log2 bins of the body counts, each bin's share of
// the worlds in sixteenths, and log2 of the world count), kept for the
// process and, when CPGPU_TUNE_FILE names one, in that file.
static std::string histogram_key(const std::vector<World*>& ws) {
    int bins[24] = {0};
    for (World* w : ws) {
        int b = 0;
        for (size_t x = w->bodies.size(); x > 1 && b < 23; x >>= 1) b++;
        bins[b]++;
    }
    int lw = 0;
    for (size_t x = ws.size(); x > 1; x >>= 1) lw++;
    std::string key = "w" + std::to_string(lw) + ":";
    for (int b = 0; b < 24; b++) {
        const int q = (int)((16LL * bins[b] + (int64_t)ws.size() / 2) / (int64_t)ws.size());
        key += std::to_string(q) + (b + 1 < 24 ? "," : "");
    }
    return key;
}

static std::mutex g_tune_mutex;
static std::map<std::string, Schedule> g_tuned;
static bool g_tune_file_loaded = false;

static void tune_file_load() {
    if (g_tune_file_loaded) return;
    g_tune_file_loaded = true;
    const char* path = std::getenv("CPGPU_TUNE_FILE");
    if (!path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    char key[256];
    Schedule S;
    while (std::fscanf(f, "%255s %d %d %d %d %d %d", key, &S.parts, &S.first_share, &S.rest_per_sm, &S.big_rows,
                       &S.second_share, &S.mid_per_sm) == 7)
        g_tuned[key] = S;
    std::fclose(f);
}

static void tune_file_save(const std::string& key, const Schedule& S) {
    const char* path = std::getenv("CPGPU_TUNE_FILE");
    if (!path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s %d %d %d %d %d %d\n", key.c_str(), S.parts, S.first_share, S.rest_per_sm, S.big_rows, S.second_share,
                 S.mid_per_sm);
    std::fclose(f);
}

// The batch object: parts built for a schedule
static std::unique_ptr<cpgpu_batch> make_batch(const std::vector<World*>& ws, const Schedule& S) {
    const int n = (int)ws.size();
    auto b = std::make_unique<cpgpu_batch>();
    b->sched = S;
    b->stagger = env_int("CPGPU_BATCH_STAGGER", 1) != 0;
    b->worlds = ws;
    b->part_of.resize(n);
    b->local_of.resize(n);
    b->row0.resize(n);
    for (int i = 0; i < n; i++) {
        b->row0[i] = (int)b->n_bodies;
        b->n_bodies += (int64_t)ws[i]->bodies.size();
    }
    const auto parts = batch_partition(ws, S);
    b->sched.parts = (int)parts.size();
    for (size_t p = 0; p < parts.size(); p++) {
        std::vector<World*> sub;
        std::vector<int> rows;
        for (size_t k = 0; k < parts[p].size(); k++) {
            const int wi = parts[p][k];
            b->part_of[wi] = (int)p;
            b->local_of[wi] = (int)k;
            sub.push_back(ws[wi]);
            for (size_t j = 0; j < ws[wi]->bodies.size(); j++) rows.push_back(b->row0[wi] + (int)j);
        }
        // the parts' solver-chain kernels run at the same time and share the
        // SMs' shared memory: the later parts take at most rest_per_sm chain
        // workers per SM so that the first part's longest chains are not
        // queued behind them
        const int rank = parts.size() > 1 && env_int("CPGPU_BATCH_PRIORITY", 1) ? (int)p : -1;
        const int per_sm = p == 0 || parts.size() == 1 ? 0 : (p == 1 && S.mid_per_sm >= 0 ? S.mid_per_sm : S.rest_per_sm);
        b->parts.push_back(build_batch(sub, per_sm, rank));
        if (S.big_rows != kDefaultBigRows) b->parts.back()->set_schedule(b->parts.back()->pgs_per_sm, S.big_rows);
        int* d_rows = nullptr;
        CK(cudaMalloc(&d_rows, sizeof(int) * std::max<size_t>(rows.size(), 1)));
        CK(cudaMemcpy(d_rows, rows.data(), sizeof(int) * rows.size(), cudaMemcpyHostToDevice));
        b->rows.push_back(d_rows);
    }
    CK(cudaMalloc(&b->stage, sizeof(float4) * 4 * std::max<int64_t>(b->n_bodies, 1)));
    CK(cudaEventCreate(&b->ev0));
    CK(cudaEventCreate(&b->ev1));
    CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->done.resize(b->parts.size());
    for (auto& e : b->done) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return b;
}

static std::vector<World*> batch_worlds(cpgpu_world* const* worlds, int n) {
    if (!worlds || n <= 0) throw ApiFail{CPGPU_ERR_INVALID_ARG, "empty batch"};
    std::vector<World*> ws;
    for (int i = 0; i < n; i++) {
        if (!worlds[i]) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null world"};
        if (worlds[i]->w.dev && worlds[i]->w.dev_valid) download_state(worlds[i]->w);
        ws.push_back(&worlds[i]->w);
    }
    return ws;
}

int cpgpu_batch_create(cpgpu_world* const* worlds, int n, cpgpu_batch** out) {
    return guarded([&] {
        if (!out) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null output"};
        const std::vector<World*> ws = batch_worlds(worlds, n);
        Schedule S = default_schedule(ws);
        bool tuned = false;
        // a schedule set through the environment takes precedence over the cache
        const bool env_set = std::getenv("CPGPU_BATCH_PARTS") || std::getenv("CPGPU_BATCH_FIRST_SHARE") ||
                             std::getenv("CPGPU_BATCH_SECOND_SHARE") || std::getenv("CPGPU_PGS_REST_PER_SM") ||
                             std::getenv("CPGPU_PGS_MID_PER_SM") || std::getenv("CPGPU_PGS_BIG_ROWS");
        if (!env_set) {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            tune_file_load();
            auto it = g_tuned.find(histogram_key(ws));
            if (it != g_tuned.end()) { S = it->second; tuned = true; }
        }
        auto b = make_batch(ws, S);
        b->tuned = tuned;
        b->pin(worlds, n);
        *out = b.release();
        return CPGPU_OK;
    });
}

// Device time of n steps of every part (graph launches, the parts
// concurrent), the parts' streams joined before and after
static double time_steps(cpgpu_batch* b, int n) {
    CK(cudaEventRecord(b->ev0, b->st0()));
    b->fan_out();
    b->step_parts(n);
    b->fan_in();
    CK(cudaEventRecord(b->ev1, b->st0()));
    CK(cudaEventSynchronize(b->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    for (auto& p : b->parts) p->check_status();
    return ms;
}

// The autotuner's score of a schedule, ms per step: the mean of a step inside
// a run of n steps (the parts drift apart, staggered) and a step run alone and
// waited for (the parts concurrent; a caller that reads the state back every
// step sees this one).  A schedule can favour one and cost the other.
static double tune_score(cpgpu_batch* b, int n) {
    const double run = time_steps(b, n) / n;
    double single = 0;
    for (int i = 0; i < n; i++) single += time_steps(b, 1);
    return 0.5 * (run + single / n);
}

// Autotuner: candidate schedules (one, two or three parts with several
// first-part shares; for each, the later parts' chain workers per SM and the
// big-island threshold) are built from the batch's current state (read back
// into the worlds' host mirrors), timed on trial steps, each trial's state
// restored afterwards, and the fastest adopted; the batch then continues from
// exactly the state it had.  Tune from a representative state (the first
// steps of a scene, before bodies touch, cost far less than later ones).  The
// choice is cached for the world-size histogram, so later batches with the
// same histogram start with it.
static void tune_batch(cpgpu_batch* b, int trial_steps) {
    const int T = std::max(1, trial_steps);
    for (size_t i = 0; i < b->worlds.size(); i++)
        if (i < b->versions.size() && b->worlds[i]->version != b->versions[i])
            throw ApiFail{CPGPU_ERR_INVALID_ARG, "a world changed after the batch was made from it: make a new batch"};
    // private copies of the worlds carry the batch's current state; the
    // worlds' own host mirrors are left as they are
    std::vector<std::unique_ptr<World>> copies(b->worlds.size());
    std::vector<World*> ws(b->worlds.size());
    for (size_t i = 0; i < copies.size(); i++) {
        copies[i] = std::make_unique<World>();
        copy_world(*b->worlds[i], *copies[i]);
        ws[i] = copies[i].get();
    }
    for (size_t p = 0; p < b->parts.size(); p++) {
        std::vector<World*> sub;
        for (size_t wi = 0; wi < ws.size(); wi++)
            if (b->part_of[wi] == (int)p) sub.push_back(ws[wi]);
        download_worlds(*b->parts[p], sub);
    }
    const Schedule dflt = default_schedule(ws);
    std::vector<Schedule> layouts{dflt};
    auto add = [&](int parts, int share, int second) {
        if (parts > (int)ws.size()) return;
        for (const Schedule& x : layouts)
            if (x.parts == parts && (parts == 1 || (x.first_share == share && x.second_share == second))) return;
        Schedule sch;
        sch.parts = parts; sch.first_share = parts > 1 ? share : 100;
        sch.second_share = parts > 2 ? second : 0;
        layouts.push_back(sch);
    };
    add(1, 100, 0);
    for (int share : {10, 20, 30}) add(2, share, 0);
    // graduated parts (the largest worlds' few percent first), whose
    // staggered first halves let the longest chains start soonest
    add(3, 5, 20);
    add(4, 3, 12);
    std::unique_ptr<cpgpu_batch> best, dcand;   // dcand: the hand-set default's layout, kept for the final check
    double best_ms = 1e300, dflt_ms = -1;
    Schedule dcfg = dflt;
    for (const Schedule& L : layouts) {
        std::unique_ptr<cpgpu_batch> cand = make_batch(ws, L);
        for (auto& p : cand->parts) p->snapshot();
        const bool dflt_layout = L.parts == dflt.parts && L.first_share == dflt.first_share && L.second_share == dflt.second_share;
        const std::vector<int> per_sms = cand->parts.size() > 1 ? std::vector<int>{1, 2, 3} : std::vector<int>{0};
        Schedule cbest = cand->sched;
        double cbest_ms = 1e300;
        for (int per_sm : per_sms)
            for (int big : {32, 48, 96}) {
                for (size_t p = 0; p < cand->parts.size(); p++) cand->parts[p]->set_schedule(p == 0 ? 0 : per_sm, big);
                time_steps(cand.get(), 1);   // warm-up
                const double ms = tune_score(cand.get(), T);
                for (auto& p : cand->parts) p->restore(false);
                const bool is_dflt = dflt_layout && big == dflt.big_rows &&
                                     (cand->parts.size() == 1 || per_sm == dflt.rest_per_sm);
                if (is_dflt) { dflt_ms = ms; dcfg = cand->sched; dcfg.rest_per_sm = cand->parts.size() > 1 ? per_sm : 0; dcfg.big_rows = big; }
                if (ms < cbest_ms) {
                    cbest_ms = ms;
                    cbest.rest_per_sm = cand->parts.size() > 1 ? per_sm : 0;
                    cbest.big_rows = big;
                }
            }
        for (size_t p = 0; p < cand->parts.size(); p++)
            cand->parts[p]->set_schedule(p == 0 ? 0 : cbest.rest_per_sm, cbest.big_rows);
        cand->sched = cbest;
        if (cbest_ms < best_ms) {
            best_ms = cbest_ms;
            if (best && !dcand && best->sched.parts == dflt.parts && best->sched.first_share == dflt.first_share &&
                best->sched.second_share == dflt.second_share)
                dcand = std::move(best);
            best = std::move(cand);
        } else if (dflt_layout) {
            dcand = std::move(cand);
        }
    }
    // A few trial steps can favour a schedule whose parts drift apart within
    // them; when the choice is not the hand-set default, the two are timed
    // again over more steps from the same state and the faster kept.
    if (dcand && dflt_ms > 0) {
        const int T2 = std::max(2 * T, 8);
        time_steps(best.get(), 1);
        const double mb = tune_score(best.get(), T2);
        for (auto& p : best->parts) p->restore(false);
        for (size_t p = 0; p < dcand->parts.size(); p++)
            dcand->parts[p]->set_schedule(p == 0 ? 0 : dcfg.rest_per_sm, dcfg.big_rows);
        dcand->sched = dcfg;
        time_steps(dcand.get(), 1);
        const double md = tune_score(dcand.get(), T2);
        for (auto& p : dcand->parts) p->restore(false);
        if (md <= mb) { best = std::move(dcand); best_ms = md; dflt_ms = md; }
        else { best_ms = mb; dflt_ms = md; }
    }
    for (auto& p : best->parts) p->restore(true);
    b->adopt(*best);
    b->tuned = true;
    b->tuned_ms = best_ms;
    b->default_ms = dflt_ms;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    const std::string key = histogram_key(ws);
    g_tuned[key] = b->sched;
    tune_file_save(key, b->sched);
}

int cpgpu_batch_tune(cpgpu_batch* b, int trial_steps) {
    if (!b) return fail(CPGPU_ERR_INVALID_ARG, "null batch");
    return guarded([&] {
        tune_batch(b, trial_steps);
        return CPGPU_OK;
    });
}

int cpgpu_batch_create_tuned(cpgpu_world* const* worlds, int n, int trial_steps, cpgpu_batch** out) {
    return guarded([&] {
        if (!out) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null output"};
        const std::vector<World*> ws = batch_worlds(worlds, n);
        auto b = make_batch(ws, default_schedule(ws));
        b->pin(worlds, n);
        tune_batch(b.get(), trial_steps);
        *out = b.release();
        return CPGPU_OK;
    });
}

int cpgpu_batch_schedule(cpgpu_batch* b, int* sched, double* times) {
    if (!b) return fail(CPGPU_ERR_INVALID_ARG, "null batch");
    if (sched) {
        sched[0] = b->sched.parts; sched[1] = b->sched.first_share; sched[2] = b->sched.rest_per_sm;
        sched[3] = b->sched.big_rows; sched[4] = b->tuned ? 1 : 0; sched[5] = b->sched.second_share;
    }
    if (times) { times[0] = b->tuned_ms; times[1] = b->default_ms; }
    return CPGPU_OK;
}
int cpgpu_batch_destroy(cpgpu_batch* b) { delete b; return CPGPU_OK; }

static int batch_check(cpgpu_batch* b) {
    for (auto& p : b->parts) p->check_status();
    return CPGPU_OK;
}

int cpgpu_batch_step(cpgpu_batch* b, int n) {
    if (!b) return fail(CPGPU_ERR_INVALID_ARG, "null batch");
    return guarded([&] {
        b->step_parts(n);
        return batch_check(b);
    });
}
int cpgpu_batch_set_audit(cpgpu_batch* b, int enabled) {
    if (!b) return fail(CPGPU_ERR_INVALID_ARG, "null batch");
    return guarded([&] {
        for (auto& p : b->parts) p->set_audit(enabled != 0);
        return CPGPU_OK;
    });
}

int cpgpu_batch_read_audit(cpgpu_batch* b, double* out) {
    if (!b) return fail(CPGPU_ERR_INVALID_ARG, "null batch");
    return guarded([&] {
        if (!out) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null output"};
        std::vector<std::vector<double>> per(b->parts.size());
        for (size_t p = 0; p < b->parts.size(); p++) {
            per[p].resize((size_t)kAuditValues * b->parts[p]->n_worlds);
            b->parts[p]->read_audit(per[p].data());
        }
        for (size_t wi = 0; wi < b->part_of.size(); wi++)
            for (int k = 0; k < kAuditValues; k++)
                out[kAuditValues * wi + k] = per[b->part_of[wi]][(size_t)kAuditValues * b->local_of[wi] + k];
        return CPGPU_OK;
    });
}

int cpgpu_batch_get_body_state(cpgpu_batch* b, int wi, double* com, double* quat, double* vel, double* ang) {
    if (!b) return fail(CPGPU_ERR_INVALID_ARG, "null batch");
    return guarded([&] {
        if (wi < 0 || wi >= (int)b->part_of.size()) throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad world index"};
        Batch& B = b->part(b->part_of[wi]);
        const int lw = b->local_of[wi];
        int s = B.world_start[lw], n = B.world_start[lw + 1] - s;
        std::vector<float4> pos(n), rot(n), vel4(n), ang4(n);
        const Dev& x = B.cur();
        CK(cudaMemcpyAsync(pos.data(), x.pos + s, n * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(rot.data(), x.rot + s, n * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(vel4.data(), x.vel + s, n * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaMemcpyAsync(ang4.data(), x.angv + s, n * 16, cudaMemcpyDeviceToHost, B.st));
        CK(cudaStreamSynchronize(B.st));
        for (int i = 0; i < n; i++) {
            bool fixed = B.movement[s + i] == CPGPU_FIXED;
            if (com) { com[3 * i] = pos[i].x; com[3 * i + 1] = pos[i].y; com[3 * i + 2] = pos[i].z; }
            if (quat) { quat[4 * i] = rot[i].x; quat[4 * i + 1] = rot[i].y; quat[4 * i + 2] = rot[i].z; quat[4 * i + 3] = rot[i].w; }
            if (vel) { vel[3 * i] = fixed ? 0 : vel4[i].x; vel[3 * i + 1] = fixed ? 0 : vel4[i].y; vel[3 * i + 2] = fixed ? 0 : vel4[i].z; }
            if (ang) { ang[3 * i] = fixed ? 0 : ang4[i].x; ang[3 * i + 1] = fixed ? 0 : ang4[i].y; ang[3 * i + 2] = fixed ? 0 : ang4[i].z; }
        }
        return CPGPU_OK;
    });
}
int cpgpu_batch_info(cpgpu_batch* b, int64_t* n_bodies, int64_t* n_worlds, int64_t* n_contacts) {
    if (!b) return fail(CPGPU_ERR_INVALID_ARG, "null batch");
    return guarded([&] {
        int64_t contacts = 0;
        for (auto& p : b->parts) {
            Batch& B = *p;
            int counts[6];
            CK(cudaMemcpyAsync(counts, B.cur().n_pairs, sizeof(counts), cudaMemcpyDeviceToHost, B.st));
            CK(cudaStreamSynchronize(B.st));
            contacts += counts[3 + B.parity];
        }
        if (n_bodies) *n_bodies = b->n_bodies;
        if (n_worlds) *n_worlds = (int64_t)b->part_of.size();
        if (n_contacts) *n_contacts = contacts;
        return CPGPU_OK;
    });
}

int cpgpu_batch_launches_per_step(cpgpu_batch* b, int* n) {
    if (!b || !n) return fail(CPGPU_ERR_INVALID_ARG, "null argument");
    int t = 0;
    for (auto& p : b->parts) t += p->launches_per_step();
    *n = t;
    return CPGPU_OK;
}

// host layout: 16 floats per body in batch order (pos with inverse mass, rot,
// vel, ang vel); one copy each way, each part gathering / scattering its rows
int cpgpu_batch_read_state(cpgpu_batch* b, float* out) {
    if (!b || !out) return fail(CPGPU_ERR_INVALID_ARG, "null argument");
    return guarded([&] {
        for (size_t p = 0; p < b->parts.size(); p++) {
            Batch& B = b->part((int)p);
            launch_scatter_state(B.cur(), b->rows[p], b->stage, Launch{B.n_sms, B.st});
        }
        b->fan_in();
        CK(cudaMemcpyAsync(out, b->stage, (size_t)b->n_bodies * 64, cudaMemcpyDeviceToHost, b->st0()));
        CK(cudaStreamSynchronize(b->st0()));
        return CPGPU_OK;
    });
}

int cpgpu_batch_write_state(cpgpu_batch* b, const float* in) {
    if (!b || !in) return fail(CPGPU_ERR_INVALID_ARG, "null argument");
    return guarded([&] {
        CK(cudaMemcpyAsync(b->stage, in, (size_t)b->n_bodies * 64, cudaMemcpyHostToDevice, b->st0()));
        b->fan_out();
        for (size_t p = 0; p < b->parts.size(); p++) {
            Batch& B = b->part((int)p);
            const Launch L{B.n_sms, B.st};
            launch_gather_state(B.cur(), b->stage, b->rows[p], L);
            launch_apply_state(B.cur(), L);
        }
        // the staging buffer is reused by the next read: order it after these gathers
        b->fan_in();
        CK(cudaStreamSynchronize(b->st0()));
        return CPGPU_OK;
    });
}

// n steps launched stage by stage with an event after every stage on every
// part's stream, one step at a time (every part's stream waits for the
// previous step of all parts), the parts concurrent as in a single step;
// `each(at)` is called after each step with at(p, m) = ms from the step's
// start to mark m of part p.
using StageClock = std::function<double(size_t, int)>;
static void profile_steps(cpgpu_batch* b, int n_steps, const std::function<void(const StageClock&)>& each) {
    const size_t np = b->parts.size();
    std::vector<std::vector<cudaEvent_t>> ev(np);
    for (size_t p = 0; p < np; p++) {
        ev[p].resize(7 + 3 * b->parts[p]->substeps);
        for (auto& e : ev[p]) CK(cudaEventCreate(&e));
    }
    for (int i = 0; i < n_steps; i++) {
        CK(cudaEventRecord(b->ev0, b->st0()));
        b->fan_out();
        for (size_t p = 0; p < np; p++) {
            Batch& B = *b->parts[p];
            B.marks = &ev[p];
            B.launch_pre(B.d[B.parity]);
            CK(cudaEventRecord(B.pre_done, B.st));
            B.launch_rest(B.d[B.parity]);
            B.marks = nullptr;
            CK(cudaGetLastError());   // a launch refused here would leave its stage untimed
            B.parity ^= 1;
        }
        b->fan_in();
        CK(cudaEventRecord(b->ev1, b->st0()));
        CK(cudaEventSynchronize(b->ev1));
        const StageClock at = [&](size_t p, int m) {
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, b->ev0, ev[p][m]));
            return (double)ms;
        };
        each(at);
    }
    for (auto& v : ev)
        for (auto& e : v) cudaEventDestroy(e);
}

int cpgpu_batch_profile(cpgpu_batch* b, int n_steps, double* stage_ms, int64_t* counts) {
    if (!b || !stage_ms) return fail(CPGPU_ERR_INVALID_ARG, "null argument");
    return guarded([&] {
        for (int k = 0; k < CPGPU_N_STAGES; k++) stage_ms[k] = 0;
        if (counts) counts[0] = counts[1] = counts[2] = 0;
        const size_t np = b->parts.size();
        const int S = b->parts[0]->substeps;   // the parts share the substep count
        profile_steps(b, n_steps, [&](const StageClock& at) {
            // the stage's time in the step: the length of the union of the
            // parts' intervals in it (a part's stages are in stream order)
            auto window = [&](auto first_mark, auto last_mark) {
                std::vector<std::pair<double, double>> iv;
                for (size_t p = 0; p < np; p++) iv.push_back({at(p, first_mark(p)), at(p, last_mark(p))});
                std::sort(iv.begin(), iv.end());
                double total = 0, lo = -1e300, hi = -1e300;
                for (const auto& x : iv) {
                    if (x.first > hi) { total += std::max(0.0, hi - lo); lo = x.first; hi = x.second; }
                    else hi = std::max(hi, x.second);
                }
                return total + std::max(0.0, hi - lo);
            };
            for (int k = 0; k < 5; k++) stage_ms[k] += window([&](size_t) { return k; }, [&](size_t) { return k + 1; });
            for (int s2 = 0; s2 < S; s2++) {
                stage_ms[5] += window([&](size_t) { return 5 + 3 * s2; }, [&](size_t) { return 6 + 3 * s2; });
                stage_ms[6] += window([&](size_t) { return 6 + 3 * s2; }, [&](size_t) { return 7 + 3 * s2; });
                stage_ms[7] += window([&](size_t) { return 7 + 3 * s2; }, [&](size_t) { return 8 + 3 * s2; });
            }
            stage_ms[8] += window([&](size_t) { return 5 + 3 * S; }, [&](size_t) { return 6 + 3 * S; });
        });
        if (counts)
            for (auto& part : b->parts) {
                Batch& B = *part;
                int c[6];
                CK(cudaMemcpyAsync(c, B.cur().n_pairs, sizeof(c), cudaMemcpyDeviceToHost, B.st));
                CK(cudaStreamSynchronize(B.st));
                counts[0] += c[0];
                counts[1] += c[3 + B.parity];
                counts[2] += c[5];
            }
        return batch_check(b);
    });
}

int cpgpu_batch_timeline(cpgpu_batch* b, int n_steps, double* out, int cap, int* n_parts, int* n_marks) {
    if (!b || !n_parts || !n_marks) return fail(CPGPU_ERR_INVALID_ARG, "null argument");
    return guarded([&] {
        const int np = (int)b->parts.size(), nm = 7 + 3 * b->parts[0]->substeps;
        *n_parts = np;
        *n_marks = nm;
        if (!out || n_steps < 1) return CPGPU_OK;
        if (cap < np * nm) throw ApiFail{CPGPU_ERR_INVALID_ARG, "timeline buffer too small"};
        for (int k = 0; k < np * nm; k++) out[k] = 0;
        profile_steps(b, n_steps, [&](const StageClock& at) {
            for (int p = 0; p < np; p++)
                for (int m = 0; m < nm; m++) out[p * nm + m] += at(p, m) / n_steps;
        });
        return batch_check(b);
    });
}

// Device time of n steps of the batch: CUDA events on part 0's stream, which
// the other parts' streams join before the start and after the last step.
int cpgpu_batch_step_timed(cpgpu_batch* b, int n, double* device_ms) {
    if (!b) return fail(CPGPU_ERR_INVALID_ARG, "null batch");
    return guarded([&] {
        CK(cudaEventRecord(b->ev0, b->st0()));
        b->fan_out();
        b->step_parts(n);
        b->fan_in();
        CK(cudaEventRecord(b->ev1, b->st0()));
        CK(cudaEventSynchronize(b->ev1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        if (device_ms) *device_ms = ms;
        return batch_check(b);
    });
}

// ------------------------------------------------------------------ serving ----
int cpgpu_world_clone(cpgpu_world* src, cpgpu_world** out) {
    W_OR_FAIL(src);
    return guarded([&] {
        if (!out) throw ApiFail{CPGPU_ERR_INVALID_ARG, "null out"};
        if (src->w.dev && src->w.dev_valid) download_state(src->w);
        auto c = std::make_unique<cpgpu_world>();
        copy_world(src->w, c->w);
        *out = c.release();
        return CPGPU_OK;
    });
}

}  // extern "C"

namespace cpgpu {

struct ServerRequest {
    World* w = nullptr;
    int remaining = 0;
    uint64_t token = 0;
    int64_t bodies = 0;
    size_t bytes = 0;   // estimated device bytes
    bool finished = false;   // result captured; still in the batch until the next re-form
};

// A cohort: requests admitted together, stepped as one batch on the batch's
// own stream.  A cohort never takes in running worlds: requests that arrive
// later form new cohorts, which step beside it; a finished request's state is
// read back in place while its cohort keeps going; a cohort is freed when its
// last request finishes.
struct Cohort {
    std::vector<ServerRequest> running;   // in batch order
    std::unique_ptr<Batch> batch;
    int inflight = 0;                     // steps launched and not yet accounted
    int stepped = 0;                      // steps completed since it was built
    cudaEvent_t ev = nullptr;             // recorded after the in-flight steps
    ~Cohort() { if (ev) cudaEventDestroy(ev); }
    int64_t live_bodies() const {
        int64_t n = 0;
        for (const auto& r : running) if (!r.finished) n += r.bodies;
        return n;
    }
    int64_t all_bodies() const {
        int64_t n = 0;
        for (const auto& r : running) n += r.bodies;
        return n;
    }
};

// One lane of the server: the requests of one world-size class
struct ServerLane {
    std::deque<ServerRequest> waiting;
    std::vector<std::unique_ptr<Cohort>> cohorts;   // oldest first
};

// Requests are worlds with a step count.  They are sorted by size into lanes
// (fewer than 128 dynamic bodies, fewer than 512, the rest): a step of a batch
// lasts as long as its largest island's serial solve, so a small world batched
// with large ones would advance at the large ones' pace.  Within a lane,
// waiting requests are admitted in arrival order under one device-memory
// budget for all lanes, at most once per `epoch_steps` steps of the lane's
// newest cohort, as a new cohort (a batch built from the new worlds only);
// running worlds are never copied to admit new ones.  A cohort whose finished
// requests hold three quarters of its bodies (compact_pct) is compacted into
// the next new cohort of its lane (its live worlds read back and packed with
// the new ones).  Every cohort steps on its own stream in chunks: advance() launches
// the next chunk on every idle cohort and returns once one has completed.
struct Server {
    int64_t budget = 0;
    int epoch_steps = 10;
    double bytes_per_body = 2048;     // updated from every batch built
    std::vector<std::unique_ptr<ServerLane>> lanes;
    std::vector<int64_t> bounds{128, 512};
    std::vector<uint64_t> done;
    uint64_t next_token = 1;
    int64_t body_steps = 0, reforms = 0;
    double reform_ms = 0;
    // a cohort whose finished requests hold this percentage of its bodies is
    // compacted into the lane's next new cohort (CPGPU_SERVE_COMPACT_PCT)
    int compact_pct = 75;

    Server() {
        compact_pct = std::max(1, std::min(100, env_int("CPGPU_SERVE_COMPACT_PCT", 75)));
        for (size_t k = 0; k <= bounds.size(); k++) lanes.push_back(std::make_unique<ServerLane>());
    }

    int lane_of(int64_t bodies) const {
        int k = 0;
        while (k < (int)bounds.size() && bodies >= bounds[k]) k++;
        return k;
    }
    size_t estimate(const World& w) const { return (size_t)(bytes_per_body * (double)w.bodies.size()) + (1u << 20); }
    size_t used_bytes() const {
        size_t u = 0;
        for (auto& L : lanes)
            for (auto& c : L->cohorts)
                for (auto& r : c->running) u += r.bytes;
        return u;
    }
    int64_t running_count() const {
        int64_t n = 0;
        for (auto& L : lanes)
            for (auto& c : L->cohorts)
                for (auto& r : c->running) n += !r.finished;
        return n;
    }
    int64_t waiting_count() const {
        int64_t n = 0;
        for (auto& L : lanes) n += (int64_t)L->waiting.size();
        return n;
    }
    int64_t device_bytes() const {
        int64_t n = 0;
        for (auto& L : lanes)
            for (auto& c : L->cohorts) n += c->batch ? (int64_t)c->batch->bytes : 0;
        return n;
    }
    int64_t running_bodies() const {
        int64_t n = 0;
        for (auto& L : lanes)
            for (auto& c : L->cohorts) n += c->live_bodies();
        return n;
    }

    void submit(const ServerRequest& r) { lanes[lane_of(r.bodies)]->waiting.push_back(r); }

    // capture the exact state of requests that reached their step count,
    // without stopping the cohort (they keep stepping as dead weight until the
    // cohort ends or is compacted)
    void capture_finished(Cohort& C) {
        std::vector<int> idx;
        std::vector<World*> ws;
        for (size_t i = 0; i < C.running.size(); i++)
            if (!C.running[i].finished && C.running[i].remaining <= 0) { idx.push_back((int)i); ws.push_back(C.running[i].w); }
        if (idx.empty()) return;
        download_subset(*C.batch, idx, ws);
        for (int i : idx) { C.running[i].finished = true; done.push_back(C.running[i].token); }
    }

    // a new cohort for the lane: the live requests of its sparse cohorts
    // (read back) and the waiting requests that fit the budget
    void admit(ServerLane& L) {
        auto t0 = std::chrono::steady_clock::now();
        std::vector<ServerRequest> take;
        for (auto it = L.cohorts.begin(); it != L.cohorts.end();) {
            Cohort& C = **it;
            const int64_t live = C.live_bodies(), all = C.all_bodies();
            if (C.inflight == 0 && live > 0 && 100 * (all - live) >= (int64_t)compact_pct * all) {
                std::vector<int> idx;
                std::vector<World*> ws;
                for (size_t i = 0; i < C.running.size(); i++)
                    if (!C.running[i].finished) { idx.push_back((int)i); ws.push_back(C.running[i].w); take.push_back(C.running[i]); }
                download_subset(*C.batch, idx, ws);
                it = L.cohorts.erase(it);
            } else {
                ++it;
            }
        }
        size_t used = used_bytes();
        for (auto& r : take) used += r.bytes;
        while (!L.waiting.empty()) {
            ServerRequest& r = L.waiting.front();
            r.bytes = estimate(*r.w);
            if ((running_count() > 0 || !take.empty()) && used + r.bytes > (size_t)budget) break;
            used += r.bytes;
            take.push_back(r);
            L.waiting.pop_front();
        }
        if (!take.empty()) {
            auto C = std::make_unique<Cohort>();
            C->running = std::move(take);
            std::vector<World*> ws;
            for (auto& r : C->running) ws.push_back(r.w);
            C->batch = build_batch(ws);
            int64_t nb = 0;
            for (auto& r : C->running) nb += r.bodies;
            if (nb > 0) bytes_per_body = (double)C->batch->bytes / (double)nb;
            for (auto& r : C->running) r.bytes = estimate(*r.w);
            CK(cudaEventCreateWithFlags(&C->ev, cudaEventDisableTiming));
            L.cohorts.push_back(std::move(C));
            reforms++;
        }
        reform_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }

    // account for a cohort's completed chunk; a cohort with no live request
    // left is freed
    void complete(Cohort& C) {
        if (C.inflight == 0) return;
        C.batch->check_status();
        for (auto& r : C.running) {
            if (r.finished) continue;
            r.remaining -= C.inflight;
            body_steps += (int64_t)C.inflight * r.bodies;
        }
        C.stepped += C.inflight;
        C.inflight = 0;
        capture_finished(C);
    }

    void launch(Cohort& C, int max_steps) {
        int n = max_steps;
        bool live = false;
        for (auto& r : C.running) if (!r.finished) { n = std::min(n, r.remaining); live = true; }
        if (!live) return;
        if (n <= 0) { capture_finished(C); return; }
        C.batch->step(n);
        CK(cudaEventRecord(C.ev, C.batch->st));
        C.inflight = n;
    }

    // Admit where due, launch on every idle cohort, then wait (bounded) until
    // one cohort's chunk completes and account for it.  Returns the steps that
    // cohort completed.
    int advance(int max_steps) {
        for (auto& L : lanes) {
            // drop finished cohorts
            L->cohorts.erase(std::remove_if(L->cohorts.begin(), L->cohorts.end(),
                                            [](const std::unique_ptr<Cohort>& c) { return c->inflight == 0 && c->live_bodies() == 0; }),
                             L->cohorts.end());
            const bool due = L->cohorts.empty() || L->cohorts.back()->stepped + L->cohorts.back()->inflight >= epoch_steps;
            if (!L->waiting.empty() && due) admit(*L);
            for (auto& c : L->cohorts)
                if (c->inflight == 0) {
                    int n = max_steps;
                    // the newest cohort stops at the epoch so that the next admission is not delayed
                    if (!L->waiting.empty() && c.get() == L->cohorts.back().get()) n = std::min(n, std::max(1, epoch_steps - c->stepped));
                    launch(*c, n);
                }
        }
        const auto t0 = std::chrono::steady_clock::now();
        while (true) {
            int stepped = 0;
            bool any = false;
            for (auto& L : lanes)
                for (auto& c : L->cohorts) {
                    if (c->inflight == 0) continue;
                    any = true;
                    const cudaError_t q = cudaEventQuery(c->ev);
                    if (q == cudaSuccess) {
                        stepped = std::max(stepped, c->inflight);
                        complete(*c);
                    } else if (q != cudaErrorNotReady) {
                        CK(q);
                    }
                }
            if (!any || stepped > 0) return stepped;
            if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(600))
                throw ApiFail{CPGPU_ERR_TIMEOUT, "server chunk did not complete within 600 s"};
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }

    // wait for every chunk in flight
    void drain() {
        for (auto& L : lanes)
            for (auto& c : L->cohorts)
                if (c->inflight) { CK(cudaEventSynchronize(c->ev)); complete(*c); }
    }
};

}  // namespace cpgpu

struct cpgpu_server { cpgpu::Server s; };

extern "C" {

int cpgpu_server_create(int64_t hbm_budget_bytes, int epoch_steps, cpgpu_server** out) {
    return guarded([&] {
        if (!out || hbm_budget_bytes <= 0 || epoch_steps < 1) throw ApiFail{CPGPU_ERR_INVALID_ARG, "bad server arguments"};
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw ApiFail{CPGPU_ERR_NO_DEVICE, "no CUDA device"};
        auto s = std::make_unique<cpgpu_server>();
        s->s.budget = hbm_budget_bytes;
        s->s.epoch_steps = epoch_steps;
        *out = s.release();
        return CPGPU_OK;
    });
}
int cpgpu_server_destroy(cpgpu_server* s) {
    if (s) {
        try { s->s.drain(); } catch (...) {}
    }
    delete s;
    return CPGPU_OK;
}

int cpgpu_server_submit(cpgpu_server* s, cpgpu_world* w, int steps, uint64_t* token) {
    if (!s || !w) return fail(CPGPU_ERR_INVALID_ARG, "null server or world");
    return guarded([&] {
        if (steps < 0) throw ApiFail{CPGPU_ERR_INVALID_ARG, "negative step count"};
        if (w->w.bodies.empty()) throw ApiFail{CPGPU_ERR_INVALID_ARG, "empty world"};
        if (w->w.dev && w->w.dev_valid) download_state(w->w);
        w->w.dev_valid = false;
        cpgpu::ServerRequest r;
        r.w = &w->w;
        r.remaining = steps;
        r.token = s->s.next_token++;
        r.bodies = 0;
        for (const auto& b : w->w.bodies) r.bodies += b.movement == CPGPU_DYNAMIC;
        s->s.submit(r);
        if (token) *token = r.token;
        return CPGPU_OK;
    });
}

int cpgpu_server_advance(cpgpu_server* s, int max_steps, int* n_running, int* n_waiting) {
    if (!s) return fail(CPGPU_ERR_INVALID_ARG, "null server");
    return guarded([&] {
        s->s.advance(max_steps);
        if (n_running) *n_running = (int)s->s.running_count();
        if (n_waiting) *n_waiting = (int)s->s.waiting_count();
        return CPGPU_OK;
    });
}

int cpgpu_server_poll(cpgpu_server* s, uint64_t* tokens, int cap, int* n) {
    if (!s || !n) return fail(CPGPU_ERR_INVALID_ARG, "null argument");
    auto& d = s->s.done;
    int k = std::min((int)d.size(), cap);
    for (int i = 0; i < k; i++) if (tokens) tokens[i] = d[i];
    d.erase(d.begin(), d.begin() + k);
    *n = k;
    return CPGPU_OK;
}

int cpgpu_server_stats(cpgpu_server* s, int64_t* body_steps, int64_t* reforms, double* reform_ms, int64_t* device_bytes,
                       int64_t* running_bodies) {
    if (!s) return fail(CPGPU_ERR_INVALID_ARG, "null server");
    if (body_steps) *body_steps = s->s.body_steps;
    if (reforms) *reforms = s->s.reforms;
    if (reform_ms) *reform_ms = s->s.reform_ms;
    if (device_bytes) *device_bytes = s->s.device_bytes();
    if (running_bodies) *running_bodies = s->s.running_bodies();
    return CPGPU_OK;
}

}  // extern "C"
