// cport.h — CPU restatement of the ConstraintPhysics per-step contact path.
//
// TEST INFRASTRUCTURE (the oracle).  Only the test-suite and the CPU-baseline
// leg of bench.py load it; the product never links it.  It restates, in FP64
// and in plain serial C++, what the reference engine computes on this path,
// with each function citing the reference lines it follows.  Arithmetic is
// written in the reference's evaluation order (left-to-right sums, the same
// matrix/vector formulas) so that runs stay within rounding of the reference;
// tests pin it against the reference engine compiled from its own sources.
//
// Unlike the reference it can import a full dynamic state (bodies and the
// persistent contact graph), so a device step can be replayed here from the
// very same input state.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <algorithm>
#include <vector>
#include <memory>
#include <unordered_map>
#include <set>
#include <functional>
#include <array>

namespace cport {

// ---------------------------------------------------------------- math ----
// Formulas follow Math/src/Vec3.h:6-125, Quaternion.h:7-112, Mat3.h:6-146.
struct V3 {
    double x = 0, y = 0, z = 0;
    V3() {}
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    double mag2() const { return x * x + y * y + z * z; }
    double mag() const { return std::sqrt(x * x + y * y + z * z); }
    V3 normalize() const {
        double m = mag();
        return (m == 0) ? V3(0, 0, 0) : V3(x / m, y / m, z / m);
    }
    V3 cross(const V3& v) const { return V3(y * v.z - z * v.y, z * v.x - x * v.z, x * v.y - y * v.x); }
    double dot(const V3& v) const { return x * v.x + y * v.y + z * v.z; }
    V3 operator+(const V3& v) const { return V3(x + v.x, y + v.y, z + v.z); }
    V3 operator-(const V3& v) const { return V3(x - v.x, y - v.y, z - v.z); }
    V3 operator-() const { return V3(-x, -y, -z); }
    V3& operator+=(const V3& v) { x += v.x; y += v.y; z += v.z; return *this; }
    V3& operator-=(const V3& v) { x -= v.x; y -= v.y; z -= v.z; return *this; }
    V3& operator*=(double d) { x *= d; y *= d; z *= d; return *this; }
    V3& operator/=(double d) { x /= d; y /= d; z /= d; return *this; }
    bool operator==(const V3& v) const { return x == v.x && y == v.y && z == v.z; }
    bool operator!=(const V3& v) const { return !(*this == v); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    // Vec3.h:53-57: two trial axes, the less parallel one wins
    void perpBasis(V3* u, V3* w) const {
        V3 a1(1, 0, 0), a2(0, 1, 0);
        *u = (std::abs(dot(a1)) < std::abs(dot(a2))) ? cross(a1).normalize() : cross(a2).normalize();
        *w = cross(*u).normalize();
    }
};
inline V3 operator*(const V3& v, double d) { return V3(v.x * d, v.y * d, v.z * d); }
inline V3 operator*(double d, const V3& v) { return V3(v.x * d, v.y * d, v.z * d); }
inline V3 operator/(const V3& v, double d) { return V3(v.x / d, v.y / d, v.z / d); }

struct M3 {
    double m[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    static M3 iden() { M3 o; o.m[0][0] = o.m[1][1] = o.m[2][2] = 1; return o; }
    static M3 crossMat(const V3& v) {
        M3 o;
        o.m[0][0] = 0;    o.m[0][1] = -v.z; o.m[0][2] = v.y;
        o.m[1][0] = v.z;  o.m[1][1] = 0;    o.m[1][2] = -v.x;
        o.m[2][0] = -v.y; o.m[2][1] = v.x;  o.m[2][2] = 0;
        return o;
    }
    double det() const {
        double a = m[0][0], b = m[0][1], c = m[0][2], d = m[1][0], e = m[1][1], f = m[1][2], g = m[2][0], h = m[2][1], i = m[2][2];
        return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
    }
    // adjugate over determinant (Mat3.h:46-57)
    M3 inverse() const {
        double a = m[0][0], b = m[0][1], c = m[0][2], d = m[1][0], e = m[1][1], f = m[1][2], g = m[2][0], h = m[2][1], i = m[2][2];
        double dt = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
        M3 o;
        o.m[0][0] = (e * i - f * h); o.m[0][1] = (c * h - b * i); o.m[0][2] = (b * f - c * e);
        o.m[1][0] = (f * g - d * i); o.m[1][1] = (a * i - c * g); o.m[1][2] = (c * d - a * f);
        o.m[2][0] = (d * h - e * g); o.m[2][1] = (b * g - a * h); o.m[2][2] = (a * e - b * d);
        for (int r = 0; r < 3; r++) for (int s = 0; s < 3; s++) o.m[r][s] /= dt;
        return o;
    }
    V3 operator*(const V3& w) const {
        return V3(m[0][0] * w.x + m[0][1] * w.y + m[0][2] * w.z,
                  m[1][0] * w.x + m[1][1] * w.y + m[1][2] * w.z,
                  m[2][0] * w.x + m[2][1] * w.y + m[2][2] * w.z);
    }
    M3 operator*(const M3& b) const {
        M3 o;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) for (int k = 0; k < 3; k++) o.m[i][j] += m[i][k] * b.m[k][j];
        return o;
    }
    M3 operator+(const M3& b) const { M3 o; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.m[i][j] = m[i][j] + b.m[i][j]; return o; }
    M3 operator-(const M3& b) const { M3 o; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.m[i][j] = m[i][j] - b.m[i][j]; return o; }
    M3& operator*=(double d) { for (auto& r : m) for (double& x : r) x *= d; return *this; }
    M3& operator/=(double d) { for (auto& r : m) for (double& x : r) x /= d; return *this; }
};
inline M3 operator*(double d, const M3& a) { M3 o; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.m[i][j] = d * a.m[i][j]; return o; }

struct Q {
    double r = 1, i = 0, j = 0, k = 0;
    Q() {}
    Q(double a, double b, double c, double d) : r(a), i(b), j(c), k(d) {}
    // rotation of `theta` about `axis` (Quaternion.h:26-33)
    static Q axisAngle(double theta, V3 axis) {
        axis = axis.normalize();
        Q q;
        q.r = std::cos(theta / 2.0);
        double s = std::sin(theta / 2.0);
        q.i = axis.x * s; q.j = axis.y * s; q.k = axis.z * s;
        return q;
    }
    V3 rotate(const V3& v) const {
        return V3(v.x * (r * r + i * i - j * j - k * k) + v.y * (2 * i * j - 2 * r * k) + v.z * (2 * i * k + 2 * r * j),
                  v.x * (2 * i * j + 2 * r * k) + v.y * (r * r - i * i + j * j - k * k) + v.z * (2 * j * k - 2 * r * i),
                  v.x * (2 * i * k - 2 * r * j) + v.y * (2 * j * k + 2 * r * i) + v.z * (r * r - i * i - j * j + k * k));
    }
    M3 rotMatrix() const {
        M3 o;
        o.m[0][0] = r * r + i * i - j * j - k * k; o.m[0][1] = 2 * i * j - 2 * r * k;         o.m[0][2] = 2 * i * k + 2 * r * j;
        o.m[1][0] = 2 * i * j + 2 * r * k;         o.m[1][1] = r * r - i * i + j * j - k * k; o.m[1][2] = 2 * j * k - 2 * r * i;
        o.m[2][0] = 2 * i * k - 2 * r * j;         o.m[2][1] = 2 * j * k + 2 * r * i;         o.m[2][2] = r * r - i * i - j * j + k * k;
        return o;
    }
    Q conj() const { return Q(r, -i, -j, -k); }
    Q operator*(const Q& q) const {
        return Q(r * q.r - i * q.i - j * q.j - k * q.k,
                 r * q.i + i * q.r + j * q.k - k * q.j,
                 r * q.j - i * q.k + j * q.r + k * q.i,
                 r * q.k + i * q.j - j * q.i + k * q.r);
    }
    Q normalize() const {
        double mg = std::sqrt(r * r + i * i + j * j + k * k);
        return Q(r / mg, i / mg, j / mg, k / mg);
    }
    bool operator==(const Q& q) const { return r == q.r && i == q.i && j == q.j && k == q.k; }
    bool operator!=(const Q& q) const { return !(*this == q); }
};

// small dense matrices with the accumulation order of Math/src/NMat.h:43-95
template <int R, int C>
struct Mat {
    double v[R][C] = {};
    template <int X>
    Mat<R, X> operator*(const Mat<C, X>& b) const {
        Mat<R, X> o;
        for (int i = 0; i < R; i++) for (int j = 0; j < X; j++) { o.v[i][j] = 0; for (int k = 0; k < C; k++) o.v[i][j] += v[i][k] * b.v[k][j]; }
        return o;
    }
    Mat<C, R> T() const { Mat<C, R> o; for (int i = 0; i < R; i++) for (int j = 0; j < C; j++) o.v[j][i] = v[i][j]; return o; }
    Mat operator-() const { Mat o; for (int i = 0; i < R; i++) for (int j = 0; j < C; j++) o.v[i][j] = -v[i][j]; return o; }
    Mat operator+(const Mat& b) const { Mat o; for (int i = 0; i < R; i++) for (int j = 0; j < C; j++) o.v[i][j] = v[i][j] + b.v[i][j]; return o; }
};
template <int N>
struct Vec {
    double v[N] = {};
    Vec operator+(const Vec& b) const { Vec o; for (int i = 0; i < N; i++) o.v[i] = v[i] + b.v[i]; return o; }
    Vec operator-(const Vec& b) const { Vec o; for (int i = 0; i < N; i++) o.v[i] = v[i] - b.v[i]; return o; }
    Vec operator-() const { Vec o; for (int i = 0; i < N; i++) o.v[i] = -v[i]; return o; }
    Vec& operator+=(const Vec& b) { for (int i = 0; i < N; i++) v[i] += b.v[i]; return *this; }
    // NVec::isZero with CUTOFF 1e-8 (NVec.h:4,12-19)
    bool isZero() const { for (int i = 0; i < N; i++) if (std::abs(v[i]) > 0.00000001) return false; return true; }
};
template <int R, int C>
inline Vec<R> mul(const Mat<R, C>& m, const Vec<C>& x) {
    Vec<R> o;
    for (int i = 0; i < R; i++) { o.v[i] = 0; for (int j = 0; j < C; j++) o.v[i] += x.v[j] * m.v[i][j]; }
    return o;
}
template <int N>
inline Vec<N> scale(double d, const Vec<N>& x) { Vec<N> o; for (int i = 0; i < N; i++) o.v[i] = x.v[i] * d; return o; }
template <int R, int C, int r, int c>
inline void put(Mat<R, C>& dst, const Mat<r, c>& src, int row, int col) {
    for (int i = 0; i < r; i++) for (int j = 0; j < c; j++) dst.v[i + row][j + col] = src.v[i][j];
}
// rowMajorOrderInverse<1..3> (NMat.cpp:5-34)
inline Mat<1, 1> inverse(const Mat<1, 1>& a) { Mat<1, 1> o; o.v[0][0] = 1.0 / a.v[0][0]; return o; }
inline Mat<2, 2> inverse(const Mat<2, 2>& s) {
    double a = s.v[0][0], b = s.v[0][1], c = s.v[1][0], d = s.v[1][1];
    double di = 1.0 / (a * d - b * c);
    Mat<2, 2> o;
    o.v[0][0] = d * di; o.v[0][1] = -b * di; o.v[1][0] = -c * di; o.v[1][1] = a * di;
    return o;
}
inline Mat<3, 3> inverse(const Mat<3, 3>& s) {
    double a = s.v[0][0], b = s.v[0][1], c = s.v[0][2], d = s.v[1][0], e = s.v[1][1], f = s.v[1][2], g = s.v[2][0], h = s.v[2][1], i = s.v[2][2];
    double di = 1.0 / (a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g));
    Mat<3, 3> o;
    o.v[0][0] = (e * i - f * h) * di; o.v[0][1] = (c * h - b * i) * di; o.v[0][2] = (b * f - c * e) * di;
    o.v[1][0] = (f * g - d * i) * di; o.v[1][1] = (a * i - c * g) * di; o.v[1][2] = (c * d - a * f) * di;
    o.v[2][0] = (d * h - e * g) * di; o.v[2][1] = (b * g - a * h) * di; o.v[2][2] = (a * e - b * d) * di;
    return o;
}
inline Mat<3, 3> toMat(const M3& a) { Mat<3, 3> o; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.v[i][j] = a.m[i][j]; return o; }
inline Mat<3, 3> skew(const V3& v) { Mat<3, 3> o; o.v[0][1] = -v.z; o.v[0][2] = v.y; o.v[1][0] = v.z; o.v[1][2] = -v.x; o.v[2][0] = -v.y; o.v[2][1] = v.x; return o; }

// constants of CollisionDetect.h:20-25 and Quaternion.h:4
constexpr double PI_FULL = 3.14159265358979323846;
constexpr double PI_TRUNC = 3.1415926535;
inline double tolAng() { return 1 * PI_FULL / 180; }
inline double cosTol() { return 1 - std::cos(tolAng()); }
inline double sinTol() { return std::sin(tolAng()); }

// ------------------------------------------------------------ geometry ----
struct AABB {
    V3 mn, mx;
    // inclusive overlap (AABB.h:10-14)
    static bool overlap(const AABB& a, const AABB& b) {
        return !(a.mx.x < b.mn.x || a.mn.x > b.mx.x || a.mx.y < b.mn.y || a.mn.y > b.mx.y || a.mx.z < b.mn.z || a.mn.z > b.mx.z);
    }
};

struct Extrema {
    int min_id = -1, max_id = -1;
    double min_v = std::numeric_limits<double>::infinity();
    double max_v = -std::numeric_limits<double>::infinity();
};

struct Material { double density = 1.0, restitution = 0.3, kinetic = 0.6, stat = 1.1; };

// A convex polyhedron with the derived data of Polyhedron::Polyhedron
// (ConvexPrimitive.cpp:582-658) and its Gauss map (:861-896).
struct Hull {
    std::vector<V3> pts;
    V3 interior;
    std::vector<std::vector<int>> faces;    // vertex indices, anticlockwise
    std::vector<int> face_nci;              // normal_calc_index
    std::vector<int> face_dir;              // normalDirection
    std::vector<int> face_id;               // surfaceID (= n_points + index)
    std::vector<std::pair<int, int>> edges; // (p1, p2)
    std::vector<std::vector<int>> vert_faces, vert_edges;
    // Gauss map
    std::vector<V3> gv;                     // face normals
    std::vector<char> g_redundant;
    std::vector<Extrema> g_cache;           // cached findExtrema along the normal
    std::vector<int> g_ref_idx;
    std::vector<double> g_ref_val;
    std::vector<std::pair<int, int>> arcs;

    V3 faceNormal(int f) const;             // Surface::normal (ConvexPrimitive.cpp:817-823)
    void build(const std::vector<V3>& points, const std::vector<std::vector<int>>& face_idx);
};
Extrema findExtrema(const Hull& h, const V3& axis);

// Sphere (ConvexPrimitive.h:79-109) and cylinder (:160-210) primitives
struct SphereG { V3 c; double r = 0; };
struct CylG {
    V3 c, axis;
    double r = 0, h = 0;
    std::vector<V3> gv;                       // Gauss vertices (2 caps + 12 around)
    std::vector<std::pair<int, int>> arcs;    // 24 arcs, as the constructor builds them
    std::vector<V3> top, bot;                 // 8-gon approximations of the caps
    V3 topCenter() const { return c + 0.5 * h * axis; }
    V3 botCenter() const { return c - 0.5 * h * axis; }
};
// Capsule (ConvexPrimitive.h:107-141): centre, radius, drum height (the
// distance between the two cap-sphere centres) and height axis
struct CapG { V3 c, axis; double r = 0, h = 0; };
enum Kind { K_HULL = 0, K_SPHERE = 1, K_CYLINDER = 2, K_MESH = 3, K_CAPSULE = 4, K_UNION = 5 };

// StaticMeshFace (Geometry.h:74-86) as built by StaticMeshGeometry's
// constructor (Geometry.cpp:675-820)
struct MeshTri {
    V3 normal;
    V3 v[3];
    int vid[3] = {0, 0, 0};
    V3 ep1[3], ep2[3], out[3];   // edges (p1, p2) and outward directions in the face plane
    int eid[3] = {0, 0, 0};
    std::vector<V3> gauss;       // gauss_region
    int concave = 0;             // concave_neighbor_count
    int id = 0;
    AABB aabb;
};

// AABBTree<unsigned int> (AABB_Tree.h) with margin 0 and the surface-area
// cost, filled by add() in triangle order as the mesh copy constructor does
// (Geometry.cpp:660-666); candidates() is getCollisionCandidatesWith.
struct MeshTree {
    struct Node { int parent = -1, left = -1, right = -1; bool leaf = false; int obj = -1; AABB box, true_box; double cost = 0; };
    std::vector<Node> nodes;
    int root = -1;
    void add(int obj, const AABB& b);
    std::vector<int> candidates(const AABB& target) const;
};
CylG makeCylinder(V3 center, double radius, double height);

// --------------------------------------------------------------- world ----
enum Movement { DYNAMIC = 0, FIXED = 1, KINEMATIC = 2 };

struct Body {
    uint32_t id = 0;
    int movement = DYNAMIC;
    Material mat;
    int kind = K_HULL;
    Hull ref_shape;       // COM-centred reference geometry
    Hull shape;           // world geometry (points and Gauss normals follow the pose)
    SphereG sph_src, sph_ref, sph;
    CylG cyl_src, cyl_ref, cyl;
    CapG cap_src, cap_ref, cap;
    // several primitives (ConvexUnionGeometry): each part holds one primitive's
    // kind, material, source / reference / world geometry and AABB; its id
    // (body id << 8 | index) names it in contact ids
    std::vector<std::unique_ptr<Body>> parts;
    std::vector<MeshTri> tris;    // static mesh (world coordinates)
    MeshTree tree;
    AABB aabb;
    V3 com, vel, ang_vel, pvel, pang_vel, prev_com;
    Q q, prev_q;
    double mass = 0;
    M3 tensor, inv_tensor, ref_tensor, ref_inv_tensor;
    std::vector<V3> track_p;
    std::set<const Body*> no_collide;   // no_collision_set (RigidBody.h), filled by joints
    // sleeping (RigidBody.h: asleep, sleep_ready_counter, non_sleepy_tick_count,
    // history, recievedWakingAction; RigidBody.cpp:318-352)
    bool asleep = false, waking = false;
    double sleep_ready = 0;
    int non_sleepy = 0;
    std::vector<std::pair<V3, V3>> history;   // (vel, ang_vel) of the last steps
    bool getAsleep() const { return asleep && movement == DYNAMIC; }
    void sleep() { if (movement != DYNAMIC) return; asleep = true; vel = V3(); ang_vel = V3(); }
    void wake() { if (asleep) { asleep = false; sleep_ready = 0; non_sleepy = 0; history.clear(); } }
    void alertWaking() { waking = true; sleep_ready = 0; non_sleepy = 0; history.clear(); }
    V3 local_origin;
    Hull src_shape;       // geometry as given at creation (geometry frame)
    V3 create_pos;
    double invMass() const { return movement == DYNAMIC ? 1.0 / mass : 0; }
    M3 invTensor() const { return movement == DYNAMIC ? inv_tensor : M3(); }
    V3 getVel() const { return movement == FIXED ? V3() : vel; }
    V3 getAngVel() const { return movement == FIXED ? V3() : ang_vel; }
    V3 trackedP(int k) const { return com + q.rotate(track_p[k]); }
    void updateGeometry();
    void updateInertiaTensor();
    void rotateWithGyro(double dt, int n_itr, bool gyro_disabled);
};

struct DV { Vec<6> v, pv, lin_err; };   // VelPair (ConstraintSolver.cpp:83-89)

// A joint row: DegreedConstraint<n> (ConstraintSolver.h:60-144) for n = 3
// (BallSocketConstraint) or 5 (HingeConstraint), stored at the largest size
// with every loop bounded by n, in the reference's accumulation order.
constexpr int kMaxDof = 6;
// impulses per joint in the joint-state layout of cpgpu_get/set_joint_state
// (the largest row, a weld's, has 6)
constexpr int kStateDof = 6;
struct JRow {
    int n = 3;
    Body* a = nullptr; Body* b = nullptr;
    DV* da = nullptr; DV* db = nullptr;
    bool in_holo = false;
    int proj = 0;                 // 1 / 2: accumulated impulse kept >= 0 / <= 0 (projectValidImpulse);
                                  // 3: powered rows, x > 0 ? min(x, lim) : max(x, -lim)
    double lim = 0;               // proj 3: the motor's or piston's impulse bound
    bool has_vt = false;          // motor / piston: target = vt - value (findTargetConstraintValue)
    double vt = 0;
    bool pos = true;              // needsPosCorrect: solved in the position passes
    double impulse[kMaxDof] = {}, pimpulse[kMaxDof] = {}, holo[kMaxDof] = {};
    double target[kMaxDof] = {}, ptarget[kMaxDof] = {};
    double ja[kMaxDof][6] = {}, jb[kMaxDof][6] = {};
    double ita[6][kMaxDof] = {}, itb[6][kMaxDof] = {};
    double itv[kMaxDof][kMaxDof] = {}, minv[kMaxDof][kMaxDof] = {};
};

struct Edge;
struct Params;
// BallSocket / Hinge (PersistentConstraint.h:118-313)
struct Joint {
    int n = 3;                    // 1 distance, 3 ball-socket, 4 sliding hinge, 5 hinge or slider, 6 weld
    bool slider = false;          // n == 5: SliderConstraint rows instead of HingeConstraint's
    // ConeRotationLimit (PersistentConstraint.h:145-172): one inequality row,
    // present only while the axes' angle is at or past max_angle; not
    // holonomic, no tracked points
    bool cone = false;
    double max_angle = 0;
    bool inactive = true;
    // TwistLimit (PersistentConstraint.h:174-215): as the cone, for the twist
    // angle about the axes, tracked across ticks in cur_angle
    bool twist = false;
    double min_angle = 0, cur_angle = 0;
    V3 u_local, w_local;          // b1's perpendicular basis (w first, as the reference)
    // Motor (PersistentConstraint.h:253-275) on a hinge's or sliding hinge's
    // axis; Piston (:217-251) on a slider's or sliding hinge's axis, held as two
    // joints: its slide limit, then its powered row (addSolverConstraints
    // lists them in that order)
    bool motor = false, slide_limit = false, piston = false;
    int seq = -1;                 // constraint id: PhysicsEngine's nextConstraintID order over joints and springs, from 0
    int mode = 0;                 // PoweredConstraitMode: 0 off, 1 constant torque / force, 2 target velocity, 3 target position
    double power_max = 0;         // max_torque / max_force
    double target_vel = 0, target_pos = 0;
    double lim_min = 0, lim_max = 0;   // motor angles / slide positions
    double position = 0;          // motor_angular_position / piston_position
    double prev_vel = 0;          // motor: prev_velocity (never written for a piston)
    bool exceeded = false;        // piston: slide_limit_exceeded of the last rebuild
    V3 ref_u, ref_w, cmp;         // motor: body 1's u, w reference axes, body 2's comparison axis (body space)
    bool powered() const { return motor || slide_limit || piston; }
    bool holonomic() const { return !cone && !twist && !powered(); }
    // addSolverConstraints: whether the joint's row is listed in its island
    bool listed() const {
        if (cone || twist) return !inactive;
        if (motor) return (mode != 0 && power_max != 0) || position < lim_min || position > lim_max;
        if (slide_limit) return exceeded;
        if (piston) return mode != 0 && power_max != 0;
        return true;
    }
    double motorPosition(const V3& axis, const V3& w1, const V3& w2, double dts) const;
    double motorTargetVelocity(const V3& axis, const V3& w1, const V3& w2) const;
    double pistonTargetVelocity(const V3& axis) const;
    double target = 0;            // distance: the attachment points' distance
    Body* b1 = nullptr; Body* b2 = nullptr;
    int k1 = 0, k2 = 0;           // tracked point keys
    V3 ax1, ax2;                  // hinge axes in body space (normalised)
    double pos_hard = 15000, rot_hard = 15000;
    JRow row;
    V3 u, w;                      // HingeConstraint::u / w of the last rebuild
    Edge* edge = nullptr;
    void rebuild(const Params& p, double dt_sub, bool in_holo);
};

// HolonomicSystem (HolonomicBlockSolver.cpp:11-132): constraint order chosen
// by minimum fill, block-sparse LDL^T of J M^-1 J^T
struct HoloSys {
    std::vector<Edge*> member_edges;
    bool changed = false;
    std::vector<JRow*> cons;      // elimination order
    int degree = 0;
    std::vector<int> table;       // block_location_table
    std::vector<int> vpos;        // vector_location_lookup
    std::vector<double> buf;      // blocks, then the diagonal-element scratch
    int cap = 0, dcap = 0;
    void build(const std::vector<JRow*>& og);
    int loc(int row, int col) const;
    int firstBelow(int col) const;
    int dloc(int row, int col) const;
    void computeInverse(double cfm);
    void solve(std::vector<double>& v) const;
    void computeAndApply(bool pseudo, double lin_err_threshold);
    double inverseError(double cfm) const;
};

// one solver row of the reference's DegreedConstraint<n> (ConstraintSolver.h:60-144)
template <int N>
struct Row {
    Body* a = nullptr; Body* b = nullptr;
    DV* da = nullptr; DV* db = nullptr;
    Vec<N> impulse, pimpulse, target, ptarget;
    Mat<N, 6> ja, jb;
    Mat<6, N> ita, itb;
    Mat<N, N> minv;
    Vec<N> value(const Vec<6>& va, const Vec<6>& vb) const { return mul(ja, va) + mul(jb, vb); }
    void applyImpulse(const Vec<N>& imp, Vec<6>* va, Vec<6>* vb) const { *va += mul(ita, imp); *vb += mul(itb, imp); }
};

struct Contact {
    Body* b1; Body* b2;
    V3 p1_local, p2_local, n_local;
    double pen, bounce, hardness, friction_coeff, cutoff;
    uint64_t magic_c, magic_b;
    int life;
    bool live;
    Row<1> normal;       // ContactConstraint
    Row<2> friction;     // FrictionConstraint
    V3 fu, fw;           // friction basis of the last rebuild
    bool static_ready = false;
    bool friction_built = false;
};

// Spring (PersistentConstraint.h:411-434): not a solver row; an impulse pair
// applied at the start of every substep
struct Spring {
    int seq = -1;                 // constraint id (creation order among joints and springs, from 0)
    Body* b1; Body* b2;
    int k1, k2;                   // tracked point keys
    double stiffness, damping, rest;
};

struct Edge {
    Body* n1; Body* n2;                       // n1 = node the edge was created from
    // SharedConstraintsEdge::constraints: joints are listed before contacts
    // (a joint forbids contacts between its bodies from then on)
    std::vector<Joint*> joints;
    std::vector<std::unique_ptr<Contact>> contacts;
    std::vector<Spring*> springs;
    HoloSys* h = nullptr;                     // holonomic system of the edge
    bool scan_needed = false;                 // holonomic_system_scan_needed
    Body* other(Body* x) const { return x == n1 ? n2 : n1; }
};

// kind 0 = normal row, 1 = friction row (of contact c), 2 = joint row (j)
struct RowRef { int kind; Contact* c; Joint* j = nullptr; };

struct Params {
    double dt = 1.0 / 90;
    V3 g = V3(0, -6, 0);
    int substeps = 8, pgs_vel = 4, pgs_pos = 1, pgs_holo = 1;
    double cfm = 0.0000025;
    int contact_life = 6;
    double hardness = 1000;
    int angle_ticks = 4;
    bool gyro_disabled = false;
    bool warm_start_disabled = false;
    bool sleeping = true;
    // sleep parameters (PhysicsEngine.h:219-224)
    double sleep_delay = 0.5;
    int non_sleepy_threshold = 3;
    double vel_sleep_coeff = 0.1, ang_vel_eps = 0.1, accel_sleep_coeff = 0.044;
    double lin_err_threshold = 15;   // excessive_linear_error_torque_threshold (PhysicsEngine.h:217)
    double cutoff_vel = 0;   // set by setStep_time / setGravity (PhysicsEngine.cpp:1142-1145,1214-1217)
};

struct ManifoldPoint { V3 pos; double pen, restitution, kinetic, stat; uint64_t magic_c, magic_b; };
struct Manifold { std::vector<ManifoldPoint> pts; V3 normal; double max_pen = -1; };

struct World {
    Params p;
    std::vector<std::unique_ptr<Body>> bodies;
    std::unordered_map<unsigned int, Body*> nodes;            // constraint_graph_nodes (iteration order matters)
    std::unordered_map<Body*, std::vector<Edge*>> adj;        // node -> edges sorted by other id
    std::vector<std::unique_ptr<Edge>> edges;
    std::vector<std::pair<uint32_t, uint32_t>> last_pairs;
    std::vector<std::unique_ptr<Joint>> joints;
    std::vector<std::unique_ptr<Spring>> springs;
    std::vector<std::unique_ptr<HoloSys>> systems;

    Body* addHull(const std::vector<V3>& pts, const std::vector<std::vector<int>>& faces, const Material& m, int movement, V3 pos);
    Body* addSphere(V3 center, double r, const Material& m, int movement, V3 pos);
    Body* addCylinder(V3 base, double r, double h, const Material& m, int movement, V3 pos);
    Body* addCapsule(V3 bot, double r, double h, const Material& m, int movement, V3 pos);
    Body* addUnion(std::vector<std::unique_ptr<Body>> parts, int movement, V3 pos);
    Body* finishBody(std::unique_ptr<Body> b, double mass, const V3& com, const M3& tensor);
    Body* addMesh(const std::vector<V3>& points, const std::vector<std::array<int, 3>>& tris, const Material& m);
    void placeBody(Body* b, double mass, const V3& com_geom, const M3& tensor);
    Edge* edgeBetween(Body* a, Body* b);
    Edge* getOrCreateEdge(Body* a, Body* b);
    void deleteEdge(Edge* e);
    void addContact(Body* b1, Body* b2, const ManifoldPoint& mp, const V3& n);
    Joint* addJoint(int n, Body* b1, Body* b2, V3 p1, V3 p2, V3 ax1, V3 ax2, double pos_hard, double rot_hard,
                    double target = -1);
    void maintainHolonomicSystems();
    void applySprings(double dt_sub);
    Joint* addTwist(Body* b1, Body* b2, V3 ax1, V3 ax2, double min_angle, double max_angle, double rot_hard);
    Joint* addMotor(Joint* base, double min_angle, double max_angle);
    int constraint_seq = 0;       // PhysicsEngine::nextConstraintID (PhysicsEngine.h:301)
    // the joint a constraint id names (a piston's two joints share its id:
    // the powered one, created last)
    Joint* jointById(uint32_t id) {
        Joint* out = nullptr;
        for (auto& j : joints) if (j->seq == (int)id) out = j.get();
        return out;
    }
    Joint* addPiston(Joint* base, double min_pos, double max_pos);
    Joint* addCone(Body* b1, Body* b2, V3 ax1, V3 ax2, double max_angle, double rot_hard);
    Spring* addSpring(Body* b1, Body* b2, V3 p1, V3 p2, double damping, double stiffness, double rest);
    void holonomicScan(Edge* e);
    void updateHolonomicInverses();
    void step();
    bool bodySleepy(const Body* b) const;
    bool readyToSleep(const Body* b) const;
    void wakeupIsland(Body* foothold);
    void applyVelocityChange(Body* b, const V3& dv, const V3& dw, const V3& dpv, const V3& dpw);
};

void jrowTarget(JRow& r);
void jrowWarm(JRow& r);
void jrowStep(JRow& r, bool pseudo);
void jrowApply(const JRow& r, const double* imp, Vec<6>* va, Vec<6>* vb);

Manifold satPolyPoly(const Hull& a, uint32_t a_id, const Material& am, const Hull& b, uint32_t b_id, const Material& bm);
Manifold satPolySphere(const Hull& a, uint32_t a_id, const Material& am, const SphereG& b, uint32_t b_id, const Material& bm);
Manifold satPolyCylinder(const Hull& a, uint32_t a_id, const Material& am, const CylG& b, uint32_t b_id, const Material& bm);
Manifold sphereSphere(const SphereG& a, uint32_t a_id, const Material& am, const SphereG& b, uint32_t b_id, const Material& bm);
Manifold sphereCylinder(const SphereG& a, uint32_t a_id, const Material& am, const CylG& b, uint32_t b_id, const Material& bm);
Manifold cylinderCylinder(const CylG& a, uint32_t a_id, const Material& am, const CylG& b, uint32_t b_id, const Material& bm);
Manifold sphereCapsule(const SphereG& a, uint32_t a_id, const Material& am, const CapG& b, uint32_t b_id, const Material& bm);
Manifold capsuleCapsule(const CapG& a, uint32_t a_id, const Material& am, const CapG& b, uint32_t b_id, const Material& bm);
Manifold satPolyCapsule(const Hull& a, uint32_t a_id, const Material& am, const CapG& b, uint32_t b_id, const Material& bm);
Manifold capsuleCylinder(const CapG& a, uint32_t a_id, const Material& am, const CylG& b, uint32_t b_id, const Material& bm);
Manifold flipped(Manifold m);
std::vector<Manifold> meshCollide(const Body* convex, const Body* mesh);   // SAT_*Mesh (CollisionDetect.cpp:2648-2778)
Manifold mergeManifold(const Manifold& a, const Manifold& b);              // merge_manifold (:2780-2793)   // normal negated, MagicID halves swapped (CollisionDetect.cpp:29-40)
Manifold cullManifold(const Manifold& m, int n);
void massProperties(const Hull& h, double density, V3* com, M3* tensor, double* mass);

}  // namespace cport
