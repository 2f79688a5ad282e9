// geometry.cpp — hull preparation, mass properties, SAT narrowphase and
// contact clipping of the CPU restatement (test infrastructure; see cport.h).
#include "cport.h"

#include <functional>

namespace cport {

static const double EPS_GAUSS = 0.0000000001;  // ConvexPrimitive.cpp:10

V3 Hull::faceNormal(int f) const {
    const std::vector<int>& s = faces[f];
    V3 p1 = pts[s[0]], p2 = pts[s[1]], p3 = pts[s[face_nci[f]]];
    return (p2 - p1).cross(p3 - p2).normalize() * (double)face_dir[f];
}

// Surface::findNormalCalcInfo (ConvexPrimitive.cpp:797-815): the third point of
// the normal is the first one not (nearly) collinear with the first edge, and
// the sign makes the normal point away from the interior point.
static void normalCalcInfo(Hull& h, int f, const V3& normalish) {
    const std::vector<int>& s = h.faces[f];
    V3 p0 = h.pts[s[0]], p1 = h.pts[s[1]];
    int nci = 2;
    V3 v1 = (p1 - p0).normalize();
    V3 v2 = (h.pts[s[nci]] - p0).normalize();
    while (std::abs(v1.dot(v2)) > 0.99 && nci + 1 < (int)s.size()) v2 = (h.pts[s[++nci]] - p0).normalize();
    h.face_nci[f] = nci;
    h.face_dir[f] = 1;
    if (normalish.dot(h.faceNormal(f)) < 0) h.face_dir[f] = -1;
}

// Surface::setWindingAntiClockwise (ConvexPrimitive.cpp:834-859)
static void windAntiClockwise(Hull& h, int f, const V3& n) {
    V3 u, w;
    n.perpBasis(&u, &w);
    std::vector<int>& s = h.faces[f];
    int np = (int)s.size();
    double area = 0;
    for (int i = 0; i < np; i++) {
        V3 p1 = h.pts[s[i]], p2 = h.pts[s[(i + 1 == np) ? 0 : i + 1]];
        double p1u = p1.dot(u), p1w = p1.dot(w), p2u = p2.dot(u), p2w = p2.dot(w);
        area += (p2w - p1w) * (p2u + p1u) / 2.0;
    }
    if (area < 0) {
        std::reverse(s.begin(), s.end());
        normalCalcInfo(h, f, n);
    }
}

Extrema findExtrema(const Hull& h, const V3& axis) {
    // CollisionDetect.cpp:627-644 (strict comparisons: the first index wins ties)
    Extrema e;
    for (int i = 0; i < (int)h.pts.size(); i++) {
        double v = h.pts[i].dot(axis);
        if (v < e.min_v) { e.min_id = i; e.min_v = v; }
        if (v > e.max_v) { e.max_id = i; e.max_v = v; }
    }
    return e;
}

void Hull::build(const std::vector<V3>& points, const std::vector<std::vector<int>>& face_idx) {
    // Polyhedron::Polyhedron (ConvexPrimitive.cpp:582-658)
    pts = points;
    interior = V3();
    for (const V3& p : pts) interior += p;
    interior /= (double)pts.size();
    int nf = (int)face_idx.size();
    faces = face_idx;
    face_nci.assign(nf, 2);
    face_dir.assign(nf, 1);
    face_id.resize(nf);
    vert_faces.assign(pts.size(), {});
    vert_edges.assign(pts.size(), {});
    for (int f = 0; f < nf; f++) {
        for (int j : faces[f]) vert_faces[j].push_back(f);
        face_id[f] = (int)pts.size() + f;
        normalCalcInfo(*this, f, pts[faces[f][0]] - interior);
        windAntiClockwise(*this, f, faceNormal(f));
    }
    edges.clear();
    for (int f = 0; f < nf; f++) {
        int n = (int)faces[f].size();
        for (int i = 0; i < n; i++) {
            int a = faces[f][i], b = faces[f][(i + 1) % n];
            bool seen = false;
            for (auto& e : edges) if ((e.first == a && e.second == b) || (e.first == b && e.second == a)) { seen = true; break; }
            if (!seen) edges.push_back({a, b});
        }
    }
    for (int i = 0; i < (int)edges.size(); i++) {
        vert_edges[edges[i].first].push_back(i);
        vert_edges[edges[i].second].push_back(i);
    }
    // Polyhedron::computeGaussMap (ConvexPrimitive.cpp:861-896)
    gv.clear(); g_redundant.clear(); g_cache.clear(); g_ref_idx.clear(); g_ref_val.clear(); arcs.clear();
    for (int i = 0; i < nf; i++) {
        V3 n = faceNormal(i);
        bool red = false;
        for (const V3& g : gv) if (n.dot(g) < -1 + EPS_GAUSS) { red = true; break; }
        int ref = faces[i][0];
        gv.push_back(n);
        g_redundant.push_back(red);
        g_cache.push_back(findExtrema(*this, n));
        g_ref_idx.push_back(ref);
        g_ref_val.push_back(n.dot(pts[ref]));
        for (int j = i + 1; j < nf; j++) {
            const std::vector<int>& s1 = faces[i];
            const std::vector<int>& s2 = faces[j];
            for (size_t k = 0; k < s1.size(); k++) {
                for (size_t w = 0; w < s2.size(); w++) {
                    int a1 = s1[k], a2 = s1[(k + 1) % s1.size()], b1 = s2[w], b2 = s2[(w + 1) % s2.size()];
                    if ((a1 == b1 && a2 == b2) || (a1 == b2 && a2 == b1)) { arcs.push_back({i, j}); break; }
                }
            }
        }
    }
}

// Volume, first and second moments of a convex polyhedron by decomposition
// into tetrahedra (interior point, face fan).  Same quantities as Mirtich's
// surface-integral method used by the reference (RigidBody.cpp:427-640),
// computed differently, so results agree to rounding.
void massProperties(const Hull& h, double density, V3* com, M3* tensor, double* mass) {
    double vol = 0;
    V3 first;
    double c[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // integral of x_i x_j dV
    V3 o = h.interior;
    for (int f = 0; f < (int)h.faces.size(); f++) {
        const std::vector<int>& s = h.faces[f];
        for (size_t t = 1; t + 1 < s.size(); t++) {
            V3 p[4] = {o, h.pts[s[0]], h.pts[s[t]], h.pts[s[t + 1]]};
            double v6 = (p[1] - p[0]).dot((p[2] - p[0]).cross(p[3] - p[0]));  // 6 * signed volume
            double v = v6 / 6.0;
            V3 sum = p[0] + p[1] + p[2] + p[3];
            vol += v;
            first += sum * (v / 4.0);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    double acc = sum[i] * sum[j];
                    for (int k = 0; k < 4; k++) acc += p[k][i] * p[k][j];
                    c[i][j] += v / 20.0 * acc;
                }
        }
    }
    *mass = density * vol;
    *com = first * density / *mass;
    M3 t;
    double tr = c[0][0] + c[1][1] + c[2][2];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) t.m[i][j] = density * ((i == j ? tr : 0.0) - c[i][j]);
    // about the centre of mass (parallel axis; RigidBody.cpp:400-420)
    V3 cm = *com;
    double m = *mass;
    double cc[3] = {cm.x, cm.y, cm.z};
    double c2 = cm.mag2();
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) t.m[i][j] -= m * ((i == j ? c2 : 0.0) - cc[i] * cc[j]);
    *tensor = t;
}

// ---------------------------------------------------------------- SAT ----
struct NormResult { int a_id, b_id; V3 n; double pen; };

// sat_checknorm (CollisionDetect.cpp:705-715)
static NormResult checkNorm(const Extrema& a, const Extrema& b, const V3& n) {
    double fwd = a.max_v - b.min_v;
    double rev = b.max_v - a.min_v;
    if (fwd < rev) return {a.max_id, b.min_id, n, fwd};
    return {a.min_id, b.max_id, -n, rev};
}

static Extrema recenter(const Extrema& e, double old_ref, double new_ref) {
    double d = new_ref - old_ref;
    Extrema o = e;
    o.min_v = e.min_v + d;
    o.max_v = e.max_v + d;
    return o;
}

struct P2 { double x = 0, y = 0; };
static P2 p2(double a, double b) { P2 p; p.x = a; p.y = b; return p; }
static P2 sub(P2 a, P2 b) { return p2(a.x - b.x, a.y - b.y); }
static P2 add(P2 a, P2 b) { return p2(a.x + b.x, a.y + b.y); }
static P2 mul(P2 a, double d) { return p2(a.x * d, a.y * d); }
static double dot2(P2 a, P2 b) { double s = 0; s += a.x * b.x; s += a.y * b.y; return s; }
static P2 norm2(P2 a) { return mul(a, 1.0 / std::sqrt(dot2(a, a))); }
// getInDirOfEdge (CollisionDetect.cpp:394-397): inward normal of a CCW edge
static P2 inDir(P2 a, P2 b) { return norm2(p2(a.y - b.y, b.x - a.x)); }

enum Origin { FACE, EDGE, VERTEX };
struct Area { std::vector<P2> ps; std::vector<int> ids; int surface; Origin origin; };

// findContactArea (CollisionDetect.cpp:237-280)
static Area contactArea(const Hull& c, const V3& n, const V3& p, int pid, const V3& u, const V3& w) {
    int best_f = -1;
    double best_ft = 1.0;
    for (int f : c.vert_faces[pid]) {
        double ca = c.faceNormal(f).dot(n);
        if (1 - ca < best_ft) { best_ft = 1 - ca; best_f = f; }
    }
    if (best_ft <= cosTol()) {
        Area a;
        for (int id : c.faces[best_f]) { V3 v = c.pts[id]; a.ps.push_back(p2(v.dot(u), v.dot(w))); a.ids.push_back(id); }
        a.surface = c.face_id[best_f];
        a.origin = FACE;
        return a;
    }
    int best_e = -1;
    double best_et = 1.0;
    for (int e : c.vert_edges[pid]) {
        V3 d = c.pts[c.edges[e].second] - c.pts[c.edges[e].first];
        double sa = std::abs(d.normalize().dot(n));
        if (sa < best_et) { best_et = sa; best_e = e; }
    }
    if (best_et <= sinTol()) {
        Area a;
        V3 e1 = c.pts[c.edges[best_e].first], e2 = c.pts[c.edges[best_e].second];
        a.ps = {p2(e1.dot(u), e1.dot(w)), p2(e2.dot(u), e2.dot(w))};
        a.ids = {c.edges[best_e].first, c.edges[best_e].second};
        a.surface = -1;
        a.origin = EDGE;
        return a;
    }
    Area a;
    a.ps = {p2(p.dot(u), p.dot(w))};
    a.ids = {pid};
    a.surface = -1;
    a.origin = VERTEX;
    return a;
}

// getEdgeID (CollisionDetect.cpp:9-21): ids are truncated to 16 bits
static uint32_t edgeId(int a, int b) {
    uint16_t p1 = (uint16_t)a, p2v = (uint16_t)b;
    int mn, mx;
    if (p1 < p2v) { mn = p1; mx = p2v; } else { mn = p2v; mx = p1; }
    return (0x0000FFFFu & (uint32_t)mn) + (0xFFFF0000u & ((uint32_t)mx << 16));
}

struct ClipP { P2 pos; int32_t src; uint64_t magic; bool skip; };

static uint64_t packMagic(uint64_t lo, uint64_t hi) {
    return (0x00000000FFFFFFFFull & lo) | (0xFFFFFFFF00000000ull & (hi << 32));
}

static bool windingCCW(const Area& c) {
    P2 in = inDir(c.ps[0], c.ps[1]);
    for (size_t i = 2; i < c.ps.size(); i++) {
        double d = dot2(sub(c.ps[i], c.ps[0]), in);
        if (d > 0.0000000001) return true;
        if (d < -0.0000000001) return false;
    }
    return false;
}

// createClipEvaluationPoly (CollisionDetect.cpp:441-460)
static std::vector<ClipP> clipPoly(const Area& c, uint32_t other_surface, bool flip) {
    std::vector<ClipP> out;
    for (size_t i = 0; i < c.ps.size(); i++) {
        uint64_t id = (uint64_t)(int64_t)c.ids[i];
        uint64_t m = flip ? packMagic(other_surface, id) : packMagic(id, other_surface);
        out.push_back({c.ps[i], c.ids[i], m, false});
    }
    if (c.ps.size() > 2 && !windingCCW(c)) std::reverse(out.begin(), out.end());
    return out;
}

// getEdgeIntersectionWithClippingEdge (CollisionDetect.cpp:462-487)
static ClipP intersect(const ClipP& e1, const ClipP& e2, P2 nrm, P2 sample, int32_t clip_edge, bool flip) {
    P2 d = sub(e2.pos, e1.pos);
    P2 pos = add(e1.pos, mul(d, dot2(nrm, sub(sample, e1.pos)) / dot2(nrm, d)));
    bool e2_kept = dot2(d, nrm) > 0;
    int32_t src = e2_kept ? e1.src : e2.src;
    uint64_t eid = edgeId(e1.src, e2.src);
    uint64_t ce = (uint64_t)(int64_t)clip_edge;
    uint64_t m = flip ? packMagic(ce, eid) : packMagic(eid, ce);
    return {pos, src, m, !e2_kept};
}

enum ClipRes { BOTH, P1_ON_P2_CLIPPED, P2_ON_P1_CLIPPED, NEITHER, ONLY_P1, ONLY_P2 };
static ClipRes checkSegment(double a, double b, double c) {
    if (a >= c && b >= c) return NEITHER;
    if (a == c && b < c) return P1_ON_P2_CLIPPED;
    if (a < c && b == c) return P2_ON_P1_CLIPPED;
    if (a < c && b >= c) return ONLY_P1;
    if (a >= c && b < c) return ONLY_P2;
    return BOTH;
}

// getClipEvaluatinPolyAfterClippingByEdge (CollisionDetect.cpp:500-576)
static std::vector<ClipP> clipByEdge(const std::vector<ClipP>& c, P2 side, P2 sample, int32_t eid, bool flip) {
    std::vector<ClipP> out;
    double cv = dot2(sample, side);
    if (c.size() >= 3) {
        double v1 = 0, v2 = 0;
        ClipP q1, q2;
        for (size_t i = 0; i < c.size(); i++) {
            if (i > 0) { v1 = v2; q1 = q2; }
            else { q1 = c[0]; v1 = dot2(q1.pos, side); }
            q2 = c[(i + 1) % c.size()];
            v2 = dot2(q2.pos, side);
            ClipRes r = checkSegment(v1, v2, cv);
            if (r == NEITHER || r == P1_ON_P2_CLIPPED) out.push_back(q1);
            else if (r == ONLY_P2) { out.push_back(q1); out.push_back(intersect(q1, q2, side, sample, eid, flip)); }
            else if (r == ONLY_P1) out.push_back(intersect(q1, q2, side, sample, eid, flip));
        }
        return out;
    }
    if (c.size() == 2) {
        double v1 = dot2(c[0].pos, side), v2 = dot2(c[1].pos, side);
        ClipRes r = checkSegment(v1, v2, cv);
        if (r == NEITHER) return c;
        if (r == P1_ON_P2_CLIPPED) return {c[0]};
        if (r == P2_ON_P1_CLIPPED) return {c[1]};
        if (r == ONLY_P1) return {intersect(c[0], c[1], side, sample, eid, flip), c[1]};
        if (r == ONLY_P2) return {c[0], intersect(c[0], c[1], side, sample, eid, flip)};
        return out;
    }
    if (dot2(c[0].pos, side) >= cv) return c;
    return out;
}

static std::vector<ClipP> clipByAll(std::vector<ClipP> c1, const std::vector<ClipP>& c2, bool flip) {
    for (size_t i = 0; i < c2.size(); i++) {
        const ClipP& e1 = c2[i];
        if (e1.skip) continue;
        const ClipP& e2 = c2[(i + 1) % c2.size()];
        c1 = clipByEdge(c1, inDir(e1.pos, e2.pos), e1.pos, (int32_t)edgeId(e1.src, e2.src), flip);
        if (c1.empty()) return c1;
    }
    return c1;
}

// clipContacts (CollisionDetect.cpp:578-620)
static std::vector<ClipP> clipContacts(const Area& c1, const Area& c2) {
    std::vector<ClipP> p1 = clipPoly(c1, (uint32_t)c2.surface, false);
    std::vector<ClipP> p2v = clipPoly(c2, (uint32_t)c1.surface, true);
    if (p1.size() == 1) return p1;
    if (p2v.size() == 1) return p2v;
    if (p1.size() == 2 && p2v.size() == 2) {
        P2 nrm = inDir(p2v[0].pos, p2v[1].pos);
        return {intersect(p1[0], p1[1], nrm, p2v[0].pos, (int32_t)edgeId(p2v[0].src, p2v[1].src), false)};
    }
    if (p1.size() == 2) return clipByAll(p1, p2v, false);
    if (p2v.size() == 2) return clipByAll(p2v, p1, true);
    p1 = clipByAll(p1, p2v, false);
    return clipByAll(p2v, p1, true);
}

// SAT_PolyPoly (CollisionDetect.cpp:717-835)
Manifold satPolyPoly(const Hull& a, uint32_t a_id, const Material& am, const Hull& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    for (size_t f = 0; f < a.gv.size(); f++) {
        if (a.g_redundant[f]) continue;
        Extrema ea = recenter(a.g_cache[f], a.g_ref_val[f], a.gv[f].dot(a.pts[a.g_ref_idx[f]]));
        NormResult x = checkNorm(ea, findExtrema(b, a.gv[f]), a.gv[f]);
        if (x.pen < 0) { out.max_pen = -1; return out; }
        if (x.pen < best.pen) best = x;
    }
    for (size_t f = 0; f < b.gv.size(); f++) {
        if (b.g_redundant[f]) continue;
        Extrema eb = recenter(b.g_cache[f], b.g_ref_val[f], b.gv[f].dot(b.pts[b.g_ref_idx[f]]));
        NormResult x = checkNorm(findExtrema(a, b.gv[f]), eb, b.gv[f]);
        if (x.pen < 0) { out.max_pen = -1; return out; }
        if (x.pen < best.pen) best = x;
    }
    for (auto& arc1 : a.arcs) {
        for (auto& arc2 : b.arcs) {
            V3 a1 = a.gv[arc1.first], a2 = a.gv[arc1.second];
            V3 b1 = -b.gv[arc2.first], b2 = -b.gv[arc2.second];
            V3 avg = a1 + a2;
            if (avg.dot(b1) + avg.dot(b2) <= 0) continue;
            V3 ap = a1.cross(a2), bp = b1.cross(b2);
            if (ap.dot(b1) * ap.dot(b2) > 0 || bp.dot(a1) * bp.dot(a2) > 0) continue;
            V3 n = ap.cross(bp);
            if (n.mag2() == 0) continue;
            n = n.normalize();
            if (avg.dot(n) < 0) n *= -1;
            NormResult x = checkNorm(findExtrema(a, n), findExtrema(b, n), n);
            if (x.pen < 0) { out.max_pen = -1; return out; }
            if (x.pen < best.pen) best = x;
        }
    }
    out.normal = best.n;
    V3 n = best.n;
    V3 amax = a.pts[best.a_id], bmax = b.pts[best.b_id];
    V3 u, w;
    n.perpBasis(&u, &w);
    Area ac = contactArea(a, n, amax, best.a_id, u, w);
    Area bc = contactArea(b, (-1) * n, bmax, best.b_id, u, w);
    std::vector<ClipP> pool = clipContacts(ac, bc);
    double a_dot = amax.dot(n);
    V3 off = n * a_dot;
    uint64_t cid = (0x00000000FFFFFFFFull & (uint64_t)a_id) | (0xFFFFFFFF00000000ull & ((uint64_t)b_id << 32));
    for (const ClipP& p : pool) {
        ManifoldPoint mp;
        mp.pos = u * p.pos.x + w * p.pos.y + off;
        mp.pen = mp.pos.dot(n) - a_dot + best.pen;
        mp.restitution = std::max(am.restitution, bm.restitution);
        mp.kinetic = (am.kinetic + bm.kinetic) / 2.0;
        mp.stat = (am.stat + bm.stat) / 2.0;
        mp.magic_c = cid;
        mp.magic_b = p.magic;
        out.pts.push_back(mp);
    }
    out.max_pen = best.pen;
    return out;
}

// ---------------------------------------------- spheres and cylinders ----
// Cylinder::Cylinder (ConvexPrimitive.cpp:222-256) for the default axis (0,1,0),
// 12 Gauss ring vertices and 8-gon cap approximations.  The arcs are built as
// the constructor builds them: {0, i} and {1, i} for i in [0, 12).
CylG makeCylinder(V3 center, double radius, double height) {
    CylG c;
    c.c = center; c.axis = V3(0, 1, 0); c.r = radius; c.h = height;
    M3 rot = M3::iden();
    c.gv.resize(14);
    c.gv[0] = rot * V3(0, 1, 0);
    c.gv[1] = rot * V3(0, -1, 0);
    double dth = 2 * PI_TRUNC / 12;
    for (int i = 0; i < 12; i++) {
        double th = i * dth;
        c.gv[i + 2] = rot * V3(std::sin(th), 0, std::cos(th));
    }
    c.arcs.resize(24);
    for (int i = 0; i < 12; i++) { c.arcs[2 * i] = {0, i}; c.arcs[2 * i + 1] = {1, i}; }
    double fth = 2 * PI_TRUNC / 8;
    double er = radius / std::cos(PI_TRUNC / 8);
    c.top.resize(8); c.bot.resize(8);
    for (int i = 0; i < 8; i++) {
        double th = i * fth;
        c.top[i] = center + rot * V3(er * std::sin(th), height / 2.0, er * std::cos(th));
        c.bot[i] = center + rot * V3(er * std::sin(th), -height / 2.0, er * std::cos(th));
    }
    return c;
}

static Extrema sphereExtrema(const SphereG& s, const V3& d) {   // getSphereExtrema (CollisionDetect.cpp:646-655)
    Extrema e;
    double cv = d.dot(s.c);
    e.max_v = cv + s.r;
    e.min_v = cv - s.r;
    e.min_id = e.max_id = -1;
    return e;
}

// Cylinder::getExtremaOfDisk (ConvexPrimitive.cpp:319-355)
static V3 diskExtremum(V3 center, V3 normal, double r, V3 target) {
    if (std::abs(normal.dot(target)) > 0.99999999) return center;
    if (std::abs(normal.dot(target)) < 0.00000001) return center + target * r;
    V3 u, v, w;
    w = target;
    target.perpBasis(&u, &v);
    V3 uvw_n(normal.dot(u), normal.dot(v), normal.dot(w));
    double dwdu = -uvw_n.x / uvw_n.z;
    double dwdv = -uvw_n.y / uvw_n.z;
    double gm = std::sqrt(dwdu * dwdu + dwdv * dwdv);
    double gu = dwdu / gm, gv = dwdv / gm;
    double uv2 = r * r / (1 + gm * gm);
    double dw = std::sqrt(r * r - uv2);
    double du = gu * std::sqrt(uv2), dv = gv * std::sqrt(uv2);
    return center + u * du + v * dv + w * dw;
}

static Extrema cylinderExtrema(const CylG& c, const V3& d) {   // getCylinderExtrema (CollisionDetect.cpp:657-683)
    V3 tc = c.topCenter();
    V3 tmax = diskExtremum(tc, c.axis, c.r, d);
    V3 tmin = 2 * tc - tmax;
    V3 bmax = 2 * c.c - tmin;
    V3 bmin = 2 * c.c - tmax;
    double a = d.dot(tmax), b = d.dot(tmin), e = d.dot(bmax), f = d.dot(bmin);
    Extrema x;
    x.max_v = std::max<double>(a, e);
    x.min_v = std::min<double>(b, f);
    x.min_id = x.max_id = -1;
    return x;
}

// apply one candidate axis: returns true when it separates
static bool axisTest(const Extrema& a, const Extrema& b, const V3& n, NormResult* best) {
    NormResult x = checkNorm(a, b, n);
    if (x.pen < 0) return true;
    if (x.pen < best->pen) *best = x;
    return false;
}

static ManifoldPoint mkPoint(const V3& pos, double pen, const Material& am, const Material& bm, uint64_t cid, uint64_t bid) {
    ManifoldPoint mp;
    mp.pos = pos;
    mp.pen = pen;
    mp.restitution = std::max(am.restitution, bm.restitution);
    mp.kinetic = (am.kinetic + bm.kinetic) / 2.0;
    mp.stat = (am.stat + bm.stat) / 2.0;
    mp.magic_c = cid;
    mp.magic_b = bid;
    return mp;
}

static uint64_t cidOf(uint32_t a, uint32_t b) {
    return (0x00000000FFFFFFFFull & (uint64_t)a) | (0xFFFFFFFF00000000ull & ((uint64_t)b << 32));
}

Manifold flipped(Manifold m) {
    m.normal = -m.normal;
    for (ManifoldPoint& p : m.pts) {
        uint64_t c1 = p.magic_c & 0xFFFFFFFFull, c2 = p.magic_c >> 32, b1 = p.magic_b & 0xFFFFFFFFull, b2 = p.magic_b >> 32;
        p.magic_c = c2 | (c1 << 32);
        p.magic_b = b2 | (b1 << 32);
    }
    return m;
}

// detectSphereSphere (CollisionDetect.cpp:837-866)
Manifold sphereSphere(const SphereG& a, uint32_t a_id, const Material& am, const SphereG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    V3 diff = b.c - a.c;
    double dist = diff.mag();
    out.max_pen = a.r + b.r - dist;
    if (out.max_pen < 0) return out;
    out.normal = diff.normalize();
    out.pts.push_back(mkPoint(a.c + out.normal * a.r, out.max_pen, am, bm, cidOf(a_id, b_id), 0));
    return out;
}

// SAT_PolySphere (CollisionDetect.cpp:1336-1411): face, vertex and edge axes
Manifold satPolySphere(const Hull& a, uint32_t a_id, const Material& am, const SphereG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    uint32_t feature = 0;
    uint32_t surf = (uint32_t)a.pts.size();
    for (size_t f = 0; f < a.gv.size(); f++, surf++) {
        if (a.g_redundant[f]) continue;
        Extrema ea = recenter(a.g_cache[f], a.g_ref_val[f], a.gv[f].dot(a.pts[a.g_ref_idx[f]]));
        double before = best.pen;
        if (axisTest(ea, sphereExtrema(b, a.gv[f]), a.gv[f], &best)) { out.max_pen = -1; return out; }
        if (best.pen < before) feature = surf;
    }
    for (int p = 0; p < (int)a.pts.size(); p++) {
        V3 n = (a.pts[p] - b.c).normalize();
        double before = best.pen;
        if (axisTest(findExtrema(a, n), sphereExtrema(b, n), n, &best)) { out.max_pen = -1; return out; }
        if (best.pen < before) feature = (uint32_t)p;
    }
    for (auto& e : a.edges) {
        V3 dir = (a.pts[e.second] - a.pts[e.first]).normalize();
        V3 sample = a.pts[e.first] - b.c;
        V3 n = (sample - dir * dir.dot(sample)).normalize();
        double before = best.pen;
        if (axisTest(findExtrema(a, n), sphereExtrema(b, n), n, &best)) { out.max_pen = -1; return out; }
        if (best.pen < before) feature = edgeId(e.first, e.second);
    }
    out.normal = best.n;
    out.pts.push_back(mkPoint(b.c - out.normal * b.r, best.pen, am, bm, cidOf(a_id, b_id), feature));
    out.max_pen = best.pen;
    return out;
}

// findCylinderContactArea (CollisionDetect.cpp:354-374) and the barrel line
// of cylinderLengthwiseLineInDirection (:346-351)
static void lengthwiseLine(const CylG& c, V3 n, V3* p1, V3* p2) {
    V3 barrel = (n - c.axis * c.axis.dot(n)).normalize();
    *p1 = c.c + barrel * c.r + 0.5 * c.h * c.axis;
    *p2 = *p1 - c.h * c.axis;
}
enum CylArea { CA_FACE, CA_EDGE, CA_BARREL };
static Area cylinderArea(const CylG& c, V3 n, V3 u, V3 w, CylArea* kind) {
    Area a;
    double ad = c.axis.dot(n);
    if (1 - std::abs(ad) <= cosTol() && n.dot(c.axis) > 0) {
        for (int i = 0; i < 8; i++) { a.ps.push_back(p2(c.top[i].dot(u), c.top[i].dot(w))); a.ids.push_back(i); }
        a.surface = 16; a.origin = FACE; *kind = CA_FACE;
        return a;
    }
    if (1 - std::abs(ad) <= cosTol()) {
        for (int i = 0; i < 8; i++) { a.ps.push_back(p2(c.bot[i].dot(u), c.bot[i].dot(w))); a.ids.push_back(i + 8); }
        a.surface = 17; a.origin = FACE; *kind = CA_FACE;
        return a;
    }
    if (std::abs(ad) <= sinTol()) {
        V3 l1, l2;
        lengthwiseLine(c, n, &l1, &l2);
        a.ps = {p2(l1.dot(u), l1.dot(w)), p2(l2.dot(u), l2.dot(w))};
        a.ids = {18, 19};
        a.surface = -1; a.origin = EDGE; *kind = CA_BARREL;
        return a;
    }
    V3 p = n.dot(c.axis) > 0 ? diskExtremum(c.topCenter(), c.axis, c.r, n) : diskExtremum(c.botCenter(), c.axis, c.r, n);
    a.ps = {p2(p.dot(u), p.dot(w))};
    a.ids = {n.dot(c.axis) > 0 ? 18 : 19};
    a.surface = -1; a.origin = EDGE; *kind = CA_EDGE;
    return a;
}

static bool arcAxes(const std::vector<V3>& ag, const std::vector<std::pair<int, int>>& aarcs, const std::vector<V3>& bg,
                    const std::vector<std::pair<int, int>>& barcs, const std::function<Extrema(const V3&)>& ea,
                    const std::function<Extrema(const V3&)>& eb, NormResult* best) {
    for (auto& arc1 : aarcs) {
        for (auto& arc2 : barcs) {
            V3 a1 = ag[arc1.first], a2 = ag[arc1.second];
            V3 b1 = -bg[arc2.first], b2 = -bg[arc2.second];
            V3 avg = a1 + a2;
            if (avg.dot(b1) + avg.dot(b2) <= 0) continue;
            V3 ap = a1.cross(a2), bp = b1.cross(b2);
            if (ap.dot(b1) * ap.dot(b2) > 0 || bp.dot(a1) * bp.dot(a2) > 0) continue;
            V3 n = ap.cross(bp);
            if (n.mag2() == 0) continue;
            n = n.normalize();
            if (avg.dot(n) < 0) n *= -1;
            if (axisTest(ea(n), eb(n), n, best)) return true;
        }
    }
    return false;
}

static Manifold pointsFromPool(const std::vector<ClipP>& pool, V3 u, V3 w, V3 n, double a_dot, double a_pen,
                               const Material& am, const Material& bm, uint64_t cid) {
    Manifold out;
    V3 off = n * a_dot;
    for (const ClipP& p : pool) {
        V3 pos = u * p.pos.x + w * p.pos.y + off;
        out.pts.push_back(mkPoint(pos, pos.dot(n) - a_dot + a_pen, am, bm, cid, p.magic));
    }
    return out;
}

// SAT_PolyCylinder (CollisionDetect.cpp:1563-1709)
Manifold satPolyCylinder(const Hull& a, uint32_t a_id, const Material& am, const CylG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    for (size_t f = 0; f < a.gv.size(); f++) {
        if (a.g_redundant[f]) continue;
        Extrema ea = recenter(a.g_cache[f], a.g_ref_val[f], a.gv[f].dot(a.pts[a.g_ref_idx[f]]));
        if (axisTest(ea, cylinderExtrema(b, a.gv[f]), a.gv[f], &best)) return out;
    }
    V3 ax = b.axis;
    if (axisTest(findExtrema(a, ax), cylinderExtrema(b, ax), ax, &best)) return out;
    for (auto& e : a.edges) {
        V3 ed = a.pts[e.second] - a.pts[e.first];
        V3 dir = ed.cross(ax);
        if (dir.mag() < 0.00000000001) continue;
        V3 dn = dir.normalize();
        if (axisTest(findExtrema(a, dn), cylinderExtrema(b, dn), dn, &best)) return out;
    }
    for (const V3& p : a.pts) {
        V3 diff = p - b.c;
        V3 n = (diff - ax * ax.dot(diff)).normalize();
        if (axisTest(findExtrema(a, n), cylinderExtrema(b, n), n, &best)) return out;
    }
    if (arcAxes(a.gv, a.arcs, b.gv, b.arcs, [&](const V3& n) { return findExtrema(a, n); },
                [&](const V3& n) { return cylinderExtrema(b, n); }, &best))
        return out;
    V3 n = best.n;
    V3 amax = a.pts[best.a_id];
    V3 u, w;
    n.perpBasis(&u, &w);
    Area ac = contactArea(a, n, amax, best.a_id, u, w);
    CylArea bk;
    Area bc = cylinderArea(b, -n, u, w, &bk);
    std::vector<ClipP> pool;
    if (bk == CA_EDGE) pool = {ClipP{bc.ps[0], 0, 0x0, false}};
    else pool = clipContacts(ac, bc);
    out = pointsFromPool(pool, u, w, n, amax.dot(n), best.pen, am, bm, cidOf(a_id, b_id));
    out.normal = n;
    out.max_pen = best.pen;
    return out;
}

// detectSphereCylinder (CollisionDetect.cpp:1712-1792).  The fourth axis uses
// the same disk as the third: the reference computes its "bottom" disk centre
// with +0.5 h along the axis (:1756), and that is reproduced here.
Manifold sphereCylinder(const SphereG& a, uint32_t a_id, const Material& am, const CylG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    V3 ax = b.axis;
    if (axisTest(sphereExtrema(a, ax), cylinderExtrema(b, ax), ax, &best)) return out;
    V3 diff = b.c - a.c;
    V3 barrel = (diff - ax * ax.dot(diff)).normalize();
    if (axisTest(sphereExtrema(a, barrel), cylinderExtrema(b, barrel), barrel, &best)) return out;
    V3 top = b.c + ax * 0.5 * b.h;
    V3 tp = diskExtremum(top, ax, b.r, -diff.normalize());
    V3 e1 = (tp - a.c).normalize();
    if (axisTest(sphereExtrema(a, e1), cylinderExtrema(b, e1), e1, &best)) return out;
    V3 bot = b.c + ax * 0.5 * b.h;
    V3 bp = diskExtremum(bot, ax, b.r, -diff.normalize());
    V3 e2 = (bp - a.c).normalize();
    if (axisTest(sphereExtrema(a, e2), cylinderExtrema(b, e2), e2, &best)) return out;
    out.normal = best.n;
    out.pts.push_back(mkPoint(a.c + out.normal * a.r, best.pen, am, bm, cidOf(a_id, b_id), 0));
    out.max_pen = best.pen;
    return out;
}

// checkCylinderEdgeApproxVsBarrel (CollisionDetect.cpp:938-956)
static bool edgeApproxVsBarrel(const CylG& a, const CylG& b, V3 barrel_axis, const std::vector<V3>& ring, NormResult* best) {
    int n = (int)ring.size();
    for (int i = 0; i < n; i++) {
        V3 ed = ring[(i + 1) % n] - ring[i];
        V3 dir = ed.cross(barrel_axis);
        if (dir.mag() < 0.00000000001) continue;
        V3 dn = dir.normalize();
        if (axisTest(cylinderExtrema(a, dn), cylinderExtrema(b, dn), dn, best)) return true;
    }
    return false;
}

// detectCylinderCylinder (CollisionDetect.cpp:958-1137)
Manifold cylinderCylinder(const CylG& a, uint32_t a_id, const Material& am, const CylG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    V3 aa = a.axis, ba = b.axis;
    if (axisTest(cylinderExtrema(a, aa), cylinderExtrema(b, aa), aa, &best)) return out;
    if (axisTest(cylinderExtrema(a, ba), cylinderExtrema(b, ba), ba, &best)) return out;
    if (edgeApproxVsBarrel(a, b, ba, a.top, &best)) return out;
    if (edgeApproxVsBarrel(a, b, ba, a.bot, &best)) return out;
    if (edgeApproxVsBarrel(a, b, aa, b.top, &best)) return out;
    if (edgeApproxVsBarrel(a, b, aa, b.bot, &best)) return out;
    V3 bb = aa.cross(ba);
    if (bb.mag2() > 0.00000001) {
        bb = bb.normalize();
        if (axisTest(cylinderExtrema(a, bb), cylinderExtrema(b, bb), bb, &best)) return out;
    }
    if (arcAxes(a.gv, a.arcs, b.gv, b.arcs, [&](const V3& n) { return cylinderExtrema(a, n); },
                [&](const V3& n) { return cylinderExtrema(b, n); }, &best))
        return out;
    V3 n = best.n;
    V3 u, w;
    n.perpBasis(&u, &w);
    CylArea ak, bk;
    Area ac = cylinderArea(a, n, u, w, &ak);
    Area bc = cylinderArea(b, -n, u, w, &bk);
    std::vector<ClipP> pool;
    if (ak == CA_EDGE) pool = {ClipP{ac.ps[0], 0, 0x0, false}};
    else if (bk == CA_EDGE) pool = {ClipP{bc.ps[0], 0, 0x0, false}};
    else if (ak == CA_BARREL && bk == CA_BARREL && std::abs(aa.dot(ba)) > 0.995) {
        V3 a1, a2, b1, b2;
        lengthwiseLine(a, n, &a1, &a2);
        lengthwiseLine(b, -n, &b1, &b2);
        if (ba.dot(aa) < 0) std::swap(b1, b2);
        double amx = a1.dot(aa), amn = a2.dot(aa), bmx = b1.dot(aa), bmn = b2.dot(aa);
        V3 imx = (amx > bmx) ? b1 : a1;
        V3 imn = (amn > bmn) ? a2 : b2;
        pool = {ClipP{p2(u.dot(imx), w.dot(imx)), 0, 0x0, false}, ClipP{p2(u.dot(imn), w.dot(imn)), 0, 0x1, false}};
    } else {
        pool = clipContacts(ac, bc);
    }
    V3 amax = aa.dot(n) > 0 ? diskExtremum(a.topCenter(), aa, a.r, n) : diskExtremum(a.botCenter(), aa, a.r, n);
    out = pointsFromPool(pool, u, w, n, amax.dot(n), best.pen, am, bm, cidOf(a_id, b_id));
    out.normal = n;
    out.max_pen = best.pen;
    return out;
}

// --------------------------------------------------------------- capsules ----
// getCapsuleExtrema (CollisionDetect.cpp:685-703): the two cap spheres
static Extrema capsuleExtrema(const CapG& c, const V3& d) {
    V3 off = c.axis * c.h / 2.0;
    double v1 = d.dot(c.c + off);
    double mn1 = v1 - c.r, mx1 = v1 + c.r;
    double v2 = d.dot(c.c - off);
    double mn2 = v2 - c.r, mx2 = v2 + c.r;
    Extrema e;
    e.max_v = std::max<double>(mx1, mx2);
    e.min_v = std::min<double>(mn1, mn2);
    e.min_id = e.max_id = -1;
    return e;
}

// cylinderLengthwiseLineInDirection (CollisionDetect.cpp:346-351) for any
// centre / axis / radius / height
static void lineAlong(const V3& c, const V3& axis, double r, double h, const V3& n, V3* p1, V3* p2) {
    V3 barrel = (n - axis * axis.dot(n)).normalize();
    *p1 = c + barrel * r + 0.5 * h * axis;
    *p2 = *p1 - h * axis;
}

// findCapsuleContactArea (CollisionDetect.cpp:376-390): the barrel line (ids
// 0 = top cap, 1 = bottom cap) or the one cap point
enum CapArea { CAP_BARREL, CAP_EDGE };
static Area capsuleArea(const CapG& c, V3 n, V3 u, V3 w, CapArea* kind) {
    Area a;
    if (std::abs(c.axis.dot(n)) <= sinTol()) {
        V3 l1, l2;
        lineAlong(c.c, c.axis, c.r, c.h, n, &l1, &l2);
        a.ps = {p2(l1.dot(u), l1.dot(w)), p2(l2.dot(u), l2.dot(w))};
        a.ids = {0, 1};
        a.surface = -1; a.origin = EDGE; *kind = CAP_BARREL;
        return a;
    }
    if (n.dot(c.axis) > 0) {
        V3 p = n * c.r + c.c + c.axis * c.h / 2.0;
        a.ps = {p2(p.dot(u), p.dot(w))};
        a.ids = {0};
    } else {
        V3 p = n * c.r + c.c - c.axis * c.h / 2.0;
        a.ps = {p2(p.dot(u), p.dot(w))};
        a.ids = {1};
    }
    a.surface = -1; a.origin = EDGE; *kind = CAP_EDGE;
    return a;
}

// the contact of two parallel barrels (lengthwise lines clipped along a's
// axis), as detectCapsuleCapsule / detectCapsuleCylinder /
// detectCylinderCylinder build it
static std::vector<ClipP> parallelBarrels(V3 a1, V3 a2, V3 b1, V3 b2, const V3& aa, const V3& ba, const V3& u, const V3& w) {
    if (ba.dot(aa) < 0) std::swap(b1, b2);
    double amx = a1.dot(aa), amn = a2.dot(aa), bmx = b1.dot(aa), bmn = b2.dot(aa);
    V3 imx = (amx > bmx) ? b1 : a1;
    V3 imn = (amn > bmn) ? a2 : b2;
    return {ClipP{p2(u.dot(imx), w.dot(imx)), 0, 0x0, false}, ClipP{p2(u.dot(imn), w.dot(imn)), 0, 0x1, false}};
}

// detectSphereCapsule (CollisionDetect.cpp:868-935)
Manifold sphereCapsule(const SphereG& a, uint32_t a_id, const Material& am, const CapG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    V3 ax = b.axis;
    V3 diff = b.c - a.c;
    V3 barrel = (diff - ax * ax.dot(diff)).normalize();
    if (axisTest(sphereExtrema(a, barrel), capsuleExtrema(b, barrel), barrel, &best)) return out;
    V3 cap1 = b.c + ax * b.h / 2.0;
    V3 e1 = (cap1 - a.c).normalize();
    if (axisTest(sphereExtrema(a, e1), capsuleExtrema(b, e1), e1, &best)) return out;
    V3 cap2 = b.c - ax * b.h / 2.0;
    V3 e2 = (cap2 - a.c).normalize();
    if (axisTest(sphereExtrema(a, e2), capsuleExtrema(b, e2), e2, &best)) return out;
    out.normal = best.n;
    out.pts.push_back(mkPoint(a.c + out.normal * a.r, best.pen, am, bm, cidOf(a_id, b_id), 0));
    out.max_pen = best.pen;
    return out;
}

// detectCapsuleCapsule (CollisionDetect.cpp:1139-1334).  The axes are those
// the reference tests, in its order: cap-centre pairs (top-top, bottom-top as
// b top minus a bottom, bottom-bottom), each of a's caps against b's barrel,
// b's caps against a's barrel (taken from b's centre), barrel-barrel.
Manifold capsuleCapsule(const CapG& a, uint32_t a_id, const Material& am, const CapG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    V3 at = a.c + a.axis * a.h / 2.0, ab = a.c - a.axis * a.h / 2.0;
    V3 bt = b.c + b.axis * b.h / 2.0, bb = b.c - b.axis * b.h / 2.0;
    auto test = [&](const V3& n) { return axisTest(capsuleExtrema(a, n), capsuleExtrema(b, n), n, &best); };
    if (test((bt - at).normalize())) return out;
    if (test((bt - ab).normalize())) return out;
    if (test((bb - ab).normalize())) return out;
    {
        V3 d = b.c - at;
        if (test((d - b.axis * b.axis.dot(d)).normalize())) return out;
    }
    {
        V3 d = b.c - ab;
        if (test((d - b.axis * b.axis.dot(d)).normalize())) return out;
    }
    {
        V3 d = b.c - bt;
        if (test((d - a.axis * a.axis.dot(d)).normalize())) return out;
    }
    {
        V3 d = b.c - bb;
        if (test((d - a.axis * a.axis.dot(d)).normalize())) return out;
    }
    V3 bx = a.axis.cross(b.axis);
    if (bx.mag2() > 0.00000001) {
        bx = bx.normalize();
        if (test(bx)) return out;
    }
    V3 n = best.n;
    V3 u, w;
    n.perpBasis(&u, &w);
    CapArea ak, bk;
    Area ac = capsuleArea(a, n, u, w, &ak);
    Area bc = capsuleArea(b, -n, u, w, &bk);
    std::vector<ClipP> pool;
    if (ak == CAP_BARREL && bk == CAP_BARREL && std::abs(a.axis.dot(b.axis)) > 0.995) {
        V3 a1, a2, b1, b2;
        lineAlong(a.c, a.axis, a.r, a.h, n, &a1, &a2);
        lineAlong(b.c, b.axis, b.r, b.h, -n, &b1, &b2);
        pool = parallelBarrels(a1, a2, b1, b2, a.axis, b.axis, u, w);
    } else {
        pool = clipContacts(ac, bc);
    }
    V3 amax = a.axis.dot(n) > 0 ? at + n * a.r : ab + n * a.r;
    out = pointsFromPool(pool, u, w, n, amax.dot(n), best.pen, am, bm, cidOf(a_id, b_id));
    out.normal = n;
    out.max_pen = best.pen;
    return out;
}

// SAT_PolyCapsule (CollisionDetect.cpp:1413-1561).  The reference places the
// caps a full drum height from the centre here (:1436-1437) and tests each
// edge's "bottom cap" axis against the top cap again (:1486-1488); both are
// reproduced.
Manifold satPolyCapsule(const Hull& a, uint32_t a_id, const Material& am, const CapG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    for (size_t f = 0; f < a.gv.size(); f++) {
        if (a.g_redundant[f]) continue;
        Extrema ea = recenter(a.g_cache[f], a.g_ref_val[f], a.gv[f].dot(a.pts[a.g_ref_idx[f]]));
        if (axisTest(ea, capsuleExtrema(b, a.gv[f]), a.gv[f], &best)) return out;
    }
    V3 ax = b.axis;
    V3 tcc = b.c + ax * b.h;
    V3 bcc = b.c - ax * b.h;
    double tv = tcc.dot(ax), bv = bcc.dot(ax);
    for (const V3& p : a.pts) {
        double v = p.dot(ax);
        V3 n;
        if (bv <= v && v <= tv) n = ((p - b.c) - ax * ax.dot(p - b.c)).normalize();
        else if (v > tv) n = (p - tcc).normalize();
        else n = (p - bcc).normalize();
        if (axisTest(findExtrema(a, n), capsuleExtrema(b, n), n, &best)) return out;
    }
    for (auto& e : a.edges) {
        V3 dir = (a.pts[e.second] - a.pts[e.first]).normalize();
        for (int k = 0; k < 2; k++) {
            V3 sample = a.pts[e.first] - tcc;
            V3 n = (sample - dir * dir.dot(sample)).normalize();
            if (axisTest(findExtrema(a, n), capsuleExtrema(b, n), n, &best)) return out;
        }
        V3 d = dir.cross(ax);
        if (d.mag() < 0.00000000001) continue;
        V3 n = d.normalize();
        if (axisTest(findExtrema(a, n), capsuleExtrema(b, n), n, &best)) return out;
    }
    V3 n = best.n;
    V3 amax = a.pts[best.a_id];
    V3 u, w;
    n.perpBasis(&u, &w);
    Area ac = contactArea(a, n, amax, best.a_id, u, w);
    CapArea bk;
    Area bc = capsuleArea(b, -n, u, w, &bk);
    std::vector<ClipP> pool = clipContacts(ac, bc);
    out = pointsFromPool(pool, u, w, n, amax.dot(n), best.pen, am, bm, cidOf(a_id, b_id));
    out.normal = n;
    out.max_pen = best.pen;
    return out;
}

// detectCapsuleCylinder (CollisionDetect.cpp:1794-2002)
Manifold capsuleCylinder(const CapG& a, uint32_t a_id, const Material& am, const CylG& b, uint32_t b_id, const Material& bm) {
    Manifold out;
    out.max_pen = -1;
    NormResult best = {-1, -1, V3(), std::numeric_limits<double>::infinity()};
    V3 aa = a.axis, ba = b.axis;
    auto test = [&](const V3& n) { return axisTest(capsuleExtrema(a, n), cylinderExtrema(b, n), n, &best); };
    if (test(ba)) return out;
    const int nr = (int)b.top.size();
    for (int i = 0; i < nr; i++) {
        V3 ed = b.top[(i + 1) % nr] - b.top[i];
        V3 dir = ed.cross(aa);
        if (dir.mag() < 0.00000000001) continue;
        if (test(dir.normalize())) return out;
    }
    V3 at = a.c + a.axis * a.h / 2.0, ab = a.c - a.axis * a.h / 2.0;
    V3 tdc = b.c + ba * 0.5 * b.h;
    {
        V3 cp = diskExtremum(tdc, ba, b.r, (at - b.c).normalize());
        if (test((cp - at).normalize())) return out;
    }
    {
        V3 cp = diskExtremum(tdc, ba, b.r, (ab - b.c).normalize());
        if (test((cp - ab).normalize())) return out;
    }
    V3 bdc = b.c - ba * 0.5 * b.h;
    {
        V3 cp = diskExtremum(bdc, ba, b.r, (at - b.c).normalize());
        if (test((cp - at).normalize())) return out;
    }
    {
        V3 cp = diskExtremum(bdc, ba, b.r, (ab - b.c).normalize());
        if (test((cp - ab).normalize())) return out;
    }
    {
        V3 d = b.c - at;
        if (test((d - ba * ba.dot(d)).normalize())) return out;
    }
    {
        V3 d = b.c - ab;
        if (test((d - ba * ba.dot(d)).normalize())) return out;
    }
    V3 bx = aa.cross(ba);
    if (bx.mag2() > 0.00000001) {
        bx = bx.normalize();
        if (test(bx)) return out;
    }
    V3 n = best.n;
    V3 u, w;
    n.perpBasis(&u, &w);
    CapArea ak;
    CylArea bk;
    Area ac = capsuleArea(a, n, u, w, &ak);
    Area bc = cylinderArea(b, -n, u, w, &bk);
    std::vector<ClipP> pool;
    if (bk == CA_EDGE) {
        pool = {ClipP{bc.ps[0], 0, 0x0, false}};
    } else if (ak == CAP_BARREL && bk == CA_BARREL && std::abs(aa.dot(ba)) > 0.995) {
        V3 a1, a2, b1, b2;
        lineAlong(a.c, a.axis, a.r, a.h, n, &a1, &a2);
        lineAlong(b.c, b.axis, b.r, b.h, -n, &b1, &b2);
        pool = parallelBarrels(a1, a2, b1, b2, aa, ba, u, w);
    } else {
        pool = clipContacts(ac, bc);
    }
    V3 amax = a.axis.dot(n) > 0 ? at + n * a.r : ab + n * a.r;
    out = pointsFromPool(pool, u, w, n, amax.dot(n), best.pen, am, bm, cidOf(a_id, b_id));
    out.normal = n;
    out.max_pen = best.pen;
    return out;
}

// ------------------------------------------------------ mesh triangles ----
// findTriangleExtrema (CollisionDetect.cpp:2004-2021)
static Extrema triExtrema(const MeshTri& t, const V3& d) {
    Extrema e;
    for (int i = 0; i < 3; i++) {
        double v = t.v[i].dot(d);
        if (v < e.min_v) { e.min_id = i; e.min_v = v; }
        if (v > e.max_v) { e.max_id = i; e.max_v = v; }
    }
    return e;
}

// normalDirectionValid (CollisionDetect.cpp:2024-2060): the normal must lie in
// the face's Gauss region (triangle of 3 directions, arc of 2, or the normal)
static bool normalValid(const MeshTri& s, const V3& n) {
    const double EPS = 0.0001;
    const std::vector<V3>& g = s.gauss;
    switch (s.concave) {
    case 0:
    case 1:
        for (size_t i = 0; i < g.size(); i++) {
            V3 inner = g[i].cross(g[(i + 1) % g.size()]);
            if (n.dot(inner) < -EPS) return false;
        }
        break;
    case 2: {
        V3 arc = g[0].cross(g[1]);
        if (std::abs(n.dot(arc)) > EPS) return false;
        V3 up = arc.cross(g[0]);
        if (n.dot(up) < -EPS) return false;
        V3 down = g[1].cross(arc);
        if (n.dot(down) < -EPS) return false;
        break;
    }
    case 3:
        if (n.dot(s.normal) < 1 - EPS) return false;
        break;
    }
    return true;
}

// findTriangleContactArea (CollisionDetect.cpp:303-329) with projectTriangleFace
// / projectTriangleEdge (:282-300): face points carry ids 0..2, edge points the
// edge id
static Area triangleArea(const MeshTri& t, const V3& n, const V3& p, int pid, const V3& u, const V3& w) {
    Area a;
    if (1 - t.normal.dot(n) <= cosTol()) {
        for (int i = 0; i < 3; i++) { a.ps.push_back(p2(t.v[i].dot(u), t.v[i].dot(w))); a.ids.push_back(i); }
        a.surface = t.id;
        a.origin = FACE;
        return a;
    }
    for (int i = 0; i < 3; i++) {
        if (i != pid && (i + 1) % 3 != pid) continue;
        double sn = std::abs((t.ep2[i] - t.ep1[i]).normalize().dot(n));
        if (sn <= sinTol()) {
            a.ps = {p2(t.ep1[i].dot(u), t.ep1[i].dot(w)), p2(t.ep2[i].dot(u), t.ep2[i].dot(w))};
            a.ids = {t.eid[i], t.eid[i]};
            a.surface = -1;
            a.origin = EDGE;
            return a;
        }
    }
    a.ps = {p2(p.dot(u), p.dot(w))};
    a.ids = {pid};
    a.surface = -1;
    a.origin = VERTEX;
    return a;
}

// the six Gauss arcs of a triangle (normal to each edge's outward direction,
// and on to the reversed normal)
static void triArcs(const MeshTri& t, V3 g1[6], V3 g2[6]) {
    for (int i = 0; i < 3; i++) {
        g1[2 * i] = t.normal; g2[2 * i] = t.out[i];
        g1[2 * i + 1] = t.out[i]; g2[2 * i + 1] = -t.normal;
    }
}

struct TriSat {
    NormResult min_pen{-1, -1, V3(), std::numeric_limits<double>::infinity()};
    NormResult min_valid{-1, -1, V3(), std::numeric_limits<double>::infinity()};
    bool sep = false;
    // one axis: false when it separates
    bool take(const MeshTri& t, const Extrema& ea, const Extrema& eb, const V3& n, bool* improved = nullptr) {
        NormResult x = checkNorm(ea, eb, n);
        if (x.pen < 0) { sep = true; return false; }
        if (improved) *improved = false;
        if (x.pen < min_pen.pen) { min_pen = x; if (improved) *improved = true; }
        if (x.pen < min_valid.pen && normalValid(t, -x.n)) min_valid = x;
        return true;
    }
    // the penalised choice; returns the unpenalised minimum as well
    NormResult choose(double penalty, NormResult* nongauss) const {
        *nongauss = min_pen;
        return (min_valid.pen < min_pen.pen + penalty) ? min_valid : min_pen;
    }
};

static bool triArcAxes(TriSat& S, const MeshTri& t, const std::vector<V3>& ag, const std::vector<std::pair<int, int>>& aarcs,
                       const std::function<Extrema(const V3&)>& ea) {
    V3 g1[6], g2[6];
    triArcs(t, g1, g2);
    for (auto& arc1 : aarcs)
        for (int k = 0; k < 6; k++) {
            V3 a1 = ag[arc1.first], a2 = ag[arc1.second];
            V3 b1 = -g1[k], b2 = -g2[k];
            V3 avg = a1 + a2;
            if (avg.dot(b1) + avg.dot(b2) <= 0) continue;
            V3 ap = a1.cross(a2), bp = b1.cross(b2);
            if (ap.dot(b1) * ap.dot(b2) > 0 || bp.dot(a1) * bp.dot(a2) > 0) continue;
            V3 n = ap.cross(bp);
            if (n.mag2() == 0) continue;
            n = n.normalize();
            if (avg.dot(n) < 0) n *= -1;
            if (!S.take(t, ea(n), triExtrema(t, n), n)) return false;
        }
    return true;
}

// SAT_PolyTriangle (CollisionDetect.cpp:2062-2194)
static Manifold satPolyTriangle(const Hull& a, uint32_t a_id, const Material& am, const MeshTri& b, const Material& bm, double penalty) {
    Manifold out;
    TriSat S;
    if (!S.take(b, findExtrema(a, b.normal), triExtrema(b, b.normal), b.normal)) return out;
    for (size_t f = 0; f < a.gv.size(); f++) {
        if (a.g_redundant[f]) continue;
        Extrema ea = recenter(a.g_cache[f], a.g_ref_val[f], a.gv[f].dot(a.pts[a.g_ref_idx[f]]));
        if (!S.take(b, ea, triExtrema(b, a.gv[f]), a.gv[f])) return out;
    }
    if (!triArcAxes(S, b, a.gv, a.arcs, [&](const V3& n) { return findExtrema(a, n); })) return out;
    NormResult ng;
    NormResult mp = S.choose(penalty, &ng);
    V3 n = mp.n;
    V3 amax = a.pts[ng.a_id], bmax = b.v[ng.b_id];
    V3 u, w;
    n.perpBasis(&u, &w);
    Area ac = contactArea(a, ng.n, amax, ng.a_id, u, w);
    Area bc = triangleArea(b, (-1) * ng.n, bmax, ng.b_id, u, w);
    std::vector<ClipP> pool = clipContacts(ac, bc);
    out = pointsFromPool(pool, u, w, n, amax.dot(n), mp.pen, am, bm, cidOf(a_id, (uint32_t)b.id));
    out.normal = n;
    out.max_pen = mp.pen;
    return out;
}

// SAT_SphereTriangle (CollisionDetect.cpp:2196-2276)
static Manifold satSphereTriangle(const SphereG& a, uint32_t a_id, const Material& am, const MeshTri& b, const Material& bm, double penalty) {
    Manifold out;
    TriSat S;
    uint32_t feature = (uint32_t)-1;
    if (!S.take(b, sphereExtrema(a, b.normal), triExtrema(b, b.normal), b.normal)) return out;
    for (int i = 0; i < 3; i++) {
        V3 n = (b.v[i] - a.c).normalize();
        bool imp;
        if (!S.take(b, sphereExtrema(a, n), triExtrema(b, n), n, &imp)) return out;
        if (imp) feature = (uint32_t)i;
    }
    for (int i = 0; i < 3; i++) {
        V3 dir = (b.ep2[i] - b.ep1[i]).normalize();
        V3 sample = b.ep1[i] - a.c;
        V3 n = (sample - dir * dir.dot(sample)).normalize();
        bool imp;
        if (!S.take(b, sphereExtrema(a, n), triExtrema(b, n), n, &imp)) return out;
        if (imp) feature = (uint32_t)b.eid[i];
    }
    NormResult ng;
    NormResult mp = S.choose(penalty, &ng);
    out.normal = mp.n;
    out.pts.push_back(mkPoint(a.c + mp.n * a.r, mp.pen, am, bm, cidOf(a_id, (uint32_t)b.id), feature));
    out.max_pen = mp.pen;
    return out;
}

// SAT_CylinderTriangle (CollisionDetect.cpp:2466-2646)
static Manifold satCylinderTriangle(const CylG& a, uint32_t a_id, const Material& am, const MeshTri& b, const Material& bm, double penalty) {
    Manifold out;
    TriSat S;
    V3 ax = a.axis;
    if (!S.take(b, cylinderExtrema(a, ax), triExtrema(b, ax), ax)) return out;
    if (!S.take(b, cylinderExtrema(a, b.normal), triExtrema(b, b.normal), b.normal)) return out;
    for (int i = 0; i < 3; i++) {
        V3 dir = (b.ep2[i] - b.ep1[i]).cross(ax);
        if (dir.mag() < 0.00000000001) continue;
        V3 dn = dir.normalize();
        if (!S.take(b, cylinderExtrema(a, dn), triExtrema(b, dn), dn)) return out;
    }
    for (int i = 0; i < 3; i++) {
        V3 diff = b.v[i] - a.c;
        V3 n = (diff - ax * ax.dot(diff)).normalize();
        if (!S.take(b, cylinderExtrema(a, n), triExtrema(b, n), n)) return out;
    }
    if (!triArcAxes(S, b, a.gv, a.arcs, [&](const V3& n) { return cylinderExtrema(a, n); })) return out;
    NormResult ng;
    NormResult mp = S.choose(penalty, &ng);
    V3 n = mp.n;
    V3 amax = ax.dot(n) > 0 ? diskExtremum(a.topCenter(), ax, a.r, n) : diskExtremum(a.botCenter(), ax, a.r, n);
    V3 bmax = b.v[ng.b_id];
    V3 u, w;
    n.perpBasis(&u, &w);
    CylArea ak;
    Area ac = cylinderArea(a, ng.n, u, w, &ak);
    Area bc = triangleArea(b, -ng.n, bmax, ng.b_id, u, w);
    std::vector<ClipP> pool;
    if (ak == CA_EDGE) pool = {ClipP{ac.ps[0], 0, 0x0, false}};
    else pool = clipContacts(ac, bc);
    out = pointsFromPool(pool, u, w, n, amax.dot(n), mp.pen, am, bm, cidOf(a_id, (uint32_t)b.id));
    out.normal = n;
    out.max_pen = mp.pen;
    return out;
}

// SAT_CapsuleTriangle (CollisionDetect.cpp:2278-2464).  The reference sets
// its "bottom" cap centre with +h/2 as well (:2286), so both cap tests use the
// top cap; reproduced.
static Manifold satCapsuleTriangle(const CapG& a, uint32_t a_id, const Material& am, const MeshTri& b, const Material& bm, double penalty) {
    Manifold out;
    TriSat S;
    V3 ax = a.axis;
    V3 at = a.c + ax * a.h / 2.0;
    V3 ab = a.c + ax * a.h / 2.0;
    if (!S.take(b, capsuleExtrema(a, b.normal), triExtrema(b, b.normal), b.normal)) return out;
    for (int i = 0; i < 3; i++) {
        V3 dir = (b.ep2[i] - b.ep1[i]).cross(ax);
        if (dir.mag() < 0.00000000001) continue;
        V3 dn = dir.normalize();
        if (!S.take(b, capsuleExtrema(a, dn), triExtrema(b, dn), dn)) return out;
    }
    for (int i = 0; i < 3; i++) {
        V3 diff = b.v[i] - a.c;
        V3 n = (diff - ax * ax.dot(diff)).normalize();
        if (!S.take(b, capsuleExtrema(a, n), triExtrema(b, n), n)) return out;
    }
    for (const V3* cc : {&at, &ab})
        for (int i = 0; i < 3; i++) {
            V3 n = (b.v[i] - *cc).normalize();
            if (!S.take(b, capsuleExtrema(a, n), triExtrema(b, n), n)) return out;
        }
    for (const V3* cc : {&at, &ab})
        for (int i = 0; i < 3; i++) {
            V3 dir = (b.ep2[i] - b.ep1[i]).normalize();
            V3 sample = b.ep1[i] - *cc;
            V3 n = (sample - dir * dir.dot(sample)).normalize();
            if (!S.take(b, capsuleExtrema(a, n), triExtrema(b, n), n)) return out;
        }
    NormResult ng;
    NormResult mp = S.choose(penalty, &ng);
    V3 n = mp.n;
    V3 amax = ax.dot(n) > 0 ? at + n * a.r : ab + n * a.r;
    V3 bmax = b.v[ng.b_id];
    V3 u, w;
    n.perpBasis(&u, &w);
    CapArea ak;
    Area ac = capsuleArea(a, ng.n, u, w, &ak);
    Area bc = triangleArea(b, -ng.n, bmax, ng.b_id, u, w);
    std::vector<ClipP> pool;
    if (ak == CAP_EDGE) pool = {ClipP{ac.ps[0], 0, 0x0, false}};
    else pool = clipContacts(ac, bc);
    out = pointsFromPool(pool, u, w, n, amax.dot(n), mp.pen, am, bm, cidOf(a_id, (uint32_t)b.id));
    out.normal = n;
    out.max_pen = mp.pen;
    return out;
}

static double longest(const AABB& b) {
    return std::max<double>(b.mx.x - b.mn.x, std::max<double>(b.mx.y - b.mn.y, b.mx.z - b.mn.z));
}

// SAT_PolyMesh / SAT_SphereMesh / SAT_CapsuleMesh / SAT_CylinderMesh (CollisionDetect.cpp:
// 2648-2778) for a fixed mesh in world coordinates: candidate triangles from
// the mesh tree in its traversal order, penalty 0 for polyhedra and
// 0.15 min(longest AABB sides) otherwise
std::vector<Manifold> meshCollide(const Body* c, const Body* m) {
    std::vector<Manifold> out;
    const Material& mm = m->mat;
    for (int ti : m->tree.candidates(c->aabb)) {
        const MeshTri& t = m->tris[ti];
        Manifold r;
        if (c->kind == K_HULL) r = satPolyTriangle(c->shape, c->id, c->mat, t, mm, 0 * std::min<double>(longest(c->aabb), longest(t.aabb)));
        else if (c->kind == K_SPHERE) r = satSphereTriangle(c->sph, c->id, c->mat, t, mm, 0.15 * std::min<double>(longest(c->aabb), longest(t.aabb)));
        else if (c->kind == K_CAPSULE) r = satCapsuleTriangle(c->cap, c->id, c->mat, t, mm, 0.15 * std::min<double>(longest(c->aabb), longest(t.aabb)));
        else r = satCylinderTriangle(c->cyl, c->id, c->mat, t, mm, 0.15 * std::min<double>(longest(c->aabb), longest(t.aabb)));
        if (r.max_pen > 0 && !r.pts.empty()) out.push_back(r);
    }
    return out;
}

// merge_manifold (CollisionDetect.cpp:2780-2793)
Manifold mergeManifold(const Manifold& a, const Manifold& b) {
    Manifold o;
    o.pts = a.pts;
    o.pts.insert(o.pts.end(), b.pts.begin(), b.pts.end());
    o.normal = (a.normal + b.normal).normalize();
    o.max_pen = std::max<double>(a.max_pen, b.max_pen);
    return o;
}

// cull_manifold (CollisionDetect.cpp:2795-2830): keep the extreme points in 4
// directions of the contact plane
Manifold cullManifold(const Manifold& m, int n) {
    if (n >= (int)m.pts.size()) return m;
    Manifold out;
    out.normal = m.normal;
    out.max_pen = 0;
    out.pts.resize(n);
    std::vector<bool> avail(m.pts.size(), true);
    V3 u, w;
    m.normal.perpBasis(&u, &w);
    for (int i = 0; i < n; i++) {
        double vu = std::cos(2 * PI_FULL * i / n);
        double vw = std::sin(2 * PI_FULL * i / n);
        V3 dir = u * vu + w * vw;
        int best = -1;
        double bv = -std::numeric_limits<double>::infinity();
        for (size_t j = 0; j < m.pts.size(); j++) {
            if (!avail[j]) continue;
            double v = m.pts[j].pos.dot(dir);
            if (v > bv) { bv = v; best = (int)j; }
        }
        out.pts[i] = m.pts[best];
        out.max_pen = std::max(out.max_pen, m.pts[best].pen);
        avail[best] = false;
    }
    return out;
}

}  // namespace cport
