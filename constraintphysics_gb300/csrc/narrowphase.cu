// narrowphase.cu — SAT narrowphase for convex-hull pairs, one warp per pair.
//
// Follows SAT_PolyPoly (ConstraintPhysics/src/CollisionDetect.cpp:717-835):
// face axes of both hulls (with the cached self-extrema recentred by the
// pose), edge-edge axes only for Gauss-map arc pairs that intersect (hemisphere
// test plus two plane-straddle tests), minimum penetration with the
// first-in-order tie-break, then contact-feature selection (:237-280),
// Sutherland-Hodgman clipping with feature-pair ids (:394-620) and the
// 4-direction cull (:2795-2830).
//
// GB300 mapping: the hot part of each hull blob (header, vertices, Gauss
// normals, arcs, cached extrema) is staged into the warp's shared-memory slot
// with one cp.async.bulk per hull completing on an mbarrier (bounded wait);
// lanes transform vertices/normals to world space in place, then each lane
// owns a strided subset of the axes (face axes, then arc pairs), keeps its
// own (pen, axis-order) minimum and the warp reduces it with shuffles.  The
// serial feature selection and polygon clipping run on lane 0 over the staged
// data.
#include "kernels.cuh"
#include "devmath.cuh"

namespace cpgpu {

namespace {

constexpr float kCosTol = (float)1.5230484360873042e-4;  // 1 - cos(1 deg), CollisionDetect.h:21-23
constexpr float kSinTol = (float)0.017452406437283512;   // sin(1 deg)
constexpr int kMaxClip = 40;
constexpr int kQueue = 64;                       // queued edge-edge axes per warp
constexpr int kQueueBytes = kQueue * (16 + 4);
constexpr int kMeshBlocksPerSm = 2;          // mesh-pair kernel grid (its scratch is per warp)

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// bounded mbarrier wait: `limit` polls (Dev::wait_limit; kDefaultWaitLimit
// when draining a giving-up warp's own copies)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
    for (long long it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ---- hull views --------------------------------------------------------------
struct HullView {
    const HullHeader* h;
    float4* v;           // world vertices (shared, transformed in place)
    float4* n;           // world Gauss normals, w = redundant flag
    const float4* cache; // reference-frame face extrema
    const uint8_t* arc;  // staged arc pairs
    const uint8_t* g;    // global blob (cold sections)
    f3 com;
    __device__ __forceinline__ f3 vert(int i) const { return mk(v[i]); }
    __device__ __forceinline__ f3 norm(int f) const { return mk(n[f]); }
};

// The same hull read from its global blob by one thread, each vertex and
// normal put in world space when it is used (the arithmetic of stage_hull, so
// both views give identical values)
struct HullG {
    const HullHeader* h;
    const float4* vref;
    const float4* nref;
    const uint8_t* g;
    f3 com;
    M33 R;
    __device__ __forceinline__ HullG(const uint8_t* blob, float4 pos, float4 rot) {
        h = reinterpret_cast<const HullHeader*>(blob);
        vref = reinterpret_cast<const float4*>(blob + sizeof(HullHeader));
        nref = reinterpret_cast<const float4*>(blob + h->off_norm);
        g = blob;
        com = mk(pos);
        R = quatRot(qnormalize(rot));
    }
    __device__ __forceinline__ f3 vert(int i) const { return com + mul(R, mk(__ldg(vref + i))); }
    __device__ __forceinline__ f3 norm(int f) const { return mul(R, mk(__ldg(nref + f))); }
};

__device__ __forceinline__ const uint16_t* u16(const uint8_t* base, int off) { return reinterpret_cast<const uint16_t*>(base + off); }

// ---- extrema / axis test -----------------------------------------------------
struct Ext { float mn, mx; int mn_id, mx_id; };

// findExtrema (CollisionDetect.cpp:627-644): strict compares, first index wins
__device__ __forceinline__ Ext extrema(const float4* v, int nv, f3 ax) {
    Ext e{INFINITY, -INFINITY, -1, -1};
    for (int i = 0; i < nv; i++) {
        float x = dot(mk(v[i]), ax);
        if (x < e.mn) { e.mn = x; e.mn_id = i; }
        if (x > e.mx) { e.mx = x; e.mx_id = i; }
    }
    return e;
}

struct Axis { float pen; int idx; int aid, bid; f3 n; };

// sat_checknorm (CollisionDetect.cpp:705-715)
__device__ __forceinline__ void check(const Ext& a, const Ext& b, f3 n, int idx, Axis* best, bool* sep) {
    float fwd = a.mx - b.mn, rev = b.mx - a.mn;
    Axis x;
    if (fwd < rev) x = Axis{fwd, idx, a.mx_id, b.mn_id, n};
    else x = Axis{rev, idx, a.mn_id, b.mx_id, -n};
    if (x.pen < 0.f) *sep = true;
    // strict minimum over the reference's axis order: ties go to the axis that
    // comes first (axes reach a lane out of order, so compare the index too)
    else if (x.pen < best->pen || (x.pen == best->pen && idx < best->idx)) *best = x;
}

// ---- 2-D clipping (lane 0) --------------------------------------------------------
struct P2 { float x, y; };
struct CP { P2 p; int src; unsigned long long magic; int skip; };

__device__ __forceinline__ float dot2(P2 a, P2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ P2 inDir(P2 a, P2 b) {  // getInDirOfEdge (CollisionDetect.cpp:394-397)
    P2 v{a.y - b.y, b.x - a.x};
    float s = 1.0f / sqrtf(dot2(v, v));
    return P2{v.x * s, v.y * s};
}
// getEdgeID (CollisionDetect.cpp:9-21): ids truncated to 16 bits
__device__ __forceinline__ uint32_t edgeId(int a, int b) {
    uint32_t p = (uint16_t)a, q = (uint16_t)b;
    uint32_t mn = p < q ? p : q, mx = p < q ? q : p;
    return (0x0000FFFFu & mn) + (0xFFFF0000u & (mx << 16));
}
__device__ __forceinline__ unsigned long long pack(unsigned long long lo, unsigned long long hi) {
    return (0x00000000FFFFFFFFull & lo) | (0xFFFFFFFF00000000ull & (hi << 32));
}

struct Area { P2 ps[kMaxClip]; int ids[kMaxClip]; int n; int surface; };

__device__ CP intersect(const CP& e1, const CP& e2, P2 nrm, P2 sample, int clip_edge, bool flip) {
    P2 d{e2.p.x - e1.p.x, e2.p.y - e1.p.y};
    P2 sd{sample.x - e1.p.x, sample.y - e1.p.y};
    float t = dot2(nrm, sd) / dot2(nrm, d);
    CP o;
    o.p = P2{e1.p.x + d.x * t, e1.p.y + d.y * t};
    bool e2_kept = dot2(d, nrm) > 0.f;
    o.src = e2_kept ? e1.src : e2.src;
    unsigned long long eid = edgeId(e1.src, e2.src);
    unsigned long long ce = (unsigned long long)(long long)clip_edge;
    o.magic = flip ? pack(ce, eid) : pack(eid, ce);
    o.skip = !e2_kept;
    return o;
}

// getClipEvaluatinPolyAfterClippingByEdge (CollisionDetect.cpp:500-576)
__device__ int clipByEdge(const CP* c, int n, CP* out, P2 side, P2 sample, int eid, bool flip, int* status) {
    int m = 0;
    float cv = dot2(sample, side);
    auto push = [&](const CP& x) { if (m < kMaxClip) out[m++] = x; else atomicOr(status, ST_CLIP_OVERFLOW); };
    if (n >= 3) {
        float v1 = 0.f, v2 = 0.f;
        CP q1, q2;
        for (int i = 0; i < n; i++) {
            if (i > 0) { v1 = v2; q1 = q2; }
            else { q1 = c[0]; v1 = dot2(q1.p, side); }
            q2 = c[(i + 1) % n];
            v2 = dot2(q2.p, side);
            if (v1 >= cv && v2 >= cv) push(q1);                                  // neither clipped
            else if (v1 == cv && v2 < cv) push(q1);                              // p1 on edge, p2 clipped
            else if (v1 < cv && v2 == cv) {}                                     // p2 on edge, p1 clipped
            else if (v1 < cv && v2 >= cv) push(intersect(q1, q2, side, sample, eid, flip));  // only p1 clipped
            else if (v1 >= cv && v2 < cv) { push(q1); push(intersect(q1, q2, side, sample, eid, flip)); }
        }
        return m;
    }
    if (n == 2) {
        float v1 = dot2(c[0].p, side), v2 = dot2(c[1].p, side);
        if (v1 >= cv && v2 >= cv) { out[0] = c[0]; out[1] = c[1]; return 2; }
        if (v1 == cv && v2 < cv) { out[0] = c[0]; return 1; }
        if (v1 < cv && v2 == cv) { out[0] = c[1]; return 1; }
        if (v1 < cv && v2 >= cv) { out[0] = intersect(c[0], c[1], side, sample, eid, flip); out[1] = c[1]; return 2; }
        if (v1 >= cv && v2 < cv) { out[0] = c[0]; out[1] = intersect(c[0], c[1], side, sample, eid, flip); return 2; }
        return 0;
    }
    if (n == 1 && dot2(c[0].p, side) >= cv) { out[0] = c[0]; return 1; }
    return 0;
}

// clipC1ByAllEdgesOfC2 (CollisionDetect.cpp:566-576); result in c1
__device__ int clipByAll(CP* c1, int n1, const CP* c2, int n2, bool flip, CP* tmp, int* status) {
    for (int i = 0; i < n2; i++) {
        const CP& e1 = c2[i];
        if (e1.skip) continue;
        const CP& e2 = c2[(i + 1) % n2];
        int m = clipByEdge(c1, n1, tmp, inDir(e1.p, e2.p), e1.p, (int)edgeId(e1.src, e2.src), flip, status);
        for (int k = 0; k < m; k++) c1[k] = tmp[k];
        n1 = m;
        if (n1 == 0) return 0;
    }
    return n1;
}

// createClipEvaluationPoly (CollisionDetect.cpp:441-460)
__device__ int toClipPoly(const Area& a, uint32_t other_surface, bool flip, CP* out) {
    for (int i = 0; i < a.n; i++) {
        unsigned long long id = (unsigned long long)(long long)a.ids[i];
        out[i].p = a.ps[i];
        out[i].src = a.ids[i];
        out[i].magic = flip ? pack(other_surface, id) : pack(id, other_surface);
        out[i].skip = 0;
    }
    if (a.n > 2) {
        P2 in = inDir(a.ps[0], a.ps[1]);
        bool ccw = false;
        for (int i = 2; i < a.n; i++) {
            float d = dot2(P2{a.ps[i].x - a.ps[0].x, a.ps[i].y - a.ps[0].y}, in);
            if (d > 0.0000000001f) { ccw = true; break; }
            if (d < -0.0000000001f) { ccw = false; break; }
        }
        if (!ccw)
            for (int i = 0, j = a.n - 1; i < j; i++, j--) { CP t = out[i]; out[i] = out[j]; out[j] = t; }
    }
    return a.n;
}

// findContactArea (CollisionDetect.cpp:237-280)
template <class HV>
__device__ void contactArea(const HV& h, f3 n, int pid, f3 u, f3 w, Area* a) {
    const HullHeader& H = *h.h;
    const uint16_t* vfofs = u16(h.g, H.off_vfofs);
    const uint8_t* vfidx = h.g + H.off_vfidx;
    int best_f = -1;
    float best_ft = 1.0f;
    for (int k = vfofs[pid]; k < vfofs[pid + 1]; k++) {
        int f = vfidx[k];
        float ca = dot(h.norm(f), n);
        if (1.f - ca < best_ft) { best_ft = 1.f - ca; best_f = f; }
    }
    if (best_ft <= kCosTol) {
        const uint16_t* fofs = u16(h.g, H.off_fofs);
        const uint8_t* fidx = h.g + H.off_fidx;
        a->n = 0;
        for (int k = fofs[best_f]; k < fofs[best_f + 1] && a->n < kMaxClip; k++) {
            int id = fidx[k];
            f3 v = h.vert(id);
            a->ps[a->n] = P2{dot(v, u), dot(v, w)};
            a->ids[a->n++] = id;
        }
        a->surface = H.nv + best_f;
        return;
    }
    const uint16_t* veofs = u16(h.g, H.off_veofs);
    const uint8_t* veidx = h.g + H.off_veidx;
    const uint8_t* edges = h.g + H.off_edge;
    int best_e = -1;
    float best_et = 1.0f;
    for (int k = veofs[pid]; k < veofs[pid + 1]; k++) {
        int e = veidx[k];
        f3 d = h.vert(edges[2 * e + 1]) - h.vert(edges[2 * e]);
        float sa = fabsf(dot(normalize(d), n));
        if (sa < best_et) { best_et = sa; best_e = e; }
    }
    if (best_et <= kSinTol) {
        int p1 = edges[2 * best_e], p2 = edges[2 * best_e + 1];
        f3 e1 = h.vert(p1), e2 = h.vert(p2);
        a->ps[0] = P2{dot(e1, u), dot(e1, w)};
        a->ps[1] = P2{dot(e2, u), dot(e2, w)};
        a->ids[0] = p1; a->ids[1] = p2;
        a->n = 2;
        a->surface = -1;
        return;
    }
    f3 p = h.vert(pid);
    a->ps[0] = P2{dot(p, u), dot(p, w)};
    a->ids[0] = pid;
    a->n = 1;
    a->surface = -1;
}

struct Scratch { CP p1[kMaxClip], p2[kMaxClip], tmp[kMaxClip]; };

// clipContacts (CollisionDetect.cpp:578-620); returns the clipped point count in out
__device__ int clipContacts(const Area& c1, const Area& c2, Scratch& s, CP* out, int* status) {
    int n1 = toClipPoly(c1, (uint32_t)c2.surface, false, s.p1);
    int n2 = toClipPoly(c2, (uint32_t)c1.surface, true, s.p2);
    if (n1 == 1) { out[0] = s.p1[0]; return 1; }
    if (n2 == 1) { out[0] = s.p2[0]; return 1; }
    if (n1 == 2 && n2 == 2) {
        P2 nrm = inDir(s.p2[0].p, s.p2[1].p);
        out[0] = intersect(s.p1[0], s.p1[1], nrm, s.p2[0].p, (int)edgeId(s.p2[0].src, s.p2[1].src), false);
        return 1;
    }
    if (n1 == 2) {
        int m = clipByAll(s.p1, n1, s.p2, n2, false, s.tmp, status);
        for (int i = 0; i < m; i++) out[i] = s.p1[i];
        return m;
    }
    if (n2 == 2) {
        int m = clipByAll(s.p2, n2, s.p1, n1, true, s.tmp, status);
        for (int i = 0; i < m; i++) out[i] = s.p2[i];
        return m;
    }
    n1 = clipByAll(s.p1, n1, s.p2, n2, false, s.tmp, status);
    int m = clipByAll(s.p2, n2, s.p1, n1, true, s.tmp, status);
    for (int i = 0; i < m; i++) out[i] = s.p2[i];
    return m;
}

__device__ __forceinline__ void stage_hull(const uint8_t* g, uint8_t* s, const float4 pos, const float4 rot, HullView* hv, int lane) {
    const HullHeader* H = reinterpret_cast<const HullHeader*>(s);
    float4* v = reinterpret_cast<float4*>(s + sizeof(HullHeader));
    float4* n = reinterpret_cast<float4*>(s + H->off_norm);
    M33 R = quatRot(qnormalize(rot));
    f3 com = mk(pos);
    for (int i = lane; i < H->nv; i += 32) {
        f3 p = com + mul(R, mk(v[i]));
        v[i] = make_float4(p.x, p.y, p.z, 0.f);
    }
    for (int i = lane; i < H->nf; i += 32) {
        float4 q = n[i];
        f3 p = mul(R, mk(q));
        n[i] = make_float4(p.x, p.y, p.z, q.w);
    }
    hv->h = H;
    hv->v = v;
    hv->n = n;
    hv->cache = reinterpret_cast<const float4*>(s + H->off_cache);
    hv->arc = s + H->off_arc;
    hv->g = g;
    hv->com = com;
}

// collisionAllowed (PhysicsEngine.cpp:570-572): bodies joined by a joint do
// not collide; the joint-edge keys are sorted, so one binary search decides
// two sleeping bodies are not tested (PhysicsEngine.cpp:174)
__device__ __forceinline__ bool both_asleep(const Dev& d, int a, int b) {
    return d.has_sleep && d.asleep[a] && d.asleep[b];
}

__device__ __forceinline__ bool jointed(const Dev& d, int a, int b) {
    if (d.n_joint_edges == 0) return false;
    const uint64_t k = ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
    int lo = 0, hi = d.n_joint_edges;
    while (lo < hi) {
        int m = (lo + hi) >> 1;
        if (d.je.key[m] < k) lo = m + 1; else hi = m;
    }
    // a pair joined only by springs still collides (addSpring adds no
    // collision exception, PhysicsEngine.cpp:974-998)
    return lo < d.n_joint_edges && d.je.key[lo] == k && d.je.jcount[lo] > 0;
}

// bodies of several primitives (ConvexUnionGeometry): their primitives'
// blobs, AABBs and materials live in the primitive tables; a body of one
// primitive is its own only primitive
__device__ __forceinline__ bool is_union(const Dev& d, int g) { return d.has_union && d.prim_start[g] >= 0; }
__device__ __forceinline__ int prim_n(const Dev& d, int g) { return is_union(d, g) ? d.prim_count[g] : 1; }
__device__ __forceinline__ const uint8_t* prim_blob(const Dev& d, int g, int k) {
    return d.shapes + (is_union(d, g) ? d.prim_shape[d.prim_start[g] + k] : d.shape[g]);
}
__device__ __forceinline__ void prim_box(const Dev& d, int g, int k, f3* lo, f3* hi) {
    if (is_union(d, g)) { *lo = mk(d.prim_lo[d.prim_start[g] + k]); *hi = mk(d.prim_hi[d.prim_start[g] + k]); }
    else { *lo = mk(d.aabb_lo[g]); *hi = mk(d.aabb_hi[g]); }
}

// cull_manifold (CollisionDetect.cpp:2795-2830) to at most 4 points and write
// the pair's manifold
__device__ void emit_manifold(const Dev& d, int p, f3 n, float maxpen, const float4* pts, const unsigned long long* magic, int m) {
    int out_n = m;
    int pick[4] = {0, 1, 2, 3};
    if (m > 4) {
        out_n = 4;
        unsigned long long avail = (m >= 64) ? ~0ull : ((1ull << m) - 1ull);
        f3 cu, cw;
        basis(n, &cu, &cw);
        const float cs[4] = {1.0f, 6.123233995736766e-17f, -1.0f, -1.8369701987210297e-16f};
        const float sn[4] = {0.0f, 1.0f, 1.2246467991473532e-16f, -1.0f};
        for (int i = 0; i < 4; i++) {
            f3 dir = cu * cs[i] + cw * sn[i];
            int bi2 = -1;
            float bv = -INFINITY;
            for (int j = 0; j < m; j++) {
                if (!((avail >> j) & 1ull)) continue;
                float v = dot(mk(pts[j]), dir);
                if (v > bv) { bv = v; bi2 = j; }
            }
            if (bi2 < 0) { out_n = i; break; }
            pick[i] = bi2;
            avail &= ~(1ull << bi2);
        }
    }
    for (int i = 0; i < out_n; i++) {
        d.mf_pt[4 * p + i] = pts[pick[i]];
        d.mf_magic[4 * p + i] = magic[pick[i]];
    }
    d.mf_n[p] = make_float4(n.x, n.y, n.z, maxpen);
    d.mf_cnt[p] = out_n;
}

__device__ __forceinline__ void no_manifold(const Dev& d, int p) {
    d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f);
    d.mf_cnt[p] = 0;
}

// warp argmin over (pen, axis order); every lane gets the winner
__device__ __forceinline__ Axis warp_best(const Axis& best) {
    float bp = best.pen;
    int bi = best.idx;
    for (int o = 16; o > 0; o >>= 1) {
        float op = __shfl_xor_sync(0xffffffffu, bp, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (op < bp || (op == bp && oi < bi)) { bp = op; bi = oi; }
    }
    unsigned owner_mask = __ballot_sync(0xffffffffu, best.idx == bi && best.pen == bp);
    int owner = owner_mask ? __ffs(owner_mask) - 1 : 0;
    Axis w;
    w.pen = bp;
    w.idx = bi;
    w.n = mk(__shfl_sync(0xffffffffu, best.n.x, owner), __shfl_sync(0xffffffffu, best.n.y, owner),
             __shfl_sync(0xffffffffu, best.n.z, owner));
    w.aid = __shfl_sync(0xffffffffu, best.aid, owner);
    w.bid = __shfl_sync(0xffffffffu, best.bid, owner);
    return w;
}

// ---- spheres, cylinders and capsules ------------------------------------------------
// Sphere (ConvexPrimitive.h:79-109), Cylinder (:160-210) and Capsule (:107-141;
// `h` is its drum height) in world space.
struct PrimView {
    uint32_t kind;
    f3 c, axis;
    float r, h;
    const float4 *gv, *top, *bot;   // cylinder: Gauss vertices, cap 8-gons
};

// world pose of a staged sphere / cylinder blob; the cylinder's Gauss vertices
// and caps are transformed in place (Cylinder::recomputeFromReference,
// ConvexPrimitive.cpp:272-287: the bottom cap is top - height * axis)
__device__ void stage_prim(uint8_t* s, float4 pos, float4 rot, PrimView* pv, int lane) {
    const HullHeader* H = reinterpret_cast<const HullHeader*>(s);
    M33 R = quatRot(qnormalize(rot));
    f3 com = mk(pos);
    float4 cref = *reinterpret_cast<const float4*>(s + sizeof(HullHeader));
    pv->kind = H->kind;
    pv->r = cref.w;
    pv->c = mul(R, mk(cref)) + com;
    pv->axis = mk(0.f, 0.f, 0.f);
    pv->h = 0.f;
    if (H->kind == SHAPE_CAPSULE) {   // Capsule::recomputeFromReference (ConvexPrimitive.cpp:383-388)
        float4 ax = *reinterpret_cast<const float4*>(s + kCylOffAxis);
        pv->axis = mul(R, mk(ax));
        pv->h = ax.w;
        return;
    }
    if (H->kind != SHAPE_CYLINDER) return;
    float4 ax = *reinterpret_cast<const float4*>(s + kCylOffAxis);
    pv->axis = mul(R, mk(ax));
    pv->h = ax.w;
    float4* gv = reinterpret_cast<float4*>(s + kCylOffGv);
    float4* top = reinterpret_cast<float4*>(s + kCylOffTop);
    float4* bot = reinterpret_cast<float4*>(s + kCylOffBot);
    if (lane < 2 + kCylRing) {
        f3 g = mul(R, mk(gv[lane]));
        gv[lane] = make_float4(g.x, g.y, g.z, 0.f);
    }
    if (lane < kCylCap) {
        f3 t = mul(R, mk(top[lane])) + com;
        f3 b = t - pv->h * pv->axis;
        top[lane] = make_float4(t.x, t.y, t.z, 0.f);
        bot[lane] = make_float4(b.x, b.y, b.z, 0.f);
    }
    pv->gv = gv;
    pv->top = top;
    pv->bot = bot;
}

// getSphereExtrema (CollisionDetect.cpp:646-655)
__device__ __forceinline__ Ext sphereExt(const PrimView& s, f3 d) {
    float cv = dot(d, s.c);
    return Ext{cv - s.r, cv + s.r, -1, -1};
}

// Cylinder::getExtremaOfDisk (ConvexPrimitive.cpp:319-355): the point of the
// disk rim furthest along `target`.  Two FP32 restatements keep the reference's
// FP64 behaviour: its parallel test |n.t| > 1 - 1e-8 is below FP32 resolution
// near 1, so it is applied as the equivalent sin(angle) < sqrt(2e-8) on the
// cross product; and the rim height dw = sqrt(r^2 - r^2 / (1 + g^2)) cancels
// catastrophically for nearly parallel directions in FP32, so it is evaluated
// as the equal r g / sqrt(1 + g^2).  (A tilt of 4e-4 rad otherwise moves the
// extremum's projection by r * 4e-4.)
__device__ f3 diskExtremum(f3 center, f3 normal, float r, f3 target) {
    if (mag(cross(normal, target)) < 1.41421356e-4f) return center;
    float nd = fabsf(dot(normal, target));
    if (nd < 1e-8f) return center + target * r;
    f3 u, v;
    basis(target, &u, &v);
    f3 w = target;
    float nu = dot(normal, u), nv = dot(normal, v), nw = dot(normal, w);
    float dwdu = -nu / nw, dwdv = -nv / nw;
    float gm = sqrtf(dwdu * dwdu + dwdv * dwdv);
    float gu = dwdu / gm, gv = dwdv / gm;
    float root = sqrtf(1.f + gm * gm);
    float su = r / root;            // sqrt(uv_mag_sqrd)
    float dw = r * gm / root;       // sqrt(r^2 - uv_mag_sqrd)
    return center + u * (gu * su) + v * (gv * su) + w * dw;
}

__device__ __forceinline__ f3 topCenter(const PrimView& c) { return c.c + (0.5f * c.h) * c.axis; }
__device__ __forceinline__ f3 botCenter(const PrimView& c) { return c.c - (0.5f * c.h) * c.axis; }

// getCylinderExtrema (CollisionDetect.cpp:657-683): extremes of the two caps by
// symmetry about the centre
__device__ Ext cylExt(const PrimView& c, f3 d) {
    f3 tc = topCenter(c);
    f3 tmax = diskExtremum(tc, c.axis, c.r, d);
    f3 tmin = 2.f * tc - tmax;
    f3 bmax = 2.f * c.c - tmin;
    f3 bmin = 2.f * c.c - tmax;
    return Ext{fminf(dot(d, tmin), dot(d, bmin)), fmaxf(dot(d, tmax), dot(d, bmax)), -1, -1};
}

// findCylinderContactArea (CollisionDetect.cpp:354-374).  Returns 0 for a cap
// face (8-gon, point ids offset + i, surface 16 / 17), 1 for the barrel line
// (ids 18, 19) and 2 for a single rim point.
__device__ int cylArea(const PrimView& c, f3 n, f3 u, f3 w, Area* a) {
    float ad = dot(c.axis, n);
    if (1.f - fabsf(ad) <= kCosTol) {
        bool top = dot(n, c.axis) > 0.f;
        const float4* ring = top ? c.top : c.bot;
        for (int i = 0; i < kCylCap; i++) {
            f3 q = mk(ring[i]);
            a->ps[i] = P2{dot(q, u), dot(q, w)};
            a->ids[i] = i + (top ? 0 : kCylCap);
        }
        a->n = kCylCap;
        a->surface = top ? 2 * kCylCap : 2 * kCylCap + 1;
        return 0;
    }
    if (fabsf(ad) <= kSinTol) {
        // cylinderLengthwiseLineInDirection (CollisionDetect.cpp:346-351)
        f3 barrel = normalize(n - c.axis * dot(c.axis, n));
        f3 p1 = c.c + barrel * c.r + (0.5f * c.h) * c.axis;
        f3 p2 = p1 - c.h * c.axis;
        a->ps[0] = P2{dot(p1, u), dot(p1, w)};
        a->ps[1] = P2{dot(p2, u), dot(p2, w)};
        a->ids[0] = 2 * kCylCap + 2;
        a->ids[1] = 2 * kCylCap + 3;
        a->n = 2;
        a->surface = -1;
        return 1;
    }
    bool top = dot(n, c.axis) > 0.f;
    f3 q = diskExtremum(top ? topCenter(c) : botCenter(c), c.axis, c.r, n);
    a->ps[0] = P2{dot(q, u), dot(q, w)};
    a->ids[0] = top ? 2 * kCylCap + 2 : 2 * kCylCap + 3;
    a->n = 1;
    a->surface = -1;
    return 2;
}

// The FP64 reference skips an axis cross(edge, axis) when its length is below
// 1e-11, i.e. only for exactly parallel directions; FP32 rounding leaves ~1e-7
// of noise there, so the skip is relative: sin(angle) below 1e-6.
__device__ __forceinline__ bool edgeAxis(f3 edge, f3 axis, f3* n) {
    f3 dir = cross(edge, axis);
    float m = mag(dir);
    if (m < 1e-6f * mag(edge) || m == 0.f) return false;
    *n = dir * (1.f / m);
    return true;
}

// Gauss-arc pair test shared by the hull-cylinder and cylinder-cylinder
// edge axes (same steps as SAT_PolyPoly's)
__device__ __forceinline__ bool arcAxis(f3 a1, f3 a2, f3 b1, f3 b2, f3* n) {
    f3 avg = a1 + a2;
    if (!(dot(avg, b1) + dot(avg, b2) > 0.f)) return false;
    f3 ap = cross(a1, a2), bp = cross(b1, b2);
    if (dot(ap, b1) * dot(ap, b2) > 0.f || dot(bp, a1) * dot(bp, a2) > 0.f) return false;
    f3 x = cross(ap, bp);
    if (mag2(x) == 0.f) return false;
    x = normalize(x);
    if (dot(avg, x) < 0.f) x = x * -1.f;
    *n = x;
    return true;
}

// cylinder Gauss arcs as the constructor builds them (ConvexPrimitive.cpp:
// 243-244): arc 2i joins Gauss vertex 0 to vertex i, arc 2i+1 vertex 1 to i
__device__ __forceinline__ void cylArc(const PrimView& c, int k, f3* g1, f3* g2) {
    *g1 = mk(c.gv[k & 1]);
    *g2 = mk(c.gv[k >> 1]);
}

// ManifoldPoint list of one detector call (before the cull)
struct PrimOut {
    int m;
    f3 n;
    float pen;
    float4 pts[kMaxClip];
    unsigned long long magic[kMaxClip];
};

__device__ void points_from_pool(const CP* pool, int m, f3 u, f3 w, f3 n, float a_dot, float pen, PrimOut* o) {
    f3 off = n * a_dot;
    for (int i = 0; i < m; i++) {
        f3 q = u * pool[i].p.x + w * pool[i].p.y + off;
        o->pts[i] = make_float4(q.x, q.y, q.z, dot(q, n) - a_dot + pen);
        o->magic[i] = pool[i].magic;
    }
    o->m = m;
}

// SAT_PolySphere (CollisionDetect.cpp:1336-1411): face, vertex and edge axes of
// the hull; the contact is the sphere's deepest point, its feature id the
// winning axis' face (n_points + f), vertex or edge id.
__device__ bool polySphere(const HullView& A, const PrimView& S, int lane, PrimOut* o) {
    const HullHeader& H = *A.h;
    const int nf = H.nf, nv = H.nv, ne = H.ne;
    const uint8_t* edges = A.g + H.off_edge;
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    for (int t = lane; t < nf + nv + ne; t += 32) {
        Ext ea;
        f3 n;
        if (t < nf) {
            float4 g = A.n[t];
            if (g.w != 0.f) continue;
            n = mk(g);
            float4 c = A.cache[t];
            float shift = dot(n, A.com);
            ea = Ext{c.y + shift, c.x + shift, __float_as_int(c.w), __float_as_int(c.z)};
        } else if (t < nf + nv) {
            n = normalize(mk(A.v[t - nf]) - S.c);
            ea = extrema(A.v, nv, n);
        } else {
            int e = t - nf - nv;
            f3 p1 = mk(A.v[edges[2 * e]]), p2 = mk(A.v[edges[2 * e + 1]]);
            f3 dir = normalize(p2 - p1);
            f3 sample = p1 - S.c;
            n = normalize(sample - dir * dot(dir, sample));
            ea = extrema(A.v, nv, n);
        }
        check(ea, sphereExt(S, n), n, t, &best, &sep);
    }
    if (__any_sync(0xffffffffu, sep)) return false;
    Axis b = warp_best(best);
    if (!(b.pen < INFINITY)) return false;
    if (lane == 0) {
        uint32_t feature;
        if (b.idx < nf) feature = (uint32_t)(nv + b.idx);
        else if (b.idx < nf + nv) feature = (uint32_t)(b.idx - nf);
        else {
            int e = b.idx - nf - nv;
            feature = edgeId(edges[2 * e], edges[2 * e + 1]);
        }
        f3 q = S.c - b.n * S.r;
        o->n = b.n;
        o->pen = b.pen;
        o->pts[0] = make_float4(q.x, q.y, q.z, b.pen);
        o->magic[0] = feature;
        o->m = 1;
    }
    return true;
}

// SAT_PolyCylinder (CollisionDetect.cpp:1563-1709): hull faces, the cylinder
// axis, hull edges x axis, hull vertices radially, Gauss-arc pairs; contact by
// clipping the hull's feature against the cylinder's cap / barrel line, or the
// single rim point.
__device__ bool polyCylinder(const HullView& A, const PrimView& C, int lane, Scratch& scratch, CP* clipped,
                             int* status, PrimOut* o) {
    const HullHeader& H = *A.h;
    const int nf = H.nf, nv = H.nv, ne = H.ne, na = H.na;
    const uint8_t* edges = A.g + H.off_edge;
    const int e0 = nf + 1, v0 = e0 + ne, a0 = v0 + nv, total = a0 + na * 2 * kCylRing;
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    for (int t = lane; t < total; t += 32) {
        Ext ea;
        f3 n;
        if (t < nf) {
            float4 g = A.n[t];
            if (g.w != 0.f) continue;
            n = mk(g);
            float4 c = A.cache[t];
            float shift = dot(n, A.com);
            ea = Ext{c.y + shift, c.x + shift, __float_as_int(c.w), __float_as_int(c.z)};
        } else {
            if (t == nf) n = C.axis;
            else if (t < v0) {
                int e = t - e0;
                if (!edgeAxis(mk(A.v[edges[2 * e + 1]]) - mk(A.v[edges[2 * e]]), C.axis, &n)) continue;
            } else if (t < a0) {
                f3 diff = mk(A.v[t - v0]) - C.c;
                n = normalize(diff - C.axis * dot(C.axis, diff));
            } else {
                int k = t - a0, ia = k / (2 * kCylRing), ib = k - ia * (2 * kCylRing);
                f3 g1, g2;
                cylArc(C, ib, &g1, &g2);
                if (!arcAxis(mk(A.n[A.arc[2 * ia]]), mk(A.n[A.arc[2 * ia + 1]]), -g1, -g2, &n)) continue;
            }
            ea = extrema(A.v, nv, n);
        }
        check(ea, cylExt(C, n), n, t, &best, &sep);
    }
    if (__any_sync(0xffffffffu, sep)) return false;
    Axis b = warp_best(best);
    if (!(b.pen < INFINITY) || b.aid < 0) return false;
    if (lane == 0) {
        f3 n = b.n, u, w;
        basis(n, &u, &w);
        Area ac, bc;
        contactArea(A, n, b.aid, u, w, &ac);
        int m;
        if (cylArea(C, -1.f * n, u, w, &bc) == 2) {
            clipped[0] = CP{bc.ps[0], 0, 0ull, 0};
            m = 1;
        } else {
            m = clipContacts(ac, bc, scratch, clipped, status);
        }
        points_from_pool(clipped, m, u, w, n, dot(mk(A.v[b.aid]), n), b.pen, o);
        o->n = n;
        o->pen = b.pen;
    }
    return true;
}

// detectSphereSphere (CollisionDetect.cpp:837-866)
__device__ bool sphereSphere(const PrimView& A, const PrimView& B, PrimOut* o) {
    f3 diff = B.c - A.c;
    float pen = A.r + B.r - mag(diff);
    if (pen < 0.f) return false;
    f3 n = normalize(diff);
    f3 q = A.c + n * A.r;
    o->n = n;
    o->pen = pen;
    o->pts[0] = make_float4(q.x, q.y, q.z, pen);
    o->magic[0] = 0ull;
    o->m = 1;
    return true;
}

// detectSphereCylinder (CollisionDetect.cpp:1712-1792): the cylinder axis, the
// radial direction and two rim directions.  The reference computes both rim
// points from the top cap (its "bottom" centre also adds half the height,
// :1756); that is kept.
__device__ bool sphereCylinder(const PrimView& S, const PrimView& C, PrimOut* o) {
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    f3 ax = C.axis;
    check(sphereExt(S, ax), cylExt(C, ax), ax, 0, &best, &sep);
    if (sep) return false;
    f3 diff = C.c - S.c;
    f3 barrel = normalize(diff - ax * dot(ax, diff));
    check(sphereExt(S, barrel), cylExt(C, barrel), barrel, 1, &best, &sep);
    if (sep) return false;
    f3 rim_c = C.c + ax * 0.5f * C.h;
    f3 rim = diskExtremum(rim_c, ax, C.r, -normalize(diff));
    f3 e = normalize(rim - S.c);
    check(sphereExt(S, e), cylExt(C, e), e, 2, &best, &sep);
    if (sep) return false;
    check(sphereExt(S, e), cylExt(C, e), e, 3, &best, &sep);
    if (sep || !(best.pen < INFINITY)) return false;
    f3 q = S.c + best.n * S.r;
    o->n = best.n;
    o->pen = best.pen;
    o->pts[0] = make_float4(q.x, q.y, q.z, best.pen);
    o->magic[0] = 0ull;
    o->m = 1;
    return true;
}

// checkCylinderEdgeApproxVsBarrel (CollisionDetect.cpp:938-956), one ring edge
__device__ __forceinline__ bool ringAxis(const float4* ring, int i, f3 barrel_axis, f3* n) {
    return edgeAxis(mk(ring[(i + 1) % kCylCap]) - mk(ring[i]), barrel_axis, n);
}

// detectCylinderCylinder (CollisionDetect.cpp:958-1137): both axes, the four cap
// 8-gons' edges against the other barrel, the barrel-barrel axis, Gauss-arc
// pairs; then the contact cases (rim point, parallel barrels, clipping).
__device__ bool cylinderCylinder(const PrimView& A, const PrimView& B, int lane, Scratch& scratch, CP* clipped,
                                 int* status, PrimOut* o) {
    const int r0 = 2, bb = r0 + 4 * kCylCap, a0 = bb + 1, total = a0 + 4 * kCylRing * kCylRing;
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    for (int t = lane; t < total; t += 32) {
        f3 n;
        if (t == 0) n = A.axis;
        else if (t == 1) n = B.axis;
        else if (t < bb) {
            int k = t - r0, ring = k / kCylCap, i = k - ring * kCylCap;
            const float4* pts = ring == 0 ? A.top : ring == 1 ? A.bot : ring == 2 ? B.top : B.bot;
            if (!ringAxis(pts, i, ring < 2 ? B.axis : A.axis, &n)) continue;
        } else if (t == bb) {
            f3 x = cross(A.axis, B.axis);
            if (!(mag2(x) > 0.00000001f)) continue;
            n = normalize(x);
        } else {
            int k = t - a0, ia = k / (2 * kCylRing), ib = k - ia * (2 * kCylRing);
            f3 a1, a2, b1, b2;
            cylArc(A, ia, &a1, &a2);
            cylArc(B, ib, &b1, &b2);
            if (!arcAxis(a1, a2, -b1, -b2, &n)) continue;
        }
        check(cylExt(A, n), cylExt(B, n), n, t, &best, &sep);
    }
    if (__any_sync(0xffffffffu, sep)) return false;
    Axis b = warp_best(best);
    if (!(b.pen < INFINITY)) return false;
    if (lane == 0) {
        f3 n = b.n, u, w;
        basis(n, &u, &w);
        Area ac, bc;
        int ka = cylArea(A, n, u, w, &ac);
        int kb = cylArea(B, -1.f * n, u, w, &bc);
        int m;
        if (ka == 2) { clipped[0] = CP{ac.ps[0], 0, 0ull, 0}; m = 1; }
        else if (kb == 2) { clipped[0] = CP{bc.ps[0], 0, 0ull, 0}; m = 1; }
        else if (ka == 1 && kb == 1 && fabsf(dot(A.axis, B.axis)) > 0.995f) {
            // parallel barrels: overlap of the two lines along A's axis
            f3 ba = normalize(n - A.axis * dot(A.axis, n));
            f3 a1 = A.c + ba * A.r + (0.5f * A.h) * A.axis, a2 = a1 - A.h * A.axis;
            f3 bbv = normalize(-1.f * n - B.axis * dot(B.axis, -1.f * n));
            f3 b1 = B.c + bbv * B.r + (0.5f * B.h) * B.axis, b2 = b1 - B.h * B.axis;
            if (dot(B.axis, A.axis) < 0.f) { f3 t = b1; b1 = b2; b2 = t; }
            float amx = dot(a1, A.axis), amn = dot(a2, A.axis), bmx = dot(b1, A.axis), bmn = dot(b2, A.axis);
            f3 imx = (amx > bmx) ? b1 : a1;
            f3 imn = (amn > bmn) ? a2 : b2;
            clipped[0] = CP{P2{dot(u, imx), dot(w, imx)}, 0, 0ull, 0};
            clipped[1] = CP{P2{dot(u, imn), dot(w, imn)}, 0, 1ull, 0};
            m = 2;
        } else {
            m = clipContacts(ac, bc, scratch, clipped, status);
        }
        f3 amax = diskExtremum(dot(A.axis, n) > 0.f ? topCenter(A) : botCenter(A), A.axis, A.r, n);
        points_from_pool(clipped, m, u, w, n, dot(amax, n), b.pen, o);
        o->n = n;
        o->pen = b.pen;
    }
    return true;
}

// ---- capsules ----------------------------------------------------------------------
__device__ __forceinline__ f3 capTop(const PrimView& c) { return c.c + c.axis * (0.5f * c.h); }
__device__ __forceinline__ f3 capBot(const PrimView& c) { return c.c - c.axis * (0.5f * c.h); }

// getCapsuleExtrema (CollisionDetect.cpp:685-703): the two cap spheres
__device__ __forceinline__ Ext capExt(const PrimView& c, f3 d) {
    float v1 = dot(d, capTop(c)), v2 = dot(d, capBot(c));
    return Ext{fminf(v1 - c.r, v2 - c.r), fmaxf(v1 + c.r, v2 + c.r), -1, -1};
}

// findCapsuleContactArea (CollisionDetect.cpp:376-390): 1 for the barrel line
// (ids 0 = top cap, 1 = bottom cap), 2 for the single cap point
__device__ int capArea(const PrimView& c, f3 n, f3 u, f3 w, Area* a) {
    if (fabsf(dot(c.axis, n)) <= kSinTol) {
        f3 barrel = normalize(n - c.axis * dot(c.axis, n));
        f3 p1 = c.c + barrel * c.r + (0.5f * c.h) * c.axis;
        f3 p2 = p1 - c.h * c.axis;
        a->ps[0] = P2{dot(p1, u), dot(p1, w)};
        a->ps[1] = P2{dot(p2, u), dot(p2, w)};
        a->ids[0] = 0;
        a->ids[1] = 1;
        a->n = 2;
        a->surface = -1;
        return 1;
    }
    const bool top = dot(n, c.axis) > 0.f;
    f3 q = top ? n * c.r + c.c + c.axis * (0.5f * c.h) : n * c.r + c.c - c.axis * (0.5f * c.h);
    a->ps[0] = P2{dot(q, u), dot(q, w)};
    a->ids[0] = top ? 0 : 1;
    a->n = 1;
    a->surface = -1;
    return 2;
}

// two parallel barrel lines (A's along n, B's along -n) clipped to their
// overlap along A's axis, as detectCapsuleCapsule / detectCapsuleCylinder build
// the contact (CollisionDetect.cpp:1277-1297, 1947-1966)
__device__ int parallelBarrels(const PrimView& A, const PrimView& B, f3 n, f3 u, f3 w, CP* out) {
    f3 ba = normalize(n - A.axis * dot(A.axis, n));
    f3 a1 = A.c + ba * A.r + (0.5f * A.h) * A.axis, a2 = a1 - A.h * A.axis;
    f3 bbv = normalize(-1.f * n - B.axis * dot(B.axis, -1.f * n));
    f3 b1 = B.c + bbv * B.r + (0.5f * B.h) * B.axis, b2 = b1 - B.h * B.axis;
    if (dot(B.axis, A.axis) < 0.f) { f3 t = b1; b1 = b2; b2 = t; }
    float amx = dot(a1, A.axis), amn = dot(a2, A.axis), bmx = dot(b1, A.axis), bmn = dot(b2, A.axis);
    f3 imx = (amx > bmx) ? b1 : a1;
    f3 imn = (amn > bmn) ? a2 : b2;
    out[0] = CP{P2{dot(u, imx), dot(w, imx)}, 0, 0ull, 0};
    out[1] = CP{P2{dot(u, imn), dot(w, imn)}, 0, 1ull, 0};
    return 2;
}

// detectSphereCapsule (CollisionDetect.cpp:868-935): the radial direction to
// the capsule axis, then the directions to both cap centres
__device__ bool sphereCapsule(const PrimView& S, const PrimView& C, PrimOut* o) {
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    f3 ax = C.axis;
    f3 diff = C.c - S.c;
    f3 barrel = normalize(diff - ax * dot(ax, diff));
    check(sphereExt(S, barrel), capExt(C, barrel), barrel, 0, &best, &sep);
    if (sep) return false;
    f3 e1 = normalize(capTop(C) - S.c);
    check(sphereExt(S, e1), capExt(C, e1), e1, 1, &best, &sep);
    if (sep) return false;
    f3 e2 = normalize(capBot(C) - S.c);
    check(sphereExt(S, e2), capExt(C, e2), e2, 2, &best, &sep);
    if (sep || !(best.pen < INFINITY)) return false;
    f3 q = S.c + best.n * S.r;
    o->n = best.n;
    o->pen = best.pen;
    o->pts[0] = make_float4(q.x, q.y, q.z, best.pen);
    o->magic[0] = 0ull;
    o->m = 1;
    return true;
}

// detectCapsuleCapsule (CollisionDetect.cpp:1139-1334): the reference's eight
// axes in its order (cap-centre pairs top-top, b top - a bottom,
// bottom-bottom; a's caps against b's barrel; b's caps against a's barrel,
// taken from b's centre; barrel x barrel), one lane each; then the parallel-
// barrel case or clipping
__device__ bool capsuleCapsule(const PrimView& A, const PrimView& B, int lane, Scratch& scratch, CP* clipped,
                               int* status, PrimOut* o) {
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    const f3 at = capTop(A), ab = capBot(A), bt = capTop(B), bb = capBot(B);
    if (lane < 8) {
        f3 n;
        bool use = true;
        switch (lane) {
        case 0: n = normalize(bt - at); break;
        case 1: n = normalize(bt - ab); break;
        case 2: n = normalize(bb - ab); break;
        case 3: { f3 d = B.c - at; n = normalize(d - B.axis * dot(B.axis, d)); } break;
        case 4: { f3 d = B.c - ab; n = normalize(d - B.axis * dot(B.axis, d)); } break;
        case 5: { f3 d = B.c - bt; n = normalize(d - A.axis * dot(A.axis, d)); } break;
        case 6: { f3 d = B.c - bb; n = normalize(d - A.axis * dot(A.axis, d)); } break;
        default: {
            f3 x = cross(A.axis, B.axis);
            use = mag2(x) > 0.00000001f;
            n = use ? normalize(x) : x;
        }
        }
        if (use) check(capExt(A, n), capExt(B, n), n, lane, &best, &sep);
    }
    if (__any_sync(0xffffffffu, sep)) return false;
    Axis b = warp_best(best);
    if (!(b.pen < INFINITY)) return false;
    if (lane == 0) {
        f3 n = b.n, u, w;
        basis(n, &u, &w);
        Area ac, bc;
        int ka = capArea(A, n, u, w, &ac);
        int kb = capArea(B, -1.f * n, u, w, &bc);
        int m;
        if (ka == 1 && kb == 1 && fabsf(dot(A.axis, B.axis)) > 0.995f) m = parallelBarrels(A, B, n, u, w, clipped);
        else m = clipContacts(ac, bc, scratch, clipped, status);
        f3 amax = dot(A.axis, n) > 0.f ? at + n * A.r : ab + n * A.r;
        points_from_pool(clipped, m, u, w, n, dot(amax, n), b.pen, o);
        o->n = n;
        o->pen = b.pen;
    }
    return true;
}

// SAT_PolyCapsule (CollisionDetect.cpp:1413-1561): the hull's faces, its
// vertices (radially to the drum, or to the nearer cap centre), and per edge
// the cap axis, again the cap axis (the reference's "bottom cap" test samples
// the top cap, :1486-1488) and edge x height axis; the reference places the
// cap centres a full drum height from the centre in this function
// (:1436-1437).  Contact by clipping the hull feature against the capsule's.
__device__ bool polyCapsule(const HullView& A, const PrimView& C, int lane, Scratch& scratch, CP* clipped,
                            int* status, PrimOut* o) {
    const HullHeader& H = *A.h;
    const int nf = H.nf, nv = H.nv, ne = H.ne;
    const uint8_t* edges = A.g + H.off_edge;
    const int v0 = nf, e0 = nf + nv, total = e0 + 3 * ne;
    const f3 ax = C.axis;
    const f3 tcc = C.c + ax * C.h, bcc = C.c - ax * C.h;
    const float tv = dot(tcc, ax), bv = dot(bcc, ax);
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    for (int t = lane; t < total; t += 32) {
        Ext ea;
        f3 n;
        if (t < nf) {
            float4 g = A.n[t];
            if (g.w != 0.f) continue;
            n = mk(g);
            float4 c = A.cache[t];
            float shift = dot(n, A.com);
            ea = Ext{c.y + shift, c.x + shift, __float_as_int(c.w), __float_as_int(c.z)};
        } else {
            if (t < e0) {
                f3 p = mk(A.v[t - v0]);
                float v = dot(p, ax);
                if (bv <= v && v <= tv) n = normalize((p - C.c) - ax * dot(ax, p - C.c));
                else if (v > tv) n = normalize(p - tcc);
                else n = normalize(p - bcc);
            } else {
                int k = t - e0, e = k / 3, which = k - 3 * e;
                f3 p1 = mk(A.v[edges[2 * e]]), p2 = mk(A.v[edges[2 * e + 1]]);
                f3 dir = normalize(p2 - p1);
                if (which < 2) {
                    f3 sample = p1 - tcc;
                    n = normalize(sample - dir * dot(dir, sample));
                } else if (!edgeAxis(dir, ax, &n)) {
                    continue;
                }
            }
            ea = extrema(A.v, nv, n);
        }
        check(ea, capExt(C, n), n, t, &best, &sep);
    }
    if (__any_sync(0xffffffffu, sep)) return false;
    Axis b = warp_best(best);
    if (!(b.pen < INFINITY) || b.aid < 0) return false;
    if (lane == 0) {
        f3 n = b.n, u, w;
        basis(n, &u, &w);
        Area ac, bc;
        contactArea(A, n, b.aid, u, w, &ac);
        capArea(C, -1.f * n, u, w, &bc);
        int m = clipContacts(ac, bc, scratch, clipped, status);
        points_from_pool(clipped, m, u, w, n, dot(mk(A.v[b.aid]), n), b.pen, o);
        o->n = n;
        o->pen = b.pen;
    }
    return true;
}

// detectCapsuleCylinder (CollisionDetect.cpp:1794-2002): the cylinder axis, its
// top 8-gon's edges x the capsule axis, both rim points (towards each cap
// centre) of both cylinder caps, each cap centre radially to the cylinder,
// barrel x barrel; then the rim point, parallel barrels or clipping
__device__ bool capsuleCylinder(const PrimView& A, const PrimView& B, int lane, Scratch& scratch, CP* clipped,
                                int* status, PrimOut* o) {
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    const f3 at = capTop(A), ab = capBot(A);
    if (lane < 16) {
        f3 n;
        bool use = true;
        if (lane == 0) n = B.axis;
        else if (lane <= kCylCap) use = ringAxis(B.top, lane - 1, A.axis, &n);
        else if (lane <= kCylCap + 4) {
            const int k = lane - kCylCap - 1;
            const f3 disk = k < 2 ? topCenter(B) : botCenter(B);
            const f3 cap = (k & 1) ? ab : at;
            f3 cp = diskExtremum(disk, B.axis, B.r, normalize(cap - B.c));
            n = normalize(cp - cap);
        } else if (lane <= kCylCap + 6) {
            f3 d = B.c - (lane == kCylCap + 5 ? at : ab);
            n = normalize(d - B.axis * dot(B.axis, d));
        } else {
            f3 x = cross(A.axis, B.axis);
            use = mag2(x) > 0.00000001f;
            n = use ? normalize(x) : x;
        }
        if (use) check(capExt(A, n), cylExt(B, n), n, lane, &best, &sep);
    }
    if (__any_sync(0xffffffffu, sep)) return false;
    Axis b = warp_best(best);
    if (!(b.pen < INFINITY)) return false;
    if (lane == 0) {
        f3 n = b.n, u, w;
        basis(n, &u, &w);
        Area ac, bc;
        int ka = capArea(A, n, u, w, &ac);
        int kb = cylArea(B, -1.f * n, u, w, &bc);
        int m;
        if (kb == 2) { clipped[0] = CP{bc.ps[0], 0, 0ull, 0}; m = 1; }
        else if (ka == 1 && kb == 1 && fabsf(dot(A.axis, B.axis)) > 0.995f) m = parallelBarrels(A, B, n, u, w, clipped);
        else m = clipContacts(ac, bc, scratch, clipped, status);
        f3 amax = dot(A.axis, n) > 0.f ? at + n * A.r : ab + n * A.r;
        points_from_pool(clipped, m, u, w, n, dot(amax, n), b.pen, o);
        o->n = n;
        o->pen = b.pen;
    }
    return true;
}

// detectCollision's primitive dispatch (CollisionDetect.cpp:57-150) for every
// pair involving a sphere, cylinder or capsule.  Pairs the detectors take the other way
// round are flipped back: normal negated, both MagicID halves swapped.
// the detector of a pair of primitives of which at least one is a sphere,
// cylinder or capsule (blobs staged at sa / sb): on lane 0, whether they
// touch and the manifold before the cull, in the pair's order (a first)
__device__ __forceinline__ bool narrow_prim_out(const Dev& d, int a, int b, uint8_t* sa, uint8_t* sb, const uint8_t* ga,
                                             const uint8_t* gb, uint32_t ka, uint32_t kb, int lane, Scratch& scratch,
                                             CP* clipped, PrimOut& o) {
    HullView hv;
    PrimView pa, pb;
    if (ka == SHAPE_HULL) stage_hull(ga, sa, d.pos[a], d.rot[a], &hv, lane);
    else stage_prim(sa, d.pos[a], d.rot[a], &pa, lane);
    if (kb == SHAPE_HULL) stage_hull(gb, sb, d.pos[b], d.rot[b], &hv, lane);
    else stage_prim(sb, d.pos[b], d.rot[b], &pb, lane);
    __syncwarp();
    o.m = 0;
    bool hit, flip = false;
    if (ka == SHAPE_HULL || kb == SHAPE_HULL) {
        flip = kb == SHAPE_HULL;
        const PrimView& q = flip ? pa : pb;
        const uint32_t kq = flip ? ka : kb;
        if (kq == SHAPE_SPHERE) hit = polySphere(hv, q, lane, &o);
        else if (kq == SHAPE_CAPSULE) hit = polyCapsule(hv, q, lane, scratch, clipped, d.status, &o);
        else hit = polyCylinder(hv, q, lane, scratch, clipped, d.status, &o);
    } else if (ka == SHAPE_SPHERE && kb == SHAPE_SPHERE) {
        hit = sphereSphere(pa, pb, &o);
    } else if (ka == SHAPE_SPHERE || kb == SHAPE_SPHERE) {
        flip = kb == SHAPE_SPHERE;
        const PrimView& s = flip ? pb : pa;
        const PrimView& q = flip ? pa : pb;
        hit = (flip ? ka : kb) == SHAPE_CAPSULE ? sphereCapsule(s, q, &o) : sphereCylinder(s, q, &o);
    } else if (ka == SHAPE_CAPSULE && kb == SHAPE_CAPSULE) {
        hit = capsuleCapsule(pa, pb, lane, scratch, clipped, d.status, &o);
    } else if (ka == SHAPE_CAPSULE || kb == SHAPE_CAPSULE) {
        flip = kb == SHAPE_CAPSULE;
        hit = flip ? capsuleCylinder(pb, pa, lane, scratch, clipped, d.status, &o)
                   : capsuleCylinder(pa, pb, lane, scratch, clipped, d.status, &o);
    } else {
        hit = cylinderCylinder(pa, pb, lane, scratch, clipped, d.status, &o);
    }
    if (lane != 0) return false;
    if (!hit || !(o.pen > 0.f) || o.m == 0) return false;
    if (flip) {
        o.n = -1.f * o.n;
        for (int i = 0; i < o.m; i++) {
            unsigned long long x = o.magic[i];
            o.magic[i] = (x >> 32) | (x << 32);
        }
    }
    return true;
}

__device__ __forceinline__ void narrow_prim(const Dev& d, int p, int a, int b, uint8_t* sa, uint8_t* sb, const uint8_t* ga,
                                         const uint8_t* gb, uint32_t ka, uint32_t kb, int lane, Scratch& scratch,
                                         CP* clipped) {
    PrimOut o;
    const bool hit = narrow_prim_out(d, a, b, sa, sb, ga, gb, ka, kb, lane, scratch, clipped, o);
    if (lane != 0) return;
    if (!hit) no_manifold(d, p);
    else emit_manifold(d, p, o.n, o.pen, o.pts, o.magic, o.m);
}

// ---- static triangle meshes --------------------------------------------------------
// One face of a StaticMeshGeometry (Geometry.h:120-175) read from the mesh blob.
struct TriView {
    f3 n;            // face normal
    int concave;     // concave neighbours (normalDirectionValid's case)
    f3 v[3], out[3]; // vertices; outward edge directions (edge i: v[i] -> v[i+1])
    f3 g[3];         // Gauss region
    int ng;
    int eid[3], id;
    f3 lo, hi;
};

__device__ __forceinline__ void load_tri(const float4* t, TriView* T) {
    float4 x = __ldg(t);
    T->n = mk(x);
    T->concave = __float_as_int(x.w);
    for (int i = 0; i < 3; i++) T->v[i] = mk(__ldg(t + 1 + i));
    for (int i = 0; i < 3; i++) T->out[i] = mk(__ldg(t + 4 + i));
    float4 g0 = __ldg(t + 7);
    T->g[0] = mk(g0);
    T->ng = __float_as_int(g0.w);
    T->g[1] = mk(__ldg(t + 8));
    T->g[2] = mk(__ldg(t + 9));
    int4 ids = __ldg(reinterpret_cast<const int4*>(t + 10));
    T->eid[0] = ids.x; T->eid[1] = ids.y; T->eid[2] = ids.z; T->id = ids.w;
    T->lo = mk(__ldg(t + 11));
    T->hi = mk(__ldg(t + 12));
}

// findTriangleExtrema (CollisionDetect.cpp:2004-2021)
__device__ __forceinline__ Ext triExt(const TriView& T, f3 d) {
    Ext e{INFINITY, -INFINITY, -1, -1};
    for (int i = 0; i < 3; i++) {
        float x = dot(T.v[i], d);
        if (x < e.mn) { e.mn = x; e.mn_id = i; }
        if (x > e.mx) { e.mx = x; e.mx_id = i; }
    }
    return e;
}

// normalDirectionValid (CollisionDetect.cpp:2024-2060): the direction lies in
// the face's Gauss region (a spherical triangle, an arc, or the normal alone)
__device__ bool triNormalValid(const TriView& T, f3 n) {
    const float eps = 0.0001f;
    if (T.concave <= 1) {
        for (int i = 0; i < T.ng; i++)
            if (dot(n, cross(T.g[i], T.g[(i + 1) % T.ng])) < -eps) return false;
        return true;
    }
    if (T.concave == 2) {
        f3 arc = cross(T.g[0], T.g[1]);
        if (fabsf(dot(n, arc)) > eps) return false;
        if (dot(n, cross(arc, T.g[0])) < -eps) return false;
        return !(dot(n, cross(T.g[1], arc)) < -eps);
    }
    return !(dot(n, T.n) < 1.f - eps);
}

// one axis of a triangle SAT: the plain minimum and the minimum whose contact
// normal (pointing into the triangle) lies in the face's Gauss region, both
// first-in-order on ties
__device__ __forceinline__ void triCheck(const Ext& a, const Ext& b, f3 n, int idx, const TriView& T, Axis* best,
                                         Axis* valid, bool* sep) {
    float fwd = a.mx - b.mn, rev = b.mx - a.mn;
    Axis x;
    if (fwd < rev) x = Axis{fwd, idx, a.mx_id, b.mn_id, n};
    else x = Axis{rev, idx, a.mn_id, b.mx_id, -n};
    if (x.pen < 0.f) { *sep = true; return; }
    if (x.pen < best->pen || (x.pen == best->pen && idx < best->idx)) *best = x;
    if ((x.pen < valid->pen || (x.pen == valid->pen && idx < valid->idx)) && triNormalValid(T, -1.f * x.n)) *valid = x;
}

// the six Gauss arcs of a face, negated as the other side of an arc pair:
// normal -> out[i], out[i] -> -normal
__device__ __forceinline__ void triArc(const TriView& T, int k, f3* b1, f3* b2) {
    const int i = k >> 1;
    if ((k & 1) == 0) { *b1 = -1.f * T.n; *b2 = -1.f * T.out[i]; }
    else { *b1 = -1.f * T.out[i]; *b2 = T.n; }
}

// findTriangleContactArea (CollisionDetect.cpp:303-329): the face (ids 0..2,
// surface = face id), an edge next to vertex pid (both ids the edge id), or
// the vertex
__device__ void triArea(const TriView& T, f3 n, f3 p, int pid, f3 u, f3 w, Area* a) {
    if (1.f - dot(T.n, n) <= kCosTol) {
        for (int i = 0; i < 3; i++) { a->ps[i] = P2{dot(T.v[i], u), dot(T.v[i], w)}; a->ids[i] = i; }
        a->n = 3;
        a->surface = T.id;
        return;
    }
    for (int i = 0; i < 3; i++) {
        if (i != pid && (i + 1) % 3 != pid) continue;
        f3 e1 = T.v[i], e2 = T.v[(i + 1) % 3];
        if (fabsf(dot(normalize(e2 - e1), n)) <= kSinTol) {
            a->ps[0] = P2{dot(e1, u), dot(e1, w)};
            a->ps[1] = P2{dot(e2, u), dot(e2, w)};
            a->ids[0] = a->ids[1] = T.eid[i];
            a->n = 2;
            a->surface = -1;
            return;
        }
    }
    a->ps[0] = P2{dot(p, u), dot(p, w)};
    a->ids[0] = pid;
    a->n = 1;
    a->surface = -1;
}

// penalised choice of a triangle SAT: the Gauss-valid minimum when it is
// within `penalty` of the plain one
__device__ __forceinline__ bool triChoose(const Axis& best, const Axis& valid, float penalty, bool sep, Axis* ng, Axis* mp) {
    if (__any_sync(0xffffffffu, sep)) return false;
    *ng = warp_best(best);
    Axis v = warp_best(valid);
    *mp = (v.pen < ng->pen + penalty) ? v : *ng;
    return mp->pen < INFINITY;
}

// SAT_PolyTriangle (CollisionDetect.cpp:2062-2194): the face normal, the hull's
// faces, hull-arc x face-arc pairs; features and clipping from the plain
// minimum, the manifold normal and depth from the penalised choice
__device__ bool polyTri(const HullView& A, const TriView& T, float penalty, int lane, Scratch& scratch, CP* clipped,
                        int* status, PrimOut* o) {
    const HullHeader& H = *A.h;
    const int nf = H.nf, nv = H.nv, na = H.na, total = 1 + nf + 6 * na;
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)}, valid = best;
    bool sep = false;
    for (int t = lane; t < total; t += 32) {
        Ext ea;
        f3 n;
        if (t == 0) {
            n = T.n;
            ea = extrema(A.v, nv, n);
        } else if (t <= nf) {
            float4 g = A.n[t - 1];
            if (g.w != 0.f) continue;
            n = mk(g);
            float4 c = A.cache[t - 1];
            float shift = dot(n, A.com);
            ea = Ext{c.y + shift, c.x + shift, __float_as_int(c.w), __float_as_int(c.z)};
        } else {
            int k = t - 1 - nf, ia = k / 6;
            f3 b1, b2;
            triArc(T, k - 6 * ia, &b1, &b2);
            if (!arcAxis(mk(A.n[A.arc[2 * ia]]), mk(A.n[A.arc[2 * ia + 1]]), b1, b2, &n)) continue;
            ea = extrema(A.v, nv, n);
        }
        triCheck(ea, triExt(T, n), n, t, T, &best, &valid, &sep);
    }
    Axis ng, mp;
    if (!triChoose(best, valid, penalty, sep, &ng, &mp) || ng.aid < 0 || ng.bid < 0) return false;
    if (lane == 0) {
        f3 n = mp.n, u, w;
        basis(n, &u, &w);
        Area ac, bc;
        contactArea(A, ng.n, ng.aid, u, w, &ac);
        triArea(T, -1.f * ng.n, T.v[ng.bid], ng.bid, u, w, &bc);
        int m = clipContacts(ac, bc, scratch, clipped, status);
        points_from_pool(clipped, m, u, w, n, dot(mk(A.v[ng.aid]), n), mp.pen, o);
        o->n = n;
        o->pen = mp.pen;
    }
    return true;
}

// SAT_SphereTriangle (CollisionDetect.cpp:2196-2276): the face normal, the
// vertices and the edges; the point is the sphere's deepest one along the
// chosen normal, its feature id the vertex (0..2) or edge id of the plain
// minimum (none, 0xFFFFFFFF, when the face normal is the minimum)
__device__ bool sphereTri(const PrimView& S, const TriView& T, float penalty, int lane, PrimOut* o) {
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)}, valid = best;
    bool sep = false;
    if (lane < 7) {
        f3 n;
        if (lane == 0) n = T.n;
        else if (lane < 4) n = normalize(T.v[lane - 1] - S.c);
        else {
            int i = lane - 4;
            f3 dir = normalize(T.v[(i + 1) % 3] - T.v[i]);
            f3 sample = T.v[i] - S.c;
            n = normalize(sample - dir * dot(dir, sample));
        }
        triCheck(sphereExt(S, n), triExt(T, n), n, lane, T, &best, &valid, &sep);
    }
    Axis ng, mp;
    if (!triChoose(best, valid, penalty, sep, &ng, &mp)) return false;
    if (lane == 0) {
        uint32_t feature = 0xFFFFFFFFu;
        if (ng.idx >= 1 && ng.idx < 4) feature = (uint32_t)(ng.idx - 1);
        else if (ng.idx >= 4) feature = (uint32_t)T.eid[ng.idx - 4];
        f3 q = S.c + mp.n * S.r;
        o->n = mp.n;
        o->pen = mp.pen;
        o->pts[0] = make_float4(q.x, q.y, q.z, mp.pen);
        o->magic[0] = feature;
        o->m = 1;
    }
    return true;
}

// SAT_CylinderTriangle (CollisionDetect.cpp:2466-2646): the cylinder axis, the
// face normal, face edges x axis, the vertices radially, cylinder-arc x
// face-arc pairs; the rim point or the clipped cap / barrel line
__device__ bool cylTri(const PrimView& C, const TriView& T, float penalty, int lane, Scratch& scratch, CP* clipped,
                       int* status, PrimOut* o) {
    const int a0 = 8, total = a0 + 2 * kCylRing * 6;
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)}, valid = best;
    bool sep = false;
    for (int t = lane; t < total; t += 32) {
        f3 n;
        if (t == 0) n = C.axis;
        else if (t == 1) n = T.n;
        else if (t < 5) {
            int i = t - 2;
            if (!edgeAxis(T.v[(i + 1) % 3] - T.v[i], C.axis, &n)) continue;
        } else if (t < a0) {
            f3 diff = T.v[t - 5] - C.c;
            n = normalize(diff - C.axis * dot(C.axis, diff));
        } else {
            int k = t - a0, ia = k / 6;
            f3 g1, g2, b1, b2;
            cylArc(C, ia, &g1, &g2);
            triArc(T, k - 6 * ia, &b1, &b2);
            if (!arcAxis(g1, g2, b1, b2, &n)) continue;
        }
        triCheck(cylExt(C, n), triExt(T, n), n, t, T, &best, &valid, &sep);
    }
    Axis ng, mp;
    if (!triChoose(best, valid, penalty, sep, &ng, &mp) || ng.bid < 0) return false;
    if (lane == 0) {
        f3 n = mp.n, u, w;
        basis(n, &u, &w);
        f3 amax = diskExtremum(dot(C.axis, n) > 0.f ? topCenter(C) : botCenter(C), C.axis, C.r, n);
        Area ac, bc;
        int ak = cylArea(C, ng.n, u, w, &ac);
        triArea(T, -1.f * ng.n, T.v[ng.bid], ng.bid, u, w, &bc);
        int m;
        if (ak == 2) { clipped[0] = CP{ac.ps[0], 0, 0ull, 0}; m = 1; }
        else m = clipContacts(ac, bc, scratch, clipped, status);
        points_from_pool(clipped, m, u, w, n, dot(amax, n), mp.pen, o);
        o->n = n;
        o->pen = mp.pen;
    }
    return true;
}

// SAT_CapsuleTriangle (CollisionDetect.cpp:2278-2464): the face normal, face
// edges x capsule axis, the vertices radially, the vertices and the edges
// against the cap centres; the reference computes its "bottom" cap centre
// with +h/2 too (:2285-2286), so both sets of cap axes use the top cap (and
// the deepest point is always on the top cap); kept.  One lane per axis.
__device__ bool capTri(const PrimView& C, const TriView& T, float penalty, int lane, Scratch& scratch, CP* clipped,
                       int* status, PrimOut* o) {
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)}, valid = best;
    bool sep = false;
    const f3 ax = C.axis;
    const f3 at = capTop(C), ab = capTop(C);
    if (lane < 19) {
        f3 n;
        bool use = true;
        if (lane == 0) n = T.n;
        else if (lane < 4) use = edgeAxis(T.v[lane % 3] - T.v[lane - 1], ax, &n);
        else if (lane < 7) {
            f3 diff = T.v[lane - 4] - C.c;
            n = normalize(diff - ax * dot(ax, diff));
        } else if (lane < 13) {
            n = normalize(T.v[(lane - 7) % 3] - (lane < 10 ? at : ab));
        } else {
            const int i = (lane - 13) % 3;
            f3 dir = normalize(T.v[(i + 1) % 3] - T.v[i]);
            f3 sample = T.v[i] - (lane < 16 ? at : ab);
            n = normalize(sample - dir * dot(dir, sample));
        }
        if (use) triCheck(capExt(C, n), triExt(T, n), n, lane, T, &best, &valid, &sep);
    }
    Axis ng, mp;
    if (!triChoose(best, valid, penalty, sep, &ng, &mp) || ng.bid < 0) return false;
    if (lane == 0) {
        f3 n = mp.n, u, w;
        basis(n, &u, &w);
        f3 amax = dot(ax, n) > 0.f ? at + n * C.r : ab + n * C.r;
        Area ac, bc;
        int ak = capArea(C, ng.n, u, w, &ac);
        triArea(T, -1.f * ng.n, T.v[ng.bid], ng.bid, u, w, &bc);
        int m;
        if (ak == 2) { clipped[0] = CP{ac.ps[0], 0, 0ull, 0}; m = 1; }
        else m = clipContacts(ac, bc, scratch, clipped, status);
        points_from_pool(clipped, m, u, w, n, dot(amax, n), mp.pen, o);
        o->n = n;
        o->pen = mp.pen;
    }
    return true;
}

__device__ __forceinline__ bool box_overlap(f3 alo, f3 ahi, f3 blo, f3 bhi) {
    return !(ahi.x < blo.x || alo.x > bhi.x || ahi.y < blo.y || alo.y > bhi.y || ahi.z < blo.z || alo.z > bhi.z);
}

__device__ __forceinline__ float longest(f3 lo, f3 hi) {
    return fmaxf(hi.x - lo.x, fmaxf(hi.y - lo.y, hi.z - lo.z));
}

// The manifolds of one (convex, mesh) pair after the per-triangle tests:
// PhysicsEngine.cpp:257-295 merges, in manifold order, every later manifold
// whose normal is within 1 degree of the current one (normal = normalised
// sum, points appended), culls each merged manifold to 4 points
// (cull_manifold) and adds its points with its normal.  Lane 0; returns the
// kept point count (their raw indices in S.out, normals in S.out_n).
__device__ int mesh_merge(MeshScratch& S, int nman, float* maxpen, int* status) {
    const float cs[4] = {1.0f, 6.123233995736766e-17f, -1.0f, -1.8369701987210297e-16f};
    const float sn[4] = {0.0f, 1.0f, 1.2246467991473532e-16f, -1.0f};
    unsigned long long merged = 0ull;
    int nout = 0;
    *maxpen = -1.f;
    for (int i = 0; i < nman; i++) {
        if ((merged >> i) & 1ull) continue;
        float4 mi = S.man_n[i];
        f3 gn = mk(mi);
        float gpen = mi.w;
        unsigned long long mem = 1ull << i;
        for (int j = i + 1; j < nman; j++) {
            if ((merged >> j) & 1ull) continue;
            float4 mj = S.man_n[j];
            if (1.f - dot(gn, mk(mj)) < kCosTol) {
                gn = normalize(gn + mk(mj));
                gpen = fmaxf(gpen, mj.w);
                merged |= 1ull << j;
                mem |= 1ull << j;
            }
        }
        *maxpen = fmaxf(*maxpen, gpen);
        int total = 0;
        for (unsigned long long b = mem; b; b &= b - 1) total += S.man_cnt[__ffsll((long long)b) - 1];
        int pick[4], np = 0;
        if (total <= 4) {
            for (unsigned long long b = mem; b; b &= b - 1) {
                const int m = __ffsll((long long)b) - 1;
                for (int k = 0; k < S.man_cnt[m]; k++) pick[np++] = S.man_first[m] + k;
            }
        } else {
            f3 cu, cw;
            basis(gn, &cu, &cw);
            for (int q = 0; q < 4; q++) {
                f3 dir = cu * cs[q] + cw * sn[q];
                int bi = -1;
                float bv = -INFINITY;
                for (unsigned long long b = mem; b; b &= b - 1) {
                    const int m = __ffsll((long long)b) - 1;
                    for (int k = 0; k < S.man_cnt[m]; k++) {
                        const int idx = S.man_first[m] + k;
                        bool used = false;
                        for (int r = 0; r < np; r++) used |= pick[r] == idx;
                        if (used) continue;
                        float v = dot(mk(S.pt[idx]), dir);
                        if (v > bv) { bv = v; bi = idx; }
                    }
                }
                if (bi < 0) break;
                pick[np++] = bi;
            }
        }
        for (int r = 0; r < np; r++) {
            if (nout >= kMeshOut) { atomicOr(status, ST_MESH_OVERFLOW); return nout; }
            S.out[nout] = pick[r];
            S.out_n[nout] = make_float4(gn.x, gn.y, gn.z, 0.f);
            nout++;
        }
    }
    return nout;
}

}  // namespace

// One warp per candidate pair; `slot_bytes` of shared memory per warp.
__global__ void __launch_bounds__(256) k_narrowphase(Dev d, int slot_bytes) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int warps_per_block = blockDim.x >> 5;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    uint8_t* qslot = smem + 16 * warps_per_block + (size_t)wib * (slot_bytes + kQueueBytes);
    uint8_t* slot = qslot + kQueueBytes;
    if (lane == 0) mbar_init(&bars[wib]);
    __syncthreads();
    uint32_t parity = 0;
    bool failed = false;
    const int n_pairs = *d.n_pairs;
    for (int p = blockIdx.x * warps_per_block + wib; p < n_pairs; p += gridDim.x * warps_per_block) {
        const int a = d.pair_a[p], b = d.pair_b[p];
        // pairs with a body of several primitives belong to k_narrow_mesh
        // (no manifold here, so that k_clip passes them over)
        if (is_union(d, a) || is_union(d, b)) {
            if (lane == 0) { d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f); d.mf_cnt[p] = 0; }
            continue;
        }
        const uint8_t* ga = d.shapes + d.shape[a];
        const uint8_t* gb = d.shapes + d.shape[b];
        // pairs with a sphere or cylinder belong to k_narrow_prim
        if ((reinterpret_cast<const HullHeader*>(ga)->kind | reinterpret_cast<const HullHeader*>(gb)->kind) != SHAPE_HULL) continue;
        // collision filter of PhysicsEngine.cpp:174 (at least one dynamic body)
        // and collisionAllowed; after a timed-out wait the warp writes empty
        // manifolds for the rest of its pairs, so no later kernel reads a
        // previous step's
        if (failed || !(d.movement[a] == 0 || d.movement[b] == 0) || both_asleep(d, a, b) || jointed(d, a, b)) {
            if (lane == 0) { d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f); d.mf_cnt[p] = 0; }
            continue;
        }
        const uint32_t hot_a = reinterpret_cast<const HullHeader*>(ga)->off_fofs;
        const uint32_t hot_b = reinterpret_cast<const HullHeader*>(gb)->off_fofs;
        uint8_t* sa = slot;
        uint8_t* sb = slot + ((hot_a + 15u) & ~15u);
        // order this warp's generic-proxy writes to the slot before the async copy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
            mbar_expect(&bars[wib], hot_a + hot_b);
            bulk_load(sa, ga, hot_a, &bars[wib]);
            bulk_load(sb, gb, hot_b, &bars[wib]);
        }
        bool ok = mbar_wait(&bars[wib], parity, d.wait_limit);
        parity ^= 1u;
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) { atomicOr(d.status, ST_TIMEOUT); d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f); d.mf_cnt[p] = 0; }
            // let the copies in flight land (bounded), then stop using the slot
            mbar_wait(&bars[wib], parity ^ 1u, kDefaultWaitLimit);
            failed = true;
            continue;
        }
        HullView A, B;
        stage_hull(ga, sa, d.pos[a], d.rot[a], &A, lane);
        stage_hull(gb, sb, d.pos[b], d.rot[b], &B, lane);
        __syncwarp();

        const int nva = A.h->nv, nvb = B.h->nv, nfa = A.h->nf, nfb = B.h->nf;
        Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
        bool sep = false;
        // face axes of A
        for (int f = lane; f < nfa; f += 32) {
            float4 g = A.n[f];
            if (g.w != 0.f) continue;
            f3 n = mk(g);
            float4 c = A.cache[f];
            float shift = dot(n, A.com);
            Ext ea{c.y + shift, c.x + shift, __float_as_int(c.w), __float_as_int(c.z)};
            check(ea, extrema(B.v, nvb, n), n, f, &best, &sep);
        }
        // face axes of B
        for (int f = lane; f < nfb; f += 32) {
            float4 g = B.n[f];
            if (g.w != 0.f) continue;
            f3 n = mk(g);
            float4 c = B.cache[f];
            float shift = dot(n, B.com);
            Ext eb{c.y + shift, c.x + shift, __float_as_int(c.w), __float_as_int(c.z)};
            check(extrema(A.v, nva, n), eb, n, nfa + f, &best, &sep);
        }
        if (__any_sync(0xffffffffu, sep)) {
            if (lane == 0) { d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f); d.mf_cnt[p] = 0; }
            continue;
        }
        // edge-edge axes from intersecting Gauss arcs.  The arc-pair tests are
        // cheap and uniform; the axes that pass need two support queries each,
        // so they are queued (ballot + prefix count) and then evaluated with
        // every lane taking one queued axis, instead of one lane at a time.
        const int naa = A.h->na, nab = B.h->na;
        const int total = naa * nab;
        float4* qn = reinterpret_cast<float4*>(qslot);
        int* qi = reinterpret_cast<int*>(qslot + kQueue * sizeof(float4));
        int qcount = 0;
        const unsigned lt_mask = (1u << lane) - 1u;
        for (int base = 0; base < total; base += 32) {
            int t = base + lane;
            bool pass = false;
            f3 n = mk(0.f, 0.f, 0.f);
            if (t < total) {
                int ia = t / nab, ib = t - ia * nab;
                f3 a1 = mk(A.n[A.arc[2 * ia]]), a2 = mk(A.n[A.arc[2 * ia + 1]]);
                f3 b1 = -mk(B.n[B.arc[2 * ib]]), b2 = -mk(B.n[B.arc[2 * ib + 1]]);
                f3 avg = a1 + a2;
                if (dot(avg, b1) + dot(avg, b2) > 0.f) {
                    f3 ap = cross(a1, a2), bp = cross(b1, b2);
                    if (!(dot(ap, b1) * dot(ap, b2) > 0.f || dot(bp, a1) * dot(bp, a2) > 0.f)) {
                        n = cross(ap, bp);
                        if (mag2(n) != 0.f) {
                            n = normalize(n);
                            if (dot(avg, n) < 0.f) n = n * -1.f;
                            pass = true;
                        }
                    }
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, pass);
            if (pass) {
                int at = qcount + __popc(m & lt_mask);
                qn[at] = make_float4(n.x, n.y, n.z, 0.f);
                qi[at] = nfa + nfb + t;
            }
            qcount += __popc(m);
            const bool last = base + 32 >= total;
            if (qcount > kQueue - 32 || last) {
                __syncwarp();
                for (int k = lane; k < qcount; k += 32) {
                    f3 ax = mk(qn[k]);
                    check(extrema(A.v, nva, ax), extrema(B.v, nvb, ax), ax, qi[k], &best, &sep);
                }
                qcount = 0;
                __syncwarp();
                if (__any_sync(0xffffffffu, sep)) break;
            }
        }
        if (__any_sync(0xffffffffu, sep)) {
            if (lane == 0) { d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f); d.mf_cnt[p] = 0; }
            continue;
        }
        // warp argmin over (pen, axis order)
        float bp = best.pen;
        int bi = best.idx;
        for (int o = 16; o > 0; o >>= 1) {
            float op = __shfl_xor_sync(0xffffffffu, bp, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (op < bp || (op == bp && oi < bi)) { bp = op; bi = oi; }
        }
        unsigned owner_mask = __ballot_sync(0xffffffffu, best.idx == bi && best.pen == bp);
        int owner = owner_mask ? __ffs(owner_mask) - 1 : 0;
        float nx = __shfl_sync(0xffffffffu, best.n.x, owner);
        float ny = __shfl_sync(0xffffffffu, best.n.y, owner);
        float nz = __shfl_sync(0xffffffffu, best.n.z, owner);
        int aid = __shfl_sync(0xffffffffu, best.aid, owner);
        int bid = __shfl_sync(0xffffffffu, best.bid, owner);
        // the axis and the two features; k_clip turns them into the manifold
        if (lane == 0) {
            if (!(bp < INFINITY) || aid < 0 || bid < 0) {
                d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f);
            } else {
                d.mf_n[p] = make_float4(nx, ny, nz, bp);
                d.mf_feat[p] = make_int2(aid, bid);
            }
            d.mf_cnt[p] = 0;
        }
    }
}

// Contact generation of the convex-hull pairs k_narrowphase found
// overlapping, one thread per pair: contact features (findContactArea,
// CollisionDetect.cpp:237-280), clipping (:394-620) and the 4-direction cull
// (:2795-2830).  The clip is serial per pair; a thread each keeps all lanes of
// a warp busy on 32 pairs, where a warp per pair would idle 31.
// the contact points of two hulls along the axis n (depth bp) between the
// features `feat`, before the cull; returns their count
__device__ int clip_hulls(const HullG& A, const HullG& B, f3 n, float bp, int2 feat, Scratch& scratch, CP* clipped, int* status,
                          float4* pts, unsigned long long* mag) {
    f3 u, w;
    basis(n, &u, &w);
    Area ac, bc;
    contactArea(A, n, feat.x, u, w, &ac);
    contactArea(B, -1.f * n, feat.y, u, w, &bc);
    const int m = clipContacts(ac, bc, scratch, clipped, status);
    const float a_dot = dot(A.vert(feat.x), n);
    const f3 off = n * a_dot;
    for (int i = 0; i < m; i++) {
        f3 q = u * clipped[i].p.x + w * clipped[i].p.y + off;
        pts[i] = make_float4(q.x, q.y, q.z, dot(q, n) - a_dot + bp);
        mag[i] = clipped[i].magic;
    }
    return m;
}

__global__ void __launch_bounds__(128) k_clip(Dev d) {
    const int n_pairs = *d.n_pairs;
    Scratch scratch;
    CP clipped[kMaxClip];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_pairs; p += gridDim.x * blockDim.x) {
        const float4 nn = d.mf_n[p];
        if (!(nn.w > 0.f)) continue;
        const int a = d.pair_a[p], b = d.pair_b[p];
        if (is_union(d, a) || is_union(d, b)) continue;
        const uint8_t* ga = d.shapes + d.shape[a];
        const uint8_t* gb = d.shapes + d.shape[b];
        if ((reinterpret_cast<const HullHeader*>(ga)->kind | reinterpret_cast<const HullHeader*>(gb)->kind) != SHAPE_HULL) continue;
        const HullG A(ga, d.pos[a], d.rot[a]), B(gb, d.pos[b], d.rot[b]);
        float4 pts[kMaxClip];
        unsigned long long mag[kMaxClip];
        const int m = clip_hulls(A, B, mk(nn), nn.w, d.mf_feat[p], scratch, clipped, d.status, pts, mag);
        emit_manifold(d, p, mk(nn), nn.w, pts, mag, m);
    }
}

// One warp per candidate pair that involves a sphere or a cylinder (the other
// pairs are k_narrowphase's).  Same staging as k_narrowphase.
__global__ void __launch_bounds__(256, 1) k_narrow_prim(Dev d, int slot_bytes) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int warps_per_block = blockDim.x >> 5;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    uint8_t* slot = smem + 16 * warps_per_block + (size_t)wib * slot_bytes;
    if (lane == 0) mbar_init(&bars[wib]);
    __syncthreads();
    uint32_t parity = 0;
    bool failed = false;
    Scratch scratch;
    CP clipped[kMaxClip];
    const int n_pairs = *d.n_pairs;
    for (int p = blockIdx.x * warps_per_block + wib; p < n_pairs; p += gridDim.x * warps_per_block) {
        const int a = d.pair_a[p], b = d.pair_b[p];
        const uint8_t* ga = d.shapes + d.shape[a];
        const uint8_t* gb = d.shapes + d.shape[b];
        const HullHeader* Ha = reinterpret_cast<const HullHeader*>(ga);
        const HullHeader* Hb = reinterpret_cast<const HullHeader*>(gb);
        const uint32_t ka = Ha->kind, kb = Hb->kind;
        if ((ka | kb) == SHAPE_HULL || ka == SHAPE_MESH || kb == SHAPE_MESH || is_union(d, a) || is_union(d, b)) continue;
        if (failed || !(d.movement[a] == 0 || d.movement[b] == 0) || both_asleep(d, a, b) || jointed(d, a, b)) {
            if (lane == 0) no_manifold(d, p);
            continue;
        }
        const uint32_t hot_a = Ha->off_fofs, hot_b = Hb->off_fofs;
        uint8_t* sa = slot;
        uint8_t* sb = slot + ((hot_a + 15u) & ~15u);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
            mbar_expect(&bars[wib], hot_a + hot_b);
            bulk_load(sa, ga, hot_a, &bars[wib]);
            bulk_load(sb, gb, hot_b, &bars[wib]);
        }
        bool ok = mbar_wait(&bars[wib], parity, d.wait_limit);
        parity ^= 1u;
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) { atomicOr(d.status, ST_TIMEOUT); no_manifold(d, p); }
            mbar_wait(&bars[wib], parity ^ 1u, kDefaultWaitLimit);
            failed = true;
            continue;
        }
        narrow_prim(d, p, a, b, sa, sb, ga, gb, ka, kb, lane, scratch, clipped);
    }
}

// SAT_PolyPoly's axis search (CollisionDetect.cpp:717-835) for two staged
// hulls by the whole warp: face normals of A, of B, then the edge pairs whose
// Gauss arcs cross, every lane taking strided axes; the minimum over
// (depth, axis order) is the same whatever lane meets an axis, so this equals
// k_narrowphase's queued form.  Returns false when an axis separates them.
__device__ bool sat_hulls(const HullView& A, const HullView& B, int lane, Axis* out) {
    const int nva = A.h->nv, nvb = B.h->nv, nfa = A.h->nf, nfb = B.h->nf;
    Axis best{INFINITY, 0x7fffffff, -1, -1, mk(0.f, 0.f, 0.f)};
    bool sep = false;
    for (int f = lane; f < nfa; f += 32) {
        float4 g = A.n[f];
        if (g.w != 0.f) continue;
        f3 n = mk(g);
        float4 c = A.cache[f];
        float shift = dot(n, A.com);
        Ext ea{c.y + shift, c.x + shift, __float_as_int(c.w), __float_as_int(c.z)};
        check(ea, extrema(B.v, nvb, n), n, f, &best, &sep);
    }
    for (int f = lane; f < nfb; f += 32) {
        float4 g = B.n[f];
        if (g.w != 0.f) continue;
        f3 n = mk(g);
        float4 c = B.cache[f];
        float shift = dot(n, B.com);
        Ext eb{c.y + shift, c.x + shift, __float_as_int(c.w), __float_as_int(c.z)};
        check(extrema(A.v, nva, n), eb, n, nfa + f, &best, &sep);
    }
    if (__any_sync(0xffffffffu, sep)) return false;
    const int naa = A.h->na, nab = B.h->na, total = naa * nab;
    for (int base = 0; base < total; base += 32) {
        const int t = base + lane;
        if (t < total) {
            int ia = t / nab, ib = t - ia * nab;
            f3 a1 = mk(A.n[A.arc[2 * ia]]), a2 = mk(A.n[A.arc[2 * ia + 1]]);
            f3 b1 = -mk(B.n[B.arc[2 * ib]]), b2 = -mk(B.n[B.arc[2 * ib + 1]]);
            f3 avg = a1 + a2;
            if (dot(avg, b1) + dot(avg, b2) > 0.f) {
                f3 ap = cross(a1, a2), bp = cross(b1, b2);
                if (!(dot(ap, b1) * dot(ap, b2) > 0.f || dot(bp, a1) * dot(bp, a2) > 0.f)) {
                    f3 n = cross(ap, bp);
                    if (mag2(n) != 0.f) {
                        n = normalize(n);
                        if (dot(avg, n) < 0.f) n = n * -1.f;
                        check(extrema(A.v, nva, n), extrema(B.v, nvb, n), n, nfa + nfb + t, &best, &sep);
                    }
                }
            }
        }
        if (__any_sync(0xffffffffu, sep)) return false;
    }
    *out = warp_best(best);
    return out->pen < INFINITY && out->aid >= 0 && out->bid >= 0;
}

// One warp per candidate pair with a static mesh (the other pairs are
// k_narrowphase's and k_narrow_prim's): SAT_PolyMesh / SAT_SphereMesh /
// SAT_CylinderMesh (CollisionDetect.cpp:2648-2778) for a fixed mesh in world
// coordinates.  The convex body is staged as in k_narrow_prim; lane 0 walks
// the mesh's AABB tree (LIFO, right child first, as AABBTree::getAllOverlapping
// does) into the candidate list; each candidate triangle is tested by the
// whole warp, its manifold (flipped when the mesh is the pair's first body)
// appended to the warp's scratch; lane 0 then merges, culls and writes the
// pair's points to the mesh store.
__global__ void __launch_bounds__(256) k_narrow_mesh(Dev d, int slot_bytes) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int warps_per_block = blockDim.x >> 5;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    uint8_t* slot = smem + 16 * warps_per_block + (size_t)wib * slot_bytes;
    if (lane == 0) mbar_init(&bars[wib]);
    __syncthreads();
    const int gw = blockIdx.x * warps_per_block + wib;
    if (gw >= d.mesh_warps) return;
    MeshScratch& S = d.msc[gw];
    uint32_t parity = 0;
    bool failed = false;
    Scratch scratch;
    CP clipped[kMaxClip];
    const int n_pairs = *d.n_pairs;
    for (int p = gw; p < n_pairs; p += d.mesh_warps) {
        const int a = d.pair_a[p], b = d.pair_b[p];
        const uint8_t* ga = d.shapes + d.shape[a];
        const uint8_t* gb = d.shapes + d.shape[b];
        const uint32_t ka = reinterpret_cast<const HullHeader*>(ga)->kind, kb = reinterpret_cast<const HullHeader*>(gb)->kind;
        const bool ua = is_union(d, a), ub = is_union(d, b);
        if (lane == 0) d.mf_ofs[p] = -1;
        const bool mesh_pair = ka == SHAPE_MESH || kb == SHAPE_MESH;
        if (!mesh_pair && !ua && !ub) continue;
        // collision filter of PhysicsEngine.cpp:174 and collisionAllowed (a
        // static mesh is never asleep)
        if (failed || (ka == SHAPE_MESH && kb == SHAPE_MESH) || !(d.movement[a] == 0 || d.movement[b] == 0) ||
            (!mesh_pair && both_asleep(d, a, b)) || jointed(d, a, b)) {
            if (lane == 0) no_manifold(d, p);
            continue;
        }
        int nman = 0, npts = 0;   // lane 0's counts
        // a manifold (before the cull) into the pair's list, on lane 0
        auto add_manifold = [&](const PrimOut& o, bool flipped, int tri) {
            if (nman >= kMeshMans || npts + o.m > kMeshRaw) {
                atomicOr(d.status, ST_MESH_OVERFLOW);
                return;
            }
            f3 n = flipped ? -1.f * o.n : o.n;
            S.man_n[nman] = make_float4(n.x, n.y, n.z, o.pen);
            S.man_first[nman] = npts;
            S.man_cnt[nman] = o.m;
            for (int i = 0; i < o.m; i++) {
                unsigned long long x = o.magic[i];
                S.pt[npts + i] = o.pts[i];
                S.magic[npts + i] = flipped ? ((x >> 32) | (x << 32)) : x;
                S.tri[npts + i] = tri;
            }
            npts += o.m;
            nman++;
        };
        bool timed_out = false;
        // stage blobs into the warp's slot (bounded wait); false on a timeout
        auto stage = [&](const uint8_t* g1, uint8_t* s1, uint32_t h1, const uint8_t* g2, uint8_t* s2, uint32_t h2) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                mbar_expect(&bars[wib], h1 + h2);
                bulk_load(s1, g1, h1, &bars[wib]);
                if (h2) bulk_load(s2, g2, h2, &bars[wib]);
            }
            bool ok = mbar_wait(&bars[wib], parity, d.wait_limit);
            parity ^= 1u;
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) atomicOr(d.status, ST_TIMEOUT);
                mbar_wait(&bars[wib], parity ^ 1u, kDefaultWaitLimit);
                timed_out = true;
                return false;
            }
            return true;
        };
        if (mesh_pair) {
            // SAT_PolyMesh and friends for each primitive of the convex body
            // (one for a body of one primitive), each behind its own AABB
            const bool flip = ka == SHAPE_MESH;
            const int c = flip ? b : a;
            const uint8_t* gm = flip ? ga : gb;
            const HullHeader* Hm = reinterpret_cast<const HullHeader*>(gm);
            const float4* nodes = reinterpret_cast<const float4*>(gm + kMeshOffNodes);
            const float4* tris = nodes + 2 * (size_t)Hm->pad[1];
            const int nc = prim_n(d, c);
            for (int k = 0; k < nc && !timed_out; k++) {
                const uint8_t* gc = prim_blob(d, c, k);
                const uint32_t kc = reinterpret_cast<const HullHeader*>(gc)->kind;
                if (!stage(gc, slot, reinterpret_cast<const HullHeader*>(gc)->off_fofs, nullptr, nullptr, 0)) break;
                HullView hv;
                PrimView pv;
                if (kc == SHAPE_HULL) stage_hull(gc, slot, d.pos[c], d.rot[c], &hv, lane);
                else stage_prim(slot, d.pos[c], d.rot[c], &pv, lane);
                f3 blo, bhi;
                prim_box(d, c, k, &blo, &bhi);
                int ncand = 0;
                if (lane == 0) {
                    int stack[kMeshStack];
                    int sp = 0;
                    stack[sp++] = 0;
                    while (sp > 0) {
                        const int x = stack[--sp];
                        const float4 lo = __ldg(nodes + 2 * x), hi = __ldg(nodes + 2 * x + 1);
                        const int l = __float_as_int(lo.w), r = __float_as_int(hi.w);
                        if (l < 0) {
                            const float4* t = tris + (size_t)kMeshTriF4 * r;
                            if (box_overlap(mk(__ldg(t + 11)), mk(__ldg(t + 12)), blo, bhi)) {
                                if (ncand < kMeshCand) S.cand[ncand++] = r;
                                else { atomicOr(d.status, ST_MESH_OVERFLOW); break; }
                            }
                        } else if (box_overlap(mk(lo), mk(hi), blo, bhi)) {
                            if (sp + 2 > kMeshStack) { atomicOr(d.status, ST_MESH_OVERFLOW); break; }
                            stack[sp++] = l;
                            stack[sp++] = r;
                        }
                    }
                }
                ncand = __shfl_sync(0xffffffffu, ncand, 0);
                __syncwarp();
                const float pen_scale = kc == SHAPE_HULL ? 0.f : 0.15f;
                const float body_long = longest(blo, bhi);
                for (int ci = 0; ci < ncand; ci++) {
                    TriView T;
                    load_tri(tris + (size_t)kMeshTriF4 * S.cand[ci], &T);
                    const float penalty = pen_scale * fminf(body_long, longest(T.lo, T.hi));
                    PrimOut o;
                    o.m = 0;
                    bool hit;
                    if (kc == SHAPE_HULL) hit = polyTri(hv, T, penalty, lane, scratch, clipped, d.status, &o);
                    else if (kc == SHAPE_SPHERE) hit = sphereTri(pv, T, penalty, lane, &o);
                    else if (kc == SHAPE_CAPSULE) hit = capTri(pv, T, penalty, lane, scratch, clipped, d.status, &o);
                    else hit = cylTri(pv, T, penalty, lane, scratch, clipped, d.status, &o);
                    // a union primitive's index rides above the triangle id
                    if (lane == 0 && hit && o.pen > 0.f && o.m > 0) add_manifold(o, flip, T.id | (is_union(d, c) ? k << 24 : 0));
                }
                __syncwarp();
            }
        } else {
            // bodies of several primitives (PhysicsEngine.cpp:182-219): every
            // primitive pair whose AABBs overlap, in order (a's primitives
            // outer), each detector's manifold before the cull
            const int na = prim_n(d, a), nb2 = prim_n(d, b);
            for (int i = 0; i < na && !timed_out; i++)
                for (int j = 0; j < nb2 && !timed_out; j++) {
                    f3 alo, ahi, blo, bhi;
                    prim_box(d, a, i, &alo, &ahi);
                    prim_box(d, b, j, &blo, &bhi);
                    if (!box_overlap(alo, ahi, blo, bhi)) continue;
                    const uint8_t* pa = prim_blob(d, a, i);
                    const uint8_t* pb = prim_blob(d, b, j);
                    const HullHeader* Ha = reinterpret_cast<const HullHeader*>(pa);
                    const HullHeader* Hb = reinterpret_cast<const HullHeader*>(pb);
                    uint8_t* sa = slot;
                    uint8_t* sb = slot + ((Ha->off_fofs + 15u) & ~15u);
                    if (!stage(pa, sa, Ha->off_fofs, pb, sb, Hb->off_fofs)) break;
                    const int tri = (i << 8) | j;
                    if (Ha->kind == SHAPE_HULL && Hb->kind == SHAPE_HULL) {
                        HullView A, B;
                        stage_hull(pa, sa, d.pos[a], d.rot[a], &A, lane);
                        stage_hull(pb, sb, d.pos[b], d.rot[b], &B, lane);
                        __syncwarp();
                        Axis best;
                        const bool touch = sat_hulls(A, B, lane, &best);
                        if (touch && lane == 0) {
                            const HullG GA(pa, d.pos[a], d.rot[a]), GB(pb, d.pos[b], d.rot[b]);
                            PrimOut o;
                            o.n = best.n;
                            o.pen = best.pen;
                            o.m = clip_hulls(GA, GB, best.n, best.pen, make_int2(best.aid, best.bid), scratch, clipped, d.status,
                                             o.pts, o.magic);
                            if (o.pen > 0.f && o.m > 0) add_manifold(o, false, tri);
                        }
                    } else {
                        PrimOut o;
                        const bool hit = narrow_prim_out(d, a, b, sa, sb, pa, pb, Ha->kind, Hb->kind, lane, scratch, clipped, o);
                        if (lane == 0 && hit) add_manifold(o, false, tri);
                    }
                    __syncwarp();
                }
        }
        if (timed_out) {
            if (lane == 0) no_manifold(d, p);
            failed = true;
            continue;
        }
        if (lane == 0) {
            float maxpen;
            const int nout = mesh_merge(S, nman, &maxpen, d.status);
            int ofs = nout > 0 ? atomicAdd(d.mm_count, nout) : 0;
            if (nout > 0 && ofs + nout > d.cap_mesh_pts) { atomicOr(d.status, ST_MESH_OVERFLOW); ofs = -1; }
            if (nout == 0 || ofs < 0) {
                no_manifold(d, p);
            } else {
                for (int i = 0; i < nout; i++) {
                    const int r = S.out[i];
                    d.mm_pt[ofs + i] = S.pt[r];
                    d.mm_n[ofs + i] = S.out_n[i];
                    d.mm_magic[ofs + i] = S.magic[r];
                    d.mm_tri[ofs + i] = S.tri[r];
                }
                d.mf_ofs[p] = ofs;
                d.mf_cnt[p] = nout;
                d.mf_n[p] = make_float4(0.f, 0.f, 0.f, maxpen);
            }
        }
        __syncwarp();
    }
}

void prepare_kernels() {
    cudaFuncSetAttribute(k_narrowphase, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_narrow_prim, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_narrow_mesh, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

int mesh_scratch_warps(int n_sms) { return n_sms * kMeshBlocksPerSm * 8; }

// ---- ray queries ------------------------------------------------------------------
// PhysicsEngine::raycastFirstIntersection (PhysicsEngine.cpp:582-609) for one
// ray per thread against the bodies [s, e) of one world: every body whose
// current AABB the ray crosses is tested with its primitive's ray test, the
// nearest hit wins (strictly nearer replaces, in body order).
namespace {
struct RayHitD { bool hit; f3 p, n; float t; };

// AABB::rayIntersectsAABB (AABB.h:143-172)
__device__ bool rayAABB(f3 lo, f3 hi, f3 o, f3 d) {
    float t_min = -INFINITY, t_max = INFINITY;
    const float los[3] = {lo.x, lo.y, lo.z}, his[3] = {hi.x, hi.y, hi.z}, os[3] = {o.x, o.y, o.z}, ds[3] = {d.x, d.y, d.z};
    for (int i = 0; i < 3; i++) {
        if (fabsf(ds[i]) < 1e-11f) {
            if (os[i] < los[i] || os[i] > his[i]) return false;
        } else {
            float t0 = (los[i] - os[i]) / ds[i], t1 = (his[i] - os[i]) / ds[i];
            if (t0 > t1) { float x = t0; t0 = t1; t1 = x; }
            t_min = fmaxf(t0, t_min);
            t_max = fminf(t1, t_max);
            if (t_max < 0.f || t_max < t_min) return false;
        }
    }
    return true;
}

// smaller non-negative root of a t^2 + b t + c (ConvexPrimitive.cpp:134-150, 179-195)
__device__ bool rayRoot(float a, float b, float c, float* t) {
    const float radical = b * b - 4.f * a * c;
    if (radical < 0.f) return false;
    if (radical == 0.f) { *t = -0.5f * b / a; return *t >= 0.f; }
    const float sr = sqrtf(radical);
    const float t1 = (-b + sr) / (2.f * a), t2 = (-b - sr) / (2.f * a);
    if (t1 < 0.f && t2 < 0.f) return false;
    *t = t1 < 0.f ? t2 : t2 < 0.f ? t1 : fminf(t1, t2);
    return true;
}

// testRayAgainstSphere (ConvexPrimitive.cpp:170-202)
__device__ RayHitD raySphere(f3 o, f3 d, f3 c, float r) {
    f3 rel = o - c;
    float t;
    if (!rayRoot(mag2(d), 2.f * dot(rel, d), mag2(rel) - r * r, &t)) return RayHitD{false};
    f3 hp = o + t * d;
    return RayHitD{true, hp, normalize(hp - c), t};
}

// testRayAgainstCylinderSide (ConvexPrimitive.cpp:113-168)
__device__ RayHitD rayCylSide(f3 o, f3 d, f3 c, float r, float h, f3 ax) {
    f3 u = d - ax * dot(ax, d);
    f3 w = o - c - ax * (dot(ax, o) - dot(ax, c));
    float t;
    if (!rayRoot(mag2(u), 2.f * dot(u, w), mag2(w) - r * r, &t)) return RayHitD{false};
    f3 hp = o + t * d;
    const float x = dot(hp - c, ax);
    if (fabsf(x) > 0.5f * h) return RayHitD{false};
    return RayHitD{true, hp, normalize((hp - c) - ax * x), t};
}

// checkDiskIntersection (ConvexPrimitive.cpp:300-306)
__device__ RayHitD rayDisk(f3 o, f3 d, f3 c, f3 n, float r) {
    const float t = dot(n, c - o) / dot(n, d);
    f3 ip = o + t * d;
    if (t < 0.f || mag2(ip - c) > r * r) return RayHitD{false};
    return RayHitD{true, ip, n, t};
}

__device__ __forceinline__ void rayNearer(RayHitD* out, const RayHitD& h) {
    if (h.hit && (!out->hit || h.t < out->t)) *out = h;
}

// Polyhedron::testRayIntersection (ConvexPrimitive.cpp:731-758): the first face
// whose plane the ray enters from outside at a point inside the face
__device__ RayHitD rayHull(const uint8_t* blob, float4 pos, float4 rot, f3 o, f3 d) {
    HullG h(blob, pos, rot);
    const HullHeader& H = *h.h;
    const uint16_t* fofs = u16(blob, H.off_fofs);
    const uint8_t* fidx = blob + H.off_fidx;
    for (int f = 0; f < H.nf; f++) {
        const int k0 = fofs[f], k1 = fofs[f + 1];
        f3 sp = h.vert(fidx[k0]);
        f3 n = h.norm(f);
        if (dot(d, n) > -0.0001f || dot(o - sp, n) < 0.f) continue;
        const float t = dot(n, sp - o) / dot(n, d);
        f3 ip = o + t * d;
        bool inside = true;
        for (int k = k0; k < k1 && inside; k++) {
            f3 e1 = h.vert(fidx[k]), e2 = h.vert(fidx[k + 1 == k1 ? k0 : k + 1]);
            if (dot(cross(e2 - e1, n), ip - e1) > 0.f) inside = false;
        }
        if (inside) return RayHitD{true, ip, n, t};
    }
    return RayHitD{false};
}

// StaticMeshGeometry::testRayIntersection (Geometry.cpp:867-897)
__device__ RayHitD rayMesh(const uint8_t* blob, f3 o, f3 d) {
    const HullHeader* H = reinterpret_cast<const HullHeader*>(blob);
    const float4* nodes = reinterpret_cast<const float4*>(blob + kMeshOffNodes);
    const float4* tris = nodes + 2 * (size_t)H->pad[1];
    RayHitD best{false};
    for (uint32_t i = 0; i < H->pad[0]; i++) {
        TriView T;
        load_tri(tris + (size_t)kMeshTriF4 * i, &T);
        if (!rayAABB(T.lo, T.hi, o, d)) continue;
        if (fabsf(dot(T.n, d)) < 1e-10f) continue;
        const float t = -dot(o - T.v[1], T.n) / dot(d, T.n);
        if (t < 0.f || (best.hit && best.t < t)) continue;
        f3 hp = o + t * d;
        if (dot(hp - T.v[0], T.out[0]) > 0.f || dot(hp - T.v[1], T.out[1]) > 0.f || dot(hp - T.v[2], T.out[2]) > 0.f) continue;
        best = RayHitD{true, hp, T.n, t};
    }
    return best;
}

__global__ void k_raycast(Dev d, int s, int e, const float* rays, int n, const uint32_t* ignore, int n_ignore, float* out) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const f3 o = mk(rays[6 * k], rays[6 * k + 1], rays[6 * k + 2]);
        const f3 dir = mk(rays[6 * k + 3], rays[6 * k + 4], rays[6 * k + 5]);
        RayHitD best{false};
        int best_id = 0;
        for (int g = s; g < e; g++) {
            const uint32_t id = (uint32_t)(g - s + 1);
            bool skip = false;
            for (int q = 0; q < n_ignore; q++) skip |= ignore[q] == id;
            if (skip || !rayAABB(mk(d.aabb_lo[g]), mk(d.aabb_hi[g]), o, dir)) continue;
            // RigidBody::checkRayIntersection (RigidBody.cpp:185-200): each
            // primitive behind its own AABB (a body of one: behind the body's),
            // the nearest primitive hit
            RayHitD h{false};
            const int nprim = prim_n(d, g);
            for (int pk = 0; pk < nprim; pk++) {
                if (nprim > 1) {
                    f3 plo, phi;
                    prim_box(d, g, pk, &plo, &phi);
                    if (!rayAABB(plo, phi, o, dir)) continue;
                }
                const uint8_t* blob = prim_blob(d, g, pk);
                const uint32_t kind = reinterpret_cast<const HullHeader*>(blob)->kind;
                RayHitD hp{false};
                if (kind == SHAPE_MESH) {
                    hp = rayMesh(blob, o, dir);
                } else if (kind == SHAPE_HULL) {
                    hp = rayHull(blob, d.pos[g], d.rot[g], o, dir);
                } else {
                    const M33 R = quatRot(qnormalize(d.rot[g]));
                    const float4 cr = *reinterpret_cast<const float4*>(blob + sizeof(HullHeader));
                    const f3 c = mul(R, mk(cr)) + mk(d.pos[g]);
                    if (kind == SHAPE_SPHERE) {
                        hp = raySphere(o, dir, c, cr.w);
                    } else {
                        const float4 ax4 = *reinterpret_cast<const float4*>(blob + kCylOffAxis);
                        const f3 ax = mul(R, mk(ax4));
                        hp = rayCylSide(o, dir, c, cr.w, ax4.w, ax);
                        if (kind == SHAPE_CYLINDER) {   // Cylinder::testRayIntersection (ConvexPrimitive.cpp:308-318)
                            const float sgn = dot(ax, dir) < 0.f ? 1.f : -1.f;
                            rayNearer(&hp, rayDisk(o, dir, c + sgn * ax * (0.5f * ax4.w), ax, cr.w));
                        } else {                        // Capsule::testRayIntersection (:403-411)
                            rayNearer(&hp, raySphere(o, dir, c + ax * (0.5f * ax4.w), cr.w));
                            rayNearer(&hp, raySphere(o, dir, c - ax * (0.5f * ax4.w), cr.w));
                        }
                    }
                }
                if (hp.hit && (!h.hit || hp.t < h.t)) h = hp;
            }
            if (h.hit && (!best.hit || h.t < best.t)) { best = h; best_id = (int)id; }
        }
        float* r = out + 8 * (size_t)k;
        r[0] = __int_as_float(best_id);
        r[1] = best.hit ? best.p.x : 0.f; r[2] = best.hit ? best.p.y : 0.f; r[3] = best.hit ? best.p.z : 0.f;
        r[4] = best.hit ? best.n.x : 0.f; r[5] = best.hit ? best.n.y : 0.f; r[6] = best.hit ? best.n.z : 0.f;
        r[7] = best.hit ? best.t : -1.f;
    }
}
}  // namespace

void launch_raycast(const Dev& d, int s, int e, const float* rays, int n, const uint32_t* ignore, int n_ignore, float* out,
                    cudaStream_t st) {
    if (n <= 0) return;
    k_raycast<<<(n + 127) / 128, 128, 0, st>>>(d, s, e, rays, n, ignore, n_ignore, out);
}

void launch_narrowphase(const Dev& d, int slot_bytes, int n_sms, bool prims, cudaStream_t st) {
    const int warps = 8;
    size_t smem = 16 * warps + (size_t)warps * (slot_bytes + kQueueBytes);
    k_narrowphase<<<n_sms * 4, warps * 32, smem, st>>>(d, slot_bytes);
    k_clip<<<n_sms * 16, 128, 0, st>>>(d);
    if (prims) k_narrow_prim<<<n_sms * 4, warps * 32, 16 * warps + (size_t)warps * slot_bytes, st>>>(d, slot_bytes);
    if (d.has_mesh || d.has_union)
        k_narrow_mesh<<<n_sms * kMeshBlocksPerSm, warps * 32, 16 * warps + (size_t)warps * slot_bytes, st>>>(d, slot_bytes);
}

}  // namespace cpgpu
