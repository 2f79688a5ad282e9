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
constexpr long long kSpinLimit = 1LL << 24;  // bounded mbarrier wait

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

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (long long it = 0; it < kSpinLimit; it++) {
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
__device__ void contactArea(const HullView& h, f3 n, int pid, f3 u, f3 w, Area* a) {
    const HullHeader& H = *h.h;
    const uint16_t* vfofs = u16(h.g, H.off_vfofs);
    const uint8_t* vfidx = h.g + H.off_vfidx;
    int best_f = -1;
    float best_ft = 1.0f;
    for (int k = vfofs[pid]; k < vfofs[pid + 1]; k++) {
        int f = vfidx[k];
        float ca = dot(mk(h.n[f]), n);
        if (1.f - ca < best_ft) { best_ft = 1.f - ca; best_f = f; }
    }
    if (best_ft <= kCosTol) {
        const uint16_t* fofs = u16(h.g, H.off_fofs);
        const uint8_t* fidx = h.g + H.off_fidx;
        a->n = 0;
        for (int k = fofs[best_f]; k < fofs[best_f + 1] && a->n < kMaxClip; k++) {
            int id = fidx[k];
            f3 v = mk(h.v[id]);
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
        f3 d = mk(h.v[edges[2 * e + 1]]) - mk(h.v[edges[2 * e]]);
        float sa = fabsf(dot(normalize(d), n));
        if (sa < best_et) { best_et = sa; best_e = e; }
    }
    if (best_et <= kSinTol) {
        int p1 = edges[2 * best_e], p2 = edges[2 * best_e + 1];
        f3 e1 = mk(h.v[p1]), e2 = mk(h.v[p2]);
        a->ps[0] = P2{dot(e1, u), dot(e1, w)};
        a->ps[1] = P2{dot(e2, u), dot(e2, w)};
        a->ids[0] = p1; a->ids[1] = p2;
        a->n = 2;
        a->surface = -1;
        return;
    }
    f3 p = mk(h.v[pid]);
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
    Scratch scratch;
    CP clipped[kMaxClip];
    const int n_pairs = *d.n_pairs;
    for (int p = blockIdx.x * warps_per_block + wib; p < n_pairs; p += gridDim.x * warps_per_block) {
        const int a = d.pair_a[p], b = d.pair_b[p];
        // collision filter of PhysicsEngine.cpp:174 (at least one dynamic body)
        if (!(d.movement[a] == 0 || d.movement[b] == 0)) {
            if (lane == 0) { d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f); d.mf_cnt[p] = 0; }
            continue;
        }
        const uint8_t* ga = d.shapes + d.shape[a];
        const uint8_t* gb = d.shapes + d.shape[b];
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
        bool ok = mbar_wait(&bars[wib], parity);
        parity ^= 1u;
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) { atomicOr(d.status, ST_TIMEOUT); d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f); d.mf_cnt[p] = 0; }
            // give the copies in flight one more bounded wait, then stop using the slot
            mbar_wait(&bars[wib], parity ^ 1u);
            return;
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
        if (lane == 0) {
            f3 n = mk(nx, ny, nz);
            if (!(bp < INFINITY) || aid < 0 || bid < 0) {
                d.mf_n[p] = make_float4(0.f, 0.f, 0.f, -1.f);
                d.mf_cnt[p] = 0;
            } else {
                f3 u, w;
                basis(n, &u, &w);
                Area ac, bc;
                contactArea(A, n, aid, u, w, &ac);
                contactArea(B, -1.f * n, bid, u, w, &bc);
                int m = clipContacts(ac, bc, scratch, clipped, d.status);
                f3 amax = mk(A.v[aid]);
                float a_dot = dot(amax, n);
                f3 off = n * a_dot;
                float4 pts[kMaxClip];
                for (int i = 0; i < m; i++) {
                    f3 q = u * clipped[i].p.x + w * clipped[i].p.y + off;
                    pts[i] = make_float4(q.x, q.y, q.z, dot(q, n) - a_dot + bp);
                }
                // cull_manifold to 4 points (CollisionDetect.cpp:2795-2830)
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
                float maxpen = bp;
                for (int i = 0; i < out_n; i++) {
                    d.mf_pt[4 * p + i] = pts[pick[i]];
                    d.mf_magic[4 * p + i] = clipped[pick[i]].magic;
                }
                d.mf_n[p] = make_float4(n.x, n.y, n.z, maxpen);
                d.mf_cnt[p] = out_n;
            }
        }
    }
}

void prepare_kernels() {
    cudaFuncSetAttribute(k_narrowphase, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

void launch_narrowphase(const Dev& d, int slot_bytes, int n_sms, cudaStream_t st) {
    const int warps = 8;
    size_t smem = 16 * warps + (size_t)warps * (slot_bytes + kQueueBytes);
    k_narrowphase<<<n_sms * 4, warps * 32, smem, st>>>(d, slot_bytes);
}

}  // namespace cpgpu
