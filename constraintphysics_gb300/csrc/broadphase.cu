// broadphase.cu — gravity, candidate pairs, geometry/AABB update and the
// device-counted exclusive scan used by the graph kernels.
//
// Pair generation returns exactly the set the reference's AABB tree returns:
// every pair of bodies of the same world whose true AABBs overlap under the
// inclusive test of AABB::intersects (ConstraintPhysics/src/AABB.h:10-14; the
// tree query AABB_Tree.h:153-224 visits every overlapping leaf pair once).
// Pairs are emitted as (lower id, higher id) sorted by (a, b): one thread per
// body counts its overlaps with the later bodies of its world, an exclusive
// scan gives each body its output offset, and a second pass writes.  Worlds
// above kTileWorld bodies (where one thread per body would loop over up to
// the whole world) run the same test over kTile x kTile blocks instead.
#include <algorithm>

#include "kernels.cuh"
#include "devmath.cuh"
#include "shapes.cuh"

namespace cpgpu {

namespace {
constexpr int kScanBlock = 1024;

__device__ __forceinline__ bool overlap(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    return !(ahi.x < blo.x || alo.x > bhi.x || ahi.y < blo.y || alo.y > bhi.y || ahi.z < blo.z || alo.z > bhi.z);
}

// inclusive block scan of one value per thread (blockDim.x == kScanBlock)
__device__ int block_scan_incl(int v, int* warp_sums) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int s = (lane < (blockDim.x >> 5)) ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    if (wid > 0) v += warp_sums[wid - 1];
    __syncthreads();
    return v;
}

__global__ void k_scan_chunks(const int* in, int* out, const int* n_dev, int n_host, int* chunk_sums) {
    __shared__ int ws[32];
    const int n = n_dev ? *n_dev : n_host;
    const int nchunks = (n + kScanBlock - 1) / kScanBlock;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        int i = c * kScanBlock + threadIdx.x;
        int v = (i < n) ? in[i] : 0;
        int inc = block_scan_incl(v, ws);
        if (i < n) out[i] = inc - v;
        if (threadIdx.x == kScanBlock - 1) chunk_sums[c] = inc;
    }
}

__global__ void k_scan_top(int* chunk_sums, const int* n_dev, int n_host, int* total) {
    __shared__ int ws[32];
    __shared__ int carry;
    const int n = n_dev ? *n_dev : n_host;
    const int nchunks = (n + kScanBlock - 1) / kScanBlock;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nchunks; base += kScanBlock) {
        int i = base + threadIdx.x;
        int v = (i < nchunks) ? chunk_sums[i] : 0;
        int inc = block_scan_incl(v, ws);
        int c0 = carry;
        if (i < nchunks) chunk_sums[i] = c0 + inc - v;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry = c0 + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int* out, const int* n_dev, int n_host, const int* chunk_sums) {
    const int n = n_dev ? *n_dev : n_host;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] += chunk_sums[i / kScanBlock];
}

__global__ void k_gravity(Dev d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n_bodies; i += gridDim.x * blockDim.x) {
        if (d.movement[i] != 0) continue;
        const WorldParams& p = d.wparams[d.world[i]];
        float4 v = d.vel[i];
        // vel += gravity * step_time (PhysicsEngine.cpp:85)
        v.x += p.gx * p.dt; v.y += p.gy * p.dt; v.z += p.gz * p.dt;
        d.vel[i] = v;
    }
}

__global__ void k_pairs(Dev d, int write) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n_bodies; i += gridDim.x * blockDim.x) {
        if (d.n_tile_tasks > 0 && d.tile_base[d.world[i]] >= 0) continue;   // a large world: k_pairs_tile
        const int end = d.world_start[d.world[i] + 1];
        const float4 lo = d.aabb_lo[i], hi = d.aabb_hi[i];
        if (!write) {
            int c = 0;
            for (int j = i + 1; j < end; j++) c += overlap(lo, hi, d.aabb_lo[j], d.aabb_hi[j]);
            d.pair_count[i] = c;
        } else {
            int o = d.pair_count[i];
            for (int j = i + 1; j < end; j++) {
                if (overlap(lo, hi, d.aabb_lo[j], d.aabb_hi[j])) {
                    if (o < d.cap_pairs) { d.pair_a[o] = i; d.pair_b[o] = j; }
                    o++;
                }
            }
        }
    }
}

// Large worlds: a block per (i tile, j tile >= i tile) of the world's bodies;
// the j tile's AABBs are staged in shared memory and each thread tests its
// body i against them (j > i).  The count pass stores, per body and j tile,
// the pairs found there; k_pairs_tile_rows turns a body's cells into their
// prefix and its total; the write pass writes each body's pairs of a tile at
// its offset plus the tile's prefix, in increasing j -- the same sorted
// (a, b) list as the per-body loop, with every thread doing kTile tests.
__global__ void __launch_bounds__(kTile) k_pairs_tile(Dev d, int write) {
    __shared__ float4 slo[kTile], shi[kTile];
    for (int q = blockIdx.x; q < d.n_tile_tasks; q += gridDim.x) {
        const int4 t = d.tile_task[q];
        const int s = d.world_start[t.x], e = d.world_start[t.x + 1];
        const int j0 = s + t.z * kTile, jn = min(kTile, e - j0);
        __syncthreads();   // the previous task's tile is no longer read
        if ((int)threadIdx.x < jn) {
            slo[threadIdx.x] = d.aabb_lo[j0 + threadIdx.x];
            shi[threadIdx.x] = d.aabb_hi[j0 + threadIdx.x];
        }
        __syncthreads();
        const int i = s + t.y * kTile + (int)threadIdx.x;
        if (i >= e) continue;
        const float4 lo = d.aabb_lo[i], hi = d.aabb_hi[i];
        int* cell = d.tile_cnt + d.tile_base[t.x] + (size_t)(i - s) * t.w + t.z;
        const int first = max(0, i + 1 - j0);   // j > i
        if (!write) {
            int c = 0;
            for (int k = first; k < jn; k++) c += overlap(lo, hi, slo[k], shi[k]);
            *cell = c;
        } else {
            int o = d.pair_count[i] + *cell;
            for (int k = first; k < jn; k++) {
                if (overlap(lo, hi, slo[k], shi[k])) {
                    if (o < d.cap_pairs) { d.pair_a[o] = i; d.pair_b[o] = j0 + k; }
                    o++;
                }
            }
        }
    }
}

// per large-world body: the prefix of its j-tile cells (from its own tile on)
// and its pair count
__global__ void k_pairs_tile_rows(Dev d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n_bodies; i += gridDim.x * blockDim.x) {
        const int w = d.world[i], base = d.tile_base[w];
        if (base < 0) continue;
        const int s = d.world_start[w], e = d.world_start[w + 1];
        const int T = (e - s + kTile - 1) / kTile;
        int* row = d.tile_cnt + base + (size_t)(i - s) * T;
        int acc = 0;
        for (int jt = (i - s) / kTile; jt < T; jt++) {
            const int c = row[jt];
            row[jt] = acc;
            acc += c;
        }
        d.pair_count[i] = acc;
    }
}

__global__ void k_clamp_pairs(Dev d) {
    if (*d.n_pairs > d.cap_pairs) { atomicOr(d.status, ST_PAIR_OVERFLOW); *d.n_pairs = d.cap_pairs; }
    if (d.has_mesh || d.has_union) *d.mm_count = 0;   // mesh store of this step's narrowphase
}

// RigidBody::updateGeometry (RigidBody.cpp:281-312) for moved bodies: the
// orientation is renormalised and the AABB recomputed from the world geometry
// (gen_AABB of the body's primitive).  `mode` 2 (a batch's first pass): every
// body's AABB, the orientations flagged in `moved` (poses set through the
// API) renormalised.
__global__ void k_geometry(Dev d, int mode) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n_bodies; i += gridDim.x * blockDim.x) {
        if (mode == 0 && (d.movement[i] == 1 || !d.moved[i])) continue;
        float4 q = d.rot[i];
        if (mode != 2 || d.moved[i]) {
            q = qnormalize(q);
            d.rot[i] = q;
        }
        M33 R = quatRot(q);
        f3 c = mk(d.pos[i]);
        f3 mn, mx;
        if (d.has_union && d.prim_start[i] >= 0) {
            // each primitive's AABB, the body's their combination in order
            // (ConvexUnionGeometry, RigidBody.cpp:286-294; AABB::combine)
            const int q0 = d.prim_start[i], nq = d.prim_count[i];
            for (int q = q0; q < q0 + nq; q++) {
                f3 pl, ph;
                shape_aabb(d.shapes + d.prim_shape[q], c, R, &pl, &ph);
                d.prim_lo[q] = make_float4(pl.x, pl.y, pl.z, 0.f);
                d.prim_hi[q] = make_float4(ph.x, ph.y, ph.z, 0.f);
                if (q == q0) { mn = pl; mx = ph; }
                else {
                    mn = mk(fminf(mn.x, pl.x), fminf(mn.y, pl.y), fminf(mn.z, pl.z));
                    mx = mk(fmaxf(mx.x, ph.x), fmaxf(mx.y, ph.y), fmaxf(mx.z, ph.z));
                }
            }
        } else {
            shape_aabb(d.shapes + d.shape[i], c, R, &mn, &mx);
        }
        d.aabb_lo[i] = make_float4(mn.x, mn.y, mn.z, 0.f);
        d.aabb_hi[i] = make_float4(mx.x, mx.y, mx.z, 0.f);
    }
}
}  // namespace

void scan_exclusive(const int* in, int* out, const int* n_dev, int n_host, int cap, int* total, int* tmp, const Launch& L) {
    int max_chunks = (cap + kScanBlock - 1) / kScanBlock;
    int g = max_chunks < L.n_sms * 2 ? (max_chunks > 0 ? max_chunks : 1) : L.n_sms * 2;
    k_scan_chunks<<<g, kScanBlock, 0, L.st>>>(in, out, n_dev, n_host, tmp);
    k_scan_top<<<1, kScanBlock, 0, L.st>>>(tmp, n_dev, n_host, total);
    k_scan_add<<<L.n_sms * 4, 256, 0, L.st>>>(out, n_dev, n_host, tmp);
}

static int grid_for(int n, int per_block, int n_sms) {
    int g = (n + per_block - 1) / per_block;
    int cap = n_sms * 8;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

void launch_gravity(const Dev& d, const Launch& L) {
    k_gravity<<<grid_for(d.n_bodies, 256, L.n_sms), 256, 0, L.st>>>(d);
}

void launch_pairs(const Dev& d, const Launch& L) {
    int g = grid_for(d.n_bodies, 128, L.n_sms);
    const int gt = std::min(d.n_tile_tasks, L.n_sms * 16);
    k_pairs<<<g, 128, 0, L.st>>>(d, 0);
    if (d.n_tile_tasks > 0) {
        k_pairs_tile<<<gt, kTile, 0, L.st>>>(d, 0);
        k_pairs_tile_rows<<<g, 128, 0, L.st>>>(d);
    }
    scan_exclusive(d.pair_count, d.pair_count, nullptr, d.n_bodies, d.n_bodies, d.n_pairs, d.scan_tmp, L);
    k_pairs<<<g, 128, 0, L.st>>>(d, 1);
    if (d.n_tile_tasks > 0) k_pairs_tile<<<gt, kTile, 0, L.st>>>(d, 1);
    k_clamp_pairs<<<1, 1, 0, L.st>>>(d);
}

void launch_geometry(const Dev& d, int mode, const Launch& L) {
    k_geometry<<<grid_for(d.n_bodies, 128, L.n_sms), 128, 0, L.st>>>(d, mode);
}

}  // namespace cpgpu
