// noalloc.cu — candidate-pair generation for callers that cannot allocate
// device memory.
//
// Some callers of this library may not call cudaMalloc at the point where
// they need the broadphase: code running inside another framework's memory
// pool or allocator (which owns all device memory and forbids side
// allocations), real-time loops that must not hit the driver's allocator, or
// plugins that are handed pre-allocated input/output buffers and nothing
// else.  cpgpu_pairs_noalloc serves them: the caller passes the AABBs and the
// output buffers (device memory it already owns) and the call allocates
// nothing.  Its only scratch (per-body overlap counts and the scan's chunk
// sums) is a file-scope __device__ array of fixed size, so the maximum body
// count per call is kNoAllocMaxBodies.
//
// Same result as the batch path's pair generation (broadphase.cu): every pair
// (i, j), i < j, whose AABBs overlap under the inclusive test, in (i, j)
// order, ids 1-based.
#include <cstdio>
#include <mutex>
#include <vector>

#include "kernels.cuh"

extern "C" {
#include "../../include/cpgpu.h"
}

namespace cpgpu {

constexpr int kNoAllocMaxBodies = 1 << 16;
constexpr int kNoAllocChunk = 1024;
constexpr int kNoAllocChunks = kNoAllocMaxBodies / kNoAllocChunk;

// Scratch of every call on a device: per-body overlap counts (turned into
// output offsets in place) followed by the chunk sums.  Every GPU that loads
// the library holds it (about 260 KB) until the process exits.
static __device__ __align__(256) int g_noalloc_scratch[kNoAllocMaxBodies + kNoAllocChunks + 32];

namespace {

__device__ __forceinline__ bool overlap6(const float* a, const float* b) {
    return !(a[3] < b[0] || a[0] > b[3] || a[4] < b[1] || a[1] > b[4] || a[5] < b[2] || a[2] > b[5]);
}

__global__ void k_na_count(const float* aabbs, int n, int* scratch) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* a = aabbs + 6 * i;
        int c = 0;
        for (int j = i + 1; j < n; j++) c += overlap6(a, aabbs + 6 * j);
        scratch[i] = c;
    }
}

// exclusive scan of scratch[0..n) in place, one chunk of 1024 per block; the
// chunk totals go to scratch[kNoAllocMaxBodies + chunk]
__global__ void k_na_scan_chunks(int n, int* scratch) {
    __shared__ int ws[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int i = blockIdx.x * kNoAllocChunk + threadIdx.x;
    int v = (i < n) ? scratch[i] : 0, x = v;
    for (int o = 1; o < 32; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += t; }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int y = ws[lane];
        for (int o = 1; o < 32; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, y, o); if (lane >= o) y += t; }
        ws[lane] = y;
    }
    __syncthreads();
    int incl = x + (wid > 0 ? ws[wid - 1] : 0);
    if (i < n) scratch[i] = incl - v;
    if (threadIdx.x == kNoAllocChunk - 1) scratch[kNoAllocMaxBodies + blockIdx.x] = incl;
}

// chunk offsets (one thread, at most 64 chunks) and the total pair count
__global__ void k_na_scan_top(int n_chunks, int* scratch, int* count) {
    int run = 0;
    for (int c = 0; c < n_chunks; c++) {
        int t = scratch[kNoAllocMaxBodies + c];
        scratch[kNoAllocMaxBodies + c] = run;
        run += t;
    }
    *count = run;
}

__global__ void k_na_write(const float* aabbs, int n, const int* scratch, uint32_t* pairs, int cap) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* a = aabbs + 6 * i;
        int o = scratch[i] + scratch[kNoAllocMaxBodies + i / kNoAllocChunk];
        for (int j = i + 1; j < n; j++) {
            if (overlap6(a, aabbs + 6 * j)) {
                if (o < cap) { pairs[2 * (size_t)o] = (uint32_t)i + 1; pairs[2 * (size_t)o + 1] = (uint32_t)j + 1; }
                o++;
            }
        }
    }
}

// Device address of the scratch array, looked up with the device current
// (host code must not use the symbol itself as a pointer).  The address is
// cached per CUDA context, identified by the driver's context id, so that a
// caller who resets the device (a new primary context, the module loaded
// again) gets the new address instead of a stale one.  If the driver entry
// points for the context id are unavailable, the address is looked up again
// on every call.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
struct NaCache { unsigned long long ctx_id; int* ptr; };
std::mutex g_na_mutex;
std::vector<NaCache> g_na_cache;
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
bool g_ctx_fns_looked_up = false;

bool current_context_id(unsigned long long* id) {
    if (!g_ctx_fns_looked_up) {
        g_ctx_fns_looked_up = true;
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess && f1 && f2) {
            g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
    }
    if (!g_ctx_current || !g_ctx_id) return false;
    void* ctx = nullptr;
    if (g_ctx_current(&ctx) != 0 || !ctx) return false;
    return g_ctx_id(ctx, id) == 0;
}

int scratch_for_current_device(int** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CPGPU_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    unsigned long long id = 0;
    if (current_context_id(&id))
        for (const NaCache& c : g_na_cache)
            if (c.ctx_id == id) { *out = c.ptr; return CPGPU_OK; }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return CPGPU_ERR_CUDA;
    // the lookup made the device's primary context current if it was not
    if (current_context_id(&id)) g_na_cache.push_back({id, static_cast<int*>(p)});
    *out = static_cast<int*>(p);
    return CPGPU_OK;
}

}  // namespace
}  // namespace cpgpu

extern "C" int cpgpu_pairs_noalloc(const float* aabbs, int n_bodies, uint32_t* pairs, int cap, int* count, void* stream) {
    using namespace cpgpu;
    if (n_bodies < 0 || cap < 0 || !count || (n_bodies > 0 && !aabbs) || (cap > 0 && !pairs)) {
        set_last_error("cpgpu_pairs_noalloc: null buffer or negative size");
        return CPGPU_ERR_INVALID_ARG;
    }
    if (n_bodies > kNoAllocMaxBodies) {
        set_last_error("cpgpu_pairs_noalloc: more than 65536 bodies (the fixed scratch holds one count per body)");
        return CPGPU_ERR_INVALID_ARG;
    }
    // an error left by earlier work on this thread is not ours to report or
    // to clear: refuse to run and leave it pending for its owner
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        char msg[256];
        std::snprintf(msg, sizeof msg, "cpgpu_pairs_noalloc: an earlier CUDA error is pending (%s); nothing launched",
                      cudaGetErrorName(pending));
        set_last_error(msg);
        return CPGPU_ERR_CUDA;
    }
    int* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != CPGPU_OK) {
        set_last_error("cpgpu_pairs_noalloc: no usable CUDA device or scratch symbol lookup failed");
        return rc;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int n_chunks = (n_bodies + kNoAllocChunk - 1) / kNoAllocChunk;
    const int grid = n_bodies > 0 ? (n_bodies + 127) / 128 : 1;
    if (n_bodies > 0) {
        k_na_count<<<grid, 128, 0, st>>>(aabbs, n_bodies, scratch);
        k_na_scan_chunks<<<n_chunks, kNoAllocChunk, 0, st>>>(n_bodies, scratch);
    }
    k_na_scan_top<<<1, 1, 0, st>>>(n_chunks, scratch, count);
    if (n_bodies > 0) k_na_write<<<grid, 128, 0, st>>>(aabbs, n_bodies, scratch, pairs, cap);
    if (cudaGetLastError() != cudaSuccess) {
        set_last_error("cpgpu_pairs_noalloc: kernel launch failed");
        return CPGPU_ERR_CUDA;
    }
    return CPGPU_OK;
}
