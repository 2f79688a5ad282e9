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
                if (o < cap) { pairs[2 * o] = (uint32_t)i + 1; pairs[2 * o + 1] = (uint32_t)j + 1; }
                o++;
            }
        }
    }
}

// device address of the scratch array, looked up once per device with that
// device current (host code must not use the symbol itself as a pointer)
std::mutex g_na_mutex;
int* g_na_ptr[64] = {nullptr};

int scratch_for_current_device(int** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return CPGPU_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return CPGPU_ERR_CUDA;
        g_na_ptr[dev] = static_cast<int*>(p);
    }
    *out = g_na_ptr[dev];
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
