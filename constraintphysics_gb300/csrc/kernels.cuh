// kernels.cuh — launch wrappers of the contact-path kernels.  All kernels take
// the batch's device-pointer table (Dev) by value and read per-step sizes from
// device counters, so one step's launch sequence can be captured in a graph.
#pragma once
#include "layout.h"

namespace cpgpu {

struct Launch {
    int n_sms;
    cudaStream_t st;
};

// device-counted exclusive scan: out[i] = sum(in[0..i)), *total = sum(in[0..n))
// where n = *n_dev (or n_host when n_dev is null); tmp needs 2 + cap/1024 ints.
void scan_exclusive(const int* in, int* out, const int* n_dev, int n_host, int cap, int* total, int* tmp, const Launch& L);

void prepare_kernels();   // one-time function attributes (outside graph capture)
void set_last_error(const char* msg);   // message returned by cpgpu_last_error
void launch_gravity(const Dev& d, const Launch& L);
// the start of a step: gravity, or with sleeping enabled in the batch the
// waking actions, the sleep bookkeeping and gravity (sleep.cu)
void launch_step_begin(const Dev& d, const Launch& L);
void launch_pairs(const Dev& d, const Launch& L);
void launch_geometry(const Dev& d, int mode, const Launch& L);   // mode 0 moved bodies, 2 a batch's first pass
// hull-hull pairs, then (when the batch holds spheres or cylinders) the pairs
// that involve one
void launch_narrowphase(const Dev& d, int slot_bytes, int n_sms, bool prims, cudaStream_t st);
int mesh_scratch_warps(int n_sms);   // per-warp scratch entries the mesh narrowphase uses
// ray queries against the bodies [s, e): rays 6 floats each (origin, unit
// direction), `out` 8 floats per ray (body id bits, 0 = no hit; point;
// normal; distance, -1 = no hit)
void launch_raycast(const Dev& d, int s, int e, const float* rays, int n, const uint32_t* ignore, int n_ignore, float* out,
                    cudaStream_t st);
void launch_merge(const Dev& d, const Launch& L);
// largest k_pgs_big shared Δv area (island bodies) and k_islands shared
// memory any batch uses: the kernels' dynamic shared memory limits are set to
// these once for all batches
constexpr int kPgsDvCapMax = 1536;
// default size threshold between the thread-per-island and the warp-per-island
// solvers (rows of the island); the autotuner may choose another
constexpr int kDefaultBigRows = 48;
constexpr int kIslandsSmemMax = 160 * 1024;
// k_islands' dynamic shared memory for worlds of up to `max_bodies` bodies
// (sets the kernel's limit); worlds that need more run from global memory
int islands_smem_bytes(int max_bodies);
void launch_islands(const Dev& d, int smem_bytes, const Launch& L);
// per-world edge / contact ranges of the current graph (4 ints per world)
void launch_world_ranges(const Dev& d, const int* worlds, int n, int* out, cudaStream_t st);
void launch_rows(const Dev& d, int first, int last, const Launch& L);
// PGS: islands are split by size after the island pass (largest first); large
// islands run one warp each with rows streamed through shared memory, small
// ones one thread each on the `side` stream, concurrently.
void launch_pgs_schedule(const Dev& d, const Launch& L);
void prepare_pgs(int dv_cap);
int pgs_big_smem_bytes(int dv_cap);
int pgs_big_blocks_per_sm(int dv_cap);
void launch_pgs(const Dev& d, int dv_cap, int big_blocks, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, const Launch& L);
void launch_integrate(const Dev& d, int last, const Launch& L);
// joints: rows every substep, the holonomic systems' factorisation on the
// first; islands with joint rows solved by their own kernel
void launch_joint_rows(const Dev& d, bool first, const Launch& L);
// springs: impulse pairs at the start of every substep (no-op without springs)
void launch_springs(const Dev& d, const Launch& L);
void launch_pgs_joint(const Dev& d, bool first, const Launch& L);
// external state write: apply the staged state (d.stage); bodies whose pose
// changed get their world inertia tensors and AABBs recomputed
void launch_apply_state(const Dev& d, const Launch& L);
// host-layout rows (pos, rot, vel, ang vel: 4 float4 per body) of a split batch
void launch_gather_state(const Dev& d, const float4* all, const int* rows, const Launch& L);   // all -> d.stage
void launch_scatter_state(const Dev& d, const int* rows, float4* all, const Launch& L);       // d -> all
// FP64 momentum / energy audit of every world (no-op when d.audit is null)
void launch_audit(const Dev& d, const Launch& L);

}  // namespace cpgpu
