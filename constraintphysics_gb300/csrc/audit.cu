// audit.cu — per-step FP64 momentum and energy audit of every world.
//
// The reference has no such audit; the device path computes in FP32, and this
// kernel checks the result in FP64: after each step (when enabled) one block
// per world sums, over the world's dynamic bodies, the linear momentum
// sum(m v), the angular momentum about the origin sum(x × m v + I ω), the
// kinetic energy sum(m |v|² / 2 + ω·I ω / 2) and the gravitational potential
// energy -sum(m g·x), every product and sum in FP64 (the FP32 state promoted
// once).  It also keeps, per world, the largest increase of kinetic plus
// potential energy over one step since the audit was enabled: contacts without
// restitution, friction and the solver's damping only remove energy, so a
// positive jump shows where the position correction or a failing solve added
// some.  Masses and world inertia tensors are the ones the step used (inverse
// mass in pos.w, world tensor iw); fixed and kinematic bodies are left out.
#include "kernels.cuh"

namespace cpgpu {

namespace {

constexpr int kAuditThreads = 128;

__device__ __forceinline__ double warp_sum(double x) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}

__global__ void __launch_bounds__(kAuditThreads) k_audit(Dev d) {
    __shared__ double part[kAuditThreads / 32][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int w = blockIdx.x; w < d.n_worlds; w += gridDim.x) {
        const WorldParams& P = d.wparams[w];
        const double gx = P.gx, gy = P.gy, gz = P.gz;
        double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = d.world_start[w] + threadIdx.x; i < d.world_start[w + 1]; i += blockDim.x) {
            if (d.movement[i] != 0) continue;
            const float4 p = d.pos[i];
            if (p.w == 0.f) continue;
            const double m = 1.0 / (double)p.w;
            const float4 v4 = d.vel[i], w4 = d.angv[i];
            const double x[3] = {p.x, p.y, p.z}, v[3] = {v4.x, v4.y, v4.z}, om[3] = {w4.x, w4.y, w4.z};
            const float* I = d.iw + 9 * (size_t)i;
            double Iw[3];
            for (int r = 0; r < 3; r++) Iw[r] = (double)I[3 * r] * om[0] + (double)I[3 * r + 1] * om[1] + (double)I[3 * r + 2] * om[2];
            acc[0] += m * v[0];
            acc[1] += m * v[1];
            acc[2] += m * v[2];
            acc[3] += m * (x[1] * v[2] - x[2] * v[1]) + Iw[0];
            acc[4] += m * (x[2] * v[0] - x[0] * v[2]) + Iw[1];
            acc[5] += m * (x[0] * v[1] - x[1] * v[0]) + Iw[2];
            acc[6] += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) + 0.5 * (om[0] * Iw[0] + om[1] * Iw[1] + om[2] * Iw[2]);
            acc[7] -= m * (gx * x[0] + gy * x[1] + gz * x[2]);
        }
        for (int k = 0; k < 8; k++) {
            const double s = warp_sum(acc[k]);
            if (lane == 0) part[wid][k] = s;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot[8];
            for (int k = 0; k < 8; k++) {
                double s = 0;
                for (int q = 0; q < kAuditThreads / 32; q++) s += part[q][k];
                tot[k] = s;
            }
            double* o = d.audit + (size_t)kAuditValues * w;
            const double steps = o[9];
            if (steps > 0) {
                const double jump = (tot[6] + tot[7]) - (o[6] + o[7]);
                if (steps == 1 || jump > o[8]) o[8] = jump;
            }
            for (int k = 0; k < 8; k++) o[k] = tot[k];
            o[9] = steps + 1;
        }
        __syncthreads();
    }
}

}  // namespace

void launch_audit(const Dev& d, const Launch& L) {
    if (!d.audit) return;
    int g = d.n_worlds < L.n_sms * 16 ? d.n_worlds : L.n_sms * 16;
    k_audit<<<g < 1 ? 1 : g, kAuditThreads, 0, L.st>>>(d);
}

}  // namespace cpgpu
