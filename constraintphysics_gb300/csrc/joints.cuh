// joints.cuh — device helpers for joint rows (ball-socket, hinge, distance,
// weld, slider, sliding hinge, cone and twist limits, motors, pistons) and the holonomic block
// solve, shared by the row-building kernels (joints.cu) and
// the joint-island PGS kernel (solver.cu).
#pragma once
#include "devmath.cuh"
#include "layout.h"

namespace cpgpu {

constexpr float kJZero = 0.00000001f;   // NVec::isZero cutoff (Math/src/NVec.h:4)

__device__ __forceinline__ bool jzero(const float* x, int n) {
    for (int i = 0; i < n; i++)
        if (fabsf(x[i]) > kJZero) return false;
    return true;
}

// Δv slots of one island: kDvF4 float4 per island body, 12 floats v xyz,
// w xyz, pv xyz, pw xyz; `which` 0 = (v, w), 1 = (pv, pw)
__device__ __forceinline__ void jload(const float4* dv, int slot, int which, float* out) {
    if (slot < 0) { for (int k = 0; k < 6; k++) out[k] = 0.f; return; }
    const float* f = reinterpret_cast<const float*>(dv + kDvF4 * slot) + 6 * which;
    for (int k = 0; k < 6; k++) out[k] = f[k];
}
__device__ __forceinline__ void jadd(float4* dv, int slot, int which, const float* x) {
    if (slot < 0) return;
    float* f = reinterpret_cast<float*>(dv + kDvF4 * slot) + 6 * which;
    for (int k = 0; k < 6; k++) f[k] += x[k];
}

// J_a v_a + J_b v_b
__device__ __forceinline__ void jvalue(const JointRow& R, const float* va, const float* vb, float* out) {
    for (int i = 0; i < R.n; i++) {
        float x = 0.f, y = 0.f;
        for (int k = 0; k < 6; k++) x += va[k] * R.ja[6 * i + k];
        for (int k = 0; k < 6; k++) y += vb[k] * R.jb[6 * i + k];
        out[i] = x + y;
    }
}

// impulse_to_velocity * imp added to both bodies' slots (`which` 0 = velocity,
// 1 = pseudo velocity)
__device__ __forceinline__ void japply(const JointRow& R, const float* imp, float4* dv, int which) {
    float xa[6], xb[6];
    for (int k = 0; k < 6; k++) {
        float x = 0.f, y = 0.f;
        for (int i = 0; i < R.n; i++) { x += imp[i] * R.ita[kJMax * k + i]; y += imp[i] * R.itb[kJMax * k + i]; }
        xa[k] = x;
        xb[k] = y;
    }
    jadd(dv, R.sa, which, xa);
    jadd(dv, R.sb, which, xb);
}

// The same steps for a row of N dofs known at compile time (1: distance and
// limits, 3: ball-socket, 4: sliding hinge, 5: hinge and slider, 6: weld):
// every loop unrolls, so the row's entries are loaded once into registers
// instead of through loops over a run-time count (identical sums)
template <int N>
__device__ __forceinline__ void japply_n(const JointRow& R, const float* imp, float4* dv, int which) {
    float xa[6], xb[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        float x = 0.f, y = 0.f;
#pragma unroll
        for (int i = 0; i < N; i++) { x += imp[i] * R.ita[kJMax * k + i]; y += imp[i] * R.itb[kJMax * k + i]; }
        xa[k] = x;
        xb[k] = y;
    }
    jadd(dv, R.sa, which, xa);
    jadd(dv, R.sb, which, xb);
}

// PGSConstraintStep<n> (ConstraintSolver.cpp:12-40): the accumulated impulse
// plus the row's correction, projected (ConeLimitConstraint /
// TwistLimitConstraint::projectValidImpulse, ConstraintSolver.cpp:434-436,
// 463-465: one-sided limits), applied when the change is not zero
template <int N>
__device__ __forceinline__ void jstep_n(JointRow& R, float4* dv, bool pseudo) {
    const int which = pseudo ? 1 : 0;
    float va[6], vb[6], delta[N], diff[N], acc[N];
    jload(dv, R.sa, which, va);
    jload(dv, R.sb, which, vb);
    float* accp = pseudo ? R.pimpulse : R.impulse;
    const float* tgt = pseudo ? R.ptarget : R.target;
#pragma unroll
    for (int i = 0; i < N; i++) {
        float x = 0.f, y = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) x += va[k] * R.ja[6 * i + k];
#pragma unroll
        for (int k = 0; k < 6; k++) y += vb[k] * R.jb[6 * i + k];
        delta[i] = tgt[i] - (x + y);
        acc[i] = accp[i];
    }
    bool zero = true;
#pragma unroll
    for (int i = 0; i < N; i++) {
        float x = 0.f;
#pragma unroll
        for (int k = 0; k < N; k++) x += delta[k] * R.minv[kJMax * i + k];
        float nw = acc[i] + x;
        if (N == 1 && R.proj == 1) nw = fmaxf(nw, 0.f);
        else if (N == 1 && R.proj == 2) nw = fminf(nw, 0.f);
        // MotorConstraint / PistonConstraint::projectValidImpulse
        // (ConstraintSolver.cpp:591-606, 728-731)
        else if (N == 1 && R.proj == 3) nw = nw > 0.f ? fminf(nw, R.lim) : fmaxf(nw, -R.lim);
        diff[i] = nw - acc[i];
        zero = zero && !(fabsf(diff[i]) > kJZero);
    }
    if (!zero) {
        japply_n<N>(R, diff, dv, which);
#pragma unroll
        for (int i = 0; i < N; i++) accp[i] = acc[i] + diff[i];
    }
}

// warm start (DegreedConstraint::applyWarmStartVelocityChange)
__device__ __forceinline__ void jwarm(const JointRow& R, float4* dv) {
    if (jzero(R.impulse, R.n)) return;
    switch (R.n) {
        case 1: japply_n<1>(R, R.impulse, dv, 0); break;
        case 3: japply_n<3>(R, R.impulse, dv, 0); break;
        case 4: japply_n<4>(R, R.impulse, dv, 0); break;
        case 5: japply_n<5>(R, R.impulse, dv, 0); break;
        default: japply_n<6>(R, R.impulse, dv, 0); break;
    }
}

// one Gauss-Seidel step of a joint row
__device__ __forceinline__ void jstep(JointRow& R, float4* dv, bool pseudo) {
    switch (R.n) {
        case 1: jstep_n<1>(R, dv, pseudo); break;
        case 3: jstep_n<3>(R, dv, pseudo); break;
        case 4: jstep_n<4>(R, dv, pseudo); break;
        case 5: jstep_n<5>(R, dv, pseudo); break;
        default: jstep_n<6>(R, dv, pseudo); break;
    }
}

// ---- holonomic systems (HolonomicBlockSolver.cpp) ------------------------------
__device__ __forceinline__ int holo_loc(const int* table, int n, int row, int col) {
    return table[row - col + ((2 * n + 1) * col - col * col) / 2];
}

// multInverseWithVector (HolonomicBlockSolver.cpp:251-317): v <- L^-T D^-1 L^-1 v.
// `eff` holds `degree` scratch values.
template <class T>
__device__ void holo_solve(const HoloStore& hs, int s, const JointRow* rows, const T* B, T* v, T* eff) {
    const int c0 = hs.cstart[s], n = hs.cstart[s + 1] - c0;
    const int* cons = hs.cons + c0;
    const int* vp = hs.vpos + c0;
    const int* table = hs.table + hs.tstart[s];
    const int* ls = hs.lstart + hs.lbase[s];   // column col's blocks below the diagonal
    for (int col = 0; col + 1 < n; col++) {
        const int bw = rows[cons[col]].n;
        for (int q = ls[col]; q < ls[col + 1]; q++) {
            const int row = hs.lrow[q], l = hs.lloc[q];
            const int bh = rows[cons[row]].n;
            for (int i = 0; i < bh; i++) {
                T x = 0;
                for (int k = 0; k < bw; k++) x += B[l + i * bw + k] * v[vp[col] + k];
                eff[vp[row] + i] = x;
            }
        }
        // only rows below `col` were written this pass: subtract and clear them
        for (int q = ls[col]; q < ls[col + 1]; q++) {
            const int row = hs.lrow[q];
            for (int i = 0; i < rows[cons[row]].n; i++) { v[vp[row] + i] -= eff[vp[row] + i]; eff[vp[row] + i] = 0; }
        }
    }
    for (int col = 0; col < n; col++) {
        const int w = rows[cons[col]].n, l = holo_loc(table, n, col, col);
        T tmp[kJMax];
        for (int i = 0; i < w; i++) {
            T x = 0;
            for (int k = 0; k < w; k++) x += B[l + i * w + k] * v[vp[col] + k];
            tmp[i] = x;
        }
        for (int i = 0; i < w; i++) v[vp[col] + i] = tmp[i];
    }
    for (int col = n - 2; col >= 0; col--) {
        const int bw = rows[cons[col]].n;
        T e6[kJMax] = {};
        for (int q = ls[col]; q < ls[col + 1]; q++) {
            const int row = hs.lrow[q], l = hs.lloc[q];
            const int bh = rows[cons[row]].n;
            for (int i = 0; i < bw; i++) {
                T dp = 0;
                for (int j = 0; j < bh; j++) dp += v[vp[row] + j] * B[l + i + bw * j];
                e6[i] += dp;
            }
        }
        for (int i = 0; i < bw; i++) v[vp[col] + i] -= e6[i];
    }
}

}  // namespace cpgpu
