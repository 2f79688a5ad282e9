// joints.cu — joint rows (ball-socket, hinge) and the factorisation of the
// holonomic systems on the device.
//
// Rows (BallSocket / Hinge ::updateSolverConstraints, PersistentConstraint.cpp:
// 225-231, 274-285; BallSocketConstraint / HingeConstraint constructors,
// ConstraintSolver.cpp:382-405, 468-550): one thread per joint rebuilds its
// Jacobians, impulse-to-velocity maps, effective-mass inverse and targets
// from the current poses every substep, warm-started from the joint's
// persistent impulse.
//
// Holonomic systems (HolonomicSystem::computeInverse, HolonomicBlockSolver.cpp:
// 427-543): one thread per system forms the blocks of A = J M^-1 J^T (with
// CFM on the diagonal) in the host-chosen elimination order and factorises
// A = L D L^T block by block, the diagonal blocks inverted in place.  Systems
// whose link-mass ratio exceeds 100 factorise in FP64, the others in FP32.
// The reference computes the factorisation at the end of a step for the next
// step's first substep; the rows it uses are the ones the first substep
// rebuilds from the same poses, so factorising there gives the same matrix.
#include "kernels.cuh"
#include "joints.cuh"

namespace cpgpu {

namespace {

__device__ __forceinline__ f3 qrot(float4 q, f3 v) {  // Quaternion::applyRotation
    float r = q.x, i = q.y, j = q.z, k = q.w;
    return mk(v.x * (r * r + i * i - j * j - k * k) + v.y * (2 * i * j - 2 * r * k) + v.z * (2 * i * k + 2 * r * j),
              v.x * (2 * i * j + 2 * r * k) + v.y * (r * r - i * i + j * j - k * k) + v.z * (2 * j * k - 2 * r * i),
              v.x * (2 * i * k - 2 * r * j) + v.y * (2 * j * k + 2 * r * i) + v.z * (r * r - i * i - j * j + k * k));
}

// rows 0-2 of a ball-socket or hinge Jacobian: [I | -[rA]x] and [-I | [rB]x]
__device__ __forceinline__ void point_rows(float* ja, float* jb, f3 rA, f3 rB) {
    const float ra[3][3] = {{0.f, -rA.z, rA.y}, {rA.z, 0.f, -rA.x}, {-rA.y, rA.x, 0.f}};
    const float rb[3][3] = {{0.f, -rB.z, rB.y}, {rB.z, 0.f, -rB.x}, {-rB.y, rB.x, 0.f}};
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) {
            ja[6 * i + k] = (i == k) ? 1.f : 0.f;
            ja[6 * i + 3 + k] = -ra[i][k];
            jb[6 * i + k] = (i == k) ? -1.f : 0.f;
            jb[6 * i + 3 + k] = rb[i][k];
        }
}

// rowMajorOrderInverse<n> (NMat.cpp:5-34, NMat.h:124-149)
template <class T>
__device__ void invert_block(int n, T* m) {
    T out[kJMax * kJMax];
    if (n == 1) {
        out[0] = T(1) / m[0];
    } else if (n == 2) {
        T di = T(1) / (m[0] * m[3] - m[1] * m[2]);
        out[0] = m[3] * di; out[1] = -m[1] * di; out[2] = -m[2] * di; out[3] = m[0] * di;
    } else if (n == 3) {
        T a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
        T di = T(1) / (a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g));
        out[0] = (e * i - f * h) * di; out[1] = (c * h - b * i) * di; out[2] = (b * f - c * e) * di;
        out[3] = (f * g - d * i) * di; out[4] = (a * i - c * g) * di; out[5] = (c * d - a * f) * di;
        out[6] = (d * h - e * g) * di; out[7] = (b * g - a * h) * di; out[8] = (a * e - b * d) * di;
    } else {
        T c[kJMax * kJMax];
        for (int k = 0; k < n * n; k++) { c[k] = m[k]; out[k] = 0; }
        for (int k = 0; k < n; k++) out[k * (n + 1)] = 1;
        // one reciprocal per pivot (FP64 division is a long instruction
        // sequence; the ratios and the final scaling multiply by it)
        for (int piv = 0; piv < n; piv++) {
            const T rp = T(1) / c[n * piv + piv];
            for (int r = 0; r < n; r++) {
                if (r == piv) continue;
                T ratio = c[n * r + piv] * rp;
                for (int k = 0; k < n; k++) {
                    c[n * r + k] -= ratio * c[n * piv + k];
                    out[n * r + k] -= ratio * out[n * piv + k];
                }
            }
        }
        for (int piv = 0; piv < n; piv++) {
            const T rp = T(1) / c[n * piv + piv];
            for (int k = 0; k < n; k++) out[n * piv + k] *= rp;
        }
    }
    for (int k = 0; k < n * n; k++) m[k] = out[k];
}

__global__ void k_joint_rows(Dev d) {
    const JointStore& J = d.jt;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < d.n_joints; j += gridDim.x * blockDim.x) {
        const int a = J.b1[j], b = J.b2[j], n = J.n[j];
        if (d.movement[a] != 0 && d.movement[b] != 0) continue;
        const WorldParams& P = d.wparams[d.world[a]];
        const float dts = P.dt_sub;
        const float4 qa = d.rot[a], qb = d.rot[b];
        const f3 ca = mk(d.pos[a]), cb = mk(d.pos[b]);
        const f3 pa = qrot(qa, mk(J.p1[j])) + ca, pb = qrot(qb, mk(J.p2[j])) + cb;
        const float2 hard = J.hard[j];
        const float pos_c = fminf(hard.x * dts, 1.0f / dts);
        JointRow& R = d.jt.rows[j];
        R.n = n;
        float warm[kJMax];
        for (int i = 0; i < n; i++) warm[i] = P.warm_disabled ? 0.f : J.impulse[kJMax * j + i];
        for (int i = 0; i < n; i++) { R.impulse[i] = warm[i]; R.pimpulse[i] = 0.f; R.holo[i] = 0.f; }
        const f3 rA = pa - ca;
        if (n == 3) {
            point_rows(R.ja, R.jb, rA, pb - cb);
            const f3 e = pb - pa;
            R.ptarget[0] = pos_c * e.x; R.ptarget[1] = pos_c * e.y; R.ptarget[2] = pos_c * e.z;
        } else {
            // the reference's hinge takes rB from body 1's anchor point
            point_rows(R.ja, R.jb, rA, pa - cb);
            const f3 h1 = qrot(qa, mk(J.ax1[j])), nn = qrot(qb, mk(J.ax2[j]));
            const float rot_c = fminf(hard.y * dts, 1.0f / dts);
            f3 uu, ww;
            basis(h1, &uu, &ww);
            const f3 su = mk(J.u[j]), sw = mk(J.w[j]);
            R.impulse[3] = dot(uu, su) * warm[3] + dot(uu, sw) * warm[4];
            R.impulse[4] = dot(ww, su) * warm[3] + dot(ww, sw) * warm[4];
            // n^T [u]x, u^T [n]x, n^T [w]x, w^T [n]x
            const f3 a3 = cross(nn, uu), b3 = cross(uu, nn), a4 = cross(nn, ww), b4 = cross(ww, nn);
            const float ar[2][3] = {{a3.x, a3.y, a3.z}, {a4.x, a4.y, a4.z}};
            const float br[2][3] = {{b3.x, b3.y, b3.z}, {b4.x, b4.y, b4.z}};
            for (int i = 0; i < 2; i++)
                for (int k = 0; k < 3; k++) {
                    R.ja[6 * (3 + i) + k] = 0.f;
                    R.jb[6 * (3 + i) + k] = 0.f;
                    R.ja[6 * (3 + i) + 3 + k] = ar[i][k];
                    R.jb[6 * (3 + i) + 3 + k] = br[i][k];
                }
            const f3 pc = (pb - pa) * pos_c;
            R.ptarget[0] = pc.x; R.ptarget[1] = pc.y; R.ptarget[2] = pc.z;
            R.ptarget[3] = dot(uu, nn) * rot_c;
            R.ptarget[4] = dot(ww, nn) * rot_c;
            d.jt.u[j] = make_float4(uu.x, uu.y, uu.z, 0.f);
            d.jt.w[j] = make_float4(ww.x, ww.y, ww.z, 0.f);
        }
        // impulse_to_{a,b}_velocity = M^-1 J^T, impulse_to_value, CFM inverse
        const float ima = d.pos[a].w, imb = d.pos[b].w;
        const M33 Ia = load9(d.iinv + 9 * a), Ib = load9(d.iinv + 9 * b);
        for (int i = 0; i < n; i++) {
            for (int k = 0; k < 3; k++) {
                R.ita[kJMax * k + i] = ima * R.ja[6 * i + k];
                R.itb[kJMax * k + i] = imb * R.jb[6 * i + k];
            }
            const f3 ta = mul(Ia, mk(R.ja[6 * i + 3], R.ja[6 * i + 4], R.ja[6 * i + 5]));
            const f3 tb = mul(Ib, mk(R.jb[6 * i + 3], R.jb[6 * i + 4], R.jb[6 * i + 5]));
            R.ita[kJMax * 3 + i] = ta.x; R.ita[kJMax * 4 + i] = ta.y; R.ita[kJMax * 5 + i] = ta.z;
            R.itb[kJMax * 3 + i] = tb.x; R.itb[kJMax * 4 + i] = tb.y; R.itb[kJMax * 5 + i] = tb.z;
        }
        float m[kJMax * kJMax];
        for (int i = 0; i < n; i++)
            for (int c = 0; c < n; c++) {
                float x = 0.f, y = 0.f;
                for (int k = 0; k < 6; k++) { x += R.ja[6 * i + k] * R.ita[kJMax * k + c]; y += R.jb[6 * i + k] * R.itb[kJMax * k + c]; }
                R.itv[kJMax * i + c] = x + y;
                m[n * i + c] = x + y;
            }
        for (int i = 0; i < n; i++) m[n * i + i] *= (1.0f + P.cfm);
        invert_block<float>(n, m);
        for (int i = 0; i < n; i++)
            for (int c = 0; c < n; c++) R.minv[kJMax * i + c] = m[n * i + c];
        // target from the bodies' velocities at the start of the solve
        float va[6] = {0, 0, 0, 0, 0, 0}, vb[6] = {0, 0, 0, 0, 0, 0}, cur[kJMax];
        if (d.movement[a] != 1) {
            float4 v = d.vel[a], w = d.angv[a];
            va[0] = v.x; va[1] = v.y; va[2] = v.z; va[3] = w.x; va[4] = w.y; va[5] = w.z;
        }
        if (d.movement[b] != 1) {
            float4 v = d.vel[b], w = d.angv[b];
            vb[0] = v.x; vb[1] = v.y; vb[2] = v.z; vb[3] = w.x; vb[4] = w.y; vb[5] = w.z;
        }
        jvalue(R, va, vb, cur);
        for (int i = 0; i < n; i++) R.target[i] = -cur[i];
    }
}

// computeBlockInitialValue (HolonomicBlockSolver.cpp:731-760)
template <class T>
__device__ void initial_block(const Dev& d, int j1, int j2, T* t, float cfm) {
    const JointRow& c1 = d.jt.rows[j1];
    const JointRow& c2 = d.jt.rows[j2];
    if (j1 == j2) {
        const int n = c1.n;
        for (int i = 0; i < n; i++)
            for (int k = 0; k < n; k++) t[i * n + k] = (T)c1.itv[kJMax * i + k];
        for (int i = 0; i < n; i++) t[i * n + i] *= (T)(1.0f + cfm);
        return;
    }
    const int a1 = d.jt.b1[j1], b1 = d.jt.b2[j1], a2 = d.jt.b1[j2], b2 = d.jt.b2[j2];
    const float* jac = nullptr;
    const float* it = nullptr;
    if (a1 == a2) { jac = c1.ja; it = c2.ita; }
    else if (a1 == b2) { jac = c1.ja; it = c2.itb; }
    else if (b1 == a2) { jac = c1.jb; it = c2.ita; }
    else if (b1 == b2) { jac = c1.jb; it = c2.itb; }
    for (int i = 0; i < c1.n * c2.n; i++) {
        const int r = i / c2.n, c = i % c2.n;
        T x = 0;
        if (jac)
            for (int k = 0; k < 6; k++) x += (T)jac[6 * r + k] * (T)it[kJMax * k + c];
        t[i] = x;
    }
}

// One warp per system: the column loop stays in order (each column needs the
// previous columns' updates); within a column the diagonal block is inverted
// by lane 0 and the entries of the L blocks and of the trailing updates are
// spread over the lanes, each entry summed in the same order as a serial
// loop would.
template <class T>
__device__ void factorise(const Dev& d, int s, T* B, float cfm, int lane) {
    const HoloStore& hs = d.hs;
    const int c0 = hs.cstart[s], n = hs.cstart[s + 1] - c0;
    const int* cons = hs.cons + c0;
    const int* table = hs.table + hs.tstart[s];
    const int* ls = hs.lstart + hs.lbase[s];   // column col's blocks below the diagonal: [ls[col], ls[col + 1])
    T* Dg = B + hs.cap[s];
    for (int col = lane; col < n; col += 32) {
        initial_block<T>(d, cons[col], cons[col], B + holo_loc(table, n, col, col), cfm);
        for (int q = ls[col]; q < ls[col + 1]; q++) initial_block<T>(d, cons[hs.lrow[q]], cons[col], B + hs.lloc[q], cfm);
    }
    __syncwarp();
    for (int col = 0; col < n; col++) {
        const int w = d.jt.rows[cons[col]].n;
        T* diag = B + holo_loc(table, n, col, col);
        if (lane == 0) invert_block<T>(w, diag);
        __syncwarp();
        if (col + 1 == n) break;
        const int q0 = ls[col], q1 = ls[col + 1];
        const int fb = q0 < q1 ? hs.lloc[q0] : -1;
        for (int q = q0; q < q1; q++) {
            const int row = hs.lrow[q], l = hs.lloc[q];
            const int h = d.jt.rows[cons[row]].n;
            T* tgt = Dg + (l - fb);
            for (int e = lane; e < h * w; e += 32) {
                const int r = e / w, c = e - r * w;
                T x = 0;
                for (int k = 0; k < w; k++) x += B[l + w * r + k] * diag[w * c + k];
                tgt[c + w * r] = x;
            }
        }
        __syncwarp();
        for (int qa = q0; qa < q1; qa++) {
            const int lc = hs.lrow[qa], llc = hs.lloc[qa];
            const int bw = d.jt.rows[cons[lc]].n;
            for (int qb = qa; qb < q1; qb++) {
                const int lr = hs.lrow[qb], l = hs.lloc[qb];
                const int bh = d.jt.rows[cons[lr]].n;
                T* tgt = B + holo_loc(table, n, lr, lc);
                const T* lsrc = Dg + (llc - fb);
                for (int e = lane; e < bh * bw; e += 32) {
                    const int r = e / bw, c = e - r * bw;
                    T x = 0;
                    for (int k = 0; k < w; k++) x += B[l + r * w + k] * lsrc[c * w + k];
                    tgt[r * bw + c] -= x;
                }
            }
        }
        __syncwarp();
        if (fb >= 0) {
            const int total = holo_loc(table, n, col + 1, col + 1) - fb;
            for (int k = lane; k < total; k += 32) B[fb + k] = Dg[k];
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(32) k_holo_factor(Dev d) {
    const int lane = threadIdx.x;
    for (int s = blockIdx.x; s < d.hs.n; s += gridDim.x) {
        const int j0 = d.hs.cons[d.hs.cstart[s]];
        const float cfm = d.wparams[d.world[d.jt.b1[j0]]].cfm;
        if (d.hs.fp64[s]) factorise<double>(d, s, d.hs.pool64 + d.hs.bstart[s], cfm, lane);
        else factorise<float>(d, s, d.hs.pool32 + d.hs.bstart[s], cfm, lane);
    }
}

}  // namespace

void launch_joint_rows(const Dev& d, bool first, const Launch& L) {
    if (d.n_joints == 0) return;
    int g = (d.n_joints + 127) / 128;
    g = g > L.n_sms * 8 ? L.n_sms * 8 : g;
    k_joint_rows<<<g, 128, 0, L.st>>>(d);
    if (first && d.hs.n > 0) {
        // a warp per system
        int gs = d.hs.n;
        gs = gs > L.n_sms * 32 ? L.n_sms * 32 : gs;
        k_holo_factor<<<gs, 32, 0, L.st>>>(d);
    }
}

}  // namespace cpgpu
