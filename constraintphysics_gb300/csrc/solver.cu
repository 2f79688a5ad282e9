// solver.cu — per-substep row rebuild, projected Gauss-Seidel and integration.
//
// Rows (Contact::updateSolverConstraints, PersistentConstraint.cpp:201-215;
// ContactConstraint / FrictionConstraint constructors, ConstraintSolver.cpp:
// 240-343): one thread per live contact rebuilds its normal row and 2-dof
// friction row from the current poses and writes them, with the warm-start
// impulses (the friction impulse re-projected onto the new tangent basis), to
// the contact's slot in island order.  The same pass advances the contact's
// lifetime (PhysicsEngine.cpp:1378-1399) and marks expired contacts.
//
// PGS (PGS_solve, ConstraintSolver.cpp:80-213): one thread per island walks
// its rows in the reference's order: targets from the bodies' velocities,
// warm start, n_vel velocity sweeps of block Gauss-Seidel with the projection
// on the accumulated impulse, n_pos pseudo-velocity sweeps of the normal rows,
// then the velocity deltas are applied to the island's bodies.  A serial chain
// per island is the latency-optimal form of Gauss-Seidel (each row depends on
// the previous one); throughput comes from running thousands of islands at
// once.
//
// Integration (PhysicsEngine.cpp:390-419, RigidBody.cpp:207-279): one thread
// per body.
#include "kernels.cuh"
#include "devmath.cuh"
#include "shapes.cuh"
#include "joints.cuh"

namespace cpgpu {

namespace {

constexpr float kZero = 0.00000001f;  // NVec::isZero cutoff (Math/src/NVec.h:4)

__device__ __forceinline__ f3 qrotate(float4 q, f3 v) {  // Quaternion::applyRotation
    float r = q.x, i = q.y, j = q.z, k = q.w;
    return mk(v.x * (r * r + i * i - j * j - k * k) + v.y * (2 * i * j - 2 * r * k) + v.z * (2 * i * k + 2 * r * j),
              v.x * (2 * i * j + 2 * r * k) + v.y * (r * r - i * i + j * j - k * k) + v.z * (2 * j * k - 2 * r * i),
              v.x * (2 * i * k - 2 * r * j) + v.y * (2 * j * k + 2 * r * i) + v.z * (r * r - i * i - j * j + k * k));
}

// J angular part n^T [r]x (ConstraintSolver.cpp:247-252)
__device__ __forceinline__ f3 nskew(f3 n, f3 r) {
    return mk(n.y * r.z - n.z * r.y, n.z * r.x - n.x * r.z, n.x * r.y - n.y * r.x);
}

__device__ __forceinline__ void it_of(float im, const M33& I, const float* j, float* out) {
    out[0] = im * j[0]; out[1] = im * j[1]; out[2] = im * j[2];
    f3 a = mul(I, mk(j[3], j[4], j[5]));
    out[3] = a.x; out[4] = a.y; out[5] = a.z;
}

__device__ __forceinline__ float dot6(const float* a, const float* b) {
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 6; k++) s += a[k] * b[k];
    return s;
}

__device__ __forceinline__ void body_vel(const Dev& d, int g, float* out) {
    if (d.movement[g] == 1) { for (int k = 0; k < 6; k++) out[k] = 0.f; return; }
    float4 v = d.vel[g], w = d.angv[g];
    out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = w.x; out[4] = w.y; out[5] = w.z;
}

__global__ void k_rows(Dev d, int first, int last) {
    const int nc = *d.n_contacts_new;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        int st = d.c_new.state[c];
        const bool live = cs_live(st);
        const int r = live ? d.row_of_contact[c] : -1;
        if (live && r >= 0) {
            const uint64_t key = d.e_new.key[d.c_new.edge[c]];
            const int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
            const WorldParams& P = d.wparams[d.world[a]];
            const float dt = P.dt_sub;
            const float4 qa = d.rot[a], qb = d.rot[b];
            const f3 ca = mk(d.pos[a]), cb = mk(d.pos[b]);
            const float ima = d.pos[a].w, imb = d.pos[b].w;
            const M33 Ia = load9(d.iinv + 9 * a), Ib = load9(d.iinv + 9 * b);
            const float4 p1 = d.c_new.p1[c], p2 = d.c_new.p2[c], nl = d.c_new.n[c], imp = d.c_new.imp[c];
            const f3 pa = qrotate(qa, mk(p1)) + ca;
            const f3 pb = qrotate(qb, mk(p2)) + cb;
            const f3 n = qrotate(qa, mk(nl));
            const float depth = dot(pb - pa, n) + p1.w;
            const float wn = P.warm_disabled ? 0.f : imp.x;
            const float wf0 = P.warm_disabled ? 0.f : imp.y, wf1 = P.warm_disabled ? 0.f : imp.z;
            const float pcc = fminf(P.hardness * dt, 1.0f / dt);
            const f3 rA = pa - ca, rB = pa - cb;
            // the row is assembled in registers and written with 16-byte stores
            // (a thread per contact writing 384 scattered bytes field by field
            // would issue 96 partial-sector stores)
            RowBlock R;
            R.sa = (d.movement[a] == 0) ? d.visited[a] : -1;
            R.sb = (d.movement[b] == 0) ? d.visited[b] : -1;
            R.contact = c;
            R.ga = a; R.gb = b;
            R.bounce = p2.w;
            R.cutoff = P.cutoff_vel;
            R.fcoeff = nl.w;
            R.stat = 0;
            // normal row
            float ja[6], jb[6], ia[6], ib[6];
            f3 t = nskew(n, rA), t2 = nskew(-n, rB);
            ja[0] = -n.x; ja[1] = -n.y; ja[2] = -n.z; ja[3] = t.x; ja[4] = t.y; ja[5] = t.z;
            jb[0] = n.x; jb[1] = n.y; jb[2] = n.z; jb[3] = t2.x; jb[4] = t2.y; jb[5] = t2.z;
            it_of(ima, Ia, ja, ia);
            it_of(imb, Ib, jb, ib);
            float itv = dot6(ja, ia) + dot6(jb, ib);
            for (int k = 0; k < 6; k++) { R.nja[k] = ja[k]; R.njb[k] = jb[k]; R.nita[k] = ia[k]; R.nitb[k] = ib[k]; }
            R.nminv = 1.0f / (itv * (1.0f + P.cfm));
            R.nptarget = fmaxf(0.0f, depth - 0.05f) * pcc;
            // friction rows in the tangent basis of n, warm impulse re-projected
            f3 u, w;
            basis(n, &u, &w);
            const f3 su = mk(d.c_new.fu[c]), sw = mk(d.c_new.fw[c]);
            R.imp = make_float4(wn, 0.f, dot(u, su) * wf0 + dot(u, sw) * wf1, dot(w, su) * wf0 + dot(w, sw) * wf1);
            float fja[12], fjb[12], fia[12], fib[12];
            f3 ta = nskew(-u, rA), tb = nskew(u, rB), wa = nskew(-w, rA), wb = nskew(w, rB);
            fja[0] = u.x; fja[1] = u.y; fja[2] = u.z; fja[3] = ta.x; fja[4] = ta.y; fja[5] = ta.z;
            fja[6] = w.x; fja[7] = w.y; fja[8] = w.z; fja[9] = wa.x; fja[10] = wa.y; fja[11] = wa.z;
            fjb[0] = -u.x; fjb[1] = -u.y; fjb[2] = -u.z; fjb[3] = tb.x; fjb[4] = tb.y; fjb[5] = tb.z;
            fjb[6] = -w.x; fjb[7] = -w.y; fjb[8] = -w.z; fjb[9] = wb.x; fjb[10] = wb.y; fjb[11] = wb.z;
            float tmp[6];
            for (int row = 0; row < 2; row++) {
                it_of(ima, Ia, fja + 6 * row, tmp);
                for (int k = 0; k < 6; k++) fia[2 * k + row] = tmp[k];
                it_of(imb, Ib, fjb + 6 * row, tmp);
                for (int k = 0; k < 6; k++) fib[2 * k + row] = tmp[k];
            }
            float fv[4];
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++) {
                    float sa = 0.f, sb = 0.f;
                    for (int k = 0; k < 6; k++) { sa += fja[6 * i + k] * fia[2 * k + j]; sb += fjb[6 * i + k] * fib[2 * k + j]; }
                    fv[2 * i + j] = sa + sb;
                }
            fv[0] *= (1.0f + P.cfm);
            fv[3] *= (1.0f + P.cfm);
            float di = 1.0f / (fv[0] * fv[3] - fv[1] * fv[2]);
            const float m00 = fv[3] * di, m01 = -fv[1] * di, m10 = -fv[2] * di, m11 = fv[0] * di;
            R.fmc[0] = m00; R.fmc[1] = m10; R.fmc[2] = m01; R.fmc[3] = m11;
            // the friction values' change per unit normal impulse (J_f M^-1 J_n^T),
            // mapped through Fm^-1 to the friction impulses' change
            const float kf0 = dot6(fja, ia) + dot6(fjb, ib);
            const float kf1 = dot6(fja + 6, ia) + dot6(fjb + 6, ib);
            R.kd0 = m00 * kf0 + m01 * kf1;
            R.kd1 = m10 * kf0 + m11 * kf1;
            for (int k = 0; k < 6; k++) {
                R.fja0[k] = fja[k]; R.fjb0[k] = fjb[k]; R.fja1[k] = fja[6 + k]; R.fjb1[k] = fjb[6 + k];
                R.fita0[k] = fia[2 * k]; R.fitb0[k] = fib[2 * k]; R.fita1[k] = fia[2 * k + 1]; R.fitb1[k] = fib[2 * k + 1];
            }
            // velocity targets from the bodies' velocities at the start of the
            // solve (ContactConstraint::findTargetConstraintValue,
            // ConstraintSolver.cpp:264-268; DegreedConstraint default, ConstraintSolver.h:78)
            {
                float va[6], vb[6];
                body_vel(d, a, va);
                body_vel(d, b, vb);
                float cur = dot6(ja, va) + dot6(jb, vb);
                R.tgt_n = (cur < -P.cutoff_vel) ? -(1.0f + p2.w) * cur : -cur;
                R.tgt_f0 = -(dot6(fja, va) + dot6(fjb, vb));
                R.tgt_f1 = -(dot6(fja + 6, va) + dot6(fjb + 6, vb));
            }
            {
                float4* dst = reinterpret_cast<float4*>(d.rows + r);
                const float4* src = reinterpret_cast<const float4*>(&R);
#pragma unroll
                for (int k = 0; k < (int)(sizeof(RowBlock) / 16); k++) dst[k] = src[k];
            }
            d.c_new.fu[c] = make_float4(u.x, u.y, u.z, 0.f);
            d.c_new.fw[c] = make_float4(w.x, w.y, w.z, 0.f);
        }
        // lifetime (PhysicsEngine.cpp:1378-1399, expiry :1434-1446)
        int life = cs_life(st);
        bool lv = live;
        if (last) { life = life > -127 ? life - 1 : life; lv = false; }   // the 8-bit store saturates
        bool dead = cs_dead(st) || (first && life < 0);
        if (dead && !cs_dead(st) && d.has_sleep) {
            // Contact::isExpired (PersistentConstraint.h:74): a contact of a
            // sleeping body does not expire
            const uint64_t key = d.e_new.key[d.c_new.edge[c]];
            if (d.asleep[(int)(key >> 32)] || d.asleep[(int)(key & 0xffffffffu)]) dead = false;
        }
        // a rebuilt FrictionConstraint starts with static_ready = false
        d.c_new.state[c] = cs_make(life, lv, live ? false : cs_static(st), dead);
    }
}

// ---- packed FP32 pairs: a row's 6-vectors and a body's Δv are handled as
// the three component pairs (x, y), (z, ax), (ay, az), two lanes of one
// fma.rn.f32x2 each (half the instructions of scalar FP32 on the chain).
// Every operation of the rows is written with an explicit round-to-nearest
// intrinsic: the row functions are inlined into several kernels (warp per
// island, thread per island, joint islands), and left to the compiler, a
// sum of two products could be contracted into a different FMA in each;
// spelled out, every kernel computes the same bits, so the island-size
// threshold between the kernels never changes a result.
struct P3 { float2 a, b, c; };
__device__ __forceinline__ P3 p3(const float* f) {
    return P3{make_float2(f[0], f[1]), make_float2(f[2], f[3]), make_float2(f[4], f[5])};
}
__device__ __forceinline__ float2 bc2(float x) { return make_float2(x, x); }
// x - y, rounded once (y times -1 is exact)
__device__ __forceinline__ float2 psub(float2 x, float2 y) { return __ffma2_rn(y, make_float2(-1.f, -1.f), x); }
// J_a v_a + J_b v_b
__device__ __forceinline__ float pdot(const P3& ja, const P3& va, const P3& jb, const P3& vb) {
    float2 s = __fmul2_rn(ja.a, va.a);
    s = __ffma2_rn(ja.b, va.b, s);
    s = __ffma2_rn(ja.c, va.c, s);
    float2 t = __fmul2_rn(jb.a, vb.a);
    t = __ffma2_rn(jb.b, vb.b, t);
    t = __ffma2_rn(jb.c, vb.c, t);
    const float2 u = __fadd2_rn(s, t);
    return __fadd_rn(u.x, u.y);
}
// v += x * s
__device__ __forceinline__ void paxpy(P3& v, const P3& x, float2 s) {
    v.a = __ffma2_rn(x.a, s, v.a);
    v.b = __ffma2_rn(x.b, s, v.b);
    v.c = __ffma2_rn(x.c, s, v.c);
}

// Δv of island body `slot`: which 0 = (v, w), 1 = (pv, pw); slot < 0 is a
// body of infinite mass (always zero)
__device__ __forceinline__ P3 dv_get(const float4* dv, int slot, int which) {
    if (slot < 0) return P3{make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    const float4* s = dv + kDvF4 * slot;
    if (which == 0) {
        const float4 A = s[0];
        const float2 B = reinterpret_cast<const float2*>(s + 1)[0];
        return P3{make_float2(A.x, A.y), make_float2(A.z, A.w), B};
    }
    const float2 A = reinterpret_cast<const float2*>(s + 1)[1];
    const float4 C = s[2];
    return P3{A, make_float2(C.x, C.y), make_float2(C.z, C.w)};
}
__device__ __forceinline__ void dv_put(float4* dv, int slot, int which, const P3& v) {
    if (slot < 0) return;
    float4* s = dv + kDvF4 * slot;
    if (which == 0) {
        s[0] = make_float4(v.a.x, v.a.y, v.b.x, v.b.y);
        reinterpret_cast<float2*>(s + 1)[0] = v.c;
    } else {
        reinterpret_cast<float2*>(s + 1)[1] = v.a;
        s[2] = make_float4(v.b.x, v.b.y, v.c.x, v.c.y);
    }
}

// ---- one row of each PGS pass (PGS_solve, ConstraintSolver.cpp:120-161) ----------
// warm start: apply the stored impulses when they are non-zero
// (DegreedConstraint::constraintWarmStarted / applyWarmStartVelocityChange)
__device__ __forceinline__ void row_warm(const RowBlock& R, const float4 imp, float4* dv) {
    const bool wn = fabsf(imp.x) > kZero, wf = fabsf(imp.z) > kZero || fabsf(imp.w) > kZero;
    if (!wn && !wf) return;
    P3 va = dv_get(dv, R.sa, 0), vb = dv_get(dv, R.sb, 0);
    if (wn) {
        paxpy(va, p3(R.nita), bc2(imp.x));
        paxpy(vb, p3(R.nitb), bc2(imp.x));
    }
    if (wf) {
        paxpy(va, p3(R.fita0), bc2(imp.z));
        paxpy(va, p3(R.fita1), bc2(imp.w));
        paxpy(vb, p3(R.fitb0), bc2(imp.z));
        paxpy(vb, p3(R.fitb1), bc2(imp.w));
    }
    dv_put(dv, R.sa, 0, va);
    dv_put(dv, R.sb, 0, vb);
}

// velocity pass: normal row clamped at zero, then the friction rows projected on
// the friction disc of the current normal impulse (PGSConstraintStep,
// ConstraintSolver.cpp:12-40; projections :270-272, :331-343).  The friction
// rows see the velocities after the normal change; their new impulses are
// evaluated as (impulses + Fm^-1 (targets - values of the incoming
// velocities)) minus the normal change times the row's constants
// kd = Fm^-1 J_f M^-1 J_n^T (the same quantity, associated differently), so
// that everything but one FMA per friction row runs alongside the normal row
// instead of after it; the normal row's velocity change is applied while the
// friction rows are evaluated.  The disc projection compares squared
// magnitudes and scales by rsqrt.  `va`, `vb` are the two bodies' Δv.
__device__ __forceinline__ void row_vel_r(const RowBlock& R, float4& imp, int& stat, P3& va, P3& vb) {
    const float cur = pdot(p3(R.nja), va, p3(R.njb), vb);
    const float b0 = pdot(p3(R.fja0), va, p3(R.fjb0), vb), b1 = pdot(p3(R.fja1), va, p3(R.fjb1), vb);
    // friction impulses for the incoming velocities: imp.zw + Fm^-1 (tgt_f - b)
    const float2 g = psub(make_float2(R.tgt_f0, R.tgt_f1), make_float2(b0, b1));
    const float2 A = __fadd2_rn(make_float2(imp.z, imp.w),
                                __ffma2_rn(make_float2(R.fmc[2], R.fmc[3]), bc2(g.y),
                                           __fmul2_rn(make_float2(R.fmc[0], R.fmc[1]), bc2(g.x))));
    const float nw = __fmaf_rn(R.nminv, __fsub_rn(R.tgt_n, cur), imp.x);
    float diff = __fsub_rn(fmaxf(nw, 0.0f), imp.x);
    if (!(fabsf(diff) > kZero)) diff = 0.f;
    const float ix = __fadd_rn(imp.x, diff);
    const float2 sd = bc2(diff);
    paxpy(va, p3(R.nita), sd);
    paxpy(vb, p3(R.nitb), sd);
    float2 nf = __ffma2_rn(bc2(-diff), make_float2(R.kd0, R.kd1), A);
    const float mx = __fmul_rn(R.fcoeff, ix);
    const float s2 = __fmaf_rn(nf.x, nf.x, __fmul_rn(nf.y, nf.y));
    if (s2 > __fmul_rn(mx, mx)) { nf = __fmul2_rn(nf, bc2(__fmul_rn(mx, rsqrtf(s2)))); stat = 0; }
    else stat = 1;
    float2 e = psub(nf, make_float2(imp.z, imp.w));
    if (!(fabsf(e.x) > kZero || fabsf(e.y) > kZero)) e = make_float2(0.f, 0.f);
    const float2 s0 = bc2(e.x), s1 = bc2(e.y);
    paxpy(va, p3(R.fita0), s0);
    paxpy(vb, p3(R.fitb0), s0);
    paxpy(va, p3(R.fita1), s1);
    paxpy(vb, p3(R.fitb1), s1);
    imp.x = ix;
    imp.z = __fadd_rn(imp.z, e.x);
    imp.w = __fadd_rn(imp.w, e.y);
}
// the same on the island's Δv array (written back unconditionally: a zero
// change writes the same values)
__device__ __forceinline__ void row_vel(const RowBlock& R, float4& imp, int& stat, float4* dv) {
    P3 va = dv_get(dv, R.sa, 0), vb = dv_get(dv, R.sb, 0);
    row_vel_r(R, imp, stat, va, vb);
    dv_put(dv, R.sa, 0, va);
    dv_put(dv, R.sb, 0, vb);
}

// pseudo-velocity (position correction) pass of the normal row
__device__ __forceinline__ void row_pos(const RowBlock& R, float4& imp, float4* dv) {
    P3 va = dv_get(dv, R.sa, 1), vb = dv_get(dv, R.sb, 1);
    const float cur = pdot(p3(R.nja), va, p3(R.njb), vb);
    const float nw = __fmaf_rn(R.nminv, __fsub_rn(R.nptarget, cur), imp.y);
    const float diff = __fsub_rn(fmaxf(nw, 0.0f), imp.y);
    if (fabsf(diff) > kZero) {
        paxpy(va, p3(R.nita), bc2(diff));
        paxpy(vb, p3(R.nitb), bc2(diff));
        imp.y = __fadd_rn(imp.y, diff);
        dv_put(dv, R.sa, 1, va);
        dv_put(dv, R.sb, 1, vb);
    }
}

// island epilogue: impulses to the contacts (warm start of the next rebuild)
// and velocity deltas to the bodies (PhysicsEngine::applyVelocityChange,
// PhysicsEngine.cpp:1113-1136); `t`/`nt` stride over the island
__device__ void island_finish(const Dev& d, int rs, int rc, int bs, int bc, const float4* dv, int t, int nt) {
    for (int r = rs + t; r < rs + rc; r += nt) {
        const RowBlock& R = d.rows[r];
        if (R.contact < 0) continue;   // joint row (k_pgs_joint writes those back)
        float4 imp = R.imp;
        d.c_new.imp[R.contact] = make_float4(imp.x, imp.z, imp.w, 0.f);
        int cst = d.c_new.state[R.contact];
        d.c_new.state[R.contact] = R.stat ? (cst | (1 << 9)) : (cst & ~(1 << 9));
    }
    bool wake = false;
    for (int k = t; k < bc; k += nt) {
        int g = d.isl_bodies[bs + k];
        if (d.movement[g] != 0) continue;
        const float4 A = dv[kDvF4 * k], B = dv[kDvF4 * k + 1], C = dv[kDvF4 * k + 2];
        float4 v = d.vel[g], w = d.angv[g], pv = d.pvel[g], pw = d.pangv[g];
        v = make_float4(v.x + A.x, v.y + A.y, v.z + A.z, 0.f);
        w = make_float4(w.x + A.w, w.y + B.x, w.z + B.y, 0.f);
        d.vel[g] = v;
        d.angv[g] = w;
        d.pvel[g] = make_float4(pv.x + B.z, pv.y + B.w, pv.z + C.x, 0.f);
        d.pangv[g] = make_float4(pw.x + C.y, pw.y + C.z, pw.z + C.w, 0.f);
        if (d.has_sleep && d.asleep[g]) {
            const float wv = d.wparams[d.world[g]].wake_vel;
            wake = wake || mag(mk(v)) > wv || mag(mk(w)) > wv;
        }
    }
    if (!d.has_sleep) return;
    // sleeping bodies of a solved island (PhysicsEngine::applyVelocityChange,
    // PhysicsEngine.cpp:1113-1136): one pushed faster than a quarter of the
    // sleep velocity wakes the island (the island is the component
    // wakeupIsland walks); otherwise they keep zero velocity.  The reference
    // visits the bodies in an unordered_map's order, and a body zeroed before
    // the waking one stays at rest there; here a wake takes precedence.
    if (nt == 32) wake = __any_sync(0xffffffffu, wake);
    for (int k = t; k < bc; k += nt) {
        const int g = d.isl_bodies[bs + k];
        if (d.movement[g] != 0 || !d.asleep[g]) continue;
        if (wake) {
            d.asleep[g] = 0;
            d.ready_cnt[g] = 0;
            d.non_sleepy[g] = 0;
            d.hist_n[g] = 0;
            d.hist_head[g] = 0;
        } else {
            d.vel[g] = make_float4(0.f, 0.f, 0.f, 0.f);
            d.angv[g] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// ---- scheduling: islands with at least d.big_rows rows get a warp each,
// largest first; the smaller ones a thread each (the two paths give identical
// results, so the threshold is a pure schedule choice)

__global__ void k_sched_reset(Dev d) {
    if (threadIdx.x < 96) d.sched[threadIdx.x] = 0;
}

__device__ __forceinline__ int size_bucket(int rows) { return 31 - __clz(rows); }

__global__ void k_sched_count(Dev d) {
    const int ni = *d.n_islands;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x) {
        if (d.n_joint_edges > 0 && d.g_isl_flags[i]) { d.joint_list[atomicAdd(&d.sched[3], 1)] = i; continue; }
        int rc = d.g_isl_row_count[i];
        if (rc >= d.big_rows) atomicAdd(&d.sched[32 + size_bucket(rc)], 1);
        else d.small_list[atomicAdd(&d.sched[1], 1)] = i;
    }
}

__global__ void k_sched_place(Dev d) {
    const int ni = *d.n_islands;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x) {
        if (d.n_joint_edges > 0 && d.g_isl_flags[i]) continue;
        int rc = d.g_isl_row_count[i];
        if (rc < d.big_rows) continue;
        int b = size_bucket(rc), off = 0;
        for (int k = 31; k > b; k--) off += d.sched[32 + k];   // larger buckets first
        d.big_list[off + atomicAdd(&d.sched[64 + b], 1)] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int n = 0;
        for (int k = 0; k < 32; k++) n += d.sched[32 + k];
        d.sched[0] = n;
    }
}

// small islands: one thread walks the island's rows in global memory
__global__ void k_pgs_small(Dev d) {
    const int n = d.sched[1];
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int i = d.small_list[q];
        const int rs = d.g_isl_row_start[i], rc = d.g_isl_row_count[i];
        const int bs = d.g_isl_body_start[i], bc = d.g_isl_body_count[i];
        const WorldParams& P = d.wparams[d.g_isl_world[i]];
        float4* dv = d.dv + kDvF4 * (size_t)bs;
        for (int k = 0; k < kDvF4 * bc; k++) dv[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int r = rs; r < rs + rc; r++) row_warm(d.rows[r], d.rows[r].imp, dv);
        for (int it = 0; it < P.pgs_vel; it++)
            for (int r = rs; r < rs + rc; r++) {
                RowBlock& R = d.rows[r];
                float4 imp = R.imp;
                int st = R.stat;
                row_vel(R, imp, st, dv);
                R.imp = imp;
                R.stat = st;
            }
        for (int it = 0; it < P.pgs_pos; it++)
            for (int r = rs; r < rs + rc; r++) {
                RowBlock& R = d.rows[r];
                float4 imp = R.imp;
                row_pos(R, imp, dv);
                R.imp = imp;
            }
        island_finish(d, rs, rc, bs, bc, dv, 0, 1);
    }
}

// ---- large islands: one warp per island, rows streamed through shared memory
constexpr int kRingSlots = 6;
constexpr int kChunkRows = 16;

__device__ __forceinline__ uint32_t saddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// `fence`: this thread wrote impulses to `src` with generic stores since its
// last proxy fence; those writes must be ordered before the async-proxy copy
// reads them.  (Its earlier reads of `dst` have completed: their values were
// used before this copy is issued.)
__device__ __forceinline__ void ring_load(RowBlock* dst, const RowBlock* src, int rows, uint64_t* bar, bool fence) {
    uint32_t bytes = (uint32_t)(rows * sizeof(RowBlock));
    if (fence) asm volatile("fence.proxy.async;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}

__device__ __forceinline__ bool ring_wait(uint64_t* bar, uint32_t parity, long long limit) {
    for (long long it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(done) : "r"(saddr(bar)), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// The serial Gauss-Seidel chain of one island on one thread: 1 warm-start pass,
// pgs_vel velocity passes and pgs_pos position passes over the island's rows,
// in order.  The first position pass is fused into the warm-start pass: the
// position rows read and write only the pseudo velocities and the pseudo
// impulse, which no other pass touches and which start at zero, so running
// position row j right after warm-start row j gives the same result as a
// separate pass, one pass sooner (the two rows' arithmetic interleaves).  Rows stream through the shared ring (look-ahead up to one pass,
// since a pass must see the impulses the previous pass wrote back); each row
// is copied to registers with 16-byte loads before it is used.
__device__ __forceinline__ bool big_chain(const Dev& d, RowBlock* ring, uint64_t* bars, uint32_t& phase, float4* dv, int rs,
                                       int rc, const WorldParams& P) {
    const int nch = (rc + kChunkRows - 1) / kChunkRows;
    const int n_vel = P.pgs_vel;   // read once: the row stores below could alias P for the compiler
    const int n_pos = P.pgs_pos;
    const bool fused = n_pos > 0;
    const int passes = 1 + n_vel + (fused ? n_pos - 1 : 0);
    const int total = passes * nch;
    const int ahead = nch < kRingSlots ? nch : kRingSlots;
    // A proxy fence covers every impulse write issued before it.  Chunk c of
    // sequence t was last written at sequence t - nch (every pass writes when
    // the position rows are fused into the warm-start pass, the others from
    // the first velocity pass on); a fence is needed only if none was issued
    // since: about once per pass on a large island, every chunk on a small one.
    int fenced = -1;
    // body pair whose Δv the velocity passes hold in registers (-1: none)
    int cur_a = -1, cur_b = -1;
    P3 ca{}, cb{};
    auto issue = [&](int t, int now) {
        int c = t % nch, slot = t % kRingSlots;
        int n = min(kChunkRows, rc - c * kChunkRows);
        const int tw = t - nch;
        const bool fence = tw >= (fused ? 0 : nch) && tw > fenced;
        if (fence) fenced = now;
        ring_load(ring + slot * kChunkRows, d.rows + rs + c * kChunkRows, n, &bars[slot], fence);
    };
    for (int t = 0; t < ahead && t < total; t++) issue(t, -1);
    for (int t = 0; t < total; t++) {
        const int slot = t % kRingSlots, pass = t / nch, c = t % nch;
        if (!ring_wait(&bars[slot], (phase >> slot) & 1u, d.wait_limit)) {
            // gave up on chunk t: let the copies already issued (chunks t to
            // t + ahead - 1) land before the ring is abandoned (bounded)
            for (int u = t; u < t + ahead && u < total; u++) {
                const int su = u % kRingSlots;
                ring_wait(&bars[su], (phase >> su) & 1u, kDefaultWaitLimit);
            }
            return false;
        }
        phase ^= 1u << slot;
        const int n = min(kChunkRows, rc - c * kChunkRows);
        const float4* rb = reinterpret_cast<const float4*>(ring + slot * kChunkRows);
        RowBlock* g = d.rows + rs + c * kChunkRows;
        auto load = [&](int j, RowBlock& R) {
            float4* dst = reinterpret_cast<float4*>(&R);
#pragma unroll
            for (int k = 0; k < (int)(sizeof(RowBlock) / 16); k++) dst[k] = rb[j * (sizeof(RowBlock) / 16) + k];
        };
        // one loop per pass kind (the pass is fixed within a chunk); the
        // friction state is read only after the last velocity pass, so only
        // that pass stores it
        if (pass == 0) {
            for (int j = 0; j < n; j++) {
                RowBlock R;
                load(j, R);
                float4 imp = R.imp;
                row_warm(R, imp, dv);
                if (fused) {
                    row_pos(R, imp, dv);
                    g[j].imp = imp;
                }
            }
        } else if (pass <= n_vel) {
            // consecutive rows of one body pair (the points of a manifold)
            // keep the pair's Δv in registers: the array is read when the
            // pair changes and written back when it changes again (at the
            // latest at the end of the pass), so the chain skips the
            // shared-memory round trip between such rows
            const bool last_vel = pass == n_vel;
            for (int j = 0; j < n; j++) {
                RowBlock R;
                load(j, R);
                if (R.sa != cur_a || R.sb != cur_b) {
                    dv_put(dv, cur_a, 0, ca);
                    dv_put(dv, cur_b, 0, cb);
                    cur_a = R.sa;
                    cur_b = R.sb;
                    ca = dv_get(dv, cur_a, 0);
                    cb = dv_get(dv, cur_b, 0);
                }
                float4 imp = R.imp;
                int st = R.stat;
                row_vel_r(R, imp, st, ca, cb);
                g[j].imp = imp;
                if (last_vel) g[j].stat = st;
            }
            if (c == nch - 1) {
                dv_put(dv, cur_a, 0, ca);
                dv_put(dv, cur_b, 0, cb);
                cur_a = cur_b = -1;
            }
        } else {
            for (int j = 0; j < n; j++) {
                RowBlock R;
                load(j, R);
                float4 imp = R.imp;
                row_pos(R, imp, dv);
                g[j].imp = imp;
            }
        }
        if (t + ahead < total) issue(t + ahead, t);
    }
    return true;
}

// One warp's solver-chain worker: takes big-island list entries q0, q0+1, ...
// (below q1) through `counter` and runs each island's chain.  `sm`: the
// warp's own shared area (mbarriers, row ring, Δv of up to `dv_cap` bodies).
// False when a bounded wait gave up (the status is set).
__device__ bool big_worker(const Dev& d, int dv_cap, uint8_t* sm, int* counter, int q0, int q1) {
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm);
    RowBlock* ring = reinterpret_cast<RowBlock*>(sm + 64);
    float4* sdv = reinterpret_cast<float4*>(sm + 64 + kRingSlots * kChunkRows * sizeof(RowBlock));
    const int lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < kRingSlots; k++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(&bars[k])), "r"(1) : "memory");
        }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncwarp();
    uint32_t phase = 0;   // bit k: parity of slot k
    while (true) {
        int q = 0;
        if (lane == 0) q = q0 + atomicAdd(counter, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= q1) break;
        const int i = d.big_list[q];
        const int rs = d.g_isl_row_start[i], rc = d.g_isl_row_count[i];
        const int bs = d.g_isl_body_start[i], bc = d.g_isl_body_count[i];
        const WorldParams& P = d.wparams[d.g_isl_world[i]];
        float4* dv = (bc <= dv_cap) ? sdv : d.dv + kDvF4 * (size_t)bs;
        for (int k = lane; k < kDvF4 * bc; k += 32) dv[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncwarp();
        bool ok = true;
        if (lane == 0) {
            ok = (bc <= dv_cap) ? big_chain(d, ring, bars, phase, sdv, rs, rc, P)
                                : big_chain(d, ring, bars, phase, d.dv + kDvF4 * (size_t)bs, rs, rc, P);
            if (!ok) atomicOr(d.status, ST_TIMEOUT);
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) return false;
        __syncwarp();
        island_finish(d, rs, rc, bs, bc, dv, lane, 32);
        __syncwarp();
    }
    return true;
}

// blockDim.x == 32; `dv_cap` island bodies fit in the shared Δv area
__global__ void __launch_bounds__(32) k_pgs_big(Dev d, int dv_cap) {
    extern __shared__ __align__(16) uint8_t sm[];
    big_worker(d, dv_cap, sm, &d.sched[2], 0, d.sched[0]);
}

// HolonomicSystem::computeAndApplyImpulses (HolonomicBlockSolver.cpp:319-378)
// for system s: solve A d = t - J dv with the factorisation, then (with a
// threshold) discard a pseudo solution whose angular velocity change exceeds
// it anywhere, else apply d.  Runs on one thread.
template <class T>
__device__ void holo_apply(const Dev& d, int s, float4* dv, float4* err, bool pseudo, float thr) {
    const HoloStore& hs = d.hs;
    const int c0 = hs.cstart[s], n = hs.cstart[s + 1] - c0, deg = hs.degree[s];
    const int* cons = hs.cons + c0;
    const int* vp = hs.vpos + c0;
    const T* B = reinterpret_cast<const T*>(hs.fp64[s] ? (const void*)(hs.pool64 + hs.bstart[s])
                                                       : (const void*)(hs.pool32 + hs.bstart[s]));
    T* v = reinterpret_cast<T*>(hs.work + hs.wstart[s]);
    T* eff = v + deg;
    const int which = pseudo ? 1 : 0;
    for (int i = 0; i < n; i++) {
        const JointRow& R = d.jt.rows[cons[i]];
        float va[6], vb[6], cur[kJMax];
        jload(dv, R.sa, which, va);
        jload(dv, R.sb, which, vb);
        jvalue(R, va, vb, cur);
        const float* tgt = pseudo ? R.ptarget : R.target;
        for (int k = 0; k < R.n; k++) { v[vp[i] + k] = (T)tgt[k] - (T)cur[k]; eff[vp[i] + k] = 0; }
    }
    holo_solve<T>(hs, s, d.jt.rows, B, v, eff);
    if (thr > 0.f) {
        for (int i = 0; i < n; i++) {
            const JointRow& R = d.jt.rows[cons[i]];
            float ic[kJMax];
            for (int k = 0; k < R.n; k++) ic[k] = (float)v[vp[i] + k];
            if (!jzero(ic, R.n)) japply(R, ic, err, 0);
        }
        for (int i = 0; i < n; i++) {
            const JointRow& R = d.jt.rows[cons[i]];
            float ea[6], eb[6];
            jload(err, R.sa, 0, ea);
            jload(err, R.sb, 0, eb);
            float r2 = 0.f;
            for (int k = 3; k < 6; k++) r2 += ea[k] * ea[k] + eb[k] * eb[k];
            if (r2 > thr * thr) return;
        }
    }
    for (int i = 0; i < n; i++) {
        JointRow& R = d.jt.rows[cons[i]];
        float ic[kJMax];
        for (int k = 0; k < R.n; k++) ic[k] = (float)v[vp[i] + k];
        if (jzero(ic, R.n)) continue;
        japply(R, ic, dv, which);
        float* acc = pseudo ? R.pimpulse : R.holo;
        for (int k = 0; k < R.n; k++) acc[k] += ic[k];
    }
}

// islands with joint rows: one warp per island, the serial chain on lane 0
// over contact rows and joint rows in island order, then the island's
// holonomic systems (first substep); Δv and the linearisation probe in global
// memory
__global__ void __launch_bounds__(32) k_pgs_joint(Dev d, int first) {
    const int lane = threadIdx.x;
    const int nj = d.sched[3];
    for (int q = blockIdx.x; q < nj; q += gridDim.x) {
        const int i = d.joint_list[q];
        const int rs = d.g_isl_row_start[i], rc = d.g_isl_row_count[i];
        const int bs = d.g_isl_body_start[i], bc = d.g_isl_body_count[i];
        const WorldParams& P = d.wparams[d.g_isl_world[i]];
        float4* dv = d.dv + kDvF4 * (size_t)bs;
        float4* err = d.dv_err + kDvF4 * (size_t)bs;
        for (int k = lane; k < kDvF4 * bc; k += 32) { dv[k] = make_float4(0.f, 0.f, 0.f, 0.f); err[k] = dv[k]; }
        __syncwarp();
        if (lane == 0) {
            for (int r = rs; r < rs + rc; r++) {
                const int c = d.rows[r].contact;
                if (c >= 0) row_warm(d.rows[r], d.rows[r].imp, dv);
                else jwarm(d.jt.rows[-c - 1], dv);
            }
            const int n_vel = P.pgs_vel, n_pos = P.pgs_pos;   // read once: the row stores could alias P
            for (int it = 0; it < n_vel; it++)
                for (int r = rs; r < rs + rc; r++) {
                    RowBlock& R = d.rows[r];
                    if (R.contact < 0) { jstep(d.jt.rows[-R.contact - 1], dv, false); continue; }
                    float4 imp = R.imp;
                    int st = R.stat;
                    row_vel(R, imp, st, dv);
                    R.imp = imp;
                    R.stat = st;
                }
            for (int it = 0; it < n_pos; it++)
                for (int r = rs; r < rs + rc; r++) {
                    RowBlock& R = d.rows[r];
                    if (R.contact < 0) {
                        JointRow& Jr = d.jt.rows[-R.contact - 1];
                        if (Jr.pos) jstep(Jr, dv, true);   // needsPosCorrect
                        continue;
                    }
                    float4 imp = R.imp;
                    row_pos(R, imp, dv);
                    R.imp = imp;
                }
            if (first && P.pgs_holo > 0) {
                const int ss = d.g_isl_sys_start[i], sn = d.g_isl_sys_count[i];
                for (int it = 0; it < P.pgs_holo; it++)
                    for (int k = 0; k < sn; k++) {
                        const int s = d.isl_sys[ss + k];
                        if (d.hs.fp64[s]) {
                            holo_apply<double>(d, s, dv, err, false, -1.f);
                            holo_apply<double>(d, s, dv, err, true, d.lin_err_threshold);
                        } else {
                            holo_apply<float>(d, s, dv, err, false, -1.f);
                            holo_apply<float>(d, s, dv, err, true, d.lin_err_threshold);
                        }
                    }
            }
        }
        __syncwarp();
        for (int r = rs + lane; r < rs + rc; r += 32) {
            const int c = d.rows[r].contact;
            if (c >= 0) continue;
            const int j = -c - 1;
            const JointRow& R = d.jt.rows[j];
            for (int k = 0; k < R.n; k++) d.jt.impulse[kJMax * j + k] = R.impulse[k];
        }
        island_finish(d, rs, rc, bs, bc, dv, lane, 32);
        __syncwarp();
    }
}

__device__ M33 crossm(f3 v) {
    M33 o;
    o.m[0] = 0.f;  o.m[1] = -v.z; o.m[2] = v.y;
    o.m[3] = v.z;  o.m[4] = 0.f;  o.m[5] = -v.x;
    o.m[6] = -v.y; o.m[7] = v.x;  o.m[8] = 0.f;
    return o;
}

__global__ void k_integrate(Dev d, int last) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n_bodies; i += gridDim.x * blockDim.x) {
        const int mv = d.movement[i];
        if (mv == 1 || (d.has_sleep && d.asleep[i])) continue;   // sleeping bodies stay put
        const WorldParams& P = d.wparams[d.world[i]];
        const float dt = P.dt_sub;
        float4 pos = d.pos[i], q = d.rot[i];
        const float4 pos0 = pos, q0 = q;
        f3 v = mk(d.vel[i]), w = mk(d.angv[i]), pv = mk(d.pvel[i]), pw = mk(d.pangv[i]);
        f3 c = mk(pos) + (v + pv) * dt;
        pos.x = c.x; pos.y = c.y; pos.z = c.z;
        if (mag2(w) != 0.f) {
            const bool no_gyro = P.gyro_disabled || mv == 2;
            if (no_gyro) {
                q = qmul(qaxis(mag(w) * dt, normalize(w)), q);
            } else {
                // RigidBody::rotateWhileApplyingGyroAccel: implicit Euler on the
                // gyroscopic term, angle_ticks sub-steps of two Newton iterations
                const M33 Iref = load9(d.iref + 9 * i);
                M33 it = load9(d.iw + 9 * i);
                float4 iq = q;
                f3 iw = w;
                const int n_itr = P.angle_ticks;
                for (int s = 0; s < n_itr; s++) {
                    f3 wv = iw;
                    float ts = dt / n_itr;
                    for (int k = 0; k < 2; k++) {
                        f3 Iw = mul(it, wv);
                        f3 f = ts * cross(wv, Iw) - mul(it, iw - wv);
                        M33 cw = mul(crossm(wv), it), ci = crossm(Iw);
                        M33 jac;
                        for (int m = 0; m < 9; m++) jac.m[m] = it.m[m] + ts * (cw.m[m] - ci.m[m]);
                        if (fabsf(det(jac)) > 0.00000000001f) wv = wv - mul(inverse(jac), f);
                    }
                    iw = wv;
                    iq = qmul(qaxis(ts * mag(iw), iw), iq);
                    if (s + 1 < n_itr) {
                        M33 R = quatRot(iq), Rc = quatRot(qconj(iq));
                        it = mul(mul(R, Iref), Rc);
                    }
                }
                q = iq;
                w = iw;
            }
            q = qmul(qaxis(dt * mag(pw), pw), q);
        }
        // RigidBody::updateInertiaTensor (RigidBody.cpp:270-279)
        q = qnormalize(q);
        if (mv == 0) {
            M33 R = quatRot(q), Rc = quatRot(qconj(q));
            store9(d.iw + 9 * i, mul(mul(R, load9(d.iref + 9 * i)), Rc));
            store9(d.iinv + 9 * i, mul(mul(R, load9(d.iinv_ref + 9 * i)), Rc));
        }
        if (!(isfinite(c.x) && isfinite(c.y) && isfinite(c.z) && isfinite(q.x))) atomicOr(d.status, ST_NAN);
        d.pos[i] = pos;
        d.rot[i] = q;
        d.angv[i] = make_float4(w.x, w.y, w.z, 0.f);
        d.pvel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        d.pangv[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (last) {
            bool moved = pos.x != pos0.x || pos.y != pos0.y || pos.z != pos0.z || q.x != q0.x || q.y != q0.y || q.z != q0.z || q.w != q0.w;
            d.moved[i] = moved;
        }
    }
}

// External state write (cpgpu_batch_write_state): velocities are taken as
// given; a body whose pose changed gets its world inertia tensors and AABB
// recomputed from the new pose, an unchanged body keeps them bit for bit.
__global__ void k_apply_state(Dev d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n_bodies; i += gridDim.x * blockDim.x) {
        const float4 p = d.stage[4 * i], q = d.stage[4 * i + 1], v = d.stage[4 * i + 2], w = d.stage[4 * i + 3];
        if (d.movement[i] != 1) {
            d.vel[i] = make_float4(v.x, v.y, v.z, 0.f);
            d.angv[i] = make_float4(w.x, w.y, w.z, 0.f);
        }
        const float4 p0 = d.pos[i], q0 = d.rot[i];
        if (p.x == p0.x && p.y == p0.y && p.z == p0.z && q.x == q0.x && q.y == q0.y && q.z == q0.z && q.w == q0.w) continue;
        d.pos[i] = make_float4(p.x, p.y, p.z, p0.w);
        d.rot[i] = q;
        M33 R = quatRot(q), Rc = quatRot(qconj(q));
        if (d.movement[i] == 0) {
            store9(d.iw + 9 * i, mul(mul(R, load9(d.iref + 9 * i)), Rc));
            store9(d.iinv + 9 * i, mul(mul(R, load9(d.iinv_ref + 9 * i)), Rc));
        }
        f3 mn, mx;
        shape_aabb(d.shapes + d.shape[i], mk(p), R, &mn, &mx);
        d.aabb_lo[i] = make_float4(mn.x, mn.y, mn.z, 0.f);
        d.aabb_hi[i] = make_float4(mx.x, mx.y, mx.z, 0.f);
    }
}

// host-layout state rows (pos, rot, vel, ang vel per body) of a batch split
// into parts: each part gathers / scatters its bodies' rows by index
__global__ void k_gather_state(const float4* __restrict__ all, const int* __restrict__ rows, int n, float4* __restrict__ stage) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = rows[i];
        for (int k = 0; k < 4; k++) stage[4 * i + k] = all[4 * (size_t)r + k];
    }
}
__global__ void k_scatter_state(Dev d, const int* __restrict__ rows, float4* __restrict__ all) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n_bodies; i += gridDim.x * blockDim.x) {
        float4* o = all + 4 * (size_t)rows[i];
        o[0] = d.pos[i]; o[1] = d.rot[i]; o[2] = d.vel[i]; o[3] = d.angv[i];
    }
}

int grid_for(int n, int per_block, int n_sms) {
    int g = (n + per_block - 1) / per_block;
    int cap = n_sms * 8;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

}  // namespace

void launch_rows(const Dev& d, int first, int last, const Launch& L) {
    k_rows<<<L.n_sms * 8, 128, 0, L.st>>>(d, first, last);
}

int pgs_big_smem_bytes(int dv_cap) {
    return 64 + kRingSlots * kChunkRows * (int)sizeof(RowBlock) + dv_cap * 16 * kDvF4;
}

// blocks of k_pgs_big resident per SM for this Δv capacity (one chain each)
int pgs_big_blocks_per_sm(int dv_cap) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_pgs_big, 32, pgs_big_smem_bytes(dv_cap)) != cudaSuccess || n < 1) n = 1;
    return n;
}

// The attribute is the kernel's, shared by every batch of the process: it is
// set for the largest Δv area any batch uses, so that a batch built later with
// a smaller one does not lower the limit under an earlier batch's launches
void prepare_pgs(int dv_cap) {
    (void)dv_cap;
    cudaFuncSetAttribute(k_pgs_big, cudaFuncAttributeMaxDynamicSharedMemorySize, pgs_big_smem_bytes(kPgsDvCapMax));
}

void launch_pgs_schedule(const Dev& d, const Launch& L) {
    k_sched_reset<<<1, 96, 0, L.st>>>(d);
    k_sched_count<<<L.n_sms * 2, 256, 0, L.st>>>(d);
    k_sched_place<<<L.n_sms * 2, 256, 0, L.st>>>(d);
}

void launch_pgs_joint(const Dev& d, bool first, const Launch& L) {
    if (d.n_joint_edges == 0) return;
    k_pgs_joint<<<L.n_sms * 8, 32, 0, L.st>>>(d, first ? 1 : 0);
}

void launch_pgs(const Dev& d, int dv_cap, int big_blocks, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, const Launch& L) {
    // large islands on the main stream, small ones concurrently on a side branch
    cudaMemsetAsync(d.sched + 2, 0, sizeof(int), L.st);
    cudaEventRecord(fork, L.st);
    cudaStreamWaitEvent(side, fork, 0);
    k_pgs_small<<<L.n_sms * 4, 64, 0, side>>>(d);
    cudaEventRecord(join, side);
    k_pgs_big<<<big_blocks, 32, pgs_big_smem_bytes(dv_cap), L.st>>>(d, dv_cap);
    cudaStreamWaitEvent(L.st, join, 0);
}

void launch_integrate(const Dev& d, int last, const Launch& L) {
    k_integrate<<<grid_for(d.n_bodies, 128, L.n_sms), 128, 0, L.st>>>(d, last);
}

void launch_apply_state(const Dev& d, const Launch& L) {
    k_apply_state<<<grid_for(d.n_bodies, 128, L.n_sms), 128, 0, L.st>>>(d);
}

void launch_gather_state(const Dev& d, const float4* all, const int* rows, const Launch& L) {
    k_gather_state<<<grid_for(d.n_bodies, 128, L.n_sms), 128, 0, L.st>>>(all, rows, d.n_bodies, d.stage);
}

void launch_scatter_state(const Dev& d, const int* rows, float4* all, const Launch& L) {
    k_scatter_state<<<grid_for(d.n_bodies, 128, L.n_sms), 128, 0, L.st>>>(d, rows, all);
}

}  // namespace cpgpu
