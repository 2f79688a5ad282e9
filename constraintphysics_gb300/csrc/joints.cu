// joints.cu — joint rows (ball-socket, hinge, distance, weld, slider, sliding
// hinge, cone and twist limits), springs, and the factorisation of the
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

// crossMat (NMat.cpp:59-67), row-major
__device__ __forceinline__ void cross_mat(f3 v, float m[3][3]) {
    m[0][0] = 0.f;  m[0][1] = -v.z; m[0][2] = v.y;
    m[1][0] = v.z;  m[1][1] = 0.f;  m[1][2] = -v.x;
    m[2][0] = -v.y; m[2][1] = v.x;  m[2][2] = 0.f;
}
// (1x3 row) * (3x3), as NMat<1,3> * NMat<3,3> accumulates it
__device__ __forceinline__ f3 row_times(f3 v, const float m[3][3]) {
    return mk(v.x * m[0][0] + v.y * m[1][0] + v.z * m[2][0], v.x * m[0][1] + v.y * m[1][1] + v.z * m[2][1],
              v.x * m[0][2] + v.y * m[1][2] + v.z * m[2][2]);
}
__device__ __forceinline__ void set_row(float* j, f3 lin, f3 ang) {
    j[0] = lin.x; j[1] = lin.y; j[2] = lin.z; j[3] = ang.x; j[4] = ang.y; j[5] = ang.z;
}

// angle * axis of q_b * conj(q_a) scaled by c (Quaternion::angleTo and
// getRotAxis, Math/src/Quaternion.h:35-49): the orientation error of the weld
// and slider rows.  The reference takes 2 acos(|q_a . q_b|) and calls angles
// below 2 acos(0.99999999999) zero; in FP32 the arc cosine of a dot product
// near 1 loses the angle (resolution ~3e-4 rad), so the same angle is taken
// as 2 atan2(|vec(dq)|, |dq.r|) (dq.r = q_a . q_b), with the same cutoff.
__device__ __forceinline__ f3 orientation_error(float4 qa, float4 qb, float c) {
    const float4 dq = qmul(qb, qconj(qa));
    const f3 v = mk(dq.y, dq.z, dq.w);
    const float s = mag(v);
    const float angle = 2.0f * atan2f(s, fabsf(dq.x));
    if (!(angle >= 8.944272e-6f) || s == 0.f) return mk(0.f, 0.f, 0.f);
    const f3 axis = (dq.x < 0.f ? -1.0f / s : 1.0f / s) * v;
    return (angle * c) * axis;
}

// 1 - cos(f) by its series to the 8th order, as the limit rows' error
// (ConstraintSolver.cpp:415-421, 447-455)
__device__ __forceinline__ float limit_error(float f) {
    const float f2 = f * f, f4 = f2 * f2, f6 = f4 * f2, f8 = f4 * f4;
    return -f8 / 40320.0f + f6 / 720.0f - f4 / 24.0f + f2 / 2.0f;
}

// Motor::calculatePosition (PersistentConstraint.cpp:30-71): the last angle
// advanced by the relative angular velocity, snapped to the angle of body 2's
// comparison axis in body 1's (u, w) plane in the 2 pi window nearest the
// prediction, unless that axis is within acos(0.999) of the motor axis.  The
// reference takes that angle as 2 pi - acos(c . u) (or acos(c . u) when
// c . w < 0); in FP32 the arc cosine of a dot product near 1 has a resolution
// of ~3.5e-4 rad, so the same angle is taken from the signed
// atan2(c . w, c . u) instead.
__device__ float motor_position(float prev, f3 axis, f3 w1, f3 w2, float dts, float4 qa, float4 qb, f3 ul, f3 wl, f3 cl) {
    const float kTwoPi = 2.0f * 3.1415926535f;
    const f3 ref_u = qrot(qa, ul), ref_w = qrot(qa, wl), cmp = qrot(qb, cl);
    const float rel = dot(axis, w1) - dot(axis, w2);
    const float pred = prev + rel * dts;
    if (fabsf(dot(cmp, axis)) > 0.999f) return pred;
    const f3 cn = normalize(cmp - axis * dot(axis, cmp));
    const float su = dot(cn, ref_u), sw = dot(cn, ref_w);
    const float th = atan2f(sw, su);                 // acos(c . u) with the sign of c . w
    const float rel_angle = sw >= 0.f ? kTwoPi - th : -th;
    const float n2 = pred - fmodf(pred, kTwoPi);
    const float c[3] = {n2 + rel_angle - kTwoPi, n2 + rel_angle, n2 + rel_angle + kTwoPi};
    float closest = INFINITY;
    for (int k = 0; k < 3; k++)
        if (fabsf(pred - c[k]) < fabsf(pred - closest)) closest = c[k];
    return closest;
}

// Motor::getConstraintTargetVelocityValue and
// Piston::getPistonTargetVelocityValue (PersistentConstraint.cpp:77-109,
// 153-185): off 0, constant torque / force an infinite target in its
// direction, target velocity as set, target position the velocity that the
// max torque / force reaches over the remaining distance, the inertia from
// the last impulse and velocity change (or from `inv_inertia` when either is
// below 1e-7; the reference's `abs(impulse < EPS)` holds for every impulse
// below 1e-7, negative ones included)
__device__ float powered_target(float4 pw, float position, float rel_vel, float prev_vel, float impulse, float inv_inertia) {
    const int mode = (int)pw.x;
    if (mode == 0) return 0.f;
    if (mode == 1) return pw.y > 0.f ? INFINITY : -INFINITY;
    if (mode == 2) return pw.z;
    const float ang_diff = position - pw.w;
    const float dir = ang_diff > 0.f ? -1.f : 1.f;
    const float vdt = fabsf(rel_vel - prev_vel);
    const float inertia = (vdt < 0.0000001f || impulse < 0.0000001f) ? 1.0f / inv_inertia : fabsf(impulse) / vdt;
    return dir * sqrtf(2.0f * fabsf(ang_diff) * pw.y / inertia);
}

__global__ void k_joint_rows(Dev d) {
    const JointStore& J = d.jt;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < d.n_joints; j += gridDim.x * blockDim.x) {
        const int a = J.b1[j], b = J.b2[j], n = J.n[j], kind = J.kind[j];
        if (d.movement[a] != 0 && d.movement[b] != 0) continue;
        const WorldParams& P = d.wparams[d.world[a]];
        const float dts = P.dt_sub;
        const float4 qa = d.rot[a], qb = d.rot[b];
        const f3 ca = mk(d.pos[a]), cb = mk(d.pos[b]);
        const float2 hard = J.hard[j];
        JointRow& R = d.jt.rows[j];
        float* jimp = J.impulse + kJMax * (size_t)j;
        bool rebuilt = true;
        if (kind == JK_MOTOR) {
            // Motor::updateSolverConstraints (PersistentConstraint.cpp:320-328)
            // with MotorConstraint (ConstraintSolver.cpp:555-585): the angle
            // advanced first; while powered or past a limit one row on body 1's
            // axis (target velocity limited to the limit's side and a one-sided
            // projection past a limit, else bounded by max torque x dt); the old
            // row kept otherwise
            const f3 axis = qrot(qa, mk(J.ax1[j]));
            const f3 w1 = d.movement[a] == 1 ? mk(0.f, 0.f, 0.f) : mk(d.angv[a]);
            const f3 w2 = d.movement[b] == 1 ? mk(0.f, 0.f, 0.f) : mk(d.angv[b]);
            const float4 pw = J.power[j];
            const float mx = J.par[j].x, mn = J.par[j].y;
            const float pos = motor_position(J.angle[j], axis, w1, w2, dts, qa, qb, mk(J.ul[j]), mk(J.wl[j]), mk(J.ax2[j]));
            J.angle[j] = pos;
            const bool listed = ((int)pw.x != 0 && pw.y != 0.f) || pos < mn || pos > mx;
            J.active[j] = listed ? 1 : 0;
            const float rel = dot(axis, w1) - dot(axis, w2);
            if (listed) {
                const M33 Ia = load9(d.iinv + 9 * a), Ib = load9(d.iinv + 9 * b);
                const float inv_i = dot(axis, mul(Ia, axis)) + dot(axis, mul(Ib, axis));
                const float tv = powered_target(pw, pos, rel, J.aux[j], jimp[0], inv_i);
                const float hc = fminf(hard.y * dts, 1.0f / dts);
                R.n = 1;
                R.impulse[0] = P.warm_disabled ? 0.f : jimp[0];
                R.pimpulse[0] = 0.f;
                R.holo[0] = 0.f;
                set_row(R.ja, mk(0.f, 0.f, 0.f), axis);
                set_row(R.jb, mk(0.f, 0.f, 0.f), -axis);
                R.has_vt = 1;
                R.pos = 1;
                if (pos > mx) { R.ptarget[0] = (mx - pos) * hc; R.vt = fminf(0.f, tv); R.proj = 2; }
                else if (pos < mn) { R.ptarget[0] = (mn - pos) * hc; R.vt = fmaxf(0.f, tv); R.proj = 1; }
                else { R.ptarget[0] = 0.f; R.vt = tv; R.proj = 3; R.lim = fabsf(pw.y * dts); R.pos = 0; }
            } else {
                rebuilt = false;
            }
            J.aux[j] = rel;
        } else if (kind == JK_SLIDE_LIMIT || kind == JK_PISTON) {
            // Piston::updateSolverConstraints (PersistentConstraint.cpp:300-318):
            // the slide position along body 1's axis between the slider's
            // tracked points; past a limit a SlideLimitConstraint row
            // (ConstraintSolver.cpp:736-775), while powered a PistonConstraint
            // row (:701-731), both along the axis (their angular Jacobian,
            // -s^T [s]x, is zero)
            const f3 pa = qrot(qa, mk(J.p1[j])) + ca, pb = qrot(qb, mk(J.p2[j])) + cb;
            const f3 axis = qrot(qa, mk(J.ax1[j]));
            const float pos = dot(pb, axis) - dot(pa, axis);
            const float mx = J.par[j].x, mn = J.par[j].y;
            const bool exceeded = pos < mn || pos > mx;
            const float4 pw = J.power[j];
            J.angle[j] = pos;
            J.aux[j] = exceeded ? 1.f : 0.f;
            const bool listed = kind == JK_SLIDE_LIMIT ? exceeded : ((int)pw.x != 0 && pw.y != 0.f);
            J.active[j] = listed ? 1 : 0;
            if (listed) {
                R.n = 1;
                R.impulse[0] = P.warm_disabled ? 0.f : jimp[0];
                R.pimpulse[0] = 0.f;
                R.holo[0] = 0.f;
                set_row(R.ja, -axis, mk(0.f, 0.f, 0.f));
                set_row(R.jb, axis, mk(0.f, 0.f, 0.f));
                if (kind == JK_SLIDE_LIMIT) {
                    const float hc = fminf(hard.x * dts, 1.0f / dts);
                    R.has_vt = 0;
                    R.pos = 1;
                    if (pos > mx) { R.ptarget[0] = (mx - pos) * hc; R.proj = 2; }
                    else { R.ptarget[0] = (mn - pos) * hc; R.proj = 1; }
                } else {
                    const f3 v1 = d.movement[a] == 1 ? mk(0.f, 0.f, 0.f) : mk(d.vel[a]);
                    const f3 v2 = d.movement[b] == 1 ? mk(0.f, 0.f, 0.f) : mk(d.vel[b]);
                    // the piston's previous velocity is never written and stays 0
                    R.vt = powered_target(pw, pos, dot(axis, v1) - dot(axis, v2), 0.f, jimp[0], d.pos[a].w + d.pos[b].w);
                    R.has_vt = 1;
                    R.proj = 3;
                    R.lim = pw.y * dts;
                    R.pos = 0;
                    R.ptarget[0] = 0.f;
                }
            } else {
                rebuilt = false;
            }
        } else if (jk_limit(kind)) {
            // ConeRotationLimit / TwistLimit::updateSolverConstraints
            // (PersistentConstraint.cpp:233-272): inside the limit the row is
            // inactive (warm impulse cleared, the old row kept, not listed in
            // the next islands); at or past it a one-dof row on the axis,
            // warm-started from the stored impulse unscaled
            bool inactive;
            float f;
            f3 ja_ang, jb_ang;
            int proj = 1;
            if (kind == JK_CONE) {
                const f3 d1 = qrot(qa, mk(J.ax1[j])), d2 = qrot(qb, mk(J.ax2[j]));
                // the reference's acos(d1 . d2) is taken on the dot product
                // clamped to [-1, 1] (FP32 rounding can leave it above 1)
                const float cur = acosf(fminf(1.0f, fmaxf(-1.0f, dot(d1, d2))));
                const float mx = J.par[j].x;
                inactive = cur < mx;
                const f3 h = normalize(cross(d1, d2));
                ja_ang = h;
                jb_ang = -h;
                f = cur - mx;
            } else {
                // getCurrentAngle (PersistentConstraint.cpp:115-131): body 1's
                // w axis carried by body 2, measured in body 1's (w, u) frame,
                // unwrapped against the previous value with the reference's
                // truncated pi
                const M33 r1 = quatRot(qa), r2 = quatRot(qb);
                const f3 t1 = mul(r1, mk(J.ax1[j])), u1 = mul(r1, mk(J.ul[j])), w1 = mul(r1, mk(J.wl[j]));
                const f3 t2 = mul(r2, mk(J.ax2[j])), r2w = mul(r2, mk(J.wl[j]));
                const float kPi = 3.1415926535f;
                const float prev = J.angle[j];
                float ang = atan2f(dot(r2w, u1), dot(r2w, w1));
                while (prev - ang > kPi) ang += 2.0f * kPi;
                while (prev - ang < -kPi) ang -= 2.0f * kPi;
                J.angle[j] = ang;
                const float mn = J.par[j].y, mx = J.par[j].x;
                inactive = mn <= ang && ang <= mx;
                const bool above = ang > mx;
                proj = above ? 2 : 1;
                ja_ang = -t1;
                jb_ang = t2;
                f = above ? ang - mx : mn - ang;
            }
            J.active[j] = inactive ? 0 : 1;
            if (inactive) {
                jimp[0] = 0.f;
                R.impulse[0] = 0.f;
                rebuilt = false;
            } else {
                R.n = 1;
                R.proj = proj;
                R.has_vt = 0;
                R.pos = 1;
                R.impulse[0] = jimp[0];
                R.pimpulse[0] = 0.f;
                R.holo[0] = 0.f;
                set_row(R.ja, mk(0.f, 0.f, 0.f), ja_ang);
                set_row(R.jb, mk(0.f, 0.f, 0.f), jb_ang);
                R.ptarget[0] = limit_error(f) * hard.y;
            }
        } else {
            const f3 pa = qrot(qa, mk(J.p1[j])) + ca, pb = qrot(qb, mk(J.p2[j])) + cb;
            const float pos_c = fminf(hard.x * dts, 1.0f / dts);
            const float rot_c = fminf(hard.y * dts, 1.0f / dts);
            R.n = n;
            R.proj = 0;
            R.has_vt = 0;
            R.pos = 1;
            float warm[kJMax];
            // Weld::updateSolverConstraints passes the previous impulse on
            // unscaled whatever the warm-start switch says
            // (PersistentConstraint.cpp:344-353)
            for (int i = 0; i < n; i++) warm[i] = (P.warm_disabled && kind != JK_WELD) ? 0.f : jimp[i];
            for (int i = 0; i < n; i++) { R.impulse[i] = warm[i]; R.pimpulse[i] = 0.f; R.holo[i] = 0.f; }
            const f3 rA = pa - ca;
            float sa[3][3], sb[3][3];
            cross_mat(rA, sa);
            if (kind == JK_BALL || kind == JK_WELD) {
                // BallSocketConstraint (ConstraintSolver.cpp:382-405), and the
                // WeldConstraint's three more rows locking the relative
                // angular velocity (:861-899)
                point_rows(R.ja, R.jb, rA, pb - cb);
                const f3 e = (pb - pa) * pos_c;
                R.ptarget[0] = e.x; R.ptarget[1] = e.y; R.ptarget[2] = e.z;
                if (kind == JK_WELD) {
                    for (int i = 0; i < 3; i++) {
                        const f3 u = mk(i == 0 ? 1.f : 0.f, i == 1 ? 1.f : 0.f, i == 2 ? 1.f : 0.f);
                        set_row(R.ja + 6 * (3 + i), mk(0.f, 0.f, 0.f), u);
                        set_row(R.jb + 6 * (3 + i), mk(0.f, 0.f, 0.f), -u);
                    }
                    const f3 oe = orientation_error(qa, qb, rot_c);
                    R.ptarget[3] = oe.x; R.ptarget[4] = oe.y; R.ptarget[5] = oe.z;
                }
            } else if (kind == JK_DISTANCE) {
                // DistanceConstraint (ConstraintSolver.cpp:348-377): one row
                // along the attachment direction, error target - |pa - pb|
                cross_mat(pb - cb, sb);
                const f3 diff = pa - pb;
                const f3 dd = normalize(diff);
                set_row(R.ja, dd, row_times(-dd, sa));
                set_row(R.jb, -dd, row_times(dd, sb));
                const float target = J.par[j].x;
                const float error = mag2(diff) < 0.00001f ? target : target - dot(dd, diff);
                R.ptarget[0] = pos_c * error;
            } else if (kind == JK_SLIDER) {
                // SliderConstraint (ConstraintSolver.cpp:611-696): two rows
                // across body 1's axis (its u, w) and three locking the
                // relative rotation; the orientation rows are corrected with
                // the position coefficient, as Slider::updateSolverConstraints
                // passes it (PersistentConstraint.cpp:287-298)
                cross_mat(pb - cb, sb);
                const f3 ax = normalize(qrot(qa, mk(J.ax1[j])));
                f3 uu, ww;
                basis(ax, &uu, &ww);
                const f3 su = mk(J.u[j]), sw = mk(J.w[j]);
                R.impulse[0] = dot(uu, su) * warm[0] + dot(uu, sw) * warm[1];
                R.impulse[1] = dot(ww, su) * warm[0] + dot(ww, sw) * warm[1];
                const f3 pe = pa - pb;
                float us[3][3], ws[3][3];
                cross_mat(uu, us);
                cross_mat(ww, ws);
                set_row(R.ja, uu, row_times(-uu, sa) - row_times(pe, us));
                set_row(R.jb, -uu, row_times(uu, sb));
                set_row(R.ja + 6, ww, row_times(-ww, sa) - row_times(pe, ws));
                set_row(R.jb + 6, -ww, row_times(ww, sb));
                for (int i = 0; i < 3; i++) {
                    const f3 u = mk(i == 0 ? 1.f : 0.f, i == 1 ? 1.f : 0.f, i == 2 ? 1.f : 0.f);
                    set_row(R.ja + 6 * (2 + i), mk(0.f, 0.f, 0.f), u);
                    set_row(R.jb + 6 * (2 + i), mk(0.f, 0.f, 0.f), -u);
                }
                const f3 oe = orientation_error(qa, qb, pos_c);
                R.ptarget[0] = -dot(pe, uu) * pos_c;
                R.ptarget[1] = -dot(pe, ww) * pos_c;
                R.ptarget[2] = oe.x; R.ptarget[3] = oe.y; R.ptarget[4] = oe.z;
                d.jt.u[j] = make_float4(uu.x, uu.y, uu.z, 0.f);
                d.jt.w[j] = make_float4(ww.x, ww.y, ww.z, 0.f);
            } else if (kind == JK_SLIDING_HINGE) {
                // SlidingHingeConstraint (ConstraintSolver.cpp:781-852): two
                // rows across body 2's axis and two keeping body 1's axis
                // parallel to it
                cross_mat(pb - cb, sb);
                const f3 na = qrot(qa, mk(J.ax1[j])), nb = qrot(qb, mk(J.ax2[j]));
                f3 uu, ww;
                basis(nb, &uu, &ww);
                const f3 su = mk(J.u[j]), sw = mk(J.w[j]);
                R.impulse[2] = dot(uu, su) * warm[2] + dot(uu, sw) * warm[3];
                R.impulse[3] = dot(ww, su) * warm[2] + dot(ww, sw) * warm[3];
                const f3 pd = pa - pb;
                float us[3][3], ws[3][3], ns[3][3];
                cross_mat(uu, us);
                cross_mat(ww, ws);
                cross_mat(na, ns);
                set_row(R.ja, uu, row_times(-uu, sa));
                set_row(R.jb, -uu, row_times(uu, sb) - row_times(pd, us));
                set_row(R.ja + 6, ww, row_times(-ww, sa));
                set_row(R.jb + 6, -ww, row_times(ww, sb) - row_times(pd, ws));
                set_row(R.ja + 12, mk(0.f, 0.f, 0.f), row_times(-uu, ns));
                set_row(R.jb + 12, mk(0.f, 0.f, 0.f), row_times(-na, us));
                set_row(R.ja + 18, mk(0.f, 0.f, 0.f), row_times(-ww, ns));
                set_row(R.jb + 18, mk(0.f, 0.f, 0.f), row_times(-na, ws));
                R.ptarget[0] = -dot(uu, pd) * pos_c;
                R.ptarget[1] = -dot(ww, pd) * pos_c;
                R.ptarget[2] = -dot(uu, na) * rot_c;
                R.ptarget[3] = -dot(ww, na) * rot_c;
                d.jt.u[j] = make_float4(uu.x, uu.y, uu.z, 0.f);
                d.jt.w[j] = make_float4(ww.x, ww.y, ww.z, 0.f);
            } else {
                // HingeConstraint (ConstraintSolver.cpp:468-550); the
                // reference's hinge takes rB from body 1's anchor point
                point_rows(R.ja, R.jb, rA, pa - cb);
                const f3 h1 = qrot(qa, mk(J.ax1[j])), nn = qrot(qb, mk(J.ax2[j]));
                f3 uu, ww;
                basis(h1, &uu, &ww);
                const f3 su = mk(J.u[j]), sw = mk(J.w[j]);
                R.impulse[3] = dot(uu, su) * warm[3] + dot(uu, sw) * warm[4];
                R.impulse[4] = dot(ww, su) * warm[3] + dot(ww, sw) * warm[4];
                // n^T [u]x, u^T [n]x, n^T [w]x, w^T [n]x
                set_row(R.ja + 18, mk(0.f, 0.f, 0.f), cross(nn, uu));
                set_row(R.jb + 18, mk(0.f, 0.f, 0.f), cross(uu, nn));
                set_row(R.ja + 24, mk(0.f, 0.f, 0.f), cross(nn, ww));
                set_row(R.jb + 24, mk(0.f, 0.f, 0.f), cross(ww, nn));
                const f3 pc = (pb - pa) * pos_c;
                R.ptarget[0] = pc.x; R.ptarget[1] = pc.y; R.ptarget[2] = pc.z;
                R.ptarget[3] = dot(uu, nn) * rot_c;
                R.ptarget[4] = dot(ww, nn) * rot_c;
                d.jt.u[j] = make_float4(uu.x, uu.y, uu.z, 0.f);
                d.jt.w[j] = make_float4(ww.x, ww.y, ww.z, 0.f);
            }
        }
        const int rn = R.n;
        if (rebuilt) {
            // impulse_to_{a,b}_velocity = M^-1 J^T, impulse_to_value, CFM inverse
            const float ima = d.pos[a].w, imb = d.pos[b].w;
            const M33 Ia = load9(d.iinv + 9 * a), Ib = load9(d.iinv + 9 * b);
            for (int i = 0; i < rn; i++) {
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
            for (int i = 0; i < rn; i++)
                for (int c = 0; c < rn; c++) {
                    float x = 0.f, y = 0.f;
                    for (int k = 0; k < 6; k++) { x += R.ja[6 * i + k] * R.ita[kJMax * k + c]; y += R.jb[6 * i + k] * R.itb[kJMax * k + c]; }
                    R.itv[kJMax * i + c] = x + y;
                    m[rn * i + c] = x + y;
                }
            for (int i = 0; i < rn; i++) m[rn * i + i] *= (1.0f + P.cfm);
            invert_block<float>(rn, m);
            for (int i = 0; i < rn; i++)
                for (int c = 0; c < rn; c++) R.minv[kJMax * i + c] = m[rn * i + c];
        }
        // target from the bodies' velocities at the start of the solve (also
        // for a limit row kept from an earlier rebuild: it is solved when its
        // island listed it)
        float va[6] = {0, 0, 0, 0, 0, 0}, vb[6] = {0, 0, 0, 0, 0, 0}, cur[kJMax];
        if (d.movement[a] != 1) {
            float4 v = d.vel[a], w = d.angv[a];
            va[0] = v.x; va[1] = v.y; va[2] = v.z; va[3] = w.x; va[4] = w.y; va[5] = w.z;
        }
        if (d.movement[b] != 1) {
            float4 v = d.vel[b], w = d.angv[b];
            vb[0] = v.x; vb[1] = v.y; vb[2] = v.z; vb[3] = w.x; vb[4] = w.y; vb[5] = w.z;
        }
        if (rn > 0) {
            jvalue(R, va, vb, cur);
            // MotorConstraint / PistonConstraint::findTargetConstraintValue
            // (ConstraintSolver.cpp:586-589, 723-726): the target velocity less the value
            if (R.has_vt) R.target[0] = R.vt - cur[0];
            else for (int i = 0; i < rn; i++) R.target[i] = -cur[i];
        }
    }
}

// Springs (maintainConstraintGraphApplyPoweredConstraints,
// PhysicsEngine.cpp:1309-1356): at the start of every substep, one thread
// per world applies its springs in the reference's order (they may share
// bodies, and each reads the velocities the previous one left): a stiffness
// impulse along the attachment direction, then a damping impulse capped so
// that it cannot reverse the relative velocity, measured at the reference's
// crossed attachment points (RigidBody::getVelOfPoint, RigidBody.cpp:153-155)
__device__ __forceinline__ void impulse_at(const Dev& d, int b, f3 imp, f3 at) {
    if (d.has_sleep) {
        // RigidBody::applyImpulse alerts the body (RigidBody.cpp:60-67,
        // alertWaking): its island wakes at the next step and its sleep
        // record restarts
        d.waking[b] = 1;
        d.ready_cnt[b] = 0;
        d.non_sleepy[b] = 0;
        d.hist_n[b] = 0;
        d.hist_head[b] = 0;
    }
    if (d.movement[b] != 0) return;   // RigidBody::applyImpulse on a fixed or kinematic body changes nothing
    const float4 p = d.pos[b];
    const f3 torque = cross(at - mk(p), imp);
    const M33 I = load9(d.iinv + 9 * b);
    const f3 dw = mul(I, torque);
    float4 v = d.vel[b], w = d.angv[b];
    v.x += p.w * imp.x; v.y += p.w * imp.y; v.z += p.w * imp.z;
    w.x += dw.x; w.y += dw.y; w.z += dw.z;
    d.vel[b] = v;
    d.angv[b] = w;
}

__global__ void k_springs(Dev d) {
    const SpringStore& S = d.sp;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < d.n_worlds; w += gridDim.x * blockDim.x) {
        const float dt = d.wparams[w].dt_sub;
        for (int k = S.world_start[w]; k < S.world_start[w + 1]; k++) {
            const int a = S.b1[k], b = S.b2[k];
            const f3 ca = mk(d.pos[a]), cb = mk(d.pos[b]);
            const f3 pa = qrot(d.rot[a], mk(S.p1[k])) + ca, pb = qrot(d.rot[b], mk(S.p2[k])) + cb;
            const float4 par = S.par[k];
            const f3 diff = pb - pa;
            const float dist = mag(diff);
            const f3 dir = dist != 0.f ? normalize(diff) : mk(0.f, -1.f, 0.f);
            const float expand = par.y * (dist - par.z);
            impulse_at(d, a, dir * (expand * dt), pa);
            impulse_at(d, b, -dir * (expand * dt), pb);
            const f3 rA = pa - ca, rB = pb - cb;
            const float ima = d.pos[a].w, imb = d.pos[b].w;
            const f3 rdA = mul(load9(d.iinv + 9 * a), cross(dir, rA));
            const f3 rdB = mul(load9(d.iinv + 9 * b), cross(dir, rB));
            const float sens = 1.0f / (ima + imb + dot(cross(rA, rdA), dir) + dot(cross(rB, rdB), dir));
            const f3 va = mk(d.vel[a]), wa = mk(d.angv[a]), vb = mk(d.vel[b]), wb = mk(d.angv[b]);
            const float velocity = dot(vb + cross(wb, pa - cb), dir) - dot(va + cross(wa, pb - ca), dir);
            float dampen = par.x * velocity;
            const float max_dampen = velocity * sens / dt;
            if (velocity > 0.f && dampen > max_dampen) dampen = max_dampen;
            else if (velocity < 0.f && dampen < max_dampen) dampen = max_dampen;
            impulse_at(d, a, dir * (dampen * dt), pa);
            impulse_at(d, b, -dir * (dampen * dt), pb);
        }
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

void launch_springs(const Dev& d, const Launch& L) {
    if (d.sp.n == 0) return;
    int g = (d.n_worlds + 127) / 128;
    g = g > L.n_sms * 8 ? L.n_sms * 8 : g;
    k_springs<<<g, 128, 0, L.st>>>(d);
}

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
