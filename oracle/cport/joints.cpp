// joints.cpp — ball-socket and hinge rows and the holonomic block solver of the
// CPU restatement (test infrastructure; see cport.h).
#include "cport.h"

namespace cport {

// ------------------------------------------------------------- rows ----
// rowMajorOrderInverse<n> for n >= 4 (Math/src/NMat.h:124-149): Gauss-Jordan
// elimination without pivoting
static void gaussJordan(int n, const double* src, double* dst) {
    double c[kMaxDof * kMaxDof * 2];
    for (int i = 0; i < n * n; i++) c[i] = src[i];
    for (int i = 0; i < n * n; i++) dst[i] = 0;
    for (int i = 0; i < n; i++) dst[i * (n + 1)] = 1.0;
    for (int piv = 0; piv < n; piv++)
        for (int r = 0; r < n; r++) {
            if (piv == r) continue;
            double ratio = c[n * r + piv] / c[n * piv + piv];
            for (int k = 0; k < n; k++) {
                c[n * r + k] -= ratio * c[n * piv + k];
                dst[n * r + k] -= ratio * dst[n * piv + k];
            }
        }
    for (int piv = 0; piv < n; piv++)
        for (int k = 0; k < n; k++) dst[n * piv + k] /= c[n * piv + piv];
}

// rowMajorOrderInverse<n> (NMat.cpp:5-34 for n <= 3), in place allowed
static void invertBlock(int n, double* m) {
    double out[kMaxDof * kMaxDof];
    if (n == 1) { out[0] = 1.0 / m[0]; }
    else if (n == 2) {
        double a = m[0], b = m[1], c = m[2], d = m[3];
        double di = 1.0 / (a * d - b * c);
        out[0] = d * di; out[1] = -b * di; out[2] = -c * di; out[3] = a * di;
    } else if (n == 3) {
        double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
        double di = 1.0 / (a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g));
        out[0] = (e * i - f * h) * di; out[1] = (c * h - b * i) * di; out[2] = (b * f - c * e) * di;
        out[3] = (f * g - d * i) * di; out[4] = (a * i - c * g) * di; out[5] = (c * d - a * f) * di;
        out[6] = (d * h - e * g) * di; out[7] = (b * g - a * h) * di; out[8] = (a * e - b * d) * di;
    } else {
        gaussJordan(n, m, out);
    }
    for (int k = 0; k < n * n; k++) m[k] = out[k];
}

static void crossMatInto(const V3& v, double m[3][3]) {   // crossMat (NMat.cpp:59-67)
    m[0][0] = 0; m[0][1] = -v.z; m[0][2] = v.y;
    m[1][0] = v.z; m[1][1] = 0; m[1][2] = -v.x;
    m[2][0] = -v.y; m[2][1] = v.x; m[2][2] = 0;
}

// (1x3 row) * (3x3) as NMat<1,3> * NMat<3,3> accumulates it
static void rowTimes(const double v[3], const double m[3][3], double out[3]) {
    for (int k = 0; k < 3; k++) {
        double x = 0;
        for (int q = 0; q < 3; q++) x += v[q] * m[q][k];
        out[k] = x;
    }
}

// angle * axis of b * conj(a) (Quaternion::angleTo, Quaternion.h:35-39, and
// getRotAxis, :41-49), the axis scaled by `c`; the orientation error of the
// weld and slider rows
static V3 orientationError(const Q& qa, const Q& qb, double c) {
    Q dq = qb * qa.conj();
    double dot = std::fabs(qa.r * qb.r + qa.i * qb.i + qa.j * qb.j + qa.k * qb.k);
    double angle = dot > 0.99999999999 ? 0.0 : 2 * std::acos(std::fabs(qa.r * qb.r + qa.i * qb.i + qa.j * qb.j + qa.k * qb.k));
    V3 axis;
    if (angle != 0) {
        V3 raw(dq.i, dq.j, dq.k);
        axis = (dq.r < 0 ? -raw.normalize() : raw.normalize()) * c;
    }
    return angle * axis;
}

// impulse_to_{a,b}_velocity = invMass(body) * J^T, impulse_to_value and its
// CFM-regularised inverse (ConstraintSolver.cpp:255-258 pattern)
static void finishRow(JRow& r, double cfm) {
    const int n = r.n;
    for (int side = 0; side < 2; side++) {
        const Body* body = side == 0 ? r.a : r.b;
        double (*j)[6] = side == 0 ? r.ja : r.jb;
        double (*it)[kMaxDof] = side == 0 ? r.ita : r.itb;
        double im[6][6] = {};
        double m = body->invMass();
        M3 t = body->invTensor();
        for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) { im[i][k] = (i == k ? 1.0 : 0.0) * m; im[3 + i][3 + k] = t.m[i][k]; }
        for (int i = 0; i < 6; i++)
            for (int c = 0; c < n; c++) {
                it[i][c] = 0;
                for (int k = 0; k < 6; k++) it[i][c] += im[i][k] * j[c][k];
            }
    }
    for (int i = 0; i < n; i++)
        for (int c = 0; c < n; c++) {
            double pa = 0, pb = 0;
            for (int k = 0; k < 6; k++) pa += r.ja[i][k] * r.ita[k][c];
            for (int k = 0; k < 6; k++) pb += r.jb[i][k] * r.itb[k][c];
            r.itv[i][c] = pa + pb;
        }
    double m[kMaxDof * kMaxDof];
    for (int i = 0; i < n; i++) for (int c = 0; c < n; c++) m[i * n + c] = r.itv[i][c];
    for (int i = 0; i < n; i++) m[i * n + i] *= (1 + cfm);   // applyCFM (ConstraintSolver.cpp:919-926)
    invertBlock(n, m);
    for (int i = 0; i < n; i++) for (int c = 0; c < n; c++) r.minv[i][c] = m[i * n + c];
}

// BallSocket::updateSolverConstraints (PersistentConstraint.cpp:225-231) with
// the BallSocketConstraint constructor (ConstraintSolver.cpp:382-405), and
// Hinge::updateSolverConstraints (:274-285) with HingeConstraint
// (ConstraintSolver.cpp:468-550).  The hinge's rB is taken from body 1's
// anchor point, as the reference's constructor does.
// Motor::calculatePosition (PersistentConstraint.cpp:30-71): the last angle
// advanced by the relative angular velocity, snapped to the angle of body 2's
// comparison axis in body 1's (u, w) plane (in the 2 pi window nearest the
// prediction) unless that axis is within acos(0.999) of the motor axis
double Joint::motorPosition(const V3& axis, const V3& w1, const V3& w2, double dts) const {
    V3 ref_axis_u = b1->q.rotate(ref_u);
    V3 ref_axis_w = b1->q.rotate(ref_w);
    V3 compare_axis = b2->q.rotate(cmp);
    double rel = axis.dot(w1) - axis.dot(w2);
    double pred = position + rel * dts;
    if (std::abs(compare_axis.dot(axis)) > 0.999) return pred;
    V3 cn = (compare_axis - axis * axis.dot(compare_axis)).normalize();
    double dv = cn.dot(ref_axis_u);
    if (dv > 1.0) dv = 1.0;
    if (dv < -1.0) dv = -1.0;
    double rel_angle = 2 * PI_TRUNC - std::acos(dv);
    if (cn.dot(ref_axis_w) < 0) rel_angle = 2 * PI_TRUNC - rel_angle;
    double r = std::fmod(pred, 2 * PI_TRUNC);
    double n2 = pred - r;
    const double cands[3] = {n2 + rel_angle - 2 * PI_TRUNC, n2 + rel_angle, n2 + rel_angle + 2 * PI_TRUNC};
    double closest = std::numeric_limits<double>::infinity();
    for (double c : cands)
        if (std::abs(pred - c) < std::abs(pred - closest)) closest = c;
    return closest;
}

// Motor::getConstraintTargetVelocityValue (PersistentConstraint.cpp:77-109):
// off 0, constant torque an infinite target in the torque's direction, target
// velocity as set, target position the velocity that a constant max torque
// reaches over the remaining angle, the inertia estimated from the last
// impulse and velocity change (or from the inverse tensors when either is
// below 1e-7; the reference tests `abs(impulse < EPS)`, true for every
// impulse below 1e-7, negative ones included)
double Joint::motorTargetVelocity(const V3& axis, const V3& w1, const V3& w2) const {
    switch (mode) {
        case 0: return 0;
        case 1: return power_max > 0 ? std::numeric_limits<double>::infinity() : -std::numeric_limits<double>::infinity();
        case 2: return target_vel;
        default: {
            double ang_diff = position - target_pos;
            double dir = (ang_diff > 0) ? -1 : 1;
            double vdt = std::abs((axis.dot(w1) - axis.dot(w2)) - prev_vel);
            const double EPS = 0.0000001;
            double inertia;
            if (vdt < EPS || row.impulse[0] < EPS)
                inertia = 1.0 / (axis.dot(b1->invTensor() * axis) + axis.dot(b2->invTensor() * axis));
            else
                inertia = std::abs(row.impulse[0]) / vdt;
            return dir * std::sqrt(2 * std::abs(ang_diff) * power_max / inertia);
        }
    }
}

// Piston::getPistonTargetVelocityValue (PersistentConstraint.cpp:153-185), the
// same with the inverse masses; the piston's previous velocity is never
// written (writePrevVel has no caller) and stays 0
double Joint::pistonTargetVelocity(const V3& axis) const {
    switch (mode) {
        case 0: return 0;
        case 1: return power_max > 0 ? std::numeric_limits<double>::infinity() : -std::numeric_limits<double>::infinity();
        case 2: return target_vel;
        default: {
            double ang_diff = position - target_pos;
            double dir = (ang_diff > 0) ? -1 : 1;
            double vdt = std::abs((axis.dot(b1->getVel()) - axis.dot(b2->getVel())) - prev_vel);
            const double EPS = 0.0000001;
            double inertia;
            if (vdt < EPS || row.impulse[0] < EPS) inertia = 1.0 / (b1->invMass() + b2->invMass());
            else inertia = std::abs(row.impulse[0]) / vdt;
            return dir * std::sqrt(2 * std::abs(ang_diff) * power_max / inertia);
        }
    }
}

void Joint::rebuild(const Params& p, double dts, bool in_holo) {
    if (motor) {
        // Motor::updateSolverConstraints (PersistentConstraint.cpp:320-328) with
        // the MotorConstraint constructor (ConstraintSolver.cpp:555-585): the
        // angle advanced first; while active one row on body 1's axis, its
        // target velocity limited to the limit's side and a one-sided
        // projection past a limit, else bounded by max torque x dt; the old
        // row is kept while inactive
        V3 axis = b1->q.rotate(ax1);
        V3 w1 = b1->getAngVel(), w2 = b2->getAngVel();
        position = motorPosition(axis, w1, w2, dts);
        const double start = p.warm_start_disabled ? 0.0 : 1.0 * row.impulse[0];
        if (listed()) {
            const double tv = 1.0 * motorTargetVelocity(axis, w1, w2);
            const double hard = std::min<double>(rot_hard * dts, 1.0 / dts);
            JRow r;
            r.n = 1; r.a = b1; r.b = b2;
            r.impulse[0] = start;
            const double ad[3] = {axis.x, axis.y, axis.z};
            for (int k = 0; k < 3; k++) {
                r.ja[0][k] = 0; r.ja[0][3 + k] = ad[k];
                r.jb[0][k] = 0; r.jb[0][3 + k] = -ad[k];
            }
            r.has_vt = true;
            if (position > lim_max) {
                r.ptarget[0] = (lim_max - position) * hard;
                r.vt = std::min<double>(0, tv);
                r.proj = 2;
            } else if (position < lim_min) {
                r.ptarget[0] = (lim_min - position) * hard;
                r.vt = std::max<double>(0, tv);
                r.proj = 1;
            } else {
                r.ptarget[0] = 0;
                r.vt = tv;
                r.proj = 3;
                r.lim = std::abs(power_max * dts);
                r.pos = false;
            }
            finishRow(r, p.cfm);
            row = r;
        }
        prev_vel = axis.dot(w1) - axis.dot(w2);
        return;
    }
    if (slide_limit || piston) {
        // Piston::updateSolverConstraints (PersistentConstraint.cpp:300-318):
        // the slide position along body 1's axis between the slider's tracked
        // points; past a limit a SlideLimitConstraint row (ConstraintSolver.cpp:
        // 736-775), while powered a PistonConstraint row (:701-731), both along
        // the axis (their angular Jacobian, -s^T [s]x, is zero)
        V3 pa = b1->trackedP(k1), pb = b2->trackedP(k2);
        V3 axis = b1->q.rotate(ax1);
        position = pb.dot(axis) - pa.dot(axis);
        exceeded = position < lim_min || position > lim_max;
        if (!listed()) return;
        const double start = p.warm_start_disabled ? 0.0 : 1.0 * row.impulse[0];
        JRow r;
        r.n = 1; r.a = b1; r.b = b2;
        r.impulse[0] = start;
        const double sd[3] = {axis.x, axis.y, axis.z}, nsd[3] = {-axis.x, -axis.y, -axis.z};
        double sx[3][3], ang[3];
        crossMatInto(axis, sx);
        rowTimes(nsd, sx, ang);
        for (int k = 0; k < 3; k++) {
            r.ja[0][k] = -sd[k]; r.ja[0][3 + k] = ang[k];
            r.jb[0][k] = sd[k]; r.jb[0][3 + k] = 0;
        }
        if (slide_limit) {
            const double hard = std::min<double>(pos_hard * dts, 1.0 / dts);
            if (position > lim_max) { r.ptarget[0] = (lim_max - position) * hard; r.proj = 2; }
            else { r.ptarget[0] = (lim_min - position) * hard; r.proj = 1; }
        } else {
            r.has_vt = true;
            r.vt = pistonTargetVelocity(axis);
            r.proj = 3;
            r.lim = power_max * dts;
            r.pos = false;
        }
        finishRow(r, p.cfm);
        row = r;
        return;
    }
    if (cone) {
        // ConeRotationLimit::updateSolverConstraints (PersistentConstraint.cpp:233-247)
        // with ConeLimitConstraint (ConstraintSolver.cpp:410-432): inactive
        // inside the cone (warm impulse cleared, the old row kept); else one
        // row on the axis across both directions, error from the 8th-order
        // series of 1 - cos(angle - limit) times the raw strength, warm
        // impulse passed on unscaled
        V3 d1 = b1->q.rotate(ax1), d2 = b2->q.rotate(ax2);
        double cur = std::acos(d1.dot(d2));
        inactive = cur < max_angle;
        if (inactive) { row.impulse[0] = 0.0; return; }
        JRow r;
        r.n = 1; r.a = b1; r.b = b2; r.proj = 1;
        r.impulse[0] = row.impulse[0];
        V3 h = d1.cross(d2).normalize();
        const double hd[3] = {h.x, h.y, h.z};
        for (int k = 0; k < 3; k++) {
            r.ja[0][k] = 0; r.ja[0][3 + k] = hd[k];
            r.jb[0][k] = 0; r.jb[0][3 + k] = -hd[k];
        }
        double f = cur - max_angle;
        double err = -f * f * f * f * f * f * f * f / 40320.0 + f * f * f * f * f * f / 720.0 - f * f * f * f / 24.0 + f * f / 2.0;
        r.ptarget[0] = err * rot_hard;
        finishRow(r, p.cfm);
        row = r;
        return;
    }
    if (twist) {
        // TwistLimit::updateSolverConstraints (PersistentConstraint.cpp:249-272),
        // getCurrentAngle (:115-131: the angle of b1's w axis carried by body 2,
        // measured in b1's (w, u) frame and unwrapped against the last
        // value; the reference's alignment rotation there is unused) and
        // TwistLimitConstraint (ConstraintSolver.cpp:439-466)
        M3 r1 = b1->q.rotMatrix(), r2 = b2->q.rotMatrix();
        V3 t1 = r1 * ax1, u1 = r1 * u_local, w1 = r1 * w_local;
        V3 t2 = r2 * ax2, r2w = r2 * w_local;
        double prev = cur_angle;
        double a = std::atan2(r2w.dot(u1), r2w.dot(w1));
        while (prev - a > PI_TRUNC) a += 2 * PI_TRUNC;
        while (prev - a < -PI_TRUNC) a -= 2 * PI_TRUNC;
        cur_angle = a;
        inactive = min_angle <= a && a <= max_angle;
        if (inactive) { row.impulse[0] = 0.0; return; }
        const bool above = a > max_angle;
        JRow r;
        r.n = 1; r.a = b1; r.b = b2; r.proj = above ? 2 : 1;
        r.impulse[0] = row.impulse[0];
        const double ta[3] = {t1.x, t1.y, t1.z}, tb[3] = {t2.x, t2.y, t2.z};
        for (int k = 0; k < 3; k++) {
            r.ja[0][k] = 0; r.ja[0][3 + k] = -ta[k];
            r.jb[0][k] = 0; r.jb[0][3 + k] = tb[k];
        }
        double f = above ? a - max_angle : min_angle - a;
        double err = -f * f * f * f * f * f * f * f / 40320.0 + f * f * f * f * f * f / 720.0 - f * f * f * f / 24.0 + f * f / 2.0;
        r.ptarget[0] = err * rot_hard;
        finishRow(r, p.cfm);
        row = r;
        return;
    }
    V3 pa = b1->trackedP(k1), pb = b2->trackedP(k2);
    double warm[kMaxDof] = {};
    for (int i = 0; i < n; i++) warm[i] = p.warm_start_disabled ? 0.0 : 1.0 * row.impulse[i];
    // Weld::updateSolverConstraints (PersistentConstraint.cpp:344-353) hands
    // the previous impulse to the constructor unscaled, whatever the
    // warm-start switch says
    if (n == 6) for (int i = 0; i < n; i++) warm[i] = row.impulse[i];
    double pos_c = std::min<double>(pos_hard * dts, 1.0 / dts);
    JRow r;
    r.n = n; r.a = b1; r.b = b2; r.in_holo = in_holo;
    for (int i = 0; i < n; i++) r.impulse[i] = warm[i];
    V3 rA = pa - b1->com;
    double sa[3][3], sb[3][3];
    crossMatInto(rA, sa);
    if (n == 1) {
        // Distance::updateSolverConstraints (PersistentConstraint.cpp:217-223)
        // with the DistanceConstraint constructor (ConstraintSolver.cpp:348-377):
        // one row along the attachment direction, position error target - |d|
        V3 rB = pb - b2->com;
        crossMatInto(rB, sb);
        V3 diff = pa - pb;
        V3 dd = diff.normalize();
        const double dv[3] = {dd.x, dd.y, dd.z};
        for (int k = 0; k < 3; k++) {
            double ta = 0, tb = 0;
            for (int i = 0; i < 3; i++) { ta += (-dv[i]) * sa[i][k]; tb += dv[i] * sb[i][k]; }
            r.ja[0][k] = dv[k];
            r.ja[0][3 + k] = ta;
            r.jb[0][k] = -dv[k];
            r.jb[0][3 + k] = tb;
        }
        double error = diff.mag2() < 0.00001 ? target : target - diff.normalize().dot(diff);
        r.ptarget[0] = pos_c * error;
    } else if (n == 3) {
        V3 rB = pb - b2->com;
        crossMatInto(rB, sb);
        for (int i = 0; i < 3; i++) {
            for (int k = 0; k < 3; k++) {
                r.ja[i][k] = (i == k) ? 1.0 : 0.0;
                r.ja[i][3 + k] = -sa[i][k];
                r.jb[i][k] = -((i == k) ? 1.0 : 0.0);
                r.jb[i][3 + k] = sb[i][k];
            }
        }
        V3 err = pb - pa;
        r.ptarget[0] = pos_c * err.x; r.ptarget[1] = pos_c * err.y; r.ptarget[2] = pos_c * err.z;
    } else if (n == 6) {
        // WeldConstraint (ConstraintSolver.cpp:861-899): the ball-socket rows
        // plus three rows locking the relative angular velocity; position
        // error (pb - pa), orientation error angle * axis of b * conj(a)
        V3 rB = pb - b2->com;
        crossMatInto(rB, sb);
        for (int i = 0; i < 3; i++) {
            for (int k = 0; k < 3; k++) {
                double id = (i == k) ? 1.0 : 0.0;
                r.ja[i][k] = id;
                r.ja[i][3 + k] = -sa[i][k];
                r.jb[i][k] = -id;
                r.jb[i][3 + k] = sb[i][k];
                r.ja[3 + i][k] = 0;
                r.ja[3 + i][3 + k] = id;
                r.jb[3 + i][k] = 0;
                r.jb[3 + i][3 + k] = -id;
            }
        }
        double rot_c = std::min<double>(rot_hard * dts, 1.0 / dts);
        V3 pc = (pb - pa) * pos_c;
        V3 rc = orientationError(b1->q, b2->q, rot_c);
        r.ptarget[0] = pc.x; r.ptarget[1] = pc.y; r.ptarget[2] = pc.z;
        r.ptarget[3] = rc.x; r.ptarget[4] = rc.y; r.ptarget[5] = rc.z;
    } else if (n == 5 && slider) {
        // Slider::updateSolverConstraints (PersistentConstraint.cpp:287-298)
        // with SliderConstraint (ConstraintSolver.cpp:611-696): two rows
        // across the slide axis (u, w of body 1's axis) and three locking the
        // relative rotation.  The reference hands the position coefficient
        // to the orientation rows as well.
        V3 rB = pb - b2->com;
        crossMatInto(rB, sb);
        V3 ax = b1->q.rotate(ax1).normalize();
        V3 uu, ww;
        ax.perpBasis(&uu, &ww);
        r.impulse[0] = uu.dot(u) * warm[0] + uu.dot(w) * warm[1];
        r.impulse[1] = ww.dot(u) * warm[0] + ww.dot(w) * warm[1];
        V3 pe = pa - pb;
        double us[3][3], ws[3][3];
        crossMatInto(uu, us); crossMatInto(ww, ws);
        const double ud[3] = {uu.x, uu.y, uu.z}, wd[3] = {ww.x, ww.y, ww.z}, ped[3] = {pe.x, pe.y, pe.z};
        const double nud[3] = {-uu.x, -uu.y, -uu.z}, nwd[3] = {-ww.x, -ww.y, -ww.z};
        double t0[3], t1[3], t2[3], t3[3], t4[3], t5[3];
        rowTimes(nud, sa, t0); rowTimes(ped, us, t1); rowTimes(ud, sb, t2);
        rowTimes(nwd, sa, t3); rowTimes(ped, ws, t4); rowTimes(wd, sb, t5);
        for (int k = 0; k < 3; k++) {
            r.ja[0][k] = ud[k];  r.ja[0][3 + k] = t0[k] - t1[k];
            r.jb[0][k] = -ud[k]; r.jb[0][3 + k] = t2[k];
            r.ja[1][k] = wd[k];  r.ja[1][3 + k] = t3[k] - t4[k];
            r.jb[1][k] = -wd[k]; r.jb[1][3 + k] = t5[k];
            for (int i = 0; i < 3; i++) {
                double id = (i == k) ? 1.0 : 0.0;
                r.ja[2 + i][k] = 0; r.ja[2 + i][3 + k] = id;
                r.jb[2 + i][k] = 0; r.jb[2 + i][3 + k] = -id;
            }
        }
        V3 rc = orientationError(b1->q, b2->q, pos_c);
        r.ptarget[0] = -pe.dot(uu) * pos_c;
        r.ptarget[1] = -pe.dot(ww) * pos_c;
        r.ptarget[2] = rc.x; r.ptarget[3] = rc.y; r.ptarget[4] = rc.z;
        u = uu;
        w = ww;
    } else if (n == 4) {
        // SlidingHinge::updateSolverConstraints (PersistentConstraint.cpp:331-342)
        // with SlidingHingeConstraint (ConstraintSolver.cpp:781-852): two rows
        // across body 2's axis and two keeping body 1's axis parallel to it
        V3 rB = pb - b2->com;
        crossMatInto(rB, sb);
        V3 na = b1->q.rotate(ax1), nb = b2->q.rotate(ax2);
        V3 uu, ww;
        nb.perpBasis(&uu, &ww);
        r.impulse[2] = uu.dot(u) * warm[2] + uu.dot(w) * warm[3];
        r.impulse[3] = ww.dot(u) * warm[2] + ww.dot(w) * warm[3];
        V3 pd = pa - pb;
        double us[3][3], ws[3][3], ns[3][3];
        crossMatInto(uu, us); crossMatInto(ww, ws); crossMatInto(na, ns);
        const double ud[3] = {uu.x, uu.y, uu.z}, wd[3] = {ww.x, ww.y, ww.z}, pdd[3] = {pd.x, pd.y, pd.z};
        const double nud[3] = {-uu.x, -uu.y, -uu.z}, nwd[3] = {-ww.x, -ww.y, -ww.z}, nnd[3] = {-na.x, -na.y, -na.z};
        double a0[3], b0a[3], b0b[3], a1[3], b1a[3], b1b[3], a2[3], b2r[3], a3[3], b3r[3];
        rowTimes(nud, sa, a0); rowTimes(ud, sb, b0a); rowTimes(pdd, us, b0b);
        rowTimes(nwd, sa, a1); rowTimes(wd, sb, b1a); rowTimes(pdd, ws, b1b);
        rowTimes(nud, ns, a2); rowTimes(nnd, us, b2r);
        rowTimes(nwd, ns, a3); rowTimes(nnd, ws, b3r);
        for (int k = 0; k < 3; k++) {
            r.ja[0][k] = ud[k];  r.ja[0][3 + k] = a0[k];
            r.jb[0][k] = -ud[k]; r.jb[0][3 + k] = b0a[k] - b0b[k];
            r.ja[1][k] = wd[k];  r.ja[1][3 + k] = a1[k];
            r.jb[1][k] = -wd[k]; r.jb[1][3 + k] = b1a[k] - b1b[k];
            r.ja[2][k] = 0; r.ja[2][3 + k] = a2[k];
            r.jb[2][k] = 0; r.jb[2][3 + k] = b2r[k];
            r.ja[3][k] = 0; r.ja[3][3 + k] = a3[k];
            r.jb[3][k] = 0; r.jb[3][3 + k] = b3r[k];
        }
        double rot_c = std::min<double>(rot_hard * dts, 1.0 / dts);
        r.ptarget[0] = -uu.dot(pd) * pos_c;
        r.ptarget[1] = -ww.dot(pd) * pos_c;
        r.ptarget[2] = -uu.dot(na) * rot_c;
        r.ptarget[3] = -ww.dot(na) * rot_c;
        u = uu;
        w = ww;
    } else {
        V3 rB = pa - b2->com;
        crossMatInto(rB, sb);
        V3 h1 = b1->q.rotate(ax1), h2 = b2->q.rotate(ax2);
        double rot_c = std::min<double>(rot_hard * dts, 1.0 / dts);
        V3 uu, ww;
        h1.perpBasis(&uu, &ww);
        V3 nn = h2;
        r.impulse[3] = uu.dot(u) * warm[3] + uu.dot(w) * warm[4];
        r.impulse[4] = ww.dot(u) * warm[3] + ww.dot(w) * warm[4];
        for (int i = 0; i < 3; i++) {
            for (int k = 0; k < 3; k++) {
                r.ja[i][k] = (i == k) ? 1.0 : 0.0;
                r.ja[i][3 + k] = -sa[i][k];
                r.jb[i][k] = -((i == k) ? 1.0 : 0.0);
                r.jb[i][3 + k] = sb[i][k];
            }
        }
        double us[3][3], ws[3][3], ns[3][3];
        crossMatInto(uu, us); crossMatInto(ww, ws); crossMatInto(nn, ns);
        const double ud[3] = {uu.x, uu.y, uu.z}, wd[3] = {ww.x, ww.y, ww.z}, nd[3] = {nn.x, nn.y, nn.z};
        for (int k = 0; k < 3; k++) {
            double a3 = 0, b3 = 0, a4 = 0, b4 = 0;
            for (int q = 0; q < 3; q++) {
                a3 += nd[q] * us[q][k];
                b3 += ud[q] * ns[q][k];
                a4 += nd[q] * ws[q][k];
                b4 += wd[q] * ns[q][k];
            }
            r.ja[3][k] = 0; r.jb[3][k] = 0; r.ja[4][k] = 0; r.jb[4][k] = 0;
            r.ja[3][3 + k] = a3; r.jb[3][3 + k] = b3;
            r.ja[4][3 + k] = a4; r.jb[4][3 + k] = b4;
        }
        V3 pc = (pb - pa) * pos_c;
        r.ptarget[0] = pc.x; r.ptarget[1] = pc.y; r.ptarget[2] = pc.z;
        r.ptarget[3] = uu.dot(nn) * rot_c;
        r.ptarget[4] = ww.dot(nn) * rot_c;
        u = uu;
        w = ww;
    }
    finishRow(r, p.cfm);
    row = r;
}

// J_a v_a + J_b v_b (NMat * NVec, then NVec + NVec)
static void jrowValue(const JRow& r, const Vec<6>& va, const Vec<6>& vb, double* out) {
    for (int i = 0; i < r.n; i++) {
        double x = 0, y = 0;
        for (int k = 0; k < 6; k++) x += va.v[k] * r.ja[i][k];
        for (int k = 0; k < 6; k++) y += vb.v[k] * r.jb[i][k];
        out[i] = x + y;
    }
}

// computeAndApplyVelocityChange (ConstraintSolver.h:72-75)
void jrowApply(const JRow& r, const double* imp, Vec<6>* va, Vec<6>* vb) {
    for (int k = 0; k < 6; k++) {
        double x = 0;
        for (int i = 0; i < r.n; i++) x += imp[i] * r.ita[k][i];
        va->v[k] += x;
    }
    for (int k = 0; k < 6; k++) {
        double x = 0;
        for (int i = 0; i < r.n; i++) x += imp[i] * r.itb[k][i];
        vb->v[k] += x;
    }
}

static bool isZero(const double* x, int n) {
    for (int i = 0; i < n; i++) if (std::abs(x[i]) > 0.00000001) return false;
    return true;
}

// DegreedConstraint::findTargetConstraintValue (ConstraintSolver.h:79)
void jrowTarget(JRow& r) {
    Vec<6> va, vb;
    V3 v = r.a->getVel(), w = r.a->getAngVel();
    va.v[0] = v.x; va.v[1] = v.y; va.v[2] = v.z; va.v[3] = w.x; va.v[4] = w.y; va.v[5] = w.z;
    v = r.b->getVel(); w = r.b->getAngVel();
    vb.v[0] = v.x; vb.v[1] = v.y; vb.v[2] = v.z; vb.v[3] = w.x; vb.v[4] = w.y; vb.v[5] = w.z;
    double cur[kMaxDof];
    jrowValue(r, va, vb, cur);
    // MotorConstraint / PistonConstraint::findTargetConstraintValue
    // (ConstraintSolver.cpp:586-589, 723-726): the target velocity less the value
    if (r.has_vt) r.target[0] = r.vt - cur[0];
    else for (int i = 0; i < r.n; i++) r.target[i] = -cur[i];
}

void jrowWarm(JRow& r) {
    if (!isZero(r.impulse, r.n)) jrowApply(r, r.impulse, &r.da->v, &r.db->v);
}

// PGSConstraintStep<n> (ConstraintSolver.cpp:12-40) for an equality row
void jrowStep(JRow& r, bool pseudo) {
    Vec<6>* va = pseudo ? &r.da->pv : &r.da->v;
    Vec<6>* vb = pseudo ? &r.db->pv : &r.db->v;
    double* acc = pseudo ? r.pimpulse : r.impulse;
    const double* tgt = pseudo ? r.ptarget : r.target;
    double cur[kMaxDof], delta[kMaxDof], diff[kMaxDof];
    jrowValue(r, *va, *vb, cur);
    for (int i = 0; i < r.n; i++) delta[i] = tgt[i] - cur[i];
    for (int i = 0; i < r.n; i++) {
        double x = 0;
        for (int k = 0; k < r.n; k++) x += delta[k] * r.minv[i][k];
        double nw = acc[i] + x;
        // ConeLimitConstraint / TwistLimitConstraint::projectValidImpulse
        // (ConstraintSolver.cpp:434-436, 463-465)
        if (r.proj == 1) nw = std::max<double>(nw, 0);
        else if (r.proj == 2) nw = std::min<double>(nw, 0);
        // MotorConstraint / PistonConstraint::projectValidImpulse (ConstraintSolver.cpp:591-606, 728-731)
        else if (r.proj == 3) nw = nw > 0 ? std::min<double>(nw, r.lim) : std::max<double>(nw, -r.lim);
        diff[i] = nw - acc[i];
    }
    if (!isZero(diff, r.n)) {
        jrowApply(r, diff, va, vb);
        for (int i = 0; i < r.n; i++) acc[i] += diff[i];
    }
}

// ------------------------------------------------- holonomic system ----
static const int kEmpty = -1;

void HoloSys::build(const std::vector<JRow*>& og) {
    cons.clear(); table.clear(); vpos.clear(); buf.clear();
    degree = 0; cap = 0;
    const int n = (int)og.size();
    if (n == 0) return;
    std::vector<char> edge((size_t)n * n, 0), empty((size_t)n * n, 1);
    auto E = [&](int i, int j) -> char& { return edge[(size_t)i + (size_t)j * n]; };
    auto shares = [](const JRow* x, const JRow* y) { return x->a == y->a || x->a == y->b || x->b == y->a || x->b == y->b; };
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            if (shares(og[i], og[j])) {
                empty[(size_t)i * n + j] = 0; empty[(size_t)j * n + i] = 0;
                E(i, j) = 1; E(j, i) = 1;
            }
        }
    std::vector<int> remaining(n);
    for (int i = 0; i < n; i++) remaining[i] = i;
    std::vector<int> order;
    while (!remaining.empty()) {
        int best_i = -1, best_count = std::numeric_limits<int>::max();
        std::vector<int> best_nb;
        for (int i = 0; i < (int)remaining.size(); i++) {
            std::vector<int> nb;
            for (int j = 0; j < n; j++)
                if (j != remaining[i] && E(remaining[i], j)) nb.push_back(j);
            int unconnected = 0;
            for (size_t a = 0; a < nb.size(); a++)
                for (size_t b = a + 1; b < nb.size(); b++)
                    if (!E(nb[a], nb[b])) unconnected++;
            if (unconnected < best_count) {
                best_count = unconnected;
                best_i = i;
                best_nb = nb;
                if (unconnected == 0) break;
            }
        }
        int x = remaining[best_i];
        order.push_back(x);
        remaining.erase(remaining.begin() + best_i);
        for (int j = 0; j < n; j++) { E(x, j) = 0; E(j, x) = 0; }
        for (size_t a = 0; a < best_nb.size(); a++)
            for (size_t b = a + 1; b < best_nb.size(); b++) {
                int p = best_nb[a], q = best_nb[b];
                empty[(size_t)p * n + q] = 0; empty[(size_t)q * n + p] = 0;
                E(p, q) = 1; E(q, p) = 1;
            }
    }
    for (int x : order) cons.push_back(og[x]);
    for (int col = 0; col < n; col++) {
        vpos.push_back(degree);
        degree += cons[col]->n;
        for (int row = col; row < n; row++) {
            if (empty[(size_t)order[row] * n + order[col]]) table.push_back(kEmpty);
            else { table.push_back(cap); cap += cons[row]->n * cons[col]->n; }
        }
    }
    dcap = 6 * degree;
    buf.assign((size_t)cap + dcap, 0.0);
}

int HoloSys::loc(int row, int col) const {   // getBlockBufferLocation (:584-595)
    int n = (int)cons.size();
    return table[row - col + ((2 * n + 1) * col - col * col) / 2];
}
int HoloSys::firstBelow(int col) const {
    for (int r = col + 1; r < (int)cons.size(); r++) { int l = loc(r, col); if (l != kEmpty) return l; }
    return kEmpty;
}
int HoloSys::dloc(int row, int col) const {
    int l = loc(row, col);
    if (l == kEmpty) return kEmpty;
    return l - firstBelow(col);
}

static double dotN(int n, const double* a, const double* b) {
    double o = 0;
    for (int i = 0; i < n; i++) o += a[i] * b[i];
    return o;
}

// computeBlockInitialValue (HolonomicBlockSolver.cpp:731-760): the diagonal
// block is impulse_to_value with CFM; an off-diagonal block couples through
// the first shared body in the order (a,a), (a,b), (b,a), (b,b)
static void initialBlock(double* t, const JRow* c1, const JRow* c2, double cfm) {
    if (c1 == c2) {
        int n = c1->n;
        for (int i = 0; i < n; i++) for (int j = 0; j < n; j++) t[i * n + j] = c1->itv[i][j];
        for (int i = 0; i < n; i++) t[i + n * i] *= (1 + cfm);
        return;
    }
    const double (*j)[6] = nullptr;
    const double (*it)[kMaxDof] = nullptr;
    if (c1->a == c2->a) { j = c1->ja; it = c2->ita; }
    else if (c1->a == c2->b) { j = c1->ja; it = c2->itb; }
    else if (c1->b == c2->a) { j = c1->jb; it = c2->ita; }
    else if (c1->b == c2->b) { j = c1->jb; it = c2->itb; }
    for (int i = 0; i < c1->n * c2->n; i++) {
        int r = i / c2->n, c = i % c2->n;
        t[i] = 0;
        if (j) for (int k = 0; k < 6; k++) t[i] += j[r][k] * it[k][c];
    }
}

// HolonomicSystem::computeInverse (HolonomicBlockSolver.cpp:427-543): block
// LDL^T with the diagonal blocks inverted in place and L = A D^-1
void HoloSys::computeInverse(double cfm) {
    const int n = (int)cons.size();
    double* B = buf.data();
    double* Dg = buf.data() + cap;
    for (int col = 0; col < n; col++)
        for (int row = col; row < n; row++) {
            int l = loc(row, col);
            if (l == kEmpty) continue;
            initialBlock(B + l, cons[row], cons[col], cfm);
        }
    for (int col = 0; col < n; col++) {
        double* diag = B + loc(col, col);
        const int w = cons[col]->n;
        invertBlock(w, diag);
        if (col + 1 == n) continue;
        for (int row = col + 1; row < n; row++) {
            int l = loc(row, col);
            if (l == kEmpty) continue;
            double* tgt = Dg + dloc(row, col);
            const int h = cons[row]->n;
            const double* src = B + l;
            for (int r = 0; r < h; r++)
                for (int c = 0; c < w; c++) tgt[c + w * r] = dotN(w, src + w * r, diag + w * c);
        }
        for (int lc = col + 1; lc < n; lc++)
            for (int lr = lc; lr < n; lr++) {
                int l = loc(lr, col);
                if (l == kEmpty || loc(lc, col) == kEmpty) continue;
                const double* a_src = B + l;
                const double* l_src = Dg + dloc(lc, col);
                double* tgt = B + loc(lr, lc);
                const int bw = cons[lc]->n, bh = cons[lr]->n;
                for (int r = 0; r < bh; r++)
                    for (int c = 0; c < bw; c++) tgt[r * bw + c] -= dotN(w, a_src + r * w, l_src + c * w);
            }
        int first = firstBelow(col);
        if (first == kEmpty) continue;
        int total = loc(col + 1, col + 1) - first;
        std::memcpy(B + first, Dg, sizeof(double) * (size_t)total);
    }
}

// multInverseWithVector (HolonomicBlockSolver.cpp:251-317): v <- L^-T D^-1 L^-1 v
void HoloSys::solve(std::vector<double>& v) const {
    const int n = (int)cons.size();
    const double* B = buf.data();
    std::vector<double> eff(degree);
    for (int col = 0; col + 1 < n; col++) {
        eff.assign(degree, 0.0);
        for (int row = col + 1; row < n; row++) {
            int l = loc(row, col);
            if (l == kEmpty) continue;
            const int bw = cons[col]->n, bh = cons[row]->n;
            for (int i = 0; i < bh; i++) eff[vpos[row] + i] = dotN(bw, B + l + i * bw, v.data() + vpos[col]);
        }
        for (int i = 0; i < degree; i++) v[i] -= eff[i];
    }
    std::vector<double> d(degree);
    for (int col = 0; col < n; col++) {
        const int w = cons[col]->n;
        const double* blk = B + loc(col, col);
        for (int i = 0; i < w; i++) d[vpos[col] + i] = dotN(w, blk + i * w, v.data() + vpos[col]);
    }
    v = d;
    std::vector<double> e6(6);
    for (int col = n - 2; col >= 0; col--) {
        e6.assign(6, 0.0);
        for (int row = col + 1; row < n; row++) {
            int l = loc(row, col);
            if (l == kEmpty) continue;
            const int bw = cons[col]->n, bh = cons[row]->n;
            for (int i = 0; i < bw; i++) {
                double dp = 0;
                for (int j = 0; j < bh; j++) dp += v[vpos[row] + j] * B[l + i + bw * j];
                e6[i] += dp;
            }
        }
        for (int i = 0; i < cons[col]->n; i++) v[vpos[col] + i] -= e6[i];
    }
}

// HolonomicSystem::computeAndApplyImpulses (HolonomicBlockSolver.cpp:319-378):
// solve A d = t - J dv for the whole system; with a threshold, a pseudo
// solution whose angular velocity change exceeds it anywhere is discarded
void HoloSys::computeAndApply(bool pseudo, double thr) {
    std::vector<double> delta(degree);
    for (size_t i = 0; i < cons.size(); i++) {
        JRow& r = *cons[i];
        double cur[kMaxDof];
        if (pseudo) jrowValue(r, r.da->pv, r.db->pv, cur);
        else jrowValue(r, r.da->v, r.db->v, cur);
        const double* tgt = pseudo ? r.ptarget : r.target;
        for (int k = 0; k < r.n; k++) delta[vpos[i] + k] = tgt[k] - cur[k];
    }
    solve(delta);
    if (thr > 0) {
        for (size_t i = 0; i < cons.size(); i++) {
            JRow& r = *cons[i];
            if (isZero(&delta[vpos[i]], r.n)) continue;
            jrowApply(r, &delta[vpos[i]], &r.da->lin_err, &r.db->lin_err);
        }
        for (size_t i = 0; i < cons.size(); i++) {
            const JRow& r = *cons[i];
            double r2 = 0;
            for (int k = 3; k < 6; k++) r2 += r.da->lin_err.v[k] * r.da->lin_err.v[k] + r.db->lin_err.v[k] * r.db->lin_err.v[k];
            if (r2 > thr * thr) return;
        }
    }
    for (size_t i = 0; i < cons.size(); i++) {
        JRow& r = *cons[i];
        const double* ic = &delta[vpos[i]];
        if (isZero(ic, r.n)) continue;
        if (pseudo) jrowApply(r, ic, &r.da->pv, &r.db->pv);
        else jrowApply(r, ic, &r.da->v, &r.db->v);
        double* acc = pseudo ? r.pimpulse : r.holo;
        for (int k = 0; k < r.n; k++) acc[k] += ic[k];
    }
}

// HolonomicSystem::verifyInverse (HolonomicBlockSolver.cpp:545-583): the
// factorisation applied to every column of A gives the identity; returns the
// Frobenius norm of the difference (the reference accepts < 1e-5)
double HoloSys::inverseError(double cfm) const {
    const int n = (int)cons.size();
    std::vector<double> A((size_t)degree * degree);
    int ro = 0;
    for (int r = 0; r < n; r++) {
        int co = 0;
        for (int c = 0; c < n; c++) {
            const int bw = cons[c]->n, bh = cons[r]->n;
            double blk[kMaxDof * kMaxDof];
            initialBlock(blk, cons[r], cons[c], cfm);
            for (int i = 0; i < bh; i++)
                for (int j = 0; j < bw; j++) A[(size_t)(j + co) + (size_t)(i + ro) * degree] = blk[j + i * bw];
            co += bw;
        }
        ro += cons[r]->n;
    }
    double diff = 0;
    for (int i = 0; i < degree; i++) {
        std::vector<double> col(degree);
        for (int j = 0; j < degree; j++) col[j] = A[(size_t)i + (size_t)degree * j];
        solve(col);
        for (int j = 0; j < degree; j++) {
            double d = (j == i ? 1.0 : 0.0) - col[j];
            diff += d * d;
        }
    }
    return std::sqrt(diff);
}

// ------------------------------------------------------ world side ----
// PhysicsEngine::addBallSocketConstraint / addHingeConstraint
// (PhysicsEngine.cpp:664-723): collisions between the two bodies are
// disallowed, the anchors become tracked points, the edge is flagged for a
// holonomic-system scan
Joint* World::addJoint(int n, Body* b1, Body* b2, V3 p1, V3 p2, V3 ax1, V3 ax2, double pos_hard, double rot_hard,
                       double target) {
    b1->no_collide.insert(b2);
    b2->no_collide.insert(b1);
    auto j = std::make_unique<Joint>();
    j->n = n;
    j->seq = constraint_seq++;
    j->b1 = b1; j->b2 = b2;
    b1->track_p.push_back(b1->local_origin + p1);
    j->k1 = (int)b1->track_p.size() - 1;
    b2->track_p.push_back(b2->local_origin + p2);
    j->k2 = (int)b2->track_p.size() - 1;
    if (n == 4 || n == 5) { j->ax1 = ax1.normalize(); j->ax2 = ax2.normalize(); }
    // PhysicsEngine::addDistanceConstraint (PhysicsEngine.cpp:630-635): -1
    // means the attachment points' current distance
    if (n == 1) j->target = target == -1 ? (b1->trackedP(j->k1) - b2->trackedP(j->k2)).mag() : target;
    j->pos_hard = pos_hard;
    j->rot_hard = rot_hard;
    j->row.n = n; j->row.a = b1; j->row.b = b2;
    Edge* e = getOrCreateEdge(b1, b2);
    if (e->h) e->h->changed = true;
    else e->scan_needed = true;
    j->edge = e;
    e->joints.push_back(j.get());
    joints.push_back(std::move(j));
    return joints.back().get();
}

// PhysicsEngine::addConeLimitConstraint (PhysicsEngine.cpp:926-946):
// collisions disallowed, no holonomic-system flags
Joint* World::addCone(Body* b1, Body* b2, V3 ax1, V3 ax2, double max_angle, double rot_hard) {
    b1->no_collide.insert(b2);
    b2->no_collide.insert(b1);
    auto j = std::make_unique<Joint>();
    j->n = 1; j->cone = true;
    j->seq = constraint_seq++;
    j->b1 = b1; j->b2 = b2;
    j->ax1 = ax1; j->ax2 = ax2;
    j->max_angle = max_angle;
    j->rot_hard = rot_hard;
    j->row.n = 1; j->row.a = b1; j->row.b = b2;
    Edge* e = getOrCreateEdge(b1, b2);
    j->edge = e;
    e->joints.push_back(j.get());
    joints.push_back(std::move(j));
    return joints.back().get();
}

// PhysicsEngine::addTwistLimitConstraint (PhysicsEngine.cpp:952-972) and the
// TwistLimit constructor (PersistentConstraint.h:177-184)
Joint* World::addTwist(Body* b1, Body* b2, V3 ax1, V3 ax2, double min_angle, double max_angle, double rot_hard) {
    Joint* j = addCone(b1, b2, ax1, ax2, 0, rot_hard);
    j->cone = false;
    j->twist = true;
    j->min_angle = min_angle;
    j->max_angle = max_angle;
    ax1.perpBasis(&j->w_local, &j->u_local);
    return j;
}

// PhysicsEngine::addMotorConstraint (PhysicsEngine.cpp:725-763) and the Motor
// constructor (PersistentConstraint.cpp:5-24): on the base hinge's (or
// sliding hinge's) axes and rotation strength, appended to the base's edge
Joint* World::addMotor(Joint* base, double min_angle, double max_angle) {
    auto j = std::make_unique<Joint>();
    j->n = 1; j->motor = true;
    j->seq = constraint_seq++;
    j->b1 = base->b1; j->b2 = base->b2;
    j->ax1 = base->ax1; j->ax2 = base->ax2;
    j->rot_hard = base->rot_hard;
    j->lim_min = min_angle; j->lim_max = max_angle;
    V3 tmp;
    j->ax1.perpBasis(&j->ref_u, &j->ref_w);
    j->ax2.perpBasis(&j->cmp, &tmp);
    j->row.n = 1; j->row.a = j->b1; j->row.b = j->b2;
    j->position = 0;
    j->position = j->motorPosition(j->b1->q.rotate(j->ax1), V3(), V3(), 0);
    Edge* e = getOrCreateEdge(j->b1, j->b2);
    j->edge = e;
    e->joints.push_back(j.get());
    joints.push_back(std::move(j));
    return joints.back().get();
}

// PhysicsEngine::addPistonConstraint (PhysicsEngine.cpp:808-852) and the
// Piston constructor (PersistentConstraint.cpp:134-143): on the base slider's
// (or sliding hinge's) tracked points, body 1 axis and position strength, as
// two joints (slide limit, powered row) appended to the base's edge.  The
// constructor's position reads body 2's point key on body 1
// (getTrackedP's (-1, -1, -1) when body 1 has no such key); every rebuild
// recomputes it from both bodies.  Returns the powered joint.
Joint* World::addPiston(Joint* base, double min_pos, double max_pos) {
    Joint* out = nullptr;
    const int seq = constraint_seq++;
    for (int part = 0; part < 2; part++) {
        auto j = std::make_unique<Joint>();
        j->n = 1;
        j->seq = seq;
        (part == 0 ? j->slide_limit : j->piston) = true;
        j->b1 = base->b1; j->b2 = base->b2;
        j->k1 = base->k1; j->k2 = base->k2;
        j->ax1 = base->ax1;
        j->pos_hard = base->pos_hard;
        j->lim_min = min_pos; j->lim_max = max_pos;
        j->row.n = 1; j->row.a = j->b1; j->row.b = j->b2;
        V3 pa = j->b1->trackedP(j->k1);
        V3 pb = j->k2 < (int)j->b1->track_p.size() ? j->b1->trackedP(j->k2) : V3(-1, -1, -1);
        V3 axis = j->b1->q.rotate(j->ax1);
        j->position = pb.dot(axis) - pa.dot(axis);
        Edge* e = getOrCreateEdge(j->b1, j->b2);
        j->edge = e;
        e->joints.push_back(j.get());
        joints.push_back(std::move(j));
        out = joints.back().get();
    }
    return out;
}

// getAllEdgesConnectedHolonomically (PhysicsEngine.cpp:1745-1777)
static std::vector<Edge*> connectedHolonomically(World& w, Edge* e) {
    std::set<Edge*> visited;
    std::vector<Edge*> to_visit{e}, out;
    while (!to_visit.empty()) {
        Edge* v = to_visit.back();
        to_visit.pop_back();
        if (visited.count(v)) continue;
        visited.insert(v);
        out.push_back(v);
        std::vector<Edge*> nb;
        if (v->n1->movement == DYNAMIC) nb.insert(nb.end(), w.adj[v->n1].begin(), w.adj[v->n1].end());
        if (v->n2->movement == DYNAMIC) nb.insert(nb.end(), w.adj[v->n2].begin(), w.adj[v->n2].end());
        for (Edge* x : nb) {
            if (visited.count(x)) continue;
            // SharedConstraintsEdge::hasHolonomicConstraint (PhysicsEngine.h:259-264)
            if (std::any_of(x->joints.begin(), x->joints.end(), [](const Joint* j) { return j->holonomic(); }))
                to_visit.push_back(x);
        }
    }
    return out;
}

// maintainAllHolonomicSystemStuffRelatedToThisEdge (PhysicsEngine.cpp:1466-1532)
void World::holonomicScan(Edge* e) {
    if (e->scan_needed) {
        e->scan_needed = false;
        std::vector<Edge*> conn = connectedHolonomically(*this, e);
        if (conn.size() <= 1) return;
        std::set<HoloSys*> seen;
        for (Edge* x : conn) seen.insert(x->h);
        if (seen.size() == 1 && *seen.begin() != nullptr) {
        } else if (seen.size() == 1) {
            auto h = std::make_unique<HoloSys>();
            h->member_edges = conn;
            h->changed = true;
            for (Edge* x : conn) { x->h = h.get(); x->scan_needed = false; }
            systems.push_back(std::move(h));
        } else {
            auto it = seen.begin();
            HoloSys* keep = (*it == nullptr) ? *std::next(it) : *it;
            for (Edge* x : conn) {
                if (x->h != keep) { keep->member_edges.push_back(x); x->h = keep; }
                x->scan_needed = false;
            }
            keep->changed = true;
            for (HoloSys* s : seen)
                if (s != nullptr && s != keep)
                    for (size_t i = 0; i < systems.size(); i++)
                        if (systems[i].get() == s) { systems.erase(systems.begin() + i); break; }
        }
    }
    if (e->h != nullptr && e->h->changed) {
        e->h->changed = false;
        std::vector<JRow*> rows;   // HolonomicSystemNodes::revaluateSystem (:1789-1802)
        for (Edge* x : e->h->member_edges)
            for (Joint* j : x->joints)
                if (j->holonomic()) rows.push_back(&j->row);
        e->h->build(rows);
        for (Edge* x : e->h->member_edges)
            for (Joint* j : x->joints)
                if (j->holonomic()) j->rebuild(p, p.dt / p.substeps, true);
        e->h->computeInverse(p.cfm);
    }
}

// PhysicsEngine::maintainHolonomicSystems (PhysicsEngine.cpp:1292-1306)
void World::maintainHolonomicSystems() {
    for (auto& kv : nodes)
        for (Edge* e : adj[kv.second]) holonomicScan(e);
}

// calculateHolonomicSystemInversesAsync (PhysicsEngine.cpp:1617-1649): at the
// end of a step the system rows are rebuilt from the new poses and the
// factorisations recomputed for the next step's first substep
void World::updateHolonomicInverses() {
    std::set<HoloSys*> seen;
    std::set<Edge*> seen_edges;
    for (auto& kv : nodes)
        for (Edge* e : adj[kv.second]) {
            if (e->h == nullptr || seen_edges.count(e)) continue;
            for (Joint* j : e->joints)
                if (j->holonomic()) j->rebuild(p, p.dt / p.substeps, true);
            seen_edges.insert(e);
            seen.insert(e->h);
        }
    for (HoloSys* h : seen) h->computeInverse(p.cfm);
}

}  // namespace cport
