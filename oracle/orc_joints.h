// Oracle joint constraints: BallJointConstraint, HingeJointConstraint and SliderJointConstraint of
// the reference's sequential-impulse solver (src/rigid/constraint/constraint/{ball,hinge,slider}
// _joint_constraint.cpp), restated with the reference's operation order.  Test infrastructure only.
#pragma once
#include <cmath>
#include "orc_collide.h"

namespace orc {

enum JointType { JT_BALL = 0, JT_HINGE = 1, JT_SLIDER = 2 };

template <class R> struct Joint {
    int type = JT_BALL, a = 0, b = 0;
    V3<R> anchor_a, anchor_b, axis_a = V3<R>(1, 0, 0), axis_b = V3<R>(1, 0, 0);
    bool use_limits = false, use_motor = false;
    R min_angle = 0, max_angle = 0, target_speed = 0;
    // per-step solver data (initSequentialImpulse)
    V3<R> r_a, r_b, w_axis_a, w_axis_b, w_t_a[2], w_t_b[2], rhs_ball;
    M3<R> jmj_ball, jmj_rot;
    R rhs2[2] = {0, 0}, jmj2[2] = {0, 0};   // hinge: rhs/jmj of the two hinge rows; slider: of the two position rows
    R jmj_ml = 0, rhs_motor = 0, rhs_limit = 0;
    bool limit_exceeded = false;
};

// Constraint::getSkewSymmetricMatrix (constraint.cpp:9-13)
template <class R> M3<R> skew(const V3<R>& v) {
    M3<R> m;
    m.m[0][1] = -v.z; m.m[0][2] = v.y;
    m.m[1][0] = v.z; m.m[1][2] = -v.x;
    m.m[2][0] = -v.y; m.m[2][1] = v.x;
    return m;
}

template <class R> M3<R> madd(const M3<R>& a, const M3<R>& b) {
    M3<R> o;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.m[i][j] = a.m[i][j] + b.m[i][j];
    return o;
}

// (E * (ima + imb) + rxA * IA * rxA^T + rxB * IB * rxB^T)^-1 of the ball rows
template <class R> M3<R> ball_jmj(const V3<R>& ra, const V3<R>& rb, R ims, const M3<R>& Ia, const M3<R>& Ib) {
    M3<R> s;
    for (int i = 0; i < 3; i++) s.m[i][i] = ims;
    const M3<R> rxa = skew(ra), rxb = skew(rb);
    return inverse3(madd(madd(s, mmt_r2l(mm(rxa, Ia), rxa)), mmt_r2l(mm(rxb, Ib), rxb)));
}

// RigidBody::getKinematicInvMass / getKinematicWorldInvInertia (rigidbody.cpp:52-62)
template <class R, class Bd> R kin_inv_mass(const Bd& b) { return b.kinematic ? R(0) : b.inv_mass; }
template <class R, class Bd> M3<R> kin_inv_inertia(const Bd& b) { return b.kinematic ? M3<R>() : b.world_inv_inertia; }

// RigidBody::applyTempImpulse / applyTempAngularImpulse (rigidbody.cpp:166-181)
template <class R, class Bd> void temp_impulse(Bd& b, const V3<R>& r, const V3<R>& imp) {
    if (b.kinematic) return;
    b.tv = b.tv + imp * b.inv_mass;
    b.tw = b.tw + mv(b.world_inv_inertia, cross(r, imp));
}
template <class R, class Bd> void temp_ang_impulse(Bd& b, const V3<R>& imp) {
    if (b.kinematic) return;
    b.tw = b.tw + mv(b.world_inv_inertia, imp);
}

template <class R, class Bd> void joint_init(Joint<R>& j, const Bd& A, const Bd& B, R dt, R kerp) {
    const Transform<R>& ta = A.t;
    const Transform<R>& tb = B.t;
    j.r_a = mv(ta.basis, j.anchor_a);
    j.r_b = mv(tb.basis, j.anchor_b);
    const R ims = kin_inv_mass<R>(A) + kin_inv_mass<R>(B);
    const M3<R> Ia = kin_inv_inertia<R>(A), Ib = kin_inv_inertia<R>(B);
    const V3<R> rel = ta.apply(j.anchor_a) - tb.apply(j.anchor_b);
    if (j.type == JT_BALL) {   // ball_joint_constraint.cpp:6-19
        j.jmj_ball = ball_jmj(j.r_a, j.r_b, ims, Ia, Ib);
        j.rhs_ball = mv(j.jmj_ball, rel) * (-kerp / dt);
        return;
    }
    j.w_axis_a = mv(ta.basis, j.axis_a);
    j.w_axis_b = mv(tb.basis, j.axis_b);
    ortho_units(j.axis_a, j.w_t_a[0], j.w_t_a[1]);
    j.w_t_a[0] = mv(ta.basis, j.w_t_a[0]);
    j.w_t_a[1] = mv(ta.basis, j.w_t_a[1]);
    if (j.type == JT_HINGE) {   // hinge_joint_constraint.cpp:6-63
        if (j.use_limits) {
            ortho_units(j.axis_b, j.w_t_b[0], j.w_t_b[1]);
            j.w_t_b[0] = mv(tb.basis, j.w_t_b[0]);
            j.w_t_b[1] = mv(tb.basis, j.w_t_b[1]);
        }
        j.jmj_ball = ball_jmj(j.r_a, j.r_b, ims, Ia, Ib);
        j.rhs_ball = mv(j.jmj_ball, rel) * (-kerp / dt);
        const M3<R> Is = madd(Ia, Ib);
        j.jmj2[0] = R(1.0) / dot(j.w_t_a[0], mv(Is, j.w_t_a[0]));
        j.jmj2[1] = R(1.0) / dot(j.w_t_a[1], mv(Is, j.w_t_a[1]));
        const V3<R> u = cross(j.w_axis_a, j.w_axis_b);
        j.rhs2[0] = j.jmj2[0] * (dot(u, j.w_t_a[0]) * kerp / dt);
        j.rhs2[1] = j.jmj2[1] * (dot(u, j.w_t_a[1]) * kerp / dt);
        if (j.use_motor || j.use_limits) j.jmj_ml = R(1.0) / dot(j.w_axis_a, mv(Is, j.w_axis_a));
        if (j.use_motor) j.rhs_motor = j.jmj_ml * -j.target_speed;
        if (j.use_limits) {
            const R c = dot(j.w_t_a[0], j.w_t_b[0]);
            const R s = dot(cross(j.w_t_a[0], j.w_t_b[0]), j.w_axis_a);
            const R angle = std::atan2(s, c);
            j.limit_exceeded = false;
            if (angle < j.min_angle) {
                j.limit_exceeded = true;
                j.rhs_limit = -j.jmj_ml * (j.min_angle - angle) * kerp / dt;
            } else if (angle > j.max_angle) {
                j.limit_exceeded = true;
                j.rhs_limit = -j.jmj_ml * (j.max_angle - angle) * kerp / dt;
            }
        }
        return;
    }
    // slider_joint_constraint.cpp:7-51
    ortho_units(j.axis_b, j.w_t_b[0], j.w_t_b[1]);
    j.w_t_b[0] = mv(tb.basis, j.w_t_b[0]);
    j.w_t_b[1] = mv(tb.basis, j.w_t_b[1]);
    for (int k = 0; k < 2; k++) {
        const V3<R> xa = cross(j.r_a, j.w_t_a[k]), xb = cross(j.r_b, j.w_t_a[k]);
        j.jmj2[k] = R(1.0) / (ims + dot(mv(Ia, xa), xa) + dot(mv(Ib, xb), xb));
    }
    // both position rows scale by the first row's jmj (slider_joint_constraint.cpp:39-40)
    j.rhs2[0] = j.jmj2[0] * (dot(rel, j.w_t_a[0]) * (-kerp / dt));
    j.rhs2[1] = j.jmj2[0] * (dot(rel, j.w_t_a[1]) * (-kerp / dt));
    j.jmj_rot = inverse3(madd(Ia, Ib));
}

template <class R, class Bd> void joint_iterate(Joint<R>& j, Bd& A, Bd& B) {
    if (j.type == JT_SLIDER) {   // slider_joint_constraint.cpp:53-65
        const V3<R> va = A.tv + cross(A.tw, j.r_a), vb = B.tv + cross(B.tw, j.r_b);
        const R p0 = j.rhs2[0] - j.jmj2[0] * dot(j.w_t_a[0], va - vb);
        const R p1 = j.rhs2[1] - j.jmj2[1] * dot(j.w_t_a[1], va - vb);
        const V3<R> pv = j.w_t_a[0] * p0 + j.w_t_a[1] * p1;
        temp_impulse<R>(A, j.r_a, pv);
        temp_impulse<R>(B, j.r_b, -pv);
        const V3<R> rot = mv(j.jmj_rot, A.tw - B.tw);
        const V3<R> ri(-rot.x, -rot.y, -rot.z);
        temp_ang_impulse<R>(A, ri);
        temp_ang_impulse<R>(B, -ri);
        return;
    }
    // ball rows (ball_joint_constraint.cpp:21-27; hinge_joint_constraint.cpp:66-71)
    const V3<R> va = A.tv + cross(A.tw, j.r_a), vb = B.tv + cross(B.tw, j.r_b);
    const V3<R> bi = j.rhs_ball - mv(j.jmj_ball, va - vb);
    temp_impulse<R>(A, j.r_a, bi);
    temp_impulse<R>(B, j.r_b, -bi);
    if (j.type == JT_BALL) return;
    // hinge rows (hinge_joint_constraint.cpp:73-80); the motor and limit rows read the angular
    // velocities after the impulses before them (the reference holds references to them)
    const V3<R> dw = A.tw - B.tw;
    const R h0 = j.rhs2[0] - j.jmj2[0] * dot(j.w_t_a[0], dw);
    const R h1 = j.rhs2[1] - j.jmj2[1] * dot(j.w_t_a[1], dw);
    const V3<R> iv = j.w_t_a[0] * h0 + j.w_t_a[1] * h1;
    temp_ang_impulse<R>(A, iv);
    temp_ang_impulse<R>(B, -iv);
    if (j.use_motor) {   // :83-87
        const R mi = j.rhs_motor - j.jmj_ml * dot(j.w_axis_a, A.tw - B.tw);
        temp_ang_impulse<R>(A, j.w_axis_a * mi);
        temp_ang_impulse<R>(B, -j.w_axis_a * mi);
    }
    if (j.use_limits && j.limit_exceeded) {   // :90-96
        const R delta = dot(j.w_axis_a, A.tw - B.tw);
        const R nd = delta * j.rhs_limit > 0 ? R(0) : delta;
        const R li = j.rhs_limit - j.jmj_ml * nd;
        temp_ang_impulse<R>(A, j.w_axis_a * li);
        temp_ang_impulse<R>(B, -j.w_axis_a * li);
    }
}

} // namespace orc
