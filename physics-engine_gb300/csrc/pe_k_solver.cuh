// Kernels of the rigid-body step, part 5: sequential-impulse rows, joints, contact islands,
// level schedules and colouring.
#pragma once
#include "pe_k_sat.cuh"

namespace pe {

// ===================================================================== solver
// FrictionContactConstraint::initSequentialImpulse (friction_contact_constraint.cpp:9-73), one thread per result
template <class R>
__device__ __forceinline__ void si_setup_result(int p, const Results<R>& res, const Bodies<R>& B, const Rows<R>& rows, const int* row_off,
                                                const StepParams& prm, int* status) {
    const int np = res.npts[p];
    if (np == 0) return;
    const int ia = res.a[p], ib = res.b[p];
    const bool ka = (B.flags[ia] & BF_KINEMATIC) != 0, kb = (B.flags[ib] & BF_KINEMATIC) != 0;
    const R ims = (ka ? R(0) : B.at(INVM, ia)) + (kb ? R(0) : B.at(INVM, ib));
    const M3<R> Ia = ka ? M3<R>() : B.mat(I00, ia);
    const M3<R> Ib = kb ? M3<R>() : B.mat(I00, ib);
    const M3<R> Ra = B.mat(B00, ia), Rb = B.mat(B00, ib);
    const V3<R> va0 = B.vec(VX, ia), wa0 = B.vec(WX, ia), vb0 = B.vec(VX, ib), wb0 = B.vec(WX, ib);
    const R dt = R(prm.dt), kerp = R(0.2), pen_th = R(0.3), rest_th = R(0.1);
    const R mu = res.fr[p], e = res.re[p];
    const int r0 = row_off[p];
    if (r0 + np > rows.cap) { atomicOr(status, ST_ROW_OVERFLOW); return; }
    for (int k = 0; k < np; k++) {
        const int o = p * kSlots + k;
        const V3<R> la(res.pt(LAX, o), res.pt(LAY, o), res.pt(LAZ, o));
        const V3<R> lb(res.pt(LBX, o), res.pt(LBY, o), res.pt(LBZ, o));
        const V3<R> n(res.pt(NX, o), res.pt(NY, o), res.pt(NZ, o));
        const V3<R> t0(res.pt(T0X, o), res.pt(T0Y, o), res.pt(T0Z, o));
        const V3<R> t1(res.pt(T1X, o), res.pt(T1Y, o), res.pt(T1Z, o));
        const V3<R> ra = mv(Ra, la), rb = mv(Rb, lb);
        auto jmj = [&](const V3<R>& d) {
            const V3<R> xa = cross(ra, d), xb = cross(rb, d);
            return R(1.0) / (ims + dot(mv(Ia, xa), xa) + dot(mv(Ib, xb), xb));
        };
        const R nj = jmj(n), j0 = jmj(t0), j1 = jmj(t1);
        const V3<R> va = va0 + cross(wa0, ra), vb = vb0 + cross(wb0, rb);
        R rev = -dot(n, va - vb);
        if (rabs(rev) < rest_th) rev = 0;
        rev *= e;
        R pen = res.dist[p * kSlots + k];
        pen = pen > -pen_th ? pen : -pen_th;
        const int r = r0 + k;
        const V3<R> fs[5] = {ra, rb, n, t0, t1};
        for (int g = 0; g < 5; g++) { rows.at(g * 3, r) = fs[g].x; rows.at(g * 3 + 1, r) = fs[g].y; rows.at(g * 3 + 2, r) = fs[g].z; }
        rows.at(NRHS, r) = (rev - kerp * pen / dt) * nj;
        rows.at(NJMJ, r) = nj;
        rows.at(T0JMJ, r) = j0;
        rows.at(T1JMJ, r) = j1;
        rows.at(MU, r) = mu;
        rows.at(NACC, r) = 0;
        rows.at(T0ACC, r) = 0;
        rows.at(T1ACC, r) = 0;
    }
}
template <class R>
__global__ void k_si_setup(const int* Rd, Results<R> res, Bodies<R> B, Rows<R> rows, const int* row_off, StepParams prm, int* status) {
    const int P = *Rd;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) si_setup_result(p, res, B, rows, row_off, prm, status);
}

// FrictionContactConstraint::iterateSequentialImpulse (friction_contact_constraint.cpp:75-108)
// for all points of one result; temporary velocities live in the body arrays
// The rows of one result applied to the two bodies' temporary velocities, held by the caller.
template <class R>
__device__ __forceinline__ void si_result_rows(const Rows<R>& rows, int r0, int np, bool ka, bool kb, V3<R>& tva, V3<R>& twa,
                                               V3<R>& tvb, V3<R>& twb, R ima, R imb, const M3<R>& Ia, const M3<R>& Ib) {
    for (int r = r0; r < r0 + np; r++) {
        const V3<R> ra(rows.at(RAX, r), rows.at(RAY, r), rows.at(RAZ, r));
        const V3<R> rb(rows.at(RBX, r), rows.at(RBY, r), rows.at(RBZ, r));
        const V3<R> n(rows.at(RNX, r), rows.at(RNY, r), rows.at(RNZ, r));
        const V3<R> t0(rows.at(R0X, r), rows.at(R0Y, r), rows.at(R0Z, r));
        const V3<R> t1(rows.at(R1X, r), rows.at(R1Y, r), rows.at(R1Z, r));
        R nacc = rows.at(NACC, r), t0acc = rows.at(T0ACC, r), t1acc = rows.at(T1ACC, r);
        const V3<R> vr = tva + cross(twa, ra) - tvb - cross(twb, rb);
        R ni = rows.at(NRHS, r) - dot(n, vr) * rows.at(NJMJ, r);
        ni = ni > -nacc ? ni : -nacc;
        nacc += ni;
        R tt0 = t0acc - dot(t0, vr) * rows.at(T0JMJ, r);
        R tt1 = t1acc - dot(t1, vr) * rows.at(T1JMJ, r);
        const R scale = rows.at(MU, r) * nacc / real_sqrt(tt0 * tt0 + tt1 * tt1);
        if (scale < 1) { tt0 *= scale; tt1 *= scale; }
        const V3<R> imp = ni * n + (tt0 - t0acc) * t0 + (tt1 - t1acc) * t1;
        rows.at(NACC, r) = nacc;
        rows.at(T0ACC, r) = tt0;
        rows.at(T1ACC, r) = tt1;
        if (!ka) { tva = tva + imp * ima; twa = twa + mv(Ia, cross(ra, imp)); }
        const V3<R> nimp = -imp;
        if (!kb) { tvb = tvb + nimp * imb; twb = twb + mv(Ib, cross(rb, nimp)); }
        // the same body can sit on both sides only through distinct results, never here
    }
}
template <class R>
__device__ __forceinline__ void si_iterate_result(const Bodies<R>& B, const Rows<R>& rows, int ia, int ib, int r0, int np) {
    const bool ka = (B.flags[ia] & BF_KINEMATIC) != 0, kb = (B.flags[ib] & BF_KINEMATIC) != 0;
    V3<R> tva = B.vec(TVX, ia), twa = B.vec(TWX, ia), tvb = B.vec(TVX, ib), twb = B.vec(TWX, ib);
    const R ima = B.at(INVM, ia), imb = B.at(INVM, ib);
    const M3<R> Ia = B.mat(I00, ia), Ib = B.mat(I00, ib);
    si_result_rows(rows, r0, np, ka, kb, tva, twa, tvb, twb, ima, imb, Ia, Ib);
    if (!ka) { B.set_vec(TVX, ia, tva); B.set_vec(TWX, ia, twa); }
    if (!kb) { B.set_vec(TVX, ib, tvb); B.set_vec(TWX, ib, twb); }
}

// ---------------------------------------------------------------- joints
// Ball/Hinge/SliderJointConstraint::initSequentialImpulse and iterateSequentialImpulse
// (ball_joint_constraint.cpp:6-27, hinge_joint_constraint.cpp:6-97, slider_joint_constraint.cpp:7-65)
// in the reference's operation order.  A kinematic body contributes no inverse mass or inertia
// (RigidBody::getKinematicInvMass / getKinematicWorldInvInertia) and takes no impulse.
template <class R> __device__ __forceinline__ M3<R> skew3(const V3<R>& v) {   // Constraint::getSkewSymmetricMatrix
    M3<R> m;
    m.m[0][0] = 0; m.m[0][1] = -v.z; m.m[0][2] = v.y;
    m.m[1][0] = v.z; m.m[1][1] = 0; m.m[1][2] = -v.x;
    m.m[2][0] = -v.y; m.m[2][1] = v.x; m.m[2][2] = 0;
    return m;
}
template <class R> __device__ __forceinline__ M3<R> madd3(const M3<R>& a, const M3<R>& b) {
    M3<R> o;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.m[i][j] = a.m[i][j] + b.m[i][j];
    return o;
}
template <class R> __device__ __forceinline__ V3<R> jp3(const R* p, int k) { return V3<R>(p[k], p[k + 1], p[k + 2]); }
template <class R> __device__ __forceinline__ void jw3(R* p, int k, const V3<R>& v) { p[k] = v.x; p[k + 1] = v.y; p[k + 2] = v.z; }
template <class R> __device__ __forceinline__ M3<R> jp9(const R* p, int k) {
    M3<R> m;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) m.m[i][j] = p[k + i * 3 + j];
    return m;
}
template <class R> __device__ __forceinline__ void jw9(R* p, int k, const M3<R>& m) {
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) p[k + i * 3 + j] = m.m[i][j];
}

template <class R>
__global__ void k_joint_init(Joints<R> J, Bodies<R> B, StepParams P) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J.n) return;
    const int ia = J.body[j].x, ib = J.body[j].y, type = J.type[j], fl = J.flag[j];
    const bool ka = (B.flags[ia] & BF_KINEMATIC) != 0, kb = (B.flags[ib] & BF_KINEMATIC) != 0;
    const R* q = J.param + (size_t)j * NJP;
    R* w = J.row + (size_t)j * NJR;
    const R dt = R(P.dt), kerp = R(0.2);
    const Xf<R> ta = B.xf(ia), tb = B.xf(ib);
    const V3<R> anc_a = jp3(q, JP_ANCHOR_A), anc_b = jp3(q, JP_ANCHOR_B);
    const V3<R> ra = mv(ta.b, anc_a), rb = mv(tb.b, anc_b);
    jw3(w, JR_RA, ra);
    jw3(w, JR_RB, rb);
    const R ims = (ka ? R(0) : B.at(INVM, ia)) + (kb ? R(0) : B.at(INVM, ib));
    const M3<R> Ia = ka ? M3<R>() : B.mat(I00, ia), Ib = kb ? M3<R>() : B.mat(I00, ib);
    const V3<R> rel = ta.apply(anc_a) - tb.apply(anc_b);
    auto ball = [&]() {
        M3<R> d;
        for (int k = 0; k < 3; k++) d.m[k][k] = ims;
        const M3<R> jmj = inverse3(madd3(madd3(d, world_inertia(skew3(ra), Ia)), world_inertia(skew3(rb), Ib)));
        jw9(w, JR_JMJ_BALL, jmj);
        jw3(w, JR_RHS_BALL, mv(jmj, rel) * (-kerp / dt));
    };
    if (type == JT_BALL) { ball(); return; }
    const V3<R> wax = mv(ta.b, jp3(q, JP_AXIS_A)), wbx = mv(tb.b, jp3(q, JP_AXIS_B));
    V3<R> t0, t1, u0, u1;
    ortho_units(jp3(q, JP_AXIS_A), t0, t1);
    t0 = mv(ta.b, t0);
    t1 = mv(ta.b, t1);
    jw3(w, JR_WAX, wax);
    jw3(w, JR_T0, t0);
    jw3(w, JR_T1, t1);
    if (type == JT_HINGE) {
        const bool lim = (fl & 1) != 0, mot = (fl & 2) != 0;
        if (lim) {
            ortho_units(jp3(q, JP_AXIS_B), u0, u1);
            u0 = mv(tb.b, u0);
        }
        ball();
        const M3<R> Is = madd3(Ia, Ib);
        const R j0 = R(1.0) / dot(t0, mv(Is, t0)), j1 = R(1.0) / dot(t1, mv(Is, t1));
        const V3<R> u = cross(wax, wbx);
        w[JR_JMJ2] = j0;
        w[JR_JMJ2 + 1] = j1;
        w[JR_RHS2] = j0 * (dot(u, t0) * kerp / dt);
        w[JR_RHS2 + 1] = j1 * (dot(u, t1) * kerp / dt);
        R jml = 0;
        if (mot || lim) jml = R(1.0) / dot(wax, mv(Is, wax));
        w[JR_JMJ_ML] = jml;
        if (mot) w[JR_RHS_MOTOR] = jml * -q[JP_SPEED];
        w[JR_LIMIT] = 0;
        if (lim) {
            const R c = dot(t0, u0), sn = dot(cross(t0, u0), wax);
            const R angle = atan2(sn, c);
            if (angle < q[JP_MIN]) {
                w[JR_LIMIT] = 1;
                w[JR_RHS_LIMIT] = -jml * (q[JP_MIN] - angle) * kerp / dt;
            } else if (angle > q[JP_MAX]) {
                w[JR_LIMIT] = 1;
                w[JR_RHS_LIMIT] = -jml * (q[JP_MAX] - angle) * kerp / dt;
            }
        }
        return;
    }
    // slider
    ortho_units(jp3(q, JP_AXIS_B), u0, u1);
    const V3<R> ts[2] = {t0, t1};
    R jp[2];
    for (int k = 0; k < 2; k++) {
        const V3<R> xa = cross(ra, ts[k]), xb = cross(rb, ts[k]);
        jp[k] = R(1.0) / (ims + dot(mv(Ia, xa), xa) + dot(mv(Ib, xb), xb));
    }
    w[JR_JMJ2] = jp[0];
    w[JR_JMJ2 + 1] = jp[1];
    w[JR_RHS2] = jp[0] * (dot(rel, t0) * (-kerp / dt));
    w[JR_RHS2 + 1] = jp[0] * (dot(rel, t1) * (-kerp / dt));   // the first row's jmj, as slider_joint_constraint.cpp:40
    jw9(w, JR_JMJ_ROT, inverse3(madd3(Ia, Ib)));
}

// RigidBody::applyTempImpulse / applyTempAngularImpulse (rigidbody.cpp:166-181)
template <class R> __device__ __forceinline__ void jt_impulse(const Bodies<R>& B, int i, const V3<R>& r, const V3<R>& imp) {
    if (B.flags[i] & BF_KINEMATIC) return;
    B.set_vec(TVX, i, B.vec(TVX, i) + imp * B.at(INVM, i));
    B.set_vec(TWX, i, B.vec(TWX, i) + mv(B.mat(I00, i), cross(r, imp)));
}
template <class R> __device__ __forceinline__ void jt_ang_impulse(const Bodies<R>& B, int i, const V3<R>& imp) {
    if (B.flags[i] & BF_KINEMATIC) return;
    B.set_vec(TWX, i, B.vec(TWX, i) + mv(B.mat(I00, i), imp));
}

template <class R> __device__ void joint_iterate(const Joints<R>& J, const Bodies<R>& B, int j) {
    const int ia = J.body[j].x, ib = J.body[j].y, type = J.type[j], fl = J.flag[j];
    const R* w = J.row + (size_t)j * NJR;
    const V3<R> ra = jp3(w, JR_RA), rb = jp3(w, JR_RB);
    const V3<R> va = B.vec(TVX, ia) + cross(B.vec(TWX, ia), ra), vb = B.vec(TVX, ib) + cross(B.vec(TWX, ib), rb);
    if (type == JT_SLIDER) {
        const V3<R> t0 = jp3(w, JR_T0), t1 = jp3(w, JR_T1);
        const R p0 = w[JR_RHS2] - w[JR_JMJ2] * dot(t0, va - vb);
        const R p1 = w[JR_RHS2 + 1] - w[JR_JMJ2 + 1] * dot(t1, va - vb);
        const V3<R> pv = t0 * p0 + t1 * p1;
        jt_impulse(B, ia, ra, pv);
        jt_impulse(B, ib, rb, -pv);
        const V3<R> rot = mv(jp9(w, JR_JMJ_ROT), B.vec(TWX, ia) - B.vec(TWX, ib));
        const V3<R> ri = -rot;
        jt_ang_impulse(B, ia, ri);
        jt_ang_impulse(B, ib, -ri);
        return;
    }
    const V3<R> bi = jp3(w, JR_RHS_BALL) - mv(jp9(w, JR_JMJ_BALL), va - vb);
    jt_impulse(B, ia, ra, bi);
    jt_impulse(B, ib, rb, -bi);
    if (type == JT_BALL) return;
    // hinge rows; motor and limit read the angular velocities left by the impulses before them
    const V3<R> t0 = jp3(w, JR_T0), t1 = jp3(w, JR_T1), wax = jp3(w, JR_WAX);
    const V3<R> dw = B.vec(TWX, ia) - B.vec(TWX, ib);
    const R h0 = w[JR_RHS2] - w[JR_JMJ2] * dot(t0, dw);
    const R h1 = w[JR_RHS2 + 1] - w[JR_JMJ2 + 1] * dot(t1, dw);
    const V3<R> iv = t0 * h0 + t1 * h1;
    jt_ang_impulse(B, ia, iv);
    jt_ang_impulse(B, ib, -iv);
    if (fl & 2) {
        const R mi = w[JR_RHS_MOTOR] - w[JR_JMJ_ML] * dot(wax, B.vec(TWX, ia) - B.vec(TWX, ib));
        jt_ang_impulse(B, ia, wax * mi);
        jt_ang_impulse(B, ib, -wax * mi);
    }
    if ((fl & 1) && w[JR_LIMIT] != 0) {
        const R delta = dot(wax, B.vec(TWX, ia) - B.vec(TWX, ib));
        const R nd = delta * w[JR_RHS_LIMIT] > 0 ? R(0) : delta;
        const R li = w[JR_RHS_LIMIT] - w[JR_JMJ_ML] * nd;
        jt_ang_impulse(B, ia, wax * li);
        jt_ang_impulse(B, ib, -wax * li);
    }
}

// Island items: a contact result index, or a joint index with kJointItem set.  Within an island
// the contacts come first in result order, then the joints in order, so one pass over an island's
// items is the reference's iteration (every contact, then every other constraint) restricted to
// the island.
constexpr uint32_t kJointItem = 0x80000000u;
template <class R> __device__ __forceinline__ int2 item_bodies(uint32_t item, const Results<R>& res, const Joints<R>& J) {
    if (item & kJointItem) return J.body[item & ~kJointItem];
    return make_int2(res.a[item], res.b[item]);
}
template <class R>
__device__ __forceinline__ void iterate_item(uint32_t item, const Results<R>& res, const Joints<R>& J, const Bodies<R>& B,
                                             const Rows<R>& rows, const int* row_off) {
    if (item & kJointItem) { joint_iterate(J, B, (int)(item & ~kJointItem)); return; }
    const int p = (int)item;
    si_iterate_result(B, rows, res.a[p], res.b[p], row_off[p], res.npts[p]);
}

// ---------------------------------------------------------------- contact islands
// Islands: connected components of dynamic bodies linked by contact results (a kinematic body
// links nothing: its temporary velocity never changes).  Results of different islands touch
// disjoint dynamic bodies, so running each island's results in the reference's global order
// (SequentialImpulseSolver::solve, sequential_impulse_solver.cpp:60-69) yields exactly the
// reference's velocities while islands proceed in parallel.
__device__ __forceinline__ int uf_find(const int* parent, int x) {
    int p = parent[x];
    while (p != x) { x = p; p = parent[x]; }   // parents always point to smaller indices
    return x;
}
__device__ __forceinline__ void uf_union(int* parent, int a, int b) {
    for (;;) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a < b) { const int t = a; a = b; b = t; }
        // hook the larger root below the smaller one; retry if another thread moved it first
        if (atomicCAS(&parent[a], a, b) == a) return;
    }
}

__global__ void k_isl_init(int n, int* parent);
template <class R>
__global__ void k_isl_union(const int* Ad, const int* active, Results<R> res, Bodies<R> B, int* parent) {
    const int A = *Ad;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < A; t += gridDim.x * blockDim.x) {
        const int p = active[t];
        const int ia = res.a[p], ib = res.b[p];
        if ((B.flags[ia] & BF_KINEMATIC) || (B.flags[ib] & BF_KINEMATIC)) continue;
        uf_union(parent, ia, ib);
    }
}
// joints link their bodies like contact results do
template <class R>
__global__ void k_isl_union_joints(Joints<R> J, Bodies<R> B, int* parent) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J.n) return;
    const int ia = J.body[j].x, ib = J.body[j].y;
    if ((B.flags[ia] & BF_KINEMATIC) || (B.flags[ib] & BF_KINEMATIC)) return;
    uf_union(parent, ia, ib);
}
// sort keys of the joints, after the A active results: the island label of a dynamic body; a joint
// between two kinematic bodies (which moves nothing) gets the label n_bodies, an island of its own
template <class R>
__global__ void k_isl_keys_joints(Joints<R> J, Bodies<R> B, const int* parent, const int* Ad, uint64_t* key, uint32_t* key2, uint32_t* val) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J.n) return;
    const int A = *Ad;
    const int ia = J.body[j].x, ib = J.body[j].y;
    const bool ka = (B.flags[ia] & BF_KINEMATIC) != 0, kb = (B.flags[ib] & BF_KINEMATIC) != 0;
    key[A + j] = ka && kb ? (uint64_t)B.n : (uint64_t)uf_find(parent, ka ? ib : ia);
    key2[A + j] = 0;
    val[A + j] = kJointItem | (uint32_t)j;
}
// sort keys: island label (smallest body index of the island) of each active result
template <class R>
__global__ void k_isl_keys(const int* Ad, const int* active, Results<R> res, Bodies<R> B, const int* parent, uint64_t* key, uint32_t* key2,
                           uint32_t* val) {
    const int A = *Ad;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < A; t += gridDim.x * blockDim.x) {
        const int p = active[t];
        const int ia = res.a[p], ib = res.b[p];
        const int dyn = (B.flags[ia] & BF_KINEMATIC) ? ib : ia;
        key[t] = (uint64_t)uf_find(parent, dyn);
        key2[t] = 0;
        val[t] = (uint32_t)p;
    }
}
// M = *Md sorted items (active results, then joints): island starts, and the islands' first slots
__global__ void k_isl_flags(const int* Md, int bound, const uint64_t* key, int* flag);
__global__ void k_isl_offsets(const int* Md, const uint64_t* key, const int* scan, int* isl_off, int* n_isl_out);
__global__ void k_count_add(const int* a, int add, int* out);

// serial order inside each island of up to max_len items, one thread per island, islands in their
// natural order (the island of the smallest body first): consecutive threads take neighbouring
// islands, whose bodies and rows lie close in memory.  (Keeping an island's bodies in registers
// through the iterations, or ordering islands by descending work, both measured slower: the
// first lowers occupancy, the second scatters the threads' memory accesses.)
template <class R>
__global__ void k_isl_serial(const int* n_isl, const int* isl_off, const uint32_t* order, Results<R> res, Joints<R> J, Bodies<R> B,
                             Rows<R> rows, const int* row_off, int iterations, int max_len) {
    const int NI = *n_isl;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < NI; s += gridDim.x * blockDim.x) {
        const int lo = isl_off[s], hi = isl_off[s + 1];
        if (hi - lo > max_len) continue;
        for (int it = 0; it < iterations; it++)
            for (int k = lo; k < hi; k++) iterate_item(order[k], res, J, B, rows, row_off);
    }
}


// coloured Gauss-Seidel of one island at a time per block (the islands of `list`, taken in turn
// through an atomic cursor): greedy colouring in rounds (a result takes
// colour c when it holds the smallest position among the uncoloured results on each of its
// dynamic bodies), then every iteration runs the colours in turn, all results of a colour in
// parallel.  Colour c is then the item's level in the serial order's level schedule, so an island
// coloured in at most kMaxColors - 1 rounds runs exactly the reference's order.  Results still
// uncoloured after kMaxColors - 1 rounds form a last colour that one thread runs in order.
constexpr int kMaxColors = 512;
template <class R>
__global__ void __launch_bounds__(256) k_isl_colored(const int* list, const int* n_list, int* cursor, const int* isl_off, const uint32_t* order,
                                                     Results<R> res, Joints<R> J, Bodies<R> B, Rows<R> rows, const int* row_off,
                                                     int iterations, int min_len, int max_len, int* claim, int* color, uint32_t* corder,
                                                     int* n_colors_out) {
    __shared__ int cnt[kMaxColors + 1];
    __shared__ int fill[kMaxColors];
    __shared__ int remaining;
    __shared__ int ncol;
    __shared__ int slot;
    for (;;) {   // islands from the list, one at a time per block
        if (threadIdx.x == 0) slot = atomicAdd(cursor, 1);
        __syncthreads();
        const int li = slot;
        __syncthreads();
        if (li >= *n_list) break;
        const int s = list[li];
        const int lo = isl_off[s], hi = isl_off[s + 1], m = hi - lo;
        if (m <= min_len || m > max_len) continue;
        for (int j = threadIdx.x; j < m; j += blockDim.x) color[lo + j] = -1;
        if (threadIdx.x == 0) ncol = 0;
        __syncthreads();
        for (int c = 0; c < kMaxColors - 1; c++) {
            for (int j = threadIdx.x; j < m; j += blockDim.x) {
                if (color[lo + j] >= 0) continue;
                const int2 q = item_bodies(order[lo + j], res, J);
                claim[q.x] = 0x7fffffff;
                claim[q.y] = 0x7fffffff;
            }
            if (threadIdx.x == 0) remaining = 0;
            __syncthreads();
            for (int j = threadIdx.x; j < m; j += blockDim.x) {
                if (color[lo + j] >= 0) continue;
                const int2 q = item_bodies(order[lo + j], res, J);
                const int ia = q.x, ib = q.y;
                if (!(B.flags[ia] & BF_KINEMATIC)) atomicMin(&claim[ia], j);
                if (!(B.flags[ib] & BF_KINEMATIC)) atomicMin(&claim[ib], j);
            }
            __syncthreads();
            for (int j = threadIdx.x; j < m; j += blockDim.x) {
                if (color[lo + j] >= 0) continue;
                const int2 q = item_bodies(order[lo + j], res, J);
                const int ia = q.x, ib = q.y;
                const bool da = !(B.flags[ia] & BF_KINEMATIC), db = !(B.flags[ib] & BF_KINEMATIC);
                if ((!da || claim[ia] == j) && (!db || claim[ib] == j)) color[lo + j] = c;
                else atomicAdd(&remaining, 1);
            }
            __syncthreads();
            if (threadIdx.x == 0) ncol = c + 1;
            const int rem = remaining;
            __syncthreads();
            if (rem == 0) break;
        }
        // leftovers (pathological degree): colour nc after the nc rounds' colours, run in island order
        // by one thread; only the colours in use are counted, placed and run
        const int nc = ncol;
        for (int j = threadIdx.x; j < m; j += blockDim.x)
            if (color[lo + j] < 0) color[lo + j] = nc;
        for (int k = threadIdx.x; k <= nc + 1; k += blockDim.x) cnt[k] = 0;
        __syncthreads();
        for (int j = threadIdx.x; j < m; j += blockDim.x) atomicAdd(&cnt[color[lo + j] + 1], 1);
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 0; k <= nc; k++) cnt[k + 1] += cnt[k];   // cnt[c] = first slot of colour c
            atomicMax(n_colors_out, nc + (cnt[nc + 1] > cnt[nc] ? 1 : 0));
        }
        __syncthreads();
        const bool left = cnt[nc + 1] > cnt[nc];
        // placement by colour: the results of a colour touch disjoint dynamic bodies, so their order
        // inside the colour does not matter and they are placed in parallel; the leftovers in order
        for (int k = threadIdx.x; k < nc; k += blockDim.x) fill[k] = cnt[k];
        __syncthreads();
        for (int j = threadIdx.x; j < m; j += blockDim.x) {
            const int c = color[lo + j];
            if (c < nc) corder[lo + atomicAdd(&fill[c], 1)] = order[lo + j];
        }
        if (threadIdx.x == 0 && left) {
            int f = cnt[nc];
            for (int j = 0; j < m; j++)
                if (color[lo + j] == nc) corder[lo + f++] = order[lo + j];
        }
        __syncthreads();
        for (int it = 0; it < iterations; it++) {
            for (int c = 0; c < nc; c++) {
                for (int j = cnt[c] + threadIdx.x; j < cnt[c + 1]; j += blockDim.x) iterate_item(corder[lo + j], res, J, B, rows, row_off);
                __syncthreads();
            }
            if (left) {
                if (threadIdx.x == 0)
                    for (int j = cnt[nc]; j < cnt[nc + 1]; j++) iterate_item(corder[lo + j], res, J, B, rows, row_off);
                __syncthreads();
            }
        }
        __syncthreads();
    }
}

// Serial-order mode for an island of min_len + 1 .. max_len items, in parallel and exact: levels in rounds
// (an item takes level r in the round where it holds the smallest position among the unleveled
// items on each of its dynamic bodies), so every item runs after all lower-position items that
// share a dynamic body with it and before all higher-position ones: each body receives its updates
// in island order, i.e. the reference's order, and items of one level touch disjoint bodies.  Every
// iteration runs the levels in turn with a block barrier between them.  An island that needs more
// than kMaxLevels levels runs in order on one thread instead.
constexpr int kMaxLevels = 256;
constexpr int kLevelBlock = 256;   // the largest block of k_isl_levels
template <class R>
__global__ void __launch_bounds__(kLevelBlock) k_isl_levels(const int* list, const int* n_list, int* cursor, const int* isl_off,
                                                            const uint32_t* order, Results<R> res, Joints<R> J, Bodies<R> B, Rows<R> rows,
                                                            const int* row_off, int iterations, int min_len, int max_len, int* claim,
                                                            int* level, uint32_t* lorder) {
    __shared__ int cnt[kMaxLevels + 1];
    __shared__ int remaining;
    __shared__ int slot;
    for (;;) {   // islands from the list, one at a time per block
        if (threadIdx.x == 0) slot = atomicAdd(cursor, 1);
        __syncthreads();
        const int li = slot;
        __syncthreads();
        if (li >= *n_list) break;
        const int s = list[li];
        const int lo = isl_off[s], hi = isl_off[s + 1], m = hi - lo;
        if (m <= min_len || m > max_len) continue;
        for (int j = threadIdx.x; j < m; j += blockDim.x) level[lo + j] = -1;
        __syncthreads();
        int rem = m;
        for (int r = 0; r < kMaxLevels && rem > 0; r++) {
            for (int j = threadIdx.x; j < m; j += blockDim.x) {
                if (level[lo + j] >= 0) continue;
                const int2 q = item_bodies(order[lo + j], res, J);
                claim[q.x] = 0x7fffffff;
                claim[q.y] = 0x7fffffff;
            }
            if (threadIdx.x == 0) remaining = 0;
            __syncthreads();
            for (int j = threadIdx.x; j < m; j += blockDim.x) {
                if (level[lo + j] >= 0) continue;
                const int2 q = item_bodies(order[lo + j], res, J);
                if (!(B.flags[q.x] & BF_KINEMATIC)) atomicMin(&claim[q.x], j);
                if (!(B.flags[q.y] & BF_KINEMATIC)) atomicMin(&claim[q.y], j);
            }
            __syncthreads();
            for (int j = threadIdx.x; j < m; j += blockDim.x) {
                if (level[lo + j] >= 0) continue;
                const int2 q = item_bodies(order[lo + j], res, J);
                const bool da = !(B.flags[q.x] & BF_KINEMATIC), db = !(B.flags[q.y] & BF_KINEMATIC);
                if ((!da || claim[q.x] == j) && (!db || claim[q.y] == j)) level[lo + j] = r;
                else atomicAdd(&remaining, 1);
            }
            __syncthreads();
            rem = remaining;
            __syncthreads();
        }
        if (rem > 0) {   // too many levels: the island in order on one thread
            if (threadIdx.x == 0)
                for (int it = 0; it < iterations; it++)
                    for (int k = lo; k < hi; k++) iterate_item(order[k], res, J, B, rows, row_off);
            continue;
        }
        for (int k = threadIdx.x; k <= kMaxLevels; k += blockDim.x) cnt[k] = 0;
        __syncthreads();
        int nl = 0;
        for (int j = threadIdx.x; j < m; j += blockDim.x) atomicAdd(&cnt[level[lo + j] + 1], 1);
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 0; k < kMaxLevels; k++) cnt[k + 1] += cnt[k];   // cnt[l] = first slot of level l
            int fill[kMaxLevels];
            for (int k = 0; k < kMaxLevels; k++) fill[k] = cnt[k];
            for (int j = 0; j < m; j++) lorder[lo + fill[level[lo + j]]++] = order[lo + j];
        }
        __syncthreads();
        for (int k = 0; k < kMaxLevels; k++) if (cnt[k + 1] > cnt[k]) nl = k + 1;
        for (int it = 0; it < iterations; it++)
            for (int l = 0; l < nl; l++) {
                for (int j = cnt[l] + threadIdx.x; j < cnt[l + 1]; j += blockDim.x) iterate_item(lorder[lo + j], res, J, B, rows, row_off);
                __syncthreads();
            }
        __syncthreads();
    }
}

// ---- islands above Tuning::big_island_items results: k_isl_colored's colouring rule in grid-wide kernels (round
// c gives colour c to every uncoloured result that holds the smallest island position among the
// uncoloured results on each of its dynamic bodies, so the colour classes follow the island order,
// i.e. the reference's solve order, as closely as colouring allows), with up to kMaxColorsBig
// colours, then one launch per colour and iteration.  Results of a colour touch disjoint dynamic
// bodies, so their order inside the colour does not matter; results left after kMaxColorsBig - 1
// rounds run in island order in one thread.
constexpr int kMaxColorsBig = 1024;
__global__ void k_isl_big(const int* n_isl, const int* isl_off, int* big, int* n_big, int big_items);
__global__ void k_isl_pick(const int* n_isl, const int* isl_off, int min_len, int max_len, int* list, int* n_list);
__global__ void k_step_counters(const int* status, const int* rows, const int* active, const int* islands, const int* big, const int* colors,
                                const int* cls, int* out);
template <class R>
__global__ void k_gc_mask_reset(int lo, int m, const uint32_t* order, Results<R> res, Joints<R> J, unsigned long long* mask) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int2 q = item_bodies(order[lo + j], res, J);
    mask[q.x] = 0ull;
    mask[q.y] = 0ull;
}
template <class R>
__global__ void k_gc_claim(int lo, int m, const uint32_t* order, Results<R> res, Joints<R> J, Bodies<R> B, const int* color, int* claim) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m || color[lo + j] >= 0) return;
    const int2 q = item_bodies(order[lo + j], res, J);
    const int ia = q.x, ib = q.y;
    if (!(B.flags[ia] & BF_KINEMATIC)) atomicMin(&claim[ia], j);
    if (!(B.flags[ib] & BF_KINEMATIC)) atomicMin(&claim[ib], j);
}
// coloured mode (mask given): winners of the round take the smallest colour that no earlier winner
// on either of their dynamic bodies holds (first fit over a 64-bit mask per body; all 64 taken: the
// leftover colour), so an island needs about as many colours as its bodies have contacts, not as
// many as it has rounds.  Serial-order mode (no mask): winners take the round number, the exact
// level schedule of k_isl_levels.  *remaining += results still uncoloured after this round
template <class R>
__global__ void k_gc_assign(int lo, int m, const uint32_t* order, Results<R> res, Joints<R> J, Bodies<R> B, const int* claim, int* color,
                            unsigned long long* mask, int round, int* remaining) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    bool left = false;
    if (j < m && color[lo + j] < 0) {
        const int2 q = item_bodies(order[lo + j], res, J);
        const int ia = q.x, ib = q.y;
        const bool da = !(B.flags[ia] & BF_KINEMATIC), db = !(B.flags[ib] & BF_KINEMATIC);
        if ((!da || claim[ia] == j) && (!db || claim[ib] == j)) {
            if (!mask) {   // levels of the exact serial-order schedule: the round number
                color[lo + j] = round;
            } else {
                const unsigned long long used = (da ? mask[ia] : 0ull) | (db ? mask[ib] : 0ull);
                const int c = used == ~0ull ? kMaxColorsBig - 1 : __ffsll((long long)~used) - 1;
                color[lo + j] = c;
                if (c < 64) {   // winners of a round hold disjoint dynamic bodies
                    if (da) mask[ia] |= 1ull << c;
                    if (db) mask[ib] |= 1ull << c;
                }
            }
        } else {
            left = true;
        }
    }
    const int n = __syncthreads_count(left);
    if (threadIdx.x == 0 && n) atomicAdd(remaining, n);
}
// All colouring rounds of a big island in one cooperative launch.  A round's claim on a body is
// ((kMaxColorsBig - round) << 32 | island position): claims of earlier rounds carry larger tags, so
// the round's smallest position wins without resetting the claims, and a round is two phases (claim,
// then assign) with a grid-wide barrier after each; the round's count of items left (read by every
// thread after the barrier) decides whether another round runs.  The winners are those of
// k_gc_claim / k_gc_assign; *n_rounds receives the rounds run.
template <class R>
__global__ void __launch_bounds__(kBlock) k_gc_rounds(int lo, int m, const uint32_t* order, Results<R> res, Joints<R> J, Bodies<R> B,
                                                      unsigned long long* claim, int* color, unsigned long long* mask, int* left,
                                                      int max_rounds, int* n_rounds, int* level) {
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    __shared__ int bleft;
    const int t = blockIdx.x * blockDim.x + threadIdx.x, T = gridDim.x * blockDim.x;
    for (int j = t; j < m; j += T) {
        const int2 q = item_bodies(order[lo + j], res, J);
        claim[q.x] = ~0ull;
        claim[q.y] = ~0ull;
    }
    grid.sync();
    for (int r = 0; r < max_rounds; r++) {
        const unsigned long long tag = (unsigned long long)(kMaxColorsBig - r) << 32;
        for (int j = t; j < m; j += T) {
            if (color[lo + j] >= 0) continue;
            const int2 q = item_bodies(order[lo + j], res, J);
            if (!(B.flags[q.x] & BF_KINEMATIC)) atomicMin(&claim[q.x], tag | (unsigned)j);
            if (!(B.flags[q.y] & BF_KINEMATIC)) atomicMin(&claim[q.y], tag | (unsigned)j);
        }
        grid.sync();
        if (threadIdx.x == 0) bleft = 0;
        __syncthreads();
        int mine = 0;
        for (int j = t; j < m; j += T) {
            if (color[lo + j] >= 0) continue;
            const int2 q = item_bodies(order[lo + j], res, J);
            const int ia = q.x, ib = q.y;
            const bool da = !(B.flags[ia] & BF_KINEMATIC), db = !(B.flags[ib] & BF_KINEMATIC);
            const unsigned long long key = tag | (unsigned)j;
            if ((!da || claim[ia] == key) && (!db || claim[ib] == key)) {
                if (!mask) {
                    color[lo + j] = r;
                } else {
                    if (level) level[lo + j] = r;   // the exact level, kept beside the first-fit colour
                    const unsigned long long used = (da ? mask[ia] : 0ull) | (db ? mask[ib] : 0ull);
                    const int c = used == ~0ull ? kMaxColorsBig - 1 : __ffsll((long long)~used) - 1;
                    color[lo + j] = c;
                    if (c < 64) {
                        if (da) mask[ia] |= 1ull << c;
                        if (db) mask[ib] |= 1ull << c;
                    }
                }
            } else {
                mine++;
            }
        }
        if (mine) atomicAdd(&bleft, mine);
        __syncthreads();
        if (threadIdx.x == 0 && bleft) atomicAdd(&left[r], bleft);
        grid.sync();
        if (*(volatile int*)&left[r] == 0) {   // the same value for every thread after the barrier
            if (t == 0) *n_rounds = r + 1;
            return;
        }
    }
    if (t == 0) *n_rounds = max_rounds;
}

// colour histogram (leftovers -> the last colour) and placement of every colour but the last
__global__ void k_gc_count(int lo, int m, int* color, int* cnt);
__global__ void k_gc_place(int lo, int m, const int* color, const uint32_t* order, int* cursor, uint32_t* corder);
// All iterations of a big island in one cooperative launch: colour after colour (the items of a
// colour spread over the whole grid), a grid-wide barrier between colours, the leftover colour in
// island order on one thread at the end of each iteration.  The same updates in the same order as
// one launch per colour and iteration, without the launch gaps that dominate when an island has
// hundreds of colours of a few hundred items.
template <class R>
__global__ void __launch_bounds__(kBlock) k_gc_solve(const uint32_t* corder, const int* cstart, const int* ccount, int ncol,
                                                     int iterations, int lo, int m, const uint32_t* order, const int* color, int last,
                                                     Results<R> res, Joints<R> J, Bodies<R> B, Rows<R> rows, const int* row_off) {
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    const int t = blockIdx.x * blockDim.x + threadIdx.x, T = gridDim.x * blockDim.x;
    for (int it = 0; it < iterations; it++) {
        for (int c = 0; c < ncol; c++) {
            const int n = ccount[c];
            if (n == 0) continue;   // the same for every thread
            const uint32_t* list = corder + cstart[c];
            for (int j = t; j < n; j += T) iterate_item(list[j], res, J, B, rows, row_off);
            grid.sync();
        }
        if (last) {
            if (t == 0)
                for (int j = 0; j < m; j++)
                    if (color[lo + j] == kMaxColorsBig - 1) iterate_item(order[lo + j], res, J, B, rows, row_off);
            grid.sync();
        }
    }
}

// one island [lo, lo + m) in order on one thread (a big island whose level schedule ran out of levels)
template <class R>
__global__ void k_isl_one(int lo, int m, const uint32_t* order, Results<R> res, Joints<R> J, Bodies<R> B, Rows<R> rows, const int* row_off,
                          int iterations) {
    for (int it = 0; it < iterations; it++)
        for (int k = lo; k < lo + m; k++) iterate_item(order[k], res, J, B, rows, row_off);
}

// RigidBody::clearTempVelocity (rigidbody.cpp:160-164) at SequentialImpulseSolver::setupSolver
template <class R>
__global__ void k_si_clear(Bodies<R> B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    if (B.flags[i] & BF_KINEMATIC) return;
    B.set_vec(TVX, i, B.vec(VX, i));
    B.set_vec(TWX, i, B.vec(WX, i));
}

// first sorted position of each scene -> offset of its first pair
__global__ void k_scene_pair_off(int n_scenes, const int* scene_off, const int* pair_scan, int n, int* pair_scene_off);
// results with at least one point, compacted
__global__ void k_rows_init(const int* Rd, int bound, const int* npts, int* row_off);
__global__ void k_active_flags(const int* Rd, int bound, const int* npts, int* flag);
__global__ void k_active_compact(const int* Rd, const int* npts, const int* scan, int* active);

// RigidBody::syncTempVelocity (rigidbody.cpp:154-158)
template <class R>
__global__ void k_si_sync(Bodies<R> B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    if (B.flags[i] & BF_KINEMATIC) return;
    B.set_vec(VX, i, B.vec(TVX, i));
    B.set_vec(WX, i, B.vec(TWX, i));
}

} // namespace pe
