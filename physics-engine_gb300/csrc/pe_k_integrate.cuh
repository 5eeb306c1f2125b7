// Kernels of the rigid-body step, part 1: integration (RigidBody::step and the world AABB).
#pragma once
#include <cstdint>
#include <cooperative_groups.h>
#include "pe_state.cuh"

namespace pe {

constexpr int kBlock = 256;

// ===================================================================== integration
// World::updateObjectStatus (world.cpp:35-119) + applyExternalForce (:121-127), fused per body.
template <class R>
__global__ void k_integrate(Bodies<R> B, ShapeTable<R> S, StepParams P, int do_move) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    const ShapeView<R> sh = S.view(B.shape[i]);
    const bool kin = (B.flags[i] & BF_KINEMATIC) != 0;
    Xf<R> t = B.xf(i);
    const R dt = R(P.dt);
    if (!kin && do_move) {
        // RigidBody::step (rigidbody.cpp:207-243)
        const V3<R> v = B.vec(VX, i), w = B.vec(WX, i);
        t.o = t.o + v * dt;
        const Quat<R> q = quat_from_basis(t.b);
        const V3<R> dr = w * dt * R(0.5);
        Quat<R> d0;
        d0.x = dr.x; d0.y = dr.y; d0.z = dr.z; d0.w = 0;
        const Quat<R> dq = quat_mul(d0, q);
        Quat<R> qn;
        qn.x = q.x + dq.x; qn.y = q.y + dq.y; qn.z = q.z + dq.z; qn.w = q.w + dq.w;
        quat_normalize(qn);
        t.b = quat_to_basis(qn);
        const M3<R> iw = world_inertia(t.b, B.mat(L00, i));
        B.set_mat(I00, i, iw);
        B.set_vec(OX, i, t.o);
        B.set_mat(B00, i, t.b);
        // applyDamping (rigidbody.cpp:201-204)
        const R ld = pow(R(1.0) - B.at(LDAMP, i), dt), ad = pow(R(1.0) - B.at(ADAMP, i), dt);
        V3<R> nv = v * ld, nw = w * ad;
        // applyExternalForce: force = 0 + g*m, v += force * inv_mass * dt, w += Iw * (torque * dt)
        const R m = B.at(MASS, i), im = B.at(INVM, i);
        const V3<R> force = V3<R>(0, 0, 0) + V3<R>(R(P.g[0]), R(P.g[1]), R(P.g[2])) * m;
        nv = nv + force * im * dt;
        nw = nw + mv(iw, V3<R>(0, 0, 0) * dt);
        B.set_vec(VX, i, nv);
        B.set_vec(WX, i, nw);
    }
    V3<R> mn, mx;
    if (sh.type == ST_COMPOUND) compound_aabb(S, B.shape[i], t, mn, mx);
    else shape_aabb(sh, t, mn, mx);
    B.set_vec(MNX, i, mn);
    B.set_vec(MXX, i, mx);
    // RigidBody::getAABBScale (rigidbody.cpp:119-123)
    const R sc = norm(mx - mn), df = norm(mx + mn - t.o * R(2));
    B.at(SCALE, i) = (sc + df) * R(0.5);
}

// unit direction of every hull edge, normalized(a - b) in the world's real type: the staged SAT
// reads these instead of normalising each edge of both shapes for every pair
template <class R>
__global__ void k_hull_edge_dirs(int n, const R* ea, const R* eb, R* ed) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const V3<R> a(ea[3 * e], ea[3 * e + 1], ea[3 * e + 2]), b(eb[3 * e], eb[3 * e + 1], eb[3 * e + 2]);
    const V3<R> d = normalized(a - b);
    ed[3 * e] = d.x; ed[3 * e + 1] = d.y; ed[3 * e + 2] = d.z;
}

} // namespace pe
