// Kernels of the rigid-body step, part 6: body-state transfer in the C ABI's layout.
#pragma once
#include "pe_k_solver.cuh"

namespace pe {

// Body-state transfer in the C ABI's layout (per field group: nk values per body, body-major) through
// a device staging buffer: the precision and layout change on the device, so the host side is plain
// copies of the caller's arrays.  Group g holds fields k0[g] .. k0[g] + nk[g] - 1 at off[g] values.
// T is the caller's type: double, or float (pe::Real of the reference's default build).
struct XferGroups {
    int k0[8], nk[8];
    size_t off[8];
    int n;
};
template <class R, class T>
__global__ void k_state_pack(Bodies<R> B, XferGroups G, T* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    for (int g = 0; g < G.n; g++)
        for (int k = 0; k < G.nk[g]; k++) out[G.off[g] + (size_t)i * G.nk[g] + k] = (T)B.at(G.k0[g] + k, i);
}
// the inverse; with so, smn, smx >= 0 (the groups of origin, AABB min and max) it also sets the
// body's AABB scale from them, as RigidBody::getAABBScale does (rigidbody.cpp:119-123)
template <class R, class T>
__global__ void k_state_unpack(Bodies<R> B, XferGroups G, const T* in, int so, int smn, int smx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    for (int g = 0; g < G.n; g++)
        for (int k = 0; k < G.nk[g]; k++) B.at(G.k0[g] + k, i) = R(in[G.off[g] + (size_t)i * G.nk[g] + k]);
    if (so >= 0) {
        auto v3 = [&](int g) {
            const T* q = in + G.off[g] + (size_t)i * 3;
            return V3<R>(R(q[0]), R(q[1]), R(q[2]));
        };
        const V3<R> a = v3(smn), d = v3(smx), org = v3(so);
        const R sc = norm(d - a), df = norm(d + a - org * R(2));
        B.at(SCALE, i) = (sc + df) * R(0.5);
    }
}

} // namespace pe
