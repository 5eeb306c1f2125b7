// World<R> member definitions, part 4: serving, repacking the scenes of a batched world.
#pragma once
#include "pe_world_io.cuh"

namespace pe {

// ------------------------------------------------------------------ serving: scene repacking
namespace {
// kept bodies: field-major gather from the old layout (stride ocap) into the new one (stride ncap)
// scene whose [off[s], off[s + 1]) holds r (the last such s when empty scenes share an offset)
__device__ __forceinline__ int segment_of(const int* off, int ns, int r) {
    int lo = 0, hi = ns;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= r) lo = mid;
        else hi = mid;
    }
    return lo;
}
template <class R>
__global__ void k_repack_bodies(const R* of, int ocap, const int* oshape, const int* oflags, R* nf, int ncap, int* nshape,
                                int* nflags, const int* koff, const int* first, int nk, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int s = segment_of(koff, nk, j);
    const int i = first[s] + j - koff[s];
    for (int k = 0; k < NBF; k++) nf[(size_t)k * ncap + j] = of[(size_t)k * ocap + i];
    nshape[j] = oshape[i];
    nflags[j] = oflags[i];
}
// added bodies: a compact field-major block [NBF x n] placed at new index `at`
template <class R>
__global__ void k_place_bodies(const R* blk, int n, R* nf, int ncap, int at) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    for (int k = 0; k < NBF; k++) nf[(size_t)k * ncap + at + j] = blk[(size_t)k * n + j];
}
// contact-result distance pools: slot t of the new pool comes from the kept scene's old segment
template <class R>
__global__ void k_repack_pool(const R* src, R* dst, const int* new_off, const int* old_start, int ns, int n_slots) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_slots) return;
    const int r = t / kSlots, k = t - r * kSlots;
    const int lo = segment_of(new_off, ns, r);
    dst[t] = src[(size_t)(old_start[lo] + r - new_off[lo]) * kSlots + k];
}
}  // namespace

template <class R>
void World<R>::repack(const int* keep, int n_keep, const SceneData* const* adds, int n_add) {
    PE_CK(cudaStreamSynchronize(st_));
    const int ons = NS_;
    std::vector<int> old_res(ons + 1, 0), old_axis(std::max(ons, 1), 0);
    PE_CK(cudaMemcpy(old_res.data(), res_scene_off_.p, (ons + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    PE_CK(cudaMemcpy(old_axis.data(), scene_axis_.p, ons * sizeof(int), cudaMemcpyDeviceToHost));
    for (int k = 0; k < n_keep; k++)
        if (keep[k] < 0 || keep[k] >= ons) throw std::runtime_error("repack: kept scene index out of range");
    // shapes of the added scenes go to the end of the shape tables
    std::vector<std::vector<int>> smap(n_add);
    for (int a = 0; a < n_add; a++) {
        const SceneData& d = *adds[a];
        for (int sh : d.body_shape)
            if (sh < 0 || sh >= d.n_shapes()) throw std::runtime_error("repack: body shape index out of range");
        append_shapes(d.n_shapes(), d.shape_type.data(), d.shape_param.data(), d.hull_vbeg.data(), d.hull_vcnt.data(),
                      d.hull_fbeg.data(), d.hull_fcnt.data(), d.hull_verts.data(), d.hull_face_off.data(), d.hull_face_idx.data(),
                      &smap[a]);
    }
    // new body layout: kept scenes in order (first old body of each), then the added ones
    std::vector<int> off(1, 0), first;
    for (int k = 0; k < n_keep; k++) {
        const int s = keep[k];
        first.push_back(h_scene_off_[s]);
        off.push_back(off.back() + h_scene_off_[s + 1] - h_scene_off_[s]);
    }
    const int n_kept = off.back();
    int n_new = 0;
    for (int a = 0; a < n_add; a++) { n_new += adds[a]->n_bodies(); off.push_back(n_kept + n_new); }
    const int N = n_kept + n_new, ncap = std::max(N, 1);
    std::vector<R> blk((size_t)NBF * std::max(n_new, 1), R(0));
    std::vector<int> ashape(std::max(n_new, 1)), aflags(std::max(n_new, 1));
    for (int a = 0, j = 0; a < n_add; a++) {
        const SceneData& d = *adds[a];
        for (int i = 0; i < d.n_bodies(); i++, j++) {
            ashape[j] = smap[a][d.body_shape[i]];
            aflags[j] = d.body_flags[i];
            fill_body(blk.data(), n_new, j, ashape[j], d.mass[i], d.friction[i], d.restitution[i], d.lin_damp[i], d.ang_damp[i],
                      &d.origin[(size_t)i * 3], &d.basis[(size_t)i * 9], &d.lin_vel[(size_t)i * 3], &d.ang_vel[(size_t)i * 3]);
        }
    }
    DBuf<R> nf;
    DBuf<int> nshape, nflags, dkoff, dfirst;
    nf.ensure((size_t)NBF * ncap);
    nshape.ensure(ncap + 1);
    nflags.ensure(ncap + 1);
    if (n_kept) {
        upload(dkoff, std::vector<int>(off.begin(), off.begin() + n_keep + 1), st_);
        upload(dfirst, first, st_);
        launch(K_MISC, grid(n_kept), k_repack_bodies<R>, (const R*)bf_.p, bcap_, (const int*)bshape_.p, (const int*)bflags_.p, nf.p,
               ncap, nshape.p, nflags.p, (const int*)dkoff.p, (const int*)dfirst.p, n_keep, n_kept);
    }
    DBuf<R> dblk;
    if (n_new) {
        upload(dblk, blk, st_);
        launch(K_MISC, grid(n_new), k_place_bodies<R>, (const R*)dblk.p, n_new, nf.p, ncap, n_kept);
        PE_CK(cudaMemcpyAsync(nshape.p + n_kept, ashape.data(), n_new * sizeof(int), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(nflags.p + n_kept, aflags.data(), n_new * sizeof(int), cudaMemcpyHostToDevice, st_));
    }
    // contact-result pools of the kept scenes (the current generation becomes the next step's "previous")
    const int ns = n_keep + n_add;
    std::vector<int> new_res(ns + 1, 0), old_start(std::max(ns, 1), 0), axis(std::max(ns, 1), 0);
    for (int k = 0; k < n_keep; k++) {
        const int s = keep[k];
        new_res[k + 1] = new_res[k] + old_res[s + 1] - old_res[s];
        old_start[k] = old_res[s];
        axis[k] = old_axis[s];
    }
    for (int a = 0; a < n_add; a++) new_res[n_keep + a + 1] = new_res[n_keep + a];
    const int T = new_res[ns];
    ensure_pair_capacity(std::max(T, 1));   // grows both pool generations keeping their contents
    if (T) {
        DBuf<int> dnew, dold;
        upload(dnew, new_res, st_);
        upload(dold, old_start, st_);
        launch(K_MISC, grid(T * kSlots), k_repack_pool<R>, (const R*)res_dist_[cur_dist_].p, res_dist_[cur_dist_ ^ 1].p,
               (const int*)dnew.p, (const int*)dold.p, ns, T * kSlots);
        PE_CK(cudaStreamSynchronize(st_));
        cur_dist_ ^= 1;
    }
    PE_CK(cudaStreamSynchronize(st_));
    std::swap(bf_.p, nf.p); std::swap(bf_.n, nf.n);
    std::swap(bshape_.p, nshape.p); std::swap(bshape_.n, nshape.n);
    std::swap(bflags_.p, nflags.p); std::swap(bflags_.n, nflags.n);
    N_ = N;
    bcap_ = ncap;
    claim_.ensure(N + 1);
    // scene tables (as set_scenes), then the kept axes and result offsets
    NS_ = std::max(ns, 1);
    if (ns == 0) off = {0, 0};
    h_scene_off_ = off;
    std::vector<int> sc(std::max(N, 1), 0);
    for (int s = 0; s < ns; s++) for (int i = off[s]; i < off[s + 1]; i++) sc[i] = s;
    upload(bscene_, sc, st_);
    upload(scene_off_, off, st_);
    upload(scene_axis_, axis, st_);
    if (ns == 0) new_res = {0, 0};
    std::vector<int> zero(NS_ + 1, 0);
    upload(pair_scene_off_, zero, st_);
    upload(prev_res_off_, zero, st_);
    upload(res_scene_off_, new_res, st_);
    h_pair_scene_off_ = zero;
    P_ = 0;
    R_ = 0;
    PE_CK(cudaMemsetAsync(dcnt_.p, 0, DC_COUNT * sizeof(int), st_));
    PE_CK(cudaStreamSynchronize(st_));
}

template <class R>
void World<R>::get_state_range(int first, int count, double* o, double* b, double* v, double* w) {
    if (first < 0 || count < 0 || first + count > N_) throw std::runtime_error("state range out of bounds");
    if (!count) return;
    // fields OX..WZ (origin, basis, linear and angular velocity) are 18 consecutive field rows
    R* h = staging((size_t)18 * count);
    PE_CK(cudaMemcpy2DAsync(h, (size_t)count * sizeof(R), bf_.p + first, (size_t)bcap_ * sizeof(R), (size_t)count * sizeof(R), 18,
                            cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
    struct G { double* dst; int k0; int nk; };
    const G groups[4] = {{o, OX, 3}, {b, B00, 9}, {v, VX, 3}, {w, WX, 3}};
    for (const G& g : groups) {
        if (!g.dst) continue;
        for (int k = 0; k < g.nk; k++)
            for (int i = 0; i < count; i++) g.dst[(size_t)i * g.nk + k] = (double)h[(size_t)(g.k0 + k) * count + i];
    }
}

} // namespace pe
