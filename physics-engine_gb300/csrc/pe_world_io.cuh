// World<R> member definitions, part 3: transfers between the caller's arrays and the device
// (body state, sweep axes, pairs, contact results).
#pragma once
#include "pe_world_step.cuh"

namespace pe {

// ------------------------------------------------------------------ transfers
// The body state moves through a device staging buffer in the caller's layout (k_state_pack /
// k_state_unpack convert precision and layout on the device); pairs copy straight into the caller's
// array, contact results through host vectors (their layout changes on the host), and the serving
// reads of finished scenes through pinned host memory (staging).  These are the host<->device copies
// a drop-in caller pays.
template <class R> R* World<R>::staging(size_t n) {
    if (n > stage_n_) {
        if (stage_) cudaFreeHost(stage_);
        stage_ = nullptr;
        PE_CK(cudaMallocHost(&stage_, n * sizeof(R)));
        stage_n_ = n;
    }
    return stage_;
}

template <class R> template <class T>
void World<R>::get_state_t(T* o, T* b, T* v, T* w, T* mn, T* mx, T* iw) {
    T* dst[7] = {o, b, v, w, mn, mx, iw};
    const int k0[7] = {OX, B00, VX, WX, MNX, MXX, I00}, nk[7] = {3, 9, 3, 3, 3, 3, 9};
    XferGroups G{};
    size_t tot = 0;
    int map[7];
    for (int g = 0; g < 7; g++) {
        if (!dst[g]) continue;
        map[G.n] = g;
        G.k0[G.n] = k0[g]; G.nk[G.n] = nk[g]; G.off[G.n] = tot;
        tot += (size_t)nk[g] * N_;
        G.n++;
    }
    if (!N_ || !G.n) return;
    xfer_.ensure((tot * sizeof(T) + sizeof(double) - 1) / sizeof(double));
    T* x = reinterpret_cast<T*>(xfer_.p);
    launch(K_MISC, grid(N_), k_state_pack<R, T>, bodies(), G, x);
    for (int q = 0; q < G.n; q++)
        PE_CK(cudaMemcpyAsync(dst[map[q]], x + G.off[q], (size_t)G.nk[q] * N_ * sizeof(T), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
}

template <class R> template <class T>
void World<R>::set_state_t(const T* o, const T* b, const T* v, const T* w, const T* mn, const T* mx, const T* iw) {
    const T* src[7] = {o, b, v, w, mn, mx, iw};
    const int k0[7] = {OX, B00, VX, WX, MNX, MXX, I00}, nk[7] = {3, 9, 3, 3, 3, 3, 9};
    XferGroups G{};
    size_t tot = 0;
    int at[7] = {-1, -1, -1, -1, -1, -1, -1};
    for (int g = 0; g < 7; g++) {
        if (!src[g]) continue;
        at[g] = G.n;
        G.k0[G.n] = k0[g]; G.nk[G.n] = nk[g]; G.off[G.n] = tot;
        tot += (size_t)nk[g] * N_;
        G.n++;
    }
    if (!N_ || !G.n) return;
    xfer_.ensure((tot * sizeof(T) + sizeof(double) - 1) / sizeof(double));
    T* x = reinterpret_cast<T*>(xfer_.p);
    for (int g = 0; g < 7; g++)
        if (src[g])
            PE_CK(cudaMemcpyAsync(x + G.off[at[g]], src[g], (size_t)nk[g] * N_ * sizeof(T), cudaMemcpyHostToDevice, st_));
    const bool scale = mn && mx && o;   // the injected box's AABB scale
    launch(K_MISC, grid(N_), k_state_unpack<R, T>, bodies(), G, (const T*)x, scale ? at[0] : -1, scale ? at[4] : -1,
           scale ? at[5] : -1);
    PE_CK(cudaStreamSynchronize(st_));
}

template <class R> void World<R>::get_axes(int* a) {
    PE_CK(cudaMemcpyAsync(a, scene_axis_.p, NS_ * sizeof(int), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
}
template <class R> void World<R>::set_axes(const int* a) {
    PE_CK(cudaMemcpyAsync(scene_axis_.p, a, NS_ * sizeof(int), cudaMemcpyHostToDevice, st_));
    PE_CK(cudaStreamSynchronize(st_));
}

template <class R> void World<R>::get_pairs(int* p) {
    if (P_) PE_CK(cudaMemcpyAsync(p, pairs_.p, (size_t)P_ * sizeof(int2), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
}

// per-scene offsets of a list grouped by scene (scene of its first body)
static std::vector<int> scene_offsets(int n, const int* a, const std::vector<int>& scene_off) {
    const int ns = (int)scene_off.size() - 1;
    std::vector<int> off(ns + 1, 0);
    int s = 0;
    for (int i = 0; i < n; i++) {
        const int b = a[i * 2];
        const int sb = (int)(std::upper_bound(scene_off.begin(), scene_off.end(), b) - scene_off.begin()) - 1;
        if (sb < s) throw std::runtime_error("list must be grouped by scene in scene order");
        while (s < sb) off[++s] = i;
    }
    while (s < ns) off[++s] = n;
    return off;
}

template <class R> void World<R>::set_pairs(int n, const int* p) {
    for (int i = 0; i < 2 * n; i++) if (p[i] < 0 || p[i] >= N_) throw std::runtime_error("pair body index out of range");
    ensure_pair_capacity(std::max(n, 1));
    if (n) PE_CK(cudaMemcpyAsync(pairs_.p, p, (size_t)n * sizeof(int2), cudaMemcpyHostToDevice, st_));
    h_pair_scene_off_ = scene_offsets(n, p, h_scene_off_);
    PE_CK(cudaMemcpyAsync(pair_scene_off_.p, h_pair_scene_off_.data(), (NS_ + 1) * sizeof(int), cudaMemcpyHostToDevice, st_));
    PE_CK(cudaMemcpyAsync(dcnt_.p + DC_P, &n, sizeof(int), cudaMemcpyHostToDevice, st_));
    PE_CK(cudaStreamSynchronize(st_));
    P_ = n;
}

template <class R> void World<R>::get_results(int* a, int* b, int* ps, double* fr, double* re, double* slots) {
    const int P = R_;
    std::vector<int> ha(P), hb(P), hn(P);
    std::vector<R> hfr(P), hre(P), hd((size_t)P * kSlots), pts((size_t)NPF * pair_cap_ * kSlots);
    if (P) {
        PE_CK(cudaMemcpyAsync(ha.data(), res_a_.p, P * sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hb.data(), res_b_.p, P * sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hn.data(), res_np_.p, P * sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hfr.data(), res_fr_.p, P * sizeof(R), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hre.data(), res_re_.p, P * sizeof(R), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hd.data(), res_dist_[cur_dist_].p, hd.size() * sizeof(R), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(pts.data(), res_pts_.p, pts.size() * sizeof(R), cudaMemcpyDeviceToHost, st_));
    }
    PE_CK(cudaStreamSynchronize(st_));
    const size_t stride = (size_t)pair_cap_ * kSlots;
    for (int p = 0; p < P; p++) {
        if (a) a[p] = ha[p];
        if (b) b[p] = hb[p];
        if (ps) ps[p] = hn[p];
        if (fr) fr[p] = hfr[p];
        if (re) re[p] = hre[p];
        if (!slots) continue;
        for (int k = 0; k < kSlots; k++) {
            double* o = slots + ((size_t)p * kSlots + k) * 19;
            for (int q = 0; q < 19; q++) o[q] = 0;
            o[12] = hd[(size_t)p * kSlots + k];
            if (k >= hn[p]) continue;
            const size_t s = (size_t)p * kSlots + k;
            for (int g = 0; g < 4; g++) for (int d = 0; d < 3; d++) o[g * 3 + d] = pts[(size_t)(g * 3 + d) * stride + s];
            for (int g = 4; g < 6; g++) for (int d = 0; d < 3; d++) o[13 + (g - 4) * 3 + d] = pts[(size_t)(g * 3 + d) * stride + s];
        }
    }
}

template <class R>
void World<R>::set_results(int n, const int* a, const int* b, const int* ps, const double* fr, const double* re,
                           const double* slots) {
    ensure_pair_capacity(std::max(n, 1));
    std::vector<int> ab(2 * n);
    for (int i = 0; i < n; i++) {
        if (a[i] < 0 || a[i] >= N_ || b[i] < 0 || b[i] >= N_ || ps[i] < 0 || ps[i] > kSlots)
            throw std::runtime_error("result " + std::to_string(i) + " out of range");
        ab[2 * i] = a[i];
        ab[2 * i + 1] = b[i];
    }
    std::vector<int> off = scene_offsets(n, ab.data(), h_scene_off_);
    std::vector<R> hfr(n), hre(n), hd((size_t)n * kSlots), pts((size_t)NPF * pair_cap_ * kSlots, R(0));
    const size_t stride = (size_t)pair_cap_ * kSlots;
    for (int p = 0; p < n; p++) {
        hfr[p] = R(fr[p]);
        hre[p] = R(re[p]);
        for (int k = 0; k < kSlots; k++) {
            const double* o = slots + ((size_t)p * kSlots + k) * 19;
            const size_t s = (size_t)p * kSlots + k;
            hd[s] = R(o[12]);
            for (int g = 0; g < 4; g++) for (int d = 0; d < 3; d++) pts[(size_t)(g * 3 + d) * stride + s] = R(o[g * 3 + d]);
            for (int g = 4; g < 6; g++) for (int d = 0; d < 3; d++) pts[(size_t)(g * 3 + d) * stride + s] = R(o[13 + (g - 4) * 3 + d]);
        }
    }
    if (n) {
        PE_CK(cudaMemcpyAsync(res_a_.p, a, n * sizeof(int), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_b_.p, b, n * sizeof(int), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_np_.p, ps, n * sizeof(int), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_fr_.p, hfr.data(), n * sizeof(R), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_re_.p, hre.data(), n * sizeof(R), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_dist_[cur_dist_].p, hd.data(), hd.size() * sizeof(R), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_pts_.p, pts.data(), pts.size() * sizeof(R), cudaMemcpyHostToDevice, st_));
    }
    PE_CK(cudaMemcpyAsync(res_scene_off_.p, off.data(), (NS_ + 1) * sizeof(int), cudaMemcpyHostToDevice, st_));
    PE_CK(cudaMemcpyAsync(dcnt_.p + DC_R, &n, sizeof(int), cudaMemcpyHostToDevice, st_));
    PE_CK(cudaStreamSynchronize(st_));
    R_ = n;
}

} // namespace pe
