// C ABI (include/pe_gpu.h): status codes, argument checks, exception barrier.
#include <cuda_runtime.h>
#include <cstdio>
#include <new>
#include <string>
#include "../../include/pe_gpu.h"
#include "pe_world.cuh"

struct pe_gpu_world {
    pe::WorldBase* w = nullptr;
    std::string err;
};

namespace {
template <class F> int guard(pe_gpu_world* h, F&& f) {
    if (!h || !h->w) return PE_GPU_ERR_ARG;
    try {
        h->err.clear();
        return f(*h->w);
    } catch (const pe::CudaError& e) {
        h->err = e.what();
        return PE_GPU_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        h->err = "host allocation failed";
        return PE_GPU_ERR_CAPACITY;
    } catch (const std::exception& e) {
        h->err = e.what();
        return PE_GPU_ERR_STATE;
    }
}
}  // namespace

extern "C" {

int pe_gpu_create(const pe_gpu_config* cfg, pe_gpu_world** out) {
    if (!cfg || !out || (cfg->real_bits != 32 && cfg->real_bits != 64)) return PE_GPU_ERR_ARG;
    *out = nullptr;
    auto* h = new (std::nothrow) pe_gpu_world();
    if (!h) return PE_GPU_ERR_CAPACITY;
    try {
        if (cfg->real_bits == 32) h->w = new pe::World<float>(cfg->device);
        else h->w = new pe::World<double>(cfg->device);
    } catch (const std::exception& e) {
        delete h;
        return PE_GPU_ERR_CUDA;
    }
    *out = h;
    return PE_GPU_OK;
}

int pe_gpu_destroy(pe_gpu_world* h) {
    if (!h) return PE_GPU_ERR_ARG;
    delete h->w;
    delete h;
    return PE_GPU_OK;
}

const char* pe_gpu_last_error(const pe_gpu_world* h) { return h ? h->err.c_str() : "null handle"; }

int pe_gpu_set_shapes(pe_gpu_world* h, int n, const int* type, const double* param, const int* vbeg, const int* vcnt,
                      const int* fbeg, const int* fcnt, int hv_n, const double* hv, int hf_n, const int* foff, const int* fidx) {
    if (n < 0 || (n > 0 && (!type || !param || !vbeg || !vcnt || !fbeg || !fcnt))) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_shapes(n, type, param, vbeg, vcnt, fbeg, fcnt, hv_n, hv, hf_n, foff, fidx); return PE_GPU_OK; });
}

int pe_gpu_set_compounds(pe_gpu_world* h, const int* child_beg, const int* child_cnt, int n_children, const int* child_shape,
                         const double* child_origin, const double* child_basis, const double* child_ratio,
                         const double* local_inertia, double* centroid) {
    if (!child_beg || !child_cnt || n_children < 0 ||
        (n_children > 0 && (!child_shape || !child_origin || !child_basis || !child_ratio)))
        return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) {
        w.set_compounds(child_beg, child_cnt, n_children, child_shape, child_origin, child_basis, child_ratio, local_inertia, centroid);
        return PE_GPU_OK;
    });
}

int pe_gpu_set_bodies(pe_gpu_world* h, int n, const int* shape, const int* flags, const double* mass, const double* fr,
                      const double* re, const double* ld, const double* ad, const double* o, const double* b, const double* v,
                      const double* w) {
    if (n < 0 || (n > 0 && (!shape || !flags || !mass || !fr || !re || !ld || !ad || !o || !b || !v || !w))) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& W) { W.set_bodies(n, shape, flags, mass, fr, re, ld, ad, o, b, v, w); return PE_GPU_OK; });
}

int pe_gpu_set_joints(pe_gpu_world* h, int n, const int* type, const int* bodies, const int* flags, const double* params) {
    if (n < 0 || (n > 0 && (!type || !bodies || !flags || !params))) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_joints(n, type, bodies, flags, params); return PE_GPU_OK; });
}

int pe_gpu_set_ignore_pairs(pe_gpu_world* h, int n, const int* pairs) {
    if (n < 0 || (n > 0 && !pairs)) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_ignore_pairs(n, pairs); return PE_GPU_OK; });
}

int pe_gpu_set_scenes(pe_gpu_world* h, int n, const int* off) {
    if (n < 1 || !off) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_scenes(n, off); return PE_GPU_OK; });
}

int pe_gpu_set_params(pe_gpu_world* h, double dt, double gx, double gy, double gz, int iterations) {
    if (!(dt > 0) || iterations < 0) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_params(dt, gx, gy, gz, iterations); return PE_GPU_OK; });
}

int pe_gpu_set_contact_margin(pe_gpu_world* h, double margin) {
    if (!(margin >= 0) || !(margin < 1e30)) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_margin(margin); return PE_GPU_OK; });
}

int pe_gpu_set_step_graphs(pe_gpu_world* h, int on) {
    return guard(h, [&](pe::WorldBase& w) { w.set_step_graphs(on != 0); return PE_GPU_OK; });
}

int pe_gpu_device_name(int device, char* name, int cap) {
    if (!name || cap < 1) return PE_GPU_ERR_ARG;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return PE_GPU_ERR_CUDA;
    std::snprintf(name, (size_t)cap, "%s", prop.name);
    return PE_GPU_OK;
}

int pe_gpu_get_tuning(pe_gpu_world* h, pe_gpu_tuning* out) {
    if (!out) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) {
        const pe::Tuning& t = w.tuning();
        *out = pe_gpu_tuning{t.sat_heavy_cost, t.small_island_items, t.big_island_items, t.color_block, t.level_block,
                             t.exact_levels_colored, t.scene_sort_max, t.side_streams};
        return PE_GPU_OK;
    });
}

int pe_gpu_set_tuning(pe_gpu_world* h, const pe_gpu_tuning* t) {
    if (!t || t->sat_heavy_cost < 1 || t->small_island_items < 0 || t->small_island_items > 64 ||
        t->big_island_items <= t->small_island_items || t->big_island_items > (1 << 24) || t->color_block < 32 ||
        t->color_block > 256 || t->color_block % 32 || t->level_block < 32 || t->level_block > 256 || t->level_block % 32 ||
        t->exact_levels_colored < 0 || t->exact_levels_colored > 1023 || t->scene_sort_max < 0 || t->scene_sort_max > 2048 ||
        t->side_streams < 1 || t->side_streams > 4)
        return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) {
        pe::Tuning& u = w.tuning();
        u.sat_heavy_cost = t->sat_heavy_cost; u.small_island_items = t->small_island_items; u.big_island_items = t->big_island_items;
        u.color_block = t->color_block; u.level_block = t->level_block; u.exact_levels_colored = t->exact_levels_colored;
        u.scene_sort_max = t->scene_sort_max; u.side_streams = t->side_streams;
        return PE_GPU_OK;
    });
}

int pe_gpu_step(pe_gpu_world* h, int n_steps, int mode) {
    if (n_steps < 0 || (mode != PE_GPU_SOLVER_SERIAL_ORDER && mode != PE_GPU_SOLVER_COLORED)) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.step(n_steps, mode); return PE_GPU_OK; });
}

int pe_gpu_integrate(pe_gpu_world* h) { return guard(h, [&](pe::WorldBase& w) { w.integrate(); w.sync(); return PE_GPU_OK; }); }

int pe_gpu_broadphase(pe_gpu_world* h, int* n_pairs) {
    return guard(h, [&](pe::WorldBase& w) { const int p = w.broadphase(); w.sync(); if (n_pairs) *n_pairs = p; return PE_GPU_OK; });
}

int pe_gpu_narrowphase(pe_gpu_world* h) { return guard(h, [&](pe::WorldBase& w) { w.narrowphase(); w.sync(); return PE_GPU_OK; }); }

int pe_gpu_solve(pe_gpu_world* h, int mode) {
    if (mode != PE_GPU_SOLVER_SERIAL_ORDER && mode != PE_GPU_SOLVER_COLORED) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.solve(mode); w.sync(); return PE_GPU_OK; });
}

int pe_gpu_n_bodies(const pe_gpu_world* h) { return h && h->w ? h->w->n_bodies() : PE_GPU_ERR_ARG; }
int pe_gpu_n_pairs(const pe_gpu_world* h) { return h && h->w ? h->w->n_pairs() : PE_GPU_ERR_ARG; }
int pe_gpu_n_results(const pe_gpu_world* h) { return h && h->w ? h->w->n_results() : PE_GPU_ERR_ARG; }

int pe_gpu_get_state(pe_gpu_world* h, double* o, double* b, double* v, double* w, double* mn, double* mx, double* iw) {
    return guard(h, [&](pe::WorldBase& W) { W.get_state(o, b, v, w, mn, mx, iw); return PE_GPU_OK; });
}
int pe_gpu_set_state(pe_gpu_world* h, const double* o, const double* b, const double* v, const double* w, const double* mn,
                     const double* mx, const double* iw) {
    return guard(h, [&](pe::WorldBase& W) { W.set_state(o, b, v, w, mn, mx, iw); return PE_GPU_OK; });
}
int pe_gpu_get_state_f32(pe_gpu_world* h, float* o, float* b, float* v, float* w, float* mn, float* mx, float* iw) {
    return guard(h, [&](pe::WorldBase& W) { W.get_state(o, b, v, w, mn, mx, iw); return PE_GPU_OK; });
}
int pe_gpu_set_state_f32(pe_gpu_world* h, const float* o, const float* b, const float* v, const float* w, const float* mn,
                         const float* mx, const float* iw) {
    return guard(h, [&](pe::WorldBase& W) { W.set_state(o, b, v, w, mn, mx, iw); return PE_GPU_OK; });
}
int pe_gpu_get_axes(pe_gpu_world* h, int* a) {
    if (!a) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.get_axes(a); return PE_GPU_OK; });
}
int pe_gpu_set_axes(pe_gpu_world* h, const int* a) {
    if (!a) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_axes(a); return PE_GPU_OK; });
}
int pe_gpu_get_pairs(pe_gpu_world* h, int* p) {
    if (!p) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.get_pairs(p); return PE_GPU_OK; });
}
int pe_gpu_set_pairs(pe_gpu_world* h, int n, const int* p) {
    if (n < 0 || (n > 0 && !p)) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_pairs(n, p); return PE_GPU_OK; });
}
int pe_gpu_get_results(pe_gpu_world* h, int* a, int* b, int* ps, double* fr, double* re, double* slots) {
    return guard(h, [&](pe::WorldBase& w) { w.get_results(a, b, ps, fr, re, slots); return PE_GPU_OK; });
}
int pe_gpu_set_results(pe_gpu_world* h, int n, const int* a, const int* b, const int* ps, const double* fr, const double* re,
                       const double* slots) {
    if (n < 0 || (n > 0 && (!a || !b || !ps || !fr || !re || !slots))) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.set_results(n, a, b, ps, fr, re, slots); return PE_GPU_OK; });
}
int pe_gpu_phase_times(pe_gpu_world* h, double* ms, int reset) {
    if (!ms) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.phase_times(ms, reset != 0); return PE_GPU_OK; });
}
int pe_gpu_last_counts(pe_gpu_world* h, int* c) {
    if (!c) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.last_counts(c); return PE_GPU_OK; });
}
int pe_gpu_set_profiling(pe_gpu_world* h, int on) {
    return guard(h, [&](pe::WorldBase& w) { w.set_profiling(on != 0); return PE_GPU_OK; });
}
int pe_gpu_kernel_count(void) { return pe::K_COUNT; }
const char* pe_gpu_kernel_name(int k) { return pe::kernel_name(k); }
int pe_gpu_kernel_stats(pe_gpu_world* h, double* ms, long long* launches) {
    if (!ms || !launches) return PE_GPU_ERR_ARG;
    return guard(h, [&](pe::WorldBase& w) { w.kernel_stats(ms, launches); return PE_GPU_OK; });
}
int pe_gpu_sync(pe_gpu_world* h) { return guard(h, [&](pe::WorldBase& w) { w.sync(); return PE_GPU_OK; }); }

}  // extern "C"
