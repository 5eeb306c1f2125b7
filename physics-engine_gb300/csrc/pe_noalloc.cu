// Sweep-and-prune pair query that allocates no device memory (pe_gpu_sap_pairs_noalloc).
//
// Same kernels and the same pair order as the world's broadphase (BroadPhaseSweepAndPrune::
// calcCollisionPairs, broad_phase_sweep_and_prune.cpp:6-41, with validateCollisionPair,
// broad_phase_base.cpp:5-19) for one scene of at most kSapMaxBodies bodies, but every temporary
// (sort keys, sorted AABBs, counts, scan totals) lives in one file-scope __device__ array.  The
// array comes into existence when the CUDA module is loaded into the device's context; its
// address is looked up with cudaGetSymbolAddress once per device and context and cached (a
// cudaDeviceReset gives the device a new primary context, and the address is looked up again).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include "../../include/pe_gpu.h"
#include "pe_kernels.cuh"

namespace pe {
namespace {

constexpr int kSapMaxBodies = 16384;
// no window of a scene this small can exceed the world's crowded-window threshold, so the warp
// sweep alone gives the world's pairs (the block sweeps of crowded windows never have work here)
static_assert(kSapMaxBodies <= kBigWindow, "crowded-window sweeps would be needed");
constexpr size_t kAlign = 256;
constexpr size_t al(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }
constexpr int kSapTiles = (kSapMaxBodies + kRadixTile - 1) / kRadixTile;
constexpr int kSapAux = (256 * kSapTiles + 1023) / 1024 + (kSapMaxBodies + 1 + 1023) / 1024 + 2;

// byte layout of the scratch array
struct SapLayout {
    size_t key[2], key2[2], val[2], hist, aux, total, axis, status, nbig, smn, smx, sflag, sscene, count, stage, big, end;
};
constexpr SapLayout sap_layout() {
    SapLayout L{};
    size_t o = 0;
    const size_t n = kSapMaxBodies;
    for (int k = 0; k < 2; k++) { L.key[k] = o; o += al(n * 8); }
    for (int k = 0; k < 2; k++) { L.key2[k] = o; o += al(n * 4); }
    for (int k = 0; k < 2; k++) { L.val[k] = o; o += al(n * 4); }
    L.hist = o; o += al((256 * kSapTiles + 1) * 4);
    L.aux = o; o += al(kSapAux * 4);
    L.total = o; o += al(4);
    L.axis = o; o += al(4);
    L.status = o; o += al(4);
    L.nbig = o; o += al(4);
    L.smn = o; o += al(3 * n * 4);
    L.smx = o; o += al(3 * n * 4);
    L.sflag = o; o += al(n * 4);
    L.sscene = o; o += al(n * 4);
    L.count = o; o += al((n + 1) * 4);
    L.stage = o; o += al(n * kStage * 4);
    L.big = o; o += al(n * 4);
    L.end = o;
    return L;
}
constexpr SapLayout kL = sap_layout();
constexpr size_t kSapScratchBytes = kL.end;   // about 1.4 MB
static_assert(kSapScratchBytes <= (size_t)2 << 20, "scratch budget");

__device__ __align__(256) unsigned char g_sap_scratch[kSapScratchBytes];

// sort keys of the bodies (AABB minimum along the axis, as in k_bp_keys); also the per-call
// values that must start known: the scene axis, one scene id for every key
__global__ void k_sap_keys(int n, const float* mn, int axis, uint64_t* key, uint32_t* key2, uint32_t* val, int* scene_axis) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) scene_axis[0] = axis;
    if (i >= n) return;
    key[i] = order_bits(mn[3 * i + axis]);
    key2[i] = 0u;
    val[i] = (uint32_t)i;
}

// sorted copies of the sweep inputs (as k_bp_gather); zeroes the scan's last count, the status and
// the count of crowded positions
__global__ void k_sap_gather(int n, const float* mn, const float* mx, const int* flags, const uint32_t* order, float* smn,
                             float* smx, int* sflag, int* sscene, int* count, int* status, int* n_big) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) { count[n] = 0; *status = 0; *n_big = 0; }
    if (k >= n) return;
    const int i = (int)order[k];
    for (int d = 0; d < 3; d++) {
        smn[(size_t)d * n + k] = mn[3 * i + d];
        smx[(size_t)d * n + k] = mx[3 * i + d];
    }
    sflag[k] = flags ? flags[i] : 0;
    sscene[k] = 0;
}

__global__ void k_sap_total(const int* total, int* n_pairs) { *n_pairs = *total; }

std::mutex g_setup_mu;
struct ScratchSlot {
    void* ctx = nullptr;   // the context the address belongs to
    void* ptr = nullptr;
};
ScratchSlot g_scratch[64];

// the current context (driver API, reached through the runtime so the library needs no -lcuda)
using CtxGetCurrent = CUresult (*)(CUcontext*);
CtxGetCurrent ctx_get_current() {
    static CtxGetCurrent fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrent>(f);
    }();
    return fn;
}

void set_err(char* err, int cap, const char* msg) {
    if (err && cap > 0) {
        std::strncpy(err, msg, (size_t)cap - 1);
        err[cap - 1] = '\0';
    }
}

}  // namespace
}  // namespace pe

extern "C" int pe_gpu_sap_pairs_noalloc(int device, int n, const float* aabb_min, const float* aabb_max, const int* flags, int axis,
                                        int* pairs, int pair_cap, int* n_pairs, void* stream, char* err, int err_cap) {
    using namespace pe;
    char msg[160];
    if (n < 0 || axis < 0 || axis > 2 || pair_cap < 0 || !n_pairs || (n > 0 && (!aabb_min || !aabb_max)) ||
        (pair_cap > 0 && !pairs) || device < 0 || device >= 64) {
        set_err(err, err_cap, "pe_gpu_sap_pairs_noalloc: bad argument");
        return PE_GPU_ERR_ARG;
    }
    // the kernels store pairs as 8-byte (int2) words and read 4-byte words everywhere else
    auto misaligned = [](const void* q, uintptr_t a) { return q && (reinterpret_cast<uintptr_t>(q) % a) != 0; };
    if (misaligned(pairs, 8) || misaligned(aabb_min, 4) || misaligned(aabb_max, 4) || misaligned(flags, 4) ||
        misaligned(n_pairs, 4)) {
        set_err(err, err_cap, "pe_gpu_sap_pairs_noalloc: misaligned pointer (pairs needs 8 bytes, the others 4)");
        return PE_GPU_ERR_ARG;
    }
    if (n > kSapMaxBodies) {
        std::snprintf(msg, sizeof msg, "pe_gpu_sap_pairs_noalloc: %d bodies exceed the fixed scratch limit of %d", n, kSapMaxBodies);
        set_err(err, err_cap, msg);
        return PE_GPU_ERR_CAPACITY;
    }
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) { set_err(err, err_cap, "cudaGetDevice failed"); return PE_GPU_ERR_CUDA; }
    if (prev != device && cudaSetDevice(device) != cudaSuccess) { set_err(err, err_cap, "cudaSetDevice failed"); return PE_GPU_ERR_CUDA; }
    auto done = [&](int rc, const char* what, cudaError_t e) {
        if (what) {
            std::snprintf(msg, sizeof msg, "pe_gpu_sap_pairs_noalloc: %s: %s", what, cudaGetErrorString(e));
            set_err(err, err_cap, msg);
        }
        if (prev != device) cudaSetDevice(prev);
        return rc;
    };
    // an error left by earlier, unrelated work would otherwise be reported as this call's
    cudaGetLastError();
    // set-up, once per device and context, with that device current
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        CUcontext ctx = nullptr;
        CtxGetCurrent get = ctx_get_current();
        if (get && get(&ctx) == CUDA_SUCCESS && !ctx) {   // no context current yet: the device's primary context
            const cudaError_t e = cudaSetDevice(device);
            if (e != cudaSuccess) return done(PE_GPU_ERR_CUDA, "cudaSetDevice", e);
            get(&ctx);
        }
        if (!get || !ctx) return done(PE_GPU_ERR_CUDA, "no current context", cudaErrorDeviceUninitialized);
        ScratchSlot& slot = g_scratch[device];
        if (!slot.ptr || slot.ctx != static_cast<void*>(ctx)) {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_sap_scratch);
            if (e != cudaSuccess || !p) return done(PE_GPU_ERR_CUDA, "cudaGetSymbolAddress", e);
            slot.ptr = p;
            slot.ctx = static_cast<void*>(ctx);
        }
        base = static_cast<unsigned char*>(slot.ptr);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n < 2) {   // no pair (the world's broadphase returns before sorting below two bodies)
        const cudaError_t e = cudaMemsetAsync(n_pairs, 0, sizeof(int), st);
        if (e != cudaSuccess) return done(PE_GPU_ERR_CUDA, "cudaMemsetAsync", e);
        return done(PE_GPU_OK, nullptr, cudaSuccess);
    }
    uint64_t* key[2] = {reinterpret_cast<uint64_t*>(base + kL.key[0]), reinterpret_cast<uint64_t*>(base + kL.key[1])};
    uint32_t* key2[2] = {reinterpret_cast<uint32_t*>(base + kL.key2[0]), reinterpret_cast<uint32_t*>(base + kL.key2[1])};
    uint32_t* val[2] = {reinterpret_cast<uint32_t*>(base + kL.val[0]), reinterpret_cast<uint32_t*>(base + kL.val[1])};
    int* hist = reinterpret_cast<int*>(base + kL.hist);
    int* aux = reinterpret_cast<int*>(base + kL.aux);
    int* total = reinterpret_cast<int*>(base + kL.total);
    int* scene_axis = reinterpret_cast<int*>(base + kL.axis);
    int* status = reinterpret_cast<int*>(base + kL.status);
    float* smn = reinterpret_cast<float*>(base + kL.smn);
    float* smx = reinterpret_cast<float*>(base + kL.smx);
    int* sflag = reinterpret_cast<int*>(base + kL.sflag);
    int* sscene = reinterpret_cast<int*>(base + kL.sscene);
    int* count = reinterpret_cast<int*>(base + kL.count);
    int* stage = reinterpret_cast<int*>(base + kL.stage);
    int* big = reinterpret_cast<int*>(base + kL.big);
    int* n_big = reinterpret_cast<int*>(base + kL.nbig);

    const int g = (n + kBlock - 1) / kBlock;
    k_sap_keys<<<g, kBlock, 0, st>>>(n, aabb_min, axis, key[0], key2[0], val[0], scene_axis);
    // stable LSD radix sort of the 32-bit keys (as World::radix_sort_keys)
    const int tiles = (n + kRadixTile - 1) / kRadixTile;
    int cur = 0;
    for (int shift = 0; shift < 32; shift += 8) {
        k_radix_hist<<<tiles, kBlock, 0, st>>>(key[cur], key2[cur], n, nullptr, -1, shift, 0, hist, tiles);
        const int m = 256 * tiles, ht = (m + 1023) / 1024;
        k_scan_tiles<<<ht, kBlock, 0, st>>>(hist, m, aux);
        k_scan_aux<<<1, kBlock, 0, st>>>(aux, ht, total);
        k_scan_add<<<ht, kBlock, 0, st>>>(hist, m, aux);
        k_radix_scatter<<<tiles, kBlock, 0, st>>>(key[cur], key2[cur], val[cur], key[cur ^ 1], key2[cur ^ 1], val[cur ^ 1], n, nullptr, -1, shift, 0,
                                                 hist, tiles);
        cur ^= 1;
    }
    const uint32_t* order = val[cur];
    k_sap_gather<<<g, kBlock, 0, st>>>(n, aabb_min, aabb_max, flags, order, smn, smx, sflag, sscene, count, status, n_big);
    const int gw = (int)(((size_t)n * 32 + kBlock - 1) / kBlock);
    const IgnoreLists no_lists;   // this entry point takes no ignored-pair lists
    k_bp_count<float><<<gw, kBlock, 0, st>>>(n, scene_axis, smn, smx, sflag, sscene, count, stage, big, n_big, no_lists);
    const int ct = (n + 1 + 1023) / 1024;
    k_scan_tiles<<<ct, kBlock, 0, st>>>(count, n + 1, aux);
    k_scan_aux<<<1, kBlock, 0, st>>>(aux, ct, total);
    k_scan_add<<<ct, kBlock, 0, st>>>(count, n + 1, aux);
    k_bp_write<float><<<gw, kBlock, 0, st>>>(n, scene_axis, smn, smx, sflag, sscene, order, count, stage, reinterpret_cast<int2*>(pairs),
                                             pair_cap, status, no_lists);
    k_sap_total<<<1, 1, 0, st>>>(total, n_pairs);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return done(PE_GPU_ERR_CUDA, "kernel launch", e);
    return done(PE_GPU_OK, nullptr, cudaSuccess);
}
