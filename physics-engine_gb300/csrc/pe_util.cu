// Precision-independent device utilities: exclusive scan, stable LSD radix sort passes,
// pair bucketing, and the constant-memory unit meshes.
#include "pe_kernels.cuh"

namespace pe {

// ---------------------------------------------------------------- scan
// tile = kBlock * 4 elements
constexpr int kScanItems = 4;
constexpr int kScanTile = kBlock * kScanItems;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the block total in *total
__device__ int block_excl_scan(int v, int* total) {
    __shared__ int warp_sums[kBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int incl = warp_incl_scan(v);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kBlock / 32 ? warp_sums[lane] : 0;
        w = warp_incl_scan(w);
        if (lane < kBlock / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    const int before = warp == 0 ? 0 : warp_sums[warp - 1];
    *total = warp_sums[kBlock / 32 - 1];
    __syncthreads();
    return before + incl - v;
}

__global__ void k_scan_tiles(int* data, int n, int* aux) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems], s = 0;
    for (int k = 0; k < kScanItems; k++) { v[k] = base + k < n ? data[base + k] : 0; s += v[k]; }
    int total;
    int run = block_excl_scan(s, &total);
    for (int k = 0; k < kScanItems; k++) { if (base + k < n) data[base + k] = run; run += v[k]; }
    if (threadIdx.x == 0) aux[blockIdx.x] = total;
}

// single block: exclusive scan of the m tile totals, grand total into *total
__global__ void k_scan_aux(int* aux, int m, int* total) {
    int carry = 0;
    for (int base = 0; base < m; base += kBlock) {
        const int i = base + threadIdx.x;
        const int v = i < m ? aux[i] : 0;
        int t;
        const int ex = block_excl_scan(v, &t);
        if (i < m) aux[i] = carry + ex;
        carry += t;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int* data, int n, const int* aux) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const int add = aux[blockIdx.x];
    for (int k = 0; k < kScanItems; k++) if (base + k < n) data[base + k] += add;
}

// ---------------------------------------------------------------- small sorts
__global__ void __launch_bounds__(kSceneSortBlock) k_sort_pairs_block(const uint64_t* key, const uint32_t* val, int n0, const int* nd,
                                                                     uint64_t* key_out, uint32_t* val_out) {
    __shared__ uint64_t k[kSceneSortMax];
    __shared__ uint32_t pos[kSceneSortMax];
    const int n = nd ? *nd : n0;
    if (n > kSceneSortMax) return;   // the radix passes sort this count
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < n) { k[i] = key[i]; pos[i] = (uint32_t)i; }
        else { k[i] = ~0ull; pos[i] = 0xffffffffu; }   // padding sorts last
    }
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < P / 2; t += blockDim.x) {
                const int i = 2 * t - (t & (stride - 1)), j = i + stride;
                const bool up = (i & size) == 0;
                const uint64_t ki = k[i], kj = k[j];
                const uint32_t pi = pos[i], pj = pos[j];
                const bool gt = ki > kj || (ki == kj && pi > pj);
                if (gt == up) { k[i] = kj; k[j] = ki; pos[i] = pj; pos[j] = pi; }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) pos[i] = val[pos[i]];   // every read of the input before any write
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) { key_out[i] = k[i]; val_out[i] = pos[i]; }
}

// ---------------------------------------------------------------- radix sort
__device__ __forceinline__ int digit_of(const uint64_t* key, const uint32_t* key2, int i, int shift, int use2) {
    return use2 ? (int)((key2[i] >> shift) & 0xffu) : (int)((key[i] >> shift) & 0xffull);
}

// per-tile digit histogram, stored digit-major: hist[d * n_tiles + tile]
__global__ void k_radix_hist(const uint64_t* key, const uint32_t* key2, int n0, const int* nd, int small, int shift, int use2, int* hist,
                             int n_tiles) {
    __shared__ int cnt[256];
    const int n = nd ? *nd : n0;
    if (n <= small) return;
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kRadixTile;
    for (int r = 0; r < kRadixItems; r++) {
        const int i = base + r * kBlock + threadIdx.x;
        if (i < n) atomicAdd(&cnt[digit_of(key, key2, i, shift, use2)], 1);
    }
    __syncthreads();
    hist[threadIdx.x * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// stable scatter: items of a tile keep their order within each digit
__global__ void k_radix_scatter(const uint64_t* key_in, const uint32_t* key2_in, const uint32_t* val_in, uint64_t* key_out,
                                uint32_t* key2_out, uint32_t* val_out, int n0, const int* nd, int small, int shift, int use2,
                                const int* hist, int n_tiles) {
    __shared__ int base_d[256];          // running output position of each digit for this tile
    const int n = nd ? *nd : n0;
    if (n <= small) return;
    __shared__ int warp_cnt[kBlock / 32][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    base_d[threadIdx.x] = hist[threadIdx.x * n_tiles + blockIdx.x];
    const int tile = blockIdx.x * kRadixTile;
    for (int r = 0; r < kRadixItems; r++) {
        for (int w = 0; w < kBlock / 32; w++) warp_cnt[w][threadIdx.x] = 0;
        __syncthreads();
        const int i = tile + r * kBlock + threadIdx.x;
        const bool live = i < n;
        const int d = live ? digit_of(key_in, key2_in, i, shift, use2) : 256 + lane;   // dead lanes never match live ones
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (live && rank == 0) warp_cnt[warp][d] = __popc(peers);
        __syncthreads();
        // exclusive prefix over warps for each digit (thread = digit)
        {
            int run = 0;
            for (int w = 0; w < kBlock / 32; w++) { const int c = warp_cnt[w][threadIdx.x]; warp_cnt[w][threadIdx.x] = run; run += c; }
            // stash the round total in the digit base after use below
            __syncthreads();
            if (live) {
                const int pos = base_d[d] + warp_cnt[warp][d] + rank;
                key_out[pos] = key_in[i];
                key2_out[pos] = key2_in[i];
                val_out[pos] = val_in[i];
            }
            __syncthreads();
            base_d[threadIdx.x] += run;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- narrowphase bucketing
// pairs grouped by class (order inside a class is free: every pair's result has its own slot);
// one atomic per class present in a warp.  The pair count is on the device; whole warps stride
// over it (the loop bound is block-uniform, so every lane takes part in the warp votes).
__global__ void k_np_bucket(const int* Pd, const int* cls, int* cursor, int* order) {
    const int P = *Pd;
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < P; base += gridDim.x * blockDim.x) {
        const int p = base + threadIdx.x;
        const int c = p < P ? cls[p] : -1 - lane;
        const unsigned peers = __match_any_sync(0xffffffffu, c);
        const int leader = __ffs(peers) - 1;
        int b = 0;
        if (c >= 0 && lane == leader) b = atomicAdd(&cursor[c], __popc(peers));
        b = __shfl_sync(0xffffffffu, b, leader);
        if (c >= 0) order[b + __popc(peers & ((1u << lane) - 1u))] = p;
    }
}

// class ranges from the class counts (one thread): range[c] = [first, end) of class c in the
// bucketed order, the bucketing cursors at each class's first slot, and the work cursors of the
// kernels that hand pairs out one at a time (they start at the class's first slot)
__global__ void k_np_ranges(const int* count, int* cursor, int2* range, int* work) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int run = 0;
    for (int c = 0; c < PC_COUNT; c++) {
        range[c] = make_int2(run, run + count[c]);
        cursor[c] = run;
        work[c] = run;
        run += count[c];
    }
}

} // namespace pe

namespace pe {

__global__ void k_scene_pair_off(int n_scenes, const int* scene_off, const int* pair_scan, int n, int* pair_scene_off) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > n_scenes) return;
    pair_scene_off[s] = pair_scan[scene_off[s]];
}

// rows of each result before the scan: its point count; zero from the result count up to `bound`
__global__ void k_rows_init(const int* Rd, int bound, const int* npts, int* row_off) {
    const int P = *Rd;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= bound; p += gridDim.x * blockDim.x) row_off[p] = p < P ? npts[p] : 0;
}

// 1 for the results with points, 0 from the result count up to `bound`
__global__ void k_active_flags(const int* Rd, int bound, const int* npts, int* flag) {
    const int P = *Rd;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= bound; p += gridDim.x * blockDim.x) flag[p] = p < P && npts[p] > 0 ? 1 : 0;
}

__global__ void k_active_compact(const int* Rd, const int* npts, const int* scan, int* active) {
    const int P = *Rd;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x)
        if (npts[p] > 0) active[scan[p]] = p;
}

// *out = *a + add (one thread)
__global__ void k_count_add(const int* a, int add, int* out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *out = *a + add;
}

__global__ void k_isl_init(int n, int* parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) parent[i] = i;
}

// island starts among the M = *Md sorted items; 0 from M up to `bound`
__global__ void k_isl_flags(const int* Md, int bound, const uint64_t* key, int* flag) {
    const int M = *Md;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= bound; k += gridDim.x * blockDim.x)
        flag[k] = k < M && (k == 0 || key[k] != key[k - 1]) ? 1 : 0;
}

// after an exclusive scan of the flags: island id = scan value at each island's first slot
__global__ void k_isl_offsets(const int* Md, const uint64_t* key, const int* scan, int* isl_off, int* n_isl_out) {
    const int M = *Md;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= M; k += gridDim.x * blockDim.x) {
        if (k < M && (k == 0 || key[k] != key[k - 1])) isl_off[scan[k]] = k;
        if (k == M) { isl_off[scan[M]] = M; *n_isl_out = scan[M]; }
    }
}

// islands with more than big_items results
__global__ void k_isl_big(const int* n_isl, const int* isl_off, int* big, int* n_big, int big_items) {
    const int NI = *n_isl;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < NI; s += gridDim.x * blockDim.x)
        if (isl_off[s + 1] - isl_off[s] > big_items) big[atomicAdd(n_big, 1)] = s;
}

// the step's counters gathered for one copy to the host (World::HostStat order; colours may be absent)
__global__ void k_step_counters(const int* status, const int* rows, const int* active, const int* islands, const int* big, const int* colors,
                                const int* cls, int* out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    out[0] = *status;
    out[1] = *rows;
    out[2] = *active;
    out[3] = *islands;
    out[4] = *big;
    out[5] = colors ? *colors : 0;
    out[6] = 0;
    for (int c = 0; c < PC_COUNT; c++) out[7 + c] = cls[c];
}

// islands of min_len + 1 .. max_len results (any order: islands share no dynamic body)
__global__ void k_isl_pick(const int* n_isl, const int* isl_off, int min_len, int max_len, int* list, int* n_list) {
    const int NI = *n_isl;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < NI; s += gridDim.x * blockDim.x) {
        const int m = isl_off[s + 1] - isl_off[s];
        if (m > min_len && m <= max_len) list[atomicAdd(n_list, 1)] = s;
    }
}

// colour histogram of an island (cnt[c + 1] counts colour c); uncoloured results join the last colour
__global__ void k_gc_count(int lo, int m, int* color, int* cnt) {
    __shared__ int h[kMaxColorsBig];
    for (int k = threadIdx.x; k < kMaxColorsBig; k += blockDim.x) h[k] = 0;
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) {
        int c = color[lo + j];
        if (c < 0) { c = kMaxColorsBig - 1; color[lo + j] = c; }
        atomicAdd(&h[c], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kMaxColorsBig; k += blockDim.x)
        if (h[k]) atomicAdd(&cnt[k + 1], h[k]);
}

// results of every colour but the last, grouped by colour (any order inside a colour)
__global__ void k_gc_place(int lo, int m, const int* color, const uint32_t* order, int* cursor, uint32_t* corder) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int c = j < m ? color[lo + j] : -1 - lane;
    const bool live = c >= 0 && c < kMaxColorsBig - 1;
    const int key = live ? c : -1 - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (live && lane == leader) base = atomicAdd(&cursor[c], __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (live) corder[base + __popc(peers & ((1u << lane) - 1u))] = order[lo + j];
}

// exclusive offsets of the crowded positions' chunks (few positions: one thread)
__global__ void k_bp_chunk_offsets(const int* n_big, const int* nchunk, int* choff, int* total) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int run = 0;
    for (int b = 0; b < *n_big; b++) { choff[b] = run; run += nchunk[b]; }
    *total = run;
}
__global__ void k_bp_chunk_sums(const int* big, const int* n_big, const int* choff, const int* nchunk, const int* ccount, int* cpref,
                                int* count) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < *n_big; b += gridDim.x * blockDim.x) {
        int run = 0;
        for (int k = choff[b]; k < choff[b] + nchunk[b]; k++) { cpref[k] = run; run += ccount[k]; }
        count[big[b]] = run;
    }
}


} // namespace pe
