// Kernels of the rigid-body step, part 2: scan, the LSD radix sort and the sweep-and-prune broadphase.
#pragma once
#include "pe_k_integrate.cuh"

namespace pe {

// ===================================================================== scan
// exclusive scan of n ints, in place, three phases; totals of each tile in aux
__global__ void k_scan_tiles(int* data, int n, int* aux);
__global__ void k_scan_aux(int* aux, int m, int* total);
__global__ void k_scan_add(int* data, int n, const int* aux);
constexpr int kSmallScanTiles = 16;   // scans of up to 16 tiles of 1024 run in one block (k_scan_aux in place)

// ===================================================================== radix sort
// Sort (key, value) pairs by a 64-bit key and then, more significantly, by a 32-bit
// secondary key (scene id); stable, least-significant digit first, 8-bit digits.
constexpr int kRadixItems = 16;                      // items per thread per tile
constexpr int kRadixTile = kBlock * kRadixItems;     // 4096 items per tile
// The item count is n, or *nd when nd is set (a count the device computed: the grid then covers an
// upper bound, tiles past the count do nothing, and with `small` >= 0 the passes do nothing at all
// when the count is at most `small`, the inputs that k_sort_pairs_block sorts instead).
__global__ void k_radix_hist(const uint64_t* key, const uint32_t* key2, int n, const int* nd, int small, int shift, int use2, int* hist,
                             int n_tiles);
// a sort of n <= kSceneSortMax (key, value) pairs inside one block (bitonic over (key, position)): the
// order of the stable LSD radix sort, in one launch instead of five per pass, for small inputs.  With
// nd set the count is *nd and the kernel does nothing when it is above kSceneSortMax; the output
// may be the input (all reads precede all writes).
__global__ void k_sort_pairs_block(const uint64_t* key, const uint32_t* val, int n, const int* nd, uint64_t* key_out, uint32_t* val_out);
__global__ void k_radix_scatter(const uint64_t* key_in, const uint32_t* key2_in, const uint32_t* val_in, uint64_t* key_out,
                                uint32_t* key2_out, uint32_t* val_out, int n, const int* nd, int small, int shift, int use2,
                                const int* hist, int n_tiles);

__device__ inline uint64_t order_bits(float x) {
    if (x == 0.0f) x = 0.0f;   // -0 and +0 compare equal: give them one key
    const uint32_t u = __float_as_uint(x);
    return (uint64_t)((u & 0x80000000u) ? ~u : (u | 0x80000000u));
}
__device__ inline uint64_t order_bits(double x) {
    if (x == 0.0) x = 0.0;
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

// sort key of each body: its AABB minimum along its scene's sweep axis
template <class R>
__global__ void k_bp_keys(Bodies<R> B, const int* scene_axis, uint64_t* key, uint32_t* key2, uint32_t* val) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    const int ax = scene_axis[B.scene[i]];
    key[i] = order_bits(B.at(MNX + ax, i));
    key2[i] = (uint32_t)B.scene[i];
    val[i] = (uint32_t)i;
}

// Sort of every scene's bodies by the AABB minimum along the scene's axis, one block per scene of
// at most kSceneSortMax bodies: a bitonic sort in shared memory of (key, body index) pairs, whose
// order, ties by body index, is the stable LSD radix sort's.  Replaces the radix passes (four
// per key byte plus one per scene-id byte, five launches each) when every scene fits a block.
constexpr int kSceneSortMax = 2048;
constexpr int kSceneSortBlock = 512;
template <class R>
__global__ void __launch_bounds__(kSceneSortBlock) k_bp_sort_scenes(Bodies<R> B, const int* scene_axis, const int* scene_off,
                                                                   uint32_t* order) {
    __shared__ uint64_t key[kSceneSortMax];
    __shared__ uint32_t idx[kSceneSortMax];
    const int s = blockIdx.x;
    const int lo = scene_off[s], cnt = scene_off[s + 1] - lo;
    if (cnt <= 0) return;   // whole block
    int P = 1;
    while (P < cnt) P <<= 1;
    const int ax = scene_axis[s];
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
        if (k < cnt) { key[k] = order_bits(B.at(MNX + ax, lo + k)); idx[k] = (uint32_t)k; }
        else { key[k] = ~0ull; idx[k] = 0xffffffffu; }   // padding sorts last
    }
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < P / 2; t += blockDim.x) {
                const int i = 2 * t - (t & (stride - 1)), j = i + stride;   // the t-th pair of this stage
                const bool up = (i & size) == 0;
                const uint64_t ki = key[i], kj = key[j];
                const uint32_t ii = idx[i], ij = idx[j];
                const bool gt = ki > kj || (ki == kj && ii > ij);
                if (gt == up) { key[i] = kj; key[j] = ki; idx[i] = ij; idx[j] = ii; }
            }
            __syncthreads();
        }
    }
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) order[lo + k] = (uint32_t)lo + idx[k];
}

// sorted copy of the sweep inputs (coalesced reads in the sweep)
template <class R>
__global__ void k_bp_gather(Bodies<R> B, const uint32_t* order, R* smn, R* smx, int* sflag, int* sscene) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= B.n) return;
    const int i = (int)order[k];
    for (int d = 0; d < 3; d++) {
        smn[(size_t)d * B.n + k] = B.at(MNX + d, i);
        smx[(size_t)d * B.n + k] = B.at(MXX + d, i);
    }
    sflag[k] = B.flags[i];
    sscene[k] = B.scene[i];
}

// BroadPhaseSweepAndPrune::calcCollisionPairs sweep (broad_phase_sweep_and_prune.cpp:24-35)
// with BroadPhaseBase::validateCollisionPair (broad_phase_base.cpp:5-19).
//
// One warp per sorted position i; the lanes test candidates j = i+1+lane, i+33+lane, ... with
// coalesced loads of the sorted AABBs.  The reference stops at the first j whose minimum along
// the axis exceeds i's maximum; minima are sorted, so the lanes still in range form a prefix and
// the warp stops after the first chunk that is not full.  Overlapping partners are compacted in
// ascending j with a ballot and a prefix popcount, which is the reference's pair order.
// Pass 0 counts the pairs of each position and keeps its first kStage partners; pass 1 writes the
// pairs at the scanned offsets, copying staged partners and re-sweeping only crowded positions.
constexpr int kStage = 4;
template <class R, bool WRITE>
__device__ __forceinline__ int sweep_warp(int i, int n, int lane, const int* scene_axis, const R* smn, const R* smx,
                                          const int* sflag, const int* sscene, int* stage, int2* out, const uint32_t* order,
                                          const IgnoreLists& ign) {
    const int sc = sscene[i];
    const int ax = scene_axis[sc];
    const R* amin = smn + (size_t)ax * n;
    const R maxi_ax = smx[(size_t)ax * n + i];
    const R mnx = smn[i], mny = smn[n + i], mnz = smn[2 * (size_t)n + i];
    const R mxx = smx[i], mxy = smx[n + i], mxz = smx[2 * (size_t)n + i];
    const int fi = sflag[i];
    if (fi & BF_IGNORE) return 0;
    const int a = WRITE ? (int)order[i] : 0;
    const unsigned lt = (1u << lane) - 1u;
    int c = 0;
    for (int j0 = i + 1; j0 < n; j0 += 32) {
        const int j = j0 + lane;
        const bool in = j < n && !(amin[j] > maxi_ax) && sscene[j] == sc;
        const unsigned live = __ballot_sync(0xffffffffu, in);
        bool hit = false;
        if (in) {
            const int fj = sflag[j];
            hit = !(fj & BF_IGNORE) && !((fi & BF_KINEMATIC) && (fj & BF_KINEMATIC)) &&
                  !(mnx > smx[j] || smn[j] > mxx) && !(mny > smx[n + j] || smn[n + j] > mxy) &&
                  !(mnz > smx[2 * (size_t)n + j] || smn[2 * (size_t)n + j] > mxz);
            if (hit && ign.off && ((fi | fj) & BF_IGN_LIST)) hit = !ign.ignored(i, j);
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int k = c + __popc(m & lt);
            if (WRITE) out[k] = make_int2(a, (int)order[j]);
            else if (k < kStage) stage[(size_t)i * kStage + k] = j;
        }
        c += __popc(m);
        if (live != 0xffffffffu) break;
    }
    return c;
}

// A position whose window along the axis holds more than kBigWindow candidates (a floor or a wall
// spanning the scene) is swept by a whole block instead of a warp: 256 candidates per iteration,
// warp ballots plus a block prefix of the warp counts keep the pairs in ascending j.
constexpr int kBigWindow = 32768;
template <class R>
__device__ __forceinline__ bool big_window(int i, int n, const int* scene_axis, const R* smn, const R* smx, const int* sscene) {
    const int j = i + kBigWindow;
    if (j >= n) return false;
    const int sc = sscene[i], ax = scene_axis[sc];
    return sscene[j] == sc && !(smn[(size_t)ax * n + j] > smx[(size_t)ax * n + i]);
}
template <class R, bool WRITE>
__device__ int sweep_block(int i, int n, const int* scene_axis, const R* smn, const R* smx, const int* sflag, const int* sscene,
                           int2* out, const uint32_t* order, int* wcnt, const IgnoreLists& ign) {
    const int sc = sscene[i];
    const int ax = scene_axis[sc];
    const R* amin = smn + (size_t)ax * n;
    const R maxi_ax = smx[(size_t)ax * n + i];
    const R mnx = smn[i], mny = smn[n + i], mnz = smn[2 * (size_t)n + i];
    const R mxx = smx[i], mxy = smx[n + i], mxz = smx[2 * (size_t)n + i];
    const int fi = sflag[i];
    if (fi & BF_IGNORE) return 0;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
    const int a = WRITE ? (int)order[i] : 0;
    const unsigned lt = (1u << lane) - 1u;
    int c = 0;
    for (int j0 = i + 1; j0 < n; j0 += blockDim.x) {
        const int j = j0 + tid;
        const bool in = j < n && !(amin[j] > maxi_ax) && sscene[j] == sc;
        bool hit = false;
        if (in) {
            const int fj = sflag[j];
            hit = !(fj & BF_IGNORE) && !((fi & BF_KINEMATIC) && (fj & BF_KINEMATIC)) &&
                  !(mnx > smx[j] || smn[j] > mxx) && !(mny > smx[n + j] || smn[n + j] > mxy) &&
                  !(mnz > smx[2 * (size_t)n + j] || smn[2 * (size_t)n + j] > mxz);
            if (hit && ign.off && ((fi | fj) & BF_IGN_LIST)) hit = !ign.ignored(i, j);
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) wcnt[w] = __popc(m);
        const int all_in = __syncthreads_and(in);
        int before = 0, total = 0;
        for (int k = 0; k < nw; k++) { if (k < w) before += wcnt[k]; total += wcnt[k]; }
        if (WRITE && hit) out[c + before + __popc(m & lt)] = make_int2(a, (int)order[j]);
        c += total;
        __syncthreads();   // wcnt is rewritten next iteration
        if (!all_in) break;
    }
    return c;
}

// A crowded position's window (the candidates j > i of its scene whose minimum along the axis does
// not exceed i's maximum: a prefix of the scene's sorted positions, found by binary search) swept in
// up to kMaxChunks chunks of at least kChunk candidates, one block per chunk: chunk counts are summed
// per position, and each chunk writes its pairs after those of the chunks before it, so the pairs
// keep ascending j.
constexpr int kChunk = 4096;
constexpr int kMaxChunks = 32;
template <class R, bool WRITE>
__device__ int sweep_range_block(int i, int jb, int je, int n, const R* smn, const R* smx, const int* sflag, int2* out,
                                 const uint32_t* order, int* wcnt, const IgnoreLists& ign) {
    const R mnx = smn[i], mny = smn[n + i], mnz = smn[2 * (size_t)n + i];
    const R mxx = smx[i], mxy = smx[n + i], mxz = smx[2 * (size_t)n + i];
    const int fi = sflag[i];
    if (fi & BF_IGNORE) return 0;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
    const int a = WRITE ? (int)order[i] : 0;
    const unsigned lt = (1u << lane) - 1u;
    int c = 0;
    for (int j0 = jb; j0 < je; j0 += blockDim.x) {
        const int j = j0 + tid;
        bool hit = false;
        if (j < je) {
            const int fj = sflag[j];
            hit = !(fj & BF_IGNORE) && !((fi & BF_KINEMATIC) && (fj & BF_KINEMATIC)) &&
                  !(mnx > smx[j] || smn[j] > mxx) && !(mny > smx[n + j] || smn[n + j] > mxy) &&
                  !(mnz > smx[2 * (size_t)n + j] || smn[2 * (size_t)n + j] > mxz);
            if (hit && ign.off && ((fi | fj) & BF_IGN_LIST)) hit = !ign.ignored(i, j);
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) wcnt[w] = __popc(m);
        __syncthreads();
        int before = 0, total = 0;
        for (int k = 0; k < nw; k++) { if (k < w) before += wcnt[k]; total += wcnt[k]; }
        if (WRITE && hit) out[c + before + __popc(m & lt)] = make_int2(a, (int)order[j]);
        c += total;
        __syncthreads();   // wcnt is rewritten next iteration
    }
    return c;
}
// per crowded position: window end, chunk size and chunk count
template <class R>
__global__ void k_bp_big_windows(int n, const int* scene_axis, const int* scene_off, const R* smn, const R* smx, const int* sscene,
                                 const int* big, const int* n_big, int* wend, int* csize, int* nchunk) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < *n_big; b += gridDim.x * blockDim.x) {
        const int i = big[b], sc = sscene[i];
        const R* amin = smn + (size_t)scene_axis[sc] * n;
        const R mx = smx[(size_t)scene_axis[sc] * n + i];
        int lo = i + 1, hi = scene_off[sc + 1];   // first j with amin[j] > mx, else the scene's end
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (amin[mid] > mx) hi = mid;
            else lo = mid + 1;
        }
        const int len = lo - (i + 1);
        int cs = (len + kMaxChunks - 1) / kMaxChunks;
        cs = cs < kChunk ? kChunk : cs;
        wend[b] = lo;
        csize[b] = cs;
        nchunk[b] = (len + cs - 1) / cs;
    }
}
__global__ void k_bp_chunk_offsets(const int* n_big, const int* nchunk, int* choff, int* total);
__device__ __forceinline__ int chunk_owner(int c, const int* choff, int nb) {   // last b with choff[b] <= c
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (choff[mid] <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
template <class R>
__global__ void k_bp_count_chunks(int n, const R* smn, const R* smx, const int* sflag, const int* big, const int* n_big, const int* wend,
                                  const int* csize, const int* choff, const int* total, int* ccount, IgnoreLists ign) {
    __shared__ int wcnt[32];
    for (int c = blockIdx.x; c < *total; c += gridDim.x) {
        const int b = chunk_owner(c, choff, *n_big), i = big[b];
        const int jb = i + 1 + (c - choff[b]) * csize[b], je = jb + csize[b] < wend[b] ? jb + csize[b] : wend[b];
        const int k = sweep_range_block<R, false>(i, jb, je, n, smn, smx, sflag, nullptr, nullptr, wcnt, ign);
        if (threadIdx.x == 0) ccount[c] = k;
    }
}
// per crowded position: its pair count and the offsets of its chunks' pairs
__global__ void k_bp_chunk_sums(const int* big, const int* n_big, const int* choff, const int* nchunk, const int* ccount, int* cpref,
                                int* count);
template <class R>
__global__ void k_bp_write_chunks(int n, const R* smn, const R* smx, const int* sflag, const uint32_t* order, const int* offset,
                                  const int* big, const int* n_big, const int* wend, const int* csize, const int* choff, const int* total,
                                  const int* cpref, int2* pairs, int pair_cap, int* status, IgnoreLists ign) {
    __shared__ int wcnt[32];
    for (int c = blockIdx.x; c < *total; c += gridDim.x) {
        const int b = chunk_owner(c, choff, *n_big), i = big[b];
        if (offset[i + 1] > pair_cap) {
            if (threadIdx.x == 0) atomicOr(status, ST_PAIR_OVERFLOW);
            continue;
        }
        const int jb = i + 1 + (c - choff[b]) * csize[b], je = jb + csize[b] < wend[b] ? jb + csize[b] : wend[b];
        sweep_range_block<R, true>(i, jb, je, n, smn, smx, sflag, pairs + offset[i] + cpref[c], order, wcnt, ign);
    }
}

template <class R>
__global__ void k_bp_count(int n, const int* scene_axis, const R* smn, const R* smx, const int* sflag, const int* sscene, int* count,
                           int* stage, int* big, int* n_big, IgnoreLists ign) {
    const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    if (big_window(i, n, scene_axis, smn, smx, sscene)) {   // left to k_bp_count_big
        if (lane == 0) big[atomicAdd(n_big, 1)] = i;
        return;
    }
    const int c = sweep_warp<R, false>(i, n, lane, scene_axis, smn, smx, sflag, sscene, stage, nullptr, nullptr, ign);
    if (lane == 0) count[i] = c;
}
// one block per listed position (blocks loop over the list)
template <class R>
__global__ void k_bp_count_big(int n, const int* scene_axis, const R* smn, const R* smx, const int* sflag, const int* sscene,
                               int* count, const int* big, const int* n_big, IgnoreLists ign) {
    __shared__ int wcnt[32];
    for (int b = blockIdx.x; b < *n_big; b += gridDim.x) {
        const int i = big[b];
        const int c = sweep_block<R, false>(i, n, scene_axis, smn, smx, sflag, sscene, nullptr, nullptr, wcnt, ign);
        if (threadIdx.x == 0) count[i] = c;
        __syncthreads();
    }
}
template <class R>
__global__ void k_bp_write_big(int n, const int* scene_axis, const R* smn, const R* smx, const int* sflag, const int* sscene,
                               const uint32_t* order, const int* offset, int2* pairs, int pair_cap, int* status, const int* big,
                               const int* n_big, IgnoreLists ign) {
    __shared__ int wcnt[32];
    for (int b = blockIdx.x; b < *n_big; b += gridDim.x) {
        const int i = big[b];
        const int base = offset[i], c = offset[i + 1] - base;
        if (c == 0) continue;   // uniform in the block
        if (base + c > pair_cap) {
            if (threadIdx.x == 0) atomicOr(status, ST_PAIR_OVERFLOW);
            continue;
        }
        sweep_block<R, true>(i, n, scene_axis, smn, smx, sflag, sscene, pairs + base, order, wcnt, ign);
        __syncthreads();
    }
}

template <class R>
__global__ void k_bp_write(int n, const int* scene_axis, const R* smn, const R* smx, const int* sflag, const int* sscene,
                           const uint32_t* order, const int* offset, const int* stage, int2* pairs, int pair_cap, int* status,
                           IgnoreLists ign) {
    const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const int base = offset[i], c = offset[i + 1] - base;
    if (c == 0 || big_window(i, n, scene_axis, smn, smx, sscene)) return;   // big windows: k_bp_write_big
    if (base + c > pair_cap) {
        if (lane == 0) atomicOr(status, ST_PAIR_OVERFLOW);
        return;
    }
    if (c <= kStage) {
        if (lane < c) pairs[base + lane] = make_int2((int)order[i], (int)order[stage[(size_t)i * kStage + lane]]);
    } else {
        sweep_warp<R, true>(i, n, lane, scene_axis, smn, smx, sflag, sscene, nullptr, pairs + base, order, ign);
    }
}

// Next sweep axis of each scene (BroadPhaseSweepAndPrune::calcCollisionPairs,
// broad_phase_sweep_and_prune.cpp:18-22, 37-40): the AABB centres (min + max) * 0.5 summed in the
// scene's sorted order, in the world's real type, one running sum per component for the centres and
// one for their squares, exactly as the reference accumulates them; then the variances
// s2 - s * s / n and the reference's strict comparisons.  A float sum is not associative, so the
// six sums run sequentially: one block of two warps per scene, warp 1 stages the next chunk of
// centres in shared memory while six lanes of warp 0 add up the current one.  A scene below two
// bodies keeps its axis (the reference returns before updating it).
template <class R> constexpr int axis_chunk() { return sizeof(R) == 4 ? 1024 : 512; }   // centres per staged chunk
template <class R>
__global__ void __launch_bounds__(64) k_bp_axis(const R* smn, const R* smx, int n, const int* scene_off, int* scene_axis) {
    constexpr int CH = axis_chunk<R>(), PAD = CH + 1;   // the padding puts the three rows in different banks
    __shared__ R cbuf[2][3 * PAD];
    __shared__ R sums[6];
    const int s = blockIdx.x, tid = threadIdx.x;
    const int lo = scene_off[s], hi = scene_off[s + 1], cnt = hi - lo;
    if (cnt < 2) return;   // whole block
    auto stage = [&](int buf, int base, int t) {   // t in [0, 32): the staging warp's lane
        const int e = min(CH, hi - base);
        for (int k = t; k < e; k += 32)
            for (int d = 0; d < 3; d++)
                cbuf[buf][d * PAD + k] = (smn[(size_t)d * n + base + k] + smx[(size_t)d * n + base + k]) * R(0.5);
    };
    if (tid >= 32) stage(0, lo, tid - 32);
    __syncthreads();
    R acc = 0;   // tid d < 3: running sum of centre component d; tid 3 + d: of its square
    int buf = 0;
    for (int base = lo; base < hi; base += CH) {
        if (tid >= 32) {
            if (base + CH < hi) stage(buf ^ 1, base + CH, tid - 32);
        } else if (tid < 6) {
            const int e = min(CH, hi - base);
            const R* c = cbuf[buf] + (tid < 3 ? tid : tid - 3) * PAD;
            const bool sq = tid >= 3;
            int k = 0;
            for (; k + 8 <= e; k += 8) {   // loads ahead of the dependent adds, which stay in order
                R v[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    v[u] = c[k + u];
                    if (sq) v[u] = v[u] * v[u];
                }
#pragma unroll
                for (int u = 0; u < 8; u++) acc = acc + v[u];
            }
            for (; k < e; k++) {
                R v = c[k];
                if (sq) v = v * v;
                acc = acc + v;
            }
        }
        __syncthreads();
        buf ^= 1;
    }
    if (tid < 6) sums[tid] = acc;
    __syncthreads();
    if (tid == 0) {
        R v[3];
        for (int d = 0; d < 3; d++) {
            const R ss = sums[d] * sums[d];
            v[d] = sums[3 + d] - ss / R(cnt);
        }
        int ax = 0;
        if (v[1] > v[0]) ax = 1;
        if (v[2] > v[ax]) ax = 2;
        scene_axis[s] = ax;
    }
}

} // namespace pe
