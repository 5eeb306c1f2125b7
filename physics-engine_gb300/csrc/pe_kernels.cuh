// Kernels of the rigid-body step.  One thread per body for integration, a project-written
// LSD radix sort plus a sweep for the broadphase, one thread per collision pair for the
// narrowphase (pairs bucketed by shape pairing), and sequential-impulse solver kernels
// (serial replay of the reference order per scene, or graph-coloured Gauss-Seidel).
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

// ===================================================================== scan
// exclusive scan of n ints, in place, three phases; totals of each tile in aux
__global__ void k_scan_tiles(int* data, int n, int* aux);
__global__ void k_scan_aux(int* aux, int m, int* total);
__global__ void k_scan_add(int* data, int n, const int* aux);

// ===================================================================== radix sort
// Sort (key, value) pairs by a 64-bit key and then, more significantly, by a 32-bit
// secondary key (scene id); stable, least-significant digit first, 8-bit digits.
constexpr int kRadixItems = 16;                      // items per thread per tile
constexpr int kRadixTile = kBlock * kRadixItems;     // 4096 items per tile
__global__ void k_radix_hist(const uint64_t* key, const uint32_t* key2, int n, int shift, int use2, int* hist, int n_tiles);
__global__ void k_radix_scatter(const uint64_t* key_in, const uint32_t* key2_in, const uint32_t* val_in, uint64_t* key_out,
                                uint32_t* key2_out, uint32_t* val_out, int n, int shift, int use2, const int* hist, int n_tiles);

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

// next sweep axis of each scene: the axis of largest AABB-centre variance (sweep_and_prune.cpp:37-40).
// One block per scene sums the sorted centres in double, in an order fixed relative to the scene
// (thread t takes positions t, t + blockDim, ... of the scene, then a fixed tree), so a scene gets
// the same sums wherever it sits in a batch and run to run.  A scene below two bodies keeps its
// axis, as the reference returns before updating it.
constexpr int kAxisTile = 4096;   // scenes above this size sum scene-relative tiles in separate blocks
template <class R>
__global__ void k_bp_axis(const R* smn, const R* smx, int n, const int* scene_off, int* scene_axis) {
    const int s = blockIdx.x;
    const int lo = scene_off[s], hi = scene_off[s + 1];
    const int cnt = hi - lo;
    if (cnt < 2 || cnt > kAxisTile) return;   // whole block
    __shared__ double red[6][kBlock];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
        for (int d = 0; d < 3; d++) {
            const double c = (double)((smn[(size_t)d * n + k] + smx[(size_t)d * n + k]) * R(0.5));
            acc[d] += c;
            acc[3 + d] += c * c;
        }
    }
    for (int q = 0; q < 6; q++) red[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) for (int q = 0; q < 6; q++) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double v[3];
        for (int d = 0; d < 3; d++) v[d] = red[3 + d][0] - red[d][0] * red[d][0] / (double)cnt;
        int ax = 0;
        if (v[1] > v[0]) ax = 1;
        if (v[2] > v[ax]) ax = 2;
        scene_axis[s] = ax;
    }
}

// large scenes: block b sums tile item[b].y (positions lo + tile * kAxisTile, ...) of scene
// item[b].x, in the same fixed order as k_bp_axis; then one thread per large scene adds its tiles
// in tile order
template <class R>
__global__ void k_bp_axis_tiles(const R* smn, const R* smx, int n, const int* scene_off, const int2* item, double* part) {
    const int s = item[blockIdx.x].x, t = item[blockIdx.x].y;
    const int lo = scene_off[s] + t * kAxisTile, hi = min(scene_off[s + 1], lo + kAxisTile);
    __shared__ double red[6][kBlock];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
        for (int d = 0; d < 3; d++) {
            const double c = (double)((smn[(size_t)d * n + k] + smx[(size_t)d * n + k]) * R(0.5));
            acc[d] += c;
            acc[3 + d] += c * c;
        }
    }
    for (int q = 0; q < 6; q++) red[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) for (int q = 0; q < 6; q++) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 6) part[(size_t)blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
}
__global__ void k_bp_axis_combine(const int* scene_off, const int2* item, int n_item, const double* part, int* scene_axis);

// ===================================================================== narrowphase
// bucket pairs by algorithm class
// Shared-memory staging limits of the SAT kernels (faces, unique edges, hull vertices per shape),
// and the scheduling split of ConvexConvexCollisionAlgorithm pairs by estimated work: candidate
// axes x projection cost (hull vertices; a box or cylinder projects in closed form).
constexpr int kSatF = 128, kSatE = 192, kSatV = 64;
constexpr int kSatWarps = 1;                 // pairs (one warp each) per block, light pairs
constexpr int kSatGroup = 8;                 // warps per pair, heavy pairs (one block each)
constexpr long long kSatHeavyCost = 200000;
template <class R> __device__ __forceinline__ bool sat_fits(const ShapeView<R>& s) {
    return s.face_count() <= kSatF && s.edge_count() <= kSatE && (s.type != ST_HULL || s.nv <= kSatV);
}
template <class R> __device__ __forceinline__ int sat_class(const ShapeView<R>& a, const ShapeView<R>& b) {
    if (!sat_fits(a) || !sat_fits(b)) return PC_CONVEX_BIG;
    auto w = [](const ShapeView<R>& s) { return s.type == ST_HULL ? s.nv : s.type == ST_CYLINDER ? 12 : s.type == ST_BOX ? 8 : 2; };
    auto ue = [](const ShapeView<R>& s) { return s.type == ST_BOX ? 3 : s.edge_count(); };   // distinct edge axes
    const long long axes = (long long)a.face_count() + b.face_count() + (long long)ue(a) * ue(b);
    if (axes * (w(a) + w(b)) >= kSatHeavyCost) return PC_CONVEX_HEAVY;
    if (a.type == ST_HULL && b.type == ST_HULL) return PC_CONVEX_HULL_HULL;
    if (a.type == ST_CYLINDER) return PC_CONVEX_CYL_CYL;
    return a.type == ST_BOX ? PC_CONVEX : PC_CONVEX_HULL_BOX;
}

template <class R>
__global__ void k_np_classify(int P, const int2* pairs, Bodies<R> B, ShapeTable<R> S, int* cls, int* cls_count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    int c = -1 - (int)(threadIdx.x & 31);   // lanes past the end never match a class
    if (p < P) {
        const int2 q = pairs[p];
        const ShapeView<R> sa = S.view(B.shape[q.x]), sb = S.view(B.shape[q.y]);
        c = pair_class(sa.type, sb.type);
        if (c == PC_CONVEX) c = sat_class(sa, sb);
        cls[p] = c;
    }
    // one atomic per class present in the warp
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    if (c >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cls_count[c], __popc(peers));
}
__global__ void k_np_bucket(int P, const int* cls, int* cursor, int* order);

// Pair setup of SimpleNarrowPhase::calcContactResults (simple_narrow_phase.cpp:24-38): the pooled
// result is reset, keeping the distances its slots had after the previous step's sort when the
// same (scene-local) result index existed then, the "fresh result" maximum otherwise.
template <class R>
__device__ __forceinline__ void np_setup(int p, const int2* pairs, const Bodies<R>& B, const ShapeTable<R>& S, const Results<R>& res,
                                         const int* pair_scene_off, const int* prev_off, Cache<R>& cache, Pair<R>& pr,
                                         bool load_cache = true) {
    const int2 q = pairs[p];
    const int ia = q.x, ib = q.y;
    pr.xa = B.xf(ia);
    pr.xb = B.xf(ib);
    const R scale_a = B.at(SCALE, ia), scale_b = B.at(SCALE, ib);
    pr.sa = S.view(B.shape[ia]);
    pr.sb = S.view(B.shape[ib]);
    pr.ref_scale = (scale_a + scale_b) * R(0.05);
    pr.c = &cache;
    if (!load_cache) return;
    cache.valid = 0;
    cache.swap = false;
    const int sc = B.scene[ia];
    const int local = p - pair_scene_off[sc];
    if (local < prev_off[sc + 1] - prev_off[sc]) {
        const int src = (prev_off[sc] + local) * kSlots;
        for (int k = 0; k < kSlots; k++) cache.dist[k] = res.prev_dist[src + k];
    } else {
        for (int k = 0; k < kSlots; k++) cache.dist[k] = Lim<R>::max();
    }
    cache.ta = pr.xa;
    cache.tb = pr.xb;
    cache.scale_a = scale_a;
    cache.scale_b = scale_b;
}

// ContactResult::sortContactPoints (stable order by distance over all 8 slots, size = first
// invalid slot) and write-out of result p
template <class R>
__device__ __forceinline__ void np_finish(int p, const int2* pairs, const Bodies<R>& B, const Results<R>& res, const Cache<R>& cache,
                                          bool swapped = false) {
    int2 q = pairs[p];
    if (swapped) q = make_int2(q.y, q.x);   // the result names its objects in swapped order
    int perm[kSlots];
    for (int k = 0; k < kSlots; k++) {
        int j = k;
        const R d = cache.dist[k];
        while (j > 0 && d < cache.dist[perm[j - 1]]) { perm[j] = perm[j - 1]; j--; }
        perm[j] = k;
    }
    int np = kSlots;
    for (int k = 0; k < kSlots; k++) if (!((cache.valid >> perm[k]) & 1u)) { np = k; break; }
    res.a[p] = q.x;
    res.b[p] = q.y;
    res.npts[p] = np;
    res.fr[p] = rsqrt_(B.at(FRIC, q.x) * B.at(FRIC, q.y));     // ContactResult::setObjects (contact_result.cpp:80-86)
    res.re[p] = rsqrt_(B.at(REST, q.x) * B.at(REST, q.y));
    for (int k = 0; k < kSlots; k++) res.dist[p * kSlots + k] = cache.dist[perm[k]];
    for (int k = 0; k < np; k++) {
        const int s = perm[k];
        const int o = p * kSlots + k;
        V3<R> t0, t1;
        ortho_units(cache.nrm[s], t0, t1);
        const V3<R> f[6] = {cache.pos[s], cache.nrm[s], cache.la[s], cache.lb[s], t0, t1};
        for (int g = 0; g < 6; g++) { res.pt(g * 3, o) = f[g].x; res.pt(g * 3 + 1, o) = f[g].y; res.pt(g * 3 + 2, o) = f[g].z; }
    }
}

// one thread per pair of one algorithm class; `order[lo..hi)` holds that class's pairs
template <class R, int CLS>
__global__ void k_np_class(int lo, int hi, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
                           const int* pair_scene_off, const int* prev_off) {
    const int t = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= hi) return;
    const int p = order[t];
    Cache<R> cache;
    Pair<R> pr;
    np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, pr);
    collide(pr, CLS);
    np_finish(p, pairs, B, res, cache);
}

// CompoundCompoundCollisionAlgorithm::processCollision (compound_compound_collision_algorithm.cpp:8-46),
// one thread per pair with a compound on either side.  A compound second swaps the pair (shapes,
// transforms and the result's objects: ContactResult::setObjects(B, A), so the result names the
// compound as object A); then every child of the compound, against every child of a second
// compound or against the other shape, runs its shape pair's algorithm into the same contact
// cache at the child's world transform (body transform * local transform).  Local contact
// positions stay relative to the bodies.
template <class R>
__global__ void k_np_compound(int lo, int hi, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
                              const int* pair_scene_off, const int* prev_off) {
    const int t = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= hi) return;
    const int p = order[t];
    Cache<R> cache;
    Pair<R> pr;
    np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, pr);
    int sa = B.shape[pairs[p].x], sb = B.shape[pairs[p].y];
    bool swapped = false;
    if (pr.sb.type == ST_COMPOUND) {
        const ShapeView<R> v = pr.sa; pr.sa = pr.sb; pr.sb = v;
        const Xf<R> x = pr.xa; pr.xa = pr.xb; pr.xb = x;
        const Xf<R> y = cache.ta; cache.ta = cache.tb; cache.tb = y;
        const R z = cache.scale_a; cache.scale_a = cache.scale_b; cache.scale_b = z;
        const int w = sa; sa = sb; sb = w;
        swapped = true;
    }
    const Xf<R> ta = pr.xa, tb = pr.xb;
    const bool b_comp = pr.sb.type == ST_COMPOUND;
    for (int i = S.c_beg[sa], ie = S.c_beg[sa] + S.c_cnt[sa]; i < ie; i++) {
        Pair<R> c = pr;
        c.sa = S.view(S.c_shape[i]);
        c.xa = ta * S.child_xf(i);
        if (b_comp) {
            for (int j = S.c_beg[sb], je = S.c_beg[sb] + S.c_cnt[sb]; j < je; j++) {
                c.sb = S.view(S.c_shape[j]);
                c.xb = tb * S.child_xf(j);
                collide(c, pair_class(c.sa.type, c.sb.type));
            }
        } else {
            collide(c, pair_class(c.sa.type, c.sb.type));
        }
    }
    np_finish(p, pairs, B, res, cache, swapped);
}

// ---------------------------------------------------------------- warp-cooperative SAT
// (convex_convex_collision_algorithm.cpp:251-432) for cylinder-cylinder, box-hull and hull-hull:
// one warp per pair, lanes over candidate axes.  The reference scans axes in order and keeps
// the first strictly smaller depth; that is the lexicographic minimum of (depth, axis index),
// which the warp reduces.  Any separating axis ends the test (the reference returns at the
// first one it meets; what it computed before that is discarded except the corner point).
template <class R> __device__ __forceinline__ void warp_argmin(R& d, int& idx) {
    for (int o = 16; o > 0; o >>= 1) {
        const R od = __shfl_xor_sync(0xffffffffu, d, o);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (od < d || (od == d && oi < idx)) { d = od; idx = oi; }
    }
}
template <class R> __device__ __forceinline__ void warp_min(R& d) {
    for (int o = 16; o > 0; o >>= 1) {
        const R od = __shfl_xor_sync(0xffffffffu, d, o);
        if (od < d) d = od;
    }
}
template <class R> __device__ __forceinline__ void warp_argmax(R& d, int& idx) {
    for (int o = 16; o > 0; o >>= 1) {
        const R od = __shfl_xor_sync(0xffffffffu, d, o);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (od > d || (od == d && oi < idx)) { d = od; idx = oi; }
    }
}
template <class R> __device__ __forceinline__ V3<R> shfl3(const V3<R>& v, int src) {
    return V3<R>(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src), __shfl_sync(0xffffffffu, v.z, src));
}

// ---- SAT with per-pair staging: world face normals, world unit edge directions and local hull
// vertices of both shapes are computed once into shared memory; support intervals are computed
// first and witness points only for an axis that becomes the current best.  Same formulas as
// Shape::project (so the same bits); only the order of evaluation across axes differs.
template <class R> constexpr int sat_stage_reals() { return 3 * (2 * kSatF + 2 * kSatE) + 4 * 2 * kSatV; }

template <class R> struct SatStage {
    R* nA; R* nB; R* dA; R* dB; R* vA; R* vB;   // vertices padded to 4 reals (16-byte aligned rows)
    __device__ void bind(R* base) {
        nA = base; nB = nA + 3 * kSatF; dA = nB + 3 * kSatF; dB = dA + 3 * kSatE; vA = dB + 3 * kSatE; vB = vA + 4 * kSatV;
    }
};
template <class R> __device__ __forceinline__ V3<R> ld3(const R* p, int i) { return V3<R>(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
template <class R> __device__ __forceinline__ void st3(R* p, int i, const V3<R>& v) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }
__device__ __forceinline__ V3<float> ldv(const float* p, int i) {
    const float4 f = reinterpret_cast<const float4*>(p)[i];
    return V3<float>(f.x, f.y, f.z);
}
__device__ __forceinline__ V3<double> ldv(const double* p, int i) {
    const double2* q = reinterpret_cast<const double2*>(p) + 2 * i;
    const double2 a = q[0], b = q[1];
    return V3<double>(a.x, a.y, b.x);
}
template <class R> __device__ __forceinline__ void stv(R* p, int i, const V3<R>& v) {
    p[4 * i] = v.x; p[4 * i + 1] = v.y; p[4 * i + 2] = v.z; p[4 * i + 3] = R(0);
}


// support interval of a shape along a world axis (Shape::project without the witness points);
// for hulls the indices of the witness vertices are returned (the first vertex never becomes
// the maximum, like convex_mesh_shape.cpp:171-175)
template <class R>
__device__ __forceinline__ void shape_interval(const ShapeView<R>& s, const Xf<R>& t, const V3<R>& axis, const R* lv, R& mnp, R& mxp,
                                               int& imn, int& imx) {
    if (s.type == ST_SPHERE) {
        const R off = dot(t.o, axis);
        mnp = off - s.radius; mxp = off + s.radius;
        return;
    }
    const V3<R> la = mtv(t.b, axis);
    const R off = dot(t.o, axis);
    if (s.type == ST_BOX) {
        const V3<R> ext(la.x > 0 ? s.half.x : -s.half.x, la.y > 0 ? s.half.y : -s.half.y, la.z > 0 ? s.half.z : -s.half.z);
        const R he = dot(ext, la);
        mnp = off - he; mxp = off + he;
        return;
    }
    if (s.type == ST_CYLINDER) {
        const R hh = s.height * R(0.5);
        if (rabs(la.x - 0) < eps<R>() && rabs(la.z - 0) < eps<R>()) { mnp = off - hh; mxp = off + hh; }
        else if (rabs(la.y - 0) < eps<R>()) { mnp = off - s.radius; mxp = off + s.radius; }
        else {
            const R r = rsqrt_(la.x * la.x + la.z * la.z);
            const R x = s.radius * la.x / r, z = s.radius * la.z / r;
            const R y = hh * (la.y > 0 ? 1 : -1);
            const R el = dot(V3<R>(x, y, z), la);
            mnp = off - el; mxp = off + el;
        }
        return;
    }
    mnp = Lim<R>::max();
    mxp = Lim<R>::min();
    imn = -1; imx = -1;
    for (int i = 0; i < s.nv; i++) {
        const R v = dot(ldv(lv, i), la);
        if (v < mnp) { mnp = v; imn = i; }
        else if (v > mxp) { mxp = v; imx = i; }
    }
    mnp += off;
    mxp += off;
}

// two axes at once: a hull's vertices are loaded once for both (same arithmetic per axis)
template <class R>
__device__ __forceinline__ void shape_interval2(const ShapeView<R>& s, const Xf<R>& t, const V3<R>* axis, const R* lv, R* mnp, R* mxp,
                                                int* imn, int* imx) {
    if (s.type != ST_HULL) {
        shape_interval(s, t, axis[0], lv, mnp[0], mxp[0], imn[0], imx[0]);
        shape_interval(s, t, axis[1], lv, mnp[1], mxp[1], imn[1], imx[1]);
        return;
    }
    const V3<R> l0 = mtv(t.b, axis[0]), l1 = mtv(t.b, axis[1]);
    R n0 = Lim<R>::max(), x0 = Lim<R>::min(), n1 = Lim<R>::max(), x1 = Lim<R>::min();
    int in0 = -1, ix0 = -1, in1 = -1, ix1 = -1;
    for (int i = 0; i < s.nv; i++) {
        const V3<R> p = ldv(lv, i);
        const R v0 = dot(p, l0), v1 = dot(p, l1);
        if (v0 < n0) { n0 = v0; in0 = i; }
        else if (v0 > x0) { x0 = v0; ix0 = i; }
        if (v1 < n1) { n1 = v1; in1 = i; }
        else if (v1 > x1) { x1 = v1; ix1 = i; }
    }
    const R o0 = dot(t.o, axis[0]), o1 = dot(t.o, axis[1]);
    mnp[0] = n0 + o0; mxp[0] = x0 + o0; imn[0] = in0; imx[0] = ix0;
    mnp[1] = n1 + o1; mxp[1] = x1 + o1; imn[1] = in1; imx[1] = ix1;
}

// Intervals of both shapes along two axes.  The larger hull's vertex loop may stop early: its
// running minimum only falls and its (first-vertex-excluding) running maximum only rises, so the
// overlap depths min(maxA - minB, maxB - minA) computed from a prefix of its vertices are lower
// bounds of the final ones (IEEE rounding is monotone).  Once both depths of an axis exceed `best`
// (an upper bound of the pair's minimum depth) the axis can neither separate nor be the minimum;
// when that holds for both axes the loop ends and both are reported not live.  Compiled out of line:
// the face and the edge passes share one copy, and the SAT kernels' instruction fetch stalls fell
// with the code size (the staged SAT group 6.52 -> 5.76 ms per batched step).
template <class R>
__device__ __noinline__ void pair_intervals2(const Pair<R>& c, const V3<R>* ax, bool* live, R best, const R* vA, const R* vB,
                                                R* min0, R* max0, R* min1, R* max1, int* a0, int* a1, int* b0, int* b1) {
    const bool part_b = c.sb.type == ST_HULL && (c.sa.type != ST_HULL || c.sb.nv >= c.sa.nv);
    const bool part_a = !part_b && c.sa.type == ST_HULL;
    if (!part_a && !part_b) {
        shape_interval2(c.sa, c.ta(), ax, vA, min0, max0, a0, a1);
        shape_interval2(c.sb, c.tb(), ax, vB, min1, max1, b0, b1);
        return;
    }
    // the complete side first
    const ShapeView<R>& sp = part_b ? c.sb : c.sa;
    const Xf<R>& tp = part_b ? c.tb() : c.ta();
    const R* lv = part_b ? vB : vA;
    R cmn[2], cmx[2];
    if (part_b) { shape_interval2(c.sa, c.ta(), ax, vA, min0, max0, a0, a1); cmn[0] = min0[0]; cmn[1] = min0[1]; cmx[0] = max0[0]; cmx[1] = max0[1]; }
    else { shape_interval2(c.sb, c.tb(), ax, vB, min1, max1, b0, b1); cmn[0] = min1[0]; cmn[1] = min1[1]; cmx[0] = max1[0]; cmx[1] = max1[1]; }
    const V3<R> l0 = mtv(tp.b, ax[0]), l1 = mtv(tp.b, ax[1]);
    const R o0 = dot(tp.o, ax[0]), o1 = dot(tp.o, ax[1]);
    R n0 = Lim<R>::max(), x0 = Lim<R>::min(), n1 = Lim<R>::max(), x1 = Lim<R>::min();
    int in0 = -1, ix0 = -1, in1 = -1, ix1 = -1;
    bool done = false;
    for (int i0 = 0; i0 < sp.nv; i0 += 8) {
        const int e = i0 + 8 < sp.nv ? i0 + 8 : sp.nv;
        for (int i = i0; i < e; i++) {
            const V3<R> p = ldv(lv, i);
            const R v0 = dot(p, l0), v1 = dot(p, l1);
            if (v0 < n0) { n0 = v0; in0 = i; }
            else if (v0 > x0) { x0 = v0; ix0 = i; }
            if (v1 < n1) { n1 = v1; in1 = i; }
            else if (v1 > x1) { x1 = v1; ix1 = i; }
        }
        if (e == sp.nv) break;
        // partial depths: d0 = maxA - minB, d1 = maxB - minA with the partial side's running values
        bool dec[2];
        const R pn[2] = {n0 + o0, n1 + o1}, px[2] = {x0 + o0, x1 + o1};
        for (int k = 0; k < 2; k++) {
            const R d0 = part_b ? cmx[k] - pn[k] : px[k] - cmn[k];
            const R d1 = part_b ? px[k] - cmn[k] : cmx[k] - pn[k];
            dec[k] = !live[k] || (d0 > best && d1 > best);
        }
        if (dec[0] && dec[1]) { done = true; break; }
    }
    if (done) { live[0] = live[1] = false; return; }
    if (part_b) { min1[0] = n0 + o0; max1[0] = x0 + o0; b0[0] = in0; b1[0] = ix0; min1[1] = n1 + o1; max1[1] = x1 + o1; b0[1] = in1; b1[1] = ix1; }
    else { min0[0] = n0 + o0; max0[0] = x0 + o0; a0[0] = in0; a1[0] = ix0; min0[1] = n1 + o1; max0[1] = x1 + o1; a0[1] = in1; a1[1] = ix1; }
}

// witness point of Shape::project on the min (want_max = false) or max side
template <class R>
__device__ V3<R> shape_witness(const ShapeView<R>& s, const Xf<R>& t, const V3<R>& axis, bool want_max, int idx, const R* lv) {
    R a, b;
    V3<R> pmin, pmax;
    if (s.type == ST_HULL) {
        // an index never set leaves the reference's witness undefined; that only happens on a
        // separating axis, whose witness is never used
        const V3<R> p = idx >= 0 ? ldv(lv, idx) : V3<R>(0, 0, 0);
        return t.apply(p);
    }
    shape_project(s, t, axis, a, b, pmin, pmax);
    return want_max ? pmax : pmin;
}

// Group primitives of the staged SAT: a group is one warp (G = 1) or a whole block of G warps.
// Reductions are lexicographic (value, axis index) minima/maxima, so their result does not depend
// on the order lanes and warps are combined in.
template <int G> __device__ __forceinline__ bool group_any(bool p) {
    if (G == 1) return __any_sync(0xffffffffu, p);
    return __syncthreads_or(p) != 0;
}
template <class R, int G> __device__ __forceinline__ void group_argmin(R& d, int& idx, int tid, R* rd, int* ri) {
    warp_argmin(d, idx);
    if (G == 1) return;
    if ((tid & 31) == 0) { rd[tid >> 5] = d; ri[tid >> 5] = idx; }
    __syncthreads();
    d = rd[0]; idx = ri[0];
    for (int k = 1; k < G; k++)
        if (rd[k] < d || (rd[k] == d && ri[k] < idx)) { d = rd[k]; idx = ri[k]; }
    __syncthreads();
}
template <class R, int G> __device__ __forceinline__ void group_argmax(R& d, int& idx, int tid, R* rd, int* ri) {
    warp_argmax(d, idx);
    if (G == 1) return;
    if ((tid & 31) == 0) { rd[tid >> 5] = d; ri[tid >> 5] = idx; }
    __syncthreads();
    d = rd[0]; idx = ri[0];
    for (int k = 1; k < G; k++)
        if (rd[k] > d || (rd[k] == d && ri[k] < idx)) { d = rd[k]; idx = ri[k]; }
    __syncthreads();
}
// value of the one thread of the group with `mine` set (the thread that evaluated the winning axis)
template <class R, int G> __device__ __forceinline__ V3<R> group_bcast3(const V3<R>& v, bool mine, R* buf) {
    if (G == 1) return shfl3(v, __ffs(__ballot_sync(0xffffffffu, mine)) - 1);
    if (mine) { buf[0] = v.x; buf[1] = v.y; buf[2] = v.z; }
    __syncthreads();
    const V3<R> r(buf[0], buf[1], buf[2]);
    __syncthreads();
    return r;
}
// reals of per-group scratch after the staging area: G reduction values, G indices, 3 broadcast,
// the queue length
template <class R> constexpr int sat_scratch_reals(int G) { return G == 1 ? 0 : 2 * G + 4; }
// candidate axes per thread of one pruning pass, and the queue of surviving axis indices after the
// scratch area
constexpr int kSatQ = 8;
template <class R> constexpr int sat_queue_reals(int G) { return (kSatQ * 32 * G * (int)sizeof(int) + (int)sizeof(R) - 1) / (int)sizeof(R); }

// Pruning bound of one shape along a world axis: lo <= the computed maximum of its projection
// interval, hi >= the computed minimum (a hull: its inner ball about the local origin; another
// shape: its closed-form interval), and mag bounds the magnitudes entering their rounding.
template <class R>
__device__ __forceinline__ void prune_side(const ShapeView<R>& s, const Xf<R>& t, const V3<R>& ax, R& lo, R& hi, R& mag) {
    if (s.type == ST_HULL) {
        const R o = dot(t.o, ax);
        lo = o + s.inner;
        hi = o - s.inner;
        mag = rabs(o) + s.outer;
        return;
    }
    int i0, i1;
    shape_interval(s, t, ax, (const R*)nullptr, hi, lo, i0, i1);
    mag = rabs(hi) + rabs(lo);
}
// True when the axis's overlap depth min(maxA - minB, maxB - minA) is certainly above `best`, a
// depth the SAT has already computed for one of the pair's axes (so best >= 0): such an axis can
// neither separate the pair nor be its minimum (the reference keeps the first strict minimum), and
// skipping it leaves the result unchanged.  The bound is lowered by 64 units of roundoff of the
// magnitudes involved, which covers the rounding of the projections the SAT would compute.  `able`
// is false when a hull of the pair has no certified inner ball.
template <class R>
__device__ __forceinline__ bool sat_prunable(const Pair<R>& c, bool able, const V3<R>& ax, R best) {
    if (!able || !(best < Lim<R>::max())) return false;
    R loA, hiA, mA, loB, hiB, mB;
    prune_side(c.sa, c.ta(), ax, loA, hiA, mA);
    prune_side(c.sb, c.tb(), ax, loB, hiB, mB);
    const R d0 = loA - hiB, d1 = loB - hiA;
    const R lb = d0 < d1 ? d0 : d1;
    constexpr R u = sizeof(R) == 4 ? R(1.1920929e-7) : R(2.220446049250313e-16);
    return lb > best + R(64) * u * (mA + mB + rabs(best));
}
// Compacts the candidate axes [base, base + span) ∩ [0, n) that `keep` accepts into the group's
// queue and returns their count (the same in every thread of the group).  With one warp the queue
// keeps ascending order; with several, warps append in any order.
template <int G, class F>
__device__ __forceinline__ int sat_queue(int base, int span, int n, int tid, int* q, int* qn, F&& keep) {
    constexpr int T = 32 * G;
    const unsigned lt = (1u << (tid & 31)) - 1u;
    int cnt = 0;
    for (int j = 0; j < span; j += T) {
        const int f = base + j + tid;
        const bool k = f < n && keep(f);
        const unsigned m = __ballot_sync(0xffffffffu, k);
        if (G == 1) {
            if (k) q[cnt + __popc(m & lt)] = f;
            cnt += __popc(m);
        } else {
            int b = 0;
            if ((tid & 31) == 0 && m) b = atomicAdd(qn, __popc(m));
            b = __shfl_sync(0xffffffffu, b, 0);
            if (k) q[b + __popc(m & lt)] = f;
        }
    }
    if (G == 1) {
        __syncwarp();
        return cnt;
    }
    __syncthreads();
    cnt = *qn;
    __syncthreads();
    if (tid == 0) *qn = 0;   // visible to the next pass's appends after sat_queue_done
    return cnt;
}
// the queue is read until here; the next pass may refill it
template <int G> __device__ __forceinline__ void sat_queue_done() {
    if (G == 1) __syncwarp(); else __syncthreads();
}

// Staged SAT of one pair by a group of G warps (tid in [0, 32 G)).  Per pass the group tests
// candidate axes against the pruning bound, queues the survivors and projects them two per thread;
// it stops at the first round holding a separating axis.
// What the staged SAT leaves for the contact step (one record of kSatOut reals per pair, written by
// thread 0): the face-stage point, the edge-stage point, the final axis and the clipping faces,
// in the order the reference adds them (convex_convex_collision_algorithm.cpp:300-308, :363-395,
// :420-430).  flags: 1 face point, 2 edge point, 4 clip.
enum SatOutField { SO_FLAGS = 0, SO_FN = 1, SO_FP = 4, SO_FD = 7, SO_EN = 8, SO_EP = 11, SO_ED = 14, SO_SEP = 15, SO_FB = 18,
                   SO_FA = 19, kSatOut = 20 };
template <class R> __device__ __forceinline__ void so_put3(R* o, int k, const V3<R>& v) { o[k] = v.x; o[k + 1] = v.y; o[k + 2] = v.z; }
template <class R> __device__ __forceinline__ V3<R> so_get3(const R* o, int k) { return V3<R>(o[k], o[k + 1], o[k + 2]); }

template <class R, int G, int TA, int TB>
__device__ void sat_staged(Pair<R>& c, int tid, R* smem, R* out) {
    constexpr int T = 32 * G;
    if (tid == 0) out[SO_FLAGS] = R(0);
    if (TA >= 0) c.sa.type = TA;   // shape types known at compile time: the other branches fold away
    if (TB >= 0) c.sb.type = TB;
    const R margin = 0;
    SatStage<R> st;
    st.bind(smem);
    R* rd = smem + sat_stage_reals<R>();
    int* ri = reinterpret_cast<int*>(rd + G);
    R* bc = rd + 2 * G;
    const int fa = c.sa.face_count(), fb = c.sb.face_count();
    const int na = c.sa.edge_count(), nb = c.sb.edge_count();
    for (int f = tid; f < fa; f += T) st3(st.nA, f, mv(c.ta().b, c.sa.face_normal(f)));
    for (int f = tid; f < fb; f += T) st3(st.nB, f, mv(c.tb().b, c.sb.face_normal(f)));
    for (int e = tid; e < na; e += T) { V3<R> a0, a1; c.sa.edge(e, a0, a1); st3(st.dA, e, mv(c.ta().b, normalized(a0 - a1))); }
    for (int e = tid; e < nb; e += T) { V3<R> b0, b1; c.sb.edge(e, b0, b1); st3(st.dB, e, mv(c.tb().b, normalized(b0 - b1))); }
    if (c.sa.type == ST_HULL) for (int i = tid; i < c.sa.nv; i += T) stv(st.vA, i, c.sa.vert(i));
    if (c.sb.type == ST_HULL) for (int i = tid; i < c.sb.nv; i += T) stv(st.vB, i, c.sb.vert(i));
    int* queue = reinterpret_cast<int*>(smem + sat_stage_reals<R>() + sat_scratch_reals<R>(G));
    int* qn = reinterpret_cast<int*>(rd + 2 * G + 3);   // several warps: the queue length
    if (G > 1 && tid == 0) *qn = 0;
    if (G == 1) __syncwarp(); else __syncthreads();
    const V3<R> dc = c.ta().o - c.tb().o;
    const bool able = (c.sa.type != ST_HULL || c.sa.inner > 0) && (c.sb.type != ST_HULL || c.sb.inner > 0);
    // ---- face axes of A, then of B (findSeparatingAxis :265-308).  Each pass compacts the axes
    // that the running minimum does not rule out (sat_prunable) and projects those, two per thread;
    // the first 2T axes run unpruned and give the bound.  A candidate compares by (depth, axis
    // index), the reference's first strict minimum in any visiting order.
    auto face_axis = [&](int f) {
        V3<R> n = f < fa ? ld3(st.nA, f) : ld3(st.nB, f - fa);
        if (dot(dc, n) < 0) n = n * R(-1.0);
        return n;
    };
    R bd = Lim<R>::max();
    int bf = 0x7fffffff, bside = 0, bia = -1, bib = -1;
    for (int pass = 0; pass < fa + fb;) {
        const int span = pass == 0 ? 2 * T : kSatQ * T;
        R pb = bd;
        warp_min(pb);
        const int cnt = sat_queue<G>(pass, span, fa + fb, tid, queue, qn, [&](int f) { return !sat_prunable(c, able, face_axis(f), pb); });
        for (int base = 0; base < cnt; base += 2 * T) {
            V3<R> n[2];
            bool ok[2];
            int fi[2];
            for (int k = 0; k < 2; k++) {
                const int qi = base + T * k + tid;
                ok[k] = qi < cnt;
                fi[k] = ok[k] ? queue[qi] : 0x7fffffff;
                n[k] = ok[k] ? face_axis(fi[k]) : V3<R>(0, 0, 0);
            }
            R min0[2], max0[2], min1[2], max1[2];
            int a0[2], a1[2], b0[2], b1[2];
            R best = bd;
            warp_min(best);
            pair_intervals2(c, n, ok, best, st.vA, st.vB, min0, max0, min1, max1, a0, a1, b0, b1);
            bool sep = false;
            for (int k = 0; k < 2; k++) sep |= ok[k] && (max0[k] < min1[k] || max1[k] < min0[k]);
            if (group_any<G>(sep)) return;
            for (int k = 0; k < 2; k++) {
                if (!ok[k]) continue;
                const R d0 = max0[k] - min1[k], d1 = max1[k] - min0[k];
                const R d = d0 < d1 ? d0 : d1;
                if (d < bd || (d == bd && fi[k] < bf)) {
                    bd = d; bf = fi[k]; bside = d0 < d1;
                    bia = d0 < d1 ? a1[k] : a0[k]; bib = d0 < d1 ? b0[k] : b1[k];
                }
            }
        }
        sat_queue_done<G>();
        pass += span;
    }
    R dmin = bd;
    int wf = bf;
    group_argmin<R, G>(dmin, wf, tid, rd, ri);
    V3<R> sep, dpt;
    const bool on_a = wf >= fa;
    if (wf < 0x7fffffff) {
        const bool mine = bf == wf;
        if (mine) {
            V3<R> n = wf < fa ? ld3(st.nA, wf) : ld3(st.nB, wf - fa);
            if (dot(dc, n) < 0) n = n * R(-1.0);
            sep = n;
            // testSepAxis witnesses: d0 < d1 -> (max of A, min of B), else (min of A, max of B)
            if (!on_a) dpt = shape_witness(c.sb, c.tb(), n, !bside, bib, st.vB);
            else dpt = shape_witness(c.sa, c.ta(), n, bside, bia, st.vA) + n * bd;
        }
        sep = group_bcast3<R, G>(sep, mine, bc);
        dpt = group_bcast3<R, G>(dpt, mine, bc);
        if (tid == 0 &&
            ((on_a && shape_inside(c.sb, c.tb().inv_apply(dpt))) || (!on_a && shape_inside(c.sa, c.ta().inv_apply(dpt))))) {
            out[SO_FLAGS] = R(1);
            so_put3(out, SO_FN, sep);
            so_put3(out, SO_FP, dpt - sep * margin);
            out[SO_FD] = -dmin + margin * 2;
        }
    }
    // ---- edge-pair axes (:323-361).  A box's 12 edges come in 3 classes of 4 whose direction
    // vectors are bit-identical (scaled unit-mesh differences), so they give identical axes,
    // projections and witnesses: each class is projected once, and a candidate takes the first
    // edge pair of the class (in the reference's e0-major order) whose lines hold the witnesses.
    // Candidates compare by (depth, reference axis index), which is the reference's first strict
    // minimum whatever order the axes are visited in.
    R ed = dmin;
    int ep = 0x7fffffff;
    V3<R> ewa, ewb, en;
    const bool boxA = c.sa.type == ST_BOX, boxB = c.sb.type == ST_BOX;
    const int ua = boxA ? 3 : na, ub = boxB ? 3 : nb;
    const int ne = ua * ub;
    auto edge_axis = [&](int q, V3<R>& a) {   // false for parallel edges
        const int iu = q / ub, ju = q - iu * ub;
        const V3<R> x = cross(ld3(st.dA, boxA ? 4 * iu : iu), ld3(st.dB, boxB ? 4 * ju : ju));
        if (rabs(norm(x) - 0) < eps<R>()) return false;
        a = normalized(x);
        if (dot(dc, a) < 0) a = a * R(-1.0);
        return true;
    };
    for (int pass = 0; pass < ne; pass += kSatQ * T) {
      R pb = ed;
      warp_min(pb);
      const int cnt = sat_queue<G>(pass, kSatQ * T, ne, tid, queue, qn, [&](int q) {
          V3<R> a;
          return edge_axis(q, a) && !sat_prunable(c, able, a, pb);
      });
      for (int qb = 0; qb < cnt; qb += 2 * T) {
        V3<R> cr[2];
        bool ok[2];
        int qa[2];
        for (int k = 0; k < 2; k++) {
            const int qi = qb + T * k + tid;
            ok[k] = qi < cnt;
            qa[k] = ok[k] ? queue[qi] : 0;
            cr[k] = V3<R>(0, 0, 0);
            if (ok[k]) edge_axis(qa[k], cr[k]);
        }
        R min0[2], max0[2], min1[2], max1[2];
        int a0[2], a1[2], b0[2], b1[2];
        R best = ed;
        warp_min(best);
        pair_intervals2(c, cr, ok, best, st.vA, st.vB, min0, max0, min1, max1, a0, a1, b0, b1);
        bool sp = false;
        for (int k = 0; k < 2; k++) sp |= ok[k] && (max0[k] < min1[k] || max1[k] < min0[k]);
        if (group_any<G>(sp)) return;
        for (int k = 0; k < 2; k++) {
            if (!ok[k]) continue;
            const R d0 = max0[k] - min1[k], d1 = max1[k] - min0[k];
            const R dist = d0 < d1 ? d0 : d1;
            if (!(dist < ed || (dist == ed && ep != 0x7fffffff))) continue;
            const int q = qa[k];
            const int iu = q / ub, ju = q - iu * ub;
            const bool side = d0 < d1;
            const V3<R> wa = shape_witness(c.sa, c.ta(), cr[k], side, side ? a1[k] : a0[k], st.vA);
            const V3<R> wb = shape_witness(c.sb, c.tb(), cr[k], !side, side ? b0[k] : b1[k], st.vB);
            const V3<R> la = c.ta().inv_apply(wa), lb = c.tb().inv_apply(wb);
            int qref = 0x7fffffff;
            for (int m0 = 0; m0 < (boxA ? 4 : 1) && qref == 0x7fffffff; m0++) {
                const int e0 = boxA ? 4 * iu + m0 : iu;
                V3<R> p0, p1;
                c.sa.edge(e0, p0, p1);
                if (!on_line(p0, p1, la)) continue;
                for (int m1 = 0; m1 < (boxB ? 4 : 1); m1++) {
                    const int e1 = boxB ? 4 * ju + m1 : ju;
                    V3<R> q0, q1;
                    c.sb.edge(e1, q0, q1);
                    if (on_line(q0, q1, lb)) { qref = e0 * nb + e1; break; }
                }
            }
            if (qref == 0x7fffffff || !(dist < ed || qref < ep)) continue;
            ed = dist; ep = qref; ewa = wa; ewb = wb; en = cr[k];
        }
      }
      sat_queue_done<G>();
    }
    R emin = ed;
    int wq = ep;
    group_argmin<R, G>(emin, wq, tid, rd, ri);
    if (wq < 0x7fffffff) {
        const bool mine = ep == wq;
        const V3<R> wpa = group_bcast3<R, G>(ewa, mine, bc), wpb = group_bcast3<R, G>(ewb, mine, bc);
        sep = group_bcast3<R, G>(en, mine, bc);
        if (tid == 0) {   // segmentsClosestPoints with unbounded half-lengths (:172-214, :363-395)
            const int e0 = wq / nb, e1 = wq - e0 * nb;
            const V3<R> wea = ld3(st.dA, e0), web = ld3(st.dB, e1);
            const V3<R> tr = wpb - wpa;
            const R ab = dot(wea, web), at = dot(wea, tr), bt = dot(web, tr);
            const R d = R(1.0) - ab * ab;
            const R ha = Lim<R>::max(), hb = Lim<R>::max();
            R ta, tb;
            if (d == 0) ta = 0;
            else { ta = (at - bt * ab) / d; if (ta < -ha) ta = -ha; else if (ta > ha) ta = ha; }
            tb = ta * ab - bt;
            if (tb < -hb) { tb = -hb; ta = tb * ab + at; if (ta < -ha) ta = -ha; else if (ta > ha) ta = ha; }
            else if (tb > hb) { tb = hb; ta = tb * ab + at; if (ta < -ha) ta = -ha; else if (ta > ha) ta = ha; }
            const V3<R> oa = wea * ta, ob = web * tb;
            V3<R> pts = tr - oa + ob;
            const R nl2 = sqnorm(pts);
            if (nl2 > eps<R>()) {
                const R nl = rsqrt_(nl2);
                pts = pts * (R(1.0) / nl);
                if (dot(pts, dc) < 0) pts = pts * R(-1.0);
                out[SO_FLAGS] += R(2);
                so_put3(out, SO_EN, pts);
                so_put3(out, SO_EP, wpb + ob - pts * margin);
                out[SO_ED] = -nl + margin * 2;
            }
        }
    }
    if (dot(dc, sep) < 0) sep = -sep;
    // ---- clipping (:63-170): incident face of B (first maximum), reference face of A (first minimum)
    R dmax = Lim<R>::min();
    int fbest = 0x7fffffff;
    for (int f = tid; f < fb; f += T) {
        const R d = dot(ld3(st.nB, f), sep);
        if (d > dmax) { dmax = d; fbest = f; }
    }
    group_argmax<R, G>(dmax, fbest, tid, rd, ri);
    R dmn = Lim<R>::max();
    int fabest = 0x7fffffff;
    for (int f = tid; f < fa; f += T) {
        const R d = dot(ld3(st.nA, f), sep);
        if (d < dmn) { dmn = d; fabest = f; }
    }
    group_argmin<R, G>(dmn, fabest, tid, rd, ri);
    if (tid == 0 && fbest < 0x7fffffff && fabest < 0x7fffffff) {
        out[SO_FLAGS] += R(4);
        so_put3(out, SO_SEP, sep);
        out[SO_FB] = R(fbest);
        out[SO_FA] = R(fabest);
    }
}

template <class R>
__device__ bool sat_warp(Pair<R>& c, int lane) {
    const R margin = 0;
    const V3<R> dc = c.ta().o - c.tb().o;
    const int fa = c.sa.face_count(), fb = c.sb.face_count();
    // face axes of A, then of B
    R bd = Lim<R>::max();
    int bf = 0x7fffffff;
    V3<R> bn, bpt;
    bool sep_found = false;
    for (int f = lane; f < fa + fb; f += 32) {
        const bool is_a = f < fa;
        V3<R> n = is_a ? mv(c.ta().b, c.sa.face_normal(f)) : mv(c.tb().b, c.sb.face_normal(f - fa));
        if (dot(dc, n) < 0) n = n * R(-1.0);
        R d;
        V3<R> wa, wb;
        if (!sep_test(c, n, d, wa, wb)) { sep_found = true; break; }
        if (d < bd) { bd = d; bf = f; bn = n; bpt = is_a ? wb : wa + n * d; }
    }
    if (__any_sync(0xffffffffu, sep_found)) return false;
    R dmin = bd;
    int wf = bf;
    warp_argmin(dmin, wf);
    const int src_lane = wf < 0x7fffffff ? wf % 32 : 0;
    V3<R> sep = shfl3(bn, src_lane);
    const V3<R> dpt = shfl3(bpt, src_lane);
    const bool on_a = wf >= fa;
    if (wf < 0x7fffffff && lane == 0) {
        if ((on_a && shape_inside(c.sb, c.tb().inv_apply(dpt))) || (!on_a && shape_inside(c.sa, c.ta().inv_apply(dpt))))
            c.add(sep, dpt - sep * margin, -dmin + margin * 2);
    }
    // edge-pair axes
    const int na = c.sa.edge_count(), nb = c.sb.edge_count();
    const int ne = na * nb;
    R ed = dmin;
    int ep = 0x7fffffff;
    V3<R> ewa, ewb, ew0, ew1, en;
    sep_found = false;
    for (int q = lane; q < ne; q += 32) {
        const int e0 = q / nb, e1 = q - e0 * nb;
        V3<R> a0, a1, b0, b1;
        c.sa.edge(e0, a0, a1);
        c.sb.edge(e1, b0, b1);
        const V3<R> w0 = mv(c.ta().b, normalized(a0 - a1));
        const V3<R> w1 = mv(c.tb().b, normalized(b0 - b1));
        V3<R> cr = cross(w0, w1);
        if (rabs(norm(cr) - 0) < eps<R>()) continue;
        cr = normalized(cr);
        if (dot(dc, cr) < 0) cr = cr * R(-1.0);
        R dist;
        V3<R> wa, wb;
        if (!sep_test(c, cr, dist, wa, wb)) { sep_found = true; break; }
        if (dist < ed) {
            if (!on_line(a0, a1, c.ta().inv_apply(wa)) || !on_line(b0, b1, c.tb().inv_apply(wb))) continue;
            ed = dist; ep = q; ewa = wa; ewb = wb; ew0 = w0; ew1 = w1; en = cr;
        }
    }
    if (__any_sync(0xffffffffu, sep_found)) return false;
    R emin = ed;
    int wq = ep;
    warp_argmin(emin, wq);
    if (wq < 0x7fffffff) {
        const int sl = wq % 32;
        const V3<R> wpa = shfl3(ewa, sl), wpb = shfl3(ewb, sl), wea = shfl3(ew0, sl), web = shfl3(ew1, sl);
        sep = shfl3(en, sl);
        if (lane == 0) {   // segmentsClosestPoints with unbounded half-lengths (:172-214, :363-395)
            const V3<R> tr = wpb - wpa;
            const R ab = dot(wea, web), at = dot(wea, tr), bt = dot(web, tr);
            const R d = R(1.0) - ab * ab;
            const R ha = Lim<R>::max(), hb = Lim<R>::max();
            R ta, tb;
            if (d == 0) ta = 0;
            else { ta = (at - bt * ab) / d; if (ta < -ha) ta = -ha; else if (ta > ha) ta = ha; }
            tb = ta * ab - bt;
            if (tb < -hb) { tb = -hb; ta = tb * ab + at; if (ta < -ha) ta = -ha; else if (ta > ha) ta = ha; }
            else if (tb > hb) { tb = hb; ta = tb * ab + at; if (ta < -ha) ta = -ha; else if (ta > ha) ta = ha; }
            const V3<R> oa = wea * ta, ob = web * tb;
            V3<R> pts = tr - oa + ob;
            const R nl2 = sqnorm(pts);
            if (nl2 > eps<R>()) {
                const R nl = rsqrt_(nl2);
                pts = pts * (R(1.0) / nl);
                if (dot(pts, dc) < 0) pts = pts * R(-1.0);
                c.add(pts, wpb + ob - pts * margin, -nl + margin * 2);
            }
        }
    }
    if (dot(dc, sep) < 0) sep = -sep;
    // clipping (:63-170): incident face of B (first maximum), reference face of A (first minimum)
    R dmax = Lim<R>::min();
    int fbest = 0x7fffffff;
    for (int f = lane; f < fb; f += 32) {
        const R d = dot(mv(c.tb().b, c.sb.face_normal(f)), sep);
        if (d > dmax) { dmax = d; fbest = f; }
    }
    warp_argmax(dmax, fbest);
    R dmn = Lim<R>::max();
    int fabest = 0x7fffffff;
    for (int f = lane; f < fa; f += 32) {
        const R d = dot(mv(c.ta().b, c.sa.face_normal(f)), sep);
        if (d < dmn) { dmn = d; fabest = f; }
    }
    warp_argmin(dmn, fabest);
    if (lane == 0 && fbest < 0x7fffffff && fabest < 0x7fffffff) clip_faces(c, sep, -c.ref_scale, R(0), fbest, fabest);
    return true;
}

// SAT pairs: G = 1 runs kSatWarps pairs per block, one warp each, instantiated per shape pairing
// (TA, TB; one launch per pairing); G = kSatGroup runs one heavy pair per block, any pairing (-1).
// Only thread 0 holds the pair's contact cache.
// per-group stride, a multiple of 4 reals so that every group's vertex rows stay 16-byte aligned
template <class R> constexpr int sat_group_reals(int G) {
    return (sat_stage_reals<R>() + sat_scratch_reals<R>(G) + sat_queue_reals<R>(G) + 3) & ~3;
}
static_assert(sat_group_reals<float>(1) % 4 == 0 && (3 * (2 * kSatF + 2 * kSatE)) % 4 == 0, "SAT staging alignment");
template <class R, int G, int TA, int TB>
__global__ void __launch_bounds__(G == 1 ? 32 * kSatWarps : 32 * G, G == 1 ? 16 / kSatWarps : 2)
k_np_sat(int lo, int hi, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, R* sat_out) {
    extern __shared__ __align__(16) unsigned char sat_smem[];
    const int grp = G == 1 ? (int)(threadIdx.x >> 5) : 0;
    const int tid = G == 1 ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
    const int t = lo + blockIdx.x * (G == 1 ? kSatWarps : 1) + grp;
    if (t >= hi) return;   // whole groups leave together
    const int2 q = pairs[order[t]];
    Pair<R> pr;
    pr.xa = B.xf(q.x);
    pr.xb = B.xf(q.y);
    pr.sa = S.view(B.shape[q.x]);
    pr.sb = S.view(B.shape[q.y]);
    pr.c = nullptr;
    sat_staged<R, G, TA, TB>(pr, tid, reinterpret_cast<R*>(sat_smem) + (size_t)grp * sat_group_reals<R>(G),
                             sat_out + (size_t)t * kSatOut);
}

// contact step of the staged SAT pairs, one thread per pair: the pooled result is set up, the
// recorded face-stage and edge-stage points are added and the faces clipped, in the reference's
// order, and the result is sorted and written out
template <class R>
__global__ void k_np_sat_finish(int lo, int hi, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
                                const int* pair_scene_off, const int* prev_off, const R* sat_out) {
    const int t = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= hi) return;
    const int p = order[t];
    Cache<R> cache;
    Pair<R> pr;
    np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, pr);
    const R* o = sat_out + (size_t)t * kSatOut;
    const int fl = (int)o[SO_FLAGS];
    if (fl & 1) pr.add(so_get3(o, SO_FN), so_get3(o, SO_FP), o[SO_FD]);
    if (fl & 2) pr.add(so_get3(o, SO_EN), so_get3(o, SO_EP), o[SO_ED]);
    if (fl & 4) clip_faces(pr, so_get3(o, SO_SEP), -pr.ref_scale, R(0), (int)o[SO_FB], (int)o[SO_FA]);
    np_finish(p, pairs, B, res, cache);
}

// CylinderConvexCollisionAlgorithm (cylinder_convex_collision_algorithm.cpp:109-203), one warp
// per pair: in rounds of 32 faces (in the reference's descending face order, lane i taking the
// i-th face of the round), each lane computes the contact points its face contributes, and lane 0
// then adds them to the pair's cache in face order and, inside a face, in the reference's segment
// order: the cache's merging depends on that order, the candidate points do not.
constexpr int kCylHullCand = 12;   // points a face can give: 6 cylinder segments x 2 ends
template <class R> constexpr int cyl_hull_warps() { return sizeof(R) == 4 ? 4 : 2; }
template <class R>
__global__ void __launch_bounds__(32 * cyl_hull_warps<R>())
k_np_cyl_hull(int lo, int hi, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
              const int* pair_scene_off, const int* prev_off) {
    constexpr int W = cyl_hull_warps<R>(), K = kCylHullCand;
    __shared__ R cand[W][32 * K][7];
    __shared__ int ccnt[W][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = lo + blockIdx.x * W + warp;
    if (t >= hi) return;   // whole warps
    const int p = order[t];
    Cache<R> cache;
    Pair<R> c;
    np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, c, lane == 0);
    const bool a_hull = c.sa.type == ST_HULL;
    const ShapeView<R>& m = a_hull ? c.sa : c.sb;
    const ShapeView<R>& cy = a_hull ? c.sb : c.sa;
    const Xf<R>& to = a_hull ? c.ta() : c.tb();
    const Xf<R>& tc = a_hull ? c.tb() : c.ta();
    const R margin = 0;
    if (lane == 0) cache.swap = a_hull;
    const R cr = cy.radius, ch = cy.height / R(2.0);
    const Xf<R> rel = to.inverse() * tc;
    const V3<R> axis = rel.b.col(1), pos = rel.o;
    V3<R> aa, bb;
    shape_aabb(cy, rel, aa, bb);
    const int dxs[4] = {1, -1, -1, 1}, dys[4] = {1, 1, -1, -1};
    auto push = [&](int& k, const V3<R>& n, const V3<R>& pt, R d) {
        R* e = cand[warp][lane * K + k];
        e[0] = n.x; e[1] = n.y; e[2] = n.z; e[3] = pt.x; e[4] = pt.y; e[5] = pt.z; e[6] = d;
        k++;
    };
    auto drain = [&]() {   // lane 0 adds the round's points in face order
        __syncwarp();
        if (lane == 0)
            for (int l = 0; l < 32; l++)
                for (int k = 0; k < ccnt[warp][l]; k++) {
                    const R* e = cand[warp][l * K + k];
                    c.add(V3<R>(e[0], e[1], e[2]), V3<R>(e[3], e[4], e[5]), e[6]);
                }
        __syncwarp();
    };
    // cylinder side segments against the faces the cylinder's box reaches
    for (int base = 0; base < m.nf; base += 32) {
        const int f = m.nf - 1 - base - lane;
        int k = 0;
        if (f >= 0 && face_hit(m, f, aa, bb)) {
            const V3<R> fn = m.face_normal(f);
            const R adc = dot(axis, fn);
            V3<R> ddx, ddz;
            const V3<R> ddy = axis;
            bool vertical = false;
            if (rabs(rabs(adc) - 1) < eps<R>()) {
                ddz = normalized(cross(axis, V3<R>(1, 0, 0)));
                ddx = normalized(cross(axis, ddz));
                vertical = true;
            } else {
                ddx = normalized(cross(cross(fn, axis), axis));
            }
            auto seg = [&](const V3<R>& ps, const V3<R>& ds, R ls) {
                R t1, t2, d1, d2;
                if (segment_face(m, f, ps, ds, ls, margin, t1, t2, d1, d2)) {
                    const V3<R> p1 = to.apply(ps + ds * t1 - fn * d1);
                    const V3<R> p2 = to.apply(ps + ds * t2 - fn * d2);
                    const V3<R> n = mv(to.b, fn);
                    push(k, n, p1 - n * margin, d1 + margin * 2);
                    push(k, n, p2 - n * margin, d2 + margin * 2);
                }
            };
            for (int i = 0; i < 4; i++) {
                const V3<R> ps = pos + ddx * R(dxs[i]) * cr + ddy * R(dys[i]) * ch;
                const V3<R> ds = (dxs[i] == dys[i] ? ddy : ddx) * R(-dxs[i]);
                const R ls = (dxs[i] == dys[i] ? ch : cr) * 2;
                seg(ps, ds, ls);
            }
            if (vertical)
                for (int i = 0; i < 3; i += 2) {
                    const V3<R> ps = pos + ddz * R(dxs[i]) * cr + ddy * R(dys[i]) * ch;
                    seg(ps, ddy * R(-dxs[i]), ch * 2);
                }
        }
        ccnt[warp][lane] = k;
        drain();
    }
    // hull edges of those faces against the cylinder (a face with more than K edges is left to
    // lane 0, in its turn)
    for (int base = 0; base < m.nf; base += 32) {
        const int f = m.nf - 1 - base - lane;
        int k = 0;
        if (f >= 0 && face_hit(m, f, aa, bb)) {
            const int n = m.face_size(f);
            if (n > K) k = -1;
            else
                for (int i = 0; i < n; i++) {
                    const V3<R> v1 = m.vert(m.face_vert(f, i));
                    const V3<R> v2 = m.vert(m.face_vert(f, (i + 1) % n));
                    R t1, t2;
                    const V3<R> start = (v1 + v2) / R(2);
                    const R ls = norm(v2 - v1) / 2;
                    const V3<R> dir = (v2 - v1) / (ls * 2);
                    if (segment_cylinder(start, dir, ls, pos, axis, ch, cr, margin, t1, t2)) {
                        const V3<R> p1 = start + dir * t1, p2 = start + dir * t2;
                        V3<R> wn, wp;
                        R wd;
                        cyl_contact((p1 + p2) / R(2), pos, axis, cr, ch, to, margin, wn, wp, wd);
                        push(k, wn, wp, wd);
                    }
                }
        }
        ccnt[warp][lane] = k;
        __syncwarp();
        if (lane == 0)
            for (int l = 0; l < 32; l++) {
                if (ccnt[warp][l] >= 0) {
                    for (int q = 0; q < ccnt[warp][l]; q++) {
                        const R* e = cand[warp][l * K + q];
                        c.add(V3<R>(e[0], e[1], e[2]), V3<R>(e[3], e[4], e[5]), e[6]);
                    }
                    continue;
                }
                const int g = m.nf - 1 - base - l, n = m.face_size(g);
                for (int i = 0; i < n; i++) {
                    const V3<R> v1 = m.vert(m.face_vert(g, i));
                    const V3<R> v2 = m.vert(m.face_vert(g, (i + 1) % n));
                    R t1, t2;
                    const V3<R> start = (v1 + v2) / R(2);
                    const R ls = norm(v2 - v1) / 2;
                    const V3<R> dir = (v2 - v1) / (ls * 2);
                    if (segment_cylinder(start, dir, ls, pos, axis, ch, cr, margin, t1, t2)) {
                        const V3<R> p1 = start + dir * t1, p2 = start + dir * t2;
                        add_on_cylinder(c, (p1 + p2) / R(2), pos, axis, cr, ch, to, margin);
                    }
                }
            }
        __syncwarp();
    }
    if (lane == 0) {
        cache.swap = false;
        np_finish(p, pairs, B, res, cache);
    }
}

// SAT pairs with a shape beyond the staging limits (PC_CONVEX_BIG): one warp each, unstaged
template <class R>
__global__ void k_np_sat_big(int lo, int hi, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
                             const int* pair_scene_off, const int* prev_off) {
    const int t = lo + (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (t >= hi) return;
    const int p = order[t];
    Cache<R> cache;
    Pair<R> pr;
    np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, pr);
    sat_warp(pr, lane);
    if (lane == 0) np_finish(p, pairs, B, res, cache);
}

// ===================================================================== solver
// FrictionContactConstraint::initSequentialImpulse (friction_contact_constraint.cpp:9-73), one thread per result
template <class R>
__global__ void k_si_setup(int P, Results<R> res, Bodies<R> B, Rows<R> rows, const int* row_off, StepParams prm, int* status) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
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

// FrictionContactConstraint::iterateSequentialImpulse (friction_contact_constraint.cpp:75-108)
// for all points of one result; temporary velocities live in the body arrays
template <class R>
__device__ __forceinline__ void si_iterate_result(const Bodies<R>& B, const Rows<R>& rows, int ia, int ib, int r0, int np) {
    const bool ka = (B.flags[ia] & BF_KINEMATIC) != 0, kb = (B.flags[ib] & BF_KINEMATIC) != 0;
    V3<R> tva = B.vec(TVX, ia), twa = B.vec(TWX, ia), tvb = B.vec(TVX, ib), twb = B.vec(TWX, ib);
    const R ima = B.at(INVM, ia), imb = B.at(INVM, ib);
    const M3<R> Ia = B.mat(I00, ia), Ib = B.mat(I00, ib);
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
        const R scale = rows.at(MU, r) * nacc / rsqrt_(tt0 * tt0 + tt1 * tt1);
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
__global__ void k_isl_union(int A, const int* active, Results<R> res, Bodies<R> B, int* parent) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A) return;
    const int p = active[t];
    const int ia = res.a[p], ib = res.b[p];
    if ((B.flags[ia] & BF_KINEMATIC) || (B.flags[ib] & BF_KINEMATIC)) return;
    uf_union(parent, ia, ib);
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
__global__ void k_isl_keys_joints(Joints<R> J, Bodies<R> B, const int* parent, int A, uint64_t* key, uint32_t* key2, uint32_t* val) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J.n) return;
    const int ia = J.body[j].x, ib = J.body[j].y;
    const bool ka = (B.flags[ia] & BF_KINEMATIC) != 0, kb = (B.flags[ib] & BF_KINEMATIC) != 0;
    key[A + j] = ka && kb ? (uint64_t)B.n : (uint64_t)uf_find(parent, ka ? ib : ia);
    key2[A + j] = 0;
    val[A + j] = kJointItem | (uint32_t)j;
}
// sort keys: island label (smallest body index of the island) of each active result
template <class R>
__global__ void k_isl_keys(int A, const int* active, Results<R> res, Bodies<R> B, const int* parent, uint64_t* key, uint32_t* key2,
                           uint32_t* val) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A) return;
    const int p = active[t];
    const int ia = res.a[p], ib = res.b[p];
    const int dyn = (B.flags[ia] & BF_KINEMATIC) ? ib : ia;
    key[t] = (uint64_t)uf_find(parent, dyn);
    key2[t] = 0;
    val[t] = (uint32_t)p;
}
__global__ void k_isl_flags(int A, const uint64_t* key, int* flag);
__global__ void k_isl_offsets(int A, const uint64_t* key, const int* scan, int* isl_off, int* n_isl_out);

// serial order inside each island: one thread per island (all islands in serial-order mode,
// islands up to `max_len` results in coloured mode)
template <class R>
__global__ void k_isl_serial(const int* n_isl, const int* isl_off, const uint32_t* order, Results<R> res, Joints<R> J, Bodies<R> B,
                             Rows<R> rows, const int* row_off, int iterations, int min_len, int max_len) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= *n_isl) return;
    const int lo = isl_off[s], hi = isl_off[s + 1];
    if (hi - lo < min_len || hi - lo > max_len) return;
    for (int it = 0; it < iterations; it++)
        for (int k = lo; k < hi; k++) iterate_item(order[k], res, J, B, rows, row_off);
}

constexpr int kSmallResults = 8;   // islands up to this size run in the reference order, one thread each

// coloured Gauss-Seidel of one island per block: greedy colouring in rounds (a result takes
// colour c when it holds the smallest position among the uncoloured results on each of its
// dynamic bodies), then every iteration runs the colours in turn, all results of a colour in
// parallel.  Results still uncoloured after kMaxColors - 1 rounds form a last colour that one
// thread runs in order.
constexpr int kMaxColors = 64;
constexpr int kColorBlock = 64;   // threads per island block: islands run tens of results per colour
constexpr int kBigIsland = 4096;  // larger islands are coloured and solved by the whole grid (k_gc_*)
template <class R>
__global__ void k_isl_colored(const int* n_isl, const int* isl_off, const uint32_t* order, Results<R> res, Joints<R> J, Bodies<R> B,
                              Rows<R> rows, const int* row_off, int iterations, int min_len, int* claim, int* color, uint32_t* corder,
                              int* n_colors_out) {
    const int s = blockIdx.x;
    if (s >= *n_isl) return;
    const int lo = isl_off[s], hi = isl_off[s + 1], m = hi - lo;
    if (m <= min_len || m > kBigIsland) return;
    __shared__ int cnt[kMaxColors + 1];
    __shared__ int remaining;
    __shared__ int ncol;
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
    // leftovers (pathological degree): one last colour, run in order by one thread
    for (int j = threadIdx.x; j < m; j += blockDim.x)
        if (color[lo + j] < 0) color[lo + j] = kMaxColors - 1;
    for (int k = threadIdx.x; k <= kMaxColors; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) atomicAdd(&cnt[color[lo + j] + 1], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < kMaxColors; k++) cnt[k + 1] += cnt[k];   // cnt[c] = first slot of colour c
        atomicMax(n_colors_out, ncol + (cnt[kMaxColors] > cnt[kMaxColors - 1] ? 1 : 0));
    }
    __syncthreads();
    // placement by colour keeping the island order within each colour
    if (threadIdx.x == 0) {
        int fill[kMaxColors];
        for (int k = 0; k < kMaxColors; k++) fill[k] = cnt[k];
        for (int j = 0; j < m; j++) corder[lo + fill[color[lo + j]]++] = order[lo + j];
    }
    __syncthreads();
    for (int it = 0; it < iterations; it++) {
        for (int c = 0; c < kMaxColors - 1; c++) {
            const int a = cnt[c], b = cnt[c + 1];
            if (a == b) continue;
            for (int j = a + threadIdx.x; j < b; j += blockDim.x) iterate_item(corder[lo + j], res, J, B, rows, row_off);
            __syncthreads();
        }
        if (threadIdx.x == 0)
            for (int j = cnt[kMaxColors - 1]; j < cnt[kMaxColors]; j++) iterate_item(corder[lo + j], res, J, B, rows, row_off);
        __syncthreads();
    }
}

// Serial-order mode for an island of up to kBigIsland items, in parallel and exact: levels in rounds
// (an item takes level r in the round where it holds the smallest position among the unleveled
// items on each of its dynamic bodies), so every item runs after all lower-position items that
// share a dynamic body with it and before all higher-position ones: each body receives its updates
// in island order, i.e. the reference's order, and items of one level touch disjoint bodies.  Every
// iteration runs the levels in turn with a block barrier between them.  An island that needs more
// than kMaxLevels levels runs in order on one thread instead.
constexpr int kMaxLevels = 256;
constexpr int kLevelBlock = 256;
template <class R>
__global__ void __launch_bounds__(kLevelBlock) k_isl_levels(const int* n_isl, const int* isl_off, const uint32_t* order, Results<R> res,
                                                            Joints<R> J, Bodies<R> B, Rows<R> rows, const int* row_off, int iterations,
                                                            int min_len, int* claim, int* level, uint32_t* lorder) {
    const int s = blockIdx.x;
    if (s >= *n_isl) return;
    const int lo = isl_off[s], hi = isl_off[s + 1], m = hi - lo;
    if (m <= min_len || m > kBigIsland) return;
    __shared__ int cnt[kMaxLevels + 1];
    __shared__ int remaining;
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
        return;
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
}

// ---- islands above kBigIsland results: k_isl_colored's colouring rule in grid-wide kernels (round
// c gives colour c to every uncoloured result that holds the smallest island position among the
// uncoloured results on each of its dynamic bodies, so the colour classes follow the island order,
// i.e. the reference's solve order, as closely as colouring allows), with up to kMaxColorsBig
// colours, then one launch per colour and iteration.  Results of a colour touch disjoint dynamic
// bodies, so their order inside the colour does not matter; results left after kMaxColorsBig - 1
// rounds run in island order in one thread.
constexpr int kMaxColorsBig = 1024;
__global__ void k_isl_big(const int* n_isl, const int* isl_off, int* big, int* n_big);
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
                                                      int max_rounds, int* n_rounds) {
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

// Body-state transfer in the C ABI's layout (per field group: nk doubles per body, body-major) through
// a device staging buffer: the precision and layout change on the device, so the host side is plain
// copies of the caller's arrays.  Group g holds fields k0[g] .. k0[g] + nk[g] - 1 at off[g] doubles.
struct XferGroups {
    int k0[8], nk[8];
    size_t off[8];
    int n;
};
template <class R>
__global__ void k_state_pack(Bodies<R> B, XferGroups G, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    for (int g = 0; g < G.n; g++)
        for (int k = 0; k < G.nk[g]; k++) out[G.off[g] + (size_t)i * G.nk[g] + k] = (double)B.at(G.k0[g] + k, i);
}
// the inverse; with so, smn, smx >= 0 (the groups of origin, AABB min and max) it also sets the
// body's AABB scale from them, as RigidBody::getAABBScale does (rigidbody.cpp:119-123)
template <class R>
__global__ void k_state_unpack(Bodies<R> B, XferGroups G, const double* in, int so, int smn, int smx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    for (int g = 0; g < G.n; g++)
        for (int k = 0; k < G.nk[g]; k++) B.at(G.k0[g] + k, i) = R(in[G.off[g] + (size_t)i * G.nk[g] + k]);
    if (so >= 0) {
        auto v3 = [&](int g) {
            const double* q = in + G.off[g] + (size_t)i * 3;
            return V3<R>(R(q[0]), R(q[1]), R(q[2]));
        };
        const V3<R> a = v3(smn), d = v3(smx), org = v3(so);
        const R sc = norm(d - a), df = norm(d + a - org * R(2));
        B.at(SCALE, i) = (sc + df) * R(0.5);
    }
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
__global__ void k_active_flags(int P, const int* npts, int* flag);
__global__ void k_active_compact(int P, const int* npts, const int* scan, int* active);

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
