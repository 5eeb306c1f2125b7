// Kernels of the rigid-body step, part 3: narrowphase classification, bucketing and the
// closed-form pair kernels.
#pragma once
#include "pe_k_broadphase.cuh"

namespace pe {

// ===================================================================== narrowphase
// bucket pairs by algorithm class
// Shared-memory staging limits of the SAT kernels (faces, unique edges, hull vertices per shape),
// and the scheduling split of ConvexConvexCollisionAlgorithm pairs by estimated work: candidate
// axes x projection cost (hull vertices; a box or cylinder projects in closed form).
constexpr int kSatF = 128, kSatE = 192, kSatV = 64;
constexpr int kSatWarps = 1;                 // pairs (one warp each) per block, light pairs
constexpr int kSatGroup = 8;                 // warps per pair, heavy pairs (one block each)
// resident light SAT blocks per SM the registers are sized for: 12 leaves the warp loop unspilled
// (16, at most 128 registers, spilled: the batched step measured 0.16 ms slower)
constexpr int kSatBlocksPerSm = 12 / kSatWarps;
template <class R> __device__ __forceinline__ bool sat_fits(const ShapeView<R>& s) {
    return s.face_count() <= kSatF && s.edge_count() <= kSatE && (s.type != ST_HULL || s.nv <= kSatV);
}
// heavy: estimated work (axes x projection cost) from which a pair gets a block of warps
template <class R> __device__ __forceinline__ int sat_class(const ShapeView<R>& a, const ShapeView<R>& b, long long heavy) {
    if (!sat_fits(a) || !sat_fits(b)) return PC_CONVEX_BIG;
    auto w = [](const ShapeView<R>& s) { return s.type == ST_HULL ? s.nv : s.type == ST_CYLINDER ? 12 : s.type == ST_BOX ? 8 : 2; };
    auto ue = [](const ShapeView<R>& s) { return s.type == ST_BOX ? 3 : s.edge_count(); };   // distinct edge axes
    const long long axes = (long long)a.face_count() + b.face_count() + (long long)ue(a) * ue(b);
    if (axes * (w(a) + w(b)) >= heavy) return PC_CONVEX_HEAVY;
    if (a.type == ST_HULL && b.type == ST_HULL) return PC_CONVEX_HULL_HULL;
    if (a.type == ST_CYLINDER) return PC_CONVEX_CYL_CYL;
    return a.type == ST_BOX ? PC_CONVEX : PC_CONVEX_HULL_BOX;
}

// The pair count is on the device (*Pd); whole warps stride over it, so that every lane takes part
// in the warp votes.
template <class R>
__global__ void k_np_classify(const int* Pd, const int2* pairs, Bodies<R> B, ShapeTable<R> S, int* cls, int* cls_count, long long heavy) {
    const int P = *Pd;
    for (int base = blockIdx.x * blockDim.x; base < P; base += gridDim.x * blockDim.x) {
        const int p = base + threadIdx.x;
        int c = -1 - (int)(threadIdx.x & 31);   // lanes past the end never match a class
        if (p < P) {
            const int2 q = pairs[p];
            const ShapeView<R> sa = S.view(B.shape[q.x]), sb = S.view(B.shape[q.y]);
            c = pair_class(sa.type, sb.type);
            if (c == PC_CONVEX) c = sat_class(sa, sb, heavy);
            cls[p] = c;
        }
        // one atomic per class present in the warp
        const unsigned peers = __match_any_sync(0xffffffffu, c);
        if (c >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cls_count[c], __popc(peers));
    }
}
__global__ void k_np_bucket(const int* Pd, const int* cls, int* cursor, int* order);
__global__ void k_np_ranges(const int* count, int* cursor, int2* range, int* work);

// Work loops over a class's range [rng.x, rng.y) of the bucketed order, whose size only the device
// knows: the grids are sized by an upper bound, at most the GPU's resident blocks.
// thread_items: one item per thread, grid-strided.
template <class F> __device__ __forceinline__ void thread_items(int2 rng, F&& f) {
    for (int t = rng.x + blockIdx.x * blockDim.x + threadIdx.x; t < rng.y; t += gridDim.x * blockDim.x) f(t);
}
// warp_items: one item per warp, handed out by an atomic cursor (which starts at rng.x), so that
// the warps that finish early take the next items while a long pair holds another warp
template <class F> __device__ __forceinline__ void warp_items(int2 rng, int* cursor, F&& f) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(cursor, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= rng.y) break;
        f(t);
        __syncwarp();
    }
}
// block_items: one item per block, from an atomic cursor
template <class F> __device__ __forceinline__ void block_items(int2 rng, int* cursor, int* slot, F&& f) {
    for (;;) {
        if (threadIdx.x == 0) *slot = atomicAdd(cursor, 1);
        __syncthreads();
        const int t = *slot;
        __syncthreads();
        if (t >= rng.y) break;
        f(t);
        __syncthreads();
    }
}

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
    pr.margin = S.margin;
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
    res.fr[p] = real_sqrt(B.at(FRIC, q.x) * B.at(FRIC, q.y));     // ContactResult::setObjects (contact_result.cpp:80-86)
    res.re[p] = real_sqrt(B.at(REST, q.x) * B.at(REST, q.y));
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

// one thread per pair of one algorithm class; `order[rng)` holds that class's pairs
template <class R, int CLS>
__global__ void k_np_class(const int2* rng, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
                           const int* pair_scene_off, const int* prev_off) {
    thread_items(*rng, [&](int t) {
        const int p = order[t];
        Cache<R> cache;
        Pair<R> pr;
        np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, pr);
        collide(pr, CLS);
        np_finish(p, pairs, B, res, cache);
    });
}

// CompoundCompoundCollisionAlgorithm::processCollision (compound_compound_collision_algorithm.cpp:8-46),
// one thread per pair with a compound on either side.  A compound second swaps the pair (shapes,
// transforms and the result's objects: ContactResult::setObjects(B, A), so the result names the
// compound as object A); then every child of the compound, against every child of a second
// compound or against the other shape, runs its shape pair's algorithm into the same contact
// cache at the child's world transform (body transform * local transform).  Local contact
// positions stay relative to the bodies.
template <class R>
__device__ __forceinline__ void compound_pair(int p, const int2* pairs, const Bodies<R>& B, const ShapeTable<R>& S, const Results<R>& res,
                                              const int* pair_scene_off, const int* prev_off) {
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

template <class R>
__global__ void k_np_compound(const int2* rng, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
                              const int* pair_scene_off, const int* prev_off) {
    thread_items(*rng, [&](int t) { compound_pair(order[t], pairs, B, S, res, pair_scene_off, prev_off); });
}

} // namespace pe
