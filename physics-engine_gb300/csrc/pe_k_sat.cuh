// Kernels of the rigid-body step, part 4: the convex SAT and face clipping (staged, pruned, and
// the contact step).
#pragma once
#include "pe_k_narrowphase.cuh"

namespace pe {

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
            const R r = real_sqrt(la.x * la.x + la.z * la.z);
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
// scratch area (16: the batched step 0.27 ms faster than with 8, 4 slower)
constexpr int kSatQ = 16;
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
// The same test on an unnormalised axis x of length nx (computed as the reference's norm): every
// projection scales by nx, so the bound and the slack are scaled by nx instead of dividing x by
// it.  The normalisation the test skips changes each projection by a few units of roundoff, well
// inside the 64-unit slack.  For boxes and hulls only (a cylinder's closed form branches on
// near-zero components of the normalised axis).
template <class R>
__device__ __forceinline__ void prune_side_scaled(const ShapeView<R>& s, const Xf<R>& t, const V3<R>& x, R nx, R& lo, R& hi, R& mag) {
    if (s.type == ST_HULL) {
        const R o = dot(t.o, x);
        lo = o + s.inner * nx;
        hi = o - s.inner * nx;
        mag = rabs(o) + s.outer * nx;
        return;
    }
    int i0, i1;
    shape_interval(s, t, x, (const R*)nullptr, hi, lo, i0, i1);
    mag = rabs(hi) + rabs(lo);
}
template <class R>
__device__ __forceinline__ bool sat_prunable_scaled(const Pair<R>& c, bool able, const V3<R>& x, R nx, R best) {
    if (!able || !(best < Lim<R>::max())) return false;
    R loA, hiA, mA, loB, hiB, mB;
    prune_side_scaled(c.sa, c.ta(), x, nx, loA, hiA, mA);
    prune_side_scaled(c.sb, c.tb(), x, nx, loB, hiB, mB);
    const R d0 = loA - hiB, d1 = loB - hiA;
    const R lb = d0 < d1 ? d0 : d1;
    constexpr R u = sizeof(R) == 4 ? R(1.1920929e-7) : R(2.220446049250313e-16);
    return lb > nx * best + R(64) * u * (mA + mB + nx * rabs(best));
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
    const R margin = c.margin;
    SatStage<R> st;
    st.bind(smem);
    R* rd = smem + sat_stage_reals<R>();
    int* ri = reinterpret_cast<int*>(rd + G);
    R* bc = rd + 2 * G;
    const int fa = c.sa.face_count(), fb = c.sb.face_count();
    const int na = c.sa.edge_count(), nb = c.sb.edge_count();
    for (int f = tid; f < fa; f += T) st3(st.nA, f, mv(c.ta().b, c.sa.face_normal(f)));
    for (int f = tid; f < fb; f += T) st3(st.nB, f, mv(c.tb().b, c.sb.face_normal(f)));
    // unit edge directions: a hull's come precomputed (k_hull_edge_dirs, the same arithmetic)
    auto edge_unit = [](const ShapeView<R>& sh, int e) {
        if (sh.type == ST_HULL) return sh.edge_dir(e);
        V3<R> a0, a1;
        sh.edge(e, a0, a1);
        return normalized(a0 - a1);
    };
    for (int e = tid; e < na; e += T) st3(st.dA, e, mv(c.ta().b, edge_unit(c.sa, e)));
    for (int e = tid; e < nb; e += T) st3(st.dB, e, mv(c.tb().b, edge_unit(c.sb, e)));
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
    const bool cyl = c.sa.type == ST_CYLINDER || c.sb.type == ST_CYLINDER;
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
          if (cyl) {
              V3<R> a;
              return edge_axis(q, a) && !sat_prunable(c, able, a, pb);
          }
          const int iu = q / ub, ju = q - iu * ub;
          const V3<R> x = cross(ld3(st.dA, boxA ? 4 * iu : iu), ld3(st.dB, boxB ? 4 * ju : ju));
          const R nx = norm(x);
          return !(rabs(nx - 0) < eps<R>()) && !sat_prunable_scaled(c, able, x, nx, pb);   // parallel edges: no axis
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
                const R nl = real_sqrt(nl2);
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
    const R margin = c.margin;
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
                const R nl = real_sqrt(nl2);
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
    if (lane == 0 && fbest < 0x7fffffff && fabest < 0x7fffffff) clip_faces(c, sep, -c.ref_scale, c.margin, fbest, fabest);
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
__global__ void __launch_bounds__(G == 1 ? 32 * kSatWarps : 32 * G, G == 1 ? kSatBlocksPerSm : 2)
k_np_sat(const int2* rng, int* cursor, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, R* sat_out) {
    extern __shared__ __align__(16) unsigned char sat_smem[];
    const int grp = G == 1 ? (int)(threadIdx.x >> 5) : 0;
    const int tid = G == 1 ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
    R* smem = reinterpret_cast<R*>(sat_smem) + (size_t)grp * sat_group_reals<R>(G);
    auto one = [&](int t) {
        const int2 q = pairs[order[t]];
        Pair<R> pr;
        pr.xa = B.xf(q.x);
        pr.xb = B.xf(q.y);
        pr.sa = S.view(B.shape[q.x]);
        pr.sb = S.view(B.shape[q.y]);
        pr.margin = S.margin;
        pr.c = nullptr;
        sat_staged<R, G, TA, TB>(pr, tid, smem, sat_out + (size_t)t * kSatOut);
    };
    if (G == 1) {
        warp_items(*rng, cursor, one);
    } else {
        __shared__ int slot;
        block_items(*rng, cursor, &slot, one);
    }
}

// contact step of the staged SAT pairs, one thread per pair: the pooled result is set up, the
// recorded face-stage and edge-stage points are added and the faces clipped, in the reference's
// order, and the result is sorted and written out
template <class R>
__global__ void k_np_sat_finish(const int2* rng, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
                                const int* pair_scene_off, const int* prev_off, const R* sat_out) {
    thread_items(*rng, [&](int t) {
        const int p = order[t];
        Cache<R> cache;
        Pair<R> pr;
        np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, pr);
        const R* o = sat_out + (size_t)t * kSatOut;
        const int fl = (int)o[SO_FLAGS];
        if (fl & 1) pr.add(so_get3(o, SO_FN), so_get3(o, SO_FP), o[SO_FD]);
        if (fl & 2) pr.add(so_get3(o, SO_EN), so_get3(o, SO_EP), o[SO_ED]);
        if (fl & 4) clip_faces(pr, so_get3(o, SO_SEP), -pr.ref_scale, pr.margin, (int)o[SO_FB], (int)o[SO_FA]);
        np_finish(p, pairs, B, res, cache);
    });
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
k_np_cyl_hull(const int2* rng, int* cursor, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
              const int* pair_scene_off, const int* prev_off) {
    constexpr int W = cyl_hull_warps<R>(), K = kCylHullCand;
    __shared__ R cand[W][32 * K][7];
    __shared__ int ccnt[W][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    warp_items(*rng, cursor, [&](int t) {
    const int p = order[t];
    Cache<R> cache;
    Pair<R> c;
    np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, c, lane == 0);
    const bool a_hull = c.sa.type == ST_HULL;
    const ShapeView<R>& m = a_hull ? c.sa : c.sb;
    const ShapeView<R>& cy = a_hull ? c.sb : c.sa;
    const Xf<R>& to = a_hull ? c.ta() : c.tb();
    const Xf<R>& tc = a_hull ? c.tb() : c.ta();
    const R margin = c.margin;
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
    });
}

// SphereConvexCollisionAlgorithm (sphere_convex_collision_algorithm.cpp:185-210) for a convex hull,
// one warp per pair: in rounds of 32 faces (the face tree's order for a hull, descending face
// index; lane i takes the i-th face of the round) each lane tests its face's box and runs the
// sphere-triangle test on its face's fan triangles; lane 0 then adds the points to the pair's cache
// in face order and, inside a face, in triangle order, as the reference's query callback does.  A
// face with more than kSphereHullCand triangles is left to lane 0 in its turn.
constexpr int kSphereHullCand = 8;
template <class R> constexpr int sphere_hull_warps() { return sizeof(R) == 4 ? 4 : 2; }
template <class R>
__global__ void __launch_bounds__(32 * sphere_hull_warps<R>())
k_np_sphere_hull(const int2* rng, int* cursor, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S, Results<R> res,
                 const int* pair_scene_off, const int* prev_off) {
    constexpr int W = sphere_hull_warps<R>(), K = kSphereHullCand;
    __shared__ R cand[W][32 * K][7];
    __shared__ int ccnt[W][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    warp_items(*rng, cursor, [&](int t) {
    const int p = order[t];
    Cache<R> cache;
    Pair<R> c;
    np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, c, lane == 0);
    const bool a_hull = c.sa.type == ST_HULL;
    const ShapeView<R>& m = a_hull ? c.sa : c.sb;
    const ShapeView<R>& sp = a_hull ? c.sb : c.sa;
    const Xf<R>& tm = a_hull ? c.ta() : c.tb();
    const Xf<R>& ts = a_hull ? c.tb() : c.ta();
    const R margin = c.margin;
    if (lane == 0) cache.swap = a_hull;
    const V3<R> rel = tm.inv_apply(ts.o);
    const R r = sp.radius;
    const V3<R> aa = rel - V3<R>(r, r, r), bb = rel + V3<R>(r, r, r);
    // the points of face f's fan triangles, in order, through emit
    auto face_points = [&](int f, auto&& emit) {
        const int n = m.face_size(f);
        for (int i = 0; i < n - 2; i++) {
            const V3<R> vs[3] = {m.vert(m.face_vert(f, 0)), m.vert(m.face_vert(f, i + 1)), m.vert(m.face_vert(f, i + 2))};
            V3<R> point, normal;
            R depth = 0;
            if (sphere_triangle(rel, r, vs, point, normal, depth)) {
                normal = mv(tm.b, normal);
                point = tm.apply(point);
                emit(normal, point - normal * margin, depth + 2 * margin);
            }
        }
    };
    for (int base = 0; base < m.nf; base += 32) {
        const int f = m.nf - 1 - base - lane;
        int k = 0;
        if (f >= 0 && face_hit(m, f, aa, bb)) {
            if (m.face_size(f) - 2 > K) k = -1;
            else
                face_points(f, [&](const V3<R>& n, const V3<R>& pt, R d) {
                    R* e = cand[warp][lane * K + k];
                    e[0] = n.x; e[1] = n.y; e[2] = n.z; e[3] = pt.x; e[4] = pt.y; e[5] = pt.z; e[6] = d;
                    k++;
                });
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
                } else {
                    face_points(m.nf - 1 - base - l, [&](const V3<R>& n, const V3<R>& pt, R d) { c.add(n, pt, d); });
                }
            }
        __syncwarp();
    }
    if (lane == 0) {
        cache.swap = false;
        np_finish(p, pairs, B, res, cache);
    }
    });
}

// SAT pairs with a shape beyond the staging limits (PC_CONVEX_BIG): one warp each, unstaged
template <class R>
__global__ void k_np_sat_big(const int2* rng, int* cursor, const int* order, const int2* pairs, Bodies<R> B, ShapeTable<R> S,
                             Results<R> res, const int* pair_scene_off, const int* prev_off) {
    const int lane = threadIdx.x & 31;
    warp_items(*rng, cursor, [&](int t) {
        const int p = order[t];
        Cache<R> cache;
        Pair<R> pr;
        np_setup(p, pairs, B, S, res, pair_scene_off, prev_off, cache, pr);
        sat_warp(pr, lane);
        if (lane == 0) np_finish(p, pairs, B, res, cache);
    });
}

} // namespace pe
