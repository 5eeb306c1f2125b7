// Kernels of the rigid-body step.  One thread per body for integration, a project-written
// LSD radix sort plus a sweep for the broadphase, one thread per collision pair for the
// narrowphase (pairs bucketed by shape pairing), and sequential-impulse solver kernels
// (serial replay of the reference order per scene, or graph-coloured Gauss-Seidel).
#pragma once
#include <cstdint>
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
    shape_aabb(sh, t, mn, mx);
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
// with BroadPhaseBase::validateCollisionPair (broad_phase_base.cpp:5-19).  Pass 0 counts the
// pairs of each sorted position, pass 1 writes them at the scanned offsets.
template <class R>
__global__ void k_bp_sweep(int n, const int* scene_axis, const R* smn, const R* smx, const int* sflag, const int* sscene,
                           const uint32_t* order, int* count, const int* offset, int2* pairs, int pair_cap, int* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int sc = sscene[i];
    const int ax = scene_axis[sc];
    const R* amin = smn + (size_t)ax * n;
    const R maxi_ax = smx[(size_t)ax * n + i];
    const R mnx = smn[i], mny = smn[n + i], mnz = smn[2 * (size_t)n + i];
    const R mxx = smx[i], mxy = smx[n + i], mxz = smx[2 * (size_t)n + i];
    const int fi = sflag[i];
    const bool write = offset != nullptr;
    int c = 0;
    int base = write ? offset[i] : 0;
    if (fi & BF_IGNORE) { if (!write) count[i] = 0; return; }
    for (int j = i + 1; j < n; j++) {
        if (sscene[j] != sc) break;
        if (amin[j] > maxi_ax) break;
        const int fj = sflag[j];
        if (fj & BF_IGNORE) continue;
        if ((fi & BF_KINEMATIC) && (fj & BF_KINEMATIC)) continue;
        const R jmnx = smn[j], jmny = smn[n + j], jmnz = smn[2 * (size_t)n + j];
        const R jmxx = smx[j], jmxy = smx[n + j], jmxz = smx[2 * (size_t)n + j];
        if (mnx > jmxx || jmnx > mxx) continue;
        if (mny > jmxy || jmny > mxy) continue;
        if (mnz > jmxz || jmnz > mxz) continue;
        if (write) {
            const int p = base + c;
            if (p < pair_cap) pairs[p] = make_int2((int)order[i], (int)order[j]);
            else atomicOr(status, ST_PAIR_OVERFLOW);
        }
        c++;
    }
    if (!write) count[i] = c;
}

// next sweep axis of each scene: the axis of largest AABB-centre variance (sweep_and_prune.cpp:37-40).
// One block per scene, sums in a fixed tree order.
template <class R>
__global__ void k_bp_axis(const R* smn, const R* smx, int n, const int* scene_off, int* scene_axis) {
    const int s = blockIdx.x;
    const int lo = scene_off[s], hi = scene_off[s + 1];
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
        const int cnt = hi - lo;
        if (cnt < 2) return;   // the reference returns before touching the axis
        double v[3];
        for (int d = 0; d < 3; d++) v[d] = red[3 + d][0] - red[d][0] * red[d][0] / (double)cnt;
        int ax = 0;
        if (v[1] > v[0]) ax = 1;
        if (v[2] > v[ax]) ax = 2;
        scene_axis[s] = ax;
    }
}

// ===================================================================== narrowphase
// bucket pairs by algorithm class
template <class R>
__global__ void k_np_classify(int P, const int2* pairs, Bodies<R> B, const int* shape_type, int* cls, int* cls_count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int2 q = pairs[p];
    const int c = pair_class(shape_type[B.shape[q.x]], shape_type[B.shape[q.y]]);
    cls[p] = c;
    atomicAdd(&cls_count[c], 1);
}
__global__ void k_np_bucket(int P, const int* cls, int* cursor, int* order);

// One thread per pair: SimpleNarrowPhase::calcContactResults body (simple_narrow_phase.cpp:24-41):
// reset the pooled result, combine materials, dispatch, sort the cache, write the result out.
// Slot distances of a pooled result persist between steps: slot k of result p starts with
// the distance that slot had after the previous step's sort when the same (scene-local)
// result index existed then, and the "fresh result" maximum otherwise.
template <class R>
__global__ void k_np(int P, const int* order, const int* cls, const int2* pairs, Bodies<R> B, ShapeTable<R> S,
                     Results<R> res, const int* pair_scene_off, const int* prev_off, int cls_lo, int cls_hi) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P) return;
    const int p = order[t];
    const int c = cls[p];
    if (c < cls_lo || c > cls_hi) return;
    const int2 q = pairs[p];
    const int ia = q.x, ib = q.y;
    Cache<R> cache;
    cache.valid = 0;
    cache.swap = false;
    {   // stale slot distances of the pooled result
        const int sc = B.scene[ia];
        const int local = p - pair_scene_off[sc];
        if (local < prev_off[sc + 1] - prev_off[sc]) {
            const int src = (prev_off[sc] + local) * kSlots;
            for (int k = 0; k < kSlots; k++) cache.dist[k] = res.prev_dist[src + k];
        } else {
            for (int k = 0; k < kSlots; k++) cache.dist[k] = Lim<R>::max();
        }
    }
    cache.ta = B.xf(ia);
    cache.tb = B.xf(ib);
    cache.scale_a = B.at(SCALE, ia);
    cache.scale_b = B.at(SCALE, ib);
    Pair<R> pr;
    pr.sa = S.view(B.shape[ia]);
    pr.sb = S.view(B.shape[ib]);
    pr.ref_scale = (cache.scale_a + cache.scale_b) * R(0.05);
    pr.c = &cache;
    collide(pr, c);
    // ContactResult::sortContactPoints: stable order by distance over all 8 slots
    int perm[kSlots];
    for (int k = 0; k < kSlots; k++) {
        int j = k;
        const R d = cache.dist[k];
        while (j > 0 && d < cache.dist[perm[j - 1]]) { perm[j] = perm[j - 1]; j--; }
        perm[j] = k;
    }
    int np = kSlots;
    for (int k = 0; k < kSlots; k++) if (!((cache.valid >> perm[k]) & 1u)) { np = k; break; }
    res.a[p] = ia;
    res.b[p] = ib;
    res.npts[p] = np;
    res.fr[p] = rsqrt_(B.at(FRIC, ia) * B.at(FRIC, ib));
    res.re[p] = rsqrt_(B.at(REST, ia) * B.at(REST, ib));
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

// serial-order mode: one thread per scene replays SequentialImpulseSolver::solve's loop
// (sequential_impulse_solver.cpp:60-69) over that scene's results in order
template <class R>
__global__ void k_si_serial(int n_scenes, const int* scene_pair_off, Results<R> res, Bodies<R> B, Rows<R> rows, const int* row_off,
                            int iterations) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_scenes) return;
    const int lo = scene_pair_off[s], hi = scene_pair_off[s + 1];
    for (int it = 0; it < iterations; it++)
        for (int p = lo; p < hi; p++) {
            const int np = res.npts[p];
            if (np) si_iterate_result(B, rows, res.a[p], res.b[p], row_off[p], np);
        }
}

// greedy colouring in rounds: an uncoloured result takes colour c when it holds the smallest
// index among the uncoloured results touching each of its dynamic bodies
template <class R>
__global__ void k_color_claim(int n_active, const int* active, const int* color, Results<R> res, Bodies<R> B, int* claim) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_active) return;
    if (color[t] >= 0) return;
    const int p = active[t];
    const int ia = res.a[p], ib = res.b[p];
    if (!(B.flags[ia] & BF_KINEMATIC)) atomicMin(&claim[ia], t);
    if (!(B.flags[ib] & BF_KINEMATIC)) atomicMin(&claim[ib], t);
}
template <class R>
__global__ void k_color_take(int n_active, const int* active, int* color, Results<R> res, Bodies<R> B, int* claim, int c, int* remaining) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_active) return;
    if (color[t] >= 0) return;
    const int p = active[t];
    const int ia = res.a[p], ib = res.b[p];
    const bool da = !(B.flags[ia] & BF_KINEMATIC), db = !(B.flags[ib] & BF_KINEMATIC);
    const bool win = (!da || claim[ia] == t) && (!db || claim[ib] == t);
    if (win) color[t] = c;
    else atomicAdd(remaining, 1);
}
template <class R>
__global__ void k_color_reset(int n_active, const int* active, const int* color, Results<R> res, int* claim) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_active) return;
    const int p = active[t];
    claim[res.a[p]] = 0x7fffffff;
    claim[res.b[p]] = 0x7fffffff;
}

// coloured Gauss-Seidel: all results of one colour in parallel (no shared dynamic body)
template <class R>
__global__ void k_si_color(int lo, int hi, const int* by_color, Results<R> res, Bodies<R> B, Rows<R> rows, const int* row_off) {
    const int t = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= hi) return;
    const int p = by_color[t];
    si_iterate_result(B, rows, res.a[p], res.b[p], row_off[p], res.npts[p]);
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
__global__ void k_color_count(int n_active, const int* color, int* cnt);
__global__ void k_color_bucket(int n_active, const int* active, const int* color, int* cursor, int* by_color);

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
