// Oracle narrowphase: the contact cache (ContactResult / ContactPoint) and the pair
// algorithms for box, sphere, cylinder and convex-mesh pairs, restating
// src/rigid/collision/narrow_phase/contact_result.cpp and
// src/rigid/collision/collision_algorithm/*.cpp.  Test infrastructure only.
#pragma once
#include <cstring>
#include <vector>
#include "orc_shapes.h"

namespace orc {

constexpr int kCache = 8;   // PE_CONTACT_CACHE_SIZE (contact_result.h:6)

template <class R> struct CPoint {
    V3<R> pos = V3<R>(Limits<R>::max(), Limits<R>::max(), Limits<R>::max());
    V3<R> normal = V3<R>(0, 1, 0);
    V3<R> la, lb;
    R dist = Limits<R>::max();
    V3<R> t0, t1;
    bool valid() const { return (double)pos.x < (double)Limits<R>::max() + 0.1; }   // contact_result.h:73
};

// contact_result.cpp:8-31
template <class R> void ortho_units(V3<R> n, V3<R>& t1, V3<R>& t2) {
    n = normalized(n);
    if (std::abs(n.z) > R(0.7071)) {
        const R a = n.y * n.y + n.z * n.z;
        const R k = R(1.0) / std::sqrt(a);
        t1.x = 0; t1.y = -n.z * k; t1.z = n.y * k;
        t2.x = a * k; t2.y = -n.x * t1.z; t2.z = n.x * t1.y;
    } else {
        const R a = n.x * n.x + n.y * n.y;
        const R k = R(1.0) / std::sqrt(a);
        t1.x = -n.y * k; t1.y = n.x * k; t1.z = 0;
        t2.x = -n.z * t1.y; t2.y = n.z * t1.x; t2.z = a * k;
    }
}

template <class R> struct BodyView {   // what the contact cache needs of a body
    const Transform<R>* t;
    R aabb_scale;
};

template <class R> struct CResult {
    int a = -1, b = -1;
    R friction = 0, restitution = 0;
    int point_size = 0;
    bool swap = false;
    CPoint<R> pts[kCache];

    // contact_result.cpp:158-164
    void clear() {
        for (auto& p : pts) p.pos = V3<R>(Limits<R>::max(), Limits<R>::max(), Limits<R>::max());
        point_size = 0;
        swap = false;
    }

    // contact_result.cpp:88-141 (+ closest-point search :166-181, threshold :183-187)
    void add(const BodyView<R>& A, const BodyView<R>& B, const V3<R>& wn, const V3<R>& wp, R depth) {
        V3<R> pa = wp, pb = wp, n = wn, point = wp;
        if (swap) {
            n = -n;
            pb = wp + wn * depth;
            point = pb;
        } else {
            pa = wp + wn * depth;
        }
        const V3<R> la = A.t->inv_apply(pa);
        const V3<R> lb = B.t->inv_apply(pb);
        R th = (A.aabb_scale < B.aabb_scale ? A.aabb_scale : B.aabb_scale) * R(0.02);
        th *= th;
        int near = -1;
        for (int i = 0; i < kCache; i++) {
            if (!pts[i].valid()) continue;
            const V3<R> d = pts[i].lb - lb;
            const R dd = dot(d, d);
            if (dd < th) { th = dd; near = i; }
        }
        auto make = [&](CPoint<R>& c) {
            c.pos = point; c.normal = n; c.la = la; c.lb = lb; c.dist = depth;
            ortho_units(n, c.t0, c.t1);
        };
        if (near >= 0) {
            if (depth < pts[near].dist) make(pts[near]);
            return;
        }
        for (int i = 0; i < kCache; i++) {
            if (!pts[i].valid()) { make(pts[i]); return; }
        }
        R mx = Limits<R>::min();
        int idx = -1;
        for (int i = 0; i < kCache; i++) {
            if (pts[i].dist > mx) { mx = pts[i].dist; idx = i; }
        }
        if (idx >= 0) make(pts[idx]);
    }

    // contact_result.cpp:144-156: stable ordering by distance over all 8 slots
    // (libstdc++ sorts 8 elements by insertion), size = first invalid slot
    void sort() {
        for (int i = 1; i < kCache; i++) {
            CPoint<R> v = pts[i];
            int j = i;
            while (j > 0 && v.dist < pts[j - 1].dist) { pts[j] = pts[j - 1]; j--; }
            pts[j] = v;
        }
        point_size = kCache;
        for (int i = 0; i < kCache; i++) if (!pts[i].valid()) { point_size = i; break; }
    }
};

template <class R> struct PairCtx {
    const Shape<R>* sa;
    const Shape<R>* sb;
    const Transform<R>* ta;
    const Transform<R>* tb;
    BodyView<R> A, B;
    R ref_scale;
    R margin = 0;   // PE_MARGIN (phys_general.h:45): 0 in the reference's build
    CResult<R>* res;
    void add(const V3<R>& n, const V3<R>& p, R d) { res->add(A, B, n, p, d); }
};

template <class R> inline R rmin(R a, R b) { return a < b ? a : b; }   // PE_MIN
template <class R> inline R rmax(R a, R b) { return a > b ? a : b; }   // PE_MAX
template <class R> inline R rclamp(R x, R lo, R hi) { return rmax(rmin(x, hi), lo); }

// ======================================================================= box-box
// box_box_collision_algorithm.cpp:20-71
template <class R> int rect_quad(const R h[2], R p[8], R ret[16]) {
    int nq = 4, nr = 0;
    R buffer[16];
    R* q = p;
    R* r = ret;
    for (int dir = 0; dir <= 1; dir++) {
        for (int sign = -1; sign <= 1; sign += 2) {
            R* pq = q;
            R* pr = r;
            nr = 0;
            for (int i = nq; i > 0; i--) {
                if (R(sign) * pq[dir] < h[dir]) {
                    pr[0] = pq[0]; pr[1] = pq[1]; pr += 2; nr++;
                    if (nr & 8) { q = r; goto done; }
                }
                R* nq_ = (i > 1) ? pq + 2 : q;
                if ((R(sign) * pq[dir] < h[dir]) ^ (R(sign) * nq_[dir] < h[dir])) {
                    pr[1 - dir] = pq[1 - dir] + (nq_[1 - dir] - pq[1 - dir]) / (nq_[dir] - pq[dir]) * (R(sign) * h[dir] - pq[dir]);
                    pr[dir] = R(sign) * h[dir];
                    pr += 2; nr++;
                    if (nr & 8) { q = r; goto done; }
                }
                pq += 2;
            }
            q = r;
            r = (q == ret) ? buffer : ret;
            nq = nr;
        }
    }
done:
    if (q != ret) std::memcpy(ret, q, nr * 2 * sizeof(R));
    return nr;
}

// box_box_collision_algorithm.cpp:73-135
template <class R> void cull_points(int n, const R p[], int m, int i0, int iret[]) {
    int i;
    R a, cx, cy, q;
    if (n == 1) { cx = p[0]; cy = p[1]; }
    else if (n == 2) { cx = R(0.5) * (p[0] + p[2]); cy = R(0.5) * (p[1] + p[3]); }
    else {
        a = 0; cx = 0; cy = 0;
        for (i = 0; i < n - 1; i++) {
            const R p0 = p[i * 2], p1 = p[i * 2 + 1], p2 = p[i * 2 + 2], p3 = p[i * 2 + 3];
            q = p0 * p3 - p2 * p1;
            a += q;
            cx += q * (p0 + p2);
            cy += q * (p1 + p3);
        }
        const R p0 = p[0], p1 = p[1], pm1 = p[n * 2 - 1], pm2 = p[n * 2 - 2];
        q = pm2 * p1 - p0 * pm1;
        if (std::abs(a + q) > kEps<R>()) a = R(1.0) / (R(3.0) * (a + q));
        else a = Limits<R>::max();
        cx = a * (cx + q * (pm2 + p0));
        cy = a * (cy + q * (pm1 + p1));
    }
    R A[8];
    int avail[8];
    for (i = 0; i < n; i++) { A[i] = std::atan2(p[i * 2 + 1] - cy, p[i * 2] - cx); avail[i] = 1; }
    avail[i0] = 0;
    iret[0] = i0;
    int* ir = iret + 1;
    for (int j = 1; j < m; j++) {
        a = R(j) * (2 * kPi<R>() / m) + A[i0];
        if (a > kPi<R>()) a -= 2 * kPi<R>();
        R maxd = Limits<R>::max();
        *ir = i0;
        for (i = 0; i < n; i++) {
            if (avail[i]) {
                R diff = std::abs(A[i] - a);
                if (diff > kPi<R>()) diff = 2 * kPi<R>() - diff;
                if (diff < maxd) { maxd = diff; *ir = i; }
            }
        }
        avail[*ir] = 0;
        ir++;
    }
}

// box_box_collision_algorithm.cpp:137-580
template <class R> bool box_box(PairCtx<R>& c) {
    const R margin = c.margin;
    const R fudge = R(1.05);
    const V3<R>& p1 = c.ta->origin;
    const V3<R>& p2 = c.tb->origin;
    const M3<R>& R1 = c.ta->basis;
    const M3<R>& R2 = c.tb->basis;
    const V3<R> p = p2 - p1;
    const V3<R> pp = mtv(R1, p);
    R A[3] = {c.sa->size.x * R(0.5), c.sa->size.y * R(0.5), c.sa->size.z * R(0.5)};
    R B[3] = {c.sb->size.x * R(0.5), c.sb->size.y * R(0.5), c.sb->size.z * R(0.5)};
    const M3<R> Rij = mtm(R1, R2);
    R Q11 = std::abs(Rij.m[0][0]), Q12 = std::abs(Rij.m[0][1]), Q13 = std::abs(Rij.m[0][2]);
    R Q21 = std::abs(Rij.m[1][0]), Q22 = std::abs(Rij.m[1][1]), Q23 = std::abs(Rij.m[1][2]);
    R Q31 = std::abs(Rij.m[2][0]), Q32 = std::abs(Rij.m[2][1]), Q33 = std::abs(Rij.m[2][2]);
    bool use_normalR = false;
    V3<R> normalC(0, 0, 0), normalR;
    R s = Limits<R>::min(), s2, l;
    int invert_normal = 0, code = 0;
    auto tst_face = [&](R e1, R e2, const V3<R>& nrm, int cc) -> bool {
        s2 = std::abs(e1) - e2;
        if (s2 > 0) return false;
        if (s2 > s) { s = s2; normalR = nrm; use_normalR = true; invert_normal = e1 < 0; code = cc; }
        return true;
    };
    if (!tst_face(pp[0], A[0] + B[0] * Q11 + B[1] * Q12 + B[2] * Q13, R1.col(0), 1)) return false;
    if (!tst_face(pp[1], A[1] + B[0] * Q21 + B[1] * Q22 + B[2] * Q23, R1.col(1), 2)) return false;
    if (!tst_face(pp[2], A[2] + B[0] * Q31 + B[1] * Q32 + B[2] * Q33, R1.col(2), 3)) return false;
    if (!tst_face(dot(R2.col(0), p), A[0] * Q11 + A[1] * Q21 + A[2] * Q31 + B[0], R2.col(0), 4)) return false;
    if (!tst_face(dot(R2.col(1), p), A[0] * Q12 + A[1] * Q22 + A[2] * Q32 + B[1], R2.col(1), 5)) return false;
    if (!tst_face(dot(R2.col(2), p), A[0] * Q13 + A[1] * Q23 + A[2] * Q33 + B[2], R2.col(2), 6)) return false;
    auto tst_edge = [&](R e1, R e2, R n1, R n2, R n3, int cc) -> bool {
        s2 = std::abs(e1) - e2;
        if (s2 > kEps<R>()) return false;
        l = std::sqrt(n1 * n1 + n2 * n2 + n3 * n3);
        if (l > kEps<R>()) {
            s2 /= l;
            if (s2 * fudge > s) {
                s = s2; use_normalR = false;
                normalC[0] = n1 / l; normalC[1] = n2 / l; normalC[2] = n3 / l;
                invert_normal = e1 < 0; code = cc;
            }
        }
        return true;
    };
    const R eps = kEps<R>();
    Q11 += eps; Q12 += eps; Q13 += eps; Q21 += eps; Q22 += eps; Q23 += eps; Q31 += eps; Q32 += eps; Q33 += eps;
    const auto& Rm = Rij.m;
    if (!tst_edge(pp[2] * Rm[1][0] - pp[1] * Rm[2][0], A[1] * Q31 + A[2] * Q21 + B[1] * Q13 + B[2] * Q12, 0, -Rm[2][0], Rm[1][0], 7)) return false;
    if (!tst_edge(pp[2] * Rm[1][1] - pp[1] * Rm[2][1], A[1] * Q32 + A[2] * Q22 + B[0] * Q13 + B[2] * Q11, 0, -Rm[2][1], Rm[1][1], 8)) return false;
    if (!tst_edge(pp[2] * Rm[1][2] - pp[1] * Rm[2][2], A[1] * Q33 + A[2] * Q23 + B[0] * Q12 + B[1] * Q11, 0, -Rm[2][2], Rm[1][2], 9)) return false;
    if (!tst_edge(pp[0] * Rm[2][0] - pp[2] * Rm[0][0], A[0] * Q31 + A[2] * Q11 + B[1] * Q23 + B[2] * Q22, Rm[2][0], 0, -Rm[0][0], 10)) return false;
    if (!tst_edge(pp[0] * Rm[2][1] - pp[2] * Rm[0][1], A[0] * Q32 + A[2] * Q12 + B[0] * Q23 + B[2] * Q21, Rm[2][1], 0, -Rm[0][1], 11)) return false;
    if (!tst_edge(pp[0] * Rm[2][2] - pp[2] * Rm[0][2], A[0] * Q33 + A[2] * Q13 + B[0] * Q22 + B[1] * Q21, Rm[2][2], 0, -Rm[0][2], 12)) return false;
    if (!tst_edge(pp[1] * Rm[0][0] - pp[0] * Rm[1][0], A[0] * Q21 + A[1] * Q11 + B[1] * Q33 + B[2] * Q32, -Rm[1][0], Rm[0][0], 0, 13)) return false;
    if (!tst_edge(pp[1] * Rm[0][1] - pp[0] * Rm[1][1], A[0] * Q22 + A[1] * Q12 + B[0] * Q33 + B[2] * Q31, -Rm[1][1], Rm[0][1], 0, 14)) return false;
    if (!tst_edge(pp[1] * Rm[0][2] - pp[0] * Rm[1][2], A[0] * Q23 + A[1] * Q13 + B[0] * Q32 + B[1] * Q31, -Rm[1][2], Rm[0][2], 0, 15)) return false;
    if (!code) return false;

    V3<R> normal = use_normalR ? normalR : mv(R1, normalC);
    if (invert_normal) normal = V3<R>(-normal[0], -normal[1], -normal[2]);
    const R depth = -s;

    if (code > 6) {
        V3<R> pa = p1;
        for (int j = 0; j < 3; j++) {
            const R sign = dot(normal, R1.col(j)) > 0 ? R(1.0) : R(-1.0);
            pa[0] += sign * A[j] * R1.m[0][j];
            pa[1] += sign * A[j] * R1.m[1][j];
            pa[2] += sign * A[j] * R1.m[2][j];
        }
        V3<R> pb = p2;
        for (int j = 0; j < 3; j++) {
            const R sign = dot(normal, R2.col(j)) > 0 ? R(-1.0) : R(1.0);
            pb[0] += sign * B[j] * R2.m[0][j];
            pb[1] += sign * B[j] * R2.m[1][j];
            pb[2] += sign * B[j] * R2.m[2][j];
        }
        const int quotient = (code - 7) / 3;   // used for both edges (reference behaviour)
        const V3<R> ua = R1.col(quotient), ub = R2.col(quotient);
        const V3<R> b_a = pb - pa;
        const R ua_ub = dot(ua, ub);
        const R q1 = dot(ua, b_a);
        const R q2 = -dot(ub, b_a);
        R d = 1 - ua_ub * ua_ub, alpha, beta;
        if (d <= kEps<R>()) { alpha = 0; beta = 0; }
        else { d = R(1.0) / d; alpha = (q1 + ua_ub * q2) * d; beta = (ua_ub * q1 + q2) * d; }
        pa[0] += ua[0] * alpha; pa[1] += ua[1] * alpha; pa[2] += ua[2] * alpha;
        pb[0] += ub[0] * beta; pb[1] += ub[1] * beta; pb[2] += ub[2] * beta;
        c.add(-normal, pb + normal * margin, -depth + margin * 2);
        return true;
    }

    const R *Sa, *Sb;
    M3<R> Ra, Rb;
    V3<R> pa, pb;
    if (code <= 3) { c.res->swap = false; Ra = R1; Rb = R2; pa = p1; pb = p2; Sa = A; Sb = B; }
    else { c.res->swap = true; Ra = R2; Rb = R1; pa = p2; pb = p1; Sa = B; Sb = A; }
    const V3<R> normal2 = code <= 3 ? normal : V3<R>(-normal[0], -normal[1], -normal[2]);
    const V3<R> nr = mtv(Rb, normal2);
    const V3<R> anr(std::abs(nr[0]), std::abs(nr[1]), std::abs(nr[2]));
    int lanr, a1, a2;
    if (anr[1] > anr[0]) {
        if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    } else {
        if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    }
    V3<R> center;
    const R sbl = Sb[lanr];
    if (nr[lanr] < 0) for (int k = 0; k < 3; k++) center[k] = pb[k] - pa[k] + sbl * Rb.m[k][lanr];
    else for (int k = 0; k < 3; k++) center[k] = pb[k] - pa[k] - sbl * Rb.m[k][lanr];
    const int codeN = code <= 3 ? code - 1 : code - 4;
    int code1, code2;
    if (codeN == 0) { code1 = 1; code2 = 2; }
    else if (codeN == 1) { code1 = 0; code2 = 2; }
    else { code1 = 0; code2 = 1; }
    R quad[8];
    const R c1 = dot(center, Ra.col(code1));
    const R c2 = dot(center, Ra.col(code2));
    R m11 = dot(Ra.col(code1), Rb.col(a1));
    R m12 = dot(Ra.col(code1), Rb.col(a2));
    R m21 = dot(Ra.col(code2), Rb.col(a1));
    R m22 = dot(Ra.col(code2), Rb.col(a2));
    {
        const R k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
        const R c1mk1 = c1 - k1, c2mk2 = c2 - k2;
        quad[0] = c1mk1 - k3; quad[1] = c2mk2 - k4; quad[2] = c1mk1 + k3; quad[3] = c2mk2 + k4;
        const R c1pk1 = c1 + k1, c2pk2 = c2 + k2;
        quad[4] = c1pk1 + k3; quad[5] = c2pk2 + k4; quad[6] = c1pk1 - k3; quad[7] = c2pk2 - k4;
    }
    const R rect[2] = {Sa[code1], Sa[code2]};
    R ret[16];
    const int n = rect_quad(rect, quad, ret);
    if (n < 1) return false;
    R point[24], dep[8];
    const R det1 = R(1) / (m11 * m22 - m12 * m21);
    m11 *= det1; m12 *= det1; m21 *= det1; m22 *= det1;
    int cnum = 0;
    for (int j = 0; j < n; j++) {
        const R k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
        const R k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
        for (int k = 0; k < 3; k++) point[cnum * 3 + k] = center[k] + k1 * Rb.m[k][a1] + k2 * Rb.m[k][a2];
        dep[cnum] = Sa[codeN] - dot(normal2, V3<R>(point[cnum * 3], point[cnum * 3 + 1], point[cnum * 3 + 2]));
        if (dep[cnum] >= 0) {
            ret[cnum * 2] = ret[j * 2];
            ret[cnum * 2 + 1] = ret[j * 2 + 1];
            cnum++;
        }
    }
    if (cnum < 1) return false;
    int maxc = cnum < 4 ? cnum : 4;
    if (maxc < 1) maxc = 1;
    const V3<R> nv = normal;
    const V3<R> mvv = nv * margin;
    if (cnum <= maxc) {
        for (int j = 0; j < cnum; j++) {
            const V3<R> w(point[j * 3] + pa[0], point[j * 3 + 1] + pa[1], point[j * 3 + 2] + pa[2]);
            if (code < 4) c.add(-nv, w + mvv, -dep[j] + margin * 2);
            else c.add(nv, w - mvv, -dep[j] + margin * 2);
        }
    } else {
        int i1 = 0;
        R maxd = dep[0];
        for (int i = 1; i < cnum; i++) if (dep[i] > maxd) { maxd = dep[i]; i1 = i; }
        int iret[8];
        cull_points(cnum, ret, maxc, i1, iret);
        for (int j = 0; j < maxc; j++) {
            const int k = iret[j];
            const V3<R> w(point[k * 3] + pa[0], point[k * 3 + 1] + pa[1], point[k * 3 + 2] + pa[2]);
            if (code < 4) c.add(-nv, w + mvv, -dep[k] + margin * 2);
            else c.add(nv, w - mvv, -dep[k] + margin * 2);
        }
    }
    return true;
}

// ======================================================================= sphere pairs
// box_sphere_collision_algorithm.cpp:31-80 (the +y branch writes half_extent.x)
template <class R> R sphere_penetration(const V3<R>& he, const V3<R>& pos, V3<R>& cp, V3<R>& n) {
    R fd = he.x - pos.x;
    R md = fd;
    cp.x = he.x;
    n = V3<R>(1, 0, 0);
    fd = he.x + pos.x;
    if (fd < md) { md = fd; cp = pos; cp.x = -he.x; n = V3<R>(-1, 0, 0); }
    fd = he.y - pos.y;
    if (fd < md) { md = fd; cp = pos; cp.y = he.x; n = V3<R>(0, 1, 0); }
    fd = he.y + pos.y;
    if (fd < md) { md = fd; cp = pos; cp.y = -he.y; n = V3<R>(0, -1, 0); }
    fd = he.z - pos.z;
    if (fd < md) { md = fd; cp = pos; cp.z = he.z; n = V3<R>(0, 0, 1); }
    fd = he.z + pos.z;
    if (fd < md) { md = fd; cp = pos; cp.z = -he.z; n = V3<R>(0, 0, -1); }
    return md;
}

// box_sphere_collision_algorithm.cpp:6-29, 82-141
template <class R> bool box_sphere(PairCtx<R>& c) {
    const bool a_is_box = c.sa->type == ST_BOX;
    const Shape<R>* sph = a_is_box ? c.sb : c.sa;
    const Shape<R>* box = a_is_box ? c.sa : c.sb;
    const Transform<R>& tsph = a_is_box ? *c.tb : *c.ta;
    const Transform<R>& tbox = a_is_box ? *c.ta : *c.tb;
    const V3<R> center = tsph.origin;
    const R radius = sph->radius;
    const R margin = c.margin;
    c.res->swap = a_is_box;
    bool ret = false;
    {
        const V3<R> he = box->size / R(2.0);
        const V3<R> pos = tbox.inv_apply(center);
        V3<R> cp = pos;
        cp.x = rmin(he.x, cp.x); cp.x = rmax(-he.x, cp.x);
        cp.y = rmin(he.y, cp.y); cp.y = rmax(-he.y, cp.y);
        cp.z = rmin(he.z, cp.z); cp.z = rmax(-he.z, cp.z);
        V3<R> normal = pos - cp;
        const R d2 = sqnorm(normal);
        if (!(d2 > radius * radius)) {
            R distance;
            if (d2 <= kEps<R>() * kEps<R>()) distance = -sphere_penetration(he, pos, cp, normal);
            else { distance = norm(normal); normal = normal / distance; }
            normal = mv(tbox.basis, normal);
            const V3<R> pt = tbox.apply(cp);
            const R dist = distance - radius;
            c.add(normal, pt - normal * margin, dist + 2 * margin);
            c.res->swap = false;
            ret = true;
        }
    }
    c.res->swap = false;
    return ret;
}

// sphere_sphere_collision_algorithm.cpp:23-37
template <class R> bool sphere_sphere(PairCtx<R>& c) {
    const R ra = c.sa->radius, rb = c.sb->radius, margin = c.margin;
    const V3<R> rel = c.ta->origin - c.tb->origin;
    const R dist = norm(rel);
    if (dist > ra + rb || std::abs(dist - 0) < kEps<R>()) return false;
    const V3<R> normal = rel / dist;
    const V3<R> ptb = c.tb->origin + normal * rb;
    const R depth = dist - ra - rb;
    c.add(normal, ptb - normal * margin, depth + 2 * margin);
    return true;
}

// sphere_cylinder_collision_algorithm.cpp:6-76
template <class R> bool sphere_cylinder(PairCtx<R>& c) {
    const bool a_is_sph = c.sa->type == ST_SPHERE;
    const Shape<R>* sph = a_is_sph ? c.sa : c.sb;
    const Shape<R>* cyl = a_is_sph ? c.sb : c.sa;
    const Transform<R>& tsph = a_is_sph ? *c.ta : *c.tb;
    const Transform<R>& tcyl = a_is_sph ? *c.tb : *c.ta;
    const R margin = c.margin;
    c.res->swap = a_is_sph;
    bool ret = [&]() {
        const R s_r = sph->radius, c_r = cyl->radius, c_h = cyl->height * R(0.5);
        const V3<R> s = tcyl.inv_apply(tsph.origin);
        const R r = std::sqrt(s.x * s.x + s.z * s.z);
        const R d = std::abs(s.y) - c_h;
        if (s.y < -c_h - s_r || s.y > c_h + s_r || r * r > (c_r + s_r) * (c_r + s_r) ||
            (d > 0 && r > c_r && (r - c_r) * (r - c_r) + d * d > s_r * s_r))
            return false;
        V3<R> normal, pt;
        R depth;
        if (s.y >= -c_h && s.y <= c_h && r > 0) {
            normal = normalized(V3<R>(-s.x, 0, -s.z));
            pt = normal * s_r + s;
            depth = c_r + s_r - r;
        } else if (r <= c_r) {
            normal = V3<R>(0, 1, 0);
            if (s.y > 0) normal = -normal;
            pt = s + normal * s_r;
            depth = s_r + c_h - std::abs(s.y);
        } else {
            V3<R> pc = normalized(V3<R>(s.x, 0, s.z)) * c_r;
            pc.y = s.y > 0 ? c_h : -c_h;
            normal = normalized(pc - s);
            pt = normal * s_r + s;
            depth = s_r - norm(s - pc);
        }
        normal = mv(tcyl.basis, normal);
        pt = tcyl.apply(pt);
        c.add(normal, pt - normal * margin, -depth + 2 * margin);
        return true;
    }();
    c.res->swap = false;
    return ret;
}

// ======================================================================= box-cylinder
// box_cylinder_collision_algorithm.cpp:79-114
template <class R> void add_on_box(PairCtx<R>& c, const V3<R>& pc, int face, const V3<R>& he, const Transform<R>& t, R margin) {
    if (!(face >= -3 && face <= 3 && face != 0)) return;
    for (int i = 0; i < 3; i++) if (pc[i] > he[i] || pc[i] < -he[i]) return;
    V3<R> p = pc, n(0, 0, 0);
    R pen;
    if (face > 0) { const int i = face - 1; p[i] = he[i]; n[i] = 1; pen = pc[i] - he[i]; }
    else { const int i = -face - 1; p[i] = -he[i]; n[i] = -1; pen = -pc[i] - he[i]; }
    const V3<R> normal = mv(t.basis, n);
    const V3<R> point = t.apply(p);
    c.add(normal, point - normal * margin, pen + 2 * margin);
}

// box_cylinder_collision_algorithm.cpp:116-139
template <class R> void add_on_cylinder(PairCtx<R>& c, const V3<R>& p, const V3<R>& pos, const V3<R>& axis, R radius, R h,
                                        const Transform<R>& t, R margin) {
    const V3<R> r = p - pos;
    const R dy = dot(r, axis);
    const R dxz = std::sqrt(sqnorm(r) - dy * dy);
    const R dside = radius - dxz;
    const R dtop = h - std::abs(dy);
    V3<R> normal;
    R dist;
    if (dside < dtop) { dist = dside; normal = normalized(axis * dy - r); }
    else { dist = dtop; normal = dy < 0 ? axis : -axis; }
    normal = mv(t.basis, normal);
    const V3<R> point = t.apply(p);
    c.add(normal, point - normal * margin, -dist + 2 * margin);
}

template <class R> int closest_box_face(const V3<R>& he, const V3<R>& loc) {   // :141-157
    int code = 0;
    R dist = Limits<R>::max();
    for (int i = 0; i < 3; i++) {
        const R pd = std::abs(loc[i] - he[i]), nd = std::abs(loc[i] + he[i]);
        if (pd < dist) { code = i + 1; dist = pd; }
        if (nd < dist) { code = -(i + 1); dist = nd; }
    }
    return code;
}

template <class R> bool line_plane(const V3<R>& s, const V3<R>& d, const V3<R>& pp, const V3<R>& pn, R tol, R& t) {   // :159-169
    const R nd = dot(pn, d);
    if (std::abs(nd) < tol) return false;
    t = dot(pn, pp - s) / nd;
    return true;
}

template <class R> bool segment_box(const V3<R>& he, const V3<R>& pos, const V3<R>& axis, R h, R tol, R& tmin, R& tmax) {   // :171-231
    tmin = Limits<R>::min();
    tmax = Limits<R>::max();
    for (int k = 0; k < 3; k++) {
        if (std::abs(axis[k]) < tol) {
            if (std::abs(pos[k]) > he[k]) return false;
        } else {
            const R t1 = (-he[k] - pos[k]) / axis[k];
            const R t2 = (+he[k] - pos[k]) / axis[k];
            tmin = rmax(tmin, rmin(t1, t2));
            tmax = rmin(tmax, rmax(t1, t2));
            if (tmin > tmax) return false;
        }
    }
    if ((tmin < -h && tmax < -h) || (tmin > +h && tmax > +h)) return false;
    tmin = rclamp(tmin, -h, +h);
    tmax = rclamp(tmax, -h, +h);
    return true;
}

template <class R> bool segment_cylinder(const V3<R>& s, const V3<R>& d, R len, const V3<R>& pos, const V3<R>& axis, R h,
                                         R radius, R tol, R& tmin, R& tmax) {   // :233-304
    tmin = Limits<R>::min();
    tmax = Limits<R>::max();
    const V3<R> v = s - pos;
    const R cd_sd = dot(axis, d), v_cd = dot(v, axis), v_sd = dot(v, d), v_v = dot(v, v);
    const R a = R(1.0) - cd_sd * cd_sd;
    const R b = v_sd - v_cd * cd_sd;
    const R cc = v_v - v_cd * v_cd - radius * radius;
    if (std::abs(a) < tol) {
        const R d2 = sqnorm(v - v_cd * axis);
        if (d2 > radius * radius) return false;
        tmin = -len; tmax = +len;
    } else {
        R delta = b * b - a * cc;
        if (delta < 0) return false;
        delta = std::sqrt(delta);
        tmin = (-b - delta) / a;
        tmax = (-b + delta) / a;
    }
    R t1, t2;
    const bool c1 = line_plane(s, d, pos + h * axis, axis, tol, t1);
    const bool c2 = line_plane(s, d, pos - h * axis, axis, tol, t2);
    if (c1 && c2) {
        if (t1 < t2) { tmin = rmax(tmin, t1); tmax = rmin(tmax, t2); }
        else { tmin = rmax(tmin, t2); tmax = rmin(tmax, t1); }
        if (tmax < tmin) return false;
    } else {
        const R d1 = std::abs(dot(axis, pos + h * axis - s));
        const R d2 = std::abs(dot(axis, pos - h * axis - s));
        if (d1 > 2 * h || d2 > 2 * h) return false;
    }
    if ((tmin < -len && tmax < -len) || (tmin > +len && tmax > +len)) return false;
    tmin = rclamp(tmin, -len, +len);
    tmax = rclamp(tmax, -len, +len);
    return true;
}

// box_cylinder_collision_algorithm.cpp:13-50, 306-389
template <class R> bool box_cylinder(PairCtx<R>& c) {
    const bool a_is_box = c.sa->type == ST_BOX;
    const Shape<R>* box = a_is_box ? c.sa : c.sb;
    const Shape<R>* cyl = a_is_box ? c.sb : c.sa;
    const Transform<R>& tbox = a_is_box ? *c.ta : *c.tb;
    const Transform<R>& tcyl = a_is_box ? *c.tb : *c.ta;
    const R cyl_r = cyl->radius, cyl_h = cyl->height / R(2.0), margin = c.margin;
    const V3<R> he = box->size / R(2.0);
    c.res->swap = a_is_box;
    const Transform<R> rel = tbox.inverse() * tcyl;
    const V3<R> axis = rel.basis.col(1);
    const V3<R> pos = rel.origin;
    for (int i = 0; i < 3; i++) {
        V3<R> nd(0, 0, 0);
        nd[i] = 1;
        if (std::abs(axis[i] - 1) < kEps<R>() || std::abs(axis[i] + 1) < kEps<R>()) continue;
        const V3<R> r = normalized(cross(cross(nd, axis), axis)) * cyl_r;
        const R dirs[2] = {-1, 1};
        for (R jd : dirs) {
            const V3<R> cs = pos + jd * r;
            R tmin, tmax;
            if (segment_box(he, cs, axis, cyl_h, kEps<R>(), tmin, tmax)) {
                const V3<R> pmin = cs + axis * tmin;
                const V3<R> pmax = cs + axis * tmax;
                const V3<R> pmid = cs + axis * ((tmin + tmax) / 2);
                const int face = closest_box_face(he, pmid);
                add_on_box(c, pmin, face, he, tbox, margin);
                add_on_box(c, pmax, face, he, tbox, margin);
            }
        }
    }
    for (int i = 0; i < 3; i++) {
        V3<R> ed(0, 0, 0);
        ed[i] = 1;
        const R eh = he[i];
        const int jd = (i + 1) % 3, kd = (i + 2) % 3;
        for (int j = -1; j <= 1; j += 2) {
            for (int k = -1; k <= 1; k += 2) {
                V3<R> ec;
                ec[i] = 0;
                ec[jd] = j * he[jd];
                ec[kd] = k * he[kd];
                R tmin, tmax;
                if (segment_cylinder(ec, ed, eh, pos, axis, cyl_h, cyl_r, kEps<R>(), tmin, tmax)) {
                    const V3<R> pmid = ec + ed * ((tmin + tmax) / 2);
                    add_on_cylinder(c, pmid, pos, axis, cyl_r, cyl_h, tbox, margin);
                }
            }
        }
    }
    c.res->swap = false;
    return true;
}

// ======================================================================= convex SAT
// convex_convex_collision_algorithm.cpp:29-61
template <class R> void clip_face(const std::vector<V3<R>>& in, std::vector<V3<R>>& out, const V3<R>& pn, R pe) {
    const int nv = (int)in.size();
    if (nv < 2) return;
    V3<R> first = in[nv - 1];
    R ds = dot(pn, first) + pe;
    for (int ve = 0; ve < nv; ve++) {
        const V3<R> end = in[ve];
        const R de = dot(pn, end) + pe;
        if (ds < 0) {
            if (de < 0) out.push_back(end);
            else out.push_back(first + (end - first) * R(ds * 1.f / (ds - de)));
        } else if (de < 0) {
            out.push_back(first + (end - first) * R(ds * 1.f / (ds - de)));
            out.push_back(end);
        }
        first = end;
        ds = de;
    }
}

template <class R> bool test_sep_axis(PairCtx<R>& c, const V3<R>& axis, R& depth, V3<R>& wa, V3<R>& wb) {   // :216-243
    R min0, max0, min1, max1;
    V3<R> a0, a1, b0, b1;
    project(*c.sa, *c.ta, axis, min0, max0, a0, a1);
    project(*c.sb, *c.tb, axis, min1, max1, b0, b1);
    if (max0 < min1 || max1 < min0) return false;
    const R d0 = max0 - min1, d1 = max1 - min0;
    if (d0 < d1) { depth = d0; wa = a1; wb = b0; }
    else { depth = d1; wa = a0; wb = b1; }
    return true;
}

template <class R> bool on_line(const V3<R>& v0, const V3<R>& v1, const V3<R>& v2) {   // :245-249
    const V3<R> e = v1 - v0;
    return sqnorm(cross(e, v2 - v0)) < kEps<R>();
}

// :172-214
template <class R> void seg_closest(V3<R>& pts, V3<R>& oa, V3<R>& ob, R& ta, R& tb, const V3<R>& tr, const V3<R>& da, R ha,
                                    const V3<R>& db, R hb) {
    const R ab = dot(da, db), at = dot(da, tr), bt = dot(db, tr);
    const R d = R(1.0) - ab * ab;
    if (d == 0) ta = 0;
    else {
        ta = (at - bt * ab) / d;
        if (ta < -ha) ta = -ha;
        else if (ta > ha) ta = ha;
    }
    tb = ta * ab - bt;
    if (tb < -hb) {
        tb = -hb;
        ta = tb * ab + at;
        if (ta < -ha) ta = -ha;
        else if (ta > ha) ta = ha;
    } else if (tb > hb) {
        tb = hb;
        ta = tb * ab + at;
        if (ta < -ha) ta = -ha;
        else if (ta > ha) ta = ha;
    }
    oa = da * ta;
    ob = db * tb;
    pts = tr - oa + ob;
}

// :251-402
template <class R> bool find_sep_axis(PairCtx<R>& c, V3<R>& sep) {
    const R margin = c.margin;
    const Shape<R>& A = *c.sa;
    const Shape<R>& B = *c.sb;
    const V3<R> dc = c.ta->origin - c.tb->origin;
    R dmin = Limits<R>::max();
    V3<R> dmin_pt;
    bool pt_on_a = false;
    for (const auto& f : A.faces) {
        V3<R> n = mv(c.ta->basis, f.normal);
        if (dot(dc, n) < 0) n = n * R(-1.0);
        R d;
        V3<R> wa, wb;
        if (!test_sep_axis(c, n, d, wa, wb)) return false;
        if (d < dmin) { dmin = d; dmin_pt = wb; pt_on_a = false; sep = n; }
    }
    for (const auto& f : B.faces) {
        V3<R> n = mv(c.tb->basis, f.normal);
        if (dot(dc, n) < 0) n = n * R(-1.0);
        R d;
        V3<R> wa, wb;
        if (!test_sep_axis(c, n, d, wa, wb)) return false;
        if (d < dmin) { dmin = d; dmin_pt = wa + n * d; pt_on_a = true; sep = n; }
    }
    if ((pt_on_a && local_inside(B, c.tb->inv_apply(dmin_pt))) || (!pt_on_a && local_inside(A, c.ta->inv_apply(dmin_pt))))
        c.add(sep, dmin_pt - sep * margin, -dmin + margin * 2);
    int ea = -1, eb = -1;
    V3<R> wea, web, wpa(0, 0, 0), wpb(0, 0, 0);
    for (int e0 = 0; e0 < (int)A.edge_a.size(); e0++) {
        const V3<R> ed0 = normalized(A.edge_a[e0] - A.edge_b[e0]);
        const V3<R> w0 = mv(c.ta->basis, ed0);
        for (int e1 = 0; e1 < (int)B.edge_a.size(); e1++) {
            const V3<R> ed1 = normalized(B.edge_a[e1] - B.edge_b[e1]);
            const V3<R> w1 = mv(c.tb->basis, ed1);
            V3<R> cr = cross(w0, w1);
            if (!(std::abs(norm(cr) - 0) < kEps<R>())) {
                cr = normalized(cr);
                if (dot(dc, cr) < 0) cr = cr * R(-1.0);
                R dist;
                V3<R> wa, wb;
                if (!test_sep_axis(c, cr, dist, wa, wb)) return false;
                if (dist < dmin) {
                    if (!on_line(A.edge_a[e0], A.edge_b[e0], c.ta->inv_apply(wa)) ||
                        !on_line(B.edge_a[e1], B.edge_b[e1], c.tb->inv_apply(wb)))
                        continue;
                    dmin = dist; sep = cr; ea = e0; eb = e1; wea = w0; web = w1; wpa = wa; wpb = wb;
                }
            }
        }
    }
    if (ea >= 0 && eb >= 0) {
        V3<R> pts, oa, ob;
        R ta, tb;
        const V3<R> tr = wpb - wpa;
        seg_closest(pts, oa, ob, ta, tb, tr, wea, Limits<R>::max(), web, Limits<R>::max());
        const R nl2 = sqnorm(pts);
        if (nl2 > kEps<R>()) {
            const R nl = std::sqrt(nl2);
            pts = pts * (R(1.0) / nl);
            if (dot(pts, dc) < 0) pts = pts * R(-1.0);
            const V3<R> ptb = wpb + ob;
            c.add(pts, ptb - pts * margin, -nl + margin * 2);
        }
    }
    if (dot(dc, sep) < 0) sep = -sep;
    return true;
}

// :63-170
template <class R> void clip_hull_hull(PairCtx<R>& c, const V3<R>& sep, R min_dist, R max_dist) {
    const R margin = c.margin;
    const Shape<R>& A = *c.sa;
    const Shape<R>& B = *c.sb;
    int fb = -1;
    {
        R dmax = Limits<R>::min();
        for (int f = 0; f < (int)B.faces.size(); f++) {
            const R d = dot(mv(c.tb->basis, B.faces[f].normal), sep);
            if (d > dmax) { dmax = d; fb = f; }
        }
    }
    if (fb < 0) return;
    std::vector<V3<R>> b1, b2;
    for (int k : B.faces[fb].idx) b1.push_back(c.tb->apply(B.verts[k]));
    std::vector<V3<R>>* pin = &b1;
    std::vector<V3<R>>* pout = &b2;
    int fa = -1;
    {
        R dmin = Limits<R>::max();
        for (int f = 0; f < (int)A.faces.size(); f++) {
            const R d = dot(mv(c.ta->basis, A.faces[f].normal), sep);
            if (d < dmin) { dmin = d; fa = f; }
        }
    }
    if (fa < 0) return;
    const Face<R>& poly = A.faces[fa];
    const int nva = (int)poly.idx.size();
    const V3<R> wpn = mv(c.ta->basis, poly.normal);
    for (int e0 = 0; e0 < nva; e0++) {
        const V3<R> a = A.verts[poly.idx[e0]];
        const V3<R> b = A.verts[poly.idx[(e0 + 1) % nva]];
        const V3<R> ew = mv(c.ta->basis, a - b);
        const V3<R> pn = -cross(ew, wpn);
        const V3<R> wa = c.ta->apply(a);
        const R pe = -dot(wa, pn);
        clip_face(*pin, *pout, pn, pe);
        std::swap(pin, pout);
        pout->clear();
    }
    const V3<R> pv = A.verts[poly.idx[0]];
    const V3<R> lpn = poly.normal;
    for (size_t i = 0; i < pin->size(); i++) {
        const V3<R> v = (*pin)[i];
        const R depth = dot(lpn, c.ta->inv_apply(v) - pv);
        if (depth <= max_dist && depth >= min_dist) c.add(sep, v - sep * margin, depth + margin * 2);
    }
}

// :408-432 (used for cylinder-cylinder, box-hull, hull-hull)
template <class R> bool convex_convex(PairCtx<R>& c) {
    V3<R> sep;
    if (!find_sep_axis(c, sep)) return false;
    clip_hull_hull(c, sep, -c.ref_scale, c.margin);   // :426-429: window [-refScale, margin]
    return true;
}

// ======================================================================= sphere-hull
// sphere_convex_collision_algorithm.cpp:36-163
template <class R> R seg_sqr_dist(const V3<R>& from, const V3<R>& to, const V3<R>& p, V3<R>& nearest) {
    V3<R> diff = p - from;
    const V3<R> v = to - from;
    R t = dot(v, diff);
    if (t > 0) {
        const R vv = dot(v, v);
        if (t < vv) { t /= vv; diff = diff - t * v; }
        else { t = 1; diff = diff - v; }
    } else t = 0;
    nearest = from + t * v;
    return dot(diff, diff);
}

template <class R> bool point_in_tri(const V3<R>* vs, const V3<R>& n, const V3<R>& p) {
    const V3<R> e1 = vs[1] - vs[0], e2 = vs[2] - vs[1], e3 = vs[0] - vs[2];
    const V3<R> p1 = p - vs[0], p2 = p - vs[1], p3 = p - vs[2];
    const R r1 = dot(cross(e1, n), p1), r2 = dot(cross(e2, n), p2), r3 = dot(cross(e3, n), p3);
    return (r1 > 0 && r2 > 0 && r3 > 0) || (r1 <= 0 && r2 <= 0 && r3 <= 0);
}

template <class R> bool sphere_triangle(const V3<R>& ctr, R radius, const V3<R>* vs, V3<R>& point, V3<R>& rn, R& depth) {
    const R rt = radius;
    V3<R> n = cross(vs[1] - vs[0], vs[2] - vs[0]);
    const R l2 = sqnorm(n);
    bool has = false;
    V3<R> cp;
    if (l2 >= kEps<R>() * kEps<R>()) {
        n = n / std::sqrt(l2);
        const V3<R> p1c = ctr - vs[0];
        R dfp = dot(p1c, n);
        if (dfp < 0) { dfp *= R(-1.); n = n * R(-1.); }
        if (dfp < rt) {
            if (point_in_tri(vs, n, ctr)) { has = true; cp = ctr - n * dfp; }
            else {
                R md = rt * rt;
                V3<R> ne;
                for (int i = 0; i < 3; i++) {
                    const R ds = seg_sqr_dist(vs[i], vs[(i + 1) % 3], ctr, ne);
                    if (ds < md) { md = ds; has = true; cp = ne; }
                }
            }
        }
    }
    if (has) {
        const V3<R> cc = ctr - cp;
        const R ds = sqnorm(cc);
        if (ds < rt * rt) {
            if (ds > kEps<R>() * kEps<R>()) {
                const R dist = std::sqrt(ds);
                rn = normalized(cc);
                point = cp;
                depth = -(radius - dist);
            } else {
                rn = n;
                point = cp;
                depth = -radius;
            }
            return true;
        }
    }
    return false;
}

// sphere_convex_collision_algorithm.cpp:11-34, 165-211
template <class R> bool sphere_hull(PairCtx<R>& c) {   // also the concave mesh (concave_sphere_collision_algorithm.cpp:8-31)
    const bool a_is_hull = c.sa->type == ST_HULL || c.sa->type == ST_CONCAVE;
    const Shape<R>& mesh = a_is_hull ? *c.sa : *c.sb;
    const Shape<R>& sph = a_is_hull ? *c.sb : *c.sa;
    const Transform<R>& tm = a_is_hull ? *c.ta : *c.tb;
    const Transform<R>& ts = a_is_hull ? *c.tb : *c.ta;
    const R margin = c.margin;
    c.res->swap = a_is_hull;
    const V3<R> rel = tm.inv_apply(ts.origin);
    const R r = sph.radius;
    const V3<R> AA = rel - V3<R>(r, r, r), BB = rel + V3<R>(r, r, r);
    std::vector<int> hit;
    bvh_search(mesh, AA, BB, hit);
    bool ret = false;
    for (int fi : hit) {
        const Face<R>& f = mesh.faces[fi];
        for (int i = 0; i < (int)f.idx.size() - 2; i++) {
            V3<R> vs[3] = {mesh.verts[f.idx[0]], mesh.verts[f.idx[i + 1]], mesh.verts[f.idx[i + 2]]};
            V3<R> point, normal;
            R depth = 0;
            const V3<R> ctr = tm.inv_apply(ts.origin);
            if (sphere_triangle(ctr, r, vs, point, normal, depth)) {
                normal = mv(tm.basis, normal);
                point = tm.apply(point);
                c.add(normal, point - normal * margin, depth + 2 * margin);
                ret = true;
            }
        }
    }
    c.res->swap = false;
    return ret;
}

// ======================================================================= cylinder-hull
// cylinder_convex_collision_algorithm.cpp:53-107
template <class R> bool segment_face(const Face<R>& f, const Shape<R>& mesh, const V3<R>& ps, const V3<R>& ds, R ls, R margin,
                                     R& t1, R& t2, R& d1, R& d2) {
    const V3<R> origin = mesh.verts[f.idx[0]];
    const V3<R> es = ps + ds * ls;
    const V3<R> r1 = ps - origin, r2 = es - origin;
    const R dist1 = dot(r1, f.normal), dist2 = dot(r2, f.normal);
    if ((dist1 > 0 && dist2 > 0) || (dist1 <= 0 && dist2 <= 0)) return false;
    const R t = dist1 / (dist1 - dist2) * ls;
    const V3<R> v = ps + ds * t;
    R tmin = 0, tmax = ls;
    R mde = Limits<R>::max();
    const int n = (int)f.idx.size();
    for (int i = 0; i < n; i++) {
        const V3<R>& v0 = mesh.verts[f.idx[i]];
        const V3<R>& v1 = mesh.verts[f.idx[(i + 1) % n]];
        const V3<R> tc = normalized(cross(f.normal, v1 - v0));
        const R dd = dot(ds, tc);
        mde = rmin(mde, std::abs(dot(v0 - v, tc)));
        if (!(std::abs(dd - 0) < kEps<R>())) {
            if (dd > 0) tmin = rmax(tmin, dot(v0 - ps, tc) / dd);
            else tmax = rmin(tmax, dot(v0 - ps, tc) / dd);
        } else {
            if (dot(cross(v0 - v, v1 - v), f.normal) < 0) return false;
        }
    }
    if (t < tmin || t > tmax) return false;
    t1 = dist1 <= 0 ? tmin : t;
    t2 = dist2 <= 0 ? tmax : t;
    d1 = dist1 <= 0 ? dist1 * (t - tmin) / t : 0;
    d2 = dist2 <= 0 ? dist2 * (tmax - t) / (ls - t) : 0;
    if (-d1 > mde + margin || -d2 > mde + margin) return false;
    return true;
}

// cylinder_convex_collision_algorithm.cpp:11-51, 109-203
template <class R> bool cylinder_hull(PairCtx<R>& c) {   // also the concave mesh (concave_cylinder_collision_algorithm.cpp:37-47)
    const bool a_is_hull = c.sa->type == ST_HULL || c.sa->type == ST_CONCAVE;
    const Shape<R>& mesh = a_is_hull ? *c.sa : *c.sb;
    const Shape<R>& cyl = a_is_hull ? *c.sb : *c.sa;
    const Transform<R>& to = a_is_hull ? *c.ta : *c.tb;
    const Transform<R>& tc = a_is_hull ? *c.tb : *c.ta;
    const R margin = c.margin;
    c.res->swap = a_is_hull;
    const R cr = cyl.radius, ch = cyl.height / R(2.0);
    const Transform<R> rel = to.inverse() * tc;
    const V3<R> axis = rel.basis.col(1);
    const V3<R> pos = rel.origin;
    std::vector<int> hit;
    {
        V3<R> AA, BB;
        get_aabb(cyl, rel, AA, BB);
        bvh_search(mesh, AA, BB, hit);
    }
    static const int dx[4] = {1, -1, -1, 1};
    static const int dy[4] = {1, 1, -1, -1};
    auto seg_on_mesh = [&](const Face<R>& f, const V3<R>& ps, const V3<R>& ds, R ls) {
        R t1, t2, d1, d2;
        if (segment_face(f, mesh, ps, ds, ls, margin, t1, t2, d1, d2)) {
            const V3<R> p1 = to.apply(ps + ds * t1 - f.normal * d1);
            const V3<R> p2 = to.apply(ps + ds * t2 - f.normal * d2);
            const V3<R> n = mv(to.basis, f.normal);
            c.add(n, p1 - n * margin, d1 + margin * 2);
            c.add(n, p2 - n * margin, d2 + margin * 2);
        }
    };
    for (int fi : hit) {
        const Face<R>& f = mesh.faces[fi];
        const R adc = dot(axis, f.normal);
        V3<R> ddx, ddy = axis, ddz;
        bool vertical = false;
        if (std::abs(std::abs(adc) - 1) < kEps<R>()) {
            ddz = normalized(cross(axis, V3<R>(1, 0, 0)));
            ddx = normalized(cross(axis, ddz));
            vertical = true;
        } else {
            ddx = normalized(cross(cross(f.normal, axis), axis));
        }
        for (int i = 0; i < 4; i++) {
            const V3<R> ps = pos + ddx * R(dx[i]) * cr + ddy * R(dy[i]) * ch;
            const V3<R> ds = (dx[i] == dy[i] ? ddy : ddx) * R(-dx[i]);
            const R ls = (dx[i] == dy[i] ? ch : cr) * 2;
            seg_on_mesh(f, ps, ds, ls);
        }
        if (vertical) {
            for (int i = 0; i < 3; i += 2) {
                const V3<R> ps = pos + ddz * R(dx[i]) * cr + ddy * R(dy[i]) * ch;
                const V3<R> ds = ddy * R(-dx[i]);
                const R ls = ch * 2;
                seg_on_mesh(f, ps, ds, ls);
            }
        }
    }
    for (int fi : hit) {
        const Face<R>& f = mesh.faces[fi];
        const int n = (int)f.idx.size();
        for (int i = 0; i < n; i++) {
            const V3<R>& v1 = mesh.verts[f.idx[i]];
            const V3<R>& v2 = mesh.verts[f.idx[(i + 1) % n]];
            R t1, t2;
            const V3<R> start = (v1 + v2) / R(2);
            const R ls = norm(v2 - v1) / 2;
            const V3<R> dir = (v2 - v1) / (ls * 2);
            if (segment_cylinder(start, dir, ls, pos, axis, ch, cr, margin, t1, t2)) {
                const V3<R> p1 = start + dir * t1;
                const V3<R> p2 = start + dir * t2;
                const V3<R> pm = (p1 + p2) / R(2);
                add_on_cylinder(c, pm, pos, axis, cr, ch, to, margin);
            }
        }
    }
    c.res->swap = false;
    return true;
}

// narrow_phase_base.cpp:20-29 dispatch restricted to box/sphere/cylinder/convex-mesh
template <class R> bool collide(PairCtx<R>& c);

// ConcaveConvexCollisionAlgorithm (concave_convex_collision_algorithm.cpp:8-67), for a box or a
// convex mesh against a concave mesh (ConcaveBoxCollisionAlgorithm routes boxes here too): the
// convex shape's box in the concave mesh's frame selects faces through the face tree; each face
// becomes a one-face convex shape (its vertices in face order, its normal, no unique edges and no
// face tree: setMesh is never called on it) run through the convex-convex algorithm with the
// convex shape first, at the concave body's transform.
template <class R> bool concave_convex(PairCtx<R>& c) {
    const bool a_concave = c.sa->type == ST_CONCAVE;
    const Shape<R>& cc = a_concave ? *c.sa : *c.sb;
    const Shape<R>* cv = a_concave ? c.sb : c.sa;
    const Transform<R>* tcc = a_concave ? c.ta : c.tb;
    const Transform<R>* tcv = a_concave ? c.tb : c.ta;
    c.res->swap = a_concave;
    V3<R> AA, BB;
    get_aabb(*cv, tcc->inverse() * *tcv, AA, BB);
    std::vector<int> hit;
    bvh_search(cc, AA, BB, hit);
    for (int fi : hit) {
        const Face<R>& f = cc.faces[fi];
        Shape<R> face;
        face.type = ST_HULL;
        Face<R> ff;
        for (size_t k = 0; k < f.idx.size(); k++) {
            face.verts.push_back(cc.verts[f.idx[k]]);
            ff.idx.push_back((int)k);
        }
        ff.normal = f.normal;
        face.faces.push_back(ff);
        PairCtx<R> s = c;
        s.sa = cv; s.sb = &face; s.ta = tcv; s.tb = tcc;
        convex_convex(s);
    }
    c.res->swap = false;
    return true;
}

// CompoundCompoundCollisionAlgorithm::processCollision (compound_compound_collision_algorithm.cpp:8-37):
// the compound goes first (a compound second swaps shapes, transforms and the result's objects,
// so the result then names the compound as object A); every child (against every child of a
// second compound) runs the algorithm of its shape pair into the same result, at the child's
// world transform (body transform * local transform, :23-29), with the pair's reference scale.
template <class R> bool compound_collide(PairCtx<R>& c) {
    if (c.sb->type == ST_COMPOUND) {
        std::swap(c.sa, c.sb);
        std::swap(c.ta, c.tb);
        std::swap(c.A, c.B);
        std::swap(c.res->a, c.res->b);
    }
    if (c.sa->type != ST_COMPOUND) return false;
    bool hit = false;
    auto sub = [&](const Shape<R>* sa, const Shape<R>* sb, const Transform<R>* ta, const Transform<R>* tb) {   // :39-46
        PairCtx<R> s = c;
        s.sa = sa; s.sb = sb; s.ta = ta; s.tb = tb;
        return collide(s);
    };
    for (auto& ch : c.sa->children) {
        const Transform<R> taw = (*c.ta) * ch.local;
        if (c.sb->type == ST_COMPOUND) {
            for (auto& chb : c.sb->children) {
                const Transform<R> tbw = (*c.tb) * chb.local;
                hit |= sub(ch.s, chb.s, &taw, &tbw);
            }
        } else {
            hit |= sub(ch.s, c.sb, &taw, c.tb);
        }
    }
    return hit;
}

template <class R> bool collide(PairCtx<R>& c) {
    const int ta = c.sa->type, tb = c.sb->type;
    if (ta == ST_COMPOUND || tb == ST_COMPOUND) return compound_collide(c);
    if (ta == ST_CONCAVE || tb == ST_CONCAVE) {   // narrow_phase_base.cpp:20-29, row and column 4
        const int o = ta == ST_CONCAVE ? tb : ta;
        if (o == ST_SPHERE) return sphere_hull(c);
        if (o == ST_CYLINDER) return cylinder_hull(c);
        if (o == ST_BOX || o == ST_HULL) return concave_convex(c);
        return false;   // concave-concave: no algorithm
    }
    auto is = [&](int x, int y) { return (ta == x && tb == y) || (ta == y && tb == x); };
    if (ta == ST_BOX && tb == ST_BOX) return box_box(c);
    if (is(ST_BOX, ST_SPHERE)) return box_sphere(c);
    if (is(ST_BOX, ST_CYLINDER)) return box_cylinder(c);
    if (is(ST_BOX, ST_HULL)) return convex_convex(c);
    if (ta == ST_SPHERE && tb == ST_SPHERE) return sphere_sphere(c);
    if (is(ST_SPHERE, ST_CYLINDER)) return sphere_cylinder(c);
    if (is(ST_SPHERE, ST_HULL)) return sphere_hull(c);
    if (ta == ST_CYLINDER && tb == ST_CYLINDER) return convex_convex(c);
    if (is(ST_CYLINDER, ST_HULL)) return cylinder_hull(c);
    if (ta == ST_HULL && tb == ST_HULL) return convex_convex(c);
    return false;
}

} // namespace orc
