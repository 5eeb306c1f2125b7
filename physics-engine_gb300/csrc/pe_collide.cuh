// Narrowphase on the device: the 8-slot contact cache of a collision pair and the pair
// algorithms for box / sphere / cylinder / convex-mesh pairs.
//
// Semantics follow the reference exactly (src/rigid/collision/narrow_phase/contact_result.cpp,
// src/rigid/collision/collision_algorithm/*.cpp), including its quirks: the slot that a new
// point replaces, the stale distances carried by invalid slots of a pooled result, the
// "+y face uses half_extent.x" branch of box-sphere, the box-box edge-edge axis pair and the
// hull projection that never lets a new minimum become the maximum.  The contact margin is the
// world's (PE_MARGIN = 0 in the reference's build, phys_general.h:45).
#pragma once
#include "pe_shapes.cuh"

namespace pe {

constexpr int kSlots = 8;   // PE_CONTACT_CACHE_SIZE

// contact_result.cpp:8-31
template <class R> __device__ void ortho_units(V3<R> n, V3<R>& t1, V3<R>& t2) {
    n = normalized(n);
    if (rabs(n.z) > R(0.7071)) {
        const R a = n.y * n.y + n.z * n.z;
        const R k = R(1.0) / real_sqrt(a);
        t1 = V3<R>(0, -n.z * k, n.y * k);
        t2 = V3<R>(a * k, -n.x * t1.z, n.x * t1.y);
    } else {
        const R a = n.x * n.x + n.y * n.y;
        const R k = R(1.0) / real_sqrt(a);
        t1 = V3<R>(-n.y * k, n.x * k, 0);
        t2 = V3<R>(-n.z * t1.y, n.z * t1.x, a * k);
    }
}

// One collision pair's contact cache (ContactResult).  Tangents are not cached: they are a
// function of the stored normal and are produced when the result is written out.
template <class R> struct Cache {
    V3<R> pos[kSlots], nrm[kSlots], la[kSlots], lb[kSlots];
    R dist[kSlots];
    unsigned valid;     // bit k: slot k holds a point (world_pos.x below the sentinel)
    bool swap;
    // body data the cache needs
    Xf<R> ta, tb;
    R scale_a, scale_b;

    __device__ void add(const V3<R>& wn, const V3<R>& wp, R depth) {   // contact_result.cpp:88-141
        V3<R> pa = wp, pb = wp, n = wn, point = wp;
        if (swap) { n = -n; pb = wp + wn * depth; point = pb; }
        else pa = wp + wn * depth;
        const V3<R> lpa = ta.inv_apply(pa);
        const V3<R> lpb = tb.inv_apply(pb);
        R th = (scale_a < scale_b ? scale_a : scale_b) * R(0.02);
        th *= th;
        int near = -1;
        for (int i = 0; i < kSlots; i++) {
            if (!((valid >> i) & 1u)) continue;
            const V3<R> d = lb[i] - lpb;
            const R dd = dot(d, d);
            if (dd < th) { th = dd; near = i; }
        }
        int slot = -1;
        if (near >= 0) {
            if (!(depth < dist[near])) return;
            slot = near;
        } else {
            for (int i = 0; i < kSlots; i++) if (!((valid >> i) & 1u)) { slot = i; break; }
            if (slot < 0) {
                R mx = Lim<R>::min();
                for (int i = 0; i < kSlots; i++) if (dist[i] > mx) { mx = dist[i]; slot = i; }
                if (slot < 0) return;
            }
        }
        pos[slot] = point; nrm[slot] = n; la[slot] = lpa; lb[slot] = lpb; dist[slot] = depth;
        if ((double)point.x < (double)Lim<R>::max() + 0.1) valid |= 1u << slot;
        else valid &= ~(1u << slot);
    }
};

// One pair being collided: shapes and transforms held by value (registers); the contact cache
// (local memory, only touched by the thread that adds points) is reached through `c`.
template <class R> struct Pair {
    ShapeView<R> sa, sb;
    Xf<R> xa, xb;
    R ref_scale;
    R margin;       // the world's contact margin (ShapeTable::margin)
    Cache<R>* c;
    __device__ void add(const V3<R>& n, const V3<R>& p, R d) { c->add(n, p, d); }
    __device__ const Xf<R>& ta() const { return xa; }
    __device__ const Xf<R>& tb() const { return xb; }
};

// ======================================================================= box-box
template <class R> __device__ int rect_quad(const R h[2], R p[8], R ret[16]) {   // box_box_collision_algorithm.cpp:20-71
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
                R* nx = (i > 1) ? pq + 2 : q;
                if ((R(sign) * pq[dir] < h[dir]) ^ (R(sign) * nx[dir] < h[dir])) {
                    pr[1 - dir] = pq[1 - dir] + (nx[1 - dir] - pq[1 - dir]) / (nx[dir] - pq[dir]) * (R(sign) * h[dir] - pq[dir]);
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
    if (q != ret) for (int k = 0; k < nr * 2; k++) ret[k] = q[k];
    return nr;
}

__device__ inline float ratan2(float y, float x) { return atan2f(y, x); }
__device__ inline double ratan2(double y, double x) { return atan2(y, x); }

template <class R> __device__ void cull_points(int n, const R p[], int m, int i0, int iret[]) {   // :73-135
    R a, cx, cy, q;
    if (n == 1) { cx = p[0]; cy = p[1]; }
    else if (n == 2) { cx = R(0.5) * (p[0] + p[2]); cy = R(0.5) * (p[1] + p[3]); }
    else {
        a = 0; cx = 0; cy = 0;
        for (int i = 0; i < n - 1; i++) {
            const R p0 = p[i * 2], p1 = p[i * 2 + 1], p2 = p[i * 2 + 2], p3 = p[i * 2 + 3];
            q = p0 * p3 - p2 * p1;
            a += q;
            cx += q * (p0 + p2);
            cy += q * (p1 + p3);
        }
        const R p0 = p[0], p1 = p[1], pm1 = p[n * 2 - 1], pm2 = p[n * 2 - 2];
        q = pm2 * p1 - p0 * pm1;
        if (rabs(a + q) > eps<R>()) a = R(1.0) / (R(3.0) * (a + q));
        else a = Lim<R>::max();
        cx = a * (cx + q * (pm2 + p0));
        cy = a * (cy + q * (pm1 + p1));
    }
    R A[8];
    int avail[8];
    for (int i = 0; i < n; i++) { A[i] = ratan2(p[i * 2 + 1] - cy, p[i * 2] - cx); avail[i] = 1; }
    avail[i0] = 0;
    iret[0] = i0;
    for (int j = 1; j < m; j++) {
        a = R(j) * (2 * pi<R>() / m) + A[i0];
        if (a > pi<R>()) a -= 2 * pi<R>();
        R maxd = Lim<R>::max();
        int pick = i0;
        for (int i = 0; i < n; i++) {
            if (avail[i]) {
                R diff = rabs(A[i] - a);
                if (diff > pi<R>()) diff = 2 * pi<R>() - diff;
                if (diff < maxd) { maxd = diff; pick = i; }
            }
        }
        iret[j] = pick;
        avail[pick] = 0;
    }
}

template <class R> __device__ bool box_box(Pair<R>& c) {   // box_box_collision_algorithm.cpp:137-580
    const R margin = c.margin, fudge = R(1.05);
    const V3<R> p1 = c.ta().o, p2 = c.tb().o;
    const M3<R>& R1 = c.ta().b;
    const M3<R>& R2 = c.tb().b;
    const V3<R> p = p2 - p1;
    const V3<R> pp = mtv(R1, p);
    const R A[3] = {c.sa.size.x * R(0.5), c.sa.size.y * R(0.5), c.sa.size.z * R(0.5)};
    const R B[3] = {c.sb.size.x * R(0.5), c.sb.size.y * R(0.5), c.sb.size.z * R(0.5)};
    const M3<R> Rij = mtm(R1, R2);
    R Q[3][3];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) Q[i][j] = rabs(Rij.m[i][j]);
    bool use_nR = false;
    V3<R> nC(0, 0, 0), nR;
    R s = Lim<R>::min(), s2, l;
    int inv = 0, code = 0;
    // face axes u1..u3, v1..v3
#define PE_TSTF(e1, e2, nrm, cc)                                                          \
    {                                                                                     \
        const R ee = (e1);                                                                \
        s2 = rabs(ee) - (e2);                                                             \
        if (s2 > 0) return false;                                                         \
        if (s2 > s) { s = s2; nR = (nrm); use_nR = true; inv = ee < 0; code = (cc); }     \
    }
    PE_TSTF(pp[0], A[0] + B[0] * Q[0][0] + B[1] * Q[0][1] + B[2] * Q[0][2], R1.col(0), 1)
    PE_TSTF(pp[1], A[1] + B[0] * Q[1][0] + B[1] * Q[1][1] + B[2] * Q[1][2], R1.col(1), 2)
    PE_TSTF(pp[2], A[2] + B[0] * Q[2][0] + B[1] * Q[2][1] + B[2] * Q[2][2], R1.col(2), 3)
    PE_TSTF(dot(R2.col(0), p), A[0] * Q[0][0] + A[1] * Q[1][0] + A[2] * Q[2][0] + B[0], R2.col(0), 4)
    PE_TSTF(dot(R2.col(1), p), A[0] * Q[0][1] + A[1] * Q[1][1] + A[2] * Q[2][1] + B[1], R2.col(1), 5)
    PE_TSTF(dot(R2.col(2), p), A[0] * Q[0][2] + A[1] * Q[1][2] + A[2] * Q[2][2] + B[2], R2.col(2), 6)
#undef PE_TSTF
#define PE_TSTE(e1, e2, n1, n2, n3, cc)                                                   \
    {                                                                                     \
        const R ee = (e1);                                                                \
        s2 = rabs(ee) - (e2);                                                             \
        if (s2 > eps<R>()) return false;                                                  \
        const R a1 = (n1), a2 = (n2), a3 = (n3);                                          \
        l = real_sqrt(a1 * a1 + a2 * a2 + a3 * a3);                                          \
        if (l > eps<R>()) {                                                               \
            s2 /= l;                                                                      \
            if (s2 * fudge > s) {                                                         \
                s = s2; use_nR = false; nC = V3<R>(a1 / l, a2 / l, a3 / l);               \
                inv = ee < 0; code = (cc);                                                \
            }                                                                             \
        }                                                                                 \
    }
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) Q[i][j] += eps<R>();
    const auto& Rm = Rij.m;
    PE_TSTE(pp[2] * Rm[1][0] - pp[1] * Rm[2][0], A[1] * Q[2][0] + A[2] * Q[1][0] + B[1] * Q[0][2] + B[2] * Q[0][1], R(0), -Rm[2][0], Rm[1][0], 7)
    PE_TSTE(pp[2] * Rm[1][1] - pp[1] * Rm[2][1], A[1] * Q[2][1] + A[2] * Q[1][1] + B[0] * Q[0][2] + B[2] * Q[0][0], R(0), -Rm[2][1], Rm[1][1], 8)
    PE_TSTE(pp[2] * Rm[1][2] - pp[1] * Rm[2][2], A[1] * Q[2][2] + A[2] * Q[1][2] + B[0] * Q[0][1] + B[1] * Q[0][0], R(0), -Rm[2][2], Rm[1][2], 9)
    PE_TSTE(pp[0] * Rm[2][0] - pp[2] * Rm[0][0], A[0] * Q[2][0] + A[2] * Q[0][0] + B[1] * Q[1][2] + B[2] * Q[1][1], Rm[2][0], R(0), -Rm[0][0], 10)
    PE_TSTE(pp[0] * Rm[2][1] - pp[2] * Rm[0][1], A[0] * Q[2][1] + A[2] * Q[0][1] + B[0] * Q[1][2] + B[2] * Q[1][0], Rm[2][1], R(0), -Rm[0][1], 11)
    PE_TSTE(pp[0] * Rm[2][2] - pp[2] * Rm[0][2], A[0] * Q[2][2] + A[2] * Q[0][2] + B[0] * Q[1][1] + B[1] * Q[1][0], Rm[2][2], R(0), -Rm[0][2], 12)
    PE_TSTE(pp[1] * Rm[0][0] - pp[0] * Rm[1][0], A[0] * Q[1][0] + A[1] * Q[0][0] + B[1] * Q[2][2] + B[2] * Q[2][1], -Rm[1][0], Rm[0][0], R(0), 13)
    PE_TSTE(pp[1] * Rm[0][1] - pp[0] * Rm[1][1], A[0] * Q[1][1] + A[1] * Q[0][1] + B[0] * Q[2][2] + B[2] * Q[2][0], -Rm[1][1], Rm[0][1], R(0), 14)
    PE_TSTE(pp[1] * Rm[0][2] - pp[0] * Rm[1][2], A[0] * Q[1][2] + A[1] * Q[0][2] + B[0] * Q[2][1] + B[1] * Q[2][0], -Rm[1][2], Rm[0][2], R(0), 15)
#undef PE_TSTE
    if (!code) return false;
    V3<R> normal = use_nR ? nR : mv(R1, nC);
    if (inv) normal = V3<R>(-normal.x, -normal.y, -normal.z);
    const R depth = -s;

    if (code > 6) {   // edge-edge
        V3<R> pa = p1;
        for (int j = 0; j < 3; j++) {
            const R sg = dot(normal, R1.col(j)) > 0 ? R(1.0) : R(-1.0);
            pa.x += sg * A[j] * R1.m[0][j]; pa.y += sg * A[j] * R1.m[1][j]; pa.z += sg * A[j] * R1.m[2][j];
        }
        V3<R> pb = p2;
        for (int j = 0; j < 3; j++) {
            const R sg = dot(normal, R2.col(j)) > 0 ? R(-1.0) : R(1.0);
            pb.x += sg * B[j] * R2.m[0][j]; pb.y += sg * B[j] * R2.m[1][j]; pb.z += sg * B[j] * R2.m[2][j];
        }
        const int qt = (code - 7) / 3;   // the reference takes both edge axes from this index
        const V3<R> ua = R1.col(qt), ub = R2.col(qt);
        const V3<R> ba = pb - pa;
        const R uab = dot(ua, ub), q1 = dot(ua, ba), q2 = -dot(ub, ba);
        R d = 1 - uab * uab, al, be;
        if (d <= eps<R>()) { al = 0; be = 0; }
        else { d = R(1.0) / d; al = (q1 + uab * q2) * d; be = (uab * q1 + q2) * d; }
        pa = V3<R>(pa.x + ua.x * al, pa.y + ua.y * al, pa.z + ua.z * al);
        pb = V3<R>(pb.x + ub.x * be, pb.y + ub.y * be, pb.z + ub.z * be);
        c.add(-normal, pb + normal * margin, -depth + margin * 2);
        return true;
    }
    // face-something: reference face on the box owning the axis
    M3<R> Ra, Rb;
    V3<R> pa, pb;
    R Sa[3], Sb[3];
    if (code <= 3) { c.c->swap = false; Ra = R1; Rb = R2; pa = p1; pb = p2; for (int k = 0; k < 3; k++) { Sa[k] = A[k]; Sb[k] = B[k]; } }
    else { c.c->swap = true; Ra = R2; Rb = R1; pa = p2; pb = p1; for (int k = 0; k < 3; k++) { Sa[k] = B[k]; Sb[k] = A[k]; } }
    const V3<R> n2 = code <= 3 ? normal : V3<R>(-normal.x, -normal.y, -normal.z);
    const V3<R> nr = mtv(Rb, n2);
    const V3<R> anr(rabs(nr.x), rabs(nr.y), rabs(nr.z));
    int lanr, a1, a2;
    if (anr[1] > anr[0]) {
        if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    } else {
        if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    }
    V3<R> ctr;
    const R sbl = Sb[lanr];
    if (nr[lanr] < 0) for (int k = 0; k < 3; k++) ctr[k] = pb[k] - pa[k] + sbl * Rb.m[k][lanr];
    else for (int k = 0; k < 3; k++) ctr[k] = pb[k] - pa[k] - sbl * Rb.m[k][lanr];
    const int codeN = code <= 3 ? code - 1 : code - 4;
    const int code1 = codeN == 0 ? 1 : 0, code2 = codeN == 2 ? 1 : 2;
    const R c1 = dot(ctr, Ra.col(code1)), c2 = dot(ctr, Ra.col(code2));
    R m11 = dot(Ra.col(code1), Rb.col(a1)), m12 = dot(Ra.col(code1), Rb.col(a2));
    R m21 = dot(Ra.col(code2), Rb.col(a1)), m22 = dot(Ra.col(code2), Rb.col(a2));
    R quad[8];
    {
        const R k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
        const R c1mk1 = c1 - k1, c2mk2 = c2 - k2, c1pk1 = c1 + k1, c2pk2 = c2 + k2;
        quad[0] = c1mk1 - k3; quad[1] = c2mk2 - k4; quad[2] = c1mk1 + k3; quad[3] = c2mk2 + k4;
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
        for (int k = 0; k < 3; k++) point[cnum * 3 + k] = ctr[k] + k1 * Rb.m[k][a1] + k2 * Rb.m[k][a2];
        dep[cnum] = Sa[codeN] - dot(n2, V3<R>(point[cnum * 3], point[cnum * 3 + 1], point[cnum * 3 + 2]));
        if (dep[cnum] >= 0) {
            ret[cnum * 2] = ret[j * 2];
            ret[cnum * 2 + 1] = ret[j * 2 + 1];
            cnum++;
        }
    }
    if (cnum < 1) return false;
    int maxc = cnum < 4 ? cnum : 4;
    if (maxc < 1) maxc = 1;
    const V3<R> mvv = normal * margin;
    auto emit = [&](int k) {
        const V3<R> w(point[k * 3] + pa.x, point[k * 3 + 1] + pa.y, point[k * 3 + 2] + pa.z);
        if (code < 4) c.add(-normal, w + mvv, -dep[k] + margin * 2);
        else c.add(normal, w - mvv, -dep[k] + margin * 2);
    };
    if (cnum <= maxc) {
        for (int j = 0; j < cnum; j++) emit(j);
    } else {
        int i1 = 0;
        R md = dep[0];
        for (int i = 1; i < cnum; i++) if (dep[i] > md) { md = dep[i]; i1 = i; }
        int iret[8];
        cull_points(cnum, ret, maxc, i1, iret);
        for (int j = 0; j < maxc; j++) emit(iret[j]);
    }
    return true;
}

// ======================================================================= sphere pairs
template <class R> __device__ bool box_sphere(Pair<R>& c) {   // box_sphere_collision_algorithm.cpp:6-141
    const bool a_box = c.sa.type == ST_BOX;
    const ShapeView<R>& sph = a_box ? c.sb : c.sa;
    const ShapeView<R>& box = a_box ? c.sa : c.sb;
    const Xf<R>& ts = a_box ? c.tb() : c.ta();
    const Xf<R>& tbx = a_box ? c.ta() : c.tb();
    const R radius = sph.radius, margin = c.margin;
    c.c->swap = a_box;
    bool ret = false;
    const V3<R> he = box.size / R(2.0);
    const V3<R> pos = tbx.inv_apply(ts.o);
    V3<R> cp = pos;
    cp.x = rmin(he.x, cp.x); cp.x = rmax(-he.x, cp.x);
    cp.y = rmin(he.y, cp.y); cp.y = rmax(-he.y, cp.y);
    cp.z = rmin(he.z, cp.z); cp.z = rmax(-he.z, cp.z);
    V3<R> normal = pos - cp;
    const R d2 = sqnorm(normal);
    if (!(d2 > radius * radius)) {
        R distance;
        if (d2 <= eps<R>() * eps<R>()) {
            // getSpherePenetration (:31-80)
            R fd = he.x - pos.x, md = fd;
            cp.x = he.x; normal = V3<R>(1, 0, 0);
            fd = he.x + pos.x; if (fd < md) { md = fd; cp = pos; cp.x = -he.x; normal = V3<R>(-1, 0, 0); }
            fd = he.y - pos.y; if (fd < md) { md = fd; cp = pos; cp.y = he.x; normal = V3<R>(0, 1, 0); }
            fd = he.y + pos.y; if (fd < md) { md = fd; cp = pos; cp.y = -he.y; normal = V3<R>(0, -1, 0); }
            fd = he.z - pos.z; if (fd < md) { md = fd; cp = pos; cp.z = he.z; normal = V3<R>(0, 0, 1); }
            fd = he.z + pos.z; if (fd < md) { md = fd; cp = pos; cp.z = -he.z; normal = V3<R>(0, 0, -1); }
            distance = -md;
        } else {
            distance = norm(normal);
            normal = normal / distance;
        }
        normal = mv(tbx.b, normal);
        const V3<R> pt = tbx.apply(cp);
        c.add(normal, pt - normal * margin, distance - radius + 2 * margin);
        ret = true;
    }
    c.c->swap = false;
    return ret;
}

template <class R> __device__ bool sphere_sphere(Pair<R>& c) {   // sphere_sphere_collision_algorithm.cpp:23-37
    const R ra = c.sa.radius, rb = c.sb.radius, margin = c.margin;
    const V3<R> rel = c.ta().o - c.tb().o;
    const R dist = norm(rel);
    if (dist > ra + rb || rabs(dist - 0) < eps<R>()) return false;
    const V3<R> n = rel / dist;
    const V3<R> ptb = c.tb().o + n * rb;
    c.add(n, ptb - n * margin, dist - ra - rb + 2 * margin);
    return true;
}

template <class R> __device__ bool sphere_cylinder(Pair<R>& c) {   // sphere_cylinder_collision_algorithm.cpp:6-76
    const bool a_sph = c.sa.type == ST_SPHERE;
    const ShapeView<R>& sph = a_sph ? c.sa : c.sb;
    const ShapeView<R>& cyl = a_sph ? c.sb : c.sa;
    const Xf<R>& ts = a_sph ? c.ta() : c.tb();
    const Xf<R>& tc = a_sph ? c.tb() : c.ta();
    const R margin = c.margin;
    c.c->swap = a_sph;
    bool ret = false;
    const R s_r = sph.radius, c_r = cyl.radius, c_h = cyl.height * R(0.5);
    const V3<R> s = tc.inv_apply(ts.o);
    const R r = real_sqrt(s.x * s.x + s.z * s.z);
    const R d = rabs(s.y) - c_h;
    if (!(s.y < -c_h - s_r || s.y > c_h + s_r || r * r > (c_r + s_r) * (c_r + s_r) ||
          (d > 0 && r > c_r && (r - c_r) * (r - c_r) + d * d > s_r * s_r))) {
        V3<R> n, pt;
        R depth;
        if (s.y >= -c_h && s.y <= c_h && r > 0) {
            n = normalized(V3<R>(-s.x, 0, -s.z));
            pt = n * s_r + s;
            depth = c_r + s_r - r;
        } else if (r <= c_r) {
            n = V3<R>(0, 1, 0);
            if (s.y > 0) n = -n;
            pt = s + n * s_r;
            depth = s_r + c_h - rabs(s.y);
        } else {
            V3<R> pc = normalized(V3<R>(s.x, 0, s.z)) * c_r;
            pc.y = s.y > 0 ? c_h : -c_h;
            n = normalized(pc - s);
            pt = n * s_r + s;
            depth = s_r - norm(s - pc);
        }
        n = mv(tc.b, n);
        pt = tc.apply(pt);
        c.add(n, pt - n * margin, -depth + 2 * margin);
        ret = true;
    }
    c.c->swap = false;
    return ret;
}

// ======================================================================= box-cylinder
template <class R> __device__ void add_on_box(Pair<R>& c, const V3<R>& pc, int face, const V3<R>& he, const Xf<R>& t, R margin) {
    if (!(face >= -3 && face <= 3 && face != 0)) return;   // box_cylinder_collision_algorithm.cpp:79-114
    for (int i = 0; i < 3; i++) if (pc[i] > he[i] || pc[i] < -he[i]) return;
    V3<R> p = pc, n(0, 0, 0);
    R pen;
    if (face > 0) { const int i = face - 1; p[i] = he[i]; n[i] = 1; pen = pc[i] - he[i]; }
    else { const int i = -face - 1; p[i] = -he[i]; n[i] = -1; pen = -pc[i] - he[i]; }
    const V3<R> nw = mv(t.b, n);
    const V3<R> pw = t.apply(p);
    c.add(nw, pw - nw * margin, pen + 2 * margin);
}

// the contact point addContactPointOnCylinder (:116-139) adds for a point p near the cylinder
template <class R> __device__ void cyl_contact(const V3<R>& p, const V3<R>& pos, const V3<R>& axis, R radius, R h, const Xf<R>& t,
                                               R margin, V3<R>& wn, V3<R>& wp, R& wd) {
    const V3<R> r = p - pos;
    const R dy = dot(r, axis);
    const R dxz = real_sqrt(sqnorm(r) - dy * dy);
    const R dside = radius - dxz, dtop = h - rabs(dy);
    V3<R> n;
    R dist;
    if (dside < dtop) { dist = dside; n = normalized(axis * dy - r); }
    else { dist = dtop; n = dy < 0 ? axis : -axis; }
    n = mv(t.b, n);
    const V3<R> pw = t.apply(p);
    wn = n;
    wp = pw - n * margin;
    wd = -dist + 2 * margin;
}
template <class R> __device__ void add_on_cylinder(Pair<R>& c, const V3<R>& p, const V3<R>& pos, const V3<R>& axis, R radius, R h,
                                                   const Xf<R>& t, R margin) {   // :116-139
    V3<R> n, pw;
    R d;
    cyl_contact(p, pos, axis, radius, h, t, margin, n, pw, d);
    c.add(n, pw, d);
}

template <class R> __device__ bool line_plane(const V3<R>& s, const V3<R>& d, const V3<R>& pp, const V3<R>& pn, R tol, R& t) {
    const R nd = dot(pn, d);
    if (rabs(nd) < tol) return false;
    t = dot(pn, pp - s) / nd;
    return true;
}

template <class R> __device__ bool segment_box(const V3<R>& he, const V3<R>& pos, const V3<R>& axis, R h, R tol, R& tmin, R& tmax) {
    tmin = Lim<R>::min();   // :171-231
    tmax = Lim<R>::max();
    for (int k = 0; k < 3; k++) {
        if (rabs(axis[k]) < tol) {
            if (rabs(pos[k]) > he[k]) return false;
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

template <class R> __device__ bool segment_cylinder(const V3<R>& s, const V3<R>& d, R len, const V3<R>& pos, const V3<R>& axis, R h,
                                                    R radius, R tol, R& tmin, R& tmax) {   // :233-304
    tmin = Lim<R>::min();
    tmax = Lim<R>::max();
    const V3<R> v = s - pos;
    const R cd_sd = dot(axis, d), v_cd = dot(v, axis), v_sd = dot(v, d), v_v = dot(v, v);
    const R a = R(1.0) - cd_sd * cd_sd;
    const R b = v_sd - v_cd * cd_sd;
    const R cc = v_v - v_cd * v_cd - radius * radius;
    if (rabs(a) < tol) {
        if (sqnorm(v - v_cd * axis) > radius * radius) return false;
        tmin = -len; tmax = +len;
    } else {
        R delta = b * b - a * cc;
        if (delta < 0) return false;
        delta = real_sqrt(delta);
        tmin = (-b - delta) / a;
        tmax = (-b + delta) / a;
    }
    R t1, t2;
    const bool k1 = line_plane(s, d, pos + h * axis, axis, tol, t1);
    const bool k2 = line_plane(s, d, pos - h * axis, axis, tol, t2);
    if (k1 && k2) {
        if (t1 < t2) { tmin = rmax(tmin, t1); tmax = rmin(tmax, t2); }
        else { tmin = rmax(tmin, t2); tmax = rmin(tmax, t1); }
        if (tmax < tmin) return false;
    } else {
        const R d1 = rabs(dot(axis, pos + h * axis - s));
        const R d2 = rabs(dot(axis, pos - h * axis - s));
        if (d1 > 2 * h || d2 > 2 * h) return false;
    }
    if ((tmin < -len && tmax < -len) || (tmin > +len && tmax > +len)) return false;
    tmin = rclamp(tmin, -len, +len);
    tmax = rclamp(tmax, -len, +len);
    return true;
}

template <class R> __device__ bool box_cylinder(Pair<R>& c) {   // box_cylinder_collision_algorithm.cpp:13-50, 306-389
    const bool a_box = c.sa.type == ST_BOX;
    const ShapeView<R>& box = a_box ? c.sa : c.sb;
    const ShapeView<R>& cyl = a_box ? c.sb : c.sa;
    const Xf<R>& tbx = a_box ? c.ta() : c.tb();
    const Xf<R>& tcy = a_box ? c.tb() : c.ta();
    const R cr = cyl.radius, ch = cyl.height / R(2.0), margin = c.margin;
    const V3<R> he = box.size / R(2.0);
    c.c->swap = a_box;
    const Xf<R> rel = tbx.inverse() * tcy;
    const V3<R> axis = rel.b.col(1), pos = rel.o;
    for (int i = 0; i < 3; i++) {
        V3<R> nd(0, 0, 0);
        nd[i] = 1;
        if (rabs(axis[i] - 1) < eps<R>() || rabs(axis[i] + 1) < eps<R>()) continue;
        const V3<R> r = normalized(cross(cross(nd, axis), axis)) * cr;
        for (int jj = 0; jj < 2; jj++) {
            const R jd = jj == 0 ? R(-1) : R(1);
            const V3<R> cs = pos + jd * r;
            R tmin, tmax;
            if (segment_box(he, cs, axis, ch, eps<R>(), tmin, tmax)) {
                const V3<R> pmin = cs + axis * tmin, pmax = cs + axis * tmax;
                const V3<R> pmid = cs + axis * ((tmin + tmax) / 2);
                int face = 0;
                R dist = Lim<R>::max();
                for (int k = 0; k < 3; k++) {   // findClosestBoxFace (:141-157)
                    const R pd = rabs(pmid[k] - he[k]), ndd = rabs(pmid[k] + he[k]);
                    if (pd < dist) { face = k + 1; dist = pd; }
                    if (ndd < dist) { face = -(k + 1); dist = ndd; }
                }
                add_on_box(c, pmin, face, he, tbx, margin);
                add_on_box(c, pmax, face, he, tbx, margin);
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
                if (segment_cylinder(ec, ed, eh, pos, axis, ch, cr, eps<R>(), tmin, tmax)) {
                    const V3<R> pmid = ec + ed * ((tmin + tmax) / 2);
                    add_on_cylinder(c, pmid, pos, axis, cr, ch, tbx, margin);
                }
            }
        }
    }
    c.c->swap = false;
    return true;
}

// ======================================================================= convex SAT + clipping
template <class R> __device__ bool sep_test(const Pair<R>& c, const V3<R>& axis, R& depth, V3<R>& wa, V3<R>& wb) {
    R min0, max0, min1, max1;   // convex_convex_collision_algorithm.cpp:216-243
    V3<R> a0, a1, b0, b1;
    shape_project(c.sa, c.ta(), axis, min0, max0, a0, a1);
    shape_project(c.sb, c.tb(), axis, min1, max1, b0, b1);
    if (max0 < min1 || max1 < min0) return false;
    const R d0 = max0 - min1, d1 = max1 - min0;
    if (d0 < d1) { depth = d0; wa = a1; wb = b0; }
    else { depth = d1; wa = a0; wb = b1; }
    return true;
}

template <class R> __device__ bool on_line(const V3<R>& v0, const V3<R>& v1, const V3<R>& v2) {
    return sqnorm(cross(v1 - v0, v2 - v0)) < eps<R>();
}

// findSeparatingAxis (:251-402), one thread
template <class R> __device__ bool find_sep_axis(Pair<R>& c, V3<R>& sep) {
    const R margin = c.margin;
    const V3<R> dc = c.ta().o - c.tb().o;
    R dmin = Lim<R>::max();
    V3<R> dpt;
    bool on_a = false;
    const int fa = c.sa.face_count(), fb = c.sb.face_count();
    for (int f = 0; f < fa + fb; f++) {
        const bool is_a = f < fa;
        V3<R> n = is_a ? mv(c.ta().b, c.sa.face_normal(f)) : mv(c.tb().b, c.sb.face_normal(f - fa));
        if (dot(dc, n) < 0) n = n * R(-1.0);
        R d;
        V3<R> wa, wb;
        if (!sep_test(c, n, d, wa, wb)) return false;
        if (d < dmin) { dmin = d; dpt = is_a ? wb : wa + n * d; on_a = !is_a; sep = n; }
    }
    if ((on_a && shape_inside(c.sb, c.tb().inv_apply(dpt))) || (!on_a && shape_inside(c.sa, c.ta().inv_apply(dpt))))
        c.add(sep, dpt - sep * margin, -dmin + margin * 2);
    int ea = -1, eb = -1;
    V3<R> wea, web, wpa(0, 0, 0), wpb(0, 0, 0);
    const int na = c.sa.edge_count(), nb = c.sb.edge_count();
    for (int e0 = 0; e0 < na; e0++) {
        V3<R> a0, a1;
        c.sa.edge(e0, a0, a1);
        const V3<R> w0 = mv(c.ta().b, normalized(a0 - a1));
        for (int e1 = 0; e1 < nb; e1++) {
            V3<R> b0, b1;
            c.sb.edge(e1, b0, b1);
            const V3<R> w1 = mv(c.tb().b, normalized(b0 - b1));
            V3<R> cr = cross(w0, w1);
            if (rabs(norm(cr) - 0) < eps<R>()) continue;
            cr = normalized(cr);
            if (dot(dc, cr) < 0) cr = cr * R(-1.0);
            R dist;
            V3<R> wa, wb;
            if (!sep_test(c, cr, dist, wa, wb)) return false;
            if (dist < dmin) {
                if (!on_line(a0, a1, c.ta().inv_apply(wa)) || !on_line(b0, b1, c.tb().inv_apply(wb))) continue;
                dmin = dist; sep = cr; ea = e0; eb = e1; wea = w0; web = w1; wpa = wa; wpb = wb;
            }
        }
    }
    if (ea >= 0 && eb >= 0) {   // segmentsClosestPoints with unbounded half-lengths (:172-214, :363-395)
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
    if (dot(dc, sep) < 0) sep = -sep;
    return true;
}

constexpr int kMaxClip = 64;   // clipped polygon capacity (incident face vertices + one per clip plane)

// clipFaceAgainstHull (:63-131): the incident face fb of B clipped against the side planes of
// the reference face fa of A; points whose depth under fa lies in [min_dist, max_dist] are kept
template <class R> __device__ void clip_faces(Pair<R>& c, const V3<R>& sep, R min_dist, R max_dist, int fb, int fa) {
    const R margin = c.margin;
    V3<R> buf[2][kMaxClip];
    int n_in = 0;
    const int nbv = c.sb.face_size(fb);
    for (int k = 0; k < nbv && n_in < kMaxClip; k++) buf[0][n_in++] = c.tb().apply(c.sb.vert(c.sb.face_vert(fb, k)));
    int cur = 0;
    const int nva = c.sa.face_size(fa);
    const V3<R> wpn = mv(c.ta().b, c.sa.face_normal(fa));
    for (int e0 = 0; e0 < nva; e0++) {
        const V3<R> a = c.sa.vert(c.sa.face_vert(fa, e0));
        const V3<R> b = c.sa.vert(c.sa.face_vert(fa, (e0 + 1) % nva));
        const V3<R> ew = mv(c.ta().b, a - b);
        const V3<R> pn = -cross(ew, wpn);
        const V3<R> wa = c.ta().apply(a);
        const R pe = -dot(wa, pn);
        // clipFace (:29-61)
        V3<R>* in = buf[cur];
        V3<R>* out = buf[cur ^ 1];
        int n_out = 0;
        if (n_in >= 2) {
            V3<R> first = in[n_in - 1];
            R ds = dot(pn, first) + pe;
            for (int ve = 0; ve < n_in; ve++) {
                const V3<R> end = in[ve];
                const R de = dot(pn, end) + pe;
                if (ds < 0) {
                    if (de < 0) { if (n_out < kMaxClip) out[n_out++] = end; }
                    else if (n_out < kMaxClip) out[n_out++] = first + (end - first) * R(ds * 1.f / (ds - de));
                } else if (de < 0) {
                    if (n_out < kMaxClip) out[n_out++] = first + (end - first) * R(ds * 1.f / (ds - de));
                    if (n_out < kMaxClip) out[n_out++] = end;
                }
                first = end;
                ds = de;
            }
        }
        cur ^= 1;
        n_in = n_out;
    }
    const V3<R> pv = c.sa.vert(c.sa.face_vert(fa, 0));
    const V3<R> lpn = c.sa.face_normal(fa);
    for (int i = 0; i < n_in; i++) {
        const V3<R> v = buf[cur][i];
        const R depth = dot(lpn, c.ta().inv_apply(v) - pv);
        if (depth <= max_dist && depth >= min_dist) c.add(sep, v - sep * margin, depth + margin * 2);
    }
}

// clipHullAgainstHull (:133-170): incident face = first maximum of n_B.sep, reference face =
// first minimum of n_A.sep
template <class R> __device__ void clip_hull_hull(Pair<R>& c, const V3<R>& sep, R min_dist, R max_dist) {
    int fb = -1;
    {
        R dmax = Lim<R>::min();
        for (int f = 0; f < c.sb.face_count(); f++) {
            const R d = dot(mv(c.tb().b, c.sb.face_normal(f)), sep);
            if (d > dmax) { dmax = d; fb = f; }
        }
    }
    if (fb < 0) return;
    int fa = -1;
    {
        R dmin = Lim<R>::max();
        for (int f = 0; f < c.sa.face_count(); f++) {
            const R d = dot(mv(c.ta().b, c.sa.face_normal(f)), sep);
            if (d < dmin) { dmin = d; fa = f; }
        }
    }
    if (fa < 0) return;
    clip_faces(c, sep, min_dist, max_dist, fb, fa);
}

template <class R> __device__ bool convex_convex(Pair<R>& c) {   // :408-432
    V3<R> sep;
    if (!find_sep_axis(c, sep)) return false;
    clip_hull_hull(c, sep, -c.ref_scale, c.margin);   // window [-refScale, margin] (:426-429)
    return true;
}

// ======================================================================= sphere-hull
template <class R> __device__ R seg_sqr_dist(const V3<R>& from, const V3<R>& to, const V3<R>& p, V3<R>& nearest) {
    V3<R> diff = p - from;   // sphere_convex_collision_algorithm.cpp:36-57
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

template <class R> __device__ bool sphere_triangle(const V3<R>& ctr, R radius, const V3<R>* vs, V3<R>& point, V3<R>& rn, R& depth) {
    V3<R> n = cross(vs[1] - vs[0], vs[2] - vs[0]);   // :91-163
    const R l2 = sqnorm(n);
    bool has = false;
    V3<R> cp;
    if (l2 >= eps<R>() * eps<R>()) {
        n = n / real_sqrt(l2);
        R dfp = dot(ctr - vs[0], n);
        if (dfp < 0) { dfp *= R(-1.); n = n * R(-1.); }
        if (dfp < radius) {
            const V3<R> e1 = vs[1] - vs[0], e2 = vs[2] - vs[1], e3 = vs[0] - vs[2];
            const R r1 = dot(cross(e1, n), ctr - vs[0]), r2 = dot(cross(e2, n), ctr - vs[1]), r3 = dot(cross(e3, n), ctr - vs[2]);
            if ((r1 > 0 && r2 > 0 && r3 > 0) || (r1 <= 0 && r2 <= 0 && r3 <= 0)) { has = true; cp = ctr - n * dfp; }
            else {
                R md = radius * radius;
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
        if (ds < radius * radius) {
            if (ds > eps<R>() * eps<R>()) { rn = normalized(cc); point = cp; depth = -(radius - real_sqrt(ds)); }
            else { rn = n; point = cp; depth = -radius; }
            return true;
        }
    }
    return false;
}

// faces of a hull whose bounding box meets [aa, bb], in the order the reference's face tree
// yields them (single-face leaves, right child first: descending face index)
template <class R> __device__ bool face_hit(const ShapeView<R>& m, int f, const V3<R>& aa, const V3<R>& bb) {
    const R* mn = m.f_min + f * 3;
    const R* mx = m.f_max + f * 3;
    if (mn[0] > bb.x || mn[1] > bb.y || mn[2] > bb.z) return false;
    if (mx[0] < aa.x || mx[1] < aa.y || mx[2] < aa.z) return false;
    return true;
}

// BVH::search (bvh.cpp:105-125) of a mesh's face tree for the box [aa, bb]: the right-first stack
// walk of a tree built on index ranges meets the leaves in descending order and reports every face
// of a leaf whose box overlaps, ascending.  Convex meshes (one face per leaf) test the face boxes.
template <class R, class Visit>
__device__ void mesh_query(const ShapeView<R>& m, const V3<R>& aa, const V3<R>& bb, Visit&& visit) {
    if (m.nl == 0) {
        for (int f = m.nf - 1; f >= 0; f--)
            if (face_hit(m, f, aa, bb)) visit(f);
        return;
    }
    for (int l = m.nl - 1; l >= 0; l--) {
        const R* mn = m.l_min + l * 3;
        const R* mx = m.l_max + l * 3;
        if (mn[0] > bb.x || mn[1] > bb.y || mn[2] > bb.z) continue;
        if (mx[0] < aa.x || mx[1] < aa.y || mx[2] < aa.z) continue;
        for (int f = m.l_beg[l], e = m.l_beg[l] + m.l_cnt[l]; f < e; f++) visit(f);
    }
}
__host__ __device__ inline bool is_mesh(int t) { return t == ST_HULL || t == ST_CONCAVE; }

template <class R> __device__ bool sphere_hull(Pair<R>& c) {   // sphere_convex_collision_algorithm.cpp:11-34, 165-211
    const bool a_hull = is_mesh(c.sa.type);
    const ShapeView<R>& m = a_hull ? c.sa : c.sb;
    const ShapeView<R>& sp = a_hull ? c.sb : c.sa;
    const Xf<R>& tm = a_hull ? c.ta() : c.tb();
    const Xf<R>& ts = a_hull ? c.tb() : c.ta();
    const R margin = c.margin;
    c.c->swap = a_hull;
    const V3<R> rel = tm.inv_apply(ts.o);
    const R r = sp.radius;
    const V3<R> aa = rel - V3<R>(r, r, r), bb = rel + V3<R>(r, r, r);
    bool ret = false;
    mesh_query(m, aa, bb, [&](int f) {
        const int n = m.face_size(f);
        for (int i = 0; i < n - 2; i++) {
            const V3<R> vs[3] = {m.vert(m.face_vert(f, 0)), m.vert(m.face_vert(f, i + 1)), m.vert(m.face_vert(f, i + 2))};
            V3<R> point, normal;
            R depth = 0;
            if (sphere_triangle(rel, r, vs, point, normal, depth)) {
                normal = mv(tm.b, normal);
                point = tm.apply(point);
                c.add(normal, point - normal * margin, depth + 2 * margin);
                ret = true;
            }
        }
    });
    c.c->swap = false;
    return ret;
}

// ======================================================================= cylinder-hull
template <class R> __device__ bool segment_face(const ShapeView<R>& m, int f, const V3<R>& ps, const V3<R>& ds, R ls, R margin,
                                                R& t1, R& t2, R& d1, R& d2) {   // cylinder_convex_collision_algorithm.cpp:53-107
    const V3<R> fn = m.face_normal(f);
    const V3<R> origin = m.vert(m.face_vert(f, 0));
    const V3<R> es = ps + ds * ls;
    const R dist1 = dot(ps - origin, fn), dist2 = dot(es - origin, fn);
    if ((dist1 > 0 && dist2 > 0) || (dist1 <= 0 && dist2 <= 0)) return false;
    const R t = dist1 / (dist1 - dist2) * ls;
    const V3<R> v = ps + ds * t;
    R tmin = 0, tmax = ls, mde = Lim<R>::max();
    const int n = m.face_size(f);
    for (int i = 0; i < n; i++) {
        const V3<R> v0 = m.vert(m.face_vert(f, i));
        const V3<R> v1 = m.vert(m.face_vert(f, (i + 1) % n));
        const V3<R> tc = normalized(cross(fn, v1 - v0));
        const R dd = dot(ds, tc);
        mde = rmin(mde, rabs(dot(v0 - v, tc)));
        if (!(rabs(dd - 0) < eps<R>())) {
            if (dd > 0) tmin = rmax(tmin, dot(v0 - ps, tc) / dd);
            else tmax = rmin(tmax, dot(v0 - ps, tc) / dd);
        } else if (dot(cross(v0 - v, v1 - v), fn) < 0) {
            return false;
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

template <class R> __device__ bool cylinder_hull(Pair<R>& c) {   // cylinder_convex_collision_algorithm.cpp:11-51, 109-203
    const bool a_hull = is_mesh(c.sa.type);
    const ShapeView<R>& m = a_hull ? c.sa : c.sb;
    const ShapeView<R>& cy = a_hull ? c.sb : c.sa;
    const Xf<R>& to = a_hull ? c.ta() : c.tb();
    const Xf<R>& tc = a_hull ? c.tb() : c.ta();
    const R margin = c.margin;
    c.c->swap = a_hull;
    const R cr = cy.radius, ch = cy.height / R(2.0);
    const Xf<R> rel = to.inverse() * tc;
    const V3<R> axis = rel.b.col(1), pos = rel.o;
    V3<R> aa, bb;
    shape_aabb(cy, rel, aa, bb);
    const int dxs[4] = {1, -1, -1, 1}, dys[4] = {1, 1, -1, -1};
    auto seg_on_mesh = [&](int f, const V3<R>& ps, const V3<R>& ds, R ls) {
        R t1, t2, d1, d2;
        if (segment_face(m, f, ps, ds, ls, margin, t1, t2, d1, d2)) {
            const V3<R> fn = m.face_normal(f);
            const V3<R> p1 = to.apply(ps + ds * t1 - fn * d1);
            const V3<R> p2 = to.apply(ps + ds * t2 - fn * d2);
            const V3<R> n = mv(to.b, fn);
            c.add(n, p1 - n * margin, d1 + margin * 2);
            c.add(n, p2 - n * margin, d2 + margin * 2);
        }
    };
    mesh_query(m, aa, bb, [&](int f) {
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
        for (int i = 0; i < 4; i++) {
            const V3<R> ps = pos + ddx * R(dxs[i]) * cr + ddy * R(dys[i]) * ch;
            const V3<R> ds = (dxs[i] == dys[i] ? ddy : ddx) * R(-dxs[i]);
            const R ls = (dxs[i] == dys[i] ? ch : cr) * 2;
            seg_on_mesh(f, ps, ds, ls);
        }
        if (vertical) {
            for (int i = 0; i < 3; i += 2) {
                const V3<R> ps = pos + ddz * R(dxs[i]) * cr + ddy * R(dys[i]) * ch;
                seg_on_mesh(f, ps, ddy * R(-dxs[i]), ch * 2);
            }
        }
    });
    mesh_query(m, aa, bb, [&](int f) {
        const int n = m.face_size(f);
        for (int i = 0; i < n; i++) {
            const V3<R> v1 = m.vert(m.face_vert(f, i));
            const V3<R> v2 = m.vert(m.face_vert(f, (i + 1) % n));
            R t1, t2;
            const V3<R> start = (v1 + v2) / R(2);
            const R ls = norm(v2 - v1) / 2;
            const V3<R> dir = (v2 - v1) / (ls * 2);
            if (segment_cylinder(start, dir, ls, pos, axis, ch, cr, margin, t1, t2)) {
                const V3<R> p1 = start + dir * t1, p2 = start + dir * t2;
                add_on_cylinder(c, (p1 + p2) / R(2), pos, axis, cr, ch, to, margin);
            }
        }
    });
    c.c->swap = false;
    return true;
}

// ======================================================================= concave meshes
// ConcaveConvexCollisionAlgorithm (concave_convex_collision_algorithm.cpp:8-67; boxes go the same
// way through ConcaveBoxCollisionAlgorithm): the convex shape's box in the concave mesh's frame
// selects faces through the face tree; each face becomes a one-face convex shape (its vertices in
// face order, its normal, no unique edges: setMesh is never called on it) that the convex-convex
// algorithm meets with the convex shape first, at the concave body's transform.
constexpr int kFaceVerts = 32;   // longest face polygon a concave mesh may hold (checked at upload)
template <class R> __device__ bool concave_convex(Pair<R>& c) {
    const bool a_cc = c.sa.type == ST_CONCAVE;
    const ShapeView<R>& cc = a_cc ? c.sa : c.sb;
    const ShapeView<R> cv = a_cc ? c.sb : c.sa;
    const Xf<R> tcc = a_cc ? c.xa : c.xb;
    const Xf<R> tcv = a_cc ? c.xb : c.xa;
    c.c->swap = a_cc;
    V3<R> aa, bb;
    shape_aabb(cv, tcc.inverse() * tcv, aa, bb);
    R fv[kFaceVerts * 3];
    int fidx[kFaceVerts];
    int foff[2];
    R fn[3], fmn[3], fmx[3];
    mesh_query(cc, aa, bb, [&](int f) {
        const int n = cc.face_size(f);
        foff[0] = 0;
        foff[1] = n;
        for (int k = 0; k < 3; k++) { fmn[k] = Lim<R>::max(); fmx[k] = Lim<R>::min(); }
        for (int i = 0; i < n; i++) {
            const V3<R> p = cc.vert(cc.face_vert(f, i));
            fv[i * 3] = p.x; fv[i * 3 + 1] = p.y; fv[i * 3 + 2] = p.z;
            fidx[i] = i;
            for (int k = 0; k < 3; k++) { fmn[k] = fmn[k] < p[k] ? fmn[k] : p[k]; fmx[k] = fmx[k] > p[k] ? fmx[k] : p[k]; }
        }
        const V3<R> nrm = cc.face_normal(f);
        fn[0] = nrm.x; fn[1] = nrm.y; fn[2] = nrm.z;
        ShapeView<R> face = cc;
        face.type = ST_HULL;
        face.hv = fv; face.nv = n;
        face.f_off = foff; face.f_idx = fidx; face.f_n = fn; face.f_min = fmn; face.f_max = fmx; face.nf = 1;
        face.e_a = nullptr; face.e_b = nullptr; face.e_d = nullptr; face.ne = 0;
        face.nl = 0;
        Pair<R> s = c;
        s.sa = cv; s.sb = face; s.xa = tcv; s.xb = tcc;
        convex_convex(s);
    });
    c.c->swap = false;
    return true;
}

// pair classes (narrow_phase_base.cpp:20-29 restricted to the four convex shape types)
// PC_CONVEX (cylinder-cylinder, box-hull, hull-hull, all run by ConvexConvexCollisionAlgorithm) is
// split for scheduling: by shape pairing for the warp-per-pair kernel (so that a launch runs one
// code path), PC_CONVEX_HEAVY pairs get a block of warps each, and PC_CONVEX_BIG (a shape beyond
// the shared-memory staging limits) the unstaged warp path.
enum PairClass { PC_BOX_BOX = 0, PC_BOX_SPHERE, PC_SPHERE_SPHERE, PC_SPHERE_CYL, PC_BOX_CYL, PC_CONVEX, PC_SPHERE_HULL,
                 PC_CYL_HULL, PC_CONVEX_HEAVY, PC_CONVEX_BIG, PC_CONVEX_HULL_HULL, PC_CONVEX_CYL_CYL, PC_CONVEX_HULL_BOX,
                 PC_COMPOUND, PC_CONCAVE, PC_COUNT };

__host__ __device__ inline int pair_class(int ta, int tb) {
    const int lo = ta < tb ? ta : tb, hi = ta < tb ? tb : ta;
    if (hi == ST_COMPOUND) return PC_COMPOUND;   // CompoundCompoundCollisionAlgorithm, either side
    if (lo == ST_CONCAVE || hi == ST_CONCAVE) return PC_CONCAVE;   // the Concave*CollisionAlgorithm family
    if (lo == ST_BOX && hi == ST_BOX) return PC_BOX_BOX;
    if (lo == ST_BOX && hi == ST_SPHERE) return PC_BOX_SPHERE;
    if (lo == ST_SPHERE && hi == ST_SPHERE) return PC_SPHERE_SPHERE;
    if (lo == ST_SPHERE && hi == ST_CYLINDER) return PC_SPHERE_CYL;
    if (lo == ST_BOX && hi == ST_CYLINDER) return PC_BOX_CYL;
    if (lo == ST_SPHERE && hi == ST_HULL) return PC_SPHERE_HULL;
    if (lo == ST_CYLINDER && hi == ST_HULL) return PC_CYL_HULL;
    return PC_CONVEX;   // cylinder-cylinder, box-hull, hull-hull
}

// a concave mesh against any convex shape (narrow_phase_base.cpp:20-29, row and column 4);
// concave-concave has no algorithm
template <class R> __device__ void concave_pair(Pair<R>& c) {
    const int o = c.sa.type == ST_CONCAVE ? c.sb.type : c.sa.type;
    if (o == ST_SPHERE) sphere_hull(c);
    else if (o == ST_CYLINDER) cylinder_hull(c);
    else if (o == ST_BOX || o == ST_HULL) concave_convex(c);
}

template <class R> __device__ void collide(Pair<R>& c, int cls) {
    switch (cls) {
        case PC_CONCAVE: concave_pair(c); break;
        case PC_BOX_BOX: box_box(c); break;
        case PC_BOX_SPHERE: box_sphere(c); break;
        case PC_SPHERE_SPHERE: sphere_sphere(c); break;
        case PC_SPHERE_CYL: sphere_cylinder(c); break;
        case PC_BOX_CYL: box_cylinder(c); break;
        case PC_SPHERE_HULL: sphere_hull(c); break;
        case PC_CYL_HULL: cylinder_hull(c); break;
        default: convex_convex(c); break;
    }
}

} // namespace pe
