// Host preprocessing of shapes (see pe_host.h).
#include <algorithm>
#include <array>
#include <map>
#include <cmath>
#include <utility>
#include "pe_host.h"
#include "pe_shapes.cuh"

namespace pe {

void build_unit_meshes(UnitMeshes& u) {
    // box: 6 quads with 4 private corners each; corner signs per face, face normals, 12 edges
    static const int corners[kBoxV][3] = {
        {-1, 1, -1}, {-1, 1, 1}, {1, 1, 1}, {1, 1, -1},      // +y
        {-1, -1, 1}, {-1, -1, -1}, {1, -1, -1}, {1, -1, 1},  // -y
        {-1, 1, 1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},      // +z
        {1, 1, -1}, {1, -1, -1}, {-1, -1, -1}, {-1, 1, -1},  // -z
        {-1, 1, -1}, {-1, -1, -1}, {-1, -1, 1}, {-1, 1, 1},  // -x
        {1, 1, 1}, {1, -1, 1}, {1, -1, -1}, {1, 1, -1}};     // +x
    static const int normals[kBoxF][3] = {{0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}, {-1, 0, 0}, {1, 0, 0}};
    static const int edges[kBoxE][6] = {
        {-1, 1, 1, 1, 1, 1}, {-1, -1, 1, 1, -1, 1}, {-1, -1, -1, 1, -1, -1}, {-1, 1, -1, 1, 1, -1},
        {1, -1, 1, 1, 1, 1}, {-1, -1, 1, -1, 1, 1}, {-1, -1, -1, -1, 1, -1}, {1, -1, -1, 1, 1, -1},
        {1, 1, 1, 1, 1, -1}, {-1, 1, 1, -1, 1, -1}, {-1, -1, 1, -1, -1, -1}, {1, -1, 1, 1, -1, -1}};
    for (int i = 0; i < kBoxV; i++) for (int k = 0; k < 3; k++) u.box_v[i][k] = 0.5 * corners[i][k];
    for (int i = 0; i < kBoxF; i++) for (int k = 0; k < 3; k++) u.box_n[i][k] = (double)normals[i][k];
    for (int i = 0; i < kBoxE; i++) for (int k = 0; k < 6; k++) u.box_e[i][k] = 0.5 * edges[i][k];

    // cylinder: the reference lists 6-decimal coordinates of a 20-gon.  First-quadrant
    // magnitudes (cos of the angle) of the top ring (0,18,..,90 deg), of the bottom ring and of
    // the upper side normals (9,27,..,81 deg, the latter scaled by 0.98769), and of the lower
    // side normals (0,18,..,90 deg, scaled by 0.999981).
    static const double top[6] = {0.5, 0.475528, 0.404508, 0.293893, 0.154508, 0.0};
    static const double bot[5] = {0.493844, 0.445503, 0.353553, 0.226995, 0.078217};
    static const double up_n[5] = {0.987670, 0.890990, 0.707093, 0.453982, 0.156432};
    static const double lo_n[6] = {0.999981, 0.951038, 0.809002, 0.587774, 0.309011, 0.0};
    // point on a circle at quadrant q with first-quadrant (cos, sin) = (c, s), as (x, z) with
    // z = -sin of the full angle; a zero entry keeps the reference's literal +0
    auto place = [](int q, double c, double s, double& x, double& z) {
        auto neg = [](double v) { return v == 0.0 ? 0.0 : -v; };
        switch (q) {
            case 0: x = c; z = neg(s); break;
            case 1: x = neg(s); z = neg(c); break;
            case 2: x = neg(c); z = s; break;
            default: x = s; z = c; break;
        }
    };
    for (int k = 0; k < 20; k++) {
        double x, z;
        place(k / 5, top[k % 5], top[5 - k % 5], x, z);
        u.cyl_v[k][0] = x; u.cyl_v[k][1] = 0.5; u.cyl_v[k][2] = z;
        place(k / 5, bot[k % 5], bot[4 - k % 5], x, z);
        u.cyl_v[20 + k][0] = x; u.cyl_v[20 + k][1] = -0.5; u.cyl_v[20 + k][2] = z;
    }
    for (int k = 0; k < 40; k++) for (int d = 0; d < 3; d++) u.cyl_v[40 + k][d] = u.cyl_v[k][d];
    int off = 0, f = 0;
    u.cyl_foff[f] = off;
    for (int k = 0; k < 20; k++) u.cyl_fidx[off++] = k;                 // top cap
    u.cyl_n[f][0] = 0; u.cyl_n[f][1] = 1; u.cyl_n[f][2] = 0;
    u.cyl_foff[++f] = off;
    for (int k = 39; k >= 20; k--) u.cyl_fidx[off++] = k;               // bottom cap
    u.cyl_n[f][0] = 0; u.cyl_n[f][1] = -1; u.cyl_n[f][2] = 0;
    u.cyl_foff[++f] = off;
    for (int k = 0; k < 20; k++) {                                      // side triangles under the top ring
        u.cyl_fidx[off++] = 60 + k; u.cyl_fidx[off++] = 40 + (k + 1) % 20; u.cyl_fidx[off++] = 40 + k;
        double x, z;
        place(k / 5, up_n[k % 5], up_n[4 - k % 5], x, z);
        if (k == 6) x = -0.493982;   // the reference's table holds this value for that face
        u.cyl_n[f][0] = x; u.cyl_n[f][1] = 0.006156; u.cyl_n[f][2] = z;
        u.cyl_foff[++f] = off;
    }
    for (int k = 0; k < 20; k++) {                                      // side triangles over the bottom ring
        u.cyl_fidx[off++] = 40 + k; u.cyl_fidx[off++] = 60 + (k + 19) % 20; u.cyl_fidx[off++] = 60 + k;
        double x, z;
        place(k / 5, lo_n[k % 5], lo_n[5 - k % 5], x, z);
        u.cyl_n[f][0] = x; u.cyl_n[f][1] = -0.006156; u.cyl_n[f][2] = z;
        u.cyl_foff[++f] = off;
    }
    // unique edges: top ring, bottom ring in cap winding, then the zig-zag between the rings
    int e = 0;
    for (int k = 0; k < 20; k++) { u.cyl_e[e][0] = k; u.cyl_e[e][1] = (k + 1) % 20; e++; }
    for (int j = 0; j < 20; j++) { u.cyl_e[e][0] = 39 - j; u.cyl_e[e][1] = j == 19 ? 39 : 38 - j; e++; }
    for (int k = 0; k < 20; k++) {
        u.cyl_e[e][0] = k; u.cyl_e[e][1] = 20 + k; e++;
        u.cyl_e[e][0] = 20 + k; u.cyl_e[e][1] = (k + 1) % 20; e++;
    }
}

template <class R> M3<R> box_inertia(const V3<R>& s) {
    const R x2 = s.x * s.x, y2 = s.y * s.y, z2 = s.z * s.z;
    M3<R> m;
    m.m[0][0] = (y2 + z2) / 12; m.m[1][1] = (x2 + z2) / 12; m.m[2][2] = (x2 + y2) / 12;
    return m;
}
template <class R> M3<R> sphere_inertia(R r) {
    const R i = R(2.0 / 5.0) * r * r;
    M3<R> m;
    m.m[0][0] = m.m[1][1] = m.m[2][2] = i;
    return m;
}
template <class R> M3<R> cylinder_inertia(R r, R h) {
    const R rr = r * r, hh = h * h;
    M3<R> m;
    m.m[0][0] = m.m[2][2] = rr / R(4.0) + hh / R(12.0);
    m.m[1][1] = rr * R(0.5);
    return m;
}

namespace {
template <class R> struct HFace { std::vector<int> idx; V3<R> n; };

// bvh.cpp:90-128: the face range is sorted in place by face centroid along the longest
// side of its bounding box, then split at the midpoint; leaves hold up to `leaf` faces.
template <class R> void face_tree(std::vector<HFace<R>>& faces, const std::vector<V3<R>>& v, int l, int r, int leaf) {
    if (l > r || r - l + 1 <= leaf) return;
    V3<R> aa(Lim<R>::max(), Lim<R>::max(), Lim<R>::max()), bb(Lim<R>::min(), Lim<R>::min(), Lim<R>::min());
    for (int i = l; i <= r; i++) {
        for (int k : faces[i].idx) {
            for (int d = 0; d < 3; d++) {
                if (v[k][d] < aa[d]) aa[d] = v[k][d];
                if (v[k][d] > bb[d]) bb[d] = v[k][d];
            }
        }
    }
    const R lx = bb.x - aa.x, ly = bb.y - aa.y, lz = bb.z - aa.z;
    const int axis = (lx >= ly && lx >= lz) ? 0 : (ly >= lz ? 1 : 2);
    auto centre = [&](const HFace<R>& f) {
        R s = 0;
        for (int k : f.idx) s += v[k][axis];
        s /= (R)f.idx.size();
        return s;
    };
    std::sort(faces.begin() + l, faces.begin() + r + 1, [&](const HFace<R>& a, const HFace<R>& b) { return centre(a) < centre(b); });
    const int mid = (l + r) / 2;
    face_tree(faces, v, l, mid, leaf);
    face_tree(faces, v, mid + 1, r, leaf);
}
} // namespace

// leaves of the face tree over [l, r] (the splits of face_tree), in tree order
static void tree_leaves(int l, int r, int leaf, std::vector<std::pair<int, int>>& out) {
    if (l > r) return;
    if (r - l + 1 <= leaf) { out.emplace_back(l, r); return; }
    const int mid = (l + r) / 2;
    tree_leaves(l, mid, leaf, out);
    tree_leaves(mid + 1, r, leaf, out);
}

// Radii of two balls about the hull's local origin, for the narrowphase's axis pruning: every
// vertex lies within `outer`, and the ball of radius `inner` lies inside the vertices' convex hull.
// `inner` is certified from the faces, in double precision on the stored coordinates: they must close
// a surface (every directed edge once, its reverse once), every face vertex must lie on or behind
// every face's plane (Newell normal; one global flip for inward windings), and the origin must lie
// strictly inside.  Then that surface bounds the hull of the face vertices, the smallest plane
// distance less each face's out-of-plane spread is a safe radius, and it is shrunk by 1e-6 of
// `outer`.  Otherwise `inner` is -1 and no axis of the hull is pruned.
template <class R> static void hull_radii(const std::vector<V3<R>>& v, const std::vector<HFace<R>>& faces, R& inner, R& outer) {
    double ro = 0;
    for (const auto& p : v) ro = std::max(ro, std::sqrt(double(p.x) * p.x + double(p.y) * p.y + double(p.z) * p.z));
    outer = R(ro * (1 + 1e-6));
    inner = R(-1);
    if (faces.empty() || ro == 0) return;
    std::map<std::pair<int, int>, int> dir;   // directed edge -> count
    std::vector<int> used;
    for (const auto& f : faces) {
        const int n = (int)f.idx.size();
        if (n < 3) return;
        for (int i = 0; i < n; i++) {
            dir[{f.idx[i], f.idx[(i + 1) % n]}]++;
            used.push_back(f.idx[i]);
        }
    }
    for (const auto& e : dir) {
        if (e.second != 1) return;
        auto back = dir.find({e.first.second, e.first.first});
        if (back == dir.end() || back->second != 1) return;
    }
    std::sort(used.begin(), used.end());
    used.erase(std::unique(used.begin(), used.end()), used.end());
    const double tol = 1e-9 * ro;
    const size_t F = faces.size();
    std::vector<double> nrm(F * 3), dmin(F), dmax(F);
    size_t pos = 0, neg = 0;
    for (size_t k = 0; k < F; k++) {
        const auto& f = faces[k];
        const int n = (int)f.idx.size();
        double nx = 0, ny = 0, nz = 0;
        for (int i = 0; i < n; i++) {   // Newell's method
            const V3<R>& a = v[f.idx[i]];
            const V3<R>& b = v[f.idx[(i + 1) % n]];
            nx += (double(a.y) - b.y) * (double(a.z) + b.z);
            ny += (double(a.z) - b.z) * (double(a.x) + b.x);
            nz += (double(a.x) - b.x) * (double(a.y) + b.y);
        }
        const double l = std::sqrt(nx * nx + ny * ny + nz * nz);
        if (!(l > 0)) return;
        nrm[3 * k] = nx / l; nrm[3 * k + 1] = ny / l; nrm[3 * k + 2] = nz / l;
        double lo = 1e300, hi = -1e300;
        for (int i = 0; i < n; i++) {
            const V3<R>& a = v[f.idx[i]];
            const double d = nrm[3 * k] * a.x + nrm[3 * k + 1] * a.y + nrm[3 * k + 2] * a.z;
            lo = std::min(lo, d); hi = std::max(hi, d);
        }
        dmin[k] = lo; dmax[k] = hi;
        if (lo > tol) pos++;
        else if (hi < -tol) neg++;
    }
    if (neg == F) {   // inward winding
        for (size_t k = 0; k < F; k++) {
            for (int d = 0; d < 3; d++) nrm[3 * k + d] = -nrm[3 * k + d];
            const double lo = -dmax[k];
            dmax[k] = -dmin[k]; dmin[k] = lo;
        }
    } else if (pos != F) {
        return;
    }
    double r = 1e300;
    for (size_t k = 0; k < F; k++) {
        for (int i : used) {
            const V3<R>& a = v[i];
            if (nrm[3 * k] * a.x + nrm[3 * k + 1] * a.y + nrm[3 * k + 2] * a.z > dmax[k] + tol) return;
        }
        r = std::min(r, dmin[k] - (dmax[k] - dmin[k]));
    }
    // The projection loop never takes vertex 0 as the maximum (convex_mesh_shape.cpp:171-175), so the
    // radius must also hold for the hull of the other vertices.  Its facets are the faces without
    // vertex 0 and new ones whose corners are neighbours of vertex 0 (vertices of its faces) or
    // vertices on no face; every plane through three such candidates that supports the remaining
    // vertices is a facet plane or lies farther out, so the smallest of these distances is that
    // hull's radius.
    const int nv = (int)v.size();
    std::vector<char> cand(nv, 0), on_face(nv, 0);
    for (int i : used) on_face[i] = 1;
    for (size_t k = 0; k < F; k++) {
        const auto& f = faces[k];
        if (std::find(f.idx.begin(), f.idx.end(), 0) == f.idx.end()) continue;
        for (int i : f.idx) cand[i] = 1;
    }
    if (on_face[0]) {
        double r1 = 1e300;
        for (size_t k = 0; k < F; k++)
            if (std::find(faces[k].idx.begin(), faces[k].idx.end(), 0) == faces[k].idx.end())
                r1 = std::min(r1, dmin[k] - (dmax[k] - dmin[k]));
        std::vector<int> C;
        for (int i = 1; i < nv; i++)
            if (cand[i] || !on_face[i]) C.push_back(i);
        auto dv = [&](int i) { return std::array<double, 3>{double(v[i].x), double(v[i].y), double(v[i].z)}; };
        for (size_t a = 0; a < C.size(); a++)
            for (size_t b = a + 1; b < C.size(); b++)
                for (size_t c = b + 1; c < C.size(); c++) {
                    const auto p0 = dv(C[a]), p1 = dv(C[b]), p2 = dv(C[c]);
                    const double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                    const double w[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                    double n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
                    const double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                    if (!(l > 1e-12 * ro * ro)) continue;
                    for (double& x : n) x /= l;
                    const double d = n[0] * p0[0] + n[1] * p0[1] + n[2] * p0[2];
                    double lo = 1e300, hi = -1e300;
                    for (int i = 1; i < nv; i++) {
                        const auto q = dv(i);
                        const double e = n[0] * q[0] + n[1] * q[1] + n[2] * q[2];
                        lo = std::min(lo, e); hi = std::max(hi, e);
                    }
                    if (hi <= d + tol) r1 = std::min(r1, d);         // outward normal
                    else if (lo >= d - tol) r1 = std::min(r1, -d);   // inward normal
                }
        r = std::min(r, r1);
    }
    r -= 1e-6 * ro;
    if (r > 0) inner = R(r);
}

template <class R>
HullPrep<R> prepare_hull(const double* verts, int nv, const int* face_off, const int* face_idx, int nf, bool concave) {
    std::vector<V3<R>> v(nv);
    for (int i = 0; i < nv; i++) v[i] = V3<R>(R(verts[i * 3]), R(verts[i * 3 + 1]), R(verts[i * 3 + 2]));
    std::vector<HFace<R>> faces(nf);
    for (int f = 0; f < nf; f++) {
        for (int k = face_off[f]; k < face_off[f + 1]; k++) faces[f].idx.push_back(face_idx[k]);
        const V3<R>& p1 = v[faces[f].idx[0]];
        faces[f].n = normalized(cross(v[faces[f].idx[1]] - p1, v[faces[f].idx[2]] - p1));   // Mesh::perFaceNormal
    }
    if (concave) {
        // ConcaveMeshShape::setMesh (concave_mesh_shape.cpp:6-17): the mesh as given, unit inertia,
        // no volume, the face tree with leaves of max(faces / 2047, 1) faces, no unique edges
        HullPrep<R> h;
        h.inertia = M3<R>();
        for (int i = 0; i < 3; i++) h.inertia.m[i][i] = R(1);
        const int leaf = std::max(nf / 2047, 1);
        face_tree(faces, v, 0, nf - 1, leaf);
        for (auto& p : v) { h.v.push_back(p.x); h.v.push_back(p.y); h.v.push_back(p.z); }
        h.f_off.push_back(0);
        std::vector<V3<R>> fmn, fmx;
        for (const auto& f : faces) {
            V3<R> mn(Lim<R>::max(), Lim<R>::max(), Lim<R>::max()), mx(Lim<R>::min(), Lim<R>::min(), Lim<R>::min());
            for (int k : f.idx) {
                h.f_idx.push_back(k);
                for (int d = 0; d < 3; d++) {
                    if (v[k][d] < mn[d]) mn[d] = v[k][d];
                    if (v[k][d] > mx[d]) mx[d] = v[k][d];
                }
            }
            h.f_off.push_back((int)h.f_idx.size());
            for (int d = 0; d < 3; d++) { h.f_n.push_back(f.n[d]); h.f_min.push_back(mn[d]); h.f_max.push_back(mx[d]); }
            fmn.push_back(mn);
            fmx.push_back(mx);
        }
        std::vector<std::pair<int, int>> lv;
        tree_leaves(0, nf - 1, leaf, lv);
        for (auto& q : lv) {
            V3<R> mn(Lim<R>::max(), Lim<R>::max(), Lim<R>::max()), mx(Lim<R>::min(), Lim<R>::min(), Lim<R>::min());
            for (int f = q.first; f <= q.second; f++)
                for (int d = 0; d < 3; d++) {
                    if (fmn[f][d] < mn[d]) mn[d] = fmn[f][d];
                    if (fmx[f][d] > mx[d]) mx[d] = fmx[f][d];
                }
            h.l_beg.push_back(q.first);
            h.l_cnt.push_back(q.second - q.first + 1);
            for (int d = 0; d < 3; d++) { h.l_min.push_back(mn[d]); h.l_max.push_back(mx[d]); }
        }
        return h;
    }
    // polyhedral mass properties (convex_mesh_shape.cpp:29-100), integrals over fan triangles
    const R mult[10] = {R(1.0) / 6, R(1.0) / 24, R(1.0) / 24, R(1.0) / 24, R(1.0) / 60,
                        R(1.0) / 60, R(1.0) / 60, R(1.0) / 120, R(1.0) / 120, R(1.0) / 120};
    R in[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    auto terms = [](R w0, R w1, R w2, R& f1, R& f2, R& f3, R& g0, R& g1, R& g2) {
        const R t0 = w0 + w1;
        f1 = t0 + w2;
        const R t1 = w0 * w0;
        const R t2 = t1 + w1 * t0;
        f2 = t2 + w2 * f1;
        f3 = w0 * t1 + w1 * t2 + w2 * f2;
        g0 = f2 + w0 * (f1 + w0);
        g1 = f2 + w1 * (f1 + w1);
        g2 = f2 + w2 * (f1 + w2);
    };
    for (const auto& face : faces) {
        const V3<R>& a = v[face.idx[0]];
        for (int i = 0; i + 2 < (int)face.idx.size(); i++) {
            const V3<R>& b = v[face.idx[i + 1]];
            const V3<R>& c = v[face.idx[i + 2]];
            const R a1 = b.x - a.x, b1 = b.y - a.y, c1 = b.z - a.z, a2 = c.x - a.x, b2 = c.y - a.y, c2 = c.z - a.z;
            const R d0 = b1 * c2 - b2 * c1, d1 = a2 * c1 - a1 * c2, d2 = a1 * b2 - a2 * b1;
            R f1x, f2x, f3x, g0x, g1x, g2x, f1y, f2y, f3y, g0y, g1y, g2y, f1z, f2z, f3z, g0z, g1z, g2z;
            terms(a.x, b.x, c.x, f1x, f2x, f3x, g0x, g1x, g2x);
            terms(a.y, b.y, c.y, f1y, f2y, f3y, g0y, g1y, g2y);
            terms(a.z, b.z, c.z, f1z, f2z, f3z, g0z, g1z, g2z);
            in[0] += d0 * f1x;
            in[1] += d0 * f2x;
            in[2] += d1 * f2y;
            in[3] += d2 * f2z;
            in[4] += d0 * f3x;
            in[5] += d1 * f3y;
            in[6] += d2 * f3z;
            in[7] += d0 * (a.y * g0x + b.y * g1x + c.y * g2x);
            in[8] += d1 * (a.z * g0y + b.z * g1y + c.z * g2y);
            in[9] += d2 * (a.x * g0z + b.x * g1z + c.x * g2z);
        }
    }
    for (int i = 0; i < 10; i++) in[i] *= mult[i];
    HullPrep<R> h;
    h.volume = in[0];
    const V3<R> cm(in[1] / h.volume, in[2] / h.volume, in[3] / h.volume);
    M3<R>& I = h.inertia;
    I.m[0][0] = in[5] + in[6] - h.volume * (cm.y * cm.y + cm.z * cm.z);
    I.m[1][1] = in[4] + in[6] - h.volume * (cm.z * cm.z + cm.x * cm.x);
    I.m[2][2] = in[4] + in[5] - h.volume * (cm.x * cm.x + cm.y * cm.y);
    I.m[0][1] = I.m[1][0] = -in[7] + h.volume * cm.x * cm.y;
    I.m[1][2] = I.m[2][1] = -in[8] + h.volume * cm.y * cm.z;
    I.m[0][2] = I.m[2][0] = -in[9] + h.volume * cm.z * cm.x;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) I.m[i][j] /= h.volume;
    for (auto& p : v) p = p - cm;
    face_tree(faces, v, 0, nf - 1, std::max(nf / 8191, 1));
    // outputs
    for (auto& p : v) { h.v.push_back(p.x); h.v.push_back(p.y); h.v.push_back(p.z); }
    h.f_off.push_back(0);
    for (const auto& f : faces) {
        V3<R> mn(Lim<R>::max(), Lim<R>::max(), Lim<R>::max()), mx(Lim<R>::min(), Lim<R>::min(), Lim<R>::min());
        for (int k : f.idx) {
            h.f_idx.push_back(k);
            for (int d = 0; d < 3; d++) {
                if (v[k][d] < mn[d]) mn[d] = v[k][d];
                if (v[k][d] > mx[d]) mx[d] = v[k][d];
            }
        }
        h.f_off.push_back((int)h.f_idx.size());
        for (int d = 0; d < 3; d++) { h.f_n.push_back(f.n[d]); h.f_min.push_back(mn[d]); h.f_max.push_back(mx[d]); }
    }
    // unique edges in face order, first winding kept (convex_mesh_shape.cpp:111-128); vertices are
    // identified by position up to 1e-5 per coordinate, in first-seen order
    std::vector<int> canon(nv, -1);
    std::vector<int> reg;
    auto vid = [&](int k) {
        if (canon[k] >= 0) return canon[k];
        for (size_t i = 0; i < reg.size(); i++) {
            const V3<R>& q = v[reg[i]];
            if (std::fabs(double(q.x - v[k].x)) < 1e-5 && std::fabs(double(q.y - v[k].y)) < 1e-5 &&
                std::fabs(double(q.z - v[k].z)) < 1e-5)
                return canon[k] = (int)i;
        }
        reg.push_back(k);
        return canon[k] = (int)reg.size() - 1;
    };
    std::vector<std::pair<int, int>> seen;
    for (const auto& f : faces) {
        const int n = (int)f.idx.size();
        for (int i = 0; i < n; i++) {
            const int k0 = f.idx[i], k1 = f.idx[(i + 1) % n];
            int a = vid(k0), b = vid(k1);
            if (a > b) std::swap(a, b);
            if (std::find(seen.begin(), seen.end(), std::make_pair(a, b)) != seen.end()) continue;
            seen.emplace_back(a, b);
            for (int d = 0; d < 3; d++) { h.e_a.push_back(v[k0][d]); h.e_b.push_back(v[k1][d]); }
        }
    }
    hull_radii(v, faces, h.inner, h.outer);
    return h;
}

template M3<float> box_inertia<float>(const V3<float>&);
template M3<double> box_inertia<double>(const V3<double>&);
template M3<float> sphere_inertia<float>(float);
template M3<double> sphere_inertia<double>(double);
template M3<float> cylinder_inertia<float>(float, float);
template M3<double> cylinder_inertia<double>(double, double);
template HullPrep<float> prepare_hull<float>(const double*, int, const int*, const int*, int, bool);
template HullPrep<double> prepare_hull<double>(const double*, int, const int*, const int*, int, bool);

} // namespace pe
