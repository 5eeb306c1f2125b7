// Collision shapes on the device: box, sphere, cylinder and convex mesh ("hull").
//
// Box and cylinder meshes are not stored per shape: they are the reference's unit meshes
// (src/rigid/shape/default_mesh.h) scaled on the fly exactly as BoxShape / CylinderShape
// scale them at construction (box_shape.cpp:7-25, cylinder_shape.cpp:6-32).  The unit
// tables live in constant memory (filled by the host at world creation).  Hull meshes are
// preprocessed on the host (mass properties, recentring, face-tree face order, unique
// edges: convex_mesh_shape.cpp:12-131) and stored in flat device arrays.
#pragma once
#include "pe_math.cuh"

namespace pe {

enum ShapeType { ST_BOX = 0, ST_SPHERE = 1, ST_CYLINDER = 2, ST_HULL = 3, ST_CONCAVE = 4, ST_COMPOUND = 5 };

// unit meshes (host builds them; device reads them from constant memory)
constexpr int kBoxV = 24, kBoxF = 6, kBoxE = 12;
constexpr int kCylV = 80, kCylF = 42, kCylE = 80, kCylFIdx = 20 + 20 + 40 * 3;
struct UnitMeshes {
    double box_v[kBoxV][3];
    double box_n[kBoxF][3];
    double box_e[kBoxE][6];
    double cyl_v[kCylV][3];
    double cyl_n[kCylF][3];
    int cyl_foff[kCylF + 1];
    int cyl_fidx[kCylFIdx];
    int cyl_e[kCylE][2];   // unique edges as vertex index pairs
};

#ifdef __CUDACC__
// one copy per translation unit; each world implementation uploads its own at creation
static __constant__ UnitMeshes g_unit;
#endif

// device view of one shape
template <class R> struct ShapeView {
    int type;
    V3<R> size, half;          // box
    R radius, height, r2;      // sphere / cylinder (r2 = radius * 2)
    // hull arrays (valid when type == ST_HULL)
    const R* hv;               // local vertices [nv*3]
    int nv;
    const int* f_off;          // [nf+1] offsets into f_idx (already based at this hull)
    const int* f_idx;          // vertex indices local to this hull
    const R* f_n;              // face normals [nf*3]
    const R* f_min;            // per-face bounding boxes [nf*3]
    const R* f_max;
    int nf;
    const R* e_a;              // unique edge endpoints [ne*3]
    const R* e_b;
    const R* e_d;              // unit edge directions normalized(e_a - e_b), computed once per hull
    int ne;
    R inner, outer;            // hulls: balls about the local origin inside / around the vertices (inner < 0: none)
    // concave meshes: the face tree's leaves in tree order, each a face range and its box
    // (nl == 0 for convex meshes, whose leaves hold one face each)
    int nl;
    const int* l_beg;
    const int* l_cnt;
    const R* l_min;            // [nl*3]
    const R* l_max;

#ifdef __CUDACC__
    __device__ int face_count() const { return type == ST_BOX ? kBoxF : (type == ST_CYLINDER ? kCylF : nf); }
    __device__ int edge_count() const { return type == ST_BOX ? kBoxE : (type == ST_CYLINDER ? kCylE : ne); }
    __device__ int vert_count() const { return type == ST_BOX ? kBoxV : (type == ST_CYLINDER ? kCylV : nv); }
    __device__ V3<R> vert(int i) const {
        if (type == ST_BOX) return cmul(V3<R>(R(g_unit.box_v[i][0]), R(g_unit.box_v[i][1]), R(g_unit.box_v[i][2])), size);
        if (type == ST_CYLINDER)
            return V3<R>(R(g_unit.cyl_v[i][0]) * r2, R(g_unit.cyl_v[i][1]) * height, R(g_unit.cyl_v[i][2]) * r2);
        return V3<R>(hv[i * 3], hv[i * 3 + 1], hv[i * 3 + 2]);
    }
    __device__ int face_size(int f) const {
        if (type == ST_BOX) return 4;
        if (type == ST_CYLINDER) return g_unit.cyl_foff[f + 1] - g_unit.cyl_foff[f];
        return f_off[f + 1] - f_off[f];
    }
    __device__ int face_vert(int f, int k) const {
        if (type == ST_BOX) return f * 4 + k;
        if (type == ST_CYLINDER) return g_unit.cyl_fidx[g_unit.cyl_foff[f] + k];
        return f_idx[f_off[f] + k];
    }
    __device__ V3<R> face_normal(int f) const {
        if (type == ST_BOX) return V3<R>(R(g_unit.box_n[f][0]), R(g_unit.box_n[f][1]), R(g_unit.box_n[f][2]));
        if (type == ST_CYLINDER) return V3<R>(R(g_unit.cyl_n[f][0]), R(g_unit.cyl_n[f][1]), R(g_unit.cyl_n[f][2]));
        return V3<R>(f_n[f * 3], f_n[f * 3 + 1], f_n[f * 3 + 2]);
    }
    // unit direction of hull edge e: normalized(a - b) of edge(e, a, b), as stored by k_hull_edge_dirs
    __device__ V3<R> edge_dir(int e) const { return V3<R>(e_d[e * 3], e_d[e * 3 + 1], e_d[e * 3 + 2]); }
    __device__ void edge(int e, V3<R>& a, V3<R>& b) const {
        if (type == ST_BOX) {
            a = cmul(V3<R>(R(g_unit.box_e[e][0]), R(g_unit.box_e[e][1]), R(g_unit.box_e[e][2])), size);
            b = cmul(V3<R>(R(g_unit.box_e[e][3]), R(g_unit.box_e[e][4]), R(g_unit.box_e[e][5])), size);
        } else if (type == ST_CYLINDER) {
            a = vert(g_unit.cyl_e[e][0]);
            b = vert(g_unit.cyl_e[e][1]);
        } else {
            a = V3<R>(e_a[e * 3], e_a[e * 3 + 1], e_a[e * 3 + 2]);
            b = V3<R>(e_b[e * 3], e_b[e * 3 + 1], e_b[e * 3 + 2]);
        }
    }
#endif
};

// device-side shape tables
template <class R> struct ShapeTable {
    const int* type;      // [S]
    const R* param;       // [S*3]  box: size; sphere: r; cylinder: r, h
    const int* hull;      // [S] hull index or -1
    const int* h_vbeg; const int* h_vcnt; const int* h_fbeg; const int* h_fcnt; const int* h_ebeg; const int* h_ecnt;
    const R* hv; const int* f_off; const int* f_idx; const R* f_n; const R* f_min; const R* f_max;
    const R* e_a; const R* e_b;
    const R* e_d;         // [E*3] unit directions of the hull edges (k_hull_edge_dirs)
    const R* h_rad;       // [H*2] per hull: inner and outer radius about the local origin
    // concave meshes (hull tables plus the face-tree leaves): leaves [h_lbeg[h], h_lbeg[h] + h_lcnt[h])
    const int* h_lbeg; const int* h_lcnt; const int* lf_beg; const int* lf_cnt; const R* lf_min; const R* lf_max;
    // compound shapes: children [c_beg[s], c_beg[s] + c_cnt[s]) of shape s, each a non-compound
    // shape c_shape[k] at local transform c_xf[12k..] (basis row-major, then origin), relocated by
    // CompoundShape::init()
    const int* c_beg; const int* c_cnt; const int* c_shape; const R* c_xf;
    // contact margin of every pair algorithm (PE_MARGIN, phys_general.h:45; 0 in the reference's build)
    R margin;

#ifdef __CUDACC__
    __device__ Xf<R> child_xf(int k) const {
        const R* x = c_xf + (size_t)k * 12;
        Xf<R> t;
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) t.b.m[r][c] = x[r * 3 + c];
        t.o = V3<R>(x[9], x[10], x[11]);
        return t;
    }
    __device__ ShapeView<R> view(int s) const {
        ShapeView<R> v;
        v.type = type[s];
        const R p0 = param[s * 3], p1 = param[s * 3 + 1], p2 = param[s * 3 + 2];
        v.size = V3<R>(p0, p1, p2);
        v.half = v.size / R(2);
        v.radius = p0;
        v.height = p1;
        v.r2 = p0 * 2;
        v.hv = nullptr; v.nv = 0; v.f_off = nullptr; v.f_idx = nullptr; v.f_n = nullptr; v.f_min = nullptr; v.f_max = nullptr;
        v.nf = 0; v.e_a = nullptr; v.e_b = nullptr; v.e_d = nullptr; v.ne = 0;
        v.inner = R(-1); v.outer = R(0);
        v.nl = 0; v.l_beg = nullptr; v.l_cnt = nullptr; v.l_min = nullptr; v.l_max = nullptr;
        if (v.type == ST_HULL || v.type == ST_CONCAVE) {
            const int h = hull[s];
            const int vb = h_vbeg[h], fb = h_fbeg[h], eb = h_ebeg[h];
            v.hv = hv + vb * 3; v.nv = h_vcnt[h];
            v.inner = h_rad[2 * h]; v.outer = h_rad[2 * h + 1];
            v.f_off = f_off + fb; v.f_idx = f_idx; v.f_n = f_n + fb * 3; v.f_min = f_min + fb * 3; v.f_max = f_max + fb * 3;
            v.nf = h_fcnt[h];
            v.e_a = e_a + eb * 3; v.e_b = e_b + eb * 3; v.e_d = e_d + eb * 3; v.ne = h_ecnt[h];
            if (v.type == ST_CONCAVE) {
                const int lb = h_lbeg[h];
                v.nl = h_lcnt[h];
                v.l_beg = lf_beg + lb; v.l_cnt = lf_cnt + lb; v.l_min = lf_min + lb * 3; v.l_max = lf_max + lb * 3;
            }
        }
        return v;
    }
#endif
};

#ifdef __CUDACC__
// Shape::getAABB (box_shape.cpp:27-43, sphere_shape.cpp:14-18, cylinder_shape.cpp:34-43,
// convex_mesh_shape.cpp:138-150)
template <class R> __device__ void shape_aabb(const ShapeView<R>& s, const Xf<R>& t, V3<R>& mn, V3<R>& mx) {
    const R MX = Lim<R>::max(), MN = Lim<R>::min();
    if (s.type == ST_SPHERE) {
        const V3<R> r(s.radius, s.radius, s.radius);
        mn = t.o - r; mx = t.o + r;
        return;
    }
    if (s.type == ST_CYLINDER) {
        const V3<R> a = t.b.col(1);
        V3<R> e = V3<R>(rabs(a.x), rabs(a.y), rabs(a.z)) * (s.height * R(0.5));
        e.y += s.radius * real_sqrt(a.x * a.x + a.z * a.z);
        e.x += s.radius * real_sqrt(a.y * a.y + a.z * a.z);
        e.z += s.radius * real_sqrt(a.x * a.x + a.y * a.y);
        mn = t.o - e; mx = t.o + e;
        return;
    }
    mn = V3<R>(MX, MX, MX);
    mx = V3<R>(MN, MN, MN);
    const int n = s.type == ST_BOX ? 8 : s.nv;
    for (int i = 0; i < n; i++) {
        V3<R> p;
        if (s.type == ST_BOX) p = V3<R>(i & 1 ? s.half.x : -s.half.x, i & 2 ? s.half.y : -s.half.y, i & 4 ? s.half.z : -s.half.z);
        else p = V3<R>(s.hv[i * 3], s.hv[i * 3 + 1], s.hv[i * 3 + 2]);
        const V3<R> v = mv(t.b, p);
        mn = V3<R>(mn.x < v.x ? mn.x : v.x, mn.y < v.y ? mn.y : v.y, mn.z < v.z ? mn.z : v.z);
        mx = V3<R>(mx.x > v.x ? mx.x : v.x, mx.y > v.y ? mx.y : v.y, mx.z > v.z ? mx.z : v.z);
    }
    mn = mn + t.o;
    mx = mx + t.o;
}

// CompoundShape::getAABB (compound_shape.cpp:49-58): the union (PE_VEC_MIN2 / PE_VEC_MAX2) of the
// children's boxes at body transform * local transform
template <class R> __device__ void compound_aabb(const ShapeTable<R>& S, int s, const Xf<R>& t, V3<R>& mn, V3<R>& mx) {
    const R MX = Lim<R>::max(), MN = Lim<R>::min();
    mn = V3<R>(MX, MX, MX);
    mx = V3<R>(MN, MN, MN);
    for (int k = S.c_beg[s], e = S.c_beg[s] + S.c_cnt[s]; k < e; k++) {
        V3<R> a, b;
        shape_aabb(S.view(S.c_shape[k]), t * S.child_xf(k), a, b);
        mn = V3<R>(mn.x < a.x ? mn.x : a.x, mn.y < a.y ? mn.y : a.y, mn.z < a.z ? mn.z : a.z);
        mx = V3<R>(mx.x > b.x ? mx.x : b.x, mx.y > b.y ? mx.y : b.y, mx.z > b.z ? mx.z : b.z);
    }
}

// Shape::localIsInside
template <class R> __device__ bool shape_inside(const ShapeView<R>& s, const V3<R>& p) {
    if (s.type == ST_BOX) return rabs(p.x) <= s.half.x && rabs(p.y) <= s.half.y && rabs(p.z) <= s.half.z;
    if (s.type == ST_SPHERE) return sqnorm(p) <= s.radius * s.radius;
    if (s.type == ST_CYLINDER)
        return p.y >= -s.height * R(0.5) && p.y <= s.height * R(0.5) && p.x * p.x + p.z * p.z <= s.radius * s.radius;
    for (int f = 0; f < s.nf; f++) {
        const V3<R> p0 = s.vert(s.f_idx[s.f_off[f]]);
        if (dot(s.face_normal(f), p - p0) >= 0) return false;
    }
    return true;
}

// Shape::project: support interval and witness points along a world axis
template <class R> __device__ void shape_project(const ShapeView<R>& s, const Xf<R>& t, const V3<R>& axis, R& mnp, R& mxp,
                                                 V3<R>& mnpt, V3<R>& mxpt) {
    if (s.type == ST_SPHERE) {   // sphere_shape.cpp:24-32
        const R off = dot(t.o, axis);
        mnp = off - s.radius; mxp = off + s.radius;
        mnpt = t.o - axis * s.radius; mxpt = t.o + axis * s.radius;
        return;
    }
    const V3<R> la = mtv(t.b, axis);
    const R off = dot(t.o, axis);
    if (s.type == ST_BOX) {   // box_shape.cpp:51-68
        const V3<R> ext(la.x > 0 ? s.half.x : -s.half.x, la.y > 0 ? s.half.y : -s.half.y, la.z > 0 ? s.half.z : -s.half.z);
        const R he = dot(ext, la);
        mnp = off - he; mxp = off + he;
        mnpt = t.apply(-ext); mxpt = t.apply(ext);
        return;
    }
    if (s.type == ST_CYLINDER) {   // cylinder_shape.cpp:50-79
        const R hh = s.height * R(0.5);
        if (rabs(la.x - 0) < eps<R>() && rabs(la.z - 0) < eps<R>()) {
            const V3<R> up = V3<R>(0, 1, 0) * hh;
            mnpt = t.apply(-up); mxpt = t.apply(up);
            mnp = off - hh; mxp = off + hh;
        } else if (rabs(la.y - 0) < eps<R>()) {
            const V3<R> r = la * s.radius;
            mnpt = t.apply(-r); mxpt = t.apply(r);
            mnp = off - s.radius; mxp = off + s.radius;
        } else {
            const R r = real_sqrt(la.x * la.x + la.z * la.z);
            const R x = s.radius * la.x / r, z = s.radius * la.z / r;
            const R y = hh * (la.y > 0 ? 1 : -1);
            const V3<R> ext(x, y, z);
            mnpt = t.apply(-ext); mxpt = t.apply(ext);
            const R el = dot(ext, la);
            mnp = off - el; mxp = off + el;
        }
        return;
    }
    // convex_mesh_shape.cpp:160-183: a new minimum never updates the maximum
    mnp = Lim<R>::max();
    mxp = Lim<R>::min();
    V3<R> a, b;
    for (int i = 0; i < s.nv; i++) {
        const V3<R> p(s.hv[i * 3], s.hv[i * 3 + 1], s.hv[i * 3 + 2]);
        const R v = dot(p, la);
        if (v < mnp) { mnp = v; a = p; }
        else if (v > mxp) { mxp = v; b = p; }
    }
    mnp += off;
    mxp += off;
    mnpt = t.apply(a);
    mxpt = t.apply(b);
}
#endif

} // namespace pe
