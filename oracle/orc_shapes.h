// Oracle shapes: box, sphere, cylinder, convex mesh and compound, restating the reference's
// src/rigid/shape/{box,sphere,cylinder,convex_mesh,compound}_shape.cpp and the default meshes of
// src/rigid/shape/default_mesh.h.  Test infrastructure only.
#pragma once
#include <algorithm>
#include <stdexcept>
#include <vector>
#include "orc_math.h"

namespace orc {

enum ShapeType { ST_BOX = 0, ST_SPHERE = 1, ST_CYLINDER = 2, ST_HULL = 3, ST_CONCAVE = 4, ST_COMPOUND = 5 };

template <class R> struct Shape;
// one CompoundShape::ShapeEle (compound_shape.h:10-14); `s` points into the world's shape table
template <class R> struct Child {
    int shape = 0;
    Transform<R> local;
    R ratio = 0;
    const Shape<R>* s = nullptr;
};

template <class R> struct Face {
    std::vector<int> idx;
    V3<R> normal;
};

template <class R> struct Shape {
    int type = ST_BOX;
    V3<R> size, half;                       // box
    R radius = 0, height = 0;               // sphere / cylinder
    std::vector<V3<R>> verts;               // box / cylinder / hull mesh positions
    std::vector<Face<R>> faces;
    std::vector<V3<R>> edge_a, edge_b;      // unique edges
    M3<R> local_inertia;                    // unit mass
    R volume = 0;
    // hull bounding-volume tree (src/utils/bvh.cpp), flattened
    struct Node { int left = -1, right = -1, n = 0, index = 0; V3<R> aa, bb; };
    std::vector<Node> bvh;
    std::vector<Child<R>> children;         // compound
};

// ---------------------------------------------------------------- default meshes
// Unit box of default_mesh.h:7-57: 6 quads, 4 private vertices each, axis normals.
template <class R> void default_box_mesh(Shape<R>& s) {
    static const signed char vtx[24][3] = {
        {-1, 1, -1}, {-1, 1, 1}, {1, 1, 1}, {1, 1, -1},     {-1, -1, 1}, {-1, -1, -1}, {1, -1, -1}, {1, -1, 1},
        {-1, 1, 1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},     {1, 1, -1}, {1, -1, -1}, {-1, -1, -1}, {-1, 1, -1},
        {-1, 1, -1}, {-1, -1, -1}, {-1, -1, 1}, {-1, 1, 1}, {1, 1, 1}, {1, -1, 1}, {1, -1, -1}, {1, 1, -1}};
    static const signed char nrm[6][3] = {{0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}, {-1, 0, 0}, {1, 0, 0}};
    static const signed char edges[12][6] = {
        {-1, 1, 1, 1, 1, 1}, {-1, -1, 1, 1, -1, 1}, {-1, -1, -1, 1, -1, -1}, {-1, 1, -1, 1, 1, -1},
        {1, -1, 1, 1, 1, 1}, {-1, -1, 1, -1, 1, 1}, {-1, -1, -1, -1, 1, -1}, {1, -1, -1, 1, 1, -1},
        {1, 1, 1, 1, 1, -1}, {-1, 1, 1, -1, 1, -1}, {-1, -1, 1, -1, -1, -1}, {1, -1, 1, 1, -1, -1}};
    const R h = R(0.5);
    s.verts.clear(); s.faces.clear(); s.edge_a.clear(); s.edge_b.clear();
    for (auto& v : vtx) s.verts.push_back(V3<R>(h * v[0], h * v[1], h * v[2]));
    for (int f = 0; f < 6; f++) {
        Face<R> face;
        for (int k = 0; k < 4; k++) face.idx.push_back(f * 4 + k);
        face.normal = V3<R>(R(nrm[f][0]), R(nrm[f][1]), R(nrm[f][2]));
        s.faces.push_back(face);
    }
    for (auto& e : edges) {
        s.edge_a.push_back(V3<R>(h * e[0], h * e[1], h * e[2]));
        s.edge_b.push_back(V3<R>(h * e[3], h * e[4], h * e[5]));
    }
}

// Unit cylinder of default_mesh.h:59-273: a 20-gon top ring (vertices 0-19, angle 18k),
// a bottom ring rotated by 9 degrees (20-39), side copies of both rings (40-79), two caps and
// 40 side triangles.  Coordinates and normals are the reference's 6-decimal literals,
// including its one deviating side normal (face 8, x = -0.493982).
template <class R> void default_cylinder_mesh(Shape<R>& s) {
    // 0.5*cos / 0.5*sin of 0,18,...,90 degrees and of 9,27,...,81 degrees (6 decimals)
    static const double top_c[6] = {0.5, 0.475528, 0.404508, 0.293893, 0.154508, 0.0};
    static const double bot_c[5] = {0.493844, 0.445503, 0.353553, 0.226995, 0.078217};
    // negation that keeps the reference's literal +0 for zero table entries
    auto neg = [](double v) { return v == 0.0 ? 0.0 : -v; };
    auto ring = [&](const double* c, int n_quarter, int k, double& x, double& z) {
        // angle index k over a full turn of 4*n_quarter steps; x = cos, z = -sin
        const int q = k / n_quarter, r = k % n_quarter;
        const double cx = c[r], sx = c[n_quarter - r];   // first-quadrant values for offset r
        switch (q) {
            case 0: x = cx; z = neg(sx); break;
            case 1: x = neg(sx); z = neg(cx); break;
            case 2: x = neg(cx); z = sx; break;
            default: x = sx; z = cx; break;
        }
    };
    s.verts.assign(80, V3<R>());
    double tx[20], tz[20], bx[20], bz[20];
    for (int k = 0; k < 20; k++) {
        ring(top_c, 5, k, tx[k], tz[k]);
        // bottom ring: angles 9+18k; first quadrant has 5 entries (9..81), symmetric table
        const int q = k / 5, r = k % 5;
        const double c = bot_c[r], sn = bot_c[4 - r];
        switch (q) {
            case 0: bx[k] = c; bz[k] = -sn; break;
            case 1: bx[k] = -sn; bz[k] = -c; break;
            case 2: bx[k] = -c; bz[k] = sn; break;
            default: bx[k] = sn; bz[k] = c; break;
        }
    }
    for (int k = 0; k < 20; k++) {
        s.verts[k] = V3<R>(R(tx[k]), R(0.5), R(tz[k]));
        s.verts[20 + k] = V3<R>(R(bx[k]), R(-0.5), R(bz[k]));
        s.verts[40 + k] = s.verts[k];
        s.verts[60 + k] = s.verts[20 + k];
    }
    s.faces.clear();
    Face<R> top, bottom;
    for (int k = 0; k < 20; k++) top.idx.push_back(k);
    top.normal = V3<R>(0, 1, 0);
    for (int k = 39; k >= 20; k--) bottom.idx.push_back(k);
    bottom.normal = V3<R>(0, -1, 0);
    s.faces.push_back(top);
    s.faces.push_back(bottom);
    // side triangles (top edge k..k+1 over bottom k): normals at angles 9+18k, y = +0.006156
    static const double n1[5] = {0.987670, 0.890990, 0.707093, 0.453982, 0.156432};
    for (int k = 0; k < 20; k++) {
        Face<R> f;
        f.idx = {60 + k, 40 + (k + 1) % 20, 40 + k};
        const int q = k / 5, r = k % 5;
        const double c = n1[r], sn = n1[4 - r];
        double x, z;
        switch (q) {
            case 0: x = c; z = -sn; break;
            case 1: x = -sn; z = -c; break;
            case 2: x = -c; z = sn; break;
            default: x = sn; z = c; break;
        }
        if (k == 6) x = -0.493982;  // the reference table's value for this face
        f.normal = V3<R>(R(x), R(0.006156), R(z));
        s.faces.push_back(f);
    }
    // side triangles (bottom edge k-1..k under top k): normals at angles 18k, y = -0.006156
    static const double n2[6] = {0.999981, 0.951038, 0.809002, 0.587774, 0.309011, 0.0};
    for (int k = 0; k < 20; k++) {
        Face<R> f;
        f.idx = {40 + k, 60 + (k + 19) % 20, 60 + k};
        double x, z;
        ring(n2, 5, k, x, z);
        f.normal = V3<R>(R(x), R(-0.006156), R(z));
        s.faces.push_back(f);
    }
    // unique edges: top ring, bottom ring (cap winding), then the side zig-zag
    s.edge_a.clear(); s.edge_b.clear();
    for (int k = 0; k < 20; k++) { s.edge_a.push_back(s.verts[k]); s.edge_b.push_back(s.verts[(k + 1) % 20]); }
    for (int j = 0; j < 20; j++) {
        const int a = 39 - j, b = j == 19 ? 39 : 38 - j;
        s.edge_a.push_back(s.verts[a]); s.edge_b.push_back(s.verts[b]);
    }
    for (int k = 0; k < 20; k++) {
        s.edge_a.push_back(s.verts[k]); s.edge_b.push_back(s.verts[20 + k]);
        s.edge_a.push_back(s.verts[20 + k]); s.edge_b.push_back(s.verts[(k + 1) % 20]);
    }
}

// ---------------------------------------------------------------- constructors
template <class R> Shape<R> make_box(const V3<R>& size) {   // box_shape.cpp:7-25
    Shape<R> s;
    s.type = ST_BOX;
    s.size = size;
    s.half = size / R(2);
    default_box_mesh(s);
    for (auto& v : s.verts) v = cmul(v, size);
    for (size_t i = 0; i < s.edge_a.size(); i++) { s.edge_a[i] = cmul(s.edge_a[i], size); s.edge_b[i] = cmul(s.edge_b[i], size); }
    const R x2 = size.x * size.x, y2 = size.y * size.y, z2 = size.z * size.z;
    s.local_inertia = M3<R>();
    s.local_inertia.m[0][0] = (y2 + z2) / 12;
    s.local_inertia.m[1][1] = (x2 + z2) / 12;
    s.local_inertia.m[2][2] = (x2 + y2) / 12;
    s.volume = size.x * size.y * size.z;
    return s;
}

template <class R> Shape<R> make_sphere(R r) {   // sphere_shape.cpp:5-12
    Shape<R> s;
    s.type = ST_SPHERE;
    s.radius = r;
    s.volume = R(4.0 / 3.0) * kPi<R>() * r * r * r;
    const R i = R(2.0 / 5.0) * r * r;
    s.local_inertia = M3<R>();
    s.local_inertia.m[0][0] = s.local_inertia.m[1][1] = s.local_inertia.m[2][2] = i;
    return s;
}

template <class R> Shape<R> make_cylinder(R radius, R height) {   // cylinder_shape.cpp:6-32
    Shape<R> s;
    s.type = ST_CYLINDER;
    s.radius = radius;
    s.height = height;
    default_cylinder_mesh(s);
    const R r2 = radius * 2;
    for (auto& v : s.verts) { v.x *= r2; v.z *= r2; v.y *= height; }
    for (size_t i = 0; i < s.edge_a.size(); i++) {
        s.edge_a[i].x *= r2; s.edge_a[i].z *= r2; s.edge_a[i].y *= height;
        s.edge_b[i].x *= r2; s.edge_b[i].z *= r2; s.edge_b[i].y *= height;
    }
    const R rr = radius * radius, hh = height * height;
    const R axis = rr * R(0.5);
    const R diag = rr / R(4.0) + hh / R(12.0);
    s.volume = kPi<R>() * rr * height;
    s.local_inertia = M3<R>();
    s.local_inertia.m[0][0] = diag; s.local_inertia.m[1][1] = axis; s.local_inertia.m[2][2] = diag;
    return s;
}

// bvh.cpp:90-128 recursive build (sorts the face range in place), flattened into s.bvh
template <class R> int build_bvh(Shape<R>& s, int l, int r, int n) {
    if (l > r) return -1;
    typename Shape<R>::Node node;
    node.aa = V3<R>(Limits<R>::max(), Limits<R>::max(), Limits<R>::max());
    node.bb = V3<R>(Limits<R>::min(), Limits<R>::min(), Limits<R>::min());
    for (int i = l; i <= r; i++) {
        V3<R> mn(Limits<R>::max(), Limits<R>::max(), Limits<R>::max()), mx(Limits<R>::min(), Limits<R>::min(), Limits<R>::min());
        for (int k : s.faces[i].idx) {
            const V3<R>& p = s.verts[k];
            if (p.x < mn.x) mn.x = p.x;
            if (p.y < mn.y) mn.y = p.y;
            if (p.z < mn.z) mn.z = p.z;
        }
        for (int k : s.faces[i].idx) {
            const V3<R>& p = s.verts[k];
            if (p.x > mx.x) mx.x = p.x;
            if (p.y > mx.y) mx.y = p.y;
            if (p.z > mx.z) mx.z = p.z;
        }
        if (mn.x < node.aa.x) node.aa.x = mn.x;
        if (mn.y < node.aa.y) node.aa.y = mn.y;
        if (mn.z < node.aa.z) node.aa.z = mn.z;
        if (mx.x > node.bb.x) node.bb.x = mx.x;
        if (mx.y > node.bb.y) node.bb.y = mx.y;
        if (mx.z > node.bb.z) node.bb.z = mx.z;
    }
    const int id = (int)s.bvh.size();
    s.bvh.push_back(node);
    if (r - l + 1 <= n) {
        s.bvh[id].n = r - l + 1;
        s.bvh[id].index = l;
        return id;
    }
    const R lx = node.bb.x - node.aa.x, ly = node.bb.y - node.aa.y, lz = node.bb.z - node.aa.z;
    const int axis = (lx >= ly && lx >= lz) ? 0 : (ly >= lz ? 1 : 2);
    auto centroid = [&](const Face<R>& f) {
        R sum = 0;
        for (int k : f.idx) sum += s.verts[k][axis];
        sum /= (R)f.idx.size();
        return sum;
    };
    std::sort(s.faces.begin() + l, s.faces.begin() + r + 1,
              [&](const Face<R>& a, const Face<R>& b) { return centroid(a) < centroid(b); });
    const int mid = (l + r) / 2;
    const int left = build_bvh(s, l, mid, n);
    const int right = build_bvh(s, mid + 1, r, n);
    s.bvh[id].left = left;
    s.bvh[id].right = right;
    return id;
}

// bvh.cpp:105-125 stack search: right child popped first
template <class R> void bvh_search(const Shape<R>& s, const V3<R>& AA, const V3<R>& BB, std::vector<int>& out) {
    if (s.bvh.empty()) return;
    std::vector<int> stack{0};
    while (!stack.empty()) {
        const int id = stack.back();
        stack.pop_back();
        if (id < 0) continue;
        const auto& nd = s.bvh[id];
        if (nd.aa.x > BB.x || nd.aa.y > BB.y || nd.aa.z > BB.z) continue;
        if (nd.bb.x < AA.x || nd.bb.y < AA.y || nd.bb.z < AA.z) continue;
        if (nd.n > 0) {
            for (int i = 0; i < nd.n; i++) out.push_back(nd.index + i);
        } else {
            stack.push_back(nd.left);
            stack.push_back(nd.right);
        }
    }
}

// convex_mesh_shape.cpp:12-131: polyhedral mass properties, recentring, face tree, unique edges.
// Faces must carry their normals already (common/mesh.cpp perFaceNormal).
template <class R> Shape<R> make_hull(std::vector<V3<R>> verts, std::vector<Face<R>> faces) {
    Shape<R> s;
    s.type = ST_HULL;
    s.verts = std::move(verts);
    s.faces = std::move(faces);
    const R mult[10] = {R(1.0) / 6, R(1.0) / 24, R(1.0) / 24, R(1.0) / 24, R(1.0) / 60,
                        R(1.0) / 60, R(1.0) / 60, R(1.0) / 120, R(1.0) / 120, R(1.0) / 120};
    R intg[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    auto sub = [](R w0, R w1, R w2, R& f1, R& f2, R& f3, R& g0, R& g1, R& g2) {
        R tmp0 = w0 + w1;
        f1 = tmp0 + w2;
        R tmp1 = w0 * w0;
        R tmp2 = tmp1 + w1 * tmp0;
        f2 = tmp2 + w2 * f1;
        f3 = w0 * tmp1 + w1 * tmp2 + w2 * f2;
        g0 = f2 + w0 * (f1 + w0);
        g1 = f2 + w1 * (f1 + w1);
        g2 = f2 + w2 * (f1 + w2);
    };
    for (auto& face : s.faces) {
        const V3<R>& v0 = s.verts[face.idx[0]];
        for (int i = 0; i < (int)face.idx.size() - 2; i++) {
            const V3<R>& v1 = s.verts[face.idx[i + 1]];
            const V3<R>& v2 = s.verts[face.idx[i + 2]];
            R x0 = v0.x, y0 = v0.y, z0 = v0.z, x1 = v1.x, y1 = v1.y, z1 = v1.z, x2 = v2.x, y2 = v2.y, z2 = v2.z;
            R a1 = x1 - x0, b1 = y1 - y0, c1 = z1 - z0, a2 = x2 - x0, b2 = y2 - y0, c2 = z2 - z0;
            R d0 = b1 * c2 - b2 * c1, d1 = a2 * c1 - a1 * c2, d2 = a1 * b2 - a2 * b1;
            R f1x, f2x, f3x, g0x, g1x, g2x, f1y, f2y, f3y, g0y, g1y, g2y, f1z, f2z, f3z, g0z, g1z, g2z;
            sub(x0, x1, x2, f1x, f2x, f3x, g0x, g1x, g2x);
            sub(y0, y1, y2, f1y, f2y, f3y, g0y, g1y, g2y);
            sub(z0, z1, z2, f1z, f2z, f3z, g0z, g1z, g2z);
            intg[0] += d0 * f1x;
            intg[1] += d0 * f2x;
            intg[2] += d1 * f2y;
            intg[3] += d2 * f2z;
            intg[4] += d0 * f3x;
            intg[5] += d1 * f3y;
            intg[6] += d2 * f3z;
            intg[7] += d0 * (y0 * g0x + y1 * g1x + y2 * g2x);
            intg[8] += d1 * (z0 * g0y + z1 * g1y + z2 * g2y);
            intg[9] += d2 * (x0 * g0z + x1 * g1z + x2 * g2z);
        }
    }
    for (int i = 0; i < 10; i++) intg[i] *= mult[i];
    s.volume = intg[0];
    const V3<R> cm(intg[1] / s.volume, intg[2] / s.volume, intg[3] / s.volume);
    M3<R>& I = s.local_inertia;
    I.m[0][0] = intg[5] + intg[6] - s.volume * (cm.y * cm.y + cm.z * cm.z);
    I.m[1][1] = intg[4] + intg[6] - s.volume * (cm.z * cm.z + cm.x * cm.x);
    I.m[2][2] = intg[4] + intg[5] - s.volume * (cm.x * cm.x + cm.y * cm.y);
    I.m[0][1] = I.m[1][0] = -intg[7] + s.volume * cm.x * cm.y;
    I.m[1][2] = I.m[2][1] = -intg[8] + s.volume * cm.y * cm.z;
    I.m[0][2] = I.m[2][0] = -intg[9] + s.volume * cm.z * cm.x;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) I.m[i][j] /= s.volume;
    for (auto& v : s.verts) v = v - cm;
    const int node_size = std::max((int)s.faces.size() / 8191, 1);
    build_bvh(s, 0, (int)s.faces.size() - 1, node_size);
    // unique edges in face order; vertex identity by first registration of an
    // approximately-equal position (hull vertices are assumed separated by > 1e-5)
    std::vector<V3<R>> reg;
    auto vid = [&](const V3<R>& p) {
        for (size_t i = 0; i < reg.size(); i++) {
            if (std::abs(reg[i].x - p.x) < kEps<R>() && std::abs(reg[i].y - p.y) < kEps<R>() && std::abs(reg[i].z - p.z) < kEps<R>()) return (int)i;
        }
        reg.push_back(p);
        return (int)reg.size() - 1;
    };
    std::vector<std::pair<int, int>> seen;
    for (auto& f : s.faces) {
        for (int i = 0; i < (int)f.idx.size(); i++) {
            const int v0 = f.idx[i], v1 = f.idx[(i + 1) % f.idx.size()];
            int id0 = vid(s.verts[v0]);
            int id1 = vid(s.verts[v1]);
            if (id0 > id1) std::swap(id0, id1);
            if (std::find(seen.begin(), seen.end(), std::make_pair(id0, id1)) == seen.end()) {
                seen.emplace_back(id0, id1);
                s.edge_a.push_back(s.verts[v0]);
                s.edge_b.push_back(s.verts[v1]);
            }
        }
    }
    return s;
}

// ConcaveMeshShape::setMesh (concave_mesh_shape.cpp:6-17): the mesh as given (no recentring, no
// unique edges), unit local inertia, zero volume, and the face tree with leaves of
// max(faces / 2047, 1) faces (the tree sorts the faces in place).
template <class R> Shape<R> make_concave(std::vector<V3<R>> verts, std::vector<Face<R>> faces) {
    Shape<R> s;
    s.type = ST_CONCAVE;
    s.verts = std::move(verts);
    s.faces = std::move(faces);
    s.local_inertia = M3<R>::identity();
    s.volume = 0;
    build_bvh(s, 0, (int)s.faces.size() - 1, std::max((int)s.faces.size() / 2047, 1));
    return s;
}

// CompoundShape::addShape for each child (compound_shape.cpp:7-21) followed by init() (:25-47):
// children relocated to their mass-ratio centroid, the compound's local inertia summed from the
// children's rotated inertia plus the parallel-axis term, weighted by mass ratio.  `shapes` holds
// the children's shapes.  Returns the centroid (init()'s relocation vector).
template <class R> V3<R> make_compound(Shape<R>& s, std::vector<Child<R>> kids, const std::vector<Shape<R>>& shapes) {
    s = Shape<R>();
    s.type = ST_COMPOUND;
    R total = 0;
    for (auto& c : kids) {
        if (shapes[c.shape].type == ST_COMPOUND) throw std::runtime_error("CompoundShape cannot contain another CompoundShape");
        if (c.ratio < kEps<R>()) throw std::runtime_error("mass ratio must be greater than 0");
        total += c.ratio;
        s.volume += shapes[c.shape].volume;
    }
    V3<R> centroid(0, 0, 0);
    for (auto& c : kids) centroid = centroid + c.local.origin * c.ratio;
    centroid = centroid / total;
    M3<R> L;
    for (auto& c : kids) {
        const M3<R>& si = shapes[c.shape].local_inertia;
        const V3<R> p = c.local.origin - centroid;
        c.local.origin = p;
        const M3<R>& rot = c.local.basis;
        M3<R> t;
        const R pp = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
        for (int i = 0; i < 3; i++) t.m[i][i] = pp;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) t.m[i][j] -= p[i] * p[j];
        const M3<R> a = mmt_r2l(mm(rot, si), rot);
        const R k = c.ratio / total;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) L.m[i][j] = L.m[i][j] + (a.m[i][j] + t.m[i][j]) * k;
    }
    s.local_inertia = L;
    s.children = kids;
    return centroid;
}

// points every compound child at its shape (once the shape table no longer grows)
template <class R> void link_children(std::vector<Shape<R>>& shapes) {
    for (auto& s : shapes)
        for (auto& c : s.children) c.s = &shapes[c.shape];
}

// ---------------------------------------------------------------- queries
template <class R> void get_aabb(const Shape<R>& s, const Transform<R>& t, V3<R>& mn, V3<R>& mx) {
    const R MX = Limits<R>::max(), MN = Limits<R>::min();
    switch (s.type) {
        case ST_COMPOUND: {   // compound_shape.cpp:49-58
            mn = V3<R>(MX, MX, MX); mx = V3<R>(MN, MN, MN);
            for (auto& c : s.children) {
                V3<R> a, b;
                get_aabb(*c.s, t * c.local, a, b);
                mn = V3<R>(mn.x < a.x ? mn.x : a.x, mn.y < a.y ? mn.y : a.y, mn.z < a.z ? mn.z : a.z);   // PE_VEC_MIN2
                mx = V3<R>(mx.x > b.x ? mx.x : b.x, mx.y > b.y ? mx.y : b.y, mx.z > b.z ? mx.z : b.z);
            }
            break;
        }
        case ST_BOX: {   // box_shape.cpp:27-43
            mn = V3<R>(MX, MX, MX); mx = V3<R>(MN, MN, MN);
            for (int i = 0; i < 8; i++) {
                V3<R> p(i & 1 ? s.half.x : -s.half.x, i & 2 ? s.half.y : -s.half.y, i & 4 ? s.half.z : -s.half.z);
                V3<R> v = mv(t.basis, p);
                mn = V3<R>(mn.x < v.x ? mn.x : v.x, mn.y < v.y ? mn.y : v.y, mn.z < v.z ? mn.z : v.z);
                mx = V3<R>(mx.x > v.x ? mx.x : v.x, mx.y > v.y ? mx.y : v.y, mx.z > v.z ? mx.z : v.z);
            }
            mn = mn + t.origin; mx = mx + t.origin;
            break;
        }
        case ST_SPHERE: {   // sphere_shape.cpp:14-18
            const V3<R> r(s.radius, s.radius, s.radius);
            mn = t.origin - r; mx = t.origin + r;
            break;
        }
        case ST_CYLINDER: {   // cylinder_shape.cpp:34-43
            const V3<R> a = t.basis.col(1);
            V3<R> e = V3<R>(std::abs(a.x), std::abs(a.y), std::abs(a.z)) * (s.height * R(0.5));
            e.y += s.radius * std::sqrt(a.x * a.x + a.z * a.z);
            e.x += s.radius * std::sqrt(a.y * a.y + a.z * a.z);
            e.z += s.radius * std::sqrt(a.x * a.x + a.y * a.y);
            mn = t.origin - e; mx = t.origin + e;
            break;
        }
        default: {   // convex_mesh_shape.cpp:138-150
            mn = V3<R>(MX, MX, MX); mx = V3<R>(MN, MN, MN);
            for (auto& p : s.verts) {
                V3<R> v = mv(t.basis, p);
                mn = V3<R>(mn.x < v.x ? mn.x : v.x, mn.y < v.y ? mn.y : v.y, mn.z < v.z ? mn.z : v.z);
                mx = V3<R>(mx.x > v.x ? mx.x : v.x, mx.y > v.y ? mx.y : v.y, mx.z > v.z ? mx.z : v.z);
            }
            mn = mn + t.origin; mx = mx + t.origin;
        }
    }
}

template <class R> bool local_inside(const Shape<R>& s, const V3<R>& p) {
    switch (s.type) {
        case ST_BOX: return std::abs(p.x) <= s.half.x && std::abs(p.y) <= s.half.y && std::abs(p.z) <= s.half.z;
        case ST_SPHERE: return sqnorm(p) <= s.radius * s.radius;
        case ST_CYLINDER:
            return p.y >= -s.height * R(0.5) && p.y <= s.height * R(0.5) && p.x * p.x + p.z * p.z <= s.radius * s.radius;
        default:
            for (auto& f : s.faces)
                if (dot(f.normal, p - s.verts[f.idx[0]]) >= 0) return false;
            return true;
    }
}

template <class R> void project(const Shape<R>& s, const Transform<R>& t, const V3<R>& axis, R& mnp, R& mxp,
                                V3<R>& mnpt, V3<R>& mxpt) {
    switch (s.type) {
        case ST_BOX: {   // box_shape.cpp:51-68
            const V3<R> la = mtv(t.basis, axis);
            const R off = dot(t.origin, axis);
            V3<R> ext(la.x > 0 ? s.half.x : -s.half.x, la.y > 0 ? s.half.y : -s.half.y, la.z > 0 ? s.half.z : -s.half.z);
            const R he = dot(ext, la);
            mnp = off - he; mxp = off + he;
            mnpt = t.apply(-ext); mxpt = t.apply(ext);
            break;
        }
        case ST_SPHERE: {   // sphere_shape.cpp:24-32
            const R off = dot(t.origin, axis);
            mnp = off - s.radius; mxp = off + s.radius;
            mnpt = t.origin - axis * s.radius; mxpt = t.origin + axis * s.radius;
            break;
        }
        case ST_CYLINDER: {   // cylinder_shape.cpp:50-79
            const V3<R> la = mtv(t.basis, axis);
            const R hh = s.height * R(0.5);
            const R off = dot(t.origin, axis);
            if (std::abs(la.x - 0) < kEps<R>() && std::abs(la.z - 0) < kEps<R>()) {
                const V3<R> up = V3<R>(0, 1, 0) * hh;
                mnpt = t.apply(-up); mxpt = t.apply(up);
                mnp = off - hh; mxp = off + hh;
            } else if (std::abs(la.y - 0) < kEps<R>()) {
                const V3<R> r = la * s.radius;
                mnpt = t.apply(-r); mxpt = t.apply(r);
                mnp = off - s.radius; mxp = off + s.radius;
            } else {
                const R r = std::sqrt(la.x * la.x + la.z * la.z);
                const R x = s.radius * la.x / r, z = s.radius * la.z / r;
                const R y = hh * (la.y > 0 ? 1 : -1);
                const V3<R> ext(x, y, z);
                mnpt = t.apply(-ext); mxpt = t.apply(ext);
                const R el = dot(ext, la);
                mnp = off - el; mxp = off + el;
            }
            break;
        }
        default: {   // convex_mesh_shape.cpp:160-183 (max only updated when not a new min)
            const V3<R> la = mtv(t.basis, axis);
            const R off = dot(t.origin, axis);
            mnp = Limits<R>::max(); mxp = Limits<R>::min();
            V3<R> a, b;
            for (auto& p : s.verts) {
                const R v = dot(p, la);
                if (v < mnp) { mnp = v; a = p; }
                else if (v > mxp) { mxp = v; b = p; }
            }
            mnp += off; mxp += off;
            mnpt = t.apply(a); mxpt = t.apply(b);
        }
    }
}

} // namespace orc
