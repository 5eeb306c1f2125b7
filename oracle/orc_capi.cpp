// C interface of the oracle for ctypes (test infrastructure only).
// All reals cross the interface as double; a float world rounds on the way in.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include "orc_world.h"

using namespace orc;

namespace {

struct SceneFile {
    int S = 0, N = 0, HV = 0, HF = 0, HI = 0, iters = 10;
    double dt = 0.01, g[3] = {0, -9.8, 0};
    std::vector<int> type, vbeg, vcnt, fbeg, fcnt, foff, fidx, shape, flags;
    std::vector<double> param, hv, mass, fr, re, ld, ad, org, bas, v, w;
    // compound children ("PESCENE2" files): per shape [cbeg, cbeg + ccnt), per child its shape,
    // local origin, local basis (row-major) and mass ratio
    std::vector<int> cbeg, ccnt, cshape;
    std::vector<double> corg, cbas, cratio;
    // tagged sections: joints (type, bodies a b, flags, 15 reals) and ignored body pairs
    std::vector<int> jtype, jbody, jflag, ign;
    std::vector<double> jreal;
};

bool read_scene(const char* path, SceneFile& s) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    char magic[8];
    bool ok = fread(magic, 1, 8, f) == 8 && (memcmp(magic, "PESCENE1", 8) == 0 || memcmp(magic, "PESCENE2", 8) == 0);
    const bool compound = ok && memcmp(magic, "PESCENE2", 8) == 0;
    int hdr[6];
    double w4[4];
    ok = ok && fread(hdr, sizeof(int), 6, f) == 6 && fread(w4, sizeof(double), 4, f) == 4;
    if (!ok) { fclose(f); return false; }
    s.S = hdr[0]; s.N = hdr[1]; s.HV = hdr[2]; s.HF = hdr[3]; s.HI = hdr[4]; s.iters = hdr[5];
    s.dt = w4[0]; s.g[0] = w4[1]; s.g[1] = w4[2]; s.g[2] = w4[3];
    auto rdi = [&](std::vector<int>& a, size_t n) { a.resize(n); return n == 0 || fread(a.data(), sizeof(int), n, f) == n; };
    auto rdd = [&](std::vector<double>& a, size_t n) { a.resize(n); return n == 0 || fread(a.data(), sizeof(double), n, f) == n; };
    ok = rdi(s.type, s.S) && rdd(s.param, s.S * 3) && rdi(s.vbeg, s.S) && rdi(s.vcnt, s.S) && rdi(s.fbeg, s.S) &&
         rdi(s.fcnt, s.S) && rdd(s.hv, s.HV * 3) && rdi(s.foff, s.HF + 1) && rdi(s.fidx, s.HI) && rdi(s.shape, s.N) &&
         rdi(s.flags, s.N) && rdd(s.mass, s.N) && rdd(s.fr, s.N) && rdd(s.re, s.N) && rdd(s.ld, s.N) && rdd(s.ad, s.N) &&
         rdd(s.org, s.N * 3) && rdd(s.bas, s.N * 9) && rdd(s.v, s.N * 3) && rdd(s.w, s.N * 3);
    if (ok && compound) {
        int C = 0;
        ok = fread(&C, sizeof(int), 1, f) == 1 && C >= 0 && rdi(s.cbeg, s.S) && rdi(s.ccnt, s.S) && rdi(s.cshape, C) &&
             rdd(s.corg, (size_t)C * 3) && rdd(s.cbas, (size_t)C * 9) && rdd(s.cratio, C);
        int th[2];
        while (ok && fread(th, sizeof(int), 2, f) == 2) {
            const int n = th[1];
            if (n < 0) { ok = false; break; }
            if (th[0] == 1) ok = rdi(s.jtype, n) && rdi(s.jbody, (size_t)2 * n) && rdi(s.jflag, n) && rdd(s.jreal, (size_t)15 * n);
            else if (th[0] == 2) ok = rdi(s.ign, (size_t)2 * n);
            else ok = false;
        }
    }
    fclose(f);
    return ok;
}

struct Handle {
    int bits = 64;
    std::unique_ptr<World<double>> w64;
    std::unique_ptr<World<float>> w32;
    std::unique_ptr<Pool> pool;
};

template <class R> void put3(double* o, const V3<R>& v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }
template <class R> void put9(double* o, const M3<R>& m) { for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) o[r * 3 + c] = m.m[r][c]; }
template <class R> V3<R> get3(const double* o) { return V3<R>(R(o[0]), R(o[1]), R(o[2])); }
template <class R> M3<R> get9(const double* o) { M3<R> m; for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) m.m[r][c] = R(o[r * 3 + c]); return m; }

template <class R> void build(World<R>& W, const SceneFile& s) {
    W.dt = R(s.dt);
    W.gravity = V3<R>(R(s.g[0]), R(s.g[1]), R(s.g[2]));
    W.iterations = s.iters;
    for (int i = 0; i < s.S; i++) {
        const double* p = &s.param[i * 3];
        if (s.type[i] == ST_COMPOUND) { W.shapes.push_back(Shape<R>()); continue; }   // built below, once its children exist
        switch (s.type[i]) {
            case ST_BOX: W.shapes.push_back(make_box<R>(V3<R>(R(p[0]), R(p[1]), R(p[2])))); break;
            case ST_SPHERE: W.shapes.push_back(make_sphere<R>(R(p[0]))); break;
            case ST_CYLINDER: W.shapes.push_back(make_cylinder<R>(R(p[0]), R(p[1]))); break;
            default: {
                std::vector<V3<R>> vs;
                for (int k = 0; k < s.vcnt[i]; k++) {
                    const double* q = &s.hv[(s.vbeg[i] + k) * 3];
                    vs.push_back(V3<R>(R(q[0]), R(q[1]), R(q[2])));
                }
                std::vector<Face<R>> fs;
                for (int fi = s.fbeg[i]; fi < s.fbeg[i] + s.fcnt[i]; fi++) {
                    Face<R> face;
                    for (int k = s.foff[fi]; k < s.foff[fi + 1]; k++) face.idx.push_back(s.fidx[k]);
                    // common/mesh.cpp perFaceNormal: (p2-p1)x(p3-p1), normalised
                    const V3<R>& p1 = vs[face.idx[0]];
                    face.normal = normalized(cross(vs[face.idx[1]] - p1, vs[face.idx[2]] - p1));
                    fs.push_back(face);
                }
                W.shapes.push_back(s.type[i] == ST_CONCAVE ? make_concave<R>(vs, fs) : make_hull<R>(vs, fs));
            }
        }
    }
    for (int i = 0; i < s.S; i++) {
        if (s.type[i] != ST_COMPOUND) continue;
        if (s.cbeg.empty()) throw std::runtime_error("compound shape without a children table");
        std::vector<Child<R>> kids;
        for (int k = s.cbeg[i]; k < s.cbeg[i] + s.ccnt[i]; k++) {
            Child<R> c;
            c.shape = s.cshape[k];
            c.local.origin = get3<R>(&s.corg[(size_t)k * 3]);
            c.local.basis = get9<R>(&s.cbas[(size_t)k * 9]);
            c.ratio = R(s.cratio[k]);
            kids.push_back(c);
        }
        make_compound(W.shapes[i], kids, W.shapes);
    }
    link_children(W.shapes);
    W.bodies.resize(s.N);
    for (int i = 0; i < s.N; i++) {
        Body<R>& b = W.bodies[i];
        b.shape = s.shape[i];
        b.kinematic = (s.flags[i] & 1) != 0;
        b.ignore_collision = (s.flags[i] & 2) != 0;
        M3<R> basis;
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) basis.m[r][c] = R(s.bas[i * 9 + r * 3 + c]);
        W.init_body(b, R(s.mass[i]), basis, V3<R>(R(s.org[i * 3]), R(s.org[i * 3 + 1]), R(s.org[i * 3 + 2])));
        b.v = V3<R>(R(s.v[i * 3]), R(s.v[i * 3 + 1]), R(s.v[i * 3 + 2]));
        b.w = V3<R>(R(s.w[i * 3]), R(s.w[i * 3 + 1]), R(s.w[i * 3 + 2]));
        b.friction = R(s.fr[i]);
        b.restitution = R(s.re[i]);
        b.lin_damp = R(s.ld[i]);
        b.ang_damp = R(s.ad[i]);
    }
    for (size_t k = 0; k + 1 < s.ign.size(); k += 2) {   // RigidBody::addIgnoreCollisionId
        W.bodies[s.ign[k]].ignore_ids.push_back(s.ign[k + 1]);
    }
    for (size_t k = 0; k < s.jtype.size(); k++) {   // World::addConstraint
        Joint<R> j;
        const double* r = &s.jreal[k * 15];
        j.type = s.jtype[k];
        j.a = s.jbody[2 * k];
        j.b = s.jbody[2 * k + 1];
        j.use_limits = (s.jflag[k] & 1) != 0;
        j.use_motor = (s.jflag[k] & 2) != 0;
        j.anchor_a = get3<R>(r); j.anchor_b = get3<R>(r + 3); j.axis_a = get3<R>(r + 6); j.axis_b = get3<R>(r + 9);
        j.min_angle = R(r[12]); j.max_angle = R(r[13]); j.target_speed = R(r[14]);
        W.joints.push_back(j);
    }
}


template <class F> auto with(void* h, F&& f) {
    Handle* H = static_cast<Handle*>(h);
    if (H->bits == 64) return f(*H->w64);
    return f(*H->w32);
}

} // namespace

extern "C" {

void* orc_create(const char* scene_path, int real_bits, int threads) {
    SceneFile s;
    if (!read_scene(scene_path, s)) return nullptr;
    auto* H = new Handle();
    H->bits = real_bits == 32 ? 32 : 64;
    if (threads > 1) H->pool.reset(new Pool(threads));
    try {
        if (H->bits == 64) { H->w64.reset(new World<double>()); build(*H->w64, s); H->w64->pool = H->pool.get(); }
        else { H->w32.reset(new World<float>()); build(*H->w32, s); H->w32->pool = H->pool.get(); }
    } catch (const std::exception& e) {
        fprintf(stderr, "orc_create: %s\n", e.what());
        delete H;
        return nullptr;
    }
    return H;
}

void orc_destroy(void* h) { delete static_cast<Handle*>(h); }

int orc_n_bodies(void* h) { return with(h, [](auto& W) { return (int)W.bodies.size(); }); }
int orc_n_pairs(void* h) { return with(h, [](auto& W) { return (int)W.pairs.size(); }); }
int orc_n_results(void* h) { return with(h, [](auto& W) { return (int)W.results.size(); }); }
int orc_get_axis(void* h) { return with(h, [](auto& W) { return W.axis; }); }
void orc_set_axis(void* h, int a) { with(h, [a](auto& W) { W.axis = a; return 0; }); }
// contact margin (PE_MARGIN, phys_general.h:45; the reference compiles it as 0)
void orc_set_margin(void* h, double m) { with(h, [m](auto& W) { W.margin = static_cast<decltype(W.margin)>(m); return 0; }); }
// broadphase sort ties in body order (std::stable_sort) instead of std::sort's order
void orc_set_stable_ties(void* h, int on) { with(h, [on](auto& W) { W.stable_ties = on != 0; return 0; }); }

void orc_step(void* h, int n) { with(h, [n](auto& W) { for (int i = 0; i < n; i++) W.step(); return 0; }); }

// wall time of n full steps (seconds)
double orc_time_steps(void* h, int n) {
    auto t0 = std::chrono::steady_clock::now();
    orc_step(h, n);
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void orc_integrate(void* h) { with(h, [](auto& W) { W.integrate(); return 0; }); }
int orc_broadphase(void* h) { return with(h, [](auto& W) { W.broadphase(); return (int)W.pairs.size(); }); }
void orc_narrowphase(void* h) { with(h, [](auto& W) { W.narrowphase(); return 0; }); }
void orc_solve(void* h) { with(h, [](auto& W) { W.solve(); return 0; }); }

// body state: origin[N*3], basis[N*9], lin_vel[N*3], ang_vel[N*3], aabb_min, aabb_max [N*3], world_inv_inertia[N*9]
void orc_get_state(void* h, double* o, double* b, double* v, double* w, double* mn, double* mx, double* iw) {
    with(h, [&](auto& W) {
        for (size_t i = 0; i < W.bodies.size(); i++) {
            const auto& B = W.bodies[i];
            put3(o + i * 3, B.t.origin); put9(b + i * 9, B.t.basis); put3(v + i * 3, B.v); put3(w + i * 3, B.w);
            put3(mn + i * 3, B.aabb_min); put3(mx + i * 3, B.aabb_max); put9(iw + i * 9, B.world_inv_inertia);
        }
        return 0;
    });
}

void orc_set_state(void* h, const double* o, const double* b, const double* v, const double* w, const double* mn,
                   const double* mx, const double* iw) {
    with(h, [&](auto& W) {
        using R = typename std::remove_reference<decltype(W.bodies[0].mass)>::type;
        for (size_t i = 0; i < W.bodies.size(); i++) {
            auto& B = W.bodies[i];
            B.t.origin = get3<R>(o + i * 3); B.t.basis = get9<R>(b + i * 9); B.v = get3<R>(v + i * 3); B.w = get3<R>(w + i * 3);
            B.aabb_min = get3<R>(mn + i * 3); B.aabb_max = get3<R>(mx + i * 3); B.world_inv_inertia = get9<R>(iw + i * 9);
        }
        return 0;
    });
}

void orc_get_pairs(void* h, int* out) {
    with(h, [&](auto& W) { for (size_t i = 0; i < W.pairs.size(); i++) { out[i * 2] = W.pairs[i].first; out[i * 2 + 1] = W.pairs[i].second; } return 0; });
}

void orc_set_pairs(void* h, const int* p, int n) {
    with(h, [&](auto& W) { W.pairs.resize(n); for (int i = 0; i < n; i++) W.pairs[i] = {p[i * 2], p[i * 2 + 1]}; return 0; });
}

// results: a, b, point_size, valid_mask [R]; friction, restitution [R]; slots [R*8*19]
void orc_get_results(void* h, int* a, int* b, int* ps, int* mask, double* fr, double* re, double* slots) {
    with(h, [&](auto& W) {
        for (size_t i = 0; i < W.results.size(); i++) {
            const auto& r = W.results[i];
            a[i] = r.a; b[i] = r.b; ps[i] = r.point_size; fr[i] = r.friction; re[i] = r.restitution;
            int m = 0;
            for (int k = 0; k < kCache; k++) {
                const auto& p = r.pts[k];
                if (p.valid()) m |= 1 << k;
                double* o = slots + (i * kCache + k) * 19;
                put3(o, p.pos); put3(o + 3, p.normal); put3(o + 6, p.la); put3(o + 9, p.lb);
                o[12] = p.dist; put3(o + 13, p.t0); put3(o + 16, p.t1);
            }
            mask[i] = m;
        }
        return 0;
    });
}

void orc_set_results(void* h, int n, const int* a, const int* b, const int* ps, const double* fr, const double* re,
                     const double* slots) {
    with(h, [&](auto& W) {
        using R = typename std::remove_reference<decltype(W.bodies[0].mass)>::type;
        W.results.assign(n, CResult<R>());
        for (int i = 0; i < n; i++) {
            auto& r = W.results[i];
            r.a = a[i]; r.b = b[i]; r.point_size = ps[i]; r.friction = R(fr[i]); r.restitution = R(re[i]);
            for (int k = 0; k < kCache; k++) {
                const double* o = slots + (i * kCache + k) * 19;
                auto& p = r.pts[k];
                p.pos = get3<R>(o); p.normal = get3<R>(o + 3); p.la = get3<R>(o + 6); p.lb = get3<R>(o + 9);
                p.dist = R(o[12]); p.t0 = get3<R>(o + 13); p.t1 = get3<R>(o + 16);
            }
        }
        return 0;
    });
}

// shape tables after preprocessing (hull face order after the face-tree sort, unique edges)
int orc_shape_counts(void* h, int s, int* nv, int* nf, int* ne) {
    return with(h, [&](auto& W) {
        if (s < 0 || s >= (int)W.shapes.size()) return -1;
        const auto& S = W.shapes[s];
        *nv = (int)S.verts.size(); *nf = (int)S.faces.size(); *ne = (int)S.edge_a.size();
        return S.type;
    });
}

} // extern "C"
