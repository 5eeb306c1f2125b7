// World<R> member definitions; included by exactly one translation unit per precision.
#pragma once
#include <algorithm>
#include "pe_world.cuh"

namespace pe {

template <class R> World<R>::World(int device) : dev_(device) {
    PE_CK(cudaSetDevice(dev_));
    PE_CK(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    for (auto& e : ev_) { PE_CK(cudaEventCreate(&e[0])); PE_CK(cudaEventCreate(&e[1])); }
    UnitMeshes u;
    std::memset(&u, 0, sizeof(u));
    build_unit_meshes(u);
    PE_CK(cudaMemcpyToSymbol(g_unit, &u, sizeof(u)));
    status_.ensure(1);
    PE_CK(cudaMemset(status_.p, 0, sizeof(int)));
    total_.ensure(1);
    set_scenes(1, nullptr);
}

template <class R> World<R>::~World() {
    if (st_) cudaStreamSynchronize(st_);
    if (stage_) cudaFreeHost(stage_);
    for (auto& q : pending_) { cudaEventDestroy(q.e0); cudaEventDestroy(q.e1); }
    for (auto e : ev_pool_) cudaEventDestroy(e);
    for (auto& e : ev_) { cudaEventDestroy(e[0]); cudaEventDestroy(e[1]); }
    if (st_) cudaStreamDestroy(st_);
}

template <class R> void World<R>::ev_begin(int k) {
    PE_CK(cudaEventRecord(ev_[k][0], st_));
    ev_open_[k] = true;
}
template <class R> void World<R>::ev_end(int k) {
    PE_CK(cudaEventRecord(ev_[k][1], st_));
    PE_CK(cudaEventSynchronize(ev_[k][1]));
    float ms = 0;
    PE_CK(cudaEventElapsedTime(&ms, ev_[k][0], ev_[k][1]));
    ms_[k] += ms;
    ev_open_[k] = false;
}
template <class R> void World<R>::phase_times(double* ms, bool reset) {
    for (int k = 0; k < 5; k++) ms[k] = ms_[k];
    if (reset) for (double& m : ms_) m = 0;
}
template <class R> void World<R>::last_counts(int* c) {
    c[0] = P_; c[1] = n_active_; c[2] = n_rows_; c[3] = n_colors_; c[4] = (int)last_step_launches_; c[5] = n_islands_;
}

template <class R> void World<R>::check_status() {
    int s = 0;
    PE_CK(cudaMemcpyAsync(&s, status_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
    if (s) {
        PE_CK(cudaMemsetAsync(status_.p, 0, sizeof(int), st_));
        throw std::runtime_error("device capacity overflow (status " + std::to_string(s) + ")");
    }
}

template <class R> ShapeTable<R> World<R>::shapes() const {
    ShapeTable<R> t;
    t.type = stype_.p; t.param = sparam_.p; t.hull = shull_.p;
    t.h_vbeg = hvbeg_.p; t.h_vcnt = hvcnt_.p; t.h_fbeg = hfbeg_.p; t.h_fcnt = hfcnt_.p; t.h_ebeg = hebeg_.p; t.h_ecnt = hecnt_.p;
    t.h_rad = hrad_.p;
    t.hv = hv_.p; t.f_off = hfoff_.p; t.f_idx = hfidx_.p; t.f_n = hfn_.p; t.f_min = hfmin_.p; t.f_max = hfmax_.p;
    t.e_a = hea_.p; t.e_b = heb_.p;
    t.c_beg = cbeg_.p; t.c_cnt = ccnt_.p; t.c_shape = cshape_.p; t.c_xf = cxf_.p;
    t.h_lbeg = hlbeg_.p; t.h_lcnt = hlcnt_.p; t.lf_beg = lfbeg_.p; t.lf_cnt = lfcnt_.p; t.lf_min = lfmin_.p; t.lf_max = lfmax_.p;
    return t;
}

template <class R> Results<R> World<R>::results() {
    Results<R> r;
    r.cap = pair_cap_;
    r.a = res_a_.p; r.b = res_b_.p; r.npts = res_np_.p; r.fr = res_fr_.p; r.re = res_re_.p; r.pts = res_pts_.p;
    r.dist = res_dist_[cur_dist_].p;
    r.prev_dist = res_dist_[cur_dist_ ^ 1].p;
    return r;
}

template <class R> Rows<R> World<R>::rows() {
    Rows<R> r;
    r.cap = rows_cap_;
    r.f = rows_.p;
    return r;
}

template <class T> static void upload(DBuf<T>& d, const std::vector<T>& h, cudaStream_t st) {
    d.ensure(h.size() + 1);
    if (!h.empty()) PE_CK(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

// ------------------------------------------------------------------ scene upload
// device copy grows geometrically keeping its contents; only the new tail is copied
template <class T> static void upload_tail(DBuf<T>& d, const std::vector<T>& h, size_t from, cudaStream_t st) {
    const size_t want = h.size() + 1;
    if (want > d.n) d.ensure(std::max(want, d.n + d.n / 2), true);
    if (h.size() > from) PE_CK(cudaMemcpyAsync(d.p + from, h.data() + from, (h.size() - from) * sizeof(T), cudaMemcpyHostToDevice, st));
}

template <class R>
void World<R>::set_shapes(int S, const int* type, const double* param, const int* vbeg, const int* vcnt, const int* fbeg,
                          const int* fcnt, int HV, const double* hv, int HF, const int* foff, const int* fidx) {
    (void)HV; (void)HF;
    S_ = 0;
    h_stype_.clear(); h_sparam_.clear(); h_sinertia_.clear(); h_shull_.clear();
    h_hvb_.clear(); h_hvc_.clear(); h_hfb_.clear(); h_hfc_.clear(); h_heb_.clear(); h_hec_.clear(); h_foff_.clear(); h_fidx_.clear();
    h_hv_.clear(); h_fn_.clear(); h_fmn_.clear(); h_fmx_.clear(); h_ea_.clear(); h_eb_.clear(); h_hrad_.clear();
    hull_by_content_.clear();
    h_cbeg_.clear(); h_ccnt_.clear(); h_cshape_.clear(); h_cready_.clear(); h_cxf_.clear();
    h_hlb_.clear(); h_hlc_.clear(); h_lfb_.clear(); h_lfc_.clear(); h_lfmn_.clear(); h_lfmx_.clear();
    append_shapes(S, type, param, vbeg, vcnt, fbeg, fcnt, hv, foff, fidx);
}

template <class R>
int World<R>::append_shapes(int S, const int* type, const double* param, const int* vbeg, const int* vcnt, const int* fbeg,
                            const int* fcnt, const double* hv, const int* foff, const int* fidx, std::vector<int>* remap) {
    const int s0 = S_;
    const size_t o_h = h_hvb_.size(), o_v = h_hv_.size(), o_f = h_fn_.size(), o_e = h_ea_.size(), o_fo = h_foff_.size(),
                 o_fi = h_fidx_.size(), o_l = h_lfb_.size();
    if (remap) remap->assign(S, -1);
    int added = 0;
    for (int s = 0; s < S; s++) {
        const int t = type[s];
        std::string key;
        if (remap && (t == ST_HULL || t == ST_CONCAVE)) {   // content key: kind, vertices, then face index lists
            key.reserve((size_t)vcnt[s] * 24 + (size_t)(foff[fbeg[s] + fcnt[s]] - foff[fbeg[s]] + fcnt[s] + 3) * 4);
            const int head[4] = {t, vcnt[s], fcnt[s], foff[fbeg[s] + fcnt[s]] - foff[fbeg[s]]};
            key.append(reinterpret_cast<const char*>(head), sizeof head);
            key.append(reinterpret_cast<const char*>(hv + (size_t)vbeg[s] * 3), (size_t)vcnt[s] * 3 * sizeof(double));
            for (int f = 0; f < fcnt[s]; f++) {
                const int n = foff[fbeg[s] + f + 1] - foff[fbeg[s] + f];
                key.append(reinterpret_cast<const char*>(&n), sizeof n);
                key.append(reinterpret_cast<const char*>(fidx + foff[fbeg[s] + f]), (size_t)n * sizeof(int));
            }
            auto it = hull_by_content_.find(key);
            if (it != hull_by_content_.end()) { (*remap)[s] = it->second; continue; }
        }
        const int gs = s0 + added++;
        if (remap) (*remap)[s] = gs;
        if (!key.empty()) hull_by_content_.emplace(std::move(key), gs);
        V3<R> p;
        for (int k = 0; k < 3; k++) h_sparam_.push_back(R(param[s * 3 + k]));
        p = V3<R>(h_sparam_[(size_t)gs * 3], h_sparam_[(size_t)gs * 3 + 1], h_sparam_[(size_t)gs * 3 + 2]);
        h_stype_.push_back(t);
        int hull = -1;
        M3<R> inertia;
        if (t == ST_BOX) inertia = box_inertia(p);
        else if (t == ST_SPHERE) inertia = sphere_inertia(p.x);
        else if (t == ST_CYLINDER) inertia = cylinder_inertia(p.x, p.y);
        else if (t == ST_HULL || t == ST_CONCAVE) {
            // local face offsets of this shape
            std::vector<int> lo(fcnt[s] + 1);
            for (int f = 0; f <= fcnt[s]; f++) lo[f] = foff[fbeg[s] + f] - foff[fbeg[s]];
            if (t == ST_HULL && fcnt[s] >= 16382) throw std::runtime_error("convex mesh with more than 16381 faces is not supported");
            if (t == ST_CONCAVE)
                for (int f = 0; f < fcnt[s]; f++)
                    if (lo[f + 1] - lo[f] > kFaceVerts)
                        throw std::runtime_error("concave mesh face with more than " + std::to_string(kFaceVerts) + " vertices");
            HullPrep<R> h = prepare_hull<R>(hv + (size_t)vbeg[s] * 3, vcnt[s], lo.data(), fidx + foff[fbeg[s]], fcnt[s],
                                            t == ST_CONCAVE);
            inertia = h.inertia;
            h_hlb_.push_back((int)h_lfb_.size());
            h_hlc_.push_back((int)h.l_beg.size());
            h_lfb_.insert(h_lfb_.end(), h.l_beg.begin(), h.l_beg.end());
            h_lfc_.insert(h_lfc_.end(), h.l_cnt.begin(), h.l_cnt.end());
            h_lfmn_.insert(h_lfmn_.end(), h.l_min.begin(), h.l_min.end());
            h_lfmx_.insert(h_lfmx_.end(), h.l_max.begin(), h.l_max.end());
            hull = (int)h_hvb_.size();
            h_hvb_.push_back((int)h_hv_.size() / 3); h_hvc_.push_back(vcnt[s]);
            h_hfb_.push_back((int)h_fn_.size() / 3); h_hfc_.push_back(fcnt[s]);
            h_heb_.push_back((int)h_ea_.size() / 3); h_hec_.push_back((int)h.e_a.size() / 3);
            h_hrad_.push_back(h.inner); h_hrad_.push_back(h.outer);
            const int ibase = (int)h_fidx_.size();
            if (h_foff_.empty()) h_foff_.push_back(0);
            for (int f = 0; f < fcnt[s]; f++) h_foff_.push_back(ibase + h.f_off[f + 1]);
            h_fidx_.insert(h_fidx_.end(), h.f_idx.begin(), h.f_idx.end());
            h_hv_.insert(h_hv_.end(), h.v.begin(), h.v.end());
            h_fn_.insert(h_fn_.end(), h.f_n.begin(), h.f_n.end());
            h_fmn_.insert(h_fmn_.end(), h.f_min.begin(), h.f_min.end());
            h_fmx_.insert(h_fmx_.end(), h.f_max.begin(), h.f_max.end());
            h_ea_.insert(h_ea_.end(), h.e_a.begin(), h.e_a.end());
            h_eb_.insert(h_eb_.end(), h.e_b.begin(), h.e_b.end());
        } else if (t == ST_COMPOUND && !remap) {
            inertia = M3<R>();   // set by set_compounds (CompoundShape::init)
        } else {
            throw std::runtime_error(t == ST_COMPOUND ? "compound shapes are not supported in batched requests"
                                                      : "unsupported shape type " + std::to_string(t));
        }
        h_cbeg_.push_back(0);
        h_ccnt_.push_back(0);
        h_cready_.push_back(t != ST_COMPOUND);
        h_shull_.push_back(hull);
        h_sinertia_.push_back(inertia);
    }
    // hull face offsets are global per face: face f of hull h sits at hfb[h] + f, its offsets at
    // f_off[hfb[h] + f] .. f_off[hfb[h] + f + 1]
    S_ = s0 + added;
    PE_CK(cudaStreamSynchronize(st_));   // growth copies below run outside the stream
    upload_tail(stype_, h_stype_, s0, st_); upload_tail(sparam_, h_sparam_, (size_t)s0 * 3, st_); upload_tail(shull_, h_shull_, s0, st_);
    upload_tail(hvbeg_, h_hvb_, o_h, st_); upload_tail(hvcnt_, h_hvc_, o_h, st_); upload_tail(hfbeg_, h_hfb_, o_h, st_);
    upload_tail(hfcnt_, h_hfc_, o_h, st_); upload_tail(hebeg_, h_heb_, o_h, st_); upload_tail(hecnt_, h_hec_, o_h, st_);
    upload_tail(hv_, h_hv_, o_v, st_); upload_tail(hfoff_, h_foff_, o_fo, st_); upload_tail(hfidx_, h_fidx_, o_fi, st_);
    upload_tail(hfn_, h_fn_, o_f, st_); upload_tail(hfmin_, h_fmn_, o_f, st_); upload_tail(hfmax_, h_fmx_, o_f, st_);
    upload_tail(hea_, h_ea_, o_e, st_); upload_tail(heb_, h_eb_, o_e, st_); upload_tail(hrad_, h_hrad_, o_h * 2, st_);
    upload_tail(cbeg_, h_cbeg_, s0, st_); upload_tail(ccnt_, h_ccnt_, s0, st_);
    upload_tail(hlbeg_, h_hlb_, o_h, st_); upload_tail(hlcnt_, h_hlc_, o_h, st_);
    upload_tail(lfbeg_, h_lfb_, o_l, st_); upload_tail(lfcnt_, h_lfc_, o_l, st_);
    upload_tail(lfmin_, h_lfmn_, o_l * 3, st_); upload_tail(lfmax_, h_lfmx_, o_l * 3, st_);
    PE_CK(cudaStreamSynchronize(st_));
    return s0;
}

// CompoundShape::addShape for each child (compound_shape.cpp:7-21) and init() (:25-47) for every
// compound shape of the table: the children are relocated to their mass-ratio centroid and the
// compound's unit-mass local inertia is the sum over children of (rot * I_child * rot^T + the
// parallel-axis term |p|^2 E - p p^T) * ratio / total ratio, in the reference's operation order.
// With `local_inertia` the children are taken as already initialised and the given inertia is used.
template <class R>
void World<R>::set_compounds(const int* cbeg, const int* ccnt, int C, const int* cshape, const double* corg, const double* cbas,
                             const double* cratio, const double* local_inertia, double* centroid) {
    if (N_ > 0) throw std::runtime_error("compound shapes must be set before the bodies");
    h_cshape_.clear();
    h_cxf_.clear();
    for (int s = 0; s < S_; s++) {
        h_cbeg_[s] = 0;
        h_ccnt_[s] = 0;
        if (centroid) centroid[s * 3] = centroid[s * 3 + 1] = centroid[s * 3 + 2] = 0;
        if (h_stype_[s] != ST_COMPOUND) continue;
        const int b = cbeg[s], n = ccnt[s];
        if (n < 1 || b < 0 || b + n > C) throw std::runtime_error("compound shape " + std::to_string(s) + ": bad children range");
        struct Kid { int shape; M3<R> basis; V3<R> origin; R ratio; };
        std::vector<Kid> kids(n);
        R total = 0;
        for (int k = 0; k < n; k++) {
            Kid& c = kids[k];
            c.shape = cshape[b + k];
            if (c.shape < 0 || c.shape >= S_ || h_stype_[c.shape] == ST_COMPOUND || h_stype_[c.shape] == ST_CONCAVE)
                throw std::runtime_error("compound shape " + std::to_string(s) +
                                         ": a child must name a shape that is neither compound nor concave");
            c.ratio = R(cratio[b + k]);
            if (c.ratio < eps<R>()) throw std::runtime_error("mass ratio must be greater than 0");
            for (int r = 0; r < 3; r++) for (int q = 0; q < 3; q++) c.basis.m[r][q] = R(cbas[(size_t)(b + k) * 9 + r * 3 + q]);
            c.origin = V3<R>(R(corg[(size_t)(b + k) * 3]), R(corg[(size_t)(b + k) * 3 + 1]), R(corg[(size_t)(b + k) * 3 + 2]));
            total += c.ratio;
        }
        M3<R> L;
        if (local_inertia) {
            for (int r = 0; r < 3; r++) for (int q = 0; q < 3; q++) L.m[r][q] = R(local_inertia[(size_t)s * 9 + r * 3 + q]);
        } else {
            V3<R> cen(0, 0, 0);
            for (auto& c : kids) cen = cen + c.origin * c.ratio;
            cen = cen / total;
            for (auto& c : kids) {
                const V3<R> p = c.origin - cen;
                c.origin = p;
                M3<R> t;
                const R pp = p.x * p.x + p.y * p.y + p.z * p.z;
                for (int i = 0; i < 3; i++) t.m[i][i] = pp;
                for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) t.m[i][j] -= p[i] * p[j];
                const M3<R> a = world_inertia(c.basis, h_sinertia_[c.shape]);
                const R k = c.ratio / total;
                for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) L.m[i][j] = L.m[i][j] + (a.m[i][j] + t.m[i][j]) * k;
            }
            if (centroid) { centroid[s * 3] = cen.x; centroid[s * 3 + 1] = cen.y; centroid[s * 3 + 2] = cen.z; }
        }
        h_sinertia_[s] = L;
        h_cbeg_[s] = (int)h_cshape_.size();
        h_ccnt_[s] = n;
        h_cready_[s] = 1;
        for (auto& c : kids) {
            h_cshape_.push_back(c.shape);
            for (int r = 0; r < 3; r++) for (int q = 0; q < 3; q++) h_cxf_.push_back(c.basis.m[r][q]);
            h_cxf_.push_back(c.origin.x); h_cxf_.push_back(c.origin.y); h_cxf_.push_back(c.origin.z);
        }
    }
    upload(cbeg_, h_cbeg_, st_);
    upload(ccnt_, h_ccnt_, st_);
    upload(cshape_, h_cshape_, st_);
    upload(cxf_, h_cxf_, st_);
    PE_CK(cudaStreamSynchronize(st_));
}

// World::addConstraint for each joint, in order (sequential_impulse_solver.cpp:46-48, 60-68 run
// them after the contacts of every iteration)
template <class R>
void World<R>::set_joints(int n, const int* type, const int* body, const int* flag, const double* param) {
    std::vector<int> t(type, type + n), f(flag, flag + n);
    std::vector<int2> b(n);
    std::vector<R> q((size_t)n * NJP);
    for (int j = 0; j < n; j++) {
        if (t[j] < JT_BALL || t[j] > JT_SLIDER) throw std::runtime_error("joint " + std::to_string(j) + ": unknown type");
        b[j] = make_int2(body[2 * j], body[2 * j + 1]);
        if (b[j].x < 0 || b[j].x >= N_ || b[j].y < 0 || b[j].y >= N_ || b[j].x == b[j].y)
            throw std::runtime_error("joint " + std::to_string(j) + ": bad bodies");
        for (int k = 0; k < NJP; k++) q[(size_t)j * NJP + k] = R(param[(size_t)j * NJP + k]);
    }
    n_joints_ = n;
    upload(jtype_, t, st_);
    upload(jflag_, f, st_);
    upload(jbody_, b, st_);
    upload(jparam_, q, st_);
    jrow_.ensure((size_t)std::max(n, 1) * NJR);
    PE_CK(cudaStreamSynchronize(st_));
}

// RigidBody::addIgnoreCollisionId: symmetric partner lists, and BF_IGN_LIST on the bodies that have one
template <class R> void World<R>::set_ignore_pairs(int n, const int* pairs) {
    std::vector<std::vector<int>> part(N_);
    for (int k = 0; k < n; k++) {
        const int a = pairs[2 * k], b = pairs[2 * k + 1];
        if (a < 0 || a >= N_ || b < 0 || b >= N_) throw std::runtime_error("ignored pair " + std::to_string(k) + ": bad body");
        part[a].push_back(b);
        part[b].push_back(a);
    }
    std::vector<int> off(N_ + 1, 0), ids;
    for (int i = 0; i < N_; i++) {
        ids.insert(ids.end(), part[i].begin(), part[i].end());
        off[i + 1] = (int)ids.size();
    }
    std::vector<int> fl(N_);
    PE_CK(cudaMemcpyAsync(fl.data(), bflags_.p, N_ * sizeof(int), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
    for (int i = 0; i < N_; i++) fl[i] = (fl[i] & ~BF_IGN_LIST) | (off[i + 1] > off[i] ? BF_IGN_LIST : 0);
    upload(bflags_, fl, st_);
    upload(ign_off_, off, st_);
    upload(ign_ids_, ids, st_);
    n_ign_ = n;
    PE_CK(cudaStreamSynchronize(st_));
}

// RigidBody::setMass + setCollisionShape (rigidbody.cpp:11-41) and the initial pose: body j of a
// field-major array with the given stride
template <class R>
void World<R>::fill_body(R* f, size_t stride, int j, int shape, double mass, double fr, double re, double ld, double ad,
                         const double* o, const double* b, const double* v, const double* w) const {
    auto F = [&](int k) -> R& { return f[(size_t)k * stride + j]; };
    const R m = R(mass);
    const R inv_m = m > eps<R>() ? R(1.0) / m : R(0);
    M3<R> li;
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) li.m[r][c] = h_sinertia_[shape].m[r][c] * m;
    const M3<R> lii = m > eps<R>() ? inverse3(li) : M3<R>();
    M3<R> basis;
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) basis.m[r][c] = R(b[r * 3 + c]);
    const M3<R> wi = world_inertia(basis, lii);
    for (int k = 0; k < 3; k++) {
        F(OX + k) = R(o[k]);
        F(VX + k) = R(v[k]);
        F(WX + k) = R(w[k]);
    }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            F(B00 + r * 3 + c) = basis.m[r][c];
            F(I00 + r * 3 + c) = wi.m[r][c];
            F(L00 + r * 3 + c) = lii.m[r][c];
        }
    F(INVM) = inv_m;
    F(MASS) = m;
    F(FRIC) = R(fr);
    F(REST) = R(re);
    F(LDAMP) = R(ld);
    F(ADAMP) = R(ad);
}

template <class R>
void World<R>::set_bodies(int n, const int* shape, const int* flags, const double* mass, const double* fr, const double* re,
                          const double* ld, const double* ad, const double* o, const double* b, const double* v,
                          const double* w) {
    N_ = n;
    bcap_ = std::max(n, 1);
    std::vector<R> f((size_t)NBF * bcap_, R(0));
    for (int i = 0; i < n; i++) {
        if (shape[i] < 0 || shape[i] >= S_) throw std::runtime_error("body " + std::to_string(i) + ": bad shape index");
        if (!h_cready_[shape[i]]) throw std::runtime_error("body " + std::to_string(i) + ": compound shape without children");
        fill_body(f.data(), bcap_, i, shape[i], mass[i], fr[i], re[i], ld[i], ad[i], o + i * 3, b + i * 9, v + i * 3, w + i * 3);
    }
    upload(bf_, f, st_);
    upload(bshape_, std::vector<int>(shape, shape + n), st_);
    std::vector<int> fl(flags, flags + n);
    for (auto& x : fl) x &= BF_KINEMATIC | BF_IGNORE;   // BF_IGN_LIST belongs to set_ignore_pairs
    upload(bflags_, fl, st_);
    n_joints_ = 0;   // joints and ignored pairs name bodies: set them again after the bodies
    n_ign_ = 0;
    claim_.ensure(n + 1);
    set_scenes(1, nullptr);
}

template <class R> void World<R>::set_scenes(int ns, const int* off) {
    std::vector<int> so(ns + 1);
    if (off) for (int s = 0; s <= ns; s++) so[s] = off[s];
    else { so[0] = 0; so[1] = N_; }
    if (so[0] != 0 || so[ns] != N_) throw std::runtime_error("scene offsets must start at 0 and end at the body count");
    for (int s = 0; s < ns; s++) if (so[s + 1] < so[s]) throw std::runtime_error("scene offsets must not decrease");
    NS_ = ns;
    h_scene_off_ = so;
    build_axis_items();
    std::vector<int> sc(std::max(N_, 1), 0);
    for (int s = 0; s < ns; s++) for (int i = so[s]; i < so[s + 1]; i++) sc[i] = s;
    upload(bscene_, sc, st_);
    upload(scene_off_, so, st_);
    upload(scene_axis_, std::vector<int>(ns, 0), st_);
    std::vector<int> zero(ns + 1, 0);
    upload(pair_scene_off_, zero, st_);
    upload(res_scene_off_, zero, st_);
    upload(prev_res_off_, zero, st_);
    h_pair_scene_off_ = zero;
    P_ = 0;
    R_ = 0;
    PE_CK(cudaStreamSynchronize(st_));
}

// (scene, tile) work items of the scenes above kAxisTile bodies, consecutive per scene
template <class R> void World<R>::build_axis_items() {
    std::vector<int2> it;
    for (size_t s = 0; s + 1 < h_scene_off_.size(); s++) {
        const int cnt = h_scene_off_[s + 1] - h_scene_off_[s];
        if (cnt <= kAxisTile) continue;
        for (int t = 0; t * kAxisTile < cnt; t++) it.push_back(make_int2((int)s, t));
    }
    axis_items_n_ = (int)it.size();
    if (axis_items_n_) upload(axis_items_, it, st_);
}

template <class R> void World<R>::set_params(double dt, double gx, double gy, double gz, int iters) {
    prm_.dt = dt; prm_.g[0] = gx; prm_.g[1] = gy; prm_.g[2] = gz; prm_.iterations = iters;
}

// ------------------------------------------------------------------ utilities
template <class R> int World<R>::scan(int* data, int n) {
    const int tiles = (n + 1023) / 1024;
    aux_.ensure(tiles + 1);
    launch(K_SCAN, tiles, k_scan_tiles, data, n, aux_.p);
    launch(K_SCAN, 1, k_scan_aux, aux_.p, tiles, total_.p);
    launch(K_SCAN, tiles, k_scan_add, data, n, aux_.p);
    int tot = 0;
    PE_CK(cudaMemcpyAsync(&tot, total_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
    return tot;
}

template <class R> void World<R>::radix_sort(int n, int scene_passes) {
    order_ = val_[radix_sort_keys(n, (int)sizeof(R), scene_passes)].p;
}

template <class R> int World<R>::radix_sort_keys(int n, int key_passes, int scene_passes) {
    const int tiles = (n + kRadixTile - 1) / kRadixTile;
    hist_.ensure((size_t)256 * tiles + 1);
    aux_.ensure((256 * tiles + 1023) / 1024 + 1);
    int cur = 0;
    auto pass = [&](int shift, int use2) {
        launch(K_RADIX, tiles, k_radix_hist, key_[cur].p, key2_[cur].p, n, shift, use2, hist_.p, tiles);
        const int m = 256 * tiles;
        const int st = (m + 1023) / 1024;
        launch(K_SCAN, st, k_scan_tiles, hist_.p, m, aux_.p);
        launch(K_SCAN, 1, k_scan_aux, aux_.p, st, total_.p);
        launch(K_SCAN, st, k_scan_add, hist_.p, m, aux_.p);
        launch(K_RADIX, tiles, k_radix_scatter, key_[cur].p, key2_[cur].p, val_[cur].p, key_[cur ^ 1].p, key2_[cur ^ 1].p,
                                                  val_[cur ^ 1].p, n, shift, use2, hist_.p, tiles);
        cur ^= 1;
    };
    for (int s = 0; s < key_passes * 8; s += 8) pass(s, 0);
    for (int s = 0; s < scene_passes * 8; s += 8) pass(s, 1);
    return cur;
}

template <class R> void World<R>::ensure_pair_capacity(int P) {
    if (P <= pair_cap_) return;
    const int cap = std::max(P + P / 2, 1024);
    pairs_.ensure(cap);
    cls_.ensure(cap); order_np_.ensure(cap);
    res_a_.ensure(cap); res_b_.ensure(cap); res_np_.ensure(cap + 1);
    res_fr_.ensure(cap); res_re_.ensure(cap);
    res_pts_.ensure((size_t)NPF * cap * kSlots);
    // result slot distances survive between steps: grow both generations keeping contents
    res_dist_[0].ensure((size_t)cap * kSlots, true);
    res_dist_[1].ensure((size_t)cap * kSlots, true);
    row_off_.ensure(cap + 1); active_.ensure(cap + 1); color_.ensure(cap + 1);
    sat_out_.ensure((size_t)cap * kSatOut);
    // point buffer: field-major over the capacity; its contents live for one step only
    pair_cap_ = cap;
}

// ------------------------------------------------------------------ phases
template <class R> void World<R>::integrate() {
    if (N_ == 0) return;
    launch(K_INTEGRATE, grid(N_), k_integrate<R>, bodies(), shapes(), prm_, 1);
    PE_CK(cudaGetLastError());
}

template <class R> int World<R>::broadphase() {
    const int n = N_;
    if (n < 2) return P_;   // the reference leaves the pair list untouched below two bodies
    for (int k = 0; k < 2; k++) { key_[k].ensure(n); key2_[k].ensure(n); val_[k].ensure(n); }
    smn_.ensure((size_t)3 * n); smx_.ensure((size_t)3 * n); sflag_.ensure(n); ssc_.ensure(n);
    count_.ensure(n + 1);
    launch(K_BP_KEYS, grid(n), k_bp_keys<R>, bodies(), scene_axis_.p, key_[0].p, key2_[0].p, val_[0].p);
    int scene_passes = 0;
    for (int m = NS_ - 1; m > 0; m >>= 8) scene_passes++;
    radix_sort(n, scene_passes);
    launch(K_BP_GATHER, grid(n), k_bp_gather<R>, bodies(), order_, smn_.p, smx_.p, sflag_.p, ssc_.p);
    bp_stage_.ensure((size_t)n * kStage);
    bp_big_.ensure(n + 1);
    bp_nbig_.ensure(1);
    PE_CK(cudaMemsetAsync(bp_nbig_.p, 0, sizeof(int), st_));
    IgnoreLists ign;
    if (n_ign_ > 0) { ign.off = ign_off_.p; ign.ids = ign_ids_.p; ign.order = order_; }
    launch(K_BP_SWEEP, grid_warps(n), k_bp_count<R>, n, scene_axis_.p, smn_.p, smx_.p, sflag_.p, ssc_.p, count_.p, bp_stage_.p,
           bp_big_.p, bp_nbig_.p, ign);
    // crowded positions: windows in chunks of one block each (at most kMaxChunks per position)
    bp_wend_.ensure(n + 1); bp_csize_.ensure(n + 1); bp_nch_.ensure(n + 1); bp_choff_.ensure(n + 1); bp_ctot_.ensure(1);
    bp_ccount_.ensure((size_t)kMaxChunks * n + 1); bp_cpref_.ensure((size_t)kMaxChunks * n + 1);
    launch(K_BP_SWEEP, kBigSweepBlocks, k_bp_big_windows<R>, n, (const int*)scene_axis_.p, (const int*)scene_off_.p, (const R*)smn_.p,
           (const R*)smx_.p, (const int*)ssc_.p, (const int*)bp_big_.p, (const int*)bp_nbig_.p, bp_wend_.p, bp_csize_.p, bp_nch_.p);
    launch_block(K_BP_SWEEP, 1, 32, k_bp_chunk_offsets, (const int*)bp_nbig_.p, (const int*)bp_nch_.p, bp_choff_.p, bp_ctot_.p);
    launch(K_BP_SWEEP, 2 * kBigSweepBlocks, k_bp_count_chunks<R>, n, (const R*)smn_.p, (const R*)smx_.p, (const int*)sflag_.p,
           (const int*)bp_big_.p, (const int*)bp_nbig_.p, (const int*)bp_wend_.p, (const int*)bp_csize_.p, (const int*)bp_choff_.p,
           (const int*)bp_ctot_.p, bp_ccount_.p, ign);
    launch(K_BP_SWEEP, kBigSweepBlocks, k_bp_chunk_sums, (const int*)bp_big_.p, (const int*)bp_nbig_.p, (const int*)bp_choff_.p,
           (const int*)bp_nch_.p, (const int*)bp_ccount_.p, bp_cpref_.p, count_.p);
    PE_CK(cudaMemsetAsync(count_.p + n, 0, sizeof(int), st_));
    const int P = scan(count_.p, n + 1);
    ensure_pair_capacity(P);
    launch(K_BP_SWEEP, grid_warps(n), k_bp_write<R>, n, scene_axis_.p, smn_.p, smx_.p, sflag_.p, ssc_.p, order_, count_.p, bp_stage_.p,
           pairs_.p, pair_cap_, status_.p, ign);
    launch(K_BP_SWEEP, 2 * kBigSweepBlocks, k_bp_write_chunks<R>, n, (const R*)smn_.p, (const R*)smx_.p, (const int*)sflag_.p,
           (const uint32_t*)order_, (const int*)count_.p, (const int*)bp_big_.p, (const int*)bp_nbig_.p, (const int*)bp_wend_.p,
           (const int*)bp_csize_.p, (const int*)bp_choff_.p, (const int*)bp_ctot_.p, (const int*)bp_cpref_.p, pairs_.p, pair_cap_,
           status_.p, ign);
    launch(K_MISC, grid(NS_ + 1), k_scene_pair_off, NS_, scene_off_.p, count_.p, n, pair_scene_off_.p);
    launch(K_BP_AXIS, NS_, k_bp_axis<R>, smn_.p, smx_.p, n, scene_off_.p, scene_axis_.p);
    if (axis_items_n_ > 0) {   // scenes above kAxisTile bodies
        axis_part_.ensure((size_t)axis_items_n_ * 6);
        launch(K_BP_AXIS, axis_items_n_, k_bp_axis_tiles<R>, (const R*)smn_.p, (const R*)smx_.p, n, (const int*)scene_off_.p,
               (const int2*)axis_items_.p, axis_part_.p);
        launch(K_BP_AXIS, grid(axis_items_n_), k_bp_axis_combine, (const int*)scene_off_.p, (const int2*)axis_items_.p,
               axis_items_n_, (const double*)axis_part_.p, scene_axis_.p);
    }
    PE_CK(cudaGetLastError());
    P_ = P;
    return P;
}

template <class R> void World<R>::narrowphase() {
    const int P = P_;
    ensure_pair_capacity(std::max(P, 1));
    // the results of the previous step become the pool the new step draws stale slots from
    PE_CK(cudaMemcpyAsync(prev_res_off_.p, res_scene_off_.p, (NS_ + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st_));
    cur_dist_ ^= 1;
    if (P > 0) {
        cls_count_.ensure(2 * PC_COUNT);
        PE_CK(cudaMemsetAsync(cls_count_.p, 0, 2 * PC_COUNT * sizeof(int), st_));
        launch(K_NP_BUCKET, grid(P), k_np_classify<R>, P, pairs_.p, bodies(), shapes(), cls_.p, cls_count_.p);
        int cnt[PC_COUNT];
        PE_CK(cudaMemcpyAsync(cnt, cls_count_.p, sizeof(cnt), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaStreamSynchronize(st_));
        int cur[PC_COUNT], run = 0;
        for (int c = 0; c < PC_COUNT; c++) { cur[c] = run; run += cnt[c]; }
        PE_CK(cudaMemcpyAsync(cls_count_.p + PC_COUNT, cur, sizeof(cur), cudaMemcpyHostToDevice, st_));
        launch(K_NP_BUCKET, grid(P), k_np_bucket, P, cls_.p, cls_count_.p + PC_COUNT, order_np_.p);
        const Results<R> rs = results();
        const Bodies<R> bd = bodies();
        const ShapeTable<R> sh = shapes();
        if (!sat_attr_) {   // dynamic shared memory of the staged SAT kernels (above the 48 KB default for FP64)
            const int light = (int)(kSatWarps * sat_group_reals<R>(1) * sizeof(R));
            PE_CK(cudaFuncSetAttribute(k_np_sat<R, 1, ST_BOX, ST_HULL>, cudaFuncAttributeMaxDynamicSharedMemorySize, light));
            PE_CK(cudaFuncSetAttribute(k_np_sat<R, 1, ST_HULL, ST_BOX>, cudaFuncAttributeMaxDynamicSharedMemorySize, light));
            PE_CK(cudaFuncSetAttribute(k_np_sat<R, 1, ST_HULL, ST_HULL>, cudaFuncAttributeMaxDynamicSharedMemorySize, light));
            PE_CK(cudaFuncSetAttribute(k_np_sat<R, 1, ST_CYLINDER, ST_CYLINDER>, cudaFuncAttributeMaxDynamicSharedMemorySize, light));
            PE_CK(cudaFuncSetAttribute(k_np_sat<R, kSatGroup, -1, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sat_group_reals<R>(kSatGroup) * sizeof(R))));
            sat_attr_ = true;
        }
        for (int c = 0; c < PC_COUNT; c++) {
            const int lo = cur[c], hi = cur[c] + cnt[c];
            if (hi == lo) continue;
            const int g = grid(hi - lo);
            switch (c) {
                case PC_BOX_BOX: launch(K_NP, g, k_np_class<R, PC_BOX_BOX>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_BOX_SPHERE: launch(K_NP, g, k_np_class<R, PC_BOX_SPHERE>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_SPHERE_SPHERE: launch(K_NP, g, k_np_class<R, PC_SPHERE_SPHERE>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_SPHERE_CYL: launch(K_NP, g, k_np_class<R, PC_SPHERE_CYL>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_BOX_CYL: launch(K_NP, g, k_np_class<R, PC_BOX_CYL>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_SPHERE_HULL: launch(K_NP, g, k_np_class<R, PC_SPHERE_HULL>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_CYL_HULL: {
                    const int w = cyl_hull_warps<R>();
                    launch_block(K_NP, (hi - lo + w - 1) / w, 32 * w, k_np_cyl_hull<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs,
                                 pair_scene_off_.p, prev_res_off_.p);
                    break;
                }
                case PC_CONVEX:
                case PC_CONVEX_HULL_BOX:
                case PC_CONVEX_HULL_HULL:
                case PC_CONVEX_CYL_CYL: {
                    const size_t smem = (size_t)kSatWarps * sat_group_reals<R>(1) * sizeof(R);
                    const int gb = (hi - lo + kSatWarps - 1) / kSatWarps, bs = 32 * kSatWarps;
                    auto kern = c == PC_CONVEX ? k_np_sat<R, 1, ST_BOX, ST_HULL>
                              : c == PC_CONVEX_HULL_BOX ? k_np_sat<R, 1, ST_HULL, ST_BOX>
                              : c == PC_CONVEX_HULL_HULL ? k_np_sat<R, 1, ST_HULL, ST_HULL>
                              : k_np_sat<R, 1, ST_CYLINDER, ST_CYLINDER>;
                    launch_smem(K_NP_SAT, gb, bs, smem, kern, lo, hi, order_np_.p, pairs_.p, bd, sh, sat_out_.p);
                    launch(K_NP_SAT, grid(hi - lo), k_np_sat_finish<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p,
                           prev_res_off_.p, (const R*)sat_out_.p);
                    break;
                }
                case PC_CONVEX_HEAVY: {
                    const size_t smem = (size_t)sat_group_reals<R>(kSatGroup) * sizeof(R);
                    launch_smem(K_NP_SAT, hi - lo, 32 * kSatGroup, smem, k_np_sat<R, kSatGroup, -1, -1>, lo, hi, order_np_.p, pairs_.p, bd,
                                sh, sat_out_.p);
                    launch(K_NP_SAT, grid(hi - lo), k_np_sat_finish<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p,
                           prev_res_off_.p, (const R*)sat_out_.p);
                    break;
                }
                case PC_COMPOUND:
                    launch(K_NP, g, k_np_compound<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p);
                    break;
                case PC_CONCAVE:
                    launch(K_NP, g, k_np_class<R, PC_CONCAVE>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p,
                           prev_res_off_.p);
                    break;
                default:   // PC_CONVEX_BIG
                    launch(K_NP_SAT, grid_warps(hi - lo), k_np_sat_big<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs,
                           pair_scene_off_.p, prev_res_off_.p);
                    break;
            }
        }
        PE_CK(cudaGetLastError());
    }
    PE_CK(cudaMemcpyAsync(res_scene_off_.p, pair_scene_off_.p, (NS_ + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st_));
    R_ = P;
}

template <class R> void World<R>::solve(int mode) {
    const int P = R_;
    if (N_ == 0) return;
    launch(K_SI_MISC, grid(N_), k_si_clear<R>, bodies());
    n_active_ = 0;
    n_colors_ = 0;
    n_islands_ = 0;
    if (P > 0) {
        // rows: one per contact point, results' rows contiguous in result order
        PE_CK(cudaMemcpyAsync(row_off_.p, res_np_.p, P * sizeof(int), cudaMemcpyDeviceToDevice, st_));
        PE_CK(cudaMemsetAsync(row_off_.p + P, 0, sizeof(int), st_));
        n_rows_ = scan(row_off_.p, P + 1);
        if (n_rows_ > rows_cap_) {
            rows_cap_ = std::max(n_rows_ + n_rows_ / 2, 1024);
            rows_.ensure((size_t)NRF * rows_cap_);
        }
        launch(K_SI_SETUP, grid(P), k_si_setup<R>, P, results(), bodies(), rows(), row_off_.p, prm_, status_.p);
        // results with points, in result order
        launch(K_SI_MISC, grid(P + 1), k_active_flags, P, res_np_.p, active_.p);
        color_.ensure(P + 1);
        PE_CK(cudaMemcpyAsync(color_.p, active_.p, (P + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st_));
        n_active_ = scan(color_.p, P + 1);
        launch(K_SI_MISC, grid(P), k_active_compact, P, res_np_.p, color_.p, active_.p);
    }
    const int A = n_active_, NJ = n_joints_;
    const Joints<R> jt = joints();
    if (NJ > 0) launch(K_SI_SETUP, grid(NJ), k_joint_init<R>, jt, bodies(), prm_);
    const int M = A + NJ;   // island items: active contact results, then joints
    if (M > 0) {
        // islands: union-find over dynamic bodies linked by contacts and joints; items grouped by
        // island keeping their order (contacts in result order, then joints in order)
        parent_.ensure(N_ + 1);
        launch(K_ISLAND, grid(N_), k_isl_init, N_, parent_.p);
        if (A > 0) launch(K_ISLAND, grid(A), k_isl_union<R>, A, active_.p, results(), bodies(), parent_.p);
        if (NJ > 0) launch(K_ISLAND, grid(NJ), k_isl_union_joints<R>, jt, bodies(), parent_.p);
        for (int k = 0; k < 2; k++) { key_[k].ensure(M); key2_[k].ensure(M); val_[k].ensure(M); }
        if (A > 0)
            launch(K_ISLAND, grid(A), k_isl_keys<R>, A, active_.p, results(), bodies(), parent_.p, key_[0].p, key2_[0].p, val_[0].p);
        if (NJ > 0) launch(K_ISLAND, grid(NJ), k_isl_keys_joints<R>, jt, bodies(), parent_.p, A, key_[0].p, key2_[0].p, val_[0].p);
        int label_passes = 0;
        for (int m = NJ > 0 ? N_ : N_ - 1; m > 0; m >>= 8) label_passes++;   // joint labels reach n_bodies
        const int cur = radix_sort_keys(M, label_passes, 0);
        const uint64_t* skey = key_[cur].p;
        const uint32_t* order = val_[cur].p;
        isl_flag_.ensure(M + 1);
        isl_off_.ensure(M + 1);
        isl_n_.ensure(1);
        launch(K_ISLAND, grid(M + 1), k_isl_flags, M, skey, isl_flag_.p);
        n_islands_ = scan(isl_flag_.p, M + 1);
        launch(K_ISLAND, grid(M + 1), k_isl_offsets, M, skey, isl_flag_.p, isl_off_.p, isl_n_.p);
        const int NI = n_islands_;
        // islands of up to kSmallResults items: one thread each
        launch(K_SI_SERIAL, grid(NI), k_isl_serial<R>, isl_n_.p, isl_off_.p, order, results(), jt, bodies(), rows(), row_off_.p,
               prm_.iterations, 0, kSmallResults);
        if (mode == 0) {
            // serial order, larger islands: the exact level schedule, a block per island up to
            // kBigIsland items, grid-wide above
            isl_corder_.ensure(M);
            color_.ensure(M + 1);
            launch_block(K_SI_SERIAL, NI, kLevelBlock, k_isl_levels<R>, isl_n_.p, isl_off_.p, order, results(), jt, bodies(), rows(),
                         row_off_.p, prm_.iterations, kSmallResults, claim_.p, color_.p, isl_corder_.p);
            solve_big_islands(NI, order, true);
        } else {
            isl_corder_.ensure(M);
            color_.ensure(M + 1);
            ncol_.ensure(1);
            PE_CK(cudaMemsetAsync(ncol_.p, 0, sizeof(int), st_));
            launch_block(K_SI_COLOR, NI, kColorBlock, k_isl_colored<R>, isl_n_.p, isl_off_.p, order, results(), jt, bodies(), rows(),
                         row_off_.p, prm_.iterations, kSmallResults, claim_.p, color_.p, isl_corder_.p, ncol_.p);
            PE_CK(cudaMemcpyAsync(&n_colors_, ncol_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
            solve_big_islands(NI, order, false);
        }
    }
    launch(K_SI_MISC, grid(N_), k_si_sync<R>, bodies());
    PE_CK(cudaGetLastError());
}

// islands above kBigIsland results (coloured mode): grid-wide colouring rounds, then one launch per
// colour and iteration (see k_gc_*)
template <class R> void World<R>::solve_big_islands(int NI, const uint32_t* order, bool exact) {
    gc_big_.ensure(NI + 1);
    gc_n_.ensure(2);
    PE_CK(cudaMemsetAsync(gc_n_.p, 0, sizeof(int), st_));
    launch(K_SI_COLOR, grid(NI), k_isl_big, (const int*)isl_n_.p, (const int*)isl_off_.p, gc_big_.p, gc_n_.p);
    int nb = 0;
    PE_CK(cudaMemcpyAsync(&nb, gc_n_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
    if (nb == 0) return;
    std::vector<int> big(nb);
    PE_CK(cudaMemcpy(big.data(), gc_big_.p, nb * sizeof(int), cudaMemcpyDeviceToHost));
    std::sort(big.begin(), big.end());
    gc_cnt_.ensure(kMaxColorsBig + 1);
    gc_cursor_.ensure(kMaxColorsBig);
    const Results<R> rs = results();
    const Joints<R> jt = joints();
    const Bodies<R> bd = bodies();
    const Rows<R> rw = rows();
    std::vector<int> cnt(kMaxColorsBig + 1), start(kMaxColorsBig), cur(kMaxColorsBig);
    for (int s : big) {
        int lh[2];
        PE_CK(cudaMemcpy(lh, isl_off_.p + s, 2 * sizeof(int), cudaMemcpyDeviceToHost));
        const int lo = lh[0], m = lh[1] - lh[0], g = grid(m);
        PE_CK(cudaMemsetAsync(color_.p + lo, 0xff, (size_t)m * sizeof(int), st_));   // -1: uncoloured
        unsigned long long* mask = nullptr;   // exact level schedule: colour = round
        if (!exact) {
            gc_mask_.ensure(N_ + 1);
            mask = gc_mask_.p;
            launch(K_GC_COLOR, g, k_gc_mask_reset<R>, lo, m, order, rs, jt, mask);
        }
        // colouring rounds, the remaining count read back every 8 rounds (extra rounds find nothing to do)
        // all rounds in one cooperative launch (up to kMaxColorsBig - 1; items left over take the last colour)
        if (coop_blocks_ == 0) {
            int per_sm = 0, sms = 0;
            PE_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gc_solve<R>, kBlock, 0));
            int per_sm2 = 0;
            PE_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_gc_rounds<R>, kBlock, 0));
            PE_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_));
            coop_blocks_ = std::max(std::min(per_sm, per_sm2), 1) * sms;
        }
        gc_left_.ensure(kMaxColorsBig);
        PE_CK(cudaMemsetAsync(gc_left_.p, 0, kMaxColorsBig * sizeof(int), st_));
        gc_claim_.ensure(N_ + 1);
        launch_coop(K_GC_COLOR, coop_blocks_, kBlock, k_gc_rounds<R>, lo, m, order, rs, jt, bd, gc_claim_.p, color_.p, mask, gc_left_.p,
                    kMaxColorsBig - 1, gc_n_.p + 1);
        int ncol = 0;
        PE_CK(cudaMemcpyAsync(&ncol, gc_n_.p + 1, sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemsetAsync(gc_cnt_.p, 0, (kMaxColorsBig + 1) * sizeof(int), st_));
        launch(K_GC_COLOR, g, k_gc_count, lo, m, color_.p, gc_cnt_.p);
        PE_CK(cudaMemcpyAsync(cnt.data(), gc_cnt_.p, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaStreamSynchronize(st_));
        if (exact && cnt[kMaxColorsBig] > 0) {   // out of levels: the island in order on one thread
            launch_block(K_GC_SOLVE, 1, 1, k_isl_one<R>, lo, m, order, rs, jt, bd, rw, (const int*)row_off_.p, prm_.iterations);
            continue;
        }
        int run = 0, used = 0;
        for (int c = 0; c < kMaxColorsBig; c++) {
            start[c] = run; cur[c] = lo + run; run += cnt[c + 1];
            if (cnt[c + 1]) used = c + 1;
        }
        PE_CK(cudaMemcpyAsync(gc_cursor_.p, cur.data(), cur.size() * sizeof(int), cudaMemcpyHostToDevice, st_));
        launch(K_GC_COLOR, g, k_gc_place, lo, m, (const int*)color_.p, order, gc_cursor_.p, isl_corder_.p);
        const bool last = cnt[kMaxColorsBig] > 0;
        n_colors_ = std::max(n_colors_, std::min(used, ncol) + (last ? 1 : 0));
        // every iteration in one cooperative launch: colour lists, then the grid-wide passes
        const int top = std::min(used, kMaxColorsBig - 1);
        std::vector<int> cs(std::max(top, 1)), cc(std::max(top, 1));
        for (int c = 0; c < top; c++) { cs[c] = lo + start[c]; cc[c] = cnt[c + 1]; }
        upload(gc_cstart_, cs, st_);
        upload(gc_ccount_, cc, st_);
        launch_coop(K_GC_SOLVE, coop_blocks_, kBlock, k_gc_solve<R>, (const uint32_t*)isl_corder_.p, (const int*)gc_cstart_.p,
                    (const int*)gc_ccount_.p, top, prm_.iterations, lo, m, order, (const int*)color_.p, last ? 1 : 0, rs, jt, bd, rw,
                    (const int*)row_off_.p);
    }
}

template <class R> void World<R>::step(int n, int mode) {
    for (int s = 0; s < n; s++) {
        step_launches_ = 0;
        ev_begin(4);
        ev_begin(0); integrate(); ev_end(0);
        ev_begin(1); broadphase(); ev_end(1);
        ev_begin(2); narrowphase(); ev_end(2);
        ev_begin(3); solve(mode); ev_end(3);
        ev_end(4);
        last_step_launches_ = step_launches_;
        check_status();
    }
    resolve_prof();
}

// ------------------------------------------------------------------ transfers
// column-wise transfers: each requested field is one contiguous column of the field-major body
// array, staged through pinned host memory (these are the host<->device copies a drop-in caller pays)
template <class R> R* World<R>::staging(size_t n) {
    if (n > stage_n_) {
        if (stage_) cudaFreeHost(stage_);
        stage_ = nullptr;
        PE_CK(cudaMallocHost(&stage_, n * sizeof(R)));
        stage_n_ = n;
    }
    return stage_;
}

template <class R>
void World<R>::get_state(double* o, double* b, double* v, double* w, double* mn, double* mx, double* iw) {
    double* dst[7] = {o, b, v, w, mn, mx, iw};
    const int k0[7] = {OX, B00, VX, WX, MNX, MXX, I00}, nk[7] = {3, 9, 3, 3, 3, 3, 9};
    XferGroups G{};
    size_t tot = 0;
    int map[7];
    for (int g = 0; g < 7; g++) {
        if (!dst[g]) continue;
        map[G.n] = g;
        G.k0[G.n] = k0[g]; G.nk[G.n] = nk[g]; G.off[G.n] = tot;
        tot += (size_t)nk[g] * N_;
        G.n++;
    }
    if (!N_ || !G.n) return;
    xfer_.ensure(tot);
    launch(K_MISC, grid(N_), k_state_pack<R>, bodies(), G, xfer_.p);
    for (int q = 0; q < G.n; q++)
        PE_CK(cudaMemcpyAsync(dst[map[q]], xfer_.p + G.off[q], (size_t)G.nk[q] * N_ * sizeof(double), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
}

template <class R>
void World<R>::set_state(const double* o, const double* b, const double* v, const double* w, const double* mn, const double* mx,
                         const double* iw) {
    const double* src[7] = {o, b, v, w, mn, mx, iw};
    const int k0[7] = {OX, B00, VX, WX, MNX, MXX, I00}, nk[7] = {3, 9, 3, 3, 3, 3, 9};
    XferGroups G{};
    size_t tot = 0;
    int at[7] = {-1, -1, -1, -1, -1, -1, -1};
    for (int g = 0; g < 7; g++) {
        if (!src[g]) continue;
        at[g] = G.n;
        G.k0[G.n] = k0[g]; G.nk[G.n] = nk[g]; G.off[G.n] = tot;
        tot += (size_t)nk[g] * N_;
        G.n++;
    }
    if (!N_ || !G.n) return;
    xfer_.ensure(tot);
    for (int g = 0; g < 7; g++)
        if (src[g])
            PE_CK(cudaMemcpyAsync(xfer_.p + G.off[at[g]], src[g], (size_t)nk[g] * N_ * sizeof(double), cudaMemcpyHostToDevice, st_));
    const bool scale = mn && mx && o;   // the injected box's AABB scale
    launch(K_MISC, grid(N_), k_state_unpack<R>, bodies(), G, (const double*)xfer_.p, scale ? at[0] : -1, scale ? at[4] : -1,
           scale ? at[5] : -1);
    PE_CK(cudaStreamSynchronize(st_));
}

template <class R> void World<R>::get_axes(int* a) {
    PE_CK(cudaMemcpyAsync(a, scene_axis_.p, NS_ * sizeof(int), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
}
template <class R> void World<R>::set_axes(const int* a) {
    PE_CK(cudaMemcpyAsync(scene_axis_.p, a, NS_ * sizeof(int), cudaMemcpyHostToDevice, st_));
    PE_CK(cudaStreamSynchronize(st_));
}

template <class R> void World<R>::get_pairs(int* p) {
    if (P_) PE_CK(cudaMemcpyAsync(p, pairs_.p, (size_t)P_ * sizeof(int2), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
}

// per-scene offsets of a list grouped by scene (scene of its first body)
static std::vector<int> scene_offsets(int n, const int* a, const std::vector<int>& scene_off) {
    const int ns = (int)scene_off.size() - 1;
    std::vector<int> off(ns + 1, 0);
    int s = 0;
    for (int i = 0; i < n; i++) {
        const int b = a[i * 2];
        const int sb = (int)(std::upper_bound(scene_off.begin(), scene_off.end(), b) - scene_off.begin()) - 1;
        if (sb < s) throw std::runtime_error("list must be grouped by scene in scene order");
        while (s < sb) off[++s] = i;
    }
    while (s < ns) off[++s] = n;
    return off;
}

template <class R> void World<R>::set_pairs(int n, const int* p) {
    for (int i = 0; i < 2 * n; i++) if (p[i] < 0 || p[i] >= N_) throw std::runtime_error("pair body index out of range");
    ensure_pair_capacity(std::max(n, 1));
    if (n) PE_CK(cudaMemcpyAsync(pairs_.p, p, (size_t)n * sizeof(int2), cudaMemcpyHostToDevice, st_));
    h_pair_scene_off_ = scene_offsets(n, p, h_scene_off_);
    PE_CK(cudaMemcpyAsync(pair_scene_off_.p, h_pair_scene_off_.data(), (NS_ + 1) * sizeof(int), cudaMemcpyHostToDevice, st_));
    PE_CK(cudaStreamSynchronize(st_));
    P_ = n;
}

template <class R> void World<R>::get_results(int* a, int* b, int* ps, double* fr, double* re, double* slots) {
    const int P = R_;
    std::vector<int> ha(P), hb(P), hn(P);
    std::vector<R> hfr(P), hre(P), hd((size_t)P * kSlots), pts((size_t)NPF * pair_cap_ * kSlots);
    if (P) {
        PE_CK(cudaMemcpyAsync(ha.data(), res_a_.p, P * sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hb.data(), res_b_.p, P * sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hn.data(), res_np_.p, P * sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hfr.data(), res_fr_.p, P * sizeof(R), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hre.data(), res_re_.p, P * sizeof(R), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(hd.data(), res_dist_[cur_dist_].p, hd.size() * sizeof(R), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaMemcpyAsync(pts.data(), res_pts_.p, pts.size() * sizeof(R), cudaMemcpyDeviceToHost, st_));
    }
    PE_CK(cudaStreamSynchronize(st_));
    const size_t stride = (size_t)pair_cap_ * kSlots;
    for (int p = 0; p < P; p++) {
        if (a) a[p] = ha[p];
        if (b) b[p] = hb[p];
        if (ps) ps[p] = hn[p];
        if (fr) fr[p] = hfr[p];
        if (re) re[p] = hre[p];
        if (!slots) continue;
        for (int k = 0; k < kSlots; k++) {
            double* o = slots + ((size_t)p * kSlots + k) * 19;
            for (int q = 0; q < 19; q++) o[q] = 0;
            o[12] = hd[(size_t)p * kSlots + k];
            if (k >= hn[p]) continue;
            const size_t s = (size_t)p * kSlots + k;
            for (int g = 0; g < 4; g++) for (int d = 0; d < 3; d++) o[g * 3 + d] = pts[(size_t)(g * 3 + d) * stride + s];
            for (int g = 4; g < 6; g++) for (int d = 0; d < 3; d++) o[13 + (g - 4) * 3 + d] = pts[(size_t)(g * 3 + d) * stride + s];
        }
    }
}

template <class R>
void World<R>::set_results(int n, const int* a, const int* b, const int* ps, const double* fr, const double* re,
                           const double* slots) {
    ensure_pair_capacity(std::max(n, 1));
    std::vector<int> ab(2 * n);
    for (int i = 0; i < n; i++) {
        if (a[i] < 0 || a[i] >= N_ || b[i] < 0 || b[i] >= N_ || ps[i] < 0 || ps[i] > kSlots)
            throw std::runtime_error("result " + std::to_string(i) + " out of range");
        ab[2 * i] = a[i];
        ab[2 * i + 1] = b[i];
    }
    std::vector<int> off = scene_offsets(n, ab.data(), h_scene_off_);
    std::vector<R> hfr(n), hre(n), hd((size_t)n * kSlots), pts((size_t)NPF * pair_cap_ * kSlots, R(0));
    const size_t stride = (size_t)pair_cap_ * kSlots;
    for (int p = 0; p < n; p++) {
        hfr[p] = R(fr[p]);
        hre[p] = R(re[p]);
        for (int k = 0; k < kSlots; k++) {
            const double* o = slots + ((size_t)p * kSlots + k) * 19;
            const size_t s = (size_t)p * kSlots + k;
            hd[s] = R(o[12]);
            for (int g = 0; g < 4; g++) for (int d = 0; d < 3; d++) pts[(size_t)(g * 3 + d) * stride + s] = R(o[g * 3 + d]);
            for (int g = 4; g < 6; g++) for (int d = 0; d < 3; d++) pts[(size_t)(g * 3 + d) * stride + s] = R(o[13 + (g - 4) * 3 + d]);
        }
    }
    if (n) {
        PE_CK(cudaMemcpyAsync(res_a_.p, a, n * sizeof(int), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_b_.p, b, n * sizeof(int), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_np_.p, ps, n * sizeof(int), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_fr_.p, hfr.data(), n * sizeof(R), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_re_.p, hre.data(), n * sizeof(R), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_dist_[cur_dist_].p, hd.data(), hd.size() * sizeof(R), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(res_pts_.p, pts.data(), pts.size() * sizeof(R), cudaMemcpyHostToDevice, st_));
    }
    PE_CK(cudaMemcpyAsync(res_scene_off_.p, off.data(), (NS_ + 1) * sizeof(int), cudaMemcpyHostToDevice, st_));
    PE_CK(cudaStreamSynchronize(st_));
    R_ = n;
}

// ------------------------------------------------------------------ serving: scene repacking
namespace {
// kept bodies: field-major gather from the old layout (stride ocap) into the new one (stride ncap)
// scene whose [off[s], off[s + 1]) holds r (the last such s when empty scenes share an offset)
__device__ __forceinline__ int segment_of(const int* off, int ns, int r) {
    int lo = 0, hi = ns;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= r) lo = mid;
        else hi = mid;
    }
    return lo;
}
template <class R>
__global__ void k_repack_bodies(const R* of, int ocap, const int* oshape, const int* oflags, R* nf, int ncap, int* nshape,
                                int* nflags, const int* koff, const int* first, int nk, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int s = segment_of(koff, nk, j);
    const int i = first[s] + j - koff[s];
    for (int k = 0; k < NBF; k++) nf[(size_t)k * ncap + j] = of[(size_t)k * ocap + i];
    nshape[j] = oshape[i];
    nflags[j] = oflags[i];
}
// added bodies: a compact field-major block [NBF x n] placed at new index `at`
template <class R>
__global__ void k_place_bodies(const R* blk, int n, R* nf, int ncap, int at) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    for (int k = 0; k < NBF; k++) nf[(size_t)k * ncap + at + j] = blk[(size_t)k * n + j];
}
// contact-result distance pools: slot t of the new pool comes from the kept scene's old segment
template <class R>
__global__ void k_repack_pool(const R* src, R* dst, const int* new_off, const int* old_start, int ns, int n_slots) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_slots) return;
    const int r = t / kSlots, k = t - r * kSlots;
    const int lo = segment_of(new_off, ns, r);
    dst[t] = src[(size_t)(old_start[lo] + r - new_off[lo]) * kSlots + k];
}
}  // namespace

template <class R>
void World<R>::repack(const int* keep, int n_keep, const SceneData* const* adds, int n_add) {
    PE_CK(cudaStreamSynchronize(st_));
    const int ons = NS_;
    std::vector<int> old_res(ons + 1, 0), old_axis(std::max(ons, 1), 0);
    PE_CK(cudaMemcpy(old_res.data(), res_scene_off_.p, (ons + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    PE_CK(cudaMemcpy(old_axis.data(), scene_axis_.p, ons * sizeof(int), cudaMemcpyDeviceToHost));
    for (int k = 0; k < n_keep; k++)
        if (keep[k] < 0 || keep[k] >= ons) throw std::runtime_error("repack: kept scene index out of range");
    // shapes of the added scenes go to the end of the shape tables
    std::vector<std::vector<int>> smap(n_add);
    for (int a = 0; a < n_add; a++) {
        const SceneData& d = *adds[a];
        for (int sh : d.body_shape)
            if (sh < 0 || sh >= d.n_shapes()) throw std::runtime_error("repack: body shape index out of range");
        append_shapes(d.n_shapes(), d.shape_type.data(), d.shape_param.data(), d.hull_vbeg.data(), d.hull_vcnt.data(),
                      d.hull_fbeg.data(), d.hull_fcnt.data(), d.hull_verts.data(), d.hull_face_off.data(), d.hull_face_idx.data(),
                      &smap[a]);
    }
    // new body layout: kept scenes in order (first old body of each), then the added ones
    std::vector<int> off(1, 0), first;
    for (int k = 0; k < n_keep; k++) {
        const int s = keep[k];
        first.push_back(h_scene_off_[s]);
        off.push_back(off.back() + h_scene_off_[s + 1] - h_scene_off_[s]);
    }
    const int n_kept = off.back();
    int n_new = 0;
    for (int a = 0; a < n_add; a++) { n_new += adds[a]->n_bodies(); off.push_back(n_kept + n_new); }
    const int N = n_kept + n_new, ncap = std::max(N, 1);
    std::vector<R> blk((size_t)NBF * std::max(n_new, 1), R(0));
    std::vector<int> ashape(std::max(n_new, 1)), aflags(std::max(n_new, 1));
    for (int a = 0, j = 0; a < n_add; a++) {
        const SceneData& d = *adds[a];
        for (int i = 0; i < d.n_bodies(); i++, j++) {
            ashape[j] = smap[a][d.body_shape[i]];
            aflags[j] = d.body_flags[i];
            fill_body(blk.data(), n_new, j, ashape[j], d.mass[i], d.friction[i], d.restitution[i], d.lin_damp[i], d.ang_damp[i],
                      &d.origin[(size_t)i * 3], &d.basis[(size_t)i * 9], &d.lin_vel[(size_t)i * 3], &d.ang_vel[(size_t)i * 3]);
        }
    }
    DBuf<R> nf;
    DBuf<int> nshape, nflags, dkoff, dfirst;
    nf.ensure((size_t)NBF * ncap);
    nshape.ensure(ncap + 1);
    nflags.ensure(ncap + 1);
    if (n_kept) {
        upload(dkoff, std::vector<int>(off.begin(), off.begin() + n_keep + 1), st_);
        upload(dfirst, first, st_);
        launch(K_MISC, grid(n_kept), k_repack_bodies<R>, (const R*)bf_.p, bcap_, (const int*)bshape_.p, (const int*)bflags_.p, nf.p,
               ncap, nshape.p, nflags.p, (const int*)dkoff.p, (const int*)dfirst.p, n_keep, n_kept);
    }
    DBuf<R> dblk;
    if (n_new) {
        upload(dblk, blk, st_);
        launch(K_MISC, grid(n_new), k_place_bodies<R>, (const R*)dblk.p, n_new, nf.p, ncap, n_kept);
        PE_CK(cudaMemcpyAsync(nshape.p + n_kept, ashape.data(), n_new * sizeof(int), cudaMemcpyHostToDevice, st_));
        PE_CK(cudaMemcpyAsync(nflags.p + n_kept, aflags.data(), n_new * sizeof(int), cudaMemcpyHostToDevice, st_));
    }
    // contact-result pools of the kept scenes (the current generation becomes the next step's "previous")
    const int ns = n_keep + n_add;
    std::vector<int> new_res(ns + 1, 0), old_start(std::max(ns, 1), 0), axis(std::max(ns, 1), 0);
    for (int k = 0; k < n_keep; k++) {
        const int s = keep[k];
        new_res[k + 1] = new_res[k] + old_res[s + 1] - old_res[s];
        old_start[k] = old_res[s];
        axis[k] = old_axis[s];
    }
    for (int a = 0; a < n_add; a++) new_res[n_keep + a + 1] = new_res[n_keep + a];
    const int T = new_res[ns];
    ensure_pair_capacity(std::max(T, 1));   // grows both pool generations keeping their contents
    if (T) {
        DBuf<int> dnew, dold;
        upload(dnew, new_res, st_);
        upload(dold, old_start, st_);
        launch(K_MISC, grid(T * kSlots), k_repack_pool<R>, (const R*)res_dist_[cur_dist_].p, res_dist_[cur_dist_ ^ 1].p,
               (const int*)dnew.p, (const int*)dold.p, ns, T * kSlots);
        PE_CK(cudaStreamSynchronize(st_));
        cur_dist_ ^= 1;
    }
    PE_CK(cudaStreamSynchronize(st_));
    std::swap(bf_.p, nf.p); std::swap(bf_.n, nf.n);
    std::swap(bshape_.p, nshape.p); std::swap(bshape_.n, nshape.n);
    std::swap(bflags_.p, nflags.p); std::swap(bflags_.n, nflags.n);
    N_ = N;
    bcap_ = ncap;
    claim_.ensure(N + 1);
    // scene tables (as set_scenes), then the kept axes and result offsets
    NS_ = std::max(ns, 1);
    if (ns == 0) off = {0, 0};
    h_scene_off_ = off;
    build_axis_items();
    std::vector<int> sc(std::max(N, 1), 0);
    for (int s = 0; s < ns; s++) for (int i = off[s]; i < off[s + 1]; i++) sc[i] = s;
    upload(bscene_, sc, st_);
    upload(scene_off_, off, st_);
    upload(scene_axis_, axis, st_);
    if (ns == 0) new_res = {0, 0};
    std::vector<int> zero(NS_ + 1, 0);
    upload(pair_scene_off_, zero, st_);
    upload(prev_res_off_, zero, st_);
    upload(res_scene_off_, new_res, st_);
    h_pair_scene_off_ = zero;
    P_ = 0;
    R_ = 0;
    PE_CK(cudaStreamSynchronize(st_));
}

template <class R>
void World<R>::get_state_range(int first, int count, double* o, double* b, double* v, double* w) {
    if (first < 0 || count < 0 || first + count > N_) throw std::runtime_error("state range out of bounds");
    if (!count) return;
    // fields OX..WZ (origin, basis, linear and angular velocity) are 18 consecutive field rows
    R* h = staging((size_t)18 * count);
    PE_CK(cudaMemcpy2DAsync(h, (size_t)count * sizeof(R), bf_.p + first, (size_t)bcap_ * sizeof(R), (size_t)count * sizeof(R), 18,
                            cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
    struct G { double* dst; int k0; int nk; };
    const G groups[4] = {{o, OX, 3}, {b, B00, 9}, {v, VX, 3}, {w, WX, 3}};
    for (const G& g : groups) {
        if (!g.dst) continue;
        for (int k = 0; k < g.nk; k++)
            for (int i = 0; i < count; i++) g.dst[(size_t)i * g.nk + k] = (double)h[(size_t)(g.k0 + k) * count + i];
    }
}

} // namespace pe
