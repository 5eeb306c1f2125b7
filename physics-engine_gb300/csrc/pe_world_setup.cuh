// World<R> member definitions, part 1: lifetime, device views, and the setup calls (shapes,
// compounds, joints, ignored pairs, bodies, scenes, parameters).
#pragma once
#include <algorithm>
#include "pe_world.cuh"

namespace pe {

template <class R> World<R>::World(int device) : dev_(device) {
    PE_CK(cudaSetDevice(dev_));
    PE_CK(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    for (int k = 0; k < kSideStreams; k++) {
        PE_CK(cudaStreamCreateWithFlags(&side_[k], cudaStreamNonBlocking));
        PE_CK(cudaEventCreateWithFlags(&join_ev_[k], cudaEventDisableTiming));
    }
    PE_CK(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming));
    for (auto& e : ev_) { PE_CK(cudaEventCreate(&e[0])); PE_CK(cudaEventCreate(&e[1])); }
    UnitMeshes u;
    std::memset(&u, 0, sizeof(u));
    build_unit_meshes(u);
    PE_CK(cudaMemcpyToSymbol(g_unit, &u, sizeof(u)));
    status_.ensure(1);
    PE_CK(cudaMemset(status_.p, 0, sizeof(int)));
    total_.ensure(1);
    rows_total_.ensure(1);
    dcnt_.ensure(DC_COUNT);
    PE_CK(cudaMemset(dcnt_.p, 0, DC_COUNT * sizeof(int)));
    std::memset(gsig_, 0, sizeof gsig_);
    std::memset(&last_sig_, 0xff, sizeof last_sig_);
    std::memset(&gsig_head_, 0, sizeof gsig_head_);
    std::memset(&last_sig_head_, 0xff, sizeof last_sig_head_);
    dstat_.ensure(HS_COUNT);
    PE_CK(cudaMallocHost(&hstat_, HS_COUNT * sizeof(int)));
    std::memset(hstat_, 0, HS_COUNT * sizeof(int));
    set_scenes(1, nullptr);
}

template <class R> World<R>::~World() {
    if (st_) cudaStreamSynchronize(st_);
    if (stage_) cudaFreeHost(stage_);
    if (hstat_) cudaFreeHost(hstat_);
    for (auto& m : gexec_) for (auto& g : m) if (g) cudaGraphExecDestroy(g);
    if (ghead_) cudaGraphExecDestroy(ghead_);
    for (auto& q : pending_) { cudaEventDestroy(q.e0); cudaEventDestroy(q.e1); }
    for (auto e : ev_pool_) cudaEventDestroy(e);
    for (auto& e : ev_) { cudaEventDestroy(e[0]); cudaEventDestroy(e[1]); }
    for (int k = 0; k < kSideStreams; k++) {
        if (side_[k]) { cudaStreamSynchronize(side_[k]); cudaStreamDestroy(side_[k]); }
        if (join_ev_[k]) cudaEventDestroy(join_ev_[k]);
    }
    if (fork_ev_) cudaEventDestroy(fork_ev_);
    if (st_) cudaStreamDestroy(st_);
}

// phase events; inside a graph capture they become event-record nodes of the graph
template <class R> void World<R>::ev_begin(int k) {
    PE_CK(cudaEventRecordWithFlags(ev_[k][0], st_, capturing_ ? cudaEventRecordExternal : cudaEventRecordDefault));
    ev_open_[k] = true;
}
template <class R> void World<R>::ev_end(int k) {
    PE_CK(cudaEventRecordWithFlags(ev_[k][1], st_, capturing_ ? cudaEventRecordExternal : cudaEventRecordDefault));
    ev_open_[k] = false;
}
// the phases' durations, once the step's last event has completed (one wait per step)
template <class R> void World<R>::ev_collect() {
    PE_CK(cudaEventSynchronize(ev_[4][1]));
    for (int k = 0; k < 5; k++) {
        float ms = 0;
        PE_CK(cudaEventElapsedTime(&ms, ev_[k][0], ev_[k][1]));
        ms_[k] += ms;
    }
}
template <class R> void World<R>::phase_times(double* ms, bool reset) {
    for (int k = 0; k < 5; k++) ms[k] = ms_[k];
    if (reset) for (double& m : ms_) m = 0;
}
template <class R> void World<R>::last_counts(int* c) {
    c[0] = P_; c[1] = n_active_; c[2] = n_rows_; c[3] = n_colors_; c[4] = (int)last_step_launches_; c[5] = n_islands_;
}

template <class R> ShapeTable<R> World<R>::shapes() const {
    ShapeTable<R> t;
    t.type = stype_.p; t.param = sparam_.p; t.hull = shull_.p;
    t.h_vbeg = hvbeg_.p; t.h_vcnt = hvcnt_.p; t.h_fbeg = hfbeg_.p; t.h_fcnt = hfcnt_.p; t.h_ebeg = hebeg_.p; t.h_ecnt = hecnt_.p;
    t.h_rad = hrad_.p;
    t.hv = hv_.p; t.f_off = hfoff_.p; t.f_idx = hfidx_.p; t.f_n = hfn_.p; t.f_min = hfmin_.p; t.f_max = hfmax_.p;
    t.e_a = hea_.p; t.e_b = heb_.p; t.e_d = hed_.p;
    t.c_beg = cbeg_.p; t.c_cnt = ccnt_.p; t.c_shape = cshape_.p; t.c_xf = cxf_.p;
    t.h_lbeg = hlbeg_.p; t.h_lcnt = hlcnt_.p; t.lf_beg = lfbeg_.p; t.lf_cnt = lfcnt_.p; t.lf_min = lfmin_.p; t.lf_max = lfmax_.p;
    t.margin = margin_;
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
    const int n_edges = (int)(h_ea_.size() / 3);
    hed_.ensure((size_t)std::max(n_edges, 1) * 3);
    if (n_edges > 0) launch(K_MISC, grid(n_edges), k_hull_edge_dirs<R>, n_edges, (const R*)hea_.p, (const R*)heb_.p, hed_.p);
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
    PE_CK(cudaMemsetAsync(dcnt_.p, 0, DC_COUNT * sizeof(int), st_));
    PE_CK(cudaStreamSynchronize(st_));
}


template <class R> void World<R>::set_params(double dt, double gx, double gy, double gz, int iters) {
    prm_.dt = dt; prm_.g[0] = gx; prm_.g[1] = gy; prm_.g[2] = gz; prm_.iterations = iters;
}

} // namespace pe
