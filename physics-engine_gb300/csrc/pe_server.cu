// Serving: a request loop over one device-resident world.  Requests (a scene and a number of steps)
// queue on arrival; before each batched step the loop retires finished requests (their final state
// is read back), admits queued requests in arrival order while their estimated device footprint
// fits the budget, and repacks the world so that the live scenes are contiguous.  Live scenes keep
// their state, sweep axes and contact-result pools on the device between steps, and each step
// advances all of them in one batched launch sequence, so a scene's result is the one it gets
// stepped alone.
#include <algorithm>
#include <cmath>
#include <deque>
#include <memory>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>
#include "../../include/pe_gpu.h"
#include "pe_world.cuh"

namespace pe {

class Server {
public:
    Server(int real_bits, int device, double dt, double gx, double gy, double gz, int iterations, int mode, double budget)
        : mode_(mode), budget_(budget) {
        if (real_bits == 32) w_.reset(new World<float>(device));
        else w_.reset(new World<double>(device));
        w_->set_shapes(0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, nullptr, 0, nullptr, nullptr);
        w_->set_bodies(0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
        w_->set_params(dt, gx, gy, gz, iterations);
        r_ = real_bits / 8;
    }

    // Device bytes a live scene is charged: body state (55 reals + ints), broadphase temporaries, and
    // room for 6 pairs (result records with 8 contact slots of 18 reals and two distance pools) and
    // 6 solver rows of 23 reals per body.
    double footprint(const SceneData& d) const {
        const double r = r_;
        const double per_body = NBF * r + 64 + 6 * (40 + kSlots * (NPF + 2) * r) + 6 * NRF * r;
        return d.n_bodies() * per_body + d.hull_verts.size() * r * 4 + d.n_shapes() * 32.0;
    }

    long long submit(SceneData&& d, int k_steps) {
        const long long id = next_id_++;
        Req& q = reqs_[id];
        q.k = k_steps;
        q.bytes = footprint(d);
        q.d = std::move(d);
        if (q.bytes > budget_) { q.state = 3; q.d = SceneData(); return id; }   // can never fit
        queue_.push_back(id);
        return id;
    }

    void step(int* n_live, int* n_queued) {
        const std::vector<int> off = w_->scene_body_offsets();
        std::vector<int> keep;
        std::vector<long long> still;
        bool changed = false;
        for (size_t k = 0; k < live_.size(); k++) {
            Req& q = reqs_[live_[k]];
            if (q.done >= q.k) {   // retire: read the final state back
                const int n = off[k + 1] - off[k];
                q.o.resize((size_t)n * 3); q.b.resize((size_t)n * 9); q.v.resize((size_t)n * 3); q.w.resize((size_t)n * 3);
                w_->get_state_range(off[k], n, q.o.data(), q.b.data(), q.v.data(), q.w.data());
                q.state = 2;
                used_ -= q.bytes;
                finished_++;
                changed = true;
            } else {
                keep.push_back((int)k);
                still.push_back(live_[k]);
            }
        }
        std::vector<const SceneData*> adds;
        std::vector<long long> added;
        while (!queue_.empty()) {   // admission in arrival order, by footprint
            Req& q = reqs_[queue_.front()];
            if (used_ + q.bytes > budget_) break;
            used_ += q.bytes;
            q.state = 1;
            adds.push_back(&q.d);
            added.push_back(queue_.front());
            queue_.pop_front();
            admitted_++;
        }
        if (changed || !adds.empty()) {
            w_->repack(keep.data(), (int)keep.size(), adds.data(), (int)adds.size());
            live_ = still;
            live_.insert(live_.end(), added.begin(), added.end());
            for (long long id : added) reqs_[id].d = SceneData();   // uploaded: free the host copy
        }
        peak_used_ = std::max(peak_used_, used_);
        if (!live_.empty()) {
            double a[5], b[5];
            w_->phase_times(a, false);
            w_->step(1, mode_);
            w_->phase_times(b, false);
            step_ms_.push_back(b[4] - a[4]);
            body_steps_ += w_->n_bodies();
            for (long long id : live_) reqs_[id].done++;
        }
        *n_live = (int)live_.size();
        *n_queued = (int)queue_.size();
    }

    // 0 queued, 1 running, 2 done (state copied out, request released), 3 rejected (never fits)
    int result(long long id, double* o, double* b, double* v, double* w) {
        auto it = reqs_.find(id);
        if (it == reqs_.end()) throw std::runtime_error("unknown request id (a finished request is released when fetched)");
        Req& q = it->second;
        const int st = q.state;
        if (st == 2) {
            if (o) std::copy(q.o.begin(), q.o.end(), o);
            if (b) std::copy(q.b.begin(), q.b.end(), b);
            if (v) std::copy(q.v.begin(), q.v.end(), v);
            if (w) std::copy(q.w.begin(), q.w.end(), w);
        }
        if (st == 2 || st == 3) reqs_.erase(it);
        return st;
    }

    void stats(double* out) const {
        std::vector<double> t = step_ms_;
        std::sort(t.begin(), t.end());
        auto pct = [&](double p) { return t.empty() ? 0.0 : t[std::min(t.size() - 1, (size_t)std::floor(p * (t.size() - 1) + 0.5))]; };
        double sum = 0;
        for (double x : t) sum += x;
        out[0] = pct(0.5);
        out[1] = pct(0.99);
        out[2] = t.empty() ? 0.0 : sum / t.size();
        out[3] = (double)t.size();
        out[4] = (double)body_steps_;
        out[5] = (double)admitted_;
        out[6] = (double)finished_;
        out[7] = peak_used_;
        out[8] = (double)live_.size();
        out[9] = (double)queue_.size();
    }

private:
    struct Req {
        SceneData d;
        int k = 0, done = 0, state = 0;
        double bytes = 0;
        std::vector<double> o, b, v, w;
    };
    std::unique_ptr<WorldBase> w_;
    int mode_, r_ = 4;
    double budget_, used_ = 0, peak_used_ = 0;
    long long next_id_ = 1, body_steps_ = 0, admitted_ = 0, finished_ = 0;
    std::unordered_map<long long, Req> reqs_;
    std::deque<long long> queue_;
    std::vector<long long> live_;
    std::vector<double> step_ms_;
};

}  // namespace pe

struct pe_gpu_server {
    pe::Server* s = nullptr;
    std::string err;
};

namespace {
template <class F> int sguard(pe_gpu_server* h, F&& f) {
    if (!h || !h->s) return PE_GPU_ERR_ARG;
    try {
        h->err.clear();
        return f(*h->s);
    } catch (const pe::CudaError& e) {
        h->err = e.what();
        return PE_GPU_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        h->err = "host allocation failed";
        return PE_GPU_ERR_CAPACITY;
    } catch (const std::exception& e) {
        h->err = e.what();
        return PE_GPU_ERR_STATE;
    }
}
}  // namespace

extern "C" {

int pe_gpu_server_create(const pe_gpu_config* cfg, double dt, double gx, double gy, double gz, int iterations, int solver_mode,
                         double hbm_budget_bytes, pe_gpu_server** out) {
    if (!cfg || !out || (cfg->real_bits != 32 && cfg->real_bits != 64) || iterations < 0 || hbm_budget_bytes <= 0 ||
        (solver_mode != PE_GPU_SOLVER_SERIAL_ORDER && solver_mode != PE_GPU_SOLVER_COLORED))
        return PE_GPU_ERR_ARG;
    *out = nullptr;
    auto* h = new (std::nothrow) pe_gpu_server();
    if (!h) return PE_GPU_ERR_CAPACITY;
    try {
        h->s = new pe::Server(cfg->real_bits, cfg->device, dt, gx, gy, gz, iterations, solver_mode, hbm_budget_bytes);
    } catch (...) {
        delete h;
        return PE_GPU_ERR_CUDA;
    }
    *out = h;
    return PE_GPU_OK;
}

int pe_gpu_server_destroy(pe_gpu_server* h) {
    if (!h) return PE_GPU_ERR_ARG;
    delete h->s;
    delete h;
    return PE_GPU_OK;
}

const char* pe_gpu_server_last_error(const pe_gpu_server* h) { return h ? h->err.c_str() : "null handle"; }

int pe_gpu_server_submit(pe_gpu_server* h, const pe_gpu_scene* sc, int n_steps, long long* id) {
    return sguard(h, [&](pe::Server& s) {
        // a request steps its scene at least once: a zero-step request would still be advanced by
        // the batched step that admits it
        if (!sc || !id || n_steps < 1 || sc->n_shapes < 0 || sc->n_bodies < 0) return PE_GPU_ERR_ARG;
        pe::SceneData d;
        const int S = sc->n_shapes, N = sc->n_bodies;
        d.shape_type.assign(sc->shape_type, sc->shape_type + S);
        d.shape_param.assign(sc->shape_param, sc->shape_param + 3 * S);
        d.hull_vbeg.assign(sc->hull_vbeg, sc->hull_vbeg + S);
        d.hull_vcnt.assign(sc->hull_vcnt, sc->hull_vcnt + S);
        d.hull_fbeg.assign(sc->hull_fbeg, sc->hull_fbeg + S);
        d.hull_fcnt.assign(sc->hull_fcnt, sc->hull_fcnt + S);
        if (sc->n_hull_verts > 0) d.hull_verts.assign(sc->hull_verts, sc->hull_verts + 3 * (size_t)sc->n_hull_verts);
        if (sc->n_hull_faces > 0) {
            d.hull_face_off.assign(sc->hull_face_off, sc->hull_face_off + sc->n_hull_faces + 1);
            d.hull_face_idx.assign(sc->hull_face_idx, sc->hull_face_idx + sc->hull_face_off[sc->n_hull_faces]);
        }
        for (int k = 0; k < S; k++)
            if (d.shape_type[k] == PE_GPU_SHAPE_CONVEX_MESH &&
                (d.hull_vbeg[k] < 0 || d.hull_vbeg[k] + d.hull_vcnt[k] > sc->n_hull_verts || d.hull_fbeg[k] < 0 ||
                 d.hull_fbeg[k] + d.hull_fcnt[k] > sc->n_hull_faces))
                return PE_GPU_ERR_ARG;
        d.body_shape.assign(sc->body_shape, sc->body_shape + N);
        d.body_flags.assign(sc->body_flags, sc->body_flags + N);
        d.mass.assign(sc->mass, sc->mass + N);
        d.friction.assign(sc->friction, sc->friction + N);
        d.restitution.assign(sc->restitution, sc->restitution + N);
        d.lin_damp.assign(sc->lin_damp, sc->lin_damp + N);
        d.ang_damp.assign(sc->ang_damp, sc->ang_damp + N);
        d.origin.assign(sc->origin, sc->origin + 3 * (size_t)N);
        d.basis.assign(sc->basis, sc->basis + 9 * (size_t)N);
        d.lin_vel.assign(sc->lin_vel, sc->lin_vel + 3 * (size_t)N);
        d.ang_vel.assign(sc->ang_vel, sc->ang_vel + 3 * (size_t)N);
        for (int i = 0; i < N; i++)
            if (d.body_shape[i] < 0 || d.body_shape[i] >= S) return PE_GPU_ERR_ARG;
        *id = s.submit(std::move(d), n_steps);
        return PE_GPU_OK;
    });
}

int pe_gpu_server_step(pe_gpu_server* h, int* n_live, int* n_queued) {
    return sguard(h, [&](pe::Server& s) {
        int a = 0, b = 0;
        s.step(&a, &b);
        if (n_live) *n_live = a;
        if (n_queued) *n_queued = b;
        return PE_GPU_OK;
    });
}

int pe_gpu_server_result(pe_gpu_server* h, long long id, int* state, double* origin, double* basis, double* lin_vel,
                         double* ang_vel) {
    return sguard(h, [&](pe::Server& s) {
        const int st = s.result(id, origin, basis, lin_vel, ang_vel);
        if (state) *state = st;
        return PE_GPU_OK;
    });
}

int pe_gpu_server_stats(pe_gpu_server* h, double* out10) {
    return sguard(h, [&](pe::Server& s) {
        if (!out10) return PE_GPU_ERR_ARG;
        s.stats(out10);
        return PE_GPU_OK;
    });
}

}  // extern "C"
