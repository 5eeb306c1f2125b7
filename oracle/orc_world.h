// Oracle world: rigid bodies and the four phases of pe_intf::World::step()
// (src/intf/world.cpp:267-300 in the reference's numbering; see each function).
// Test infrastructure only: the CPU restatement that checks the GPU path and that is
// timed as the CPU baseline.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>
#include "orc_collide.h"
#include "orc_joints.h"

namespace orc {

// Fork/join pool with the reference's batching (src/utils/thread_pool.h:85-102):
// batch = count / threads / 2 + 1, batches handed to persistent workers.
class Pool {
public:
    explicit Pool(int n) : n_(n < 1 ? 1 : n) {
        for (int i = 1; i < n_; i++) workers_.emplace_back([this] { loop(); });
    }
    ~Pool() {
        { std::lock_guard<std::mutex> g(m_); stop_ = true; }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }
    int size() const { return n_; }
    void for_loop(int count, const std::function<void(int)>& fn) {
        if (count <= 0) return;
        if (n_ == 1) { for (int i = 0; i < count; i++) fn(i); return; }
        const int batch = count / n_ / 2 + 1;
        {
            std::lock_guard<std::mutex> g(m_);
            fn_ = &fn; count_ = count; batch_ = batch; next_.store(0); pending_ = (count + batch - 1) / batch;
            gen_++;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(m_);
        done_cv_.wait(lk, [&] { return pending_ == 0; });
        fn_ = nullptr;
    }

private:
    void work() {
        for (;;) {
            const int b = next_.fetch_add(1);
            const int lo = b * batch_;
            if (lo >= count_) return;
            const int hi = std::min(count_, lo + batch_);
            for (int i = lo; i < hi; i++) (*fn_)(i);
            std::lock_guard<std::mutex> g(m_);
            if (--pending_ == 0) done_cv_.notify_all();
        }
    }
    void loop() {
        long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }
    int n_;
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)>* fn_ = nullptr;
    int count_ = 0, batch_ = 1, pending_ = 0;
    std::atomic<int> next_{0};
    long gen_ = 0;
    bool stop_ = false;
};

template <class R> struct Body {
    int shape = 0;
    bool kinematic = false;
    bool ignore_collision = false;
    std::vector<int> ignore_ids;   // RigidBody::_ignore_collision_ids, as body indices
    R mass = 1, inv_mass = 1, friction = R(0.5), restitution = R(0.5), lin_damp = 0, ang_damp = 0;
    M3<R> local_inv_inertia = M3<R>::identity(), world_inv_inertia = M3<R>::identity();
    Transform<R> t;
    V3<R> v, w, tv, tw;   // tv/tw: solver's temporary velocities (zero-initialised like the reference)
    V3<R> aabb_min, aabb_max;
};

// friction_contact_constraint.h:10-24
template <class R> struct Row {
    V3<R> ra, rb, n, t0, t1;
    R n_rhs = 0, n_jmj = 0, t0_jmj = 0, t1_jmj = 0, n_acc = 0, t0_acc = 0, t1_acc = 0, mu = 0;
};

template <class R> class World {
public:
    std::vector<Shape<R>> shapes;
    std::vector<Body<R>> bodies;
    R dt = R(0.01);
    V3<R> gravity = V3<R>(0, R(-9.8), 0);
    int iterations = 10;
    int axis = 0;                           // BroadPhaseSweepAndPrune::_target_axis
    R margin = 0;                           // contact margin, PE_MARGIN (phys_general.h:45)
    bool stable_ties = false;               // broadphase ties in body order (std::stable_sort)
    std::vector<std::pair<int, int>> pairs;
    std::vector<CResult<R>> results;        // pooled: slots survive between steps (stale distances)
    std::vector<std::vector<Row<R>>> rows;
    std::vector<Joint<R>> joints;           // World::_constraints (joint constraints, in order)
    Pool* pool = nullptr;

    void for_loop(int n, const std::function<void(int)>& f) { if (pool) pool->for_loop(n, f); else for (int i = 0; i < n; i++) f(i); }

    R aabb_scale(const Body<R>& b) const {   // rigidbody.cpp:119-123
        const R sc = norm(b.aabb_max - b.aabb_min);
        const R df = norm(b.aabb_max + b.aabb_min - b.t.origin * R(2));
        return (sc + df) * R(0.5);
    }

    void update_world_inertia(Body<R>& b) {   // rigidbody.cpp:43-46
        b.world_inv_inertia = mmt_r2l(mm(b.t.basis, b.local_inv_inertia), b.t.basis);
    }

    // RigidBody::setMass then setCollisionShape then setTransform (rigidbody.cpp:11-46)
    void init_body(Body<R>& b, R mass, const M3<R>& basis, const V3<R>& origin) {
        b.mass = mass;
        b.inv_mass = mass > kEps<R>() ? R(1.0) / mass : 0;
        const M3<R> li = mscale(shapes[b.shape].local_inertia, mass);
        b.local_inv_inertia = mass > kEps<R>() ? inverse3(li) : M3<R>();
        b.t.basis = basis;
        b.t.origin = origin;
        update_world_inertia(b);
    }

    // ---------------------------------------------------------------- phase 1
    // World::updateObjectStatus (world.cpp:35-119) + applyExternalForce (:121-127)
    void integrate() {
        for_loop((int)bodies.size(), [&](int i) {
            Body<R>& b = bodies[i];
            const Shape<R>& s = shapes[b.shape];
            if (b.kinematic) { get_aabb(s, b.t, b.aabb_min, b.aabb_max); return; }
            // RigidBody::step (rigidbody.cpp:207-243)
            b.t.origin = b.t.origin + b.v * dt;
            Quat<R> q = quat_from_basis(b.t.basis);
            const V3<R> dr = b.w * dt * R(0.5);
            Quat<R> d0; d0.w = 0; d0.x = dr.x; d0.y = dr.y; d0.z = dr.z;
            const Quat<R> dq = quat_mul(d0, q);
            Quat<R> qn; qn.w = q.w + dq.w; qn.x = q.x + dq.x; qn.y = q.y + dq.y; qn.z = q.z + dq.z;
            quat_normalize(qn);
            b.t.basis = quat_to_basis(qn);
            update_world_inertia(b);
            get_aabb(s, b.t, b.aabb_min, b.aabb_max);
            // RigidBody::applyDamping (rigidbody.cpp:201-204)
            b.v = b.v * R(std::pow(R(1.0) - b.lin_damp, dt));
            b.w = b.w * R(std::pow(R(1.0) - b.ang_damp, dt));
        });
        for (auto& b : bodies) {   // serial, like the reference
            if (b.kinematic) continue;
            const V3<R> force = V3<R>(0, 0, 0) + gravity * b.mass;
            b.v = b.v + force * b.inv_mass * dt;
            b.w = b.w + mv(b.world_inv_inertia, V3<R>(0, 0, 0) * dt);
        }
    }

    // ---------------------------------------------------------------- phase 2
    // BroadPhaseBase::validateCollisionPair (broad_phase_base.cpp:5-19)
    bool validate(int i, int j) const {
        const Body<R>& a = bodies[i];
        const Body<R>& b = bodies[j];
        if (a.ignore_collision || b.ignore_collision) return false;
        if (a.kinematic && b.kinematic) return false;
        if (i == j) return false;
        for (int k : a.ignore_ids) if (k == j) return false;
        for (int k : b.ignore_ids) if (k == i) return false;
        if (a.aabb_min.x > b.aabb_max.x || b.aabb_min.x > a.aabb_max.x) return false;
        if (a.aabb_min.y > b.aabb_max.y || b.aabb_min.y > a.aabb_max.y) return false;
        if (a.aabb_min.z > b.aabb_max.z || b.aabb_min.z > a.aabb_max.z) return false;
        return true;
    }

    // BroadPhaseSweepAndPrune::calcCollisionPairs (broad_phase_sweep_and_prune.cpp:6-41)
    void broadphase() {
        const int n = (int)bodies.size();
        if (n < 2) return;
        pairs.clear();
        std::vector<int> order(n);
        for (int i = 0; i < n; i++) order[i] = i;
        const int ax = axis;
        auto by_min = [&](int a, int b) { return bodies[a].aabb_min[ax] < bodies[b].aabb_min[ax]; };
        // the reference sorts with std::sort, whose order among equal keys is unspecified; the
        // stable variant (ties in body order) is the other valid order this oracle can take
        if (stable_ties) std::stable_sort(order.begin(), order.end(), by_min);
        else std::sort(order.begin(), order.end(), by_min);
        V3<R> s(0, 0, 0), s2(0, 0, 0);
        for (int i = 0; i < n; i++) {
            const Body<R>& b1 = bodies[order[i]];
            const V3<R> c = (b1.aabb_min + b1.aabb_max) * R(0.5);
            s = s + c;
            s2 = s2 + cmul(c, c);
            for (int j = i + 1; j < n; j++) {
                const Body<R>& b2 = bodies[order[j]];
                if (b2.aabb_min[ax] > b1.aabb_max[ax]) break;
                if (validate(order[i], order[j])) pairs.emplace_back(order[i], order[j]);
            }
        }
        const V3<R> v = s2 - cmul(s, s) / R(n);
        axis = 0;
        if (v.y > v.x) axis = 1;
        if (v.z > v[axis]) axis = 2;
    }

    // ---------------------------------------------------------------- phase 3
    // SimpleNarrowPhase::calcContactResults (simple_narrow_phase.cpp:7-63)
    void narrowphase() {
        results.resize(pairs.size());   // new slots are fresh, surviving slots keep stale distances
        for_loop((int)pairs.size(), [&](int i) {
            CResult<R>& r = results[i];
            r.clear();
            const int ia = pairs[i].first, ib = pairs[i].second;
            r.a = ia; r.b = ib;
            const Body<R>& A = bodies[ia];
            const Body<R>& B = bodies[ib];
            r.friction = std::sqrt(A.friction * B.friction);       // contact_result.cpp:80-86
            r.restitution = std::sqrt(A.restitution * B.restitution);
            PairCtx<R> c;
            c.sa = &shapes[A.shape]; c.sb = &shapes[B.shape];
            c.ta = &A.t; c.tb = &B.t;
            c.A = {&A.t, aabb_scale(A)};
            c.B = {&B.t, aabb_scale(B)};
            c.ref_scale = (c.A.aabb_scale + c.B.aabb_scale) * R(0.05);
            c.margin = margin;
            c.res = &r;
            collide(c);
            r.sort();
        });
    }

    // ---------------------------------------------------------------- phase 4
    // SequentialImpulseSolver::setupSolver + solve (sequential_impulse_solver.cpp:11-80)
    void solve() {
        for (auto& b : bodies) if (!b.kinematic) { b.tv = b.v; b.tw = b.w; }   // clearTempVelocity
        rows.resize(results.size());
        const R kerp = R(0.2), pen_th = R(0.3), rest_th = R(0.1);
        for_loop((int)results.size(), [&](int i) {   // FrictionContactConstraint::initSequentialImpulse
            const CResult<R>& cr = results[i];
            const int np = cr.point_size < kCache ? cr.point_size : kCache;
            auto& rw = rows[i];
            rw.resize(np);
            const Body<R>& A = bodies[cr.a];
            const Body<R>& B = bodies[cr.b];
            const R ims = (A.kinematic ? R(0) : A.inv_mass) + (B.kinematic ? R(0) : B.inv_mass);
            const M3<R> Ia = A.kinematic ? M3<R>() : A.world_inv_inertia;
            const M3<R> Ib = B.kinematic ? M3<R>() : B.world_inv_inertia;
            for (int k = 0; k < np; k++) {
                const CPoint<R>& cp = cr.pts[k];
                Row<R>& ci = rw[k];
                ci.ra = mv(A.t.basis, cp.la);
                ci.rb = mv(B.t.basis, cp.lb);
                ci.n = cp.normal; ci.t0 = cp.t0; ci.t1 = cp.t1;
                auto jmj = [&](const V3<R>& dir) {
                    const V3<R> xa = cross(ci.ra, dir), xb = cross(ci.rb, dir);
                    return R(1.0) / (ims + dot(mv(Ia, xa), xa) + dot(mv(Ib, xb), xb));
                };
                ci.n_jmj = jmj(ci.n);
                ci.t0_jmj = jmj(ci.t0);
                ci.t1_jmj = jmj(ci.t1);
                const V3<R> va = A.v + cross(A.w, ci.ra);
                const V3<R> vb = B.v + cross(B.w, ci.rb);
                R rev = -dot(ci.n, va - vb);
                if (std::abs(rev) < rest_th) rev = 0;
                rev *= cr.restitution;
                R pen = cp.dist;
                pen = pen > -pen_th ? pen : -pen_th;
                ci.n_rhs = (rev - kerp * pen / dt) * ci.n_jmj;
                ci.n_acc = ci.t0_acc = ci.t1_acc = 0;
                ci.mu = cr.friction;
            }
        });
        for (auto& j : joints) joint_init(j, bodies[j.a], bodies[j.b], dt, kerp);   // sequential_impulse_solver.cpp:46-48
        for (int it = 0; it < iterations; it++) {   // :60-68: contacts, then the other constraints
            for (size_t i = 0; i < results.size(); i++) iterate(i);
            for (auto& j : joints) joint_iterate(j, bodies[j.a], bodies[j.b]);
        }
        for_loop((int)bodies.size(), [&](int i) {   // syncTempVelocity
            Body<R>& b = bodies[i];
            if (b.kinematic) return;
            b.v = b.tv; b.w = b.tw;
        });
    }

    // FrictionContactConstraint::iterateSequentialImpulse (friction_contact_constraint.cpp:75-108)
    void iterate(size_t i) {
        Body<R>& A = bodies[results[i].a];
        Body<R>& B = bodies[results[i].b];
        for (auto& ci : rows[i]) {
            const V3<R> vr = A.tv + cross(A.tw, ci.ra) - B.tv - cross(B.tw, ci.rb);
            R ni = ci.n_rhs - dot(ci.n, vr) * ci.n_jmj;
            ni = ni > -ci.n_acc ? ni : -ci.n_acc;
            ci.n_acc += ni;
            R t0 = ci.t0_acc - dot(ci.t0, vr) * ci.t0_jmj;
            R t1 = ci.t1_acc - dot(ci.t1, vr) * ci.t1_jmj;
            const R scale = ci.mu * ci.n_acc / std::sqrt(t0 * t0 + t1 * t1);
            if (scale < 1) { t0 *= scale; t1 *= scale; }
            const V3<R> imp = ni * ci.n + (t0 - ci.t0_acc) * ci.t0 + (t1 - ci.t1_acc) * ci.t1;
            ci.t0_acc = t0;
            ci.t1_acc = t1;
            apply_temp_impulse(A, ci.ra, imp);
            apply_temp_impulse(B, ci.rb, -imp);
        }
    }

    static void apply_temp_impulse(Body<R>& b, const V3<R>& r, const V3<R>& imp) {   // rigidbody.cpp:166-170
        if (b.kinematic) return;
        b.tv = b.tv + imp * b.inv_mass;
        b.tw = b.tw + mv(b.world_inv_inertia, cross(r, imp));
    }

    void step() {
        integrate();
        broadphase();
        narrowphase();
        solve();
    }
};

} // namespace orc
