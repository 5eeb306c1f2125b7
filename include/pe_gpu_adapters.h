/* Reference-side binding of the GB300 step: adapter classes that subclass the reference engine's
 * own phase interfaces and call the C ABI of include/pe_gpu.h.
 *
 * Installed with World::setBroadPhase / setNarrowPhase / setConstraintSolver
 * (src/intf/world.h:97-99), they let the unchanged World::step (src/intf/world.cpp:267-300) run its
 * phases on the GPU:
 *
 *   GpuBroadPhase               replaces BroadPhaseBase::calcCollisionPairs   (broad_phase_base.h:15-17)
 *   GpuNarrowPhase              replaces NarrowPhaseBase::calcContactResults  (narrow_phase_base.h:16)
 *   GpuSequentialImpulseSolver  replaces ConstraintSolver::setupSolver/solve  (constraint_solver.h:14-28)
 *   GpuStepper                  the whole step on the device (pe_gpu_step), poses and velocities
 *                               copied back into the RigidBody objects after each step
 *
 * Header-only C++14, compiled in the reference's tree (its include paths: src, ThirdParty,
 * SimpleViewer/include) and linked against libpe_gpu.so.  Every failing C ABI call is raised as
 * pe_gpu_adapter::Error, which carries the PE_GPU_* status and the library's message; a device
 * that cannot be used surfaces as PE_GPU_ERR_CUDA from the first phase that needs it (the handle
 * is created lazily, so constructing and installing the adapters never touches the GPU).
 */
#ifndef PE_GPU_ADAPTERS_H
#define PE_GPU_ADAPTERS_H

#include "intf/world.h"
#include "rigid/shape/box_shape.h"
#include "rigid/shape/sphere_shape.h"
#include "rigid/shape/cylinder_shape.h"
#include "rigid/shape/convex_mesh_shape.h"
#include "rigid/shape/compound_shape.h"
#include "rigid/shape/concave_mesh_shape.h"
#include "rigid/constraint/constraint/ball_joint_constraint.h"
#include "rigid/constraint/constraint/hinge_joint_constraint.h"
#include "rigid/constraint/constraint/slider_joint_constraint.h"
#include "rigid/collision/broad_phase/broad_phase_base.h"
#include "rigid/collision/narrow_phase/narrow_phase_base.h"
#include "rigid/constraint/constraint_solver/constraint_solver.h"
#include "pe_gpu.h"

#include <algorithm>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace pe_gpu_adapter {

// a failed C ABI call: the PE_GPU_* status and the library's message
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(pe_gpu_world* w, int rc, const char* call) {
    if (rc != PE_GPU_OK) throw Error(rc, std::string(call) + ": " + (w ? pe_gpu_last_error(w) : "no handle"));
}

// Flattens the bodies of a World into the C ABI's arrays (one shape record per body, SoA state).
// The device handle is created on first use.
struct Mirror {
    pe_gpu_world* w = nullptr;
    int real_bits;
    double margin;
    std::vector<pe_phys_object::RigidBody*> bodies;
    std::unordered_map<const pe_phys_object::RigidBody*, int> index;
    explicit Mirror(int bits, double contact_margin = 0.0) : real_bits(bits), margin(contact_margin) {}
    Mirror(const Mirror&) = delete;
    Mirror& operator=(const Mirror&) = delete;
    ~Mirror() { if (w) pe_gpu_destroy(w); }

    pe_gpu_world* handle() {
        if (!w) {
            pe_gpu_config cfg{real_bits, 0};
            pe_gpu_world* h = nullptr;
            const int rc = pe_gpu_create(&cfg, &h);
            if (rc != PE_GPU_OK) throw Error(rc, "pe_gpu_create: no usable CUDA device");
            w = h;
            if (margin != 0.0) check(w, pe_gpu_set_contact_margin(w, margin), "pe_gpu_set_contact_margin");
        }
        return w;
    }

    void upload(const pe::Array<pe_phys_object::RigidBody*>& objs) {
        handle();
        bodies.assign(objs.begin(), objs.end());
        index.clear();
        const int n = (int)bodies.size();
        std::vector<int> type, hvb, hvc, hfb, hfc, foff{0}, fidx, shape(n), flags(n);
        std::vector<double> param, hv, mass(n), fr(n), re(n), ld(n), ad(n), o(3 * n), b(9 * n), v(3 * n), wv(3 * n);
        auto put_mesh = [&](int k, const pe::Mesh& m) {
            hvb[k] = (int)hv.size() / 3;
            hvc[k] = (int)m.vertices.size();
            for (auto& vx : m.vertices) { hv.push_back(vx.position.x()); hv.push_back(vx.position.y()); hv.push_back(vx.position.z()); }
            hfb[k] = (int)foff.size() - 1;
            hfc[k] = (int)m.faces.size();
            for (auto& f : m.faces) {
                for (auto q : f.indices) fidx.push_back((int)q);
                foff.push_back((int)fidx.size());
            }
        };
        // one shape record; returns its index
        auto add_shape = [&](pe_phys_shape::Shape* s) {
            const int k = (int)type.size();
            type.push_back(0); hvb.push_back(0); hvc.push_back(0); hfb.push_back(0); hfc.push_back(0);
            param.insert(param.end(), {0.0, 0.0, 0.0});
            switch (s->getType()) {
                case pe_phys_shape::ShapeType::ST_Box: {
                    type[k] = PE_GPU_SHAPE_BOX;
                    const pe::Vector3& sz = static_cast<pe_phys_shape::BoxShape*>(s)->getSize();
                    param[3 * k] = sz.x(); param[3 * k + 1] = sz.y(); param[3 * k + 2] = sz.z();
                    break;
                }
                case pe_phys_shape::ShapeType::ST_Sphere:
                    type[k] = PE_GPU_SHAPE_SPHERE;
                    param[3 * k] = static_cast<pe_phys_shape::SphereShape*>(s)->getRadius();
                    break;
                case pe_phys_shape::ShapeType::ST_Cylinder: {
                    type[k] = PE_GPU_SHAPE_CYLINDER;
                    auto* c = static_cast<pe_phys_shape::CylinderShape*>(s);
                    param[3 * k] = c->getRadius(); param[3 * k + 1] = c->getHeight();
                    break;
                }
                case pe_phys_shape::ShapeType::ST_ConvexMesh:
                    // the mesh as stored after setMesh's recentring, which setMesh maps onto itself:
                    // the library repeats setMesh's preprocessing on it
                    type[k] = PE_GPU_SHAPE_CONVEX_MESH;
                    put_mesh(k, static_cast<pe_phys_shape::ConvexMeshShape*>(s)->getMesh());
                    break;
                case pe_phys_shape::ShapeType::ST_ConcaveMesh:   // the mesh as stored (setMesh keeps it)
                    type[k] = PE_GPU_SHAPE_CONCAVE_MESH;
                    put_mesh(k, static_cast<pe_phys_shape::ConcaveMeshShape*>(s)->getMesh());
                    break;
                case pe_phys_shape::ShapeType::ST_Compound:
                    type[k] = PE_GPU_SHAPE_COMPOUND;   // children below
                    break;
                default:
                    throw Error(PE_GPU_ERR_ARG, "shape type not handled by the GPU path");
            }
            return k;
        };
        std::vector<pe_phys_shape::CompoundShape*> compounds;   // per body, or null
        for (int i = 0; i < n; i++) {
            pe_phys_object::RigidBody* rb = bodies[i];
            index[rb] = i;
            pe_phys_shape::Shape* s = rb->getCollisionShape();
            shape[i] = add_shape(s);
            compounds.push_back(s->getType() == pe_phys_shape::ShapeType::ST_Compound ? static_cast<pe_phys_shape::CompoundShape*>(s)
                                                                                    : nullptr);
            flags[i] = (rb->isKinematic() ? PE_GPU_BODY_KINEMATIC : 0) | (rb->isIgnoreCollision() ? PE_GPU_BODY_IGNORE_COLLISION : 0);
            mass[i] = rb->getMass(); fr[i] = rb->getFrictionCoeff(); re[i] = rb->getRestitutionCoeff();
            ld[i] = rb->getLinearDamping(); ad[i] = rb->getAngularDamping();
            const pe::Transform& t = rb->getTransform();
            for (int k = 0; k < 3; k++) {
                o[3 * i + k] = t.getOrigin()[k];
                v[3 * i + k] = rb->getLinearVelocity()[k];
                wv[3 * i + k] = rb->getAngularVelocity()[k];
            }
            for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) b[9 * i + 3 * r + c] = t.getBasis()(r, c);
        }
        // compound children: extra shape records after the bodies' own.  The compounds' init()
        // already ran, so the children go as stored, with each compound's local inertia.
        std::vector<int> cbeg(n, 0), ccnt(n, 0), cshape;
        std::vector<double> corg, cbas, cratio, inertia(9 * (size_t)n, 0.0);
        for (int i = 0; i < n; i++) {
            pe_phys_shape::CompoundShape* cs = compounds[i];
            if (!cs) continue;
            const int si = shape[i];
            cbeg[si] = (int)cshape.size();
            ccnt[si] = (int)cs->getShapes().size();
            for (auto& e : cs->getShapes()) {
                cshape.push_back(add_shape(e.shape));
                for (int k = 0; k < 3; k++) corg.push_back(e.local_transform.getOrigin()[k]);
                for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) cbas.push_back(e.local_transform.getBasis()(r, c));
                cratio.push_back(e.mass_ratio);
            }
            for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) inertia[9 * (size_t)si + 3 * r + c] = cs->getLocalInertia()(r, c);
        }
        if (hv.empty()) hv.push_back(0.0);
        if (fidx.empty()) fidx.push_back(0);
        const int S = (int)type.size();
        check(w, pe_gpu_set_shapes(w, S, type.data(), param.data(), hvb.data(), hvc.data(), hfb.data(), hfc.data(),
                                   (int)hv.size() / 3, hv.data(), (int)foff.size() - 1, foff.data(), fidx.data()),
              "pe_gpu_set_shapes");
        if (!cshape.empty()) {
            cbeg.resize(S, 0); ccnt.resize(S, 0); inertia.resize(9 * (size_t)S, 0.0);
            check(w, pe_gpu_set_compounds(w, cbeg.data(), ccnt.data(), (int)cshape.size(), cshape.data(), corg.data(), cbas.data(),
                                          cratio.data(), inertia.data(), nullptr),
                  "pe_gpu_set_compounds");
        }
        check(w, pe_gpu_set_bodies(w, n, shape.data(), flags.data(), mass.data(), fr.data(), re.data(), ld.data(), ad.data(),
                                   o.data(), b.data(), v.data(), wv.data()),
              "pe_gpu_set_bodies");
    }

    // World::_constraints -> pe_gpu_set_joints (after upload, which clears them)
    void push_joints(const pe::Array<pe_phys_constraint::Constraint*>& cs) {
        std::vector<int> type, body, flag;
        std::vector<double> q;
        auto put3 = [&](const pe::Vector3& v) { q.push_back(v.x()); q.push_back(v.y()); q.push_back(v.z()); };
        for (pe_phys_constraint::Constraint* c : cs) {
            pe::Vector3 aa, ab, xa = pe::Vector3::UnitX(), xb = pe::Vector3::UnitX();
            double lo = 0, hi = 0, speed = 0;
            int f = 0;
            if (auto* j = dynamic_cast<pe_phys_constraint::BallJointConstraint*>(c)) {
                type.push_back(PE_GPU_JOINT_BALL);
                aa = j->getAnchorA(); ab = j->getAnchorB();
            } else if (auto* j = dynamic_cast<pe_phys_constraint::HingeJointConstraint*>(c)) {
                type.push_back(PE_GPU_JOINT_HINGE);
                aa = j->getAnchorA(); ab = j->getAnchorB(); xa = j->getAxisA(); xb = j->getAxisB();
                f = (j->isUseLimits() ? PE_GPU_JOINT_USE_LIMITS : 0) | (j->isUseMotor() ? PE_GPU_JOINT_USE_MOTOR : 0);
                lo = j->getMinAngle(); hi = j->getMaxAngle(); speed = j->getTargetSpeed();
            } else if (auto* j = dynamic_cast<pe_phys_constraint::SliderJointConstraint*>(c)) {
                type.push_back(PE_GPU_JOINT_SLIDER);
                aa = j->getAnchorA(); ab = j->getAnchorB(); xa = j->getAxisA(); xb = j->getAxisB();
            } else {
                throw Error(PE_GPU_ERR_ARG, "constraint type not handled by the GPU path");
            }
            body.push_back(index.at(c->getObjectA()));
            body.push_back(index.at(c->getObjectB()));
            flag.push_back(f);
            put3(aa); put3(ab); put3(xa); put3(xb);
            q.push_back(lo); q.push_back(hi); q.push_back(speed);
        }
        const int nj = (int)type.size();
        if (type.empty()) { type.push_back(0); body.insert(body.end(), {0, 0}); flag.push_back(0); q.resize(15, 0.0); }
        check(w, pe_gpu_set_joints(w, nj, type.data(), body.data(), flag.data(), q.data()), "pe_gpu_set_joints");
    }

    // body poses / AABBs / velocities of the reference objects -> device
    void push_state() {
        const int n = (int)bodies.size();
        std::vector<double> o(3 * n), b(9 * n), v(3 * n), wv(3 * n), mn(3 * n), mx(3 * n), iw(9 * n);
        for (int i = 0; i < n; i++) {
            pe_phys_object::RigidBody* rb = bodies[i];
            const pe::Transform& t = rb->getTransform();
            for (int k = 0; k < 3; k++) {
                o[3 * i + k] = t.getOrigin()[k];
                v[3 * i + k] = rb->getLinearVelocity()[k];
                wv[3 * i + k] = rb->getAngularVelocity()[k];
                mn[3 * i + k] = rb->getAABBMin()[k];
                mx[3 * i + k] = rb->getAABBMax()[k];
            }
            for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) {
                b[9 * i + 3 * r + c] = t.getBasis()(r, c);
                iw[9 * i + 3 * r + c] = rb->getWorldInvInertia()(r, c);
            }
        }
        check(w, pe_gpu_set_state(w, o.data(), b.data(), v.data(), wv.data(), mn.data(), mx.data(), iw.data()), "pe_gpu_set_state");
    }
};

// BroadPhaseBase replacement (broad_phase_base.h:15-17)
class GpuBroadPhase : public pe_phys_collision::BroadPhaseBase {
    Mirror m_{(int)sizeof(pe::Real) * 8};
public:
    void calcCollisionPairs(pe::Array<pe_phys_object::RigidBody*> objects,
                            pe::Array<pe_phys_collision::CollisionPair>& pairs) override {
        if (objects.size() < 2) return;   // the reference leaves the list untouched below two bodies
        if (objects.size() != m_.bodies.size() || !std::equal(objects.begin(), objects.end(), m_.bodies.begin()))
            m_.upload(objects);
        m_.push_state();
        int n = 0;
        check(m_.w, pe_gpu_broadphase(m_.w, &n), "pe_gpu_broadphase");
        std::vector<int> p(2 * (size_t)n + 2);
        check(m_.w, pe_gpu_get_pairs(m_.w, p.data()), "pe_gpu_get_pairs");
        pairs.clear();
        for (int i = 0; i < n; i++) {
            pe_phys_object::RigidBody* a = m_.bodies[p[2 * i]];
            pe_phys_object::RigidBody* b = m_.bodies[p[2 * i + 1]];
            // the reference keeps ignore sets private; its own check (broad_phase_base.cpp:11-12)
            // filters the device's pairs, keeping their order
            if (a->ignoreCollisionId(b->getGlobalId()) || b->ignoreCollisionId(a->getGlobalId())) continue;
            pairs.push_back(pe_phys_collision::CollisionPair(a, b));
        }
    }
};

// NarrowPhaseBase replacement (narrow_phase_base.h:16).  ContactResult objects stay the
// reference's; the GPU fills all eight slots of each (the valid points, then the invalid slots with
// the distances they carry, as the reference's pooled results do), and the handle keeps the
// previous step's slot distances itself.
class GpuNarrowPhase : public pe_phys_collision::NarrowPhaseBase {
    Mirror m_{(int)sizeof(pe::Real) * 8};
    std::vector<pe_phys_collision::ContactResult*> pool_;
    pe::Array<pe_phys_object::RigidBody*> world_bodies_;
public:
    // the narrowphase interface sees only pairs: the world's body list (World::getRigidBodies)
    explicit GpuNarrowPhase(const pe::Array<pe_phys_object::RigidBody*>* bodies = nullptr) {
        if (bodies) world_bodies_ = *bodies;
    }
    void setBodies(const pe::Array<pe_phys_object::RigidBody*>& bodies) { world_bodies_ = bodies; }
    ~GpuNarrowPhase() override { for (auto* r : pool_) delete r; }
    void calcContactResults(const pe::Array<pe_phys_collision::CollisionPair>& pairs,
                            pe::Array<pe_phys_collision::ContactResult*>& results) override {
        if (pairs.empty()) { results.clear(); return; }
        pe::Array<pe_phys_object::RigidBody*> objs = world_bodies_;
        if (objs.empty()) {   // no body list given: the bodies of the pairs, in address order
            for (auto& p : pairs) { objs.push_back(p.first); objs.push_back(p.second); }
            std::sort(objs.begin(), objs.end());
            objs.erase(std::unique(objs.begin(), objs.end()), objs.end());
        }
        if (objs.size() != m_.bodies.size() || !std::equal(objs.begin(), objs.end(), m_.bodies.begin())) m_.upload(objs);
        m_.push_state();
        std::vector<int> p;
        for (auto& q : pairs) { p.push_back(m_.index.at(q.first)); p.push_back(m_.index.at(q.second)); }
        check(m_.w, pe_gpu_set_pairs(m_.w, (int)pairs.size(), p.data()), "pe_gpu_set_pairs");
        check(m_.w, pe_gpu_narrowphase(m_.w), "pe_gpu_narrowphase");
        const int n = (int)pairs.size();
        std::vector<int> a(n), b(n), ps(n);
        std::vector<double> fr(n), re(n), slots((size_t)n * 8 * 19);
        check(m_.w, pe_gpu_get_results(m_.w, a.data(), b.data(), ps.data(), fr.data(), re.data(), slots.data()),
              "pe_gpu_get_results");
        while ((int)pool_.size() < n) pool_.push_back(new pe_phys_collision::ContactResult());
        results.assign(pool_.begin(), pool_.begin() + n);
        for (int i = 0; i < n; i++) {
            pe_phys_collision::ContactResult* r = results[i];
            r->clearContactPoints();
            r->setObjects(m_.bodies[a[i]], m_.bodies[b[i]]);
            for (int k = 0; k < 8; k++) {
                const double* s = &slots[((size_t)i * 8 + k) * 19];
                pe_phys_collision::ContactPoint& cp = r->getContactPoint(k);
                if (k < ps[i])
                    cp = pe_phys_collision::ContactPoint(pe::Vector3(s[0], s[1], s[2]), pe::Vector3(s[3], s[4], s[5]),
                                                         m_.bodies[a[i]], m_.bodies[b[i]], pe::Vector3(s[6], s[7], s[8]),
                                                         pe::Vector3(s[9], s[10], s[11]), s[12]);
                else
                    cp.setDistance(s[12]);   // invalidated by clearContactPoints; keeps its distance
            }
            r->sortContactPoints();   // the slots come sorted: this sets the point count
        }
    }
};

// ConstraintSolver replacement (constraint_solver.h:14-28).  getType() stays
// CST_SEQUENTIAL_IMPULSE so World::step still applies gravity (world.cpp:276-278).
class GpuSequentialImpulseSolver : public pe_phys_constraint::ConstraintSolver {
    Mirror m_{(int)sizeof(pe::Real) * 8};
    std::vector<pe_phys_constraint::Constraint*> joints_;
    int mode_;
public:
    explicit GpuSequentialImpulseSolver(int mode = PE_GPU_SOLVER_SERIAL_ORDER) : mode_(mode) { _iteration = 10; }
    pe_phys_constraint::ConstraintSolverType getType() const override {
        return pe_phys_constraint::ConstraintSolverType::CST_SEQUENTIAL_IMPULSE;
    }
    void setupSolver(pe::Real dt, const pe::Vector3& g, const pe::Array<pe_phys_object::RigidBody*>& objects,
                     const pe::Array<pe_phys_collision::ContactResult*>& results,
                     const pe::Array<pe_phys_constraint::Constraint*>& constraints) override {
        if (objects.size() != m_.bodies.size() || !std::equal(objects.begin(), objects.end(), m_.bodies.begin()) ||
            constraints.size() != joints_.size() || !std::equal(constraints.begin(), constraints.end(), joints_.begin())) {
            m_.upload(objects);
            m_.push_joints(constraints);
            joints_.assign(constraints.begin(), constraints.end());
        }
        check(m_.w, pe_gpu_set_params(m_.w, dt, g.x(), g.y(), g.z(), _iteration), "pe_gpu_set_params");
        m_.push_state();
        const int n = (int)results.size();
        std::vector<int> a(n), b(n), ps(n);
        std::vector<double> fr(n), re(n), slots((size_t)n * 8 * 19, 0.0);
        for (int i = 0; i < n; i++) {
            const pe_phys_collision::ContactResult* r = results[i];
            a[i] = m_.index.at(r->getObjectA());
            b[i] = m_.index.at(r->getObjectB());
            ps[i] = r->getPointSize();
            fr[i] = r->getFrictionCoeff();
            re[i] = r->getRestitutionCoeff();
            for (int k = 0; k < 8; k++) {
                const pe_phys_collision::ContactPoint& cp = r->getContactPoint(k);
                double* s = &slots[((size_t)i * 8 + k) * 19];
                for (int q = 0; q < 3; q++) {
                    s[q] = cp.getWorldPos()[q]; s[3 + q] = cp.getWorldNormal()[q];
                    s[6 + q] = cp.getLocalPosA()[q]; s[9 + q] = cp.getLocalPosB()[q];
                    s[13 + q] = cp.getTangent(0)[q]; s[16 + q] = cp.getTangent(1)[q];
                }
                s[12] = cp.getDistance();
            }
        }
        check(m_.w, pe_gpu_set_results(m_.w, n, a.data(), b.data(), ps.data(), fr.data(), re.data(), slots.data()),
              "pe_gpu_set_results");
    }
    void solve() override {
        check(m_.w, pe_gpu_solve(m_.w, mode_), "pe_gpu_solve");
        const int n = (int)m_.bodies.size();
        std::vector<double> v(3 * (size_t)n), wv(3 * (size_t)n);
        check(m_.w, pe_gpu_get_state(m_.w, nullptr, nullptr, v.data(), wv.data(), nullptr, nullptr, nullptr), "pe_gpu_get_state");
        for (int i = 0; i < n; i++) {
            pe_phys_object::RigidBody* rb = m_.bodies[i];
            if (rb->isKinematic()) continue;
            rb->setLinearVelocity(pe::Vector3(v[3 * i], v[3 * i + 1], v[3 * i + 2]));
            rb->setAngularVelocity(pe::Vector3(wv[3 * i], wv[3 * i + 1], wv[3 * i + 2]));
        }
    }
};

// Fused stepper: World::step for a whole world on the device.  Poses and velocities are read back
// into the RigidBody objects after every step so that the rest of the engine (callbacks, viewer)
// sees them.
class GpuStepper {
    Mirror m_;
public:
    explicit GpuStepper(double contact_margin = 0.0) : m_((int)sizeof(pe::Real) * 8, contact_margin) {}
    // `ignored`: the body pairs the application gave addIgnoreCollisionId (the reference cannot
    // enumerate a body's ignore set)
    void attach(pe_intf::World& world, int iterations,
                const std::vector<std::pair<pe_phys_object::RigidBody*, pe_phys_object::RigidBody*>>& ignored = {}) {
        m_.upload(world.getRigidBodies());
        m_.push_joints(world.getConstraints());
        std::vector<int> ip;
        for (auto& q : ignored) { ip.push_back(m_.index.at(q.first)); ip.push_back(m_.index.at(q.second)); }
        if (ip.empty()) ip.assign(2, 0);
        check(m_.w, pe_gpu_set_ignore_pairs(m_.w, (int)ignored.size(), ip.data()), "pe_gpu_set_ignore_pairs");
        const pe::Vector3 g = world.getGravity();
        check(m_.w, pe_gpu_set_params(m_.w, world.getDt(), g.x(), g.y(), g.z(), iterations), "pe_gpu_set_params");
    }
    void step(int mode = PE_GPU_SOLVER_COLORED) {
        check(m_.w, pe_gpu_step(m_.w, 1, mode), "pe_gpu_step");
        const int n = (int)m_.bodies.size();
        std::vector<double> o(3 * (size_t)n), b(9 * (size_t)n), v(3 * (size_t)n), wv(3 * (size_t)n);
        check(m_.w, pe_gpu_get_state(m_.w, o.data(), b.data(), v.data(), wv.data(), nullptr, nullptr, nullptr), "pe_gpu_get_state");
        for (int i = 0; i < n; i++) {
            pe_phys_object::RigidBody* rb = m_.bodies[i];
            pe::Matrix3 basis;
            for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) basis(r, c) = b[9 * i + 3 * r + c];
            rb->setTransform(pe::Transform(basis, pe::Vector3(o[3 * i], o[3 * i + 1], o[3 * i + 2])));
            rb->setLinearVelocity(pe::Vector3(v[3 * i], v[3 * i + 1], v[3 * i + 2]));
            rb->setAngularVelocity(pe::Vector3(wv[3 * i], wv[3 * i + 1], wv[3 * i + 2]));
        }
    }
};

}  // namespace pe_gpu_adapter

#endif /* PE_GPU_ADAPTERS_H */
