// Reference harness: drives the UNMODIFIED reference engine (pe_intf::World with its
// default BroadPhaseSweepAndPrune / SimpleNarrowPhase / SequentialImpulseSolver) on a
// scene file and records every phase boundary of the chosen steps.
//
// Test infrastructure only: it is built by oracle/build_ref.py from the reference
// sources in place (into oracle/_ref/), and only the golden-fixture generator runs it.
// The phases are observed through subclasses installed with World::setBroadPhase /
// World::setConstraintSolver (src/intf/world.h:97-100); each subclass calls the
// reference base implementation unchanged and only copies data out.
//
// Usage: ref_harness <scene.pescene> <out.pedump> <steps> <threads> [dump_step ...]
//        (no dump steps = dump every step; "-1" = dump none, time only)
// With PE_TRAJ_OUT set, the body states after every step (origin 3, basis 9 row-major, linear
// and angular velocity 3 + 3, as doubles, bodies in scene order) are also appended to that file.

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
#include "rigid/collision/broad_phase/broad_phase_sweep_and_prune.h"
#include "rigid/constraint/constraint_solver/sequential_impulse_solver.h"
#include "utils/thread_pool.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <unistd.h>
#include <unordered_map>
#include <vector>

namespace {

struct Scene {
    int n_shapes = 0, n_bodies = 0, n_hull_verts = 0, n_hull_faces = 0, n_hull_face_idx = 0, iterations = 10;
    double dt = 0.01, g[3] = {0, -9.8, 0};
    std::vector<int> type, hvbeg, hvcnt, hfbeg, hfcnt, face_off, face_idx, shape, flags;
    std::vector<double> param, hverts, mass, friction, restitution, lin_damp, ang_damp, origin, basis, v, w;
    std::vector<int> cbeg, ccnt, cshape;   // compound children ("PESCENE2")
    std::vector<double> corigin, cbasis, cratio;
    std::vector<int> jtype, jbody, jflag, ign;   // tagged sections: joints, ignored body pairs
    std::vector<double> jreal;
};

template <class T> void rd(FILE* f, T* p, size_t n) {
    if (n && fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); _exit(2); }
}

Scene load(const char* path) {
    Scene s;
    FILE* f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); _exit(2); }
    char magic[8];
    rd(f, magic, 8);
    const bool compound = memcmp(magic, "PESCENE2", 8) == 0;
    if (memcmp(magic, "PESCENE1", 8) != 0 && !compound) { fprintf(stderr, "bad magic\n"); _exit(2); }
    int hdr[6];
    rd(f, hdr, 6);
    s.n_shapes = hdr[0]; s.n_bodies = hdr[1]; s.n_hull_verts = hdr[2];
    s.n_hull_faces = hdr[3]; s.n_hull_face_idx = hdr[4]; s.iterations = hdr[5];
    double w4[4];
    rd(f, w4, 4);
    s.dt = w4[0]; s.g[0] = w4[1]; s.g[1] = w4[2]; s.g[2] = w4[3];
    const int S = s.n_shapes, N = s.n_bodies;
    s.type.resize(S); rd(f, s.type.data(), S);
    s.param.resize(S * 3); rd(f, s.param.data(), S * 3);
    s.hvbeg.resize(S); rd(f, s.hvbeg.data(), S);
    s.hvcnt.resize(S); rd(f, s.hvcnt.data(), S);
    s.hfbeg.resize(S); rd(f, s.hfbeg.data(), S);
    s.hfcnt.resize(S); rd(f, s.hfcnt.data(), S);
    s.hverts.resize(s.n_hull_verts * 3); rd(f, s.hverts.data(), s.hverts.size());
    s.face_off.resize(s.n_hull_faces + 1); rd(f, s.face_off.data(), s.face_off.size());
    s.face_idx.resize(s.n_hull_face_idx); rd(f, s.face_idx.data(), s.face_idx.size());
    s.shape.resize(N); rd(f, s.shape.data(), N);
    s.flags.resize(N); rd(f, s.flags.data(), N);
    for (auto* a : {&s.mass, &s.friction, &s.restitution, &s.lin_damp, &s.ang_damp}) { a->resize(N); rd(f, a->data(), N); }
    s.origin.resize(N * 3); rd(f, s.origin.data(), N * 3);
    s.basis.resize(N * 9); rd(f, s.basis.data(), N * 9);
    s.v.resize(N * 3); rd(f, s.v.data(), N * 3);
    s.w.resize(N * 3); rd(f, s.w.data(), N * 3);
    if (compound) {
        int C = 0;
        rd(f, &C, 1);
        s.cbeg.resize(S); rd(f, s.cbeg.data(), S);
        s.ccnt.resize(S); rd(f, s.ccnt.data(), S);
        s.cshape.resize(C); rd(f, s.cshape.data(), C);
        s.corigin.resize(C * 3); rd(f, s.corigin.data(), C * 3);
        s.cbasis.resize(C * 9); rd(f, s.cbasis.data(), C * 9);
        s.cratio.resize(C); rd(f, s.cratio.data(), C);
        int th[2];
        while (fread(th, sizeof(int), 2, f) == 2) {
            const int n = th[1];
            if (th[0] == 1) {
                s.jtype.resize(n); rd(f, s.jtype.data(), n);
                s.jbody.resize(2 * n); rd(f, s.jbody.data(), 2 * n);
                s.jflag.resize(n); rd(f, s.jflag.data(), n);
                s.jreal.resize(15 * n); rd(f, s.jreal.data(), 15 * n);
            } else if (th[0] == 2) {
                s.ign.resize(2 * n); rd(f, s.ign.data(), 2 * n);
            } else {
                fprintf(stderr, "unknown scene section %d\n", th[0]); _exit(2);
            }
        }
    }
    fclose(f);
    return s;
}

pe_phys_shape::Shape* make_shape(const Scene& s, int i) {
    const double* p = &s.param[i * 3];
    switch (s.type[i]) {
        case 0: return new pe_phys_shape::BoxShape(pe::Vector3(PE_R(p[0]), PE_R(p[1]), PE_R(p[2])));
        case 1: return new pe_phys_shape::SphereShape(PE_R(p[0]));
        case 2: return new pe_phys_shape::CylinderShape(PE_R(p[0]), PE_R(p[1]));
        case 3:
        case 4: {
            pe::Mesh mesh;
            for (int k = 0; k < s.hvcnt[i]; k++) {
                const double* q = &s.hverts[(s.hvbeg[i] + k) * 3];
                mesh.vertices.push_back({pe::Vector3(PE_R(q[0]), PE_R(q[1]), PE_R(q[2])), pe::Vector3::Zero()});
            }
            for (int fi = s.hfbeg[i]; fi < s.hfbeg[i] + s.hfcnt[i]; fi++) {
                pe::Mesh::Face face;
                for (int k = s.face_off[fi]; k < s.face_off[fi + 1]; k++) face.indices.push_back((uint32_t)s.face_idx[k]);
                mesh.faces.push_back(face);
            }
            pe::Mesh::perFaceNormal(mesh);
            if (s.type[i] == 4) {
                auto* cc = new pe_phys_shape::ConcaveMeshShape();
                cc->setMesh(mesh);
                return cc;
            }
            auto* cm = new pe_phys_shape::ConvexMeshShape();
            cm->setMesh(mesh);
            return cm;
        }
        default: fprintf(stderr, "unsupported shape type %d\n", s.type[i]); _exit(2);
    }
}

struct Dumper {
    FILE* f = nullptr;
    bool active = false;
    int step = 0;
    std::unordered_map<const pe_phys_object::RigidBody*, int> index;
    const pe::Array<pe_phys_object::RigidBody*>* bodies = nullptr;
    int axis_before = 0, axis_after = 0;
    std::vector<double> pre;   // pre-broadphase body state
    std::vector<int> pairs;
    std::vector<int> ri;       // per result: a, b, point_size, valid mask
    std::vector<double> rf;    // per result: friction, restitution
    std::vector<double> slots; // per result: 8 slots x 19 reals

    template <class T> void wr(const T* p, size_t n) { if (n) fwrite(p, sizeof(T), n, f); }

    static void put3(std::vector<double>& o, const pe::Vector3& v) { o.push_back(v.x()); o.push_back(v.y()); o.push_back(v.z()); }
    static void put9(std::vector<double>& o, const pe::Matrix3& m) {
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) o.push_back(m(r, c));
    }

    void record_pre(const pe::Array<pe_phys_object::RigidBody*>& objs, int axis) {
        axis_before = axis;
        const size_t N = objs.size();
        std::vector<double> o3, b9, v3, w3, mn, mx, iw;
        for (size_t i = 0; i < N; i++) {
            auto* rb = objs[i];
            put3(o3, rb->getTransform().getOrigin());
            put9(b9, rb->getTransform().getBasis());
            put3(v3, rb->getLinearVelocity());
            put3(w3, rb->getAngularVelocity());
            put3(mn, rb->getAABBMin());
            put3(mx, rb->getAABBMax());
            put9(iw, rb->getWorldInvInertia());
        }
        pre.clear();
        for (auto* a : {&o3, &b9, &v3, &w3, &mn, &mx, &iw}) pre.insert(pre.end(), a->begin(), a->end());
    }

    void record_pairs(const pe::Array<pe_phys_collision::CollisionPair>& ps, int axis) {
        axis_after = axis;
        pairs.clear();
        for (auto& p : ps) { pairs.push_back(index.at(p.first)); pairs.push_back(index.at(p.second)); }
    }

    void record_results(const pe::Array<pe_phys_collision::ContactResult*>& rs) {
        ri.clear(); rf.clear(); slots.clear();
        for (auto* r : rs) {
            int mask = 0;
            for (int k = 0; k < PE_CONTACT_CACHE_SIZE; k++) if (r->getContactPoint(k).isValid()) mask |= 1 << k;
            ri.push_back(index.at(r->getObjectA()));
            ri.push_back(index.at(r->getObjectB()));
            ri.push_back(r->getPointSize());
            ri.push_back(mask);
            rf.push_back(r->getFrictionCoeff());
            rf.push_back(r->getRestitutionCoeff());
            for (int k = 0; k < PE_CONTACT_CACHE_SIZE; k++) {
                const auto& cp = r->getContactPoint(k);
                put3(slots, cp.getWorldPos());
                put3(slots, cp.getWorldNormal());
                put3(slots, cp.getLocalPosA());
                put3(slots, cp.getLocalPosB());
                slots.push_back(cp.getDistance());
                put3(slots, cp.getTangent(0));
                put3(slots, cp.getTangent(1));
            }
        }
    }

    void write_step(const pe::Array<pe_phys_object::RigidBody*>& objs) {
        const int N = (int)objs.size();
        const int P = (int)pairs.size() / 2;
        const int R = (int)rf.size() / 2;
        int hdr[6] = {step, N, axis_before, axis_after, P, R};
        wr(hdr, 6);
        wr(pre.data(), pre.size());
        wr(pairs.data(), pairs.size());
        // results: columns a, b, point_size, mask
        std::vector<int> col(R);
        for (int c = 0; c < 4; c++) { for (int r = 0; r < R; r++) col[r] = ri[r * 4 + c]; wr(col.data(), col.size()); }
        std::vector<double> fc(R), rc(R);
        for (int r = 0; r < R; r++) { fc[r] = rf[r * 2]; rc[r] = rf[r * 2 + 1]; }
        wr(fc.data(), fc.size());
        wr(rc.data(), rc.size());
        wr(slots.data(), slots.size());
        std::vector<double> v3, w3;
        for (auto* rb : objs) { put3(v3, rb->getLinearVelocity()); put3(w3, rb->getAngularVelocity()); }
        wr(v3.data(), v3.size());
        wr(w3.data(), w3.size());
    }
};

Dumper g_dump;

class RecordingSAP : public pe_phys_collision::BroadPhaseSweepAndPrune {
public:
    void calcCollisionPairs(pe::Array<pe_phys_object::RigidBody*> objects,
                            pe::Array<pe_phys_collision::CollisionPair>& pairs) override {
        if (g_dump.active) g_dump.record_pre(objects, _target_axis);
        BroadPhaseSweepAndPrune::calcCollisionPairs(objects, pairs);
        if (g_dump.active) g_dump.record_pairs(pairs, _target_axis);
    }
};

class RecordingSIS : public pe_phys_constraint::SequentialImpulseSolver {
public:
    void setupSolver(pe::Real dt, const pe::Vector3& gravity,
                     const pe::Array<pe_phys_object::RigidBody*>& objects,
                     const pe::Array<pe_phys_collision::ContactResult*>& contact_results,
                     const pe::Array<pe_phys_constraint::Constraint*>& constraints) override {
        if (g_dump.active) g_dump.record_results(contact_results);
        SequentialImpulseSolver::setupSolver(dt, gravity, objects, contact_results, constraints);
    }
};

} // namespace

int main(int argc, char** argv) {
    if (argc < 5) { fprintf(stderr, "usage: %s scene out steps threads [dump_steps...]\n", argv[0]); return 2; }
    Scene s = load(argv[1]);
    const int steps = atoi(argv[3]);
    const int threads = atoi(argv[4]);
    std::set<int> dump_steps;
    bool dump_all = argc == 5, dump_none = false;
    for (int i = 5; i < argc; i++) { int k = atoi(argv[i]); if (k < 0) dump_none = true; else dump_steps.insert(k); }

    utils::ThreadPool::init(threads > 0 ? threads : 0);
    auto* world = new pe_intf::World();
    world->setDt(PE_R(s.dt));
    world->setGravity(pe::Vector3(PE_R(s.g[0]), PE_R(s.g[1]), PE_R(s.g[2])));
    world->setBroadPhase(new RecordingSAP());
    auto* solver = new RecordingSIS();
    solver->setIteration(s.iterations);
    world->setConstraintSolver(solver);

    std::vector<pe_phys_shape::Shape*> shapes;
    for (int i = 0; i < s.n_shapes; i++) shapes.push_back(s.type[i] == 5 ? nullptr : make_shape(s, i));
    // compound shapes: CompoundShape::addShape per child, then init() (children relocated to their
    // centroid, local inertia), as examples/compound_demo/main.cpp builds them
    for (int i = 0; i < s.n_shapes; i++) {
        if (s.type[i] != 5) continue;
        auto* cs = new pe_phys_shape::CompoundShape();
        for (int k = s.cbeg[i]; k < s.cbeg[i] + s.ccnt[i]; k++) {
            pe::Matrix3 b;
            for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) b(r, c) = PE_R(s.cbasis[k * 9 + r * 3 + c]);
            const double* o = &s.corigin[k * 3];
            cs->addShape(pe::Transform(b, pe::Vector3(PE_R(o[0]), PE_R(o[1]), PE_R(o[2]))), PE_R(s.cratio[k]), shapes[s.cshape[k]]);
        }
        cs->init();
        shapes[i] = cs;
    }
    std::vector<pe_phys_object::RigidBody*> rbs;
    for (int i = 0; i < s.n_bodies; i++) {
        auto* rb = new pe_phys_object::RigidBody();
        rbs.push_back(rb);
        rb->setMass(PE_R(s.mass[i]));
        rb->setCollisionShape(shapes[s.shape[i]]);
        pe::Matrix3 b;
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) b(r, c) = PE_R(s.basis[i * 9 + r * 3 + c]);
        rb->setTransform(pe::Transform(b, pe::Vector3(PE_R(s.origin[i * 3]), PE_R(s.origin[i * 3 + 1]), PE_R(s.origin[i * 3 + 2]))));
        rb->setLinearVelocity(pe::Vector3(PE_R(s.v[i * 3]), PE_R(s.v[i * 3 + 1]), PE_R(s.v[i * 3 + 2])));
        rb->setAngularVelocity(pe::Vector3(PE_R(s.w[i * 3]), PE_R(s.w[i * 3 + 1]), PE_R(s.w[i * 3 + 2])));
        rb->setFrictionCoeff(PE_R(s.friction[i]));
        rb->setRestitutionCoeff(PE_R(s.restitution[i]));
        rb->setLinearDamping(PE_R(s.lin_damp[i]));
        rb->setAngularDamping(PE_R(s.ang_damp[i]));
        rb->setKinematic((s.flags[i] & 1) != 0);
        rb->setIgnoreCollision((s.flags[i] & 2) != 0);
        world->addRigidBody(rb);
        g_dump.index[rb] = i;
    }

    for (size_t k = 0; k + 1 < s.ign.size(); k += 2) rbs[s.ign[k]]->addIgnoreCollisionId(rbs[s.ign[k + 1]]->getGlobalId());
    for (size_t k = 0; k < s.jtype.size(); k++) {
        const double* r = &s.jreal[k * 15];
        auto v3 = [&](int o) { return pe::Vector3(PE_R(r[o]), PE_R(r[o + 1]), PE_R(r[o + 2])); };
        pe_phys_constraint::Constraint* c = nullptr;
        if (s.jtype[k] == 0) {
            auto* j = new pe_phys_constraint::BallJointConstraint();
            j->setAnchorA(v3(0)); j->setAnchorB(v3(3));
            c = j;
        } else if (s.jtype[k] == 1) {
            auto* j = new pe_phys_constraint::HingeJointConstraint();
            j->setAnchorA(v3(0)); j->setAnchorB(v3(3)); j->setAxisA(v3(6)); j->setAxisB(v3(9));
            j->setUseLimits((s.jflag[k] & 1) != 0); j->setMinAngle(PE_R(r[12])); j->setMaxAngle(PE_R(r[13]));
            j->setUseMotor((s.jflag[k] & 2) != 0); j->setTargetSpeed(PE_R(r[14]));
            c = j;
        } else {
            auto* j = new pe_phys_constraint::SliderJointConstraint();
            j->setAnchorA(v3(0)); j->setAnchorB(v3(3)); j->setAxisA(v3(6)); j->setAxisB(v3(9));
            c = j;
        }
        c->setObjectA(rbs[s.jbody[2 * k]]);
        c->setObjectB(rbs[s.jbody[2 * k + 1]]);
        world->addConstraint(c);
    }

    g_dump.f = dump_none ? nullptr : fopen(argv[2], "wb");
    if (!dump_none && !g_dump.f) { fprintf(stderr, "cannot write %s\n", argv[2]); _exit(2); }
    if (g_dump.f) {
        const char magic[8] = {'P', 'E', 'D', 'U', 'M', 'P', '1', 0};
        fwrite(magic, 1, 8, g_dump.f);
        int real_bytes = (int)sizeof(pe::Real);
        fwrite(&real_bytes, sizeof(int), 1, g_dump.f);
    }

    FILE* traj = getenv("PE_TRAJ_OUT") ? fopen(getenv("PE_TRAJ_OUT"), "wb") : nullptr;
    double total_s = 0;
    for (int k = 0; k < steps; k++) {
        g_dump.step = k;
        g_dump.active = !dump_none && (dump_all || dump_steps.count(k));
        auto t0 = std::chrono::steady_clock::now();
        world->step();
        auto t1 = std::chrono::steady_clock::now();
        total_s += std::chrono::duration<double>(t1 - t0).count();
        if (g_dump.active) g_dump.write_step(world->getRigidBodies());
        if (traj) {
            std::vector<double> row(18);
            for (auto* rb : rbs) {
                const pe::Transform& t = rb->getTransform();
                for (int d = 0; d < 3; d++) row[d] = (double)t.getOrigin()[d];
                for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) row[3 + r * 3 + c] = (double)t.getBasis()(r, c);
                for (int d = 0; d < 3; d++) row[12 + d] = (double)rb->getLinearVelocity()[d];
                for (int d = 0; d < 3; d++) row[15 + d] = (double)rb->getAngularVelocity()[d];
                fwrite(row.data(), sizeof(double), 18, traj);
            }
        }
    }
    if (traj) fclose(traj);
    printf("{\"steps\": %d, \"bodies\": %d, \"threads\": %d, \"seconds\": %.6f, "
           "\"update_s\": %.6f, \"bp_s\": %.6f, \"np_s\": %.6f, \"solver_s\": %.6f, \"real_bytes\": %d}\n",
           steps, s.n_bodies, threads, total_s, (double)world->update_status_time, (double)world->broad_phase_time,
           (double)world->narrow_phase_time, (double)world->constraint_solver_time, (int)sizeof(pe::Real));
    fflush(stdout);
    if (g_dump.f) fclose(g_dump.f);
    // the reference thread pool's workers never exit; leave without running static destructors
    _exit(0);
}
