// Driver of tests/test_adapters.py (test infrastructure): builds a small world of the reference
// engine (src/intf/world.h), installs the adapters of include/pe_gpu_adapters.h in place of its
// broadphase, narrowphase and constraint solver (World::setBroadPhase / setNarrowPhase /
// setConstraintSolver, world.h:97-99) and runs World::step; then attaches the fused GpuStepper.
// Prints one line per path: "<path> ok" after a successful step, or "<path> error <status> <msg>"
// for the pe_gpu_adapter::Error the step raised.  Leaves with _exit (the reference's thread pool
// never joins its workers).
#include "pe_gpu_adapters.h"
#include "utils/thread_pool.h"

#include <cstdio>
#include <unistd.h>

namespace {

pe_intf::World* make_world(std::vector<pe_phys_object::RigidBody*>& bodies) {
    auto* world = new pe_intf::World();
    world->setDt(pe::Real(1.0 / 60.0));
    world->setGravity(pe::Vector3(0, pe::Real(-9.8), 0));
    auto add = [&](pe_phys_shape::Shape* s, const pe::Vector3& p, pe::Real mass, bool kinematic) {
        auto* rb = new pe_phys_object::RigidBody();
        rb->setMass(mass);
        rb->setCollisionShape(s);
        rb->setTransform(pe::Transform(pe::Matrix3::Identity(), p));
        rb->setKinematic(kinematic);
        world->addRigidBody(rb);
        bodies.push_back(rb);
        return rb;
    };
    add(new pe_phys_shape::BoxShape(pe::Vector3(20, 1, 20)), pe::Vector3(0, -0.5, 0), 0, true);
    auto* a = add(new pe_phys_shape::BoxShape(pe::Vector3(1, 1, 1)), pe::Vector3(0, 0.5, 0), 1, false);
    auto* b = add(new pe_phys_shape::SphereShape(pe::Real(0.5)), pe::Vector3(0, 1.5, 0), 1, false);
    add(new pe_phys_shape::CylinderShape(pe::Real(0.4), pe::Real(1.0)), pe::Vector3(2, 0.5, 0), 1, false);
    auto* joint = new pe_phys_constraint::BallJointConstraint();
    joint->setObjectA(a);
    joint->setObjectB(b);
    joint->setAnchorA(pe::Vector3(0, pe::Real(0.5), 0));
    joint->setAnchorB(pe::Vector3(0, pe::Real(-0.5), 0));
    world->addConstraint(joint);
    return world;
}

template <class F> void run(const char* path, F&& f) {
    try {
        f();
        std::printf("%s ok\n", path);
    } catch (const pe_gpu_adapter::Error& e) {
        std::printf("%s error %d %s\n", path, e.status, e.what());
    } catch (const std::exception& e) {
        std::printf("%s other %s\n", path, e.what());
    }
}

}  // namespace

int main() {
    utils::ThreadPool::init(2);
    std::vector<pe_phys_object::RigidBody*> bodies;
    pe_intf::World* world = make_world(bodies);
    run("phases", [&] {
        auto* np = new pe_gpu_adapter::GpuNarrowPhase();
        np->setBodies(world->getRigidBodies());
        world->setBroadPhase(new pe_gpu_adapter::GpuBroadPhase());
        world->setNarrowPhase(np);
        world->setConstraintSolver(new pe_gpu_adapter::GpuSequentialImpulseSolver(PE_GPU_SOLVER_SERIAL_ORDER));
        world->step();
    });
    std::vector<pe_phys_object::RigidBody*> bodies2;
    pe_intf::World* world2 = make_world(bodies2);
    run("stepper", [&] {
        pe_gpu_adapter::GpuStepper stepper(0.005);
        stepper.attach(*world2, 10);
        stepper.step(PE_GPU_SOLVER_COLORED);
    });
    std::fflush(stdout);
    _exit(0);
}
