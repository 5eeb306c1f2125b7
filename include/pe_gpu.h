/*
 * pe_gpu.h - C ABI of the GB300 rigid-body step.
 *
 * One handle = one device-resident world (or a batch of independent scenes) on one GPU.
 * All functions return an int status (PE_GPU_OK = 0, negative on error; the message is
 * available from pe_gpu_last_error).  No exception crosses this boundary.  A handle is
 * not thread-safe, like the reference World ("NOT thread-safe", src/intf/world.h:17-21):
 * callers serialise calls on one handle.
 *
 * Reals cross the boundary as double (the reference's default pe::Real, PE_USE_DOUBLE in
 * CMakeLists.txt:28); a world created with real_bits = 32 computes in float and rounds on
 * the way in.  Matrices are row-major 3x3.  Body / shape / pair indices are 0-based
 * positions in the arrays the caller supplied.
 *
 * Each entry point names the reference interface it replaces.
 */
#ifndef PE_GPU_H
#define PE_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define PE_GPU_OK 0
#define PE_GPU_ERR_ARG (-1)
#define PE_GPU_ERR_CUDA (-2)
#define PE_GPU_ERR_CAPACITY (-3)
#define PE_GPU_ERR_STATE (-4)

/* shape types, in the order of pe_phys_shape::ShapeType (src/rigid/shape/shape.h:7-9) */
#define PE_GPU_SHAPE_BOX 0
#define PE_GPU_SHAPE_SPHERE 1
#define PE_GPU_SHAPE_CYLINDER 2
#define PE_GPU_SHAPE_CONVEX_MESH 3
#define PE_GPU_SHAPE_CONCAVE_MESH 4   /* ConcaveMeshShape::setMesh (concave_mesh_shape.cpp:6-17): the hull tables' layout */
#define PE_GPU_SHAPE_COMPOUND 5       /* ShapeType::ST_Compound (shape.h:7-9); children via pe_gpu_set_compounds */

/* body flags */
#define PE_GPU_BODY_KINEMATIC 1        /* RigidBody::setKinematic (rigidbody.h:14) */
#define PE_GPU_BODY_IGNORE_COLLISION 2 /* RigidBody::setIgnoreCollision (rigidbody.h:15) */

/* solver modes */
#define PE_GPU_SOLVER_SERIAL_ORDER 0   /* the reference's constraint order, one thread per scene */
#define PE_GPU_SOLVER_COLORED 1        /* graph-coloured Gauss-Seidel */

typedef struct pe_gpu_world pe_gpu_world;

typedef struct pe_gpu_config {
    int real_bits; /* 32 or 64 */
    int device;    /* CUDA device ordinal */
} pe_gpu_config;

/* Creates / destroys a world.  Replaces constructing pe_intf::World (src/intf/world.cpp:10-27). */
int pe_gpu_create(const pe_gpu_config* cfg, pe_gpu_world** out);
int pe_gpu_destroy(pe_gpu_world* w);
const char* pe_gpu_last_error(const pe_gpu_world* w);

/* Collision shapes.  Replaces new BoxShape(size) / SphereShape(r) / CylinderShape(r, h) /
 * ConvexMeshShape::setMesh(mesh) (box_shape.cpp:7, sphere_shape.cpp:5, cylinder_shape.cpp:6,
 * convex_mesh_shape.cpp:12).  param[3*i..]: box size xyz; sphere radius; cylinder radius, height.
 * Convex meshes: hull_vbeg/vcnt index hull_verts (3 doubles per vertex), hull_fbeg/fcnt index
 * hull_face_off (n_hull_faces+1 offsets into hull_face_idx, indices local to the shape).  Faces
 * are wound counter-clockwise seen from outside; normals are computed like Mesh::perFaceNormal. */
int pe_gpu_set_shapes(pe_gpu_world* w, int n_shapes, const int* type, const double* param, const int* hull_vbeg,
                      const int* hull_vcnt, const int* hull_fbeg, const int* hull_fcnt, int n_hull_verts,
                      const double* hull_verts, int n_hull_faces, const int* hull_face_off, const int* hull_face_idx);

/* Compound shapes.  Replaces CompoundShape::addShape(local_transform, mass_ratio, child) for each
 * child followed by CompoundShape::init() (compound_shape.cpp:7-47), for every shape that
 * pe_gpu_set_shapes declared PE_GPU_SHAPE_COMPOUND.  Call after pe_gpu_set_shapes and before
 * pe_gpu_set_bodies.  child_beg / child_cnt [n_shapes]: the children of shape s are
 * [child_beg[s], child_beg[s] + child_cnt[s]) (ignored for other shapes); per child: child_shape
 * (a non-compound shape of the same table), child_origin [3], child_basis [9, row-major] and
 * child_ratio (mass ratio, >= 1e-5).  With local_inertia NULL the library runs init(): the
 * children are relocated to their mass-ratio centroid, the compound's unit-mass inertia is
 * computed from theirs, and centroid (optional, [3 n_shapes]) receives the relocation vector
 * init() returns (zero for other shapes).  With local_inertia [9 n_shapes, row-major] the children
 * are taken as already initialised (CompoundShape::getShapes() of a shape whose init() ran) and
 * local_inertia[9 s..] is CompoundShape::getLocalInertia().  Collisions of a compound follow
 * CompoundCompoundCollisionAlgorithm (compound_compound_collision_algorithm.cpp:8-46): a result
 * whose second body is a compound names the compound as body A. */
int pe_gpu_set_compounds(pe_gpu_world* w, const int* child_beg, const int* child_cnt, int n_children, const int* child_shape,
                         const double* child_origin, const double* child_basis, const double* child_ratio,
                         const double* local_inertia, double* centroid);

/* Rigid bodies, all at once.  Replaces RigidBody::setMass / setCollisionShape / setTransform /
 * setLinearVelocity / setAngularVelocity / setFrictionCoeff / setRestitutionCoeff /
 * setLinearDamping / setAngularDamping / setKinematic followed by World::addRigidBody
 * (rigidbody.cpp:11-67, world.cpp:218-221). */
int pe_gpu_set_bodies(pe_gpu_world* w, int n, const int* shape, const int* flags, const double* mass,
                      const double* friction, const double* restitution, const double* lin_damp, const double* ang_damp,
                      const double* origin, const double* basis, const double* lin_vel, const double* ang_vel);

/* Joint constraints, all at once, in World::addConstraint order (world.h:90); call after
 * pe_gpu_set_bodies, which clears them.  Replaces BallJointConstraint / HingeJointConstraint /
 * SliderJointConstraint with setObjectA/B, setAnchorA/B, setAxisA/B, setUseLimits, setMinAngle,
 * setMaxAngle, setUseMotor, setTargetSpeed (ball_joint_constraint.h, hinge_joint_constraint.h,
 * slider_joint_constraint.h).  type[j]: PE_GPU_JOINT_*; bodies[2j..]: bodies A and B; flags[j]:
 * PE_GPU_JOINT_USE_LIMITS | PE_GPU_JOINT_USE_MOTOR (hinge); params[15j..]: anchor_a, anchor_b,
 * axis_a, axis_b (3 each, in the bodies' frames), min_angle, max_angle, target_speed.  The solver
 * runs every contact and then every joint in each iteration, as SequentialImpulseSolver::solve
 * (sequential_impulse_solver.cpp:60-68); in coloured mode joints take part in the colouring. */
#define PE_GPU_JOINT_BALL 0
#define PE_GPU_JOINT_HINGE 1
#define PE_GPU_JOINT_SLIDER 2
#define PE_GPU_JOINT_USE_LIMITS 1
#define PE_GPU_JOINT_USE_MOTOR 2
int pe_gpu_set_joints(pe_gpu_world* w, int n, const int* type, const int* bodies, const int* flags, const double* params);

/* Body pairs that never collide: RigidBody::addIgnoreCollisionId (rigidbody.h:126) as checked by
 * BroadPhaseBase::validateCollisionPair (broad_phase_base.cpp:11-12), which excludes a pair when
 * either body lists the other.  pairs[2k..]: body indices.  Call after pe_gpu_set_bodies, which
 * clears them; a call replaces the previous pairs. */
int pe_gpu_set_ignore_pairs(pe_gpu_world* w, int n, const int* pairs);

/* Independent scenes in one world: bodies [body_off[s], body_off[s+1]) form scene s.  Each scene
 * behaves as its own pe_intf::World (own sweep axis, own contact-result pool).  Default: one scene. */
int pe_gpu_set_scenes(pe_gpu_world* w, int n_scenes, const int* body_off);

/* World::setDt / setGravity (world.h:24-25) and ConstraintSolver::setIteration (constraint_solver.h:72). */
int pe_gpu_set_params(pe_gpu_world* w, double dt, double gx, double gy, double gz, int iterations);

/* Contact margin of every pair algorithm: the reference's compile-time PE_MARGIN
 * (src/rigid/phys_general.h:45, pe::Real(0) in its build), read into each algorithm's `margin`
 * (e.g. convex_convex_collision_algorithm.cpp:23, its clipping window [-refScale, margin] at
 * :426-429).  Default 0; a margin >= 0 reproduces the reference compiled with that PE_MARGIN. */
int pe_gpu_set_contact_margin(pe_gpu_world* w, double margin);

/* Scheduling settings of the step: which kernel takes which work, with how many threads.  They
 * replace the reference's fixed work split of its thread pool (batch = count / threads / 2 + 1,
 * src/utils/thread_pool.h:85-102).  In serial-order mode no valid setting changes a result bit; in
 * coloured mode none does while every island needs at most exact_levels_colored levels (above, a
 * big island is coloured first-fit).  pe_gb300.autotune picks them by timing a small batched case;
 * the defaults are those below. */
typedef struct pe_gpu_tuning {
    int sat_heavy_cost;       /* SAT pairs whose estimated work reaches this run on a block of warps (200000) */
    int small_island_items;   /* islands up to this many items run on one thread each, 0..64 (8) */
    int big_island_items;     /* islands above this many items are coloured and solved grid-wide (4096) */
    int color_block;          /* threads per island block in coloured mode, 32..256, multiple of 32 (64) */
    int level_block;          /* threads per island block in serial-order mode, 32..256, multiple of 32 (256) */
    int exact_levels_colored; /* coloured mode keeps a big island's exact levels up to this many, 0..1023 (512) */
    int scene_sort_max;       /* scenes up to this many bodies are sorted inside one block, 0..2048 (2048) */
    int side_streams;         /* streams for the narrowphase's per-class kernels, 1..4 (4) */
} pe_gpu_tuning;
int pe_gpu_get_tuning(pe_gpu_world* w, pe_gpu_tuning* out);
int pe_gpu_set_tuning(pe_gpu_world* w, const pe_gpu_tuning* t);
/* the name of CUDA device `device` (cudaGetDeviceProperties), the key of the autotuner's tables */
int pe_gpu_device_name(int device, char* name, int cap);

/* World::step (world.cpp:267-300): n_steps full steps on the device without host round trips
 * of body state. */
int pe_gpu_step(pe_gpu_world* w, int n_steps, int solver_mode);

/* ---- per-phase entry points (the reference's phase interfaces) ---- */
/* World::updateObjectStatus + applyExternalForce (world.cpp:35-127). */
int pe_gpu_integrate(pe_gpu_world* w);
/* BroadPhaseBase::calcCollisionPairs (broad_phase_base.h:15-17); *n_pairs receives the count. */
int pe_gpu_broadphase(pe_gpu_world* w, int* n_pairs);
/* NarrowPhaseBase::calcContactResults (narrow_phase_base.h:16) on the current pair list. */
int pe_gpu_narrowphase(pe_gpu_world* w);
/* ConstraintSolver::setupSolver + solve (constraint_solver.h:14-28) on the current results. */
int pe_gpu_solve(pe_gpu_world* w, int solver_mode);

/* ---- state transfer (host arrays, doubles) ----
 * Each array is row-major per body (3 or 9 doubles); a null pointer skips that field.  One copy per
 * field moves the caller's array to or from a device staging buffer, and a kernel changes the
 * precision and layout on the device, so page-locked caller arrays make the transfers plain DMA.
 * pe_gpu_set_state recomputes the AABB scale of every body when origin, aabb_min and aabb_max are
 * all given.  Both return after the copies have completed. */
int pe_gpu_n_bodies(const pe_gpu_world* w);
int pe_gpu_get_state(pe_gpu_world* w, double* origin, double* basis, double* lin_vel, double* ang_vel, double* aabb_min,
                     double* aabb_max, double* world_inv_inertia);
int pe_gpu_set_state(pe_gpu_world* w, const double* origin, const double* basis, const double* lin_vel,
                     const double* ang_vel, const double* aabb_min, const double* aabb_max,
                     const double* world_inv_inertia);
/* The same with float arrays: the state as the reference's default build holds it (pe::Real is
 * float unless PE_USE_DOUBLE, src/rigid/phys_general.h:79-83), half the bytes of the double calls. */
int pe_gpu_get_state_f32(pe_gpu_world* w, float* origin, float* basis, float* lin_vel, float* ang_vel, float* aabb_min,
                         float* aabb_max, float* world_inv_inertia);
int pe_gpu_set_state_f32(pe_gpu_world* w, const float* origin, const float* basis, const float* lin_vel,
                         const float* ang_vel, const float* aabb_min, const float* aabb_max,
                         const float* world_inv_inertia);
/* sweep axis of each scene (BroadPhaseSweepAndPrune::_target_axis) */
int pe_gpu_get_axes(pe_gpu_world* w, int* axes);
int pe_gpu_set_axes(pe_gpu_world* w, const int* axes);
/* pairs as (body A, body B) in broadphase order; set_pairs replaces the list fed to the narrowphase */
int pe_gpu_n_pairs(const pe_gpu_world* w);
int pe_gpu_get_pairs(pe_gpu_world* w, int* pairs);
int pe_gpu_set_pairs(pe_gpu_world* w, int n, const int* pairs);
/* contact results, one per pair: bodies, point count, combined friction / restitution and the 8
 * cache slots x 19 reals (world_pos 3, world_normal 3, local_a 3, local_b 3, distance 1,
 * tangent0 3, tangent1 3).  Slots at or beyond point_size carry only their distance (the value a
 * pooled ContactResult keeps in an empty slot); their other fields are zero. */
int pe_gpu_n_results(const pe_gpu_world* w);
int pe_gpu_get_results(pe_gpu_world* w, int* a, int* b, int* point_size, double* friction, double* restitution,
                       double* slots);
int pe_gpu_set_results(pe_gpu_world* w, int n, const int* a, const int* b, const int* point_size,
                       const double* friction, const double* restitution, const double* slots);

/* Per-phase device time accumulated since the last reset, in milliseconds, measured with CUDA
 * events on the world's stream (the GPU counterpart of World's update_status_time /
 * broad_phase_time / narrow_phase_time / constraint_solver_time, world.h:58-61).
 * ms[0] integrate, ms[1] broadphase, ms[2] narrowphase, ms[3] solver, ms[4] whole steps. */
int pe_gpu_phase_times(pe_gpu_world* w, double* ms, int reset);
/* counts6: pairs, non-empty results, contact points (solver rows), colours, kernel launches of the
 * last pe_gpu_step step (a replayed step graph counts its kernel nodes), contact islands */
int pe_gpu_last_counts(pe_gpu_world* w, int* counts6);
/* Per-kernel-group device time: with profiling on, every kernel launch is bracketed by CUDA events
 * on the world's stream.  ms[k] / launches[k] for k < pe_gpu_kernel_count() (cumulative). */
int pe_gpu_set_profiling(pe_gpu_world* w, int on);
int pe_gpu_kernel_count(void);
const char* pe_gpu_kernel_name(int k);
int pe_gpu_kernel_stats(pe_gpu_world* w, double* ms, long long* launches);
/* blocks until all work on the world's stream finished */
int pe_gpu_sync(pe_gpu_world* w);
/* Steps through CUDA graphs (on by default).  A step waits on the host twice: for the pair count
 * (the pair capacity follows it) and for its counters at the end.  Between the two, the pair list,
 * the narrowphase and the solver size every grid from device-side counts, so that part is captured
 * once as a CUDA graph per solver mode and replayed while the world's sizes, capacities, parameters
 * and settings stay the same; off, the same kernels are launched one by one from the host.  Results
 * are identical either way.  With profiling on (pe_gpu_set_profiling) steps launch one by one. */
int pe_gpu_set_step_graphs(pe_gpu_world* w, int on);

/* Serving (no counterpart in the reference, which steps one World per caller): a request loop over
 * one device-resident world.  A request is a scene (the arrays of pe_gpu_set_shapes and
 * pe_gpu_set_bodies, indices local to the scene) and a number of steps.  Requests queue on
 * submission; each pe_gpu_server_step retires the requests that have run all their steps (their
 * final state is read back), admits queued requests in arrival order while their estimated device
 * footprint fits hbm_budget_bytes, and advances every live scene by one step in one batched step.
 * Live scenes keep their state, sweep axes and contact-result pools on the device between steps,
 * so a request's result is the one its scene gives stepped alone in a world of its own.  All
 * requests share dt, gravity, iterations and solver mode. */
typedef struct pe_gpu_scene {
    int n_shapes;
    const int* shape_type;
    const double* shape_param;                     /* [3 n_shapes] */
    const int* hull_vbeg; const int* hull_vcnt;    /* [n_shapes] */
    const int* hull_fbeg; const int* hull_fcnt;    /* [n_shapes] */
    int n_hull_verts; const double* hull_verts;    /* [3 n_hull_verts] */
    int n_hull_faces; const int* hull_face_off;    /* [n_hull_faces + 1] */
    const int* hull_face_idx;
    int n_bodies;
    const int* body_shape; const int* body_flags;
    const double* mass; const double* friction; const double* restitution; const double* lin_damp; const double* ang_damp;
    const double* origin; const double* basis; const double* lin_vel; const double* ang_vel;
} pe_gpu_scene;

typedef struct pe_gpu_server pe_gpu_server;
int pe_gpu_server_create(const pe_gpu_config* cfg, double dt, double gx, double gy, double gz, int iterations, int solver_mode,
                         double hbm_budget_bytes, pe_gpu_server** out);
int pe_gpu_server_destroy(pe_gpu_server* s);
const char* pe_gpu_server_last_error(const pe_gpu_server* s);
/* copies the scene; *id identifies the request.  n_steps must be at least 1 (PE_GPU_ERR_ARG otherwise). */
int pe_gpu_server_submit(pe_gpu_server* s, const pe_gpu_scene* scene, int n_steps, long long* id);
/* retire, admit, one batched step of all live scenes */
int pe_gpu_server_step(pe_gpu_server* s, int* n_live, int* n_queued);
/* *state: 0 queued, 1 running, 2 done (final origin / basis / velocities copied to the caller's
 * arrays of the scene's body count, and the request released), 3 rejected (larger than the budget) */
int pe_gpu_server_result(pe_gpu_server* s, long long id, int* state, double* origin, double* basis, double* lin_vel,
                         double* ang_vel);
/* out10: p50, p99 and mean device time per batched step (ms), batched steps, body-steps, requests
 * admitted, requests finished, peak charged footprint (bytes), live requests, queued requests */
int pe_gpu_server_stats(pe_gpu_server* s, double* out10);

/* Sweep-and-prune pairs of caller-supplied AABBs, allocating no memory.  This entry point has
 * no counterpart in the reference; it is a variant of the broadphase above (the same sort keys,
 * sweep, validation and pair order as BroadPhaseSweepAndPrune::calcCollisionPairs,
 * broad_phase_sweep_and_prune.cpp:6-41, for one scene, sorting along `axis`) for callers that may
 * not allocate device memory at the moment they need pairs: cudaMalloc and cudaFree can block or
 * synchronise the whole device, which stalls the other streams of a loop that keeps many scenes in
 * flight, and they are not allowed while a stream is being captured into a graph.
 *
 * All temporaries live in one fixed scratch array of about 1.4 MB per device, which limits n to
 * 16384 bodies; a larger n returns PE_GPU_ERR_CAPACITY with a message.  The first call on a device
 * looks the scratch up (cudaGetSymbolAddress, the device current) and caches it for the context
 * that is current; make that first call before any stream capture.  A call in another context of
 * the device (after cudaDeviceReset, or a context of the caller's own) looks it up again, and that
 * call, too, must come before any capture.  Without a current context the call makes the device's
 * primary context current.  The scratch is shared: calls on one device whose work overlaps (other
 * streams, other threads) race on it, so serialise them.  Nothing needs to start at zero: the call
 * initialises every scratch value it reads.
 *
 * Device pointers: aabb_min / aabb_max [3 n] floats (x, y, z per body), flags [n] PE_GPU_BODY_*
 * bits or NULL (all dynamic), pairs [2 pair_cap] ints (body indices, lower sweep position first),
 * n_pairs one int.  pairs must be 8-byte aligned (pairs are stored as 8-byte words) and the other
 * pointers 4-byte aligned; a misaligned pointer returns PE_GPU_ERR_ARG before any device work.
 * The work is queued on `stream` (a cudaStream_t, NULL for the default stream); *n_pairs holds
 * the pair count when it completes.  If that count exceeds pair_cap the output is incomplete:
 * call again with a larger buffer.  The call clears the runtime's last-error state on entry, so a
 * launch error it reports is its own.  err (optional) receives a message on failure. */
int pe_gpu_sap_pairs_noalloc(int device, int n, const float* aabb_min, const float* aabb_max, const int* flags, int axis,
                             int* pairs, int pair_cap, int* n_pairs, void* stream, char* err, int err_cap);

#ifdef __cplusplus
}
#endif
#endif /* PE_GPU_H */
