// Host-side preprocessing shared by the world implementations: unit meshes, convex-mesh
// preparation and per-body mass properties.  Runs once per scene upload, never per step.
#pragma once
#include <vector>
#include "pe_math.cuh"

namespace pe {

struct UnitMeshes;

// Fills the reference's unit box and 20-gon cylinder meshes (default_mesh.h:7-273).
void build_unit_meshes(UnitMeshes& u);

// A convex mesh after ConvexMeshShape::setMesh (convex_mesh_shape.cpp:12-131): vertices
// recentred on the centre of mass, faces in the order the face tree leaves them, per-face
// bounding boxes, unique edges, unit-density inertia about the centre of mass.
template <class R> struct HullPrep {
    std::vector<R> v;                 // [nv*3]
    std::vector<int> f_off, f_idx;    // [nf+1], local vertex indices
    std::vector<R> f_n, f_min, f_max; // [nf*3]
    std::vector<R> e_a, e_b;          // [ne*3]
    M3<R> inertia;                    // per unit mass (divided by the volume)
    R volume = 0;
    R inner = -1, outer = 0;          // balls about the local origin inside / around the hull (-1: none certified)
    std::vector<int> l_beg, l_cnt;    // concave meshes: face-tree leaves in tree order (face ranges)
    std::vector<R> l_min, l_max;      // [nl*3] leaf boxes
};
// ConvexMeshShape::setMesh, or ConcaveMeshShape::setMesh with `concave`
template <class R> HullPrep<R> prepare_hull(const double* verts, int nv, const int* face_off, const int* face_idx, int nf,
                                            bool concave = false);

// A scene as a caller describes it (the arrays of pe_gpu_set_shapes and pe_gpu_set_bodies), owned
// on the host; shape indices of the bodies and hull indices are local to the scene.
struct SceneData {
    std::vector<int> shape_type, hull_vbeg, hull_vcnt, hull_fbeg, hull_fcnt, hull_face_off, hull_face_idx;
    std::vector<double> shape_param, hull_verts;
    std::vector<int> body_shape, body_flags;
    std::vector<double> mass, friction, restitution, lin_damp, ang_damp, origin, basis, lin_vel, ang_vel;
    int n_shapes() const { return (int)shape_type.size(); }
    int n_bodies() const { return (int)body_shape.size(); }
};

// unit-mass local inertia of the analytic shapes (box_shape.cpp:16-23, sphere_shape.cpp:7-11,
// cylinder_shape.cpp:25-31)
template <class R> M3<R> box_inertia(const V3<R>& size);
template <class R> M3<R> sphere_inertia(R r);
template <class R> M3<R> cylinder_inertia(R r, R h);

} // namespace pe
