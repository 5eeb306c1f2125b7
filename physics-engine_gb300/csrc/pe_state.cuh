// Device-resident world state: structure-of-arrays layouts shared by the kernels.
#pragma once
#include <cstdint>
#include "pe_collide.cuh"

namespace pe {

// body fields, field-major: field k of body i at f[k * cap + i]
enum BodyField {
    OX = 0, OY, OZ,
    B00, B01, B02, B10, B11, B12, B20, B21, B22,
    VX, VY, VZ, WX, WY, WZ,
    TVX, TVY, TVZ, TWX, TWY, TWZ,       // solver temporary velocities
    MNX, MNY, MNZ, MXX, MXY, MXZ,       // AABB
    I00, I01, I02, I10, I11, I12, I20, I21, I22,   // world inverse inertia
    L00, L01, L02, L10, L11, L12, L20, L21, L22,   // local inverse inertia
    INVM, MASS, FRIC, REST, LDAMP, ADAMP, SCALE,   // SCALE: RigidBody::getAABBScale of the current AABB
    NBF
};
enum BodyFlag { BF_KINEMATIC = 1, BF_IGNORE = 2 };

template <class R> struct Bodies {
    R* f;
    int cap;
    int n;
    int* shape;
    int* flags;
    int* scene;
    __host__ __device__ R& at(int k, int i) const { return f[(size_t)k * cap + i]; }
#ifdef __CUDACC__
    __device__ Xf<R> xf(int i) const {
        Xf<R> t;
        t.o = V3<R>(at(OX, i), at(OY, i), at(OZ, i));
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) t.b.m[r][c] = at(B00 + r * 3 + c, i);
        return t;
    }
    __device__ M3<R> mat(int k0, int i) const {
        M3<R> m;
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) m.m[r][c] = at(k0 + r * 3 + c, i);
        return m;
    }
    __device__ V3<R> vec(int k0, int i) const { return V3<R>(at(k0, i), at(k0 + 1, i), at(k0 + 2, i)); }
    __device__ void set_vec(int k0, int i, const V3<R>& v) const { at(k0, i) = v.x; at(k0 + 1, i) = v.y; at(k0 + 2, i) = v.z; }
    __device__ void set_mat(int k0, int i, const M3<R>& m) const {
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) at(k0 + r * 3 + c, i) = m.m[r][c];
    }
#endif
};

// contact point fields written by the narrowphase, field-major over [cap*8] slots
enum PointField { PX = 0, PY, PZ, NX, NY, NZ, LAX, LAY, LAZ, LBX, LBY, LBZ, T0X, T0Y, T0Z, T1X, T1Y, T1Z, NPF };

template <class R> struct Results {
    int cap;          // result (pair) capacity
    int* a;           // [cap] body A
    int* b;           // [cap] body B
    int* npts;        // [cap] point_size
    R* fr;            // [cap] combined friction
    R* re;            // [cap] combined restitution
    R* pts;           // [NPF][cap*8]
    R* dist;          // [cap*8] slot distances after sorting (this step)
    const R* prev_dist;   // [prev_cap*8] slot distances of the previous step (stale-slot source)
    __host__ __device__ R& pt(int k, int slot) const { return pts[(size_t)k * cap * kSlots + slot]; }
};

// solver rows (FrictionContactConstraint::ConstraintInfo), field-major over [cap] rows
enum RowField { RAX = 0, RAY, RAZ, RBX, RBY, RBZ, RNX, RNY, RNZ, R0X, R0Y, R0Z, R1X, R1Y, R1Z,
                NRHS, NJMJ, T0JMJ, T1JMJ, MU, NACC, T0ACC, T1ACC, NRF };

template <class R> struct Rows {
    int cap;
    R* f;
    __host__ __device__ R& at(int k, int i) const { return f[(size_t)k * cap + i]; }
};

struct StepParams {
    double dt;
    double g[3];
    int iterations;
};

// device status word bits
enum StatusBits { ST_PAIR_OVERFLOW = 1, ST_ROW_OVERFLOW = 2, ST_COLOR_OVERFLOW = 4 };

} // namespace pe
