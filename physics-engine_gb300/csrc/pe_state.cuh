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
enum BodyFlag { BF_KINEMATIC = 1, BF_IGNORE = 2, BF_IGN_LIST = 4 };   // BF_IGN_LIST: the body has ignored partners

// RigidBody::_ignore_collision_ids as symmetric partner lists: body i never pairs with
// ids[off[i] .. off[i+1]); `order` maps sorted positions to bodies.  off == nullptr: no lists.
struct IgnoreLists {
    const int* off = nullptr;
    const int* ids = nullptr;
    const uint32_t* order = nullptr;
#ifdef __CUDACC__
    __device__ bool ignored(int pi, int pj) const {   // sorted positions pi, pj
        const int a = (int)order[pi], b = (int)order[pj];
        for (int k = off[a], e = off[a + 1]; k < e; k++)
            if (ids[k] == b) return true;
        return false;
    }
#endif
};

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

// joint constraints (World::addConstraint, in order): Ball/Hinge/SliderJointConstraint
enum JointType { JT_BALL = 0, JT_HINGE = 1, JT_SLIDER = 2 };
enum JointParam { JP_ANCHOR_A = 0, JP_ANCHOR_B = 3, JP_AXIS_A = 6, JP_AXIS_B = 9, JP_MIN = 12, JP_MAX = 13, JP_SPEED = 14, NJP = 15 };
// per-step solver data of one joint (initSequentialImpulse), joint-major
enum JointRow { JR_RA = 0, JR_RB = 3, JR_WAX = 6, JR_T0 = 9, JR_T1 = 12, JR_RHS_BALL = 15, JR_JMJ_BALL = 18, JR_JMJ_ROT = 27,
                JR_RHS2 = 36, JR_JMJ2 = 38, JR_JMJ_ML = 40, JR_RHS_MOTOR = 41, JR_RHS_LIMIT = 42, JR_LIMIT = 43, NJR = 44 };
template <class R> struct Joints {
    int n = 0;
    const int* type = nullptr;
    const int2* body = nullptr;    // (a, b)
    const int* flag = nullptr;     // bit 0 use_limits, bit 1 use_motor
    const R* param = nullptr;      // [NJP * n]
    R* row = nullptr;              // [NJR * n]
};

struct StepParams {
    double dt;
    double g[3];
    int iterations;
};

// Scheduling settings of the step: which kernel takes which work and with how many threads.  In
// serial-order mode no setting changes a result bit.  In coloured mode none does either while every
// island needs at most exact_levels_colored levels (above, a big island takes first-fit colours and
// a block-path island runs its leftover items last): the autotuner leaves that one setting alone.
struct Tuning {
    int sat_heavy_cost = 200000;      // SAT pairs whose estimated work reaches this run on a block of warps
    int small_island_items = 8;       // islands up to this many items run on one thread each
    int big_island_items = 4096;      // islands above this many items are coloured and solved grid-wide
    int color_block = 64;             // threads per island block, coloured mode
    int level_block = 256;            // threads per island block, serial-order mode
    int exact_levels_colored = 512;   // coloured mode keeps a big island's exact levels up to this many
    int scene_sort_max = 2048;        // scenes up to this many bodies are sorted inside one block
    int side_streams = 4;             // streams the narrowphase's per-class kernels are spread over
};

// device status word bits
enum StatusBits { ST_PAIR_OVERFLOW = 1, ST_ROW_OVERFLOW = 2, ST_COLOR_OVERFLOW = 4 };

} // namespace pe
