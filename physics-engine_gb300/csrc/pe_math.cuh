// Device (and host) math for the rigid-body step: 3-vectors, row-major 3x3 matrices,
// rigid transforms and quaternions, templated on the scalar type R (float or double).
//
// Every reduction reproduces the rounding order the reference engine gets from Eigen 3.4
// (g++ -O2, x86-64), so that results match the reference bit for bit when the kernels are
// compiled without FMA contraction (--fmad=false):
//   double: M*v and M*M rows 0,1 summed left-to-right, row 2 right-to-left;
//           M^T*v, M^T*M, dot, squaredNorm left-to-right;
//           R*I*R^T of RigidBody::updateWorldInertia: inner product as M*M, outer right-to-left.
//   float : every 3-term sum right-to-left.
//   both  : quaternion trace right-to-left, norm (x^2+z^2)+(y^2+w^2), product in the order of
//           Eigen's SSE quaternion kernel (it differs between float and double).
// Reference call sites: src/rigid/object/rigidbody.cpp:43-46, :207-243 and
// SimpleViewer/include/common/transform.cpp.
#pragma once
#include <cmath>
#include <type_traits>

#ifdef __CUDACC__
#define PE_HD __host__ __device__ __forceinline__
#else
#define PE_HD inline
#endif

namespace pe {

template <class R> struct Lim;
template <> struct Lim<double> {
    PE_HD static double max() { return 1e100; }
    PE_HD static double min() { return -1e100; }
};
template <> struct Lim<float> {
    PE_HD static float max() { return static_cast<float>(1e30); }
    PE_HD static float min() { return static_cast<float>(-1e30); }
};
template <class R> PE_HD R eps() { return R(0.00001); }
template <class R> PE_HD R pi() { return R(3.141592653589); }
template <class R> PE_HD constexpr bool dbl() { return std::is_same<R, double>::value; }

PE_HD float real_sqrt(float x) { return sqrtf(x); }
PE_HD double real_sqrt(double x) { return sqrt(x); }
PE_HD float rabs(float x) { return fabsf(x); }
PE_HD double rabs(double x) { return fabs(x); }
template <class R> PE_HD R rmin(R a, R b) { return a < b ? a : b; }
template <class R> PE_HD R rmax(R a, R b) { return a > b ? a : b; }
template <class R> PE_HD R rclamp(R x, R lo, R hi) { return rmax(rmin(x, hi), lo); }

template <class R> PE_HD R sum3(R a, R b, R c, bool l2r) { return l2r ? (a + b) + c : a + (b + c); }

template <class R> struct V3 {
    R x, y, z;
    PE_HD V3() : x(0), y(0), z(0) {}
    PE_HD V3(R a, R b, R c) : x(a), y(b), z(c) {}
    PE_HD R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    PE_HD R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> PE_HD V3<R> operator+(const V3<R>& a, const V3<R>& b) { return V3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> PE_HD V3<R> operator-(const V3<R>& a, const V3<R>& b) { return V3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> PE_HD V3<R> operator-(const V3<R>& a) { return V3<R>(-a.x, -a.y, -a.z); }
template <class R> PE_HD V3<R> operator*(const V3<R>& a, R s) { return V3<R>(a.x * s, a.y * s, a.z * s); }
template <class R> PE_HD V3<R> operator*(R s, const V3<R>& a) { return V3<R>(s * a.x, s * a.y, s * a.z); }
template <class R> PE_HD V3<R> operator/(const V3<R>& a, R s) { return V3<R>(a.x / s, a.y / s, a.z / s); }
template <class R> PE_HD V3<R> cmul(const V3<R>& a, const V3<R>& b) { return V3<R>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class R> PE_HD V3<R> cross(const V3<R>& a, const V3<R>& b) {
    return V3<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> PE_HD R dot(const V3<R>& a, const V3<R>& b) { return sum3(a.x * b.x, a.y * b.y, a.z * b.z, dbl<R>()); }
template <class R> PE_HD R sqnorm(const V3<R>& a) { return dot(a, a); }
template <class R> PE_HD R norm(const V3<R>& a) { return real_sqrt(sqnorm(a)); }
template <class R> PE_HD V3<R> normalized(const V3<R>& a) {
    const R n = sqnorm(a);
    return n > R(0) ? a / real_sqrt(n) : a;
}

template <class R> struct M3 {
    R m[3][3];
    PE_HD M3() { for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) m[i][j] = 0; }
    PE_HD static M3 identity() { M3 o; o.m[0][0] = o.m[1][1] = o.m[2][2] = R(1); return o; }
    PE_HD V3<R> col(int c) const { return V3<R>(m[0][c], m[1][c], m[2][c]); }
    PE_HD M3 transpose() const { M3 o; for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) o.m[r][c] = m[c][r]; return o; }
};

template <class R> PE_HD V3<R> mv(const M3<R>& a, const V3<R>& v) {   // M*v
    return V3<R>(sum3(a.m[0][0] * v.x, a.m[0][1] * v.y, a.m[0][2] * v.z, dbl<R>()),
                 sum3(a.m[1][0] * v.x, a.m[1][1] * v.y, a.m[1][2] * v.z, dbl<R>()),
                 sum3(a.m[2][0] * v.x, a.m[2][1] * v.y, a.m[2][2] * v.z, false));
}
template <class R> PE_HD V3<R> mtv(const M3<R>& a, const V3<R>& v) {   // M^T*v
    return V3<R>(sum3(a.m[0][0] * v.x, a.m[1][0] * v.y, a.m[2][0] * v.z, dbl<R>()),
                 sum3(a.m[0][1] * v.x, a.m[1][1] * v.y, a.m[2][1] * v.z, dbl<R>()),
                 sum3(a.m[0][2] * v.x, a.m[1][2] * v.y, a.m[2][2] * v.z, dbl<R>()));
}
template <class R> PE_HD M3<R> mm(const M3<R>& a, const M3<R>& b) {   // A*B
    M3<R> o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            o.m[i][j] = sum3(a.m[i][0] * b.m[0][j], a.m[i][1] * b.m[1][j], a.m[i][2] * b.m[2][j], dbl<R>() && i < 2);
    return o;
}
template <class R> PE_HD M3<R> mtm(const M3<R>& a, const M3<R>& b) {   // A^T*B
    M3<R> o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            o.m[i][j] = sum3(a.m[0][i] * b.m[0][j], a.m[1][i] * b.m[1][j], a.m[2][i] * b.m[2][j], dbl<R>());
    return o;
}
// world inverse inertia R * I * R^T as RigidBody::updateWorldInertia evaluates it
template <class R> PE_HD M3<R> world_inertia(const M3<R>& rot, const M3<R>& local) {
    const M3<R> t = mm(rot, local);
    M3<R> o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            o.m[i][j] = t.m[i][0] * rot.m[j][0] + (t.m[i][1] * rot.m[j][1] + t.m[i][2] * rot.m[j][2]);
    return o;
}
// Eigen's closed-form 3x3 inverse
// (compute_inverse<..., 3>: the determinant expands the cofactors of column 0, and entry (r, c)
// of the inverse is cofactor (c, r) / det; exact for matrices that are not bitwise symmetric)
template <class R> PE_HD M3<R> inverse3(const M3<R>& a) {
    auto cof = [&](int i, int j) {   // cofactor_3x3<i, j>
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        return a.m[i1][j1] * a.m[i2][j2] - a.m[i1][j2] * a.m[i2][j1];
    };
    const R det = sum3(cof(0, 0) * a.m[0][0], cof(1, 0) * a.m[1][0], cof(2, 0) * a.m[2][0], dbl<R>());
    const R inv = R(1) / det;
    M3<R> o;
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) o.m[r][c] = cof(c, r) * inv;
    return o;
}

template <class R> struct Xf {   // rigid transform: basis + origin
    M3<R> b;
    V3<R> o;
    PE_HD V3<R> apply(const V3<R>& v) const { return mv(b, v) + o; }
    PE_HD V3<R> inv_apply(const V3<R>& v) const { return mtv(b, v - o); }
    PE_HD Xf inverse() const {
        Xf r;
        r.b = b.transpose();
        r.o = V3<R>(sum3((-b.m[0][0]) * o.x, (-b.m[1][0]) * o.y, (-b.m[2][0]) * o.z, dbl<R>()),
                    sum3((-b.m[0][1]) * o.x, (-b.m[1][1]) * o.y, (-b.m[2][1]) * o.z, dbl<R>()),
                    sum3((-b.m[0][2]) * o.x, (-b.m[1][2]) * o.y, (-b.m[2][2]) * o.z, dbl<R>()));
        return r;
    }
    PE_HD Xf operator*(const Xf& t) const { Xf r; r.b = mm(b, t.b); r.o = mv(b, t.o) + o; return r; }
};

template <class R> struct Quat { R x, y, z, w; };

template <class R> PE_HD Quat<R> quat_from_basis(const M3<R>& m) {
    Quat<R> q;
    R t = m.m[0][0] + (m.m[1][1] + m.m[2][2]);
    if (t > R(0)) {
        t = real_sqrt(t + R(1));
        q.w = R(0.5) * t;
        t = R(0.5) / t;
        q.x = (m.m[2][1] - m.m[1][2]) * t;
        q.y = (m.m[0][2] - m.m[2][0]) * t;
        q.z = (m.m[1][0] - m.m[0][1]) * t;
    } else {
        int i = 0;
        if (m.m[1][1] > m.m[0][0]) i = 1;
        if (m.m[2][2] > m.m[i][i]) i = 2;
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        t = real_sqrt(m.m[i][i] - m.m[j][j] - m.m[k][k] + R(1));
        R c[3];
        c[i] = R(0.5) * t;
        t = R(0.5) / t;
        q.w = (m.m[k][j] - m.m[j][k]) * t;
        c[j] = (m.m[j][i] + m.m[i][j]) * t;
        c[k] = (m.m[k][i] + m.m[i][k]) * t;
        q.x = c[0]; q.y = c[1]; q.z = c[2];
    }
    return q;
}

template <class R> PE_HD Quat<R> quat_mul(const Quat<R>& a, const Quat<R>& b) {
    Quat<R> r;
    if (dbl<R>()) {
        r.x = (a.w * b.x + a.y * b.z) - (a.z * b.y - a.x * b.w);
        r.y = (a.w * b.y + a.y * b.w) + (a.z * b.x - a.x * b.z);
        r.z = (a.w * b.z - a.y * b.x) + (a.z * b.w + a.x * b.y);
        r.w = (a.w * b.w - a.y * b.y) - (a.z * b.z + a.x * b.x);
    } else {
        r.x = (a.x * b.w - a.z * b.y) + (a.y * b.z + a.w * b.x);
        r.y = (a.y * b.w - a.x * b.z) + (a.z * b.x + a.w * b.y);
        r.z = (a.z * b.w - a.y * b.x) + (a.x * b.y + a.w * b.z);
        r.w = (a.w * b.w - a.x * b.x) - (a.z * b.z + a.y * b.y);
    }
    return r;
}

template <class R> PE_HD void quat_normalize(Quat<R>& q) {
    const R n2 = (q.x * q.x + q.z * q.z) + (q.y * q.y + q.w * q.w);
    if (n2 > R(0)) {
        const R n = real_sqrt(n2);
        q.x = q.x / n; q.y = q.y / n; q.z = q.z / n; q.w = q.w / n;
    }
}

template <class R> PE_HD M3<R> quat_to_basis(const Quat<R>& q) {
    const R tx = R(2) * q.x, ty = R(2) * q.y, tz = R(2) * q.z;
    const R twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const R txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const R tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    M3<R> r;
    r.m[0][0] = R(1) - (tyy + tzz); r.m[0][1] = txy - twz;          r.m[0][2] = txz + twy;
    r.m[1][0] = txy + twz;          r.m[1][1] = R(1) - (txx + tzz); r.m[1][2] = tyz - twx;
    r.m[2][0] = txz - twy;          r.m[2][1] = tyz + twx;          r.m[2][2] = R(1) - (txx + tyy);
    return r;
}

} // namespace pe
