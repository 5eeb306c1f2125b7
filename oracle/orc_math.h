// Oracle math layer: 3-vectors, 3x3 matrices, transforms and quaternions with the
// exact floating-point evaluation order the reference gets from Eigen 3.4
// (ThirdParty/Eigen, compiled by g++ -O2 for x86-64/SSE2).  Test infrastructure only.
//
// Order rules (measured against Eigen itself; a 3-term sum is either
// left-to-right  (a+b)+c  or right-to-left  a+(b+c)):
//   double: M*v and M*M   -> rows 0,1 left-to-right, row 2 right-to-left
//           M^T*v, M^T*M  -> left-to-right;  dot / squaredNorm -> left-to-right
//   float : every 3-term reduction right-to-left
//   both  : trace right-to-left; quaternion norm (x^2+z^2)+(y^2+w^2);
//           quaternion product = Eigen's SSE path (Geometry/arch/Geometry_SIMD.h).
// The reference's own usage: src/rigid/object/rigidbody.cpp:43-46 (world inertia),
// :220-227 (quaternion integration), SimpleViewer/include/common/transform.cpp (Transform).
#pragma once
#include <cmath>
#include <cstdint>
#include <type_traits>

namespace orc {

template <class R> struct V3 {
    R x = 0, y = 0, z = 0;
    V3() = default;
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <class R> inline V3<R> operator+(const V3<R>& a, const V3<R>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(const V3<R>& a, const V3<R>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(const V3<R>& a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(const V3<R>& a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, const V3<R>& a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(const V3<R>& a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline V3<R> cmul(const V3<R>& a, const V3<R>& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> cross(const V3<R>& a, const V3<R>& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

template <class R> constexpr bool is_double() { return std::is_same<R, double>::value; }
template <class R> inline R sum3(R a, R b, R c, bool l2r) { return l2r ? (a + b) + c : a + (b + c); }

template <class R> inline R dot(const V3<R>& a, const V3<R>& b) { return sum3(a.x * b.x, a.y * b.y, a.z * b.z, is_double<R>()); }
template <class R> inline R sqnorm(const V3<R>& a) { return dot(a, a); }
template <class R> inline R norm(const V3<R>& a) { return std::sqrt(sqnorm(a)); }
template <class R> inline V3<R> normalized(const V3<R>& a) {
    R n = sqnorm(a);
    return n > R(0) ? a / std::sqrt(n) : a;
}

// row-major storage m[r][c]
template <class R> struct M3 {
    R m[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    static M3 identity() { M3 o; o.m[0][0] = o.m[1][1] = o.m[2][2] = R(1); return o; }
    V3<R> col(int c) const { return {m[0][c], m[1][c], m[2][c]}; }
    M3 transpose() const { M3 o; for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) o.m[r][c] = m[c][r]; return o; }
};

// M*v
template <class R> inline V3<R> mv(const M3<R>& a, const V3<R>& v) {
    V3<R> o;
    for (int i = 0; i < 3; i++) o[i] = sum3(a.m[i][0] * v.x, a.m[i][1] * v.y, a.m[i][2] * v.z, is_double<R>() && i < 2);
    return o;
}
// M^T*v (Eigen transpose expression)
template <class R> inline V3<R> mtv(const M3<R>& a, const V3<R>& v) {
    V3<R> o;
    for (int i = 0; i < 3; i++) o[i] = sum3(a.m[0][i] * v.x, a.m[1][i] * v.y, a.m[2][i] * v.z, is_double<R>());
    return o;
}
// A*B (B plain or a transpose expression)
template <class R> inline M3<R> mm(const M3<R>& a, const M3<R>& b) {
    M3<R> o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            o.m[i][j] = sum3(a.m[i][0] * b.m[0][j], a.m[i][1] * b.m[1][j], a.m[i][2] * b.m[2][j], is_double<R>() && i < 2);
    return o;
}
// A*B^T summed right-to-left in every row: the order Eigen produces for the outer product of
// RigidBody::updateWorldInertia (rigidbody.cpp:43-46), measured at that call site
template <class R> inline M3<R> mmt_r2l(const M3<R>& a, const M3<R>& b) {
    M3<R> o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            o.m[i][j] = a.m[i][0] * b.m[j][0] + (a.m[i][1] * b.m[j][1] + a.m[i][2] * b.m[j][2]);
    return o;
}
// A^T*B (A a transpose expression)
template <class R> inline M3<R> mtm(const M3<R>& a, const M3<R>& b) {
    M3<R> o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            o.m[i][j] = sum3(a.m[0][i] * b.m[0][j], a.m[1][i] * b.m[1][j], a.m[2][i] * b.m[2][j], is_double<R>());
    return o;
}
template <class R> inline M3<R> mscale(const M3<R>& a, R s) {
    M3<R> o;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.m[i][j] = a.m[i][j] * s;
    return o;
}

// Eigen's closed-form 3x3 inverse (Eigen/src/LU/InverseImpl.h, compute_inverse<..., 3>): the
// determinant expands the cofactors of column 0; entry (r, c) of the inverse is cofactor (c, r) / det
template <class R> inline M3<R> inverse3(const M3<R>& a) {
    auto cof = [&](int i, int j) {   // cofactor_3x3<i, j>
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        return a.m[i1][j1] * a.m[i2][j2] - a.m[i1][j2] * a.m[i2][j1];
    };
    const R det = sum3(cof(0, 0) * a.m[0][0], cof(1, 0) * a.m[1][0], cof(2, 0) * a.m[2][0], is_double<R>());
    const R inv = R(1) / det;
    M3<R> o;
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) o.m[r][c] = cof(c, r) * inv;
    return o;
}

template <class R> struct Transform {
    M3<R> basis = M3<R>::identity();
    V3<R> origin;
    V3<R> apply(const V3<R>& v) const { return mv(basis, v) + origin; }              // T * v
    V3<R> inv_apply(const V3<R>& v) const { return mtv(basis, v - origin); }         // inverseTransform
    Transform inverse() const {                                                       // transform.cpp inverse()
        Transform o;
        o.basis = basis.transpose();
        V3<R> r;
        for (int i = 0; i < 3; i++) r[i] = sum3((-basis.m[0][i]) * origin.x, (-basis.m[1][i]) * origin.y, (-basis.m[2][i]) * origin.z, is_double<R>());
        o.origin = r;
        return o;
    }
    Transform operator*(const Transform& t) const { return {mm(basis, t.basis), mv(basis, t.origin) + origin}; }
};

// quaternion stored (x, y, z, w) like Eigen's coeffs()
template <class R> struct Quat { R x = 0, y = 0, z = 0, w = 1; };

// Quaternion(Matrix3): Eigen's branch on the trace (trace summed right-to-left)
template <class R> inline Quat<R> quat_from_basis(const M3<R>& m) {
    Quat<R> q;
    R t = m.m[0][0] + (m.m[1][1] + m.m[2][2]);
    if (t > R(0)) {
        t = std::sqrt(t + R(1));
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
        t = std::sqrt(m.m[i][i] - m.m[j][j] - m.m[k][k] + R(1));
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

// a*b with Eigen's vectorised operation order (differs between float and double)
template <class R> inline Quat<R> quat_mul(const Quat<R>& a, const Quat<R>& b) {
    Quat<R> r;
    if (is_double<R>()) {
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

template <class R> inline void quat_normalize(Quat<R>& q) {
    const R n2 = (q.x * q.x + q.z * q.z) + (q.y * q.y + q.w * q.w);
    if (n2 > R(0)) {
        const R n = std::sqrt(n2);
        q.x /= n; q.y /= n; q.z /= n; q.w /= n;
    }
}

template <class R> inline M3<R> quat_to_basis(const Quat<R>& q) {
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

template <class R> struct Limits;
template <> struct Limits<double> { static constexpr double max() { return 1e100; } static constexpr double min() { return -1e100; } };
template <> struct Limits<float> { static constexpr float max() { return static_cast<float>(1e30); } static constexpr float min() { return static_cast<float>(-1e30); } };

template <class R> constexpr R kEps() { return R(0.00001); }
template <class R> constexpr R kPi() { return R(3.141592653589); }

} // namespace orc
