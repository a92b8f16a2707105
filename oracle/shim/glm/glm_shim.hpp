// Oracle test infrastructure: a minimal glm-compatible header set, written from
// the mathematics, covering exactly the glm surface that the reference's
// collision path uses (inMyRoom_vulkan/src/Geometry/{OBB,OBBtree,Paralgram,
// Triangle,Plane,Ray}.cpp and src/CollisionDetection/*.cpp).
//
// glm itself is an un-vendored submodule of the reference (a fork whose pinned
// commit is not available), so the operation order inside these functions is a
// convention of this shim, shared bit-for-bit by the CUDA path:
//   dot(a,b)          = (a.x*b.x + a.y*b.y) + a.z*b.z           (left to right)
//   length(v)         = sqrt(dot(v,v))
//   normalize(v)      = v * (1 / sqrt(dot(v,v)))
//   mat4 * vec4       = (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w)   (pairwise)
//   mat3 * vec3       = (c0*v.x + c1*v.y) + c2*v.z              (left to right)
//   mat4 * mat4       = column j: ((a0*b.x + a1*b.y) + a2*b.z) + a3*b.w
//   inverse(mat4)     = adjugate from 2x2 minors, times 1/det
// Default constructors zero-initialise (value semantics without indeterminate
// reads).
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <utility>
#include <algorithm>

namespace glm {

template <class T> struct tvec2 {
    T x{}, y{};
    constexpr tvec2() = default;
    constexpr explicit tvec2(T s) : x(s), y(s) {}
    constexpr tvec2(T a, T b) : x(a), y(b) {}
    template <class U> constexpr tvec2(const tvec2<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)) {}
    T& operator[](std::size_t i) { return i == 0 ? x : y; }
    const T& operator[](std::size_t i) const { return i == 0 ? x : y; }
};

template <class T> struct tvec4;

template <class T> struct tvec3 {
    T x{}, y{}, z{};
    constexpr tvec3() = default;
    constexpr explicit tvec3(T s) : x(s), y(s), z(s) {}
    constexpr tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <class U> constexpr tvec3(const tvec3<U>& o)
        : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    // implicit, as glm's own (no GLM_FORCE_EXPLICIT_CTOR): the reference
    // returns a vec4 where a vec3 is expected (ShootUncollideRays.cpp:94)
    template <class U> constexpr tvec3(const tvec4<U>& o)
        : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    T& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
    tvec3& operator+=(const tvec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    tvec3& operator-=(const tvec3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    tvec3& operator*=(T s) { x = x * s; y = y * s; z = z * s; return *this; }
    tvec3& operator/=(T s) { x = x / s; y = y / s; z = z / s; return *this; }
};

template <class T> struct tvec4 {
    T x{}, y{}, z{}, w{};
    constexpr tvec4() = default;
    constexpr explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
    constexpr tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    constexpr tvec4(const tvec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    template <class U> constexpr tvec4(const tvec4<U>& o)
        : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)), w(static_cast<T>(o.w)) {}
    T& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const T& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    tvec4& operator+=(const tvec4& o) { x = x + o.x; y = y + o.y; z = z + o.z; w = w + o.w; return *this; }
    tvec4& operator-=(const tvec4& o) { x = x - o.x; y = y - o.y; z = z - o.z; w = w - o.w; return *this; }
};

// ---- vector arithmetic (component-wise, one rounding per component) ----
template <class T> inline tvec2<T> operator+(const tvec2<T>& a, const tvec2<T>& b) { return {a.x + b.x, a.y + b.y}; }
template <class T> inline tvec2<T> operator-(const tvec2<T>& a, const tvec2<T>& b) { return {a.x - b.x, a.y - b.y}; }
template <class T> inline tvec2<T> operator*(T s, const tvec2<T>& v) { return {s * v.x, s * v.y}; }

template <class T> inline tvec3<T> operator+(const tvec3<T>& a, const tvec3<T>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline tvec3<T> operator-(const tvec3<T>& a, const tvec3<T>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline tvec3<T> operator-(const tvec3<T>& a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline tvec3<T> operator*(const tvec3<T>& a, const tvec3<T>& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline tvec3<T> operator*(const tvec3<T>& v, T s) { return {v.x * s, v.y * s, v.z * s}; }
template <class T> inline tvec3<T> operator*(T s, const tvec3<T>& v) { return {s * v.x, s * v.y, s * v.z}; }
template <class T> inline tvec3<T> operator/(const tvec3<T>& v, T s) { return {v.x / s, v.y / s, v.z / s}; }
template <class T> inline tvec3<T> operator/(const tvec3<T>& a, const tvec3<T>& b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> inline bool operator==(const tvec3<T>& a, const tvec3<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class T> inline bool operator!=(const tvec3<T>& a, const tvec3<T>& b) { return !(a == b); }

template <class T> inline tvec4<T> operator+(const tvec4<T>& a, const tvec4<T>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class T> inline tvec4<T> operator-(const tvec4<T>& a, const tvec4<T>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
template <class T> inline tvec4<T> operator*(const tvec4<T>& v, T s) { return {v.x * s, v.y * s, v.z * s, v.w * s}; }
template <class T> inline tvec4<T> operator*(T s, const tvec4<T>& v) { return {s * v.x, s * v.y, s * v.z, s * v.w}; }
template <class T> inline bool operator==(const tvec4<T>& a, const tvec4<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }
template <class T> inline bool operator!=(const tvec4<T>& a, const tvec4<T>& b) { return !(a == b); }

// ---- matrices: column-major, m[i] is column i ----
template <class T> struct tmat4;

template <class T> struct tmat3 {
    tvec3<T> c[3];
    constexpr tmat3() = default;
    constexpr explicit tmat3(T s) : c{tvec3<T>(s, 0, 0), tvec3<T>(0, s, 0), tvec3<T>(0, 0, s)} {}
    constexpr tmat3(T a0, T a1, T a2, T b0, T b1, T b2, T d0, T d1, T d2)
        : c{tvec3<T>(a0, a1, a2), tvec3<T>(b0, b1, b2), tvec3<T>(d0, d1, d2)} {}
    constexpr tmat3(const tvec3<T>& a, const tvec3<T>& b, const tvec3<T>& d) : c{a, b, d} {}
    explicit tmat3(const tmat4<T>& m);
    tvec3<T>& operator[](std::size_t i) { return c[i]; }
    const tvec3<T>& operator[](std::size_t i) const { return c[i]; }
    tmat3& operator/=(T s) { for (auto& col : c) col /= s; return *this; }
};

template <class T> struct tmat4 {
    tvec4<T> c[4];
    constexpr tmat4() = default;
    constexpr explicit tmat4(T s)
        : c{tvec4<T>(s, 0, 0, 0), tvec4<T>(0, s, 0, 0), tvec4<T>(0, 0, s, 0), tvec4<T>(0, 0, 0, s)} {}
    constexpr tmat4(const tvec4<T>& a, const tvec4<T>& b, const tvec4<T>& d, const tvec4<T>& e) : c{a, b, d, e} {}
    tvec4<T>& operator[](std::size_t i) { return c[i]; }
    const tvec4<T>& operator[](std::size_t i) const { return c[i]; }
};

template <class T> inline tmat3<T>::tmat3(const tmat4<T>& m)
    : c{tvec3<T>(m[0]), tvec3<T>(m[1]), tvec3<T>(m[2])} {}

template <class T> inline bool operator==(const tmat4<T>& a, const tmat4<T>& b) {
    return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
}
template <class T> inline bool operator!=(const tmat4<T>& a, const tmat4<T>& b) { return !(a == b); }

template <class T> inline tvec4<T> operator*(const tmat4<T>& m, const tvec4<T>& v) {
    tvec4<T> p0 = m[0] * v.x;
    tvec4<T> p1 = m[1] * v.y;
    tvec4<T> p2 = m[2] * v.z;
    tvec4<T> p3 = m[3] * v.w;
    return (p0 + p1) + (p2 + p3);
}

template <class T> inline tvec3<T> operator*(const tmat3<T>& m, const tvec3<T>& v) {
    tvec3<T> p0 = m[0] * v.x;
    tvec3<T> p1 = m[1] * v.y;
    tvec3<T> p2 = m[2] * v.z;
    return (p0 + p1) + p2;
}

template <class T> inline tmat4<T> operator*(const tmat4<T>& a, const tmat4<T>& b) {
    tmat4<T> r;
    for (int j = 0; j < 4; ++j) {
        tvec4<T> acc = a[0] * b[j].x;
        acc = acc + a[1] * b[j].y;
        acc = acc + a[2] * b[j].z;
        acc = acc + a[3] * b[j].w;
        r[j] = acc;
    }
    return r;
}

// ---- functions ----
template <class T> inline T dot(const tvec3<T>& a, const tvec3<T>& b) {
    T s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}
template <class T> inline tvec3<T> cross(const tvec3<T>& a, const tvec3<T>& b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class T> inline T length(const tvec3<T>& v) { return std::sqrt(dot(v, v)); }
template <class T> inline tvec3<T> normalize(const tvec3<T>& v) {
    T inv = T(1) / std::sqrt(dot(v, v));
    return v * inv;
}
template <class T> inline T radians(T deg) { return deg * static_cast<T>(0.01745329251994329576923690768489); }

template <class T> inline T* value_ptr(tmat3<T>& m) { return &m.c[0].x; }
template <class T> inline const T* value_ptr(const tmat3<T>& m) { return &m.c[0].x; }
template <class T> inline T* value_ptr(tmat4<T>& m) { return &m.c[0].x; }
template <class T> inline const T* value_ptr(const tmat4<T>& m) { return &m.c[0].x; }
template <class T> inline T* value_ptr(tvec3<T>& v) { return &v.x; }
template <class T> inline const T* value_ptr(const tvec3<T>& v) { return &v.x; }

// Cofactor matrix of a 3x3 (the transpose of its adjugate): the matrix that maps
// normals under the linear part of a transform, up to the factor det.
template <class T> inline tmat3<T> adjointTranspose(const tmat3<T>& m) {
    tmat3<T> r;
    // r[col][row] = cofactor(row, col) of m indexed m[col][row]
    r[0][0] = m[1][1] * m[2][2] - m[2][1] * m[1][2];
    r[0][1] = m[2][0] * m[1][2] - m[1][0] * m[2][2];
    r[0][2] = m[1][0] * m[2][1] - m[2][0] * m[1][1];
    r[1][0] = m[2][1] * m[0][2] - m[0][1] * m[2][2];
    r[1][1] = m[0][0] * m[2][2] - m[2][0] * m[0][2];
    r[1][2] = m[2][0] * m[0][1] - m[0][0] * m[2][1];
    r[2][0] = m[0][1] * m[1][2] - m[1][1] * m[0][2];
    r[2][1] = m[1][0] * m[0][2] - m[0][0] * m[1][2];
    r[2][2] = m[0][0] * m[1][1] - m[1][0] * m[0][1];
    return r;
}

// Inverse of a 4x4 by the Laplace expansion over 2x2 minors of rows {0,1}
// and rows {2,3}; a(r,c) = m[c][r].
template <class T> inline tmat4<T> inverse(const tmat4<T>& m) {
    auto a = [&](int r, int c) { return m[c][r]; };
    // 2x2 minors of the top two rows (s) and the bottom two rows (q), columns (i,j)
    T s01 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1);
    T s02 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2);
    T s03 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3);
    T s12 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2);
    T s13 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3);
    T s23 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
    T q01 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
    T q02 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2);
    T q03 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3);
    T q12 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2);
    T q13 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3);
    T q23 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3);

    T det = s01 * q23 - s02 * q13 + s03 * q12 + s12 * q03 - s13 * q02 + s23 * q01;
    T inv = T(1) / det;

    T b[4][4];  // b[r][c] of the inverse
    b[0][0] = ( a(1, 1) * q23 - a(1, 2) * q13 + a(1, 3) * q12) * inv;
    b[0][1] = (-a(0, 1) * q23 + a(0, 2) * q13 - a(0, 3) * q12) * inv;
    b[0][2] = ( a(3, 1) * s23 - a(3, 2) * s13 + a(3, 3) * s12) * inv;
    b[0][3] = (-a(2, 1) * s23 + a(2, 2) * s13 - a(2, 3) * s12) * inv;
    b[1][0] = (-a(1, 0) * q23 + a(1, 2) * q03 - a(1, 3) * q02) * inv;
    b[1][1] = ( a(0, 0) * q23 - a(0, 2) * q03 + a(0, 3) * q02) * inv;
    b[1][2] = (-a(3, 0) * s23 + a(3, 2) * s03 - a(3, 3) * s02) * inv;
    b[1][3] = ( a(2, 0) * s23 - a(2, 2) * s03 + a(2, 3) * s02) * inv;
    b[2][0] = ( a(1, 0) * q13 - a(1, 1) * q03 + a(1, 3) * q01) * inv;
    b[2][1] = (-a(0, 0) * q13 + a(0, 1) * q03 - a(0, 3) * q01) * inv;
    b[2][2] = ( a(3, 0) * s13 - a(3, 1) * s03 + a(3, 3) * s01) * inv;
    b[2][3] = (-a(2, 0) * s13 + a(2, 1) * s03 - a(2, 3) * s01) * inv;
    b[3][0] = (-a(1, 0) * q12 + a(1, 1) * q02 - a(1, 2) * q01) * inv;
    b[3][1] = ( a(0, 0) * q12 - a(0, 1) * q02 + a(0, 2) * q01) * inv;
    b[3][2] = (-a(3, 0) * s12 + a(3, 1) * s02 - a(3, 2) * s01) * inv;
    b[3][3] = ( a(2, 0) * s12 - a(2, 1) * s02 + a(2, 2) * s01) * inv;

    tmat4<T> r;
    for (int c = 0; c < 4; ++c)
        for (int rr = 0; rr < 4; ++rr) r[c][rr] = b[rr][c];
    return r;
}

using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using vec4 = tvec4<float>;
using ivec3 = tvec3<int>;
using dvec3 = tvec3<double>;
using mat3 = tmat3<float>;
using mat3x3 = tmat3<float>;
using mat4 = tmat4<float>;
using mat4x4 = tmat4<float>;
using dmat3 = tmat3<double>;
using dmat3x3 = tmat3<double>;

// Ray/triangle test with the signature the reference's glm fork exposes
// (inMyRoom_vulkan/src/Geometry/Ray.cpp:31): Moller-Trumbore, two-sided,
// reporting whether the hit is on the back face. Only the uncollide-ray
// response uses it; its semantics are not pinned by the reference.
template <class T>
inline bool intersectRayTriangle(const tvec3<T>& orig, const tvec3<T>& dir, const tvec3<T>& v0,
                                 const tvec3<T>& v1, const tvec3<T>& v2, tvec2<T>& bary, T& distance,
                                 bool& backfaces) {
    tvec3<T> e1 = v1 - v0;
    tvec3<T> e2 = v2 - v0;
    tvec3<T> p = cross(dir, e2);
    T det = dot(e1, p);
    backfaces = det < T(0);
    if (std::abs(det) <= std::numeric_limits<T>::epsilon()) return false;
    T inv = T(1) / det;
    tvec3<T> s = orig - v0;
    T u = dot(s, p) * inv;
    if (u < T(0) || u > T(1)) return false;
    tvec3<T> q = cross(s, e1);
    T v = dot(dir, q) * inv;
    if (v < T(0) || u + v > T(1)) return false;
    T t = dot(e2, q) * inv;
    if (t < T(0)) return false;
    bary = tvec2<T>(u, v);
    distance = t;
    return true;
}

}  // namespace glm
