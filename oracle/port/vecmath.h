// Oracle test infrastructure (C++ restatement of the reference's collision path).
//
// Vector arithmetic with the operation order of the glm shim the reference is
// compiled against (oracle/shim/glm/glm_shim.hpp): every function here rounds
// exactly where that shim rounds, so that results are bit-identical to the
// reference build with -ffp-contract=off.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>

namespace port {

struct V3 {
    float x, y, z;
};
struct D3 {
    double x, y, z;
};

// Column-major 4x4, m[4*c + r].
struct M4 {
    float m[16];
};

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scale(float s, V3 v) { return V3{s * v.x, s * v.y, s * v.z}; }
inline V3 divs(V3 v, float s) { return V3{v.x / s, v.y / s, v.z / s}; }
inline V3 neg(V3 v) { return V3{-v.x, -v.y, -v.z}; }
inline bool eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// ((a.x*b.x + a.y*b.y) + a.z*b.z)
inline float dot(V3 a, V3 b) {
    float s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}
inline double dotd(D3 a, D3 b) {
    double s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}
inline V3 cross(V3 a, V3 b) { return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
inline float length(V3 v) { return std::sqrt(dot(v, v)); }
inline V3 normalize(V3 v) {
    float inv = 1.0f / std::sqrt(dot(v, v));
    return V3{v.x * inv, v.y * inv, v.z * inv};
}

// M * (p, w) with the pairwise column sum (c0*x + c1*y) + (c2*z + c3*w), xyz kept.
inline V3 xform(const M4& M, V3 p, float w) {
    const float* m = M.m;
    float r[3];
    for (int k = 0; k < 3; ++k) {
        float a = m[0 + k] * p.x;
        float b = m[4 + k] * p.y;
        float c = m[8 + k] * p.z;
        float d = m[12 + k] * w;
        r[k] = (a + b) + (c + d);
    }
    return V3{r[0], r[1], r[2]};
}

// (A * B): column j = ((a0*b.x + a1*b.y) + a2*b.z) + a3*b.w
inline M4 mul(const M4& A, const M4& B) {
    M4 R;
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k) {
            float acc = A.m[0 + k] * B.m[4 * j + 0];
            acc = acc + A.m[4 + k] * B.m[4 * j + 1];
            acc = acc + A.m[8 + k] * B.m[4 * j + 2];
            acc = acc + A.m[12 + k] * B.m[4 * j + 3];
            R.m[4 * j + k] = acc;
        }
    return R;
}

// Inverse by the Laplace expansion over 2x2 minors of rows {0,1} and {2,3},
// the same expression tree as the shim.
inline M4 inverse(const M4& M) {
    auto a = [&](int r, int c) { return M.m[4 * c + r]; };
    float s01 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1);
    float s02 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2);
    float s03 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3);
    float s12 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2);
    float s13 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3);
    float s23 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
    float q01 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
    float q02 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2);
    float q03 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3);
    float q12 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2);
    float q13 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3);
    float q23 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3);
    float det = s01 * q23 - s02 * q13 + s03 * q12 + s12 * q03 - s13 * q02 + s23 * q01;
    float inv = 1.0f / det;
    float b[4][4];
    b[0][0] = (a(1, 1) * q23 - a(1, 2) * q13 + a(1, 3) * q12) * inv;
    b[0][1] = (-a(0, 1) * q23 + a(0, 2) * q13 - a(0, 3) * q12) * inv;
    b[0][2] = (a(3, 1) * s23 - a(3, 2) * s13 + a(3, 3) * s12) * inv;
    b[0][3] = (-a(2, 1) * s23 + a(2, 2) * s13 - a(2, 3) * s12) * inv;
    b[1][0] = (-a(1, 0) * q23 + a(1, 2) * q03 - a(1, 3) * q02) * inv;
    b[1][1] = (a(0, 0) * q23 - a(0, 2) * q03 + a(0, 3) * q02) * inv;
    b[1][2] = (-a(3, 0) * s23 + a(3, 2) * s03 - a(3, 3) * s02) * inv;
    b[1][3] = (a(2, 0) * s23 - a(2, 2) * s03 + a(2, 3) * s02) * inv;
    b[2][0] = (a(1, 0) * q13 - a(1, 1) * q03 + a(1, 3) * q01) * inv;
    b[2][1] = (-a(0, 0) * q13 + a(0, 1) * q03 - a(0, 3) * q01) * inv;
    b[2][2] = (a(3, 0) * s13 - a(3, 1) * s03 + a(3, 3) * s01) * inv;
    b[2][3] = (-a(2, 0) * s13 + a(2, 1) * s03 - a(2, 3) * s01) * inv;
    b[3][0] = (-a(1, 0) * q12 + a(1, 1) * q02 - a(1, 2) * q01) * inv;
    b[3][1] = (a(0, 0) * q12 - a(0, 1) * q02 + a(0, 2) * q01) * inv;
    b[3][2] = (-a(3, 0) * s12 + a(3, 1) * s02 - a(3, 2) * s01) * inv;
    b[3][3] = (a(2, 0) * s12 - a(2, 1) * s02 + a(2, 2) * s01) * inv;
    M4 R;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) R.m[4 * c + r] = b[r][c];
    return R;
}

// Cofactor matrix of the upper-left 3x3 (normal transform up to det), as
// column-major 3x3 n[3*c + r].
struct M3 {
    float m[9];
};
inline M3 cofactor3(const M4& M) {
    auto g = [&](int c, int r) { return M.m[4 * c + r]; };
    M3 R;
    auto s = [&](int c, int r, float v) { R.m[3 * c + r] = v; };
    s(0, 0, g(1, 1) * g(2, 2) - g(2, 1) * g(1, 2));
    s(0, 1, g(2, 0) * g(1, 2) - g(1, 0) * g(2, 2));
    s(0, 2, g(1, 0) * g(2, 1) - g(2, 0) * g(1, 1));
    s(1, 0, g(2, 1) * g(0, 2) - g(0, 1) * g(2, 2));
    s(1, 1, g(0, 0) * g(2, 2) - g(2, 0) * g(0, 2));
    s(1, 2, g(2, 0) * g(0, 1) - g(0, 0) * g(2, 1));
    s(2, 0, g(0, 1) * g(1, 2) - g(1, 1) * g(0, 2));
    s(2, 1, g(1, 0) * g(0, 2) - g(0, 0) * g(1, 2));
    s(2, 2, g(0, 0) * g(1, 1) - g(1, 0) * g(0, 1));
    return R;
}
// (c0*x + c1*y) + c2*z
inline V3 mul3(const M3& N, V3 v) {
    float r[3];
    for (int k = 0; k < 3; ++k) {
        float a = N.m[0 + k] * v.x;
        float b = N.m[3 + k] * v.y;
        float c = N.m[6 + k] * v.z;
        r[k] = (a + b) + c;
    }
    return V3{r[0], r[1], r[2]};
}

}  // namespace port
