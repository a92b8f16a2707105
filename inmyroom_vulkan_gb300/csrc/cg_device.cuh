// Device geometry for the collision kernels: box transform, 15-axis SAT,
// surface, triangle transform and the Moller triangle-triangle test with
// intersection segment.
//
// Every routine rounds exactly where the reference's CPU code rounds (the
// reference is compiled with IEEE semantics against glm-convention math:
// dot = (x*x' + y*y') + z*z', mat4*vec4 = (c0*x + c1*y) + (c2*z + c3*w),
// normalize = v * (1/sqrt(dot))). The translation units that include this file
// are built with -fmad=false (no FMA contraction), IEEE division and square
// root, and no flush-to-zero, so that colliding sets and segments are
// bit-identical to the reference CPU path.
#pragma once

#include <cstdint>

namespace cg {

struct Box {
    float3 c, u, v, w;
};

__device__ __forceinline__ float dot3(float3 a, float3 b) {
    float s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float length3(float3 v) { return sqrtf(dot3(v, v)); }
__device__ __forceinline__ float3 normalize3(float3 v) {
    const float inv = 1.0f / sqrtf(dot3(v, v));
    return make_float3(v.x * inv, v.y * inv, v.z * inv);
}

// Column-major 4x4 held as four columns.
struct Mat4 {
    float4 c0, c1, c2, c3;
};

// glm::vec3(M * glm::vec4(p, w)) with the pairwise column sum. The w terms
// are multiplied even when w is 0 or 1 so that signed zeros and infinities
// round exactly as on the CPU.
__device__ __forceinline__ float3 xform(const Mat4& M, float3 p, float w) {
    float3 r;
    r.x = (M.c0.x * p.x + M.c1.x * p.y) + (M.c2.x * p.z + M.c3.x * w);
    r.y = (M.c0.y * p.x + M.c1.y * p.y) + (M.c2.y * p.z + M.c3.y * w);
    r.z = (M.c0.z * p.x + M.c1.z * p.y) + (M.c2.z * p.z + M.c3.z * w);
    return r;
}

// glm-convention inverse (Laplace expansion over 2x2 minors), the expression
// tree of the host's cg_relative_matrix.
__device__ inline Mat4 inverse4(const Mat4& M) {
    const float4 col[4] = {M.c0, M.c1, M.c2, M.c3};
    auto a = [&](int r, int c) { return r == 0 ? col[c].x : (r == 1 ? col[c].y : (r == 2 ? col[c].z : col[c].w)); };
    const float s01 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1);
    const float s02 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2);
    const float s03 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3);
    const float s12 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2);
    const float s13 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3);
    const float s23 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
    const float q01 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
    const float q02 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2);
    const float q03 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3);
    const float q12 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2);
    const float q13 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3);
    const float q23 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3);
    const float det = s01 * q23 - s02 * q13 + s03 * q12 + s12 * q03 - s13 * q02 + s23 * q01;
    const float inv = 1.0f / det;
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
    return Mat4{make_float4(b[0][0], b[1][0], b[2][0], b[3][0]), make_float4(b[0][1], b[1][1], b[2][1], b[3][1]),
                make_float4(b[0][2], b[1][2], b[2][2], b[3][2]), make_float4(b[0][3], b[1][3], b[2][3], b[3][3])};
}

// glm-convention product A * B of column-major 4x4s (a left-to-right sum over
// k), the host's mat_mul.
__device__ inline Mat4 mul4(const Mat4& A, const Mat4& B) {
    const float4 a[4] = {A.c0, A.c1, A.c2, A.c3}, b[4] = {B.c0, B.c1, B.c2, B.c3};
    auto e = [](const float4& v, int r) { return r == 0 ? v.x : (r == 1 ? v.y : (r == 2 ? v.z : v.w)); };
    float4 out[4];
    for (int j = 0; j < 4; ++j) {
        float r[4];
        for (int k = 0; k < 4; ++k) {
            float acc = e(a[0], k) * e(b[j], 0);
            acc = acc + e(a[1], k) * e(b[j], 1);
            acc = acc + e(a[2], k) * e(b[j], 2);
            acc = acc + e(a[3], k) * e(b[j], 3);
            r[k] = acc;
        }
        out[j] = make_float4(r[0], r[1], r[2], r[3]);
    }
    return Mat4{out[0], out[1], out[2], out[3]};
}

// Paralgram::MultiplyBy4x4Matrix (src/Geometry/Paralgram.cpp:4-15).
__device__ __forceinline__ Box xform_box(const Mat4& M, const Box& b) {
    return Box{xform(M, b.c, 1.0f), xform(M, b.u, 0.0f), xform(M, b.v, 0.0f), xform(M, b.w, 0.0f)};
}

// Paralgram::GetMinMaxProjectionToAxis + DoMinMaxProjectionsToAxisIntersept
// (Paralgram.cpp:175-201).
__device__ __forceinline__ void project(const Box& b, float3 axis, float& lo, float& hi) {
    const float cp = dot3(b.c, axis);
    const float e = (fabsf(dot3(axis, b.u)) + fabsf(dot3(axis, b.v))) + fabsf(dot3(axis, b.w));
    lo = cp - e;
    hi = cp + e;
}
__device__ __forceinline__ bool overlap_on(const Box& a, const Box& b, float3 axis) {
    float alo, ahi, blo, bhi;
    project(a, axis, alo, ahi);
    project(b, axis, blo, bhi);
    return (ahi >= blo) && (bhi >= alo);
}

// Paralgram::IntersectParalgramsBoolean (Paralgram.cpp:17-173): a's face
// normals, b's face normals, then a_i x b_j, in the reference's order.
__device__ __forceinline__ bool sat(const Box& a, const Box& b) {
    if (!overlap_on(a, b, cross3(a.v, a.w))) return false;
    if (!overlap_on(a, b, cross3(a.u, a.w))) return false;
    if (!overlap_on(a, b, cross3(a.u, a.v))) return false;
    if (!overlap_on(a, b, cross3(b.v, b.w))) return false;
    if (!overlap_on(a, b, cross3(b.u, b.w))) return false;
    if (!overlap_on(a, b, cross3(b.u, b.v))) return false;
    if (!overlap_on(a, b, cross3(a.u, b.u))) return false;
    if (!overlap_on(a, b, cross3(a.u, b.v))) return false;
    if (!overlap_on(a, b, cross3(a.u, b.w))) return false;
    if (!overlap_on(a, b, cross3(a.v, b.u))) return false;
    if (!overlap_on(a, b, cross3(a.v, b.v))) return false;
    if (!overlap_on(a, b, cross3(a.v, b.w))) return false;
    if (!overlap_on(a, b, cross3(a.w, b.u))) return false;
    if (!overlap_on(a, b, cross3(a.w, b.v))) return false;
    if (!overlap_on(a, b, cross3(a.w, b.w))) return false;
    return true;
}

// Paralgram::GetSurface (Paralgram.cpp:203-210).
__device__ __forceinline__ float surface(const Box& b) {
    const float uv = length3(cross3(b.u, b.v));
    const float uw = length3(cross3(b.u, b.w));
    const float vw = length3(cross3(b.v, b.w));
    return 2.0f * ((uv + uw) + vw);
}

__device__ __forceinline__ float comp(float3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// ------------------------------------------------------------- Moller ----
// Triangle/triangle test with intersection line after T. Moller, "A Fast
// Triangle-Triangle Intersection Test", JGT 2(2), 1997 (2001 revision), in the
// form the reference uses (src/Geometry/Triangle.cpp:325-1003).

// |x| < 1e-6 with x promoted to double (Triangle.cpp:332, 898-902) equals
// |x| < 0x1.0c6f7cp-20f (1.0000001e-6f, the smallest float above 1e-6): 1e-6
// is not a float, so no float lies in [1e-6, 0x1.0c6f7cp-20f).
__device__ __forceinline__ bool tiny(float x) { return fabsf(x) < 0x1.0c6f7cp-20f; }

// isect2 (Triangle.cpp:764-778).
__device__ __forceinline__ void edge_points(float3 x0, float3 x1, float3 x2, float p0, float p1, float p2, float d0,
                                            float d1, float d2, float& t0, float& t1, float3& q0, float3& q1) {
    float s = d0 / (d0 - d1);
    t0 = p0 + (p1 - p0) * s;
    q0 = make_float3(s * (x1.x - x0.x) + x0.x, s * (x1.y - x0.y) + x0.y, s * (x1.z - x0.z) + x0.z);
    s = d0 / (d0 - d2);
    t1 = p0 + (p2 - p0) * s;
    q1 = make_float3(x0.x + s * (x2.x - x0.x), x0.y + s * (x2.y - x0.y), x0.z + s * (x2.z - x0.z));
}

// compute_intervals_isectline (Triangle.cpp:795-830); returns true for
// "all distances zero".
__device__ __forceinline__ bool interval(float3 x0, float3 x1, float3 x2, float p0, float p1, float p2, float d0,
                                         float d1, float d2, float d0d1, float d0d2, float& t0, float& t1, float3& q0,
                                         float3& q1) {
    if (d0d1 > 0.0f)
        edge_points(x2, x0, x1, p2, p0, p1, d2, d0, d1, t0, t1, q0, q1);
    else if (d0d2 > 0.0f)
        edge_points(x1, x0, x2, p1, p0, p2, d1, d0, d2, t0, t1, q0, q1);
    else if (d1 * d2 > 0.0f || d0 != 0.0f)
        edge_points(x0, x1, x2, p0, p1, p2, d0, d1, d2, t0, t1, q0, q1);
    else if (d1 != 0.0f)
        edge_points(x1, x0, x2, p1, p0, p2, d1, d0, d2, t0, t1, q0, q1);
    else if (d2 != 0.0f)
        edge_points(x2, x0, x1, p2, p0, p1, d2, d0, d1, t0, t1, q0, q1);
    else
        return true;
    return false;
}

// Outcome of one triangle-pair test.
enum : int { TT_MISS = 0, TT_HIT = 1, TT_COPLANAR = 2, TT_FRAGILE = 3 };

// ---- FP64 recheck of the orientation determinants ----
//
// The six plane distances of the test (du_k of the second triangle's corners
// to the first's plane, dv_k the other way) are the orientation determinants
// det[a1 - a0, a2 - a0, p - a0] as the reference computes them in FP32:
// d = (n . p) + (-(n . a0)) with n = (a1 - a0) x (a2 - a0). The test only
// looks at each one's class: zero when |d| < 1e-6 (Triangle.cpp:898-915),
// else its sign. The FP32 value's error against the exact determinant is at
// most 16 u C |a1 - a0|_1 |a2 - a0|_1 (u = 2^-24, C the largest coordinate
// magnitude of a0 and the three tested corners: the edges and the cross
// product round at 4u relative, the two dot products at 3u, the last sum at
// u). The filter bound is twice that,
//   B = 32 u C |a1 - a0|_1 |a2 - a0|_1,
// and a distance whose FP32 magnitude lies within B of 0 or of 1e-6 is
// uncertain: it is recomputed in FP64 from the same corners (det form, with
// differences of floats, exact in FP64 for the meshes' coordinate ranges)
// and classified again. Outside the band the FP32 class is the exact one.
constexpr float kRecheckU32 = 32.0f * 0x1p-24f;

__device__ __forceinline__ float amax3(float3 p) { return fmaxf(fmaxf(fabsf(p.x), fabsf(p.y)), fabsf(p.z)); }
__device__ __forceinline__ float norm1(float3 p) { return (fabsf(p.x) + fabsf(p.y)) + fabsf(p.z); }

__device__ __forceinline__ float filter_bound(float3 a0, float3 e1, float3 e2, float3 p0, float3 p1, float3 p2) {
    const float C = fmaxf(fmaxf(amax3(a0), amax3(p0)), fmaxf(amax3(p1), amax3(p2)));
    return kRecheckU32 * C * norm1(e1) * norm1(e2);
}
__device__ __forceinline__ bool uncertain(float d, float bound) {
    const float a = fabsf(d);
    return a < bound || fabsf(a - 1e-6f) < bound;
}
__device__ __forceinline__ int class32(float d) { return tiny(d) ? 0 : (d > 0.0f ? 1 : -1); }
__device__ __forceinline__ int class64(double d) { return fabs(d) < 1e-6 ? 0 : (d > 0.0 ? 1 : -1); }
static __device__ __noinline__ double orient64(float3 a0, float3 a1, float3 a2, float3 p) {
    const double e1x = double(a1.x) - double(a0.x), e1y = double(a1.y) - double(a0.y), e1z = double(a1.z) - double(a0.z);
    const double e2x = double(a2.x) - double(a0.x), e2y = double(a2.y) - double(a0.y), e2z = double(a2.z) - double(a0.z);
    const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    return (nx * (double(p.x) - double(a0.x)) + ny * (double(p.y) - double(a0.y))) + nz * (double(p.z) - double(a0.z));
}

// Recheck state of one test: distances recomputed in FP64, and whether any
// of them changed class.
struct Recheck {
    uint32_t checked = 0;
    bool disagree = false;
};

// The zero snap of three distances of one plane (a0, a1, a2 the plane's
// triangle, p the other's corners, d their FP32 distances). kMode 0: the
// reference's snap; 1: the same values, uncertain ones rechecked and counted;
// 2: uncertain ones replaced by the FP64 class (0, or the FP64 value in FP32).
template <int kMode>
__device__ __forceinline__ void snap3(float3 a0, float3 a1, float3 a2, float3 e1, float3 e2, const float3 p[3],
                                      float d[3], Recheck& rc) {
    bool unc[3] = {false, false, false};
    if (kMode != 0) {
        const float B = filter_bound(a0, e1, e2, p[0], p[1], p[2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) unc[k] = uncertain(d[k], B);
        if (unc[0] | unc[1] | unc[2]) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (!unc[k]) continue;
                const double x = orient64(a0, a1, a2, p[k]);
                const int c = class64(x);
                ++rc.checked;
                if (c != class32(d[k])) rc.disagree = true;
                if (kMode == 2) d[k] = c == 0 ? 0.0f : float(x);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (!(kMode == 2 && unc[k]) && tiny(d[k])) d[k] = 0.0f;
}

// tri_tri_intersect_with_isectline (Triangle.cpp:866-1003). TT_HIT means
// doIntersept && !areCoplanar (the pairs CreateUncollideRays.cpp:88 keeps);
// TT_COPLANAR covers every coplanar outcome (never kept); TT_FRAGILE is the
// case where the second interval degenerates (U's distances all zero while V's
// are not), in which the reference reads uninitialised values: it is defined
// here, as in the oracle, as "not colliding" and counted. kMode: the FP64
// recheck of the plane distances (snap3: 0 off, 1 counted, 2 FP64 verdict).
template <int kMode>
__device__ __forceinline__ int tri_tri_mode(float3 V0, float3 V1, float3 V2, float3 U0, float3 U1, float3 U2,
                                            float3& src, float3& tgt, Recheck& rc) {
    float3 e1 = sub3(V1, V0), e2 = sub3(V2, V0);
    const float3 n1 = make_float3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
    const float d1 = -((n1.x * V0.x + n1.y * V0.y) + n1.z * V0.z);
    float du[3];
    du[0] = ((n1.x * U0.x + n1.y * U0.y) + n1.z * U0.z) + d1;
    du[1] = ((n1.x * U1.x + n1.y * U1.y) + n1.z * U1.z) + d1;
    du[2] = ((n1.x * U2.x + n1.y * U2.y) + n1.z * U2.z) + d1;
    {
        const float3 U[3] = {U0, U1, U2};
        snap3<kMode>(V0, V1, V2, e1, e2, U, du, rc);
    }
    const float du0 = du[0], du1 = du[1], du2 = du[2];
    const float du0du1 = du0 * du1;
    const float du0du2 = du0 * du2;
    if (du0du1 > 0.0f && du0du2 > 0.0f) return TT_MISS;

    e1 = sub3(U1, U0);
    e2 = sub3(U2, U0);
    const float3 n2 = make_float3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
    const float d2 = -((n2.x * U0.x + n2.y * U0.y) + n2.z * U0.z);
    float dv[3];
    dv[0] = ((n2.x * V0.x + n2.y * V0.y) + n2.z * V0.z) + d2;
    dv[1] = ((n2.x * V1.x + n2.y * V1.y) + n2.z * V1.z) + d2;
    dv[2] = ((n2.x * V2.x + n2.y * V2.y) + n2.z * V2.z) + d2;
    {
        const float3 V[3] = {V0, V1, V2};
        snap3<kMode>(U0, U1, U2, e1, e2, V, dv, rc);
    }
    const float dv0 = dv[0], dv1 = dv[1], dv2 = dv[2];
    const float dv0dv1 = dv0 * dv1;
    const float dv0dv2 = dv0 * dv2;
    if (dv0dv1 > 0.0f && dv0dv2 > 0.0f) return TT_MISS;

    const float3 D = make_float3(n1.y * n2.z - n1.z * n2.y, n1.z * n2.x - n1.x * n2.z, n1.x * n2.y - n1.y * n2.x);
    float mx = fabsf(D.x);
    int index = 0;
    const float b = fabsf(D.y);
    const float c = fabsf(D.z);
    if (b > mx) mx = b, index = 1;
    if (c > mx) mx = c, index = 2;

    const float vp0 = comp(V0, index), vp1 = comp(V1, index), vp2 = comp(V2, index);
    const float up0 = comp(U0, index), up1 = comp(U1, index), up2 = comp(U2, index);

    float i10, i11, i20, i21;
    float3 pa1, pa2, pb1, pb2;
    // Coplanar pairs go to coplanar_tri_tri in the reference, whose verdict
    // never counts as colliding (areCoplanar is set), so it is not evaluated.
    if (interval(V0, V1, V2, vp0, vp1, vp2, dv0, dv1, dv2, dv0dv1, dv0dv2, i10, i11, pa1, pa2)) return TT_COPLANAR;
    if (interval(U0, U1, U2, up0, up1, up2, du0, du1, du2, du0du1, du0du2, i20, i21, pb1, pb2)) return TT_FRAGILE;

    int smallest1, smallest2;
    if (i10 > i11) {
        const float t = i10;
        i10 = i11;
        i11 = t;
        smallest1 = 1;
    } else {
        smallest1 = 0;
    }
    if (i20 > i21) {
        const float t = i20;
        i20 = i21;
        i21 = t;
        smallest2 = 1;
    } else {
        smallest2 = 0;
    }
    if (i11 < i20 || i21 < i10) return TT_MISS;

    if (i20 < i10) {
        src = smallest1 == 0 ? pa1 : pa2;
        if (i21 < i11)
            tgt = smallest2 == 0 ? pb2 : pb1;
        else
            tgt = smallest1 == 0 ? pa2 : pa1;
    } else {
        src = smallest2 == 0 ? pb1 : pb2;
        if (i21 > i11)
            tgt = smallest1 == 0 ? pa2 : pa1;
        else
            tgt = smallest2 == 0 ? pb2 : pb1;
    }
    return TT_HIT;
}

__device__ __forceinline__ int tri_tri(float3 V0, float3 V1, float3 V2, float3 U0, float3 U1, float3 U2, float3& src,
                                       float3& tgt) {
    Recheck rc;
    return tri_tri_mode<0>(V0, V1, V2, U0, U1, U2, src, tgt, rc);
}

}  // namespace cg
