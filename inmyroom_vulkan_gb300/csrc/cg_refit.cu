// Refit of an uploaded tree to deformed vertices: the topology stays, every
// box is fitted again to the points of its subtree (the corners of its
// triangles) the way OBB::CreateOBBfromPoints (src/Geometry/OBB.cpp:33-89)
// fits a box: mean and covariance of the points, the eig3 eigensystem of the
// covariance (eig3/eig3.cpp:21-265: Householder reduction, implicit-shift QL,
// ascending sort) with the rows of its eigenvector matrix as the box axes,
// min/max projections on the axes padded by 2 FLT_EPSILON.
//
// The reference builds trees on the CPU and has no refit; this one is shaped
// for a part whose FP64 pipe is narrow (a sequential FP64 fit of a
// 12k-triangle tube's root takes tens of milliseconds here):
//   refit_moments  compensated FP32 sums of the points and of their centred
//                  products: a thread per box of up to kSmallPoints points, a
//                  warp per larger box, a block per box of more than
//                  kBlockPoints (lane sums combined with error-free FP32
//                  sums); the larger boxes come from a per-tree list made at
//                  upload, largest first
//   refit_axes     a thread per box: the eig3 procedure in FP32
//   refit_box      FP32 projections (thread, warp or block per box as above); the box
//                  is padded by 2 FLT_EPSILON plus a bound on the FP32
//                  rounding of the projections, the axes' departure from
//                  orthonormal and the box's assembly, so it contains every
//                  point of its subtree
// The boxes are conservative like the reference's but not its bits; the
// colliding triangle pairs found with them are the same.
#include <cuda_runtime.h>

#include <cfloat>

#include "cg_device.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr unsigned kAll = 0xffffffffu;
constexpr int kRefitWarps = 4;           // warps per block of the warp-per-box kernels

template <typename R>
__device__ __forceinline__ R hyp(R x, R y) {
    return sqrt(x * x + y * y);
}

// Householder reduction of the symmetric 3x3 in v to tridiagonal form
// (eig3.cpp:21-134): v becomes the accumulated transform, d the diagonal,
// e[1..2] the sub-diagonal.
template <typename R>
__device__ void tridiagonalize(R v[3][3], R d[3], R e[3]) {
    for (int c = 0; c < 3; ++c) d[c] = v[2][c];
    for (int i = 2; i >= 1; --i) {
        R scale = R(0), h = R(0);
        for (int k = 0; k < i; ++k) scale = scale + fabs(d[k]);
        if (scale == R(0)) {
            e[i] = d[i - 1];
            for (int c = 0; c < i; ++c) {
                d[c] = v[i - 1][c];
                v[i][c] = R(0);
                v[c][i] = R(0);
            }
        } else {
            for (int k = 0; k < i; ++k) {
                d[k] = d[k] / scale;
                h = h + d[k] * d[k];
            }
            R f = d[i - 1];
            R g = sqrt(h);
            if (f > 0) g = -g;
            e[i] = scale * g;
            h = h - f * g;
            d[i - 1] = f - g;
            for (int c = 0; c < i; ++c) e[c] = R(0);
            for (int c = 0; c < i; ++c) {
                f = d[c];
                v[c][i] = f;
                g = e[c] + v[c][c] * f;
                for (int k = c + 1; k <= i - 1; ++k) {
                    g = g + v[k][c] * d[k];
                    e[k] = e[k] + v[k][c] * f;
                }
                e[c] = g;
            }
            f = R(0);
            for (int c = 0; c < i; ++c) {
                e[c] = e[c] / h;
                f = f + e[c] * d[c];
            }
            const R hh = f / (h + h);
            for (int c = 0; c < i; ++c) e[c] = e[c] - hh * d[c];
            for (int c = 0; c < i; ++c) {
                f = d[c];
                g = e[c];
                for (int k = c; k <= i - 1; ++k) v[k][c] = v[k][c] - (f * e[k] + g * d[k]);
                d[c] = v[i - 1][c];
                v[i][c] = R(0);
            }
        }
        d[i] = h;
    }
    for (int i = 0; i < 2; ++i) {
        v[2][i] = v[i][i];
        v[i][i] = R(1);
        const R h = d[i + 1];
        if (h != R(0)) {
            for (int k = 0; k <= i; ++k) d[k] = v[k][i + 1] / h;
            for (int c = 0; c <= i; ++c) {
                R g = R(0);
                for (int k = 0; k <= i; ++k) g = g + v[k][i + 1] * v[k][c];
                for (int k = 0; k <= i; ++k) v[k][c] = v[k][c] - g * d[k];
            }
        }
        for (int k = 0; k <= i; ++k) v[k][i + 1] = R(0);
    }
    for (int c = 0; c < 3; ++c) {
        d[c] = v[2][c];
        v[2][c] = R(0);
    }
    v[2][2] = R(1);
    e[0] = R(0);
}

// Implicit-shift QL on the tridiagonal form, then the ascending sort of the
// eigenvalues with their eigenvector columns (eig3.cpp:138-254). A sweep
// count limit stops what only a non-finite input could run forever.
template <typename R>
__device__ void ql_sort(R v[3][3], R d[3], R e[3], R eps) {
    for (int i = 1; i < 3; ++i) e[i - 1] = e[i];
    e[2] = R(0);
    R f = 0, tst1 = 0;
    for (int l = 0; l < 3; ++l) {
        const R t = fabs(d[l]) + fabs(e[l]);
        tst1 = (tst1 > t) ? tst1 : t;
        int m = l;
        while (m < 3) {
            if (fabs(e[m]) <= eps * tst1) break;
            ++m;
        }
        if (m > l) {
            int sweeps = 0;
            do {
                ++sweeps;
                R g = d[l];
                R p = (d[l + 1] - g) / (R(2) * e[l]);
                R r = hyp(p, R(1));
                if (p < 0) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                const R dl1 = d[l + 1];
                R h = g - d[l];
                for (int i = l + 2; i < 3; ++i) d[i] = d[i] - h;
                f = f + h;
                p = d[m];
                R c = R(1), c2 = c, c3 = c;
                const R el1 = e[l + 1];
                R s = R(0), s2 = R(0);
                for (int i = m - 1; i >= l; --i) {
                    c3 = c2;
                    c2 = c;
                    s2 = s;
                    g = c * e[i];
                    h = c * p;
                    r = hyp(p, e[i]);
                    e[i + 1] = s * r;
                    s = e[i] / r;
                    c = p / r;
                    p = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                    for (int k = 0; k < 3; ++k) {
                        h = v[k][i + 1];
                        v[k][i + 1] = s * v[k][i] + c * h;
                        v[k][i] = c * v[k][i] - s * h;
                    }
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
            } while (fabs(e[l]) > eps * tst1 && sweeps < 10000);
        }
        d[l] = d[l] + f;
        e[l] = R(0);
    }
    for (int i = 0; i < 2; ++i) {
        int k = i;
        R p = d[i];
        for (int j = i + 1; j < 3; ++j)
            if (d[j] < p) {
                k = j;
                p = d[j];
            }
        if (k != i) {
            d[k] = d[i];
            d[i] = p;
            for (int r = 0; r < 3; ++r) {
                const R tmp = v[r][i];
                v[r][i] = v[r][k];
                v[r][k] = tmp;
            }
        }
    }
}

// Compensated running sum (Kahan): s - c carries the sum of the added values.
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// Error-free sum of two floats (Knuth's two-sum): a + b = hi + lo exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& hi, float& lo) {
    hi = a + b;
    const float bb = hi - a;
    lo = (a - (hi - bb)) + (b - bb);
}

// Sum over the warp of the lanes' (hi, lo) pairs, kept as a float pair.
__device__ __forceinline__ void warp_sum2(float& hi, float& lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(kAll, hi, o), ol = __shfl_xor_sync(kAll, lo, o);
        float h, l;
        two_sum(hi, oh, h, l);
        hi = h;
        lo = (lo + ol) + l;
    }
}

__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kAll, v, o));
    return v;
}
__device__ __forceinline__ float warp_minf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kAll, v, o));
    return v;
}

// New corner positions: p_k = positions[vertex index k] for every triangle.
__global__ void refit_tris_kernel(float4* tris, const RefitTree* trees) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3u * T.n_tris) return;
    float4* q = tris + 3ull * T.tri_base + i;
    const uint32_t vi = __float_as_uint(q->w);
    const float nan = __int_as_float(0x7fc00000);
    const float4 p = vi < T.n_positions ? T.positions[vi] : make_float4(nan, nan, nan, 0.f);
    q->x = p.x;
    q->y = p.y;
    q->z = p.z;
}

// The moments of one box's points, by one lane (lanes = 1) or a whole warp.
struct Moments {
    KSum s[3];    // x, y, z
    KSum c[6];    // xx, yy, zz, xy, xz, yz of the centred points
    float mabs = 0.f;
    bool differ = false;
};

__device__ __forceinline__ void record_out(RefitScratch& out, float4 p0, bool differ, float mabs, const float* cov) {
    if (!differ) {
        out.kind = kRefitPoint;
        out.p0[0] = p0.x;
        out.p0[1] = p0.y;
        out.p0[2] = p0.z;
        return;
    }
    out.kind = kRefitBox;
    out.maxabs = mabs;
    for (int i = 0; i < 6; ++i) out.cov[i] = cov[i];
}

// Thread per small box: the count, whether two points differ, the largest
// |x| + |y| + |z| and the covariance.
__global__ void refit_moments_small_kernel(const float4* tris, const RefitTree* trees, RefitScratch* scratch) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= T.n_recs) return;
    const uint2 rg = T.ranges[r];
    RefitScratch& out = scratch[T.scratch_base + r];
    if (rg.y == ~0u || rg.y == 0u) {
        out.kind = rg.y == ~0u ? kRefitSkip : kRefitEmpty;
        return;
    }
    const uint32_t n_pts = 3u * rg.y;
    if (n_pts > kSmallPoints) return;  // a warp or block kernel's
    const float4* pt = tris + 3ull * (T.tri_base + rg.x);
    const float4 p0 = pt[0];
    KSum sx, sy, sz;
    float mabs = 0.f;
    bool differ = false;
    for (uint32_t k = 0; k < n_pts; ++k) {
        const float4 p = pt[k];
        sx.add(p.x);
        sy.add(p.y);
        sz.add(p.z);
        mabs = fmaxf(mabs, (fabsf(p.x) + fabsf(p.y)) + fabsf(p.z));
        differ |= p.x != p0.x || p.y != p0.y || p.z != p0.z;
    }
    const float fn = float(n_pts);
    const float mx = (sx.s - sx.c) / fn, my = (sy.s - sy.c) / fn, mz = (sz.s - sz.c) / fn;
    KSum c[6];
    for (uint32_t k = 0; k < n_pts && differ; ++k) {
        const float4 p = pt[k];
        const float dx = p.x - mx, dy = p.y - my, dz = p.z - mz;
        c[0].add(dx * dx);
        c[1].add(dy * dy);
        c[2].add(dz * dz);
        c[3].add(dx * dy);
        c[4].add(dx * dz);
        c[5].add(dy * dz);
    }
    float cov[6];
    for (int i = 0; i < 6; ++i) cov[i] = (c[i].s - c[i].c) / fn;
    record_out(out, p0, differ, mabs, cov);
}

// Reductions over the points of one box by a warp (G = 32) or a whole block
// (G = 256, `red` = 18 floats of shared memory); the result is the same on
// every thread of the group.
template <int G>
struct Group;
template <>
struct Group<32> {
    __device__ static void sum2(float& h, float& l, float*) { warp_sum2(h, l); }
    __device__ static float maxf(float v, float*) { return warp_maxf(v); }
    __device__ static float minf(float v, float*) { return warp_minf(v); }
    __device__ static bool any(bool b, float*) { return __any_sync(kAll, b); }
};
template <>
struct Group<256> {
    __device__ static void sum2(float& h, float& l, float* red) {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        warp_sum2(h, l);
        if (lane == 0) red[2 * w] = h, red[2 * w + 1] = l;
        __syncthreads();
        if (w == 0) {
            float hh = lane < 8 ? red[2 * lane] : 0.f, ll = lane < 8 ? red[2 * lane + 1] : 0.f;
            warp_sum2(hh, ll);
            if (lane == 0) red[16] = hh, red[17] = ll;
        }
        __syncthreads();
        h = red[16];
        l = red[17];
        __syncthreads();
    }
    template <bool kMax>
    __device__ static float ext(float v, float* red) {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        v = kMax ? warp_maxf(v) : warp_minf(v);
        if (lane == 0) red[w] = v;
        __syncthreads();
        if (w == 0) {
            float x = lane < 8 ? red[lane] : red[0];
            x = kMax ? warp_maxf(x) : warp_minf(x);
            if (lane == 0) red[16] = x;
        }
        __syncthreads();
        v = red[16];
        __syncthreads();
        return v;
    }
    __device__ static float maxf(float v, float* red) { return ext<true>(v, red); }
    __device__ static float minf(float v, float* red) { return ext<false>(v, red); }
    __device__ static bool any(bool b, float*) { return __syncthreads_or(b) != 0; }
};

// The moments of a large box's points by a group of G threads (thread t),
// lane sums combined with error-free sums.
template <int G>
__device__ __forceinline__ void group_moments(const float4* pt, uint32_t n_pts, uint32_t t, RefitScratch& out,
                                              float* red) {
    const float4 p0 = pt[0];
    KSum sx, sy, sz;
    float mabs = 0.f;
    bool differ = false;
#pragma unroll 4
    for (uint32_t k = t; k < n_pts; k += G) {
        const float4 p = pt[k];
        sx.add(p.x);
        sy.add(p.y);
        sz.add(p.z);
        mabs = fmaxf(mabs, (fabsf(p.x) + fabsf(p.y)) + fabsf(p.z));
        differ |= p.x != p0.x || p.y != p0.y || p.z != p0.z;
    }
    differ = Group<G>::any(differ, red);
    mabs = Group<G>::maxf(mabs, red);
    if (!differ) {
        if (t == 0) record_out(out, p0, false, mabs, nullptr);
        return;
    }
    float hx = sx.s, lx = -sx.c, hy = sy.s, ly = -sy.c, hz = sz.s, lz = -sz.c;
    Group<G>::sum2(hx, lx, red);
    Group<G>::sum2(hy, ly, red);
    Group<G>::sum2(hz, lz, red);
    const float fn = float(n_pts);
    const float mx = (hx + lx) / fn, my = (hy + ly) / fn, mz = (hz + lz) / fn;
    KSum c[6];
#pragma unroll 4
    for (uint32_t k = t; k < n_pts; k += G) {
        const float4 p = pt[k];
        const float dx = p.x - mx, dy = p.y - my, dz = p.z - mz;
        c[0].add(dx * dx);
        c[1].add(dy * dy);
        c[2].add(dz * dz);
        c[3].add(dx * dy);
        c[4].add(dx * dz);
        c[5].add(dy * dz);
    }
    float cov[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        float h = c[i].s, l = -c[i].c;
        Group<G>::sum2(h, l, red);
        cov[i] = (h + l) / fn;
    }
    if (t == 0) record_out(out, p0, true, mabs, cov);
}

// Large boxes come from the tree's list of records with more than
// kSmallPoints points, largest first: the first n_block (more than
// kBlockPoints points) take a block each, the rest a warp each.
__global__ void __launch_bounds__(256) refit_moments_block_kernel(const float4* tris, const RefitTree* trees,
                                                                  RefitScratch* scratch) {
    __shared__ float red[32];
    const RefitTree T = trees[blockIdx.y];
    if (blockIdx.x >= T.n_block) return;
    const uint32_t r = T.big[blockIdx.x];
    const uint2 rg = T.ranges[r];
    group_moments<256>(tris + 3ull * (T.tri_base + rg.x), 3u * rg.y, threadIdx.x, scratch[T.scratch_base + r], red);
}

__global__ void __launch_bounds__(32 * kRefitWarps) refit_moments_kernel(const float4* tris, const RefitTree* trees,
                                                                          RefitScratch* scratch) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t i = T.n_block + blockIdx.x * kRefitWarps + uint32_t(threadIdx.x >> 5);
    if (i >= T.n_big) return;  // whole warps
    const uint32_t r = T.big[i];
    const uint2 rg = T.ranges[r];
    group_moments<32>(tris + 3ull * (T.tri_base + rg.x), 3u * rg.y, threadIdx.x & 31u, scratch[T.scratch_base + r],
                      nullptr);
}

// One thread per record: the eigensystem of the covariance by the eig3
// procedure in FP32 (the covariance carries FP32 accuracy); the box axes are
// the rows of the eigenvector matrix, as the reference takes them.
__global__ void refit_axes_kernel(const RefitTree* trees, RefitScratch* scratch) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= T.n_recs) return;
    RefitScratch& sc = scratch[T.scratch_base + r];
    if (sc.kind != kRefitBox) return;
    const float* c = sc.cov;  // xx, yy, zz, xy, xz, yz
    float v[3][3] = {{c[0], c[3], c[4]}, {c[3], c[1], c[5]}, {c[4], c[5], c[2]}};
    float d[3], e[3];
    tridiagonalize(v, d, e);
    ql_sort(v, d, e, FLT_EPSILON);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) sc.axes[3 * i + j] = v[i][j];
}

// The box from its axes and the projections' min and max per axis. The pad
// adds to the reference's 2 FLT_EPSILON a bound, 2^-20 * (M + extent) with M
// the largest |x| + |y| + |z|, on the FP32 rounding of a projection
// (3 * 2^-24 * M), of the axes' departure from orthonormal and of the box's
// FP32 assembly, so every point stays inside.
__device__ __forceinline__ Box assemble(const float ax[9], const float lo[3], const float hi[3], float maxabs) {
    float cx = 0.f, cy = 0.f, cz = 0.f;
    float3 half[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float ext = hi[a] - lo[a];
        const float pad = 2.f * FLT_EPSILON + 8.f * FLT_EPSILON * (maxabs + ext);
        const float mid = 0.5f * (hi[a] + lo[a]);
        const float h2 = 0.5f * ext + pad;
        cx = cx + mid * ax[3 * a];
        cy = cy + mid * ax[3 * a + 1];
        cz = cz + mid * ax[3 * a + 2];
        half[a] = make_float3(h2 * ax[3 * a], h2 * ax[3 * a + 1], h2 * ax[3 * a + 2]);
    }
    return Box{make_float3(cx, cy, cz), half[0], half[1], half[2]};
}

__device__ __forceinline__ Box special_box(const RefitScratch& sc) {
    Box b;
    b.c = sc.kind == kRefitPoint ? make_float3(sc.p0[0], sc.p0[1], sc.p0[2]) : make_float3(0.f, 0.f, 0.f);
    b.u = make_float3(FLT_EPSILON, 0.f, 0.f);
    b.v = make_float3(0.f, FLT_EPSILON, 0.f);
    b.w = make_float3(0.f, 0.f, FLT_EPSILON);
    return b;
}

__device__ __forceinline__ void write_box(float4* recs, uint32_t rec, const Box& b) {
    float4* out = recs + 4ull * rec;
    const float4 q3 = out[3];
    out[0] = make_float4(b.c.x, b.c.y, b.c.z, b.u.x);
    out[1] = make_float4(b.u.y, b.u.z, b.v.x, b.v.y);
    out[2] = make_float4(b.v.z, b.w.x, b.w.y, b.w.z);
    out[3] = make_float4(q3.x, q3.y, surface(b), q3.w);
}

// Thread per small box (and every empty or point box).
__global__ void refit_box_small_kernel(float4* recs, const float4* tris, const RefitTree* trees,
                                       const RefitScratch* scratch) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= T.n_recs) return;
    const RefitScratch& sc = scratch[T.scratch_base + r];
    if (sc.kind == kRefitSkip) return;
    const uint2 rg = T.ranges[r];
    const uint32_t n_pts = 3u * rg.y;
    if (sc.kind != kRefitBox) {
        write_box(recs, T.rec_base + r, special_box(sc));
        return;
    }
    if (n_pts > kSmallPoints) return;  // a warp or block kernel's
    const float4* pt = tris + 3ull * (T.tri_base + rg.x);
    float ax[9];
    for (int i = 0; i < 9; ++i) ax[i] = sc.axes[i];
    const float inf = __int_as_float(0x7f800000);
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    for (uint32_t k = 0; k < n_pts; ++k) {
        const float4 p = pt[k];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float pr = (ax[3 * a] * p.x + ax[3 * a + 1] * p.y) + ax[3 * a + 2] * p.z;
            lo[a] = fminf(lo[a], pr);
            hi[a] = fmaxf(hi[a], pr);
        }
    }
    write_box(recs, T.rec_base + r, assemble(ax, lo, hi, sc.maxabs));
}

// Extent of a large box's points on its axes by a group of G threads.
template <int G>
__device__ __forceinline__ void group_box(float4* recs, uint32_t rec, const float4* pt, uint32_t n_pts, uint32_t t,
                                          const RefitScratch& sc, float* red) {
    float ax[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) ax[i] = sc.axes[i];
    const float inf = __int_as_float(0x7f800000);
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
#pragma unroll 4
    for (uint32_t k = t; k < n_pts; k += G) {
        const float4 p = pt[k];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float pr = (ax[3 * a] * p.x + ax[3 * a + 1] * p.y) + ax[3 * a + 2] * p.z;
            lo[a] = fminf(lo[a], pr);
            hi[a] = fmaxf(hi[a], pr);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = Group<G>::minf(lo[a], red);
        hi[a] = Group<G>::maxf(hi[a], red);
    }
    if (t == 0) write_box(recs, rec, assemble(ax, lo, hi, sc.maxabs));
}

__global__ void __launch_bounds__(256) refit_box_block_kernel(float4* recs, const float4* tris, const RefitTree* trees,
                                                              const RefitScratch* scratch) {
    __shared__ float red[32];
    const RefitTree T = trees[blockIdx.y];
    if (blockIdx.x >= T.n_block) return;
    const uint32_t r = T.big[blockIdx.x];
    const RefitScratch& sc = scratch[T.scratch_base + r];
    if (sc.kind != kRefitBox) return;  // written by the small kernel (whole block)
    const uint2 rg = T.ranges[r];
    group_box<256>(recs, T.rec_base + r, tris + 3ull * (T.tri_base + rg.x), 3u * rg.y, threadIdx.x, sc, red);
}

__global__ void __launch_bounds__(32 * kRefitWarps) refit_box_kernel(float4* recs, const float4* tris,
                                                                      const RefitTree* trees,
                                                                      const RefitScratch* scratch) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t i = T.n_block + blockIdx.x * kRefitWarps + uint32_t(threadIdx.x >> 5);
    if (i >= T.n_big) return;  // whole warps
    const uint32_t r = T.big[i];
    const RefitScratch& sc = scratch[T.scratch_base + r];
    if (sc.kind != kRefitBox) return;  // written by the small kernel
    const uint2 rg = T.ranges[r];
    group_box<32>(recs, T.rec_base + r, tris + 3ull * (T.tri_base + rg.x), 3u * rg.y, threadIdx.x & 31u, sc,
                  nullptr);
}

}  // namespace

cudaError_t launch_refit(float4* recs, float4* tris, const RefitTree* d_trees, uint32_t n_trees, uint32_t max_tris,
                         uint32_t max_recs, uint32_t max_block, uint32_t max_warp, RefitScratch* scratch,
                         cudaStream_t s) {
    if (n_trees == 0) return cudaSuccess;
    if (max_tris) refit_tris_kernel<<<dim3((3u * max_tris + 255u) / 256u, n_trees), 256, 0, s>>>(tris, d_trees);
    const dim3 threads((max_recs + 127u) / 128u, n_trees);
    const dim3 blocks(max_block, n_trees);
    const dim3 warps((max_warp + kRefitWarps - 1) / kRefitWarps, n_trees);
    refit_moments_small_kernel<<<threads, 128, 0, s>>>(tris, d_trees, scratch);
    if (max_block) refit_moments_block_kernel<<<blocks, 256, 0, s>>>(tris, d_trees, scratch);
    if (max_warp) refit_moments_kernel<<<warps, 32 * kRefitWarps, 0, s>>>(tris, d_trees, scratch);
    refit_axes_kernel<<<threads, 128, 0, s>>>(d_trees, scratch);
    refit_box_small_kernel<<<threads, 128, 0, s>>>(recs, tris, d_trees, scratch);
    if (max_block) refit_box_block_kernel<<<blocks, 256, 0, s>>>(recs, tris, d_trees, scratch);
    if (max_warp) refit_box_kernel<<<warps, 32 * kRefitWarps, 0, s>>>(recs, tris, d_trees, scratch);
    return cudaGetLastError();
}

}  // namespace cg
