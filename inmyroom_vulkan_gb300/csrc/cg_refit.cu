// Refit of an uploaded tree to deformed vertices: the topology stays, every
// box is fitted again to the points of its subtree with
// OBB::CreateOBBfromPoints (src/Geometry/OBB.cpp:33-89) -- FP64 mean and
// covariance accumulated point by point, the eig3 eigensystem
// (eig3/eig3.cpp:21-265: Householder reduction, implicit-shift QL, ascending
// sort; eigenvectors of the covariance as the box axes), FP64 min/max
// projections padded by 2 FLT_EPSILON, float cast.
//
// A box's points are the corners of its subtree's triangles in the tree's leaf
// (DFS) order, corner 0, 1, 2 of each. The sums run in that order, one lane per
// sum, so every box is the same bits as the host restatement on the same
// order; the min/max projections are order-free and run over all lanes. One
// warp per box; the points pass through shared memory 32 triangles at a time.
#include <cuda_runtime.h>

#include <cfloat>

#include "cg_device.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr unsigned kAll = 0xffffffffu;
constexpr int kRefitWarps = 4;  // warps per block

struct D3 {
    double x, y, z;
};

__device__ __forceinline__ double dotd(D3 a, D3 b) {
    double s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}

__device__ __forceinline__ double hyp(double x, double y) { return sqrt(x * x + y * y); }

// Householder reduction of the symmetric 3x3 in v to tridiagonal form
// (eig3.cpp:21-134): v becomes the accumulated transform, d the diagonal,
// e[1..2] the sub-diagonal.
__device__ void tridiagonalize(double v[3][3], double d[3], double e[3]) {
    for (int c = 0; c < 3; ++c) d[c] = v[2][c];
    for (int i = 2; i >= 1; --i) {
        double scale = 0.0, h = 0.0;
        for (int k = 0; k < i; ++k) scale = scale + fabs(d[k]);
        if (scale == 0.0) {
            e[i] = d[i - 1];
            for (int c = 0; c < i; ++c) {
                d[c] = v[i - 1][c];
                v[i][c] = 0.0;
                v[c][i] = 0.0;
            }
        } else {
            for (int k = 0; k < i; ++k) {
                d[k] = d[k] / scale;
                h = h + d[k] * d[k];
            }
            double f = d[i - 1];
            double g = sqrt(h);
            if (f > 0) g = -g;
            e[i] = scale * g;
            h = h - f * g;
            d[i - 1] = f - g;
            for (int c = 0; c < i; ++c) e[c] = 0.0;
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
            f = 0.0;
            for (int c = 0; c < i; ++c) {
                e[c] = e[c] / h;
                f = f + e[c] * d[c];
            }
            const double hh = f / (h + h);
            for (int c = 0; c < i; ++c) e[c] = e[c] - hh * d[c];
            for (int c = 0; c < i; ++c) {
                f = d[c];
                g = e[c];
                for (int k = c; k <= i - 1; ++k) v[k][c] = v[k][c] - (f * e[k] + g * d[k]);
                d[c] = v[i - 1][c];
                v[i][c] = 0.0;
            }
        }
        d[i] = h;
    }
    for (int i = 0; i < 2; ++i) {
        v[2][i] = v[i][i];
        v[i][i] = 1.0;
        const double h = d[i + 1];
        if (h != 0.0) {
            for (int k = 0; k <= i; ++k) d[k] = v[k][i + 1] / h;
            for (int c = 0; c <= i; ++c) {
                double g = 0.0;
                for (int k = 0; k <= i; ++k) g = g + v[k][i + 1] * v[k][c];
                for (int k = 0; k <= i; ++k) v[k][c] = v[k][c] - g * d[k];
            }
        }
        for (int k = 0; k <= i; ++k) v[k][i + 1] = 0.0;
    }
    for (int c = 0; c < 3; ++c) {
        d[c] = v[2][c];
        v[2][c] = 0.0;
    }
    v[2][2] = 1.0;
    e[0] = 0.0;
}

// Implicit-shift QL on the tridiagonal form, then the ascending sort of the
// eigenvalues with their eigenvector columns (eig3.cpp:138-254). A sweep
// count limit stops what only a non-finite input could run forever.
__device__ void ql_sort(double v[3][3], double d[3], double e[3]) {
    for (int i = 1; i < 3; ++i) e[i - 1] = e[i];
    e[2] = 0.0;
    double f = 0.0, tst1 = 0.0;
    const double eps = 2.220446049250313e-16;  // 2^-52
    for (int l = 0; l < 3; ++l) {
        const double t = fabs(d[l]) + fabs(e[l]);
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
                double g = d[l];
                double p = (d[l + 1] - g) / (2.0 * e[l]);
                double r = hyp(p, 1.0);
                if (p < 0) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                const double dl1 = d[l + 1];
                double h = g - d[l];
                for (int i = l + 2; i < 3; ++i) d[i] = d[i] - h;
                f = f + h;
                p = d[m];
                double c = 1.0, c2 = c, c3 = c;
                const double el1 = e[l + 1];
                double s = 0.0, s2 = 0.0;
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
        e[l] = 0.0;
    }
    for (int i = 0; i < 2; ++i) {
        int k = i;
        double p = d[i];
        for (int j = i + 1; j < 3; ++j)
            if (d[j] < p) {
                k = j;
                p = d[j];
            }
        if (k != i) {
            d[k] = d[i];
            d[i] = p;
            for (int r = 0; r < 3; ++r) {
                const double tmp = v[r][i];
                v[r][i] = v[r][k];
                v[r][k] = tmp;
            }
        }
    }
}

__device__ __forceinline__ float3 corner(const float4* tris, uint32_t tri, int k) {
    const float4 q = tris[3ull * tri + k];
    return make_float3(q.x, q.y, q.z);
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_xor_sync(kAll, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_xor_sync(kAll, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// New corner positions: p_k = positions[vertex index k] for every triangle.
__global__ void refit_tris_kernel(float4* tris, const RefitTree* trees) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3u * T.n_tris) return;
    float4* q = tris + 3ull * T.tri_base + i;
    const float4* positions = T.positions;
    const uint32_t n_positions = T.n_positions;
    const uint32_t vi = __float_as_uint(q->w);
    const float nan = __int_as_float(0x7fc00000);
    const float4 p = vi < n_positions ? positions[vi] : make_float4(nan, nan, nan, 0.f);
    q->x = p.x;
    q->y = p.y;
    q->z = p.z;
}

// One warp per record of the tree; record r covers tree-local triangles
// [range.x, range.x + range.y).
__global__ void __launch_bounds__(32 * kRefitWarps) refit_boxes_kernel(float4* recs, const float4* tris,
                                                                        const RefitTree* trees) {
    __shared__ float stage[kRefitWarps][3][96];
    const RefitTree T = trees[blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const uint32_t r = blockIdx.x * kRefitWarps + uint32_t(w);
    if (r >= T.n_recs) return;  // whole warps
    const uint32_t rec_base = T.rec_base, tri_base = T.tri_base;
    const uint2* ranges = T.ranges;
    const uint2 rg = ranges[r];
    if (rg.y == ~0u) return;  // the unused record of the tree's first pair
    float* sx = stage[w][0];
    float* sy = stage[w][1];
    float* sz = stage[w][2];
    const uint32_t t0 = tri_base + rg.x;
    const uint32_t n_pts = 3u * rg.y;
    float4* out = recs + 4ull * (rec_base + r);

    Box b;
    if (n_pts == 0) {
        b.c = make_float3(0.f, 0.f, 0.f);
        b.u = make_float3(FLT_EPSILON, 0.f, 0.f);
        b.v = make_float3(0.f, FLT_EPSILON, 0.f);
        b.w = make_float3(0.f, 0.f, FLT_EPSILON);
    } else {
        // fewer than two distinct points: the point box (OBB.cpp:36-44)
        const float3 p0 = corner(tris, t0, 0);
        bool differ = false;
        for (uint32_t k = lane; k < n_pts; k += 32) {
            const float3 p = corner(tris, t0 + k / 3u, int(k % 3u));
            differ |= p.x != p0.x || p.y != p0.y || p.z != p0.z;
        }
        if (!__any_sync(kAll, differ)) {
            b.c = p0;
            b.u = make_float3(FLT_EPSILON, 0.f, 0.f);
            b.v = make_float3(0.f, FLT_EPSILON, 0.f);
            b.w = make_float3(0.f, 0.f, FLT_EPSILON);
        } else {
            const double n = double(n_pts);
            // pass 1: sums of x, y, z (lanes 0, 1, 2), point by point
            double acc = 0.0;
            double mx = 0.0, my = 0.0, mz = 0.0;
            for (int pass = 0; pass < 2; ++pass) {
                acc = 0.0;
                for (uint32_t c0 = 0; c0 < rg.y; c0 += 32) {
                    const uint32_t nt = min(32u, rg.y - c0);
                    __syncwarp();
                    if (uint32_t(lane) < nt)
                        for (int k = 0; k < 3; ++k) {
                            const float3 p = corner(tris, t0 + c0 + lane, k);
                            sx[3 * lane + k] = p.x;
                            sy[3 * lane + k] = p.y;
                            sz[3 * lane + k] = p.z;
                        }
                    __syncwarp();
                    const uint32_t np = 3u * nt;
                    if (pass == 0) {
                        if (lane < 3) {
                            const float* s = lane == 0 ? sx : (lane == 1 ? sy : sz);
                            for (uint32_t k = 0; k < np; ++k) acc = acc + double(s[k]);
                        }
                    } else if (lane < 6) {
                        // cxx, cyy, czz, cxy, cxz, cyz
                        const float* s1 = (lane == 0 || lane == 3 || lane == 4) ? sx : (lane == 1 || lane == 5 ? sy : sz);
                        const float* s2 = (lane == 0) ? sx : (lane == 1 || lane == 3) ? sy : sz;
                        const double m1 = (lane == 0 || lane == 3 || lane == 4) ? mx : (lane == 1 || lane == 5 ? my : mz);
                        const double m2 = (lane == 0) ? mx : (lane == 1 || lane == 3) ? my : mz;
                        for (uint32_t k = 0; k < np; ++k) acc = acc + (double(s1[k]) - m1) * (double(s2[k]) - m2);
                    }
                }
                if (pass == 0) {
                    mx = __shfl_sync(kAll, acc, 0) / n;
                    my = __shfl_sync(kAll, acc, 1) / n;
                    mz = __shfl_sync(kAll, acc, 2) / n;
                }
            }
            const double cxx = __shfl_sync(kAll, acc, 0), cyy = __shfl_sync(kAll, acc, 1);
            const double czz = __shfl_sync(kAll, acc, 2), cxy = __shfl_sync(kAll, acc, 3);
            const double cxz = __shfl_sync(kAll, acc, 4), cyz = __shfl_sync(kAll, acc, 5);
            double ax[9];
            if (lane == 0) {
                double v[3][3] = {{cxx / n, cxy / n, cxz / n}, {cxy / n, cyy / n, cyz / n}, {cxz / n, cyz / n, czz / n}};
                double d[3], e[3];
                tridiagonalize(v, d, e);
                ql_sort(v, d, e);
                // the box axes are the rows of the eigenvector matrix
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) ax[3 * i + j] = v[i][j];
            }
#pragma unroll
            for (int i = 0; i < 9; ++i) ax[i] = __shfl_sync(kAll, ax[i], 0);
            // OBB::CreateAABBfromPoints on those axes (OBB.cpp:105-166)
            const double pad = 2.0 * double(FLT_EPSILON);
            double cx = 0.0, cy = 0.0, cz = 0.0;
            float3 half[3];
            for (int a = 0; a < 3; ++a) {
                const D3 axis{ax[3 * a], ax[3 * a + 1], ax[3 * a + 2]};
                double lo = __longlong_as_double(0x7ff0000000000000ll), hi = -lo;
                for (uint32_t k = lane; k < n_pts; k += 32) {
                    const float3 p = corner(tris, t0 + k / 3u, int(k % 3u));
                    const double pr = dotd(axis, D3{double(p.x), double(p.y), double(p.z)});
                    lo = (lo < pr) ? lo : pr;
                    hi = (pr < hi) ? hi : pr;
                }
                lo = warp_min(lo);
                hi = warp_max(hi);
                const double delta = (hi - lo) + pad;
                const double mid = (hi + lo) / 2.0;
                cx = cx + mid * axis.x;
                cy = cy + mid * axis.y;
                cz = cz + mid * axis.z;
                const double h = delta / 2.0;
                half[a] = make_float3(float(h * axis.x), float(h * axis.y), float(h * axis.z));
            }
            b.c = make_float3(float(cx), float(cy), float(cz));
            b.u = half[0];
            b.v = half[1];
            b.w = half[2];
        }
    }
    if (lane == 0) {
        const float4 q3 = out[3];
        out[0] = make_float4(b.c.x, b.c.y, b.c.z, b.u.x);
        out[1] = make_float4(b.u.y, b.u.z, b.v.x, b.v.y);
        out[2] = make_float4(b.v.z, b.w.x, b.w.y, b.w.z);
        out[3] = make_float4(q3.x, q3.y, surface(b), q3.w);
    }
}

}  // namespace

cudaError_t launch_refit(float4* recs, float4* tris, const RefitTree* d_trees, uint32_t n_trees, uint32_t max_tris,
                         uint32_t max_recs, cudaStream_t s) {
    if (n_trees == 0) return cudaSuccess;
    if (max_tris)
        refit_tris_kernel<<<dim3((3u * max_tris + 255u) / 256u, n_trees), 256, 0, s>>>(tris, d_trees);
    refit_boxes_kernel<<<dim3((max_recs + kRefitWarps - 1) / kRefitWarps, n_trees), 32 * kRefitWarps, 0, s>>>(
        recs, tris, d_trees);
    return cudaGetLastError();
}

}  // namespace cg
