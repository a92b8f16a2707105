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
// 12k-triangle tube's root takes tens of milliseconds here) and so that no
// box reads its subtree's points itself (a root box would read them all):
//   refit_tris     the triangles' corners from the new vertex positions
//   refit_climb    a thread per leaf box: count, mean and centred second
//                  moments of its points in FP32; then up the tree, the
//                  second child to arrive at a parent (an arrival counter per
//                  record, no waiting) merges the two children's moments
//                  (Chan, Golub and LeVeque's pairwise update: mean += d nb/n,
//                  M2 = M2a + M2b + d d^T na nb / n)
//   refit_axes     a thread per box: the eig3 procedure in FP32 on M2 / n
//   refit_extent   a thread per leaf box: up its chain of boxes, the extent
//                  of the leaf's points on each box's axes as the floats'
//                  order-preserving integer keys; lanes of a warp at the same
//                  box reduce their keys with one warp min/max each, and one
//                  lane per box and warp adds the result with an integer
//                  atomic min/max where it moves the box's current extent
//   refit_assemble a thread per box: the box from its axes and extents (and
//                  resets the extents for the next refit). The box is padded
//                  by 2 FLT_EPSILON plus a bound on the FP32 rounding of the
//                  projections, the axes' departure from orthonormal and the
//                  box's assembly, so it contains every point of its subtree
// The boxes are conservative like the reference's but not its bits; the
// colliding triangle pairs found with them are the same.
#include <cuda_runtime.h>

#include <cfloat>

#include "cg_device.cuh"
#include "cg_eig.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr unsigned kAll = 0xffffffffu;
constexpr uint32_t kNoRec = 0xffffffffu;

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

using Mom = RefitMom;

// Read through L2: another SM wrote it in this launch.
__device__ __forceinline__ Mom load_mom(const Mom* s) {
    Mom m;
    const uint4* q = reinterpret_cast<const uint4*>(s);
    uint4 w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = __ldcg(q + i);
    memcpy(&m, w, sizeof(Mom));
    return m;
}

// The moments of a leaf's points, two passes over them (held in registers
// for the usual leaf of up to 4 triangles).
constexpr uint32_t kLeafRegPoints = 12;

__device__ Mom leaf_mom(const float4* pt, uint32_t n_pts) {
    if (n_pts > 0 && n_pts <= kLeafRegPoints) {
        float4 q[kLeafRegPoints];
        q[0] = pt[0];
#pragma unroll
        for (uint32_t k = 1; k < kLeafRegPoints; ++k) {
            q[k] = q[0];
            if (k < n_pts) q[k] = pt[k];
        }
        Mom m{};
        m.n = n_pts;
        m.p0[0] = q[0].x, m.p0[1] = q[0].y, m.p0[2] = q[0].z;
        float sx = 0.f, sy = 0.f, sz = 0.f;
        bool differ = false;
#pragma unroll
        for (uint32_t k = 0; k < kLeafRegPoints; ++k)
            if (k < n_pts) {
                sx = sx + q[k].x;
                sy = sy + q[k].y;
                sz = sz + q[k].z;
                m.mabs = fmaxf(m.mabs, (fabsf(q[k].x) + fabsf(q[k].y)) + fabsf(q[k].z));
                differ |= q[k].x != q[0].x || q[k].y != q[0].y || q[k].z != q[0].z;
            }
        const float fn = float(n_pts);
        m.mean[0] = sx / fn, m.mean[1] = sy / fn, m.mean[2] = sz / fn;
#pragma unroll
        for (uint32_t k = 0; k < kLeafRegPoints; ++k)
            if (k < n_pts && differ) {
                const float dx = q[k].x - m.mean[0], dy = q[k].y - m.mean[1], dz = q[k].z - m.mean[2];
                m.m2[0] = m.m2[0] + dx * dx;
                m.m2[1] = m.m2[1] + dy * dy;
                m.m2[2] = m.m2[2] + dz * dz;
                m.m2[3] = m.m2[3] + dx * dy;
                m.m2[4] = m.m2[4] + dx * dz;
                m.m2[5] = m.m2[5] + dy * dz;
            }
        m.kind = differ ? kRefitBox : kRefitPoint;
        return m;
    }
    Mom m{};
    m.n = n_pts;
    if (n_pts == 0) {
        m.kind = kRefitEmpty;
        return m;
    }
    const float4 p0 = pt[0];
    m.p0[0] = p0.x, m.p0[1] = p0.y, m.p0[2] = p0.z;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    bool differ = false;
    for (uint32_t k = 0; k < n_pts; ++k) {
        const float4 p = pt[k];
        sx = sx + p.x;
        sy = sy + p.y;
        sz = sz + p.z;
        m.mabs = fmaxf(m.mabs, (fabsf(p.x) + fabsf(p.y)) + fabsf(p.z));
        differ |= p.x != p0.x || p.y != p0.y || p.z != p0.z;
    }
    const float fn = float(n_pts);
    m.mean[0] = sx / fn, m.mean[1] = sy / fn, m.mean[2] = sz / fn;
    for (uint32_t k = 0; k < n_pts && differ; ++k) {
        const float4 p = pt[k];
        const float dx = p.x - m.mean[0], dy = p.y - m.mean[1], dz = p.z - m.mean[2];
        m.m2[0] = m.m2[0] + dx * dx;
        m.m2[1] = m.m2[1] + dy * dy;
        m.m2[2] = m.m2[2] + dz * dz;
        m.m2[3] = m.m2[3] + dx * dy;
        m.m2[4] = m.m2[4] + dx * dz;
        m.m2[5] = m.m2[5] + dy * dz;
    }
    m.kind = differ ? kRefitBox : kRefitPoint;
    return m;
}

// The moments of the union of two disjoint point sets (a first in leaf
// order).
__device__ Mom merge_mom(const Mom& a, const Mom& b) {
    if (b.n == 0) return a;
    if (a.n == 0) return b;
    Mom m;
    m.n = a.n + b.n;
    const float fa = float(a.n), fb = float(b.n), fn = float(m.n);
    const float d[3] = {b.mean[0] - a.mean[0], b.mean[1] - a.mean[1], b.mean[2] - a.mean[2]};
    const float f = fb / fn, w = (fa * fb) / fn;
    for (int i = 0; i < 3; ++i) m.mean[i] = a.mean[i] + d[i] * f, m.p0[i] = a.p0[i];
    const int r[6] = {0, 1, 2, 0, 0, 1}, c[6] = {0, 1, 2, 1, 2, 2};
    for (int i = 0; i < 6; ++i) m.m2[i] = (a.m2[i] + b.m2[i]) + (d[r[i]] * d[c[i]]) * w;
    m.mabs = fmaxf(a.mabs, b.mabs);
    const bool same = a.kind == kRefitPoint && b.kind == kRefitPoint && a.p0[0] == b.p0[0] && a.p0[1] == b.p0[1] &&
                      a.p0[2] == b.p0[2];
    m.kind = same ? kRefitPoint : kRefitBox;
    return m;
}

__device__ __forceinline__ unsigned arrive_acq_rel(unsigned* p) {
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// A thread per leaf box; the second child to arrive at a parent merges and
// climbs on. The arrival counter is reset by the thread that merges.
__global__ void __launch_bounds__(128) refit_climb_kernel(const float4* recs, const float4* tris,
                                                          const RefitTree* trees, const RefitBufs B) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.n_leaves) return;
    Mom* M = B.mom + T.scratch_base;
    uint32_t* arrive = B.arrive + T.scratch_base;
    uint32_t r = T.leaves[i];
    const uint2 rg = T.ranges[r];
    Mom m = leaf_mom(tris + 3ull * (T.tri_base + rg.x), 3u * rg.y);
    M[r] = m;
    for (;;) {
        const uint32_t p = T.parent[r];
        if (p == kNoRec) break;
        // the arrival releases this box's moments and acquires the sibling's
        if (arrive_acq_rel(arrive + p) == 0u) break;  // the sibling merges
        arrive[p] = 0u;
        const uint32_t c0 = __float_as_uint(__ldg(&recs[4ull * (T.rec_base + p) + 3].x)) - T.rec_base;
        const Mom a = c0 == r ? m : load_mom(M + c0);
        const Mom b = c0 + 1u == r ? m : load_mom(M + c0 + 1u);
        m = merge_mom(a, b);
        M[p] = m;
        r = p;
    }
}

// One thread per record: the eigensystem of M2 / n by the eig3 procedure in
// FP32; the box axes are the rows of the eigenvector matrix, as the reference
// takes them.
__global__ void refit_axes_kernel(const RefitTree* trees, const RefitBufs B) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= T.n_recs || T.ranges[r].y == ~0u) return;
    const Mom& m = B.mom[T.scratch_base + r];
    float4* ax = B.axes + 3ull * (T.scratch_base + r);
    if (m.kind != kRefitBox) {
        ax[0] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float fn = float(m.n);
    float c[6];
    for (int i = 0; i < 6; ++i) c[i] = m.m2[i] / fn;  // xx, yy, zz, xy, xz, yz
    float v[3][3] = {{c[0], c[3], c[4]}, {c[3], c[1], c[5]}, {c[4], c[5], c[2]}};
    float d[3], e[3];
    tridiagonalize(v, d, e);
    ql_sort(v, d, e, FLT_EPSILON);
    ax[0] = make_float4(v[0][0], v[0][1], v[0][2], 1.f);
    ax[1] = make_float4(v[1][0], v[1][1], v[1][2], 0.f);
    ax[2] = make_float4(v[2][0], v[2][1], v[2][2], 0.f);
}

// Order-preserving int key of a float (and its inverse): integer min/max of
// keys is float min/max.
__device__ __forceinline__ int fkey(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unkey(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }

// A thread per leaf box: the projections of its points (held in registers
// for the usual leaf of up to 4 triangles) on the axes of the leaf and of
// every box above it. Leaves are in tree order, so a warp's leaves share most
// of their chains.
__global__ void __launch_bounds__(128) refit_extent_kernel(const float4* tris, const RefitTree* trees,
                                                           const RefitBufs B) {
    const RefitTree T = trees[blockIdx.y];
    if (blockIdx.x * blockDim.x >= T.n_leaves) return;  // whole block
    const float4* AX = B.axes + 3ull * T.scratch_base;
    int4* EX = B.ext + 2ull * T.scratch_base;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint32_t r = kNoRec, n_pts = 0;
    const float4* pt = nullptr;
    float4 q[kLeafRegPoints];
    if (i < T.n_leaves) {
        r = T.leaves[i];
        const uint2 rg = T.ranges[r];
        n_pts = 3u * rg.y;
        pt = tris + 3ull * (T.tri_base + rg.x);
        if (n_pts) q[0] = pt[0];
#pragma unroll
        for (uint32_t k = 1; k < kLeafRegPoints; ++k) {
            q[k] = q[0];
            if (k < n_pts) q[k] = pt[k];
        }
    }
    while (__any_sync(kAll, r != kNoRec)) {
        int lo[3] = {kExtLo, kExtLo, kExtLo}, hi[3] = {kExtHi, kExtHi, kExtHi};
        bool box = false;
        uint32_t next = kNoRec;
        int4 cur_lo = make_int4(kExtHi, kExtHi, kExtHi, 0), cur_hi = make_int4(kExtLo, kExtLo, kExtLo, 0);
        if (r != kNoRec) {
            next = T.parent[r];  // issued with the axes' loads
            // the box's extents so far (a stale value only makes an atomic
            // that was not needed: the keys only move outwards)
            cur_lo = __ldcg(EX + 2ull * r);
            cur_hi = __ldcg(EX + 2ull * r + 1);
            const float4 a0 = AX[3ull * r], a1 = AX[3ull * r + 1], a2 = AX[3ull * r + 2];
            box = a0.w != 0.f && n_pts != 0;
            if (box) {
                const float4 a[3] = {a0, a1, a2};
                float flo[3], fhi[3];
#pragma unroll
                for (int j = 0; j < 3; ++j) flo[j] = fhi[j] = (a[j].x * q[0].x + a[j].y * q[0].y) + a[j].z * q[0].z;
                if (n_pts <= kLeafRegPoints) {
#pragma unroll
                    for (uint32_t k = 1; k < kLeafRegPoints; ++k)
#pragma unroll
                        for (int j = 0; j < 3; ++j) {
                            const float pr = (a[j].x * q[k].x + a[j].y * q[k].y) + a[j].z * q[k].z;
                            flo[j] = fminf(flo[j], pr);
                            fhi[j] = fmaxf(fhi[j], pr);
                        }
                } else {
                    for (uint32_t k = 1; k < n_pts; ++k) {
                        const float4 p = pt[k];
#pragma unroll
                        for (int j = 0; j < 3; ++j) {
                            const float pr = (a[j].x * p.x + a[j].y * p.y) + a[j].z * p.z;
                            flo[j] = fminf(flo[j], pr);
                            fhi[j] = fmaxf(fhi[j], pr);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < 3; ++j) lo[j] = fkey(flo[j]), hi[j] = fkey(fhi[j]);
            }
        }
        // lanes at the same box reduce together; the lowest one adds the result
        const unsigned grp = __match_any_sync(kAll, r);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            lo[j] = __reduce_min_sync(grp, lo[j]);
            hi[j] = __reduce_max_sync(grp, hi[j]);
        }
        if (box && lane == __ffs(grp) - 1) {
            int* e = reinterpret_cast<int*>(EX + 2ull * r);
            const int clo[3] = {cur_lo.x, cur_lo.y, cur_lo.z}, chi[3] = {cur_hi.x, cur_hi.y, cur_hi.z};
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                if (lo[j] < clo[j]) atomicMin(e + j, lo[j]);
                if (hi[j] > chi[j]) atomicMax(e + 4 + j, hi[j]);
            }
        }
        r = next;
    }
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

__device__ __forceinline__ Box special_box(const Mom& m) {
    Box b;
    b.c = m.kind == kRefitPoint ? make_float3(m.p0[0], m.p0[1], m.p0[2]) : make_float3(0.f, 0.f, 0.f);
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

__global__ void refit_assemble_kernel(float4* recs, const RefitTree* trees, const RefitBufs B) {
    const RefitTree T = trees[blockIdx.y];
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= T.n_recs || T.ranges[r].y == ~0u) return;
    const size_t q = size_t(T.scratch_base) + r;
    const Mom& m = B.mom[q];
    if (m.kind != kRefitBox) {
        write_box(recs, T.rec_base + r, special_box(m));
        return;
    }
    const float4* A = B.axes + 3 * q;
    float ax[9], lo[3], hi[3];
    for (int j = 0; j < 3; ++j) {
        const float4 a = A[j];
        ax[3 * j] = a.x, ax[3 * j + 1] = a.y, ax[3 * j + 2] = a.z;
    }
    int4* E = B.ext + 2 * q;
    const int4 el = E[0], eh = E[1];
    lo[0] = unkey(el.x), lo[1] = unkey(el.y), lo[2] = unkey(el.z);
    hi[0] = unkey(eh.x), hi[1] = unkey(eh.y), hi[2] = unkey(eh.z);
    E[0] = make_int4(kExtLo, kExtLo, kExtLo, 0);
    E[1] = make_int4(kExtHi, kExtHi, kExtHi, 0);
    write_box(recs, T.rec_base + r, assemble(ax, lo, hi, m.mabs));
}

__global__ void refit_scratch_init_kernel(const RefitBufs B, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        B.arrive[i] = 0u;
        B.ext[2ull * i] = make_int4(kExtLo, kExtLo, kExtLo, 0);
        B.ext[2ull * i + 1] = make_int4(kExtHi, kExtHi, kExtHi, 0);
    }
}

}  // namespace

cudaError_t init_refit_scratch(const RefitBufs& b, uint32_t n, cudaStream_t s) {
    if (n) refit_scratch_init_kernel<<<(n + 255u) / 256u < 4096u ? (n + 255u) / 256u : 4096u, 256, 0, s>>>(b, n);
    return cudaGetLastError();
}

cudaError_t launch_refit(float4* recs, float4* tris, const RefitTree* d_trees, uint32_t n_trees, uint32_t max_tris,
                         uint32_t max_recs, uint32_t max_leaves, const RefitBufs& b, cudaStream_t s) {
    if (n_trees == 0) return cudaSuccess;
    if (max_tris) refit_tris_kernel<<<dim3((3u * max_tris + 255u) / 256u, n_trees), 256, 0, s>>>(tris, d_trees);
    if (max_leaves)
        refit_climb_kernel<<<dim3((max_leaves + 127u) / 128u, n_trees), 128, 0, s>>>(recs, tris, d_trees, b);
    const dim3 per_rec((max_recs + 127u) / 128u, n_trees);
    refit_axes_kernel<<<per_rec, 128, 0, s>>>(d_trees, b);
    if (max_leaves)
        refit_extent_kernel<<<dim3((max_leaves + 127u) / 128u, n_trees), 128, 0, s>>>(tris, d_trees, b);
    refit_assemble_kernel<<<per_rec, 128, 0, s>>>(recs, d_trees, b);
    return cudaGetLastError();
}

}  // namespace cg
