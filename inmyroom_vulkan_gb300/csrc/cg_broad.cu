// Broad phase: SweepAndPrune::ExecuteSweepAndPrune
// (src/CollisionDetection/SweepAndPrune.cpp:15-88) for a batch of entities.
//
// The reference sorts each axis's projections and sweeps an active list; the
// pairs it keeps are exactly those whose projections on all three axes
// overlap as closed intervals (an active entry stays while its end is not
// before the new start) with at least one entity that calls back, oriented
// as (the entity that starts earlier on U, the later one). The GPU tests that
// condition directly for every pair:
//   broad_project_kernel  a thread per entity: the world root box
//                         (Paralgram::MultiplyBy4x4Matrix) and its min/max
//                         projections on U, V, W
//                         (Paralgram::GetMinMaxProjectionToAxis)
//   broad_pairs_kernel    a thread per pair of a 32 x 32 tile (entities staged
//                         in shared memory), the three overlaps, the callback
//                         filter, one warp append per tile row
// Equal starts on U (where std::sort's order is unspecified) put the lower
// index first.
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr int kTile = 32;

__global__ void broad_project_kernel(const BroadParams P) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const DevTree& T = P.trees[P.tree_ids[i]];
    const float4* r = P.recs + 4ull * (T.rec_base + 1u);  // the root's box
    const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
    const Box root{make_float3(a.x, a.y, a.z), make_float3(a.w, b.x, b.y), make_float3(b.z, b.w, c.x),
                   make_float3(c.y, c.z, c.w)};
    const float* g = P.globals + 16ull * i;
    const Mat4 G{make_float4(g[0], g[1], g[2], g[3]), make_float4(g[4], g[5], g[6], g[7]),
                 make_float4(g[8], g[9], g[10], g[11]), make_float4(g[12], g[13], g[14], g[15])};
    const Box w = xform_box(G, root);
    float* out = P.proj + 6ull * i;
#pragma unroll
    for (int k = 0; k < 3; ++k) project(w, P.axes[k], out[2 * k], out[2 * k + 1]);
}

__global__ void __launch_bounds__(kTile * 8) broad_pairs_kernel(const BroadParams P) {
    __shared__ float pi[kTile][7], pj[kTile][7];
    const uint32_t bi = blockIdx.y * kTile, bj = blockIdx.x * kTile;
    if (bj + kTile <= bi) return;  // below the diagonal: whole tile
    const int tid = threadIdx.x;
    for (int e = tid; e < kTile * 7; e += blockDim.x) {
        const int r = e / 7, f = e % 7;
        const uint32_t ii = bi + r, jj = bj + r;
        pi[r][f] = ii < P.n ? (f < 6 ? P.proj[6ull * ii + f] : float(P.callback ? P.callback[ii] : 1u)) : 0.f;
        pj[r][f] = jj < P.n ? (f < 6 ? P.proj[6ull * jj + f] : float(P.callback ? P.callback[jj] : 1u)) : 0.f;
    }
    __syncthreads();
    const int lane = tid & 31, warp = tid >> 5;
    for (int r = warp; r < kTile; r += blockDim.x / 32) {
        const uint32_t i = bi + r, j = bj + lane;
        bool keep = i < P.n && j < P.n && i < j;
        if (keep) {
            const float* a = pi[r];
            const float* b = pj[lane];
            keep = (a[6] != 0.f || b[6] != 0.f) && a[1] >= b[0] && b[1] >= a[0] && a[3] >= b[2] && b[3] >= a[2] &&
                   a[5] >= b[4] && b[5] >= a[4];
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (!m) continue;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(P.count, (unsigned long long)__popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (keep) {
            const unsigned long long o = base + __popc(m & ((1u << lane) - 1u));
            if (o < P.cap) {
                const bool j_first = pj[lane][0] < pi[r][0];  // earlier start on U first; ties: lower index
                P.pairs[o] = j_first ? make_uint2(j, i) : make_uint2(i, j);
            }
        }
    }
}

}  // namespace

cudaError_t launch_broad(const BroadParams& p, cudaStream_t s) {
    if (p.n == 0) return cudaSuccess;
    broad_project_kernel<<<(p.n + 127u) / 128u, 128, 0, s>>>(p);
    const uint32_t tiles = (p.n + kTile - 1u) / kTile;
    broad_pairs_kernel<<<dim3(tiles, tiles), kTile * 8, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace cg
