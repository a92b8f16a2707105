// One frame of CollisionDetection::ExecuteCollisionDetection
// (src/CollisionDetection/CollisionDetection.cpp:38-129) on the device, up to
// the per-pair callback data (the ancestor fan-out, :106-124, needs the
// engine's entity tree and stays with the caller):
//   broad phase (cg_broad.cu) -> frame_queries_kernel: one collide query per
//   broad pair, relative = inverse(first current) * second current
//   (OBBtreesCollision.cpp:15) -> the collide step with contacts and rays ->
//   ray_pack: the step's rays, which come grouped per pair and side in the
//   reference's order (its unordered_map's iteration order), into the
//   shooting's layout -> frame_shoot_kernel: the shooting table (pairs where
//   an entity moved, :80-82) -> the shooting kernels (cg_shoot.cu) ->
//   frame_split_kernel: per pair with rays, the delta split by each entity's
//   movement of its mean ray origin (:84-97), appended to the results.
// Every step is the reference's arithmetic on the reference's rays in the
// reference's order.
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

__device__ __forceinline__ Mat4 mat16(const float* m) {
    return Mat4{make_float4(m[0], m[1], m[2], m[3]), make_float4(m[4], m[5], m[6], m[7]),
                make_float4(m[8], m[9], m[10], m[11]), make_float4(m[12], m[13], m[14], m[15])};
}

__device__ __forceinline__ void store16(float* o, const Mat4& M) {
    const float4 c[4] = {M.c0, M.c1, M.c2, M.c3};
#pragma unroll
    for (int k = 0; k < 4; ++k) o[4 * k] = c[k].x, o[4 * k + 1] = c[k].y, o[4 * k + 2] = c[k].z, o[4 * k + 3] = c[k].w;
}

__device__ __forceinline__ bool moved(const cg_frame_entity& e) {
    bool m = false;
#pragma unroll
    for (int k = 0; k < 16; ++k) m |= e.current_global[k] != e.previous_global[k];
    return m;
}

__global__ void frame_queries_kernel(const FrameParams P) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n_pairs) return;
    const uint2 pr = P.pairs[k];
    const cg_frame_entity& a = P.entities[pr.x];
    const cg_frame_entity& b = P.entities[pr.y];
    cg_query q;
    q.tree_a = a.tree;
    q.tree_b = b.tree;
    store16(q.relative, mul4(inverse4(mat16(a.current_global)), mat16(b.current_global)));
    P.queries[k] = q;
}

__device__ __forceinline__ uint32_t stored_rays(const FrameParams& P) {
    const uint32_t n = *reinterpret_cast<const volatile unsigned*>(P.n_rays);
    return n < P.max_rays ? n : P.max_rays;
}

// The rays, grouped per pair and side by the contact step, as origin +
// direction and a tag (pair | from the second entity << 31), in place.
__global__ void ray_pack_kernel(const FrameParams P) {
    const uint32_t n = stored_rays(P);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const cg_ray& r = P.rays[i];
        float* o = P.grouped + 6ull * i;
        o[0] = r.origin[0], o[1] = r.origin[1], o[2] = r.origin[2];
        o[3] = r.direction[0], o[4] = r.direction[1], o[5] = r.direction[2];
        P.tags[i] = r.query | (r.side ? 0x80000000u : 0u);
    }
}

__global__ void frame_shoot_kernel(const FrameParams P) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n_pairs) return;
    const uint2 pr = P.pairs[k];
    const cg_frame_entity& a = P.entities[pr.x];
    const cg_frame_entity& b = P.entities[pr.y];
    ShootQuery s;
    for (int i = 0; i < 16; ++i) s.relative[i] = P.queries[k].relative[i], s.first_global[i] = a.current_global[i];
    s.tree_a = a.tree;
    s.tree_b = b.tree;
    s.ray_first = P.offsets[2u * k];
    s.n_first = P.counts[2u * k];
    s.n_second = P.counts[2u * k + 1u];
    s.pad[0] = (moved(a) || moved(b)) ? 1u : 0u;  // CollisionDetection.cpp:80-82: shoot only when one moved
    s.pad[1] = s.pad[2] = 0u;
    P.shoot[k] = s;
}

// CollisionDetection::PointMovementBetweenFrames (CollisionDetection.cpp:143-151).
__device__ __forceinline__ float movement(float3 p, const float* cur, const float* prev) {
    const float3 a = xform(mat16(cur), p, 1.0f), b = xform(mat16(prev), p, 1.0f);
    return length3(sub3(a, b));
}

__global__ void frame_split_kernel(const FrameParams P) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n_pairs) return;
    const uint32_t nf = P.counts[2u * k], ns = P.counts[2u * k + 1u];
    if (nf + ns == 0u) return;  // CollisionDetection.cpp:62-66: no rays, no callback
    const uint2 pr = P.pairs[k];
    const cg_frame_entity& a = P.entities[pr.x];
    const cg_frame_entity& b = P.entities[pr.y];
    cg_frame_result r;
    r.first = pr.x;
    r.second = pr.y;
    float3 d1 = make_float3(0.f, 0.f, 0.f), d2 = d1;
    if (P.shoot[k].pad[0]) {
        const float* dl = P.deltas + 3ull * k;
        const float3 delta = make_float3(dl[0], dl[1], dl[2]);
        const cg_ray_average& av = P.averages[k];
        const float m1 = movement(make_float3(av.first[0], av.first[1], av.first[2]), a.current_global,
                                  a.previous_global);
        const float m2 = movement(make_float3(av.second[0], av.second[1], av.second[2]), b.current_global,
                                  b.previous_global);
        const float total = m1 + m2;
        const float f1 = m1 / total, f2 = m2 / total;
        d1 = make_float3(-delta.x * f1, -delta.y * f1, -delta.z * f1);
        d2 = make_float3(delta.x * f2, delta.y * f2, delta.z * f2);
    }
    r.first_delta[0] = d1.x, r.first_delta[1] = d1.y, r.first_delta[2] = d1.z;
    r.second_delta[0] = d2.x, r.second_delta[1] = d2.y, r.second_delta[2] = d2.z;
    r.query = k;
    r.reserved = 0u;
    const unsigned long long o = atomicAdd(P.n_results, 1ull);
    if (o < P.results_cap) P.results[o] = r;
}

}  // namespace

cudaError_t launch_frame_queries(const FrameParams& p, cudaStream_t s) {
    if (p.n_pairs) frame_queries_kernel<<<(p.n_pairs + 127u) / 128u, 128, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_frame_rays(const FrameParams& p, uint32_t blocks, cudaStream_t s) {
    if (!p.n_pairs) return cudaSuccess;
    ray_pack_kernel<<<blocks, 256, 0, s>>>(p);
    frame_shoot_kernel<<<(p.n_pairs + 127u) / 128u, 128, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_frame_split(const FrameParams& p, cudaStream_t s) {
    if (p.n_pairs) frame_split_kernel<<<(p.n_pairs + 127u) / 128u, 128, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace cg
