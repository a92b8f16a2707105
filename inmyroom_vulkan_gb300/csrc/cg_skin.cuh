// Morph + linear-blend skin of one vertex, shared by the deform kernel and the
// penetration-energy adjoint (which recomputes deformed vertices instead of
// keeping them): the same operations in the same order, so both give the same
// bits. The shader's position path (shaders/dynamicMeshShader_glsl.comp:78-145,
// no NORMALIZE, no ZERO_W):
//
//   morphed = base + sum_i w_i * target_i            (vec4, per component)
//   result  = sum over joint groups, joints x, y, z, w:
//             weight * ((joint_matrix * inverse_bind) * morphed)
//
// The product joint_matrix * inverse_bind is glm's column-major product with a
// left-to-right sum over k; the vec4 product is (c0 x + c1 y) + (c2 z + c3 w).
// Translation units that include this file are built without contraction.
#pragma once

#include <cuda_runtime.h>

#include "cg_internal.h"

namespace cg {

// Entry e (column e >> 2, row e & 3) of A * B, both column-major 4x4.
__device__ __forceinline__ float skin_entry(const float* A, const float* B, uint32_t e) {
    const uint32_t col = (e >> 2) & 3u, row = e & 3u;
    float acc = A[0 + row] * B[4 * col + 0];
    acc = acc + A[4 + row] * B[4 * col + 1];
    acc = acc + A[8 + row] * B[4 * col + 2];
    acc = acc + A[12 + row] * B[4 * col + 3];
    return acc;
}

// base + sum_i w_i * target_i of vertex x.
__device__ __forceinline__ float4 morph_vertex(const DeformParams& P, uint32_t x) {
    const float4* vx = reinterpret_cast<const float4*>(P.vertices) + size_t(P.n_targets + 1u) * x;
    float4 v = vx[0];
    for (uint32_t i = 0; i < P.n_targets; ++i) {
        const float w = P.morph_weights[i];
        const float4 t = vx[i + 1];
        v.x = v.x + w * t.x;
        v.y = v.y + w * t.y;
        v.z = v.z + w * t.z;
        v.w = v.w + w * t.w;
    }
    return v;
}

__device__ __forceinline__ float4 nan4() {
    const float q = __int_as_float(0x7fc00000);
    return make_float4(q, q, q, q);
}

// The skinned vertex x from its morphed position v. `mat(j, m)` gives joint
// j's skin matrix (joint_matrix * inverse_bind) as 16 floats: from shared
// memory in the deform kernel, formed on the spot with skin_entry elsewhere.
template <class MatFn>
__device__ __forceinline__ float4 skin_vertex(const DeformParams& P, uint32_t x, float4 v, MatFn mat) {
    float4 r = P.n_groups ? make_float4(0.f, 0.f, 0.f, 0.f) : v;
    for (uint32_t g = 0; g < P.n_groups; ++g) {
        const size_t k = size_t(P.n_groups) * x + g;
        const float4 w4 = reinterpret_cast<const float4*>(P.weights)[k];
        const ushort4 j4 = reinterpret_cast<const ushort4*>(P.joints)[k];
        const float we[4] = {w4.x, w4.y, w4.z, w4.w};
        const uint32_t je[4] = {j4.x, j4.y, j4.z, j4.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            if (je[e] >= P.n_joints) {  // a joint outside the matrices: the vertex comes out NaN
                r = nan4();
                continue;
            }
            float m[16];
            mat(je[e], m);
            const float tx = (m[0] * v.x + m[4] * v.y) + (m[8] * v.z + m[12] * v.w);
            const float ty = (m[1] * v.x + m[5] * v.y) + (m[9] * v.z + m[13] * v.w);
            const float tz = (m[2] * v.x + m[6] * v.y) + (m[10] * v.z + m[14] * v.w);
            const float tw = (m[3] * v.x + m[7] * v.y) + (m[11] * v.z + m[15] * v.w);
            r.x = r.x + we[e] * tx;
            r.y = r.y + we[e] * ty;
            r.z = r.z + we[e] * tz;
            r.w = r.w + we[e] * tw;
        }
    }
    return r;
}

// Vertex x deformed, forming each skin matrix on the spot (no shared table).
__device__ __forceinline__ float4 deform_vertex(const DeformParams& P, uint32_t x) {
    const float4 v = morph_vertex(P, x);
    return skin_vertex(P, x, v, [&](uint32_t j, float* m) {
        const float* A = P.joint_matrices + 16ull * j;
        const float* B = P.inverse_bind + 16ull * j;
#pragma unroll
        for (uint32_t e = 0; e < 16; ++e) m[e] = skin_entry(A, B, e);
    });
}

}  // namespace cg
