// Morph targets, then linear-blend skinning, of the engine's skinning compute
// shader (shaders/dynamicMeshShader_glsl.comp:78-145, position path: no
// NORMALIZE, no ZERO_W): one thread per vertex.
//
//   morphed = base + sum_i w_i * target_i            (vec4, per component)
//   result  = sum over joint groups, joints x, y, z, w:
//             weight * ((joint_matrix * inverse_bind) * morphed)
//
// Each joint's product joint_matrix * inverse_bind (glm convention, the same
// for every vertex) is formed once per block in shared memory; the vec4
// product is (c0 x + c1 y) + (c2 z + c3 w). Built without contraction, so the
// result is the same bits as the host restatement of the shader.
#include <cuda_runtime.h>

#include "cg_internal.h"

namespace cg {

namespace {

__global__ void __launch_bounds__(256) deform_kernel(const DeformParams* meshes) {
    extern __shared__ float mats[];  // n_joints x 16
    const DeformParams P = meshes[blockIdx.y];
    if (blockIdx.x * blockDim.x >= P.n_vertices) return;  // whole block
    for (uint32_t e = threadIdx.x; e < 16u * P.n_joints; e += blockDim.x) {
        const uint32_t j = e >> 4, col = (e >> 2) & 3u, row = e & 3u;
        const float* A = P.joint_matrices + 16ull * j;
        const float* B = P.inverse_bind + 16ull * j;
        float acc = A[0 + row] * B[4 * col + 0];
        acc = acc + A[4 + row] * B[4 * col + 1];
        acc = acc + A[8 + row] * B[4 * col + 2];
        acc = acc + A[12 + row] * B[4 * col + 3];
        mats[e] = acc;
    }
    __syncthreads();
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= P.n_vertices) return;
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
                r = make_float4(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000),
                                __int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
                continue;
            }
            const float* m = mats + 16u * je[e];
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
    reinterpret_cast<float4*>(P.out)[x] = r;
}

}  // namespace

cudaError_t deform_smem_limit() {
    return cudaFuncSetAttribute(deform_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(sizeof(float) * 16u * kMaxJoints));
}

cudaError_t launch_deform(const DeformParams* d_meshes, uint32_t n_meshes, uint32_t max_vertices, uint32_t max_joints,
                          cudaStream_t s) {
    if (n_meshes == 0 || max_vertices == 0) return cudaSuccess;
    const size_t smem = sizeof(float) * 16u * max_joints;
    deform_kernel<<<dim3((max_vertices + 255u) / 256u, n_meshes), 256, smem, s>>>(d_meshes);
    return cudaGetLastError();
}

}  // namespace cg
