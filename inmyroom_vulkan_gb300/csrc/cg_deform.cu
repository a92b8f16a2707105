// Morph targets, then linear-blend skinning, of the engine's skinning compute
// shader (shaders/dynamicMeshShader_glsl.comp:78-145, position path): one
// thread per vertex, the per-vertex math in cg_skin.cuh.
//
// Each joint's product joint_matrix * inverse_bind (the same for every vertex)
// is formed once per block in shared memory. Built without contraction, so the
// result is the same bits as the host restatement of the shader.
#include <cuda_runtime.h>

#include "cg_internal.h"
#include "cg_skin.cuh"

namespace cg {

namespace {

__global__ void __launch_bounds__(256) deform_kernel(const DeformParams* meshes) {
    extern __shared__ float mats[];  // n_joints x 16
    const DeformParams P = meshes[blockIdx.y];
    if (blockIdx.x * blockDim.x >= P.n_vertices) return;  // whole block
    for (uint32_t e = threadIdx.x; e < 16u * P.n_joints; e += blockDim.x)
        mats[e] = skin_entry(P.joint_matrices + 16ull * (e >> 4), P.inverse_bind + 16ull * (e >> 4), e & 15u);
    __syncthreads();
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= P.n_vertices) return;
    const float4 v = morph_vertex(P, x);
    const float4 r = skin_vertex(P, x, v, [&](uint32_t j, float* m) {
#pragma unroll
        for (uint32_t e = 0; e < 16; ++e) m[e] = mats[16u * j + e];
    });
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
