// Differentiable penetration energy of the colliding triangle pairs, and its
// hand-written adjoint back through skinning, morph targets and the skeleton
// to per-bone axis-angle rotations and morph weights.
//
// Energy. For every colliding pair (doIntersept && !areCoplanar, the pairs
// the narrow phase stores) both directions of the reference's vertex-vs-plane
// test (src/CollisionDetection/CreateUncollideRays.cpp:102-112) add the squared
// depth of each vertex below the other triangle's plane:
//
//   E = sum over pairs, over (plane triangle T, the other triangle's vertex p)
//       of min(0, s)^2,   s = n_T . (p - T.p0),   n_T = unit face normal
//
// (Plane::CreatePlaneFromTriangle, src/Geometry/Plane.cpp:5-20: the normal of
// cross(p1 - p0, p2 - p0), normalised; s is Plane::IntersectPoint's n.p + d
// with d = -n.p0, taken about p0). Computed in the first tree's space, the
// second triangle moved by the query's matrix as the narrow phase moves it;
// terms in FP32, the sum in FP64.
//
// Adjoint, three kernels after the forward's collide and energy:
//   vertex_grad   one thread per pair: recomputes the deformed vertices of a
//                 deforming side (cg_skin.cuh, the deform kernel's bits; the
//                 forward keeps no vertex buffer for it), the gradient of the
//                 pair's terms with respect to its six vertices (the plane's
//                 through the normal: dn = (I - n n^T) dc / |c|), into a
//                 per-vertex buffer (side B's turned back into its model space
//                 by the transposed matrix)
//   skin_adjoint  one thread per vertex with a gradient g (and clears it):
//                 recomputes the morphed vertex u; for each influence (w, j)
//                 of skin matrix S_j = G_j IBM_j: dE/dS_j += w g u^T,
//                 dE/du += w S_j^T g; dE/dw_i = dE/du . target_i; block sums
//                 in shared memory, dE/dG_j = dE/dS_j IBM_j^T per block.
//   pose_backward a half-warp per pose (lane = matrix entry), bones in reverse
//                 order: dE/dG_parent += dE/dG_j L_j^T, dE/dL_j = G_parent^T
//                 dE/dG_j; then every axis-angle rotation's adjoint in parallel.
//
// Rotation of an axis-angle a (t = |a|, K = [a]x): R = I + A K + B K^2 with
// A = sin t / t, B = (1 - cos t) / t^2 (Rodrigues), and
// dR/da_m = A' a_m / t K + A [e_m]x + B' a_m / t K^2 + B ([e_m]x K + K [e_m]x),
// so with gR = dE/dR, w = the axial vector of gR - gR^T and tr = trace(gR):
// dE/da = a (A'/t a.w + B'/t (a^T gR a - t^2 tr)) + A w + B (gR^T a + gR a - 2 tr a).
// Below t = 0.25 the four coefficients come from their Taylor series.
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_internal.h"
#include "cg_skin.cuh"

namespace cg {

namespace {

// ---- rotation ----

struct RotCoef {
    float A, B, dA, dB;  // sin t / t, (1 - cos t) / t^2, A'(t) / t, B'(t) / t
};

__device__ __forceinline__ RotCoef rot_coef(float t2) {
    RotCoef k;
    if (t2 < 0.0625f) {
        k.A = 1.0f - t2 * (1.0f / 6.0f - t2 * (1.0f / 120.0f - t2 * (1.0f / 5040.0f)));
        k.B = 0.5f - t2 * (1.0f / 24.0f - t2 * (1.0f / 720.0f - t2 * (1.0f / 40320.0f)));
        k.dA = -1.0f / 3.0f + t2 * (1.0f / 30.0f - t2 * (1.0f / 840.0f - t2 * (1.0f / 45360.0f)));
        k.dB = -1.0f / 12.0f + t2 * (1.0f / 180.0f - t2 * (1.0f / 6720.0f - t2 * (1.0f / 453600.0f)));
    } else {
        const float t = sqrtf(t2);
        float s, c;
        sincosf(t, &s, &c);
        const float h = sinf(0.5f * t);
        const float omc = 2.0f * h * h;  // 1 - cos t without cancellation
        k.A = s / t;
        k.B = omc / t2;
        k.dA = (t * c - s) / (t2 * t);
        k.dB = (t * s - 2.0f * omc) / (t2 * t2);
    }
    return k;
}

// a[i] by selects (a run-time index would put a in local memory)
__device__ __forceinline__ float pick3(const float a[3], uint32_t i) { return i == 0u ? a[0] : (i == 1u ? a[1] : a[2]); }

// [a]x entry (r, c), r, c < 3.
__device__ __forceinline__ float skew(const float a[3], uint32_t r, uint32_t c) {
    if (r == c) return 0.0f;
    const float v = pick3(a, 3u - r - c);
    return ((r + 1u) % 3u == c) ? -v : v;
}

// Entry (r, c) of the local matrix T(offset) * R(a).
__device__ __forceinline__ float local_entry(const float a[3], float t2, const RotCoef& k, const float* off,
                                             uint32_t r, uint32_t c) {
    if (r == 3u) return c == 3u ? 1.0f : 0.0f;
    if (c == 3u) return off[r];
    const float diag = r == c ? 1.0f : 0.0f;
    return diag + k.A * skew(a, r, c) + k.B * (pick3(a, r) * pick3(a, c) - diag * t2);
}

// ---- posing ----

// A half-warp per pose; lane l holds entry l of the column-major 4x4 (row
// l & 3, column l >> 2). Three phases: every bone's local matrix
// T(offset) R(a) (the rotation's sines and divisions) in parallel over the
// bones, then the chain in bone order (a parent precedes its children), only
// 4x4 products on it; the adjoint runs the chain in reverse and then every
// rotation's adjoint in parallel again. What the chain touches (parents,
// offsets, angles, matrices, accumulators) is staged in shared memory when it
// fits (P.staged).
struct PoseStage {
    const int32_t* parent;
    const float* offsets;
    const float* aa;
    float* G;    // forward: local matrices, then the world matrices in place
    float* acc;  // adjoint: dE/dG accumulated over children
    float* L;    // adjoint: local matrices, rows 0-2 (12 per bone, column-major)
    float* gR;   // adjoint: dE/dR (9 per bone, row-major)
};

// Shared layout: parent[nb] (int), offsets[3 nb], then per pose slot aa[3 nb]
// and G[16 nb], and for the adjoint acc[16 nb], L[12 nb], gR[9 nb]. Unstaged,
// the adjoint's acc, L and gR are in P.grad_acc (37 nb per pose).
constexpr uint32_t kPoseFwdFloats = 19u, kPoseAdjFloats = 56u, kPoseAdjScratch = 37u;

__device__ __forceinline__ PoseStage pose_stage(const PoseParams& P, uint32_t slot, uint32_t pose, bool live,
                                                bool adjoint) {
    extern __shared__ float sh[];
    const uint32_t nb = P.n_bones;
    PoseStage st;
    if (!P.staged) {
        st.parent = P.parent;
        st.offsets = P.offsets;
        st.aa = P.axis_angles + 3ull * nb * pose;
        st.G = P.joint_matrices + 16ull * nb * pose;
        float* sc = adjoint ? P.grad_acc + size_t(kPoseAdjScratch) * nb * pose : nullptr;
        st.acc = sc;
        st.L = adjoint ? sc + 16u * nb : nullptr;
        st.gR = adjoint ? sc + 28u * nb : nullptr;
        return st;
    }
    int32_t* par = reinterpret_cast<int32_t*>(sh);
    float* off = sh + nb;
    float* mine = sh + 4u * nb + size_t(slot) * (adjoint ? kPoseAdjFloats : kPoseFwdFloats) * nb;
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) par[i] = P.parent[i];
    for (uint32_t i = threadIdx.x; i < 3u * nb; i += blockDim.x) off[i] = P.offsets[i];
    const uint32_t l = threadIdx.x & 15u;
    if (live) {
        const float* aa = P.axis_angles + 3ull * nb * pose;
        for (uint32_t i = l; i < 3u * nb; i += 16u) mine[i] = aa[i];
        if (adjoint) {
            const float* G = P.joint_matrices + 16ull * nb * pose;
            for (uint32_t i = l; i < 16u * nb; i += 16u) mine[3u * nb + i] = G[i];
        }
    }
    __syncthreads();
    st.parent = par;
    st.offsets = off;
    st.aa = mine;
    st.G = mine + 3u * nb;
    st.acc = adjoint ? mine + 19u * nb : nullptr;
    st.L = adjoint ? mine + 35u * nb : nullptr;
    st.gR = adjoint ? mine + 47u * nb : nullptr;
    return st;
}

// The local matrix of bone j: all 16 entries (column-major) into out[16], or
// rows 0-2 into out[12] (column-major, 3 per column).
template <int kRows>
__device__ __forceinline__ void local_matrix(const PoseStage& S, uint32_t j, float* out) {
    const float a[3] = {S.aa[3 * j], S.aa[3 * j + 1], S.aa[3 * j + 2]};
    const float t2 = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2];
    const RotCoef k = rot_coef(t2);
    const float* off = S.offsets + 3ull * j;
#pragma unroll
    for (uint32_t c = 0; c < 4; ++c)
#pragma unroll
        for (uint32_t r = 0; r < uint32_t(kRows); ++r) out[kRows * c + r] = local_entry(a, t2, k, off, r, c);
}

__global__ void __launch_bounds__(256) pose_kernel(const PoseParams P) {
    const uint32_t slot = threadIdx.x >> 4, l = threadIdx.x & 15u, r = l & 3u, c = l >> 2;
    const uint32_t pose = blockIdx.x * P.per_block + slot;
    const bool live = slot < P.per_block && pose < P.n_poses;
    const PoseStage S = pose_stage(P, slot, pose, live, false);
    const uint32_t nb = P.n_bones;
    // local matrices, bones spread over the half-warp
    if (live)
        for (uint32_t j = l; j < nb; j += 16u) local_matrix<4>(S, j, S.G + 16ull * j);
    __syncwarp();
    for (uint32_t j = 0; j < nb; ++j) {
        float g = 0.0f;
        if (live) {
            const float* Lc = S.G + 16ull * j + 4u * c;  // column c of the local matrix
            const float L0 = Lc[0], L1 = Lc[1], L2 = Lc[2], L3 = Lc[3];
            const int par = S.parent[j];
            if (par < 0) {
                g = r == 0u ? L0 : (r == 1u ? L1 : (r == 2u ? L2 : L3));
            } else {
                const float* Gp = S.G + 16ull * par;
                g = (Gp[r] * L0 + Gp[4 + r] * L1) + (Gp[8 + r] * L2 + Gp[12 + r] * L3);
            }
        }
        __syncwarp();  // every lane has read the column it needs before any lane writes
        if (live) S.G[16ull * j + l] = g;
        __syncwarp();  // the bone's entries are visible to the half-warp before a child reads them
    }
    if (P.staged && live) {
        float* out = P.joint_matrices + 16ull * nb * pose;
        for (uint32_t i = l; i < 16u * nb; i += 16u) out[i] = S.G[i];
    }
}

__global__ void __launch_bounds__(256) pose_backward_kernel(const PoseParams P) {
    const uint32_t lane = threadIdx.x & 31u, base = lane & 16u, l = lane & 15u, r = l & 3u, c = l >> 2;
    const uint32_t slot = threadIdx.x >> 4;
    const uint32_t pose_w = blockIdx.x * P.per_block + slot;
    const bool live = slot < P.per_block && pose_w < P.n_poses;
    // a spare half-warp follows a real pose's chain (its shuffles need the
    // whole warp) and writes nothing; staged, it has no shared slot and
    // shuffles zeros
    const uint32_t pose = live ? pose_w : P.n_poses - 1u;
    const bool stage_live = live || !P.staged;
    const PoseStage S = pose_stage(P, slot, pose, live, true);
    const uint32_t nb = P.n_bones;
    if (live) {
        const float* gin = P.grad_joint + 16ull * nb * pose;
        for (uint32_t i = l; i < 16u * nb; i += 16u) S.acc[i] = gin[i];
        for (uint32_t j = l; j < nb; j += 16u) local_matrix<3>(S, j, S.L + 12ull * j);
    }
    __syncwarp();
    for (uint32_t jj = nb; jj-- > 0;) {
        // every lane reads and writes only its own entry of acc; the entries
        // of other lanes come by shuffle
        const float g = stage_live ? S.acc[16ull * jj + l] : 0.0f;  // dE/dG_j, children's shares included
        float grow[4], gcol[4];
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
            grow[i] = __shfl_sync(0xffffffffu, g, base + 4u * i + r);  // g[r][i]
            gcol[i] = __shfl_sync(0xffffffffu, g, base + 4u * c + i);  // g[i][c]
        }
        const int par = S.parent[jj];
        float gL = g;
        if (par >= 0 && stage_live) {
            // dE/dG_par[r][c] += sum_i g[r][i] L[c][i] (row 3 of L: 0 0 0 1)
            const float* Lj = S.L + 12ull * jj;
            float add = c == 3u ? grow[3] : 0.0f;
            if (c < 3u)
                add = ((grow[0] * Lj[c] + grow[1] * Lj[3 + c]) + grow[2] * Lj[6 + c]) + grow[3] * Lj[9 + c];
            if (live) S.acc[16ull * par + l] += add;
            // dE/dL[r][c] = sum_i G_par[i][r] g[i][c]
            const float* Gp = S.G + 16ull * par;
            gL = (Gp[4 * r] * gcol[0] + Gp[4 * r + 1] * gcol[1]) + (Gp[4 * r + 2] * gcol[2] + Gp[4 * r + 3] * gcol[3]);
        }
        if (live && r < 3u && c < 3u) S.gR[9ull * jj + 3u * r + c] = gL;
        __syncwarp();
    }
    // the rotations' adjoints, bones spread over the half-warp
    if (live) {
        float* ga = P.grad_axis_angles + 3ull * nb * pose;
        for (uint32_t j = l; j < nb; j += 16u) {
            const float a[3] = {S.aa[3 * j], S.aa[3 * j + 1], S.aa[3 * j + 2]};
            const float t2 = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2];
            const RotCoef k = rot_coef(t2);
            const float* R = S.gR + 9ull * j;
            const float gR[3][3] = {{R[0], R[1], R[2]}, {R[3], R[4], R[5]}, {R[6], R[7], R[8]}};
            const float w[3] = {gR[2][1] - gR[1][2], gR[0][2] - gR[2][0], gR[1][0] - gR[0][1]};
            const float tr = (gR[0][0] + gR[1][1]) + gR[2][2];
            float Ra[3], Rta[3];
#pragma unroll
            for (uint32_t i = 0; i < 3; ++i) {
                Ra[i] = (gR[i][0] * a[0] + gR[i][1] * a[1]) + gR[i][2] * a[2];
                Rta[i] = (gR[0][i] * a[0] + gR[1][i] * a[1]) + gR[2][i] * a[2];
            }
            const float aw = (a[0] * w[0] + a[1] * w[1]) + a[2] * w[2];
            const float aRa = (a[0] * Ra[0] + a[1] * Ra[1]) + a[2] * Ra[2];
            const float radial = k.dA * aw + k.dB * (aRa - t2 * tr);
#pragma unroll
            for (uint32_t i = 0; i < 3; ++i)
                ga[3 * j + i] = a[i] * radial + k.A * w[i] + k.B * ((Rta[i] + Ra[i]) - 2.0f * tr * a[i]);
        }
    }
}

// ---- energy ----

__device__ __forceinline__ void load_tri(const float4* tris, uint32_t i, float3 p[3], uint32_t vi[3]) {
    const float4* t = tris + 3ull * i;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 v = __ldg(t + k);
        p[k] = make_float3(v.x, v.y, v.z);
        vi[k] = __float_as_uint(v.w);
    }
}

__device__ __forceinline__ Mat4 pair_matrix(const PackedQuery& Q) {
    return Mat4{__ldg(&Q.m[0]), __ldg(&Q.m[1]), __ldg(&Q.m[2]), __ldg(&Q.m[3])};
}

__device__ __forceinline__ float3 scale3f(float s, float3 v) { return make_float3(s * v.x, s * v.y, s * v.z); }
__device__ __forceinline__ float3 add3f(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }

// Terms of the points p below the plane of triangle q.
__device__ __forceinline__ float plane_energy(const float3 q[3], const float3 p[3]) {
    const float3 cr = cross3(sub3(q[1], q[0]), sub3(q[2], q[0]));
    const float len = length3(cr);
    const float3 n = make_float3(cr.x / len, cr.y / len, cr.z / len);
    float e = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float s = dot3(n, sub3(p[k], q[0]));
        if (s < 0.0f) e = e + s * s;
    }
    return e;
}

// Gradient of plane_energy(q, p) times g into gq, gp (added).
__device__ __forceinline__ void plane_energy_grad(const float3 q[3], const float3 p[3], float g, float3 gq[3],
                                                  float3 gp[3]) {
    const float3 e1 = sub3(q[1], q[0]), e2 = sub3(q[2], q[0]);
    const float3 cr = cross3(e1, e2);
    const float len = length3(cr);
    const float3 n = make_float3(cr.x / len, cr.y / len, cr.z / len);
    float3 gn = make_float3(0.f, 0.f, 0.f);
    bool any = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float3 d = sub3(p[k], q[0]);
        const float s = dot3(n, d);
        if (s < 0.0f) {
            const float f = 2.0f * g * s;
            gp[k] = add3f(gp[k], scale3f(f, n));
            gq[0] = sub3(gq[0], scale3f(f, n));
            gn = add3f(gn, scale3f(f, d));
            any = true;
        }
    }
    if (!any) return;
    const float ng = dot3(n, gn);
    const float3 gc = make_float3((gn.x - n.x * ng) / len, (gn.y - n.y * ng) / len, (gn.z - n.z * ng) / len);
    const float3 g1 = cross3(e2, gc), g2 = cross3(gc, e1);
    gq[1] = add3f(gq[1], g1);
    gq[2] = add3f(gq[2], g2);
    gq[0] = sub3(gq[0], add3f(g1, g2));
}

__device__ __forceinline__ unsigned long long stored_pairs(const EnergyParams& P) {
    const unsigned long long n = *reinterpret_cast<const volatile unsigned long long*>(&P.ctr->n_pairs);
    return n < P.pairs_cap ? n : P.pairs_cap;
}

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double part[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const uint32_t w = threadIdx.x >> 5;
    if ((threadIdx.x & 31u) == 0) part[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (uint32_t i = 0; i < (blockDim.x + 31u) / 32u; ++i) s += part[i];
    return s;
}

__global__ void __launch_bounds__(256) energy_kernel(const EnergyParams P) {
    const unsigned long long n = stored_pairs(P);
    double acc = 0.0;
    for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < n; i += gridDim.x * 256ull) {
        const cg_tri_pair pr = P.pairs[i];
        const PackedQuery& Q = P.q[pr.query];
        float3 pa[3], pb[3];
        uint32_t vi[3];
        load_tri(P.tris, __ldg(&Q.tri_base_a) + pr.tri_a, pa, vi);
        load_tri(P.tris, __ldg(&Q.tri_base_b) + pr.tri_b, pb, vi);
        const Mat4 M = pair_matrix(Q);
#pragma unroll
        for (int k = 0; k < 3; ++k) pb[k] = xform(M, pb[k], 1.0f);
        const float e = plane_energy(pb, pa) + plane_energy(pa, pb);
        if (e == e) acc += double(e);  // a degenerate triangle (NaN normal) adds nothing
    }
    const double s = block_sum(acc);
    if (threadIdx.x == 0 && s != 0.0) atomicAdd(P.energy, s);
}

// The side's three vertices: recomputed from its view when it deforms, else
// the stored triangle. False when a vertex index is outside the view.
__device__ __forceinline__ bool side_vertices(const EnergySide& S, const uint32_t vi[3], float3 p[3]) {
    if (S.d.n_vertices == 0) return true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (vi[k] >= S.d.n_vertices) return false;
        const float4 v = deform_vertex(S.d, vi[k]);
        p[k] = make_float3(v.x, v.y, v.z);
    }
    return true;
}

__device__ __forceinline__ void add_vgrad(float* vgrad, uint32_t base, uint32_t v, float3 g) {
    float* p = vgrad + 3ull * (base + v);
    atomicAdd(p, g.x);
    atomicAdd(p + 1, g.y);
    atomicAdd(p + 2, g.z);
}

__global__ void __launch_bounds__(256) vertex_grad_kernel(const EnergyParams P) {
    const unsigned long long n = stored_pairs(P);
    const float g = float(*P.grad_energy);
    for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < n; i += gridDim.x * 256ull) {
        const cg_tri_pair pr = P.pairs[i];
        const PackedQuery& Q = P.q[pr.query];
        const EnergySide& SA = P.sides[pr.query];
        const EnergySide& SB = P.sides[P.n_queries + pr.query];
        const bool da = SA.d.n_vertices != 0, db = SB.d.n_vertices != 0;
        if (!da && !db) continue;
        float3 pa[3], pb[3];
        uint32_t va[3], vb[3];
        load_tri(P.tris, __ldg(&Q.tri_base_a) + pr.tri_a, pa, va);
        load_tri(P.tris, __ldg(&Q.tri_base_b) + pr.tri_b, pb, vb);
        if (!side_vertices(SA, va, pa) || !side_vertices(SB, vb, pb)) continue;
        const Mat4 M = pair_matrix(Q);
#pragma unroll
        for (int k = 0; k < 3; ++k) pb[k] = xform(M, pb[k], 1.0f);
        float3 ga[3], gb[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) ga[k] = gb[k] = make_float3(0.f, 0.f, 0.f);
        plane_energy_grad(pb, pa, g, gb, ga);
        plane_energy_grad(pa, pb, g, ga, gb);
        if (da)
#pragma unroll
            for (int k = 0; k < 3; ++k) add_vgrad(P.vgrad, SA.grad_base, va[k], ga[k]);
        if (db)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                // back to the second tree's space: M^T g over the upper 3x3
                const float3 t = make_float3(dot3(make_float3(M.c0.x, M.c0.y, M.c0.z), gb[k]),
                                             dot3(make_float3(M.c1.x, M.c1.y, M.c1.z), gb[k]),
                                             dot3(make_float3(M.c2.x, M.c2.y, M.c2.z), gb[k]));
                add_vgrad(P.vgrad, SB.grad_base, vb[k], t);
            }
    }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// dE/dS_j (S_j = G_j * IBM_j, the skin matrix) is summed per block in shared
// memory: when every vertex of a warp with a gradient has the same joint in an
// influence slot (a tube's ring shares its joints), the warp sums its terms
// with shuffles and one lane adds them; otherwise each lane adds its own. At
// the end dE/dG_j = dE/dS_j IBM_j^T goes to the output once per block.
__global__ void __launch_bounds__(256) skin_adjoint_kernel(const EnergyParams P) {
    extern __shared__ float sh[];  // [nj][12] dE/dS (column-major rows 0-2), [nt] dE/dw, [nj][16] S when staged
    const EnergySide& ES = P.sides[P.deforming[blockIdx.y]];
    const DeformParams& D = ES.d;
    if (blockIdx.x * blockDim.x >= D.n_vertices) return;  // whole block
    const uint32_t nj = D.n_groups ? D.n_joints : 0u, nt = D.n_targets;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    float* gp = P.vgrad + 3ull * (ES.grad_base + x);
    if (x < D.n_vertices) gx = gp[0], gy = gp[1], gz = gp[2];
    const bool has = gx != 0.0f || gy != 0.0f || gz != 0.0f;
    if (!__syncthreads_or(has)) return;  // most blocks: no vertex of theirs touches a colliding pair
    if (has) gp[0] = gp[1] = gp[2] = 0.0f;  // the buffer is zero again for the next call
    float* gS = sh;
    float* gw = sh + 12u * nj;
    float* Ms = P.skin_in_smem ? gw + nt : nullptr;
    for (uint32_t e = threadIdx.x; e < 12u * nj + nt; e += blockDim.x) sh[e] = 0.0f;
    if (Ms)
        for (uint32_t e = threadIdx.x; e < 16u * nj; e += blockDim.x)
            Ms[e] = skin_entry(D.joint_matrices + 16ull * (e >> 4), D.inverse_bind + 16ull * (e >> 4), e & 15u);
    __syncthreads();
    const unsigned act = __ballot_sync(0xffffffffu, has);
    if (act) {
        const uint32_t leader = __ffs(act) - 1u;
        const float4 u = has ? morph_vertex(D, x) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float uc[4] = {u.x, u.y, u.z, u.w};
        float gu[4] = {0.f, 0.f, 0.f, 0.f};
        if (D.n_groups == 0) gu[0] = gx, gu[1] = gy, gu[2] = gz;
        for (uint32_t grp = 0; grp < D.n_groups; ++grp) {
            float4 w4 = make_float4(0.f, 0.f, 0.f, 0.f);
            ushort4 j4 = make_ushort4(0xffff, 0xffff, 0xffff, 0xffff);
            if (has) {
                const size_t kk = size_t(D.n_groups) * x + grp;
                w4 = reinterpret_cast<const float4*>(D.weights)[kk];
                j4 = reinterpret_cast<const ushort4*>(D.joints)[kk];
            }
            const float we[4] = {w4.x, w4.y, w4.z, w4.w};
            const uint32_t je[4] = {j4.x, j4.y, j4.z, j4.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const uint32_t j = je[e];
                const bool ok = has && j < nj && we[e] != 0.0f;
                const float wg[3] = {ok ? we[e] * gx : 0.f, ok ? we[e] * gy : 0.f, ok ? we[e] * gz : 0.f};
                const uint32_t jl = __shfl_sync(0xffffffffu, j, leader);
                const bool uniform = __all_sync(0xffffffffu, !ok || j == jl) && jl < nj;
                if (uniform) {
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc)
#pragma unroll
                        for (int rr = 0; rr < 3; ++rr) {
                            const float v = warp_sum(wg[rr] * uc[cc]);
                            if (lane == leader && v != 0.0f) atomicAdd(gS + 12u * jl + 3 * cc + rr, v);
                        }
                } else if (ok) {
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc)
#pragma unroll
                        for (int rr = 0; rr < 3; ++rr) atomicAdd(gS + 12u * j + 3 * cc + rr, wg[rr] * uc[cc]);
                }
                if (ok) {
                    float m[16];
                    if (Ms) {
#pragma unroll
                        for (int i = 0; i < 16; ++i) m[i] = Ms[16u * j + i];
                    } else {
#pragma unroll
                        for (uint32_t i = 0; i < 16; ++i)
                            m[i] = skin_entry(D.joint_matrices + 16ull * j, D.inverse_bind + 16ull * j, i);
                    }
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc)  // S_j^T (w g)
                        gu[cc] = gu[cc] + ((m[4 * cc] * wg[0] + m[4 * cc + 1] * wg[1]) + m[4 * cc + 2] * wg[2]);
                }
            }
        }
        const float4* tg = reinterpret_cast<const float4*>(D.vertices) + size_t(nt + 1u) * x + 1;
        for (uint32_t i = 0; i < nt; ++i) {
            float v = 0.0f;
            if (has) {
                const float4 d = tg[i];
                v = (gu[0] * d.x + gu[1] * d.y) + (gu[2] * d.z + gu[3] * d.w);
            }
            v = warp_sum(v);
            if (lane == leader && v != 0.0f) atomicAdd(gw + i, v);
        }
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < 12u * nj; e += blockDim.x) {
        const uint32_t j = e / 12u, cc = (e % 12u) / 3u, rr = e % 3u;
        const float* d = gS + 12u * j;
        const float* I = D.inverse_bind + 16ull * j;  // dE/dG = dE/dS IBM^T: sum_k dS[rr][k] IBM[cc][k]
        const float v = (d[rr] * I[cc] + d[3 + rr] * I[4 + cc]) + (d[6 + rr] * I[8 + cc] + d[9 + rr] * I[12 + cc]);
        if (v != 0.0f) atomicAdd(ES.grad_joint + 16ull * j + 4u * cc + rr, v);
    }
    for (uint32_t i = threadIdx.x; i < nt; i += blockDim.x)
        if (gw[i] != 0.0f) atomicAdd(ES.grad_morph + i, gw[i]);
}

}  // namespace

// Shared memory of the skin adjoint: dE/dS (12 floats per joint) and the skin
// matrices (16 per joint, up to kSkinStagedJoints joints; more joints form
// them on the spot), plus up to 256 morph weights.
constexpr uint32_t kSkinStagedJoints = 1024u;
constexpr uint32_t kSkinAdjointSmemFloats =
    (28u * kSkinStagedJoints > 12u * kMaxJoints ? 28u * kSkinStagedJoints : 12u * kMaxJoints) + 256u;

// Poses per block and whether the chain is staged in shared memory (at most
// kPoseSmem bytes: the adjoint's 56 floats per bone and pose, plus 4 per bone
// for the skeleton).
constexpr uint32_t kPoseSmem = 96u * 1024u;

void pose_shape(PoseParams& p, bool adjoint, uint32_t* threads, size_t* smem) {
    const size_t per_pose = sizeof(float) * (adjoint ? kPoseAdjFloats : kPoseFwdFloats) * p.n_bones;
    const size_t common = sizeof(float) * 4u * p.n_bones;
    const size_t fit = common < kPoseSmem ? (kPoseSmem - common) / per_pose : 0;
    p.staged = fit >= 1 ? 1u : 0u;
    p.per_block = p.staged ? uint32_t(fit < 8 ? fit : 8) : 8u;
    *threads = (16u * p.per_block + 31u) / 32u * 32u;
    *smem = p.staged ? common + per_pose * p.per_block : 0;
}

cudaError_t launch_pose(const PoseParams& p_in, cudaStream_t s) {
    if (p_in.n_poses == 0 || p_in.n_bones == 0) return cudaSuccess;
    PoseParams p = p_in;
    uint32_t threads;
    size_t smem;
    pose_shape(p, false, &threads, &smem);
    pose_kernel<<<(p.n_poses + p.per_block - 1u) / p.per_block, threads, smem, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_pose_backward(const PoseParams& p_in, cudaStream_t s) {
    if (p_in.n_poses == 0 || p_in.n_bones == 0) return cudaSuccess;
    PoseParams p = p_in;
    uint32_t threads;
    size_t smem;
    pose_shape(p, true, &threads, &smem);
    pose_backward_kernel<<<(p.n_poses + p.per_block - 1u) / p.per_block, threads, smem, s>>>(p);
    return cudaGetLastError();
}

cudaError_t energy_occupancy(int* blocks_per_sm) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, energy_kernel, 256, 0);
    if (e != cudaSuccess) return e;
    int b = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, vertex_grad_kernel, 256, 0);
    if (b < *blocks_per_sm) *blocks_per_sm = b;
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(pose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kPoseSmem));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(pose_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kPoseSmem));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(skin_adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(sizeof(float) * kSkinAdjointSmemFloats));
}

cudaError_t launch_energy(const EnergyParams& p, uint32_t blocks, cudaStream_t s) {
    energy_kernel<<<blocks, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_energy_backward(const EnergyParams& p, uint32_t blocks, uint32_t max_vertices, cudaStream_t s) {
    vertex_grad_kernel<<<blocks, 256, 0, s>>>(p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || p.n_deforming == 0 || max_vertices == 0) return e;
    EnergyParams q = p;
    // skin matrices staged in shared memory up to kSkinStagedJoints joints
    q.skin_in_smem = p.max_joints <= kSkinStagedJoints ? 1u : 0u;
    const size_t smem = sizeof(float) * ((q.skin_in_smem ? 28u : 12u) * p.max_joints + p.max_targets);
    skin_adjoint_kernel<<<dim3((max_vertices + 255u) / 256u, p.n_deforming), 256, smem, s>>>(q);
    return cudaGetLastError();
}

}  // namespace cg
