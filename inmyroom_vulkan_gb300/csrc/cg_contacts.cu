// Contacts and uncollide rays on the device: the part of
// CreateUncollideRays::ExecuteCreateUncollideRays
// (src/CollisionDetection/CreateUncollideRays.cpp:60-258) that follows the
// triangle-pair tests, for every query of a launch at once.
//
// The reference keeps one TriangleCandidateRays per triangle of a leaf pair,
// adds every colliding pair of that leaf pair into it, and merges the records
// of non-zero weight into a per-triangle map. Here every colliding pair adds
// directly into a hash table keyed by (side, query, triangle). A pair whose
// segment has zero length adds no weight and no midpoint, so it only matters
// for its "not outside" bits, and only when its leaf pair gave the same
// triangle some weight; such pairs are rare and take a side path:
//
//   contacts_accumulate  pairs of non-zero length: planes (Plane.cpp:5-28),
//                        weight, weighted midpoint, vertex bits -> table;
//                        pairs of zero length: listed, and their (side, leaf
//                        pair, triangle) groups entered into a group table
//   contacts_mark        (only when some pair had zero length) pairs of
//                        non-zero length flag their groups in that table
//   contacts_apply       zero-length pairs of flagged groups AND their vertex
//                        bits into the triangle's contact
//   contacts_emit        one thread per contact: the cg_contact record and its
//                        rays (find_rays_lambda, CreateUncollideRays.cpp:
//                        131-178), vertex rays deduplicated per (side, query,
//                        vertex index) through a set; the slot is emptied
//   ray_averages         per query: the mean ray origins
//                        (CreateUncollideRays.cpp:240-258); the vertex set and
//                        group table are emptied
//
// Geometry uses the reference's arithmetic (no contraction, IEEE division and
// square root), so masks, weights of single pairs and ray directions are the
// CPU's bits. Sums are kept in double: the weighted averages and mean origins
// agree with the CPU's float sums to float rounding, not bit for bit (the
// CPU's own order of addition follows its hash-map iteration).
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

__device__ __forceinline__ uint32_t hash64(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return uint32_t(k);
}

__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 divs3(float3 v, float s) { return make_float3(v.x / s, v.y / s, v.z / s); }
__device__ __forceinline__ float3 neg3(float3 v) { return make_float3(-v.x, -v.y, -v.z); }
__device__ __forceinline__ float3 scale3(float s, float3 v) { return make_float3(s * v.x, s * v.y, s * v.z); }

// Plane::Plane(normal, point) + CreatePlaneFromTriangle (Plane.cpp:5-20).
struct Plane {
    float3 n;
    float d;
};
__device__ __forceinline__ float3 face_normal(float3 p0, float3 p1, float3 p2) {
    return normalize3(cross3(sub3(p1, p0), sub3(p2, p0)));
}
__device__ __forceinline__ Plane plane_of(float3 p0, float3 p1, float3 p2) {
    const float3 fn = face_normal(p0, p1, p2);
    const float d = -dot3(p0, fn);
    const float len = length3(fn);
    return Plane{divs3(fn, len), d / len};
}
// Plane::IntersectPoint == OUTSIDE (Plane.cpp:22-28).
__device__ __forceinline__ bool outside(const Plane& pl, float3 p) { return dot3(p, pl.n) + pl.d > 0; }

// glm::adjointTranspose(glm::mat3(M)) as columns, and its product with a
// vector, (c0 * x + c1 * y) + c2 * z.
struct Mat3 {
    float3 c0, c1, c2;
};
__device__ __forceinline__ Mat3 cofactor3(const Mat4& M) {
    const float m00 = M.c0.x, m01 = M.c0.y, m02 = M.c0.z;  // m<column><row>
    const float m10 = M.c1.x, m11 = M.c1.y, m12 = M.c1.z;
    const float m20 = M.c2.x, m21 = M.c2.y, m22 = M.c2.z;
    Mat3 R;
    R.c0 = make_float3(m11 * m22 - m21 * m12, m20 * m12 - m10 * m22, m10 * m21 - m20 * m11);
    R.c1 = make_float3(m21 * m02 - m01 * m22, m00 * m22 - m20 * m02, m20 * m01 - m00 * m21);
    R.c2 = make_float3(m01 * m12 - m11 * m02, m10 * m02 - m00 * m12, m00 * m11 - m10 * m01);
    return R;
}
__device__ __forceinline__ float3 mul3(const Mat3& N, float3 v) {
    return make_float3((N.c0.x * v.x + N.c1.x * v.y) + N.c2.x * v.z, (N.c0.y * v.x + N.c1.y * v.y) + N.c2.y * v.z,
                       (N.c0.z * v.x + N.c1.z * v.y) + N.c2.z * v.z);
}

// glm-convention inverse (Laplace expansion over 2x2 minors), the expression
// tree of the host's cg_relative_matrix.
__device__ Mat4 inverse4(const Mat4& M) {
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

__device__ __forceinline__ Mat4 query_mat(const PackedQuery* Q) {
    return Mat4{__ldg(&Q->m[0]), __ldg(&Q->m[1]), __ldg(&Q->m[2]), __ldg(&Q->m[3])};
}

__device__ __forceinline__ void tri_at(const float4* tris, uint32_t i, float3 p[3], uint32_t vi[3]) {
    const float4* t = tris + 3ull * i;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 v = __ldg(t + k);
        p[k] = make_float3(v.x, v.y, v.z);
        vi[k] = __float_as_uint(v.w);
    }
}

// (side, query or leaf pair, index) in one word; queries and leaf pairs are < 2^31.
__device__ __forceinline__ unsigned long long make_key(uint32_t side, uint32_t hi, uint32_t lo) {
    return ((unsigned long long)side << 63) | ((unsigned long long)hi << 32) | lo;
}

// Everything the contact step needs of one colliding pair.
struct PairGeom {
    uint32_t q, tri_a, tri_b, leaf;
    float w;
    float3 mid;
    unsigned mask_a, mask_b;
};

// CreateUncollideRays.cpp:148-172 for pair i: the second triangle is moved
// into the first tree's space, each triangle's vertices are tested against
// the other's plane, w = |source - target| and mid = w * (source + target) / 2.
__device__ PairGeom pair_geom(const ContactParams& P, unsigned long long i, bool need_masks) {
    const cg_tri_pair r = P.pairs[i];
    PairGeom g;
    g.q = r.query;
    g.tri_a = r.tri_a;
    g.tri_b = r.tri_b;
    g.leaf = P.pair_leaf[i];
    const float3 s = make_float3(r.source[0], r.source[1], r.source[2]);
    const float3 t = make_float3(r.target[0], r.target[1], r.target[2]);
    g.w = length3(sub3(s, t));
    g.mid = divs3(scale3(g.w, add3(s, t)), 2.0f);
    g.mask_a = g.mask_b = 7u;
    if (!need_masks) return g;
    const PackedQuery* Q = P.q + r.query;
    const Mat4 M = query_mat(Q);
    float3 pa[3], pb[3];
    uint32_t vi[3];
    tri_at(P.tris, __ldg(&Q->tri_base_a) + r.tri_a, pa, vi);
    tri_at(P.tris, __ldg(&Q->tri_base_b) + r.tri_b, pb, vi);
#pragma unroll
    for (int k = 0; k < 3; ++k) pb[k] = xform(M, pb[k], 1.0f);
    const Plane plane_a = plane_of(pa[0], pa[1], pa[2]);
    const Plane plane_b = plane_of(pb[0], pb[1], pb[2]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (outside(plane_b, pa[k])) g.mask_a &= ~(1u << k);
        if (outside(plane_a, pb[k])) g.mask_b &= ~(1u << k);
    }
    return g;
}

// Hash sets with open addressing and linear probing over 64-bit keys stored
// `stride` words apart. No key is removed while a table is in use: each
// launch empties the slots it took once it is done with them.
__device__ int table_insert(unsigned long long* keys, uint32_t stride, uint32_t mask, unsigned long long key,
                            uint32_t* slot_out) {
    uint32_t slot = hash64(key) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        unsigned long long* k = keys + size_t(stride) * slot;
        unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(k);
        if (cur == kEmptyKey) cur = atomicCAS(k, kEmptyKey, key);
        if (cur == kEmptyKey || cur == key) {
            *slot_out = slot;
            return cur == kEmptyKey ? 1 : 0;  // 1: inserted now, 0: present
        }
        slot = (slot + 1u) & mask;
    }
    return -1;  // full
}

__device__ bool table_find(const unsigned long long* keys, uint32_t stride, uint32_t mask, unsigned long long key,
                           uint32_t* slot_out) {
    uint32_t slot = hash64(key) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long cur = keys[size_t(stride) * slot];
        if (cur == key) {
            *slot_out = slot;
            return true;
        }
        if (cur == kEmptyKey) return false;
        slot = (slot + 1u) & mask;
    }
    return false;
}

constexpr uint32_t kSlotWords = sizeof(ContactSlot) / sizeof(unsigned long long);
static_assert(sizeof(ContactSlot) % sizeof(unsigned long long) == 0, "contact slots hold whole key words");

__device__ void add_contact(const ContactParams& P, unsigned long long key, float3 mid, float w, unsigned mask) {
    uint32_t slot = 0;
    const int r = table_insert(&P.table->key, kSlotWords, P.table_mask, key, &slot);
    if (r < 0) {
        atomicOr(&P.ctr->c_overflow, CONTACT_TABLE);
        return;
    }
    if (r == 1) P.occupied[atomicAdd(&P.ctr->n_contacts, 1u)] = slot;  // once per slot: fits the list
    ContactSlot* s = P.table + slot;
    atomicAdd(&s->sx, double(mid.x));
    atomicAdd(&s->sy, double(mid.y));
    atomicAdd(&s->sz, double(mid.z));
    atomicAdd(&s->sw, double(w));
    if (mask != 7u) atomicAnd(&s->mask, mask);
}

__device__ void group_insert(const ContactParams& P, unsigned long long key) {
    uint32_t slot = 0;
    const int r = table_insert(P.gkeys, 1u, P.gtable_mask, key, &slot);
    if (r < 0)
        atomicOr(&P.ctr->c_overflow, CONTACT_ZERO);
    else if (r == 1)
        P.gocc[atomicAdd(&P.ctr->n_groups, 1u)] = slot;
}

__device__ void emit_ray(const ContactParams& P, uint32_t q, uint32_t side, float3 o, float3 d) {
    const unsigned idx = atomicAdd(&P.ctr->n_rays, 1u);
    if (idx < P.max_rays) {
        cg_ray r;
        r.query = q;
        r.side = side;
        r.origin[0] = o.x;
        r.origin[1] = o.y;
        r.origin[2] = o.z;
        r.direction[0] = d.x;
        r.direction[1] = d.y;
        r.direction[2] = d.z;
        P.rays[idx] = r;
    } else {
        atomicOr(&P.ctr->c_overflow, CONTACT_RAYS);
    }
    double* s = P.sums + 8ull * q + 4ull * side;
    atomicAdd(s + 0, double(o.x));
    atomicAdd(s + 1, double(o.y));
    atomicAdd(s + 2, double(o.z));
    atomicAdd(s + 3, 1.0);
}

__device__ __forceinline__ unsigned long long n_written_pairs(const ContactParams& P) {
    const unsigned long long n = P.ctr->n_pairs;
    return n < P.pairs_cap ? n : P.pairs_cap;
}

}  // namespace

__global__ void contacts_accumulate_kernel(const ContactParams P) {
    const unsigned long long tid = blockIdx.x * 1ull * blockDim.x + threadIdx.x;
    const unsigned long long stride = 1ull * gridDim.x * blockDim.x;
    for (unsigned long long j = tid; j < 8ull * P.n_queries; j += stride) P.sums[j] = 0.0;
    const unsigned long long n = n_written_pairs(P);
    for (unsigned long long i = tid; i < n; i += stride) {
        const PairGeom g = pair_geom(P, i, true);
        if (g.w != 0.0f) {
            add_contact(P, make_key(0u, g.q, g.tri_a), g.mid, g.w, g.mask_a);
            add_contact(P, make_key(1u, g.q, g.tri_b), g.mid, g.w, g.mask_b);
        } else {
            const unsigned z = atomicAdd(&P.ctr->n_zero, 1u);
            if (z < P.zero_cap) {
                P.zero[z] = uint32_t(i);
                group_insert(P, make_key(0u, g.leaf, g.tri_a));
                group_insert(P, make_key(1u, g.leaf, g.tri_b));
            } else {
                atomicOr(&P.ctr->c_overflow, CONTACT_ZERO);
            }
        }
    }
}

__global__ void contacts_mark_kernel(const ContactParams P) {
    if (P.ctr->n_zero == 0u) return;
    const unsigned long long n = n_written_pairs(P);
    for (unsigned long long i = blockIdx.x * 1ull * blockDim.x + threadIdx.x; i < n;
         i += 1ull * gridDim.x * blockDim.x) {
        const PairGeom g = pair_geom(P, i, false);
        if (g.w == 0.0f) continue;
        uint32_t slot = 0;
        if (table_find(P.gkeys, 1u, P.gtable_mask, make_key(0u, g.leaf, g.tri_a), &slot)) P.gflag[slot] = 1u;
        if (table_find(P.gkeys, 1u, P.gtable_mask, make_key(1u, g.leaf, g.tri_b), &slot)) P.gflag[slot] = 1u;
    }
}

__global__ void contacts_apply_kernel(const ContactParams P) {
    const uint32_t nz = min(P.ctr->n_zero, P.zero_cap);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nz; j += gridDim.x * blockDim.x) {
        const PairGeom g = pair_geom(P, P.zero[j], true);
        uint32_t gs = 0, cs = 0;
        if (table_find(P.gkeys, 1u, P.gtable_mask, make_key(0u, g.leaf, g.tri_a), &gs) && P.gflag[gs] &&
            table_find(&P.table->key, kSlotWords, P.table_mask, make_key(0u, g.q, g.tri_a), &cs))
            atomicAnd(&P.table[cs].mask, g.mask_a);
        if (table_find(P.gkeys, 1u, P.gtable_mask, make_key(1u, g.leaf, g.tri_b), &gs) && P.gflag[gs] &&
            table_find(&P.table->key, kSlotWords, P.table_mask, make_key(1u, g.q, g.tri_b), &cs))
            atomicAnd(&P.table[cs].mask, g.mask_b);
    }
}

__global__ void contacts_emit_kernel(const ContactParams P) {
    const uint32_t n = P.ctr->n_contacts;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        ContactSlot* s = P.table + P.occupied[j];
        const unsigned long long key = s->key;
        const uint32_t side = uint32_t(key >> 63);
        const uint32_t q = uint32_t(key >> 32) & 0x7fffffffu;
        const uint32_t tri = uint32_t(key);
        const float3 wsum = make_float3(float(s->sx), float(s->sy), float(s->sz));
        const float weight = float(s->sw);
        const unsigned mask = s->mask;
        s->sx = s->sy = s->sz = s->sw = 0.0;  // the slot is empty again for the next launch
        s->mask = 7u;
        s->key = kEmptyKey;
        // TriangleCandidateRays::GetWeightedAvg
        const float3 avg = divs3(wsum, weight);
        if (j < P.max_contacts) {
            cg_contact c;
            c.query = q;
            c.side = side;
            c.tri = tri;
            c.mask = mask;
            c.weighted_avg[0] = avg.x;
            c.weighted_avg[1] = avg.y;
            c.weighted_avg[2] = avg.z;
            c.weight = weight;
            P.contacts[j] = c;
        }

        const PackedQuery* Q = P.q + q;
        const float* nrm = P.trees[side ? __ldg(&Q->tree_b) : __ldg(&Q->tree_a)].nrm;
        const Mat4 M = query_mat(Q);
        float3 p[3], n3[3];
        uint32_t vi[3];
        tri_at(P.tris, (side ? __ldg(&Q->tri_base_b) : __ldg(&Q->tri_base_a)) + tri, p, vi);
        if (nrm) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float* np = nrm + 9ull * tri + 3 * k;
                n3[k] = make_float3(__ldg(np), __ldg(np + 1), __ldg(np + 2));
            }
        } else {  // a tree without vertex normals carries the face normal on all corners
            n3[0] = n3[1] = n3[2] = face_normal(p[0], p[1], p[2]);
        }
        if (side) {
#pragma unroll
            for (int k = 0; k < 3; ++k) p[k] = xform(M, p[k], 1.0f);
        }
        const Mat3 N = cofactor3(M);
        if (mask != 0u) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (!(mask & (1u << k))) continue;
                uint32_t vs = 0;
                const int r = table_insert(P.vkeys, 1u, P.vtable_mask, make_key(side, q, vi[k]), &vs);
                if (r < 0) atomicOr(&P.ctr->c_overflow, CONTACT_VERTICES);
                if (r != 1) continue;  // this vertex already has its ray
                P.vocc[atomicAdd(&P.ctr->n_vertices, 1u)] = vs;
                // TriangleNormal::GetNormal(index[, corrected_matrix]) (Triangle.cpp:180-195)
                const float3 nn = side ? normalize3(mul3(N, n3[k])) : normalize3(n3[k]);
                emit_ray(P, q, side, p[k], neg3(nn));
            }
        } else {
            // TrianglePosition::GetBarycentricOfPoint (Triangle.cpp:148-163) and
            // TriangleNormal::GetNormal(bary[, corrected_matrix]) (Triangle.cpp:197-212)
            const float3 v0 = sub3(p[1], p[0]), v1 = sub3(p[2], p[0]), v2 = sub3(avg, p[0]);
            const float d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1);
            const float d20 = dot3(v2, v0), d21 = dot3(v2, v1);
            const float den = d00 * d11 - d01 * d01;
            const float bx = (d11 * d20 - d01 * d21) / den;
            const float by = (d00 * d21 - d01 * d20) / den;
            const float b0 = 1.f - bx - by;
            const float3 in = add3(add3(scale3(b0, n3[0]), scale3(bx, n3[1])), scale3(by, n3[2]));
            const float3 nn = side ? normalize3(mul3(N, in)) : normalize3(in);
            emit_ray(P, q, side, avg, neg3(nn));
        }
    }
}

__global__ void ray_averages_kernel(const ContactParams P) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t nv = P.ctr->n_vertices;
    for (uint32_t j = i; j < nv; j += stride) P.vkeys[P.vocc[j]] = kEmptyKey;
    const uint32_t ng = P.ctr->n_groups;
    for (uint32_t j = i; j < ng; j += stride) {
        P.gkeys[P.gocc[j]] = kEmptyKey;
        P.gflag[P.gocc[j]] = 0u;
    }
    if (i >= P.n_queries) return;
    const double* s = P.sums + 8ull * i;
    float3 avg[2];
    for (int side = 0; side < 2; ++side) {
        const float3 sum = make_float3(float(s[4 * side]), float(s[4 * side + 1]), float(s[4 * side + 2]));
        avg[side] = divs3(sum, float(s[4 * side + 3]));
    }
    const float3 back = xform(inverse4(query_mat(P.q + i)), avg[1], 1.0f);
    cg_ray_average a;
    a.first[0] = avg[0].x;
    a.first[1] = avg[0].y;
    a.first[2] = avg[0].z;
    a.second[0] = back.x;
    a.second[1] = back.y;
    a.second[2] = back.z;
    a.rays_first = uint32_t(s[3]);
    a.rays_second = uint32_t(s[7]);
    P.averages[i] = a;
}

__global__ void init_tables_kernel(ContactSlot* table, uint32_t n_slots, unsigned long long* vkeys, uint32_t n_vslots,
                                   unsigned long long* gkeys, unsigned int* gflag, uint32_t n_gslots) {
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t i = i0; i < n_slots; i += stride) {
        ContactSlot s;
        s.key = kEmptyKey;
        s.sx = s.sy = s.sz = s.sw = 0.0;
        s.mask = 7u;
        s.pad = 0u;
        table[i] = s;
    }
    for (uint32_t i = i0; i < n_vslots; i += stride) vkeys[i] = kEmptyKey;
    for (uint32_t i = i0; i < n_gslots; i += stride) {
        gkeys[i] = kEmptyKey;
        gflag[i] = 0u;
    }
}

cudaError_t init_contact_tables(ContactSlot* table, uint32_t n_slots, unsigned long long* vkeys, uint32_t n_vslots,
                                unsigned long long* gkeys, unsigned int* gflag, uint32_t n_gslots, cudaStream_t s) {
    init_tables_kernel<<<1024, 256, 0, s>>>(table, n_slots, vkeys, n_vslots, gkeys, gflag, n_gslots);
    return cudaGetLastError();
}

cudaError_t launch_contacts(const ContactParams& p, uint32_t grid, cudaStream_t s) {
    contacts_accumulate_kernel<<<grid, 256, 0, s>>>(p);
    contacts_mark_kernel<<<grid, 256, 0, s>>>(p);
    contacts_apply_kernel<<<grid, 256, 0, s>>>(p);
    contacts_emit_kernel<<<grid, 256, 0, s>>>(p);
    const uint32_t qgrid = (p.n_queries + 255u) / 256u;
    ray_averages_kernel<<<qgrid > grid ? qgrid : grid, 256, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace cg
