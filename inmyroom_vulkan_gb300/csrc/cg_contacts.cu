// Contacts and uncollide rays on the device: the part of
// CreateUncollideRays::ExecuteCreateUncollideRays
// (src/CollisionDetection/CreateUncollideRays.cpp:60-201) that follows the
// triangle-pair tests, for every query of a launch at once.
//
// The reference keeps one TriangleCandidateRays per triangle of a leaf pair,
// adds every colliding pair of that leaf pair into it, and merges the records
// of non-zero weight into a per-triangle map. Here every colliding pair adds
// directly into a hash table keyed by (side, query, triangle). A pair whose
// segment has zero length adds no weight and no midpoint, so it only matters
// for its "not outside" bits, and only when its leaf pair gives the same
// triangle some weight: such a pair (rare) re-runs the triangle tests of its
// leaf pair for that triangle (at most a leaf's four triangles) to find out.
//
//   contacts_accumulate  one thread per colliding pair: planes (Plane.cpp:
//                        5-28), weight, weighted midpoint, vertex bits ->
//                        table; also empties the vertex set of the previous
//                        contacts launch and the per-query origin sums
//   contacts_emit        one thread per contact: the cg_contact record and its
//                        rays (find_rays_lambda, CreateUncollideRays.cpp:
//                        131-178), vertex rays deduplicated per (side, query,
//                        vertex index) through a set; the slot is emptied.
//                        The last block to finish computes the per-query mean
//                        origins (CreateUncollideRays.cpp:183-198).
//
// Appends to the shared lists (contacts, vertices, rays) take one atomic per
// warp. Geometry uses the reference's arithmetic (no contraction, IEEE division and
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

// (side, query, index) in one word; queries are < 2^31.
__device__ __forceinline__ unsigned long long make_key(uint32_t side, uint32_t hi, uint32_t lo) {
    return ((unsigned long long)side << 63) | ((unsigned long long)hi << 32) | lo;
}

constexpr unsigned kFullMask = 0xffffffffu;

__device__ __forceinline__ unsigned lanes_below() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// One atomic per warp: lane l gets base + (number of its lanes below l that
// take a slot) when `take` is set. All 32 lanes must call it together.
__device__ __forceinline__ unsigned warp_append(unsigned* counter, unsigned take) {
    const unsigned lane = threadIdx.x & 31u;
    unsigned incl = take;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= unsigned(o)) incl += t;
    }
    const unsigned total = __shfl_sync(kFullMask, incl, 31);
    unsigned base = 0;
    if (lane == 31 && total) base = atomicAdd(counter, total);
    base = __shfl_sync(kFullMask, base, 31);
    return base + incl - take;
}

// warp_append for two adjacent counters (lo, and hi at lo + 1, an 8-byte
// aligned pair) with one 64-bit atomic.
__device__ __forceinline__ void warp_append2(unsigned* lo, unsigned take_lo, unsigned take_hi, unsigned* base_lo,
                                             unsigned* base_hi) {
    const unsigned lane = threadIdx.x & 31u;
    unsigned a = take_lo, b = take_hi;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned ta = __shfl_up_sync(kFullMask, a, o);
        const unsigned tb = __shfl_up_sync(kFullMask, b, o);
        if (lane >= unsigned(o)) {
            a += ta;
            b += tb;
        }
    }
    const unsigned total_a = __shfl_sync(kFullMask, a, 31), total_b = __shfl_sync(kFullMask, b, 31);
    unsigned long long old = 0;
    if (lane == 31 && (total_a | total_b))
        old = atomicAdd(reinterpret_cast<unsigned long long*>(lo),
                        (unsigned long long)total_a | ((unsigned long long)total_b << 32));
    old = __shfl_sync(kFullMask, old, 31);
    *base_lo = unsigned(old) + a - take_lo;
    *base_hi = unsigned(old >> 32) + b - take_hi;
}

// Everything the contact step needs of one colliding pair.
struct PairGeom {
    uint32_t q, tri_a, tri_b, leaf;  // query, tree-local triangles, leaf-list index
    uint32_t ia, ib;                 // arena triangles
    float w;
    float3 mid;
    unsigned mask_a, mask_b;
};

// CreateUncollideRays.cpp:87-112 for pair i: the second triangle is moved
// into the first tree's space, each triangle's vertices are tested against
// the other's plane, w = |source - target| and mid = w * (source + target) / 2.
// The pair record and its side record load together, then the matrix and
// both triangles.
__device__ PairGeom pair_geom(const ContactParams& P, unsigned long long i) {
    const cg_tri_pair r = P.pairs[i];
    const uint4 x = P.pair_aux[i];
    PairGeom g;
    g.q = x.w;
    g.tri_a = r.tri_a;
    g.tri_b = r.tri_b;
    g.leaf = x.z;
    g.ia = x.x;
    g.ib = x.y;
    const float3 s = make_float3(r.source[0], r.source[1], r.source[2]);
    const float3 t = make_float3(r.target[0], r.target[1], r.target[2]);
    g.w = length3(sub3(s, t));
    g.mid = divs3(scale3(g.w, add3(s, t)), 2.0f);
    const Mat4 M = query_mat(P.q + x.w);
    float3 pa[3], pb[3];
    uint32_t vi[3];
    tri_at(P.tris, x.x, pa, vi);
    tri_at(P.tris, x.y, pb, vi);
#pragma unroll
    for (int k = 0; k < 3; ++k) pb[k] = xform(M, pb[k], 1.0f);
    const Plane plane_a = plane_of(pa[0], pa[1], pa[2]);
    const Plane plane_b = plane_of(pb[0], pb[1], pb[2]);
    g.mask_a = g.mask_b = 7u;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (outside(plane_b, pa[k])) g.mask_a &= ~(1u << k);
        if (outside(plane_a, pb[k])) g.mask_b &= ~(1u << k);
    }
    return g;
}

// True when the leaf pair of a zero-length pair gives its triangle on `side`
// some weight: the triangle tests of that triangle against the other leaf's
// triangles (the narrow phase's own tests, re-run) have a colliding pair of
// non-zero length.
__device__ bool group_has_weight(const ContactParams& P, const PairGeom& g, uint32_t side) {
    const uint4 lp = P.leaf_list[g.leaf];  // (query, first triangle a, first triangle b, counts)
    const Mat4 M = query_mat(P.q + g.q);
    const uint32_t cnt_a = lp.w & 0xffffu, cnt_b = lp.w >> 16;
    const uint32_t n = side ? cnt_a : cnt_b;
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t ia = side ? lp.y + k : g.ia;
        const uint32_t ib = side ? g.ib : lp.z + k;
        float3 a[3], b[3];
        uint32_t vi[3];
        tri_at(P.tris, ia, a, vi);
        tri_at(P.tris, ib, b, vi);
#pragma unroll
        for (int j = 0; j < 3; ++j) b[j] = xform(M, b[j], 1.0f);
        float3 src, tgt;
        if (tri_tri(a[0], a[1], a[2], b[0], b[1], b[2], src, tgt) == TT_HIT && length3(sub3(src, tgt)) != 0.0f)
            return true;
    }
    return false;
}

// Hash sets with open addressing and linear probing over 64-bit keys stored
// `stride` words apart. No key is removed while a set is in use: each launch
// empties the slots it took once it is done with them. An insert is a CAS at
// the key's home slot (issued by the caller, so that a thread's inserts are
// in flight together) and, after a collision, at the following slots.
struct Probe {
    unsigned long long* keys;
    uint32_t stride, mask;
    __device__ unsigned long long* at(uint32_t slot) const { return keys + size_t(stride) * slot; }
    __device__ uint32_t home(unsigned long long key) const { return hash64(key) & mask; }
};

// Result of an insert whose home-slot CAS returned `cur`: 1 inserted, 0
// already present (*slot set either way), -1 the table is full.
__device__ int finish_insert(const Probe& T, unsigned long long key, unsigned long long cur, uint32_t home,
                             uint32_t* slot) {
    uint32_t s = home;
    for (uint32_t probe = 0;; ++probe) {
        if (cur == kEmptyKey || cur == key) {
            *slot = s;
            return cur == kEmptyKey ? 1 : 0;
        }
        if (probe == T.mask) return -1;
        s = (s + 1u) & T.mask;
        cur = atomicCAS(T.at(s), kEmptyKey, key);
    }
}

constexpr uint32_t kSlotWords = sizeof(ContactSlot) / sizeof(unsigned long long);
static_assert(sizeof(ContactSlot) % sizeof(unsigned long long) == 0, "contact slots hold whole key words");

__device__ __forceinline__ Probe contact_table(const ContactParams& P) {
    return Probe{&P.table->key, kSlotWords, P.table_mask};
}

__device__ __forceinline__ void add_to_slot(const ContactParams& P, uint32_t slot, float3 mid, float w, unsigned mask) {
    ContactSlot* s = P.table + slot;
    atomicAdd(&s->sx, double(mid.x));
    atomicAdd(&s->sy, double(mid.y));
    atomicAdd(&s->sz, double(mid.z));
    atomicAdd(&s->sw, double(w));
    if (mask != 7u) atomicAnd(&s->mask, mask);
}

__device__ __forceinline__ unsigned long long n_written_pairs(const ContactParams& P) {
    const unsigned long long n = P.ctr->n_pairs;
    return n < P.pairs_cap ? n : P.pairs_cap;
}

}  // namespace

__global__ void __launch_bounds__(256) contacts_accumulate_kernel(const ContactParams P) {
    const unsigned long long tid = blockIdx.x * 1ull * blockDim.x + threadIdx.x;
    const unsigned long long stride = 1ull * gridDim.x * blockDim.x;
    // vertex set of the previous contacts launch, and this launch's origin sums
    const uint32_t nv = P.ctr->prev_vertices;
    for (unsigned long long j = tid; j < nv; j += stride) P.vkeys[P.vocc[j]] = kEmptyKey;
    for (unsigned long long j = tid; j < 8ull * P.n_queries; j += stride) P.sums[j] = 0.0;

    const unsigned long long n = n_written_pairs(P);
    const unsigned long long warp0 = tid & ~31ull;  // warp-uniform loop: warp_append needs all lanes
    for (unsigned long long base = warp0; base < n; base += stride) {
        const unsigned long long i = base + (threadIdx.x & 31u);
        int ra = -2, rb = -2;  // -2: no slot wanted, else the insert's result
        uint32_t sa = 0, sb = 0;
        if (i < n) {
            const PairGeom g = pair_geom(P, i);
            const Probe T = contact_table(P);
            const unsigned long long ka = make_key(0u, g.q, g.tri_a), kb = make_key(1u, g.q, g.tri_b);
            // a pair of zero length only ANDs its vertex bits, and only where
            // its leaf pair gives the triangle weight
            const bool want_a = g.w != 0.0f || group_has_weight(P, g, 0u);
            const bool want_b = g.w != 0.0f || group_has_weight(P, g, 1u);
            const uint32_t ha = T.home(ka), hb = T.home(kb);
            const unsigned long long ca = want_a ? atomicCAS(T.at(ha), kEmptyKey, ka) : 0ull;
            const unsigned long long cb = want_b ? atomicCAS(T.at(hb), kEmptyKey, kb) : 0ull;
            if (want_a) ra = finish_insert(T, ka, ca, ha, &sa);
            if (want_b) rb = finish_insert(T, kb, cb, hb, &sb);
            if (ra == -1 || rb == -1) atomicOr(&P.ctr->c_overflow, CONTACT_TABLE);
            if (ra >= 0) {
                if (g.w != 0.0f) add_to_slot(P, sa, g.mid, g.w, g.mask_a);
                else atomicAnd(&P.table[sa].mask, g.mask_a);
            }
            if (rb >= 0) {
                if (g.w != 0.0f) add_to_slot(P, sb, g.mid, g.w, g.mask_b);
                else atomicAnd(&P.table[sb].mask, g.mask_b);
            }
        }
        __syncwarp();
        const unsigned new_a = ra == 1, new_b = rb == 1;
        const unsigned o = warp_append(&P.ctr->n_contacts, new_a + new_b);
        if (new_a) P.occupied[o] = sa;  // one entry per slot: the list never outgrows the table
        if (new_b) P.occupied[o + new_a] = sb;
    }
}

// Three lanes per contact (lanes 0..29 of a warp, ten contacts per warp and
// turn): lane k of a contact makes the ray of the contact's vertex k, and
// lane 0 also writes the contact record and, when no vertex is "not outside",
// the ray from the weighted average.
constexpr uint32_t kContactsPerWarp = 10;

__global__ void __launch_bounds__(256, 3) contacts_emit_kernel(const ContactParams P) {
    __shared__ bool last_block;
    if (blockIdx.x == 0 && threadIdx.x == 0) P.ctr->prev_vertices = 0u;  // the accumulate kernel emptied them
    const uint32_t n = P.ctr->n_contacts;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t k = lane % 3u;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t cb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kContactsPerWarp; cb < n;
         cb += n_warps * kContactsPerWarp) {
        const uint32_t j = cb + lane / 3u;
        const bool valid = lane < 3u * kContactsPerWarp && j < n;
        ContactSlot* s = nullptr;
        unsigned long long key = 0;
        double sx = 0, sy = 0, sz = 0, sw = 0;
        unsigned mask = 0;
        if (valid) {
            s = P.table + P.occupied[j];
            key = s->key;
            sx = s->sx;
            sy = s->sy;
            sz = s->sz;
            sw = s->sw;
            mask = s->mask;
        }
        __syncwarp();  // the contact's three lanes have read the slot
        bool ray = false, vertex = false;
        float3 ro_ = make_float3(0.f, 0.f, 0.f), rd = ro_;
        uint32_t vs = 0, q = 0, side = 0;
        if (valid) {
            side = uint32_t(key >> 63);
            q = uint32_t(key >> 32) & 0x7fffffffu;
            const uint32_t tri = uint32_t(key);
            // TriangleCandidateRays::GetWeightedAvg
            const float3 avg = divs3(make_float3(float(sx), float(sy), float(sz)), float(sw));
            if (k == 0) {
                s->sx = s->sy = s->sz = s->sw = 0.0;  // the slot is empty again for the next launch
                s->mask = 7u;
                s->key = kEmptyKey;
                if (j < P.max_contacts) {
                    cg_contact c;
                    c.query = q;
                    c.side = side;
                    c.tri = tri;
                    c.mask = mask;
                    c.weighted_avg[0] = avg.x;
                    c.weighted_avg[1] = avg.y;
                    c.weighted_avg[2] = avg.z;
                    c.weight = float(sw);
                    P.contacts[j] = c;
                }
            }
            const bool mine = mask != 0u ? (mask >> k) & 1u : k == 0;
            if (mine) {
                const PackedQuery* Q = P.q + q;
                const float* nrm = P.trees[side ? __ldg(&Q->tree_b) : __ldg(&Q->tree_a)].nrm;
                const Mat4 M = query_mat(Q);
                float3 p[3], n3[3];
                uint32_t vi[3];
                tri_at(P.tris, (side ? __ldg(&Q->tri_base_b) : __ldg(&Q->tri_base_a)) + tri, p, vi);
                if (nrm) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float* np = nrm + 9ull * tri + 3 * c;
                        n3[c] = make_float3(__ldg(np), __ldg(np + 1), __ldg(np + 2));
                    }
                } else {  // a tree without vertex normals carries the face normal on all corners
                    n3[0] = n3[1] = n3[2] = face_normal(p[0], p[1], p[2]);
                }
                if (side) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) p[c] = xform(M, p[c], 1.0f);
                }
                const Mat3 N = cofactor3(M);
                if (mask != 0u) {
                    // one ray per vertex index and side of the query
                    const Probe V{P.vkeys, 1u, P.vtable_mask};
                    const unsigned long long vk = make_key(side, q, k == 0 ? vi[0] : (k == 1 ? vi[1] : vi[2]));
                    const uint32_t home = V.home(vk);
                    const int r = finish_insert(V, vk, atomicCAS(V.at(home), kEmptyKey, vk), home, &vs);
                    if (r < 0) atomicOr(&P.ctr->c_overflow, CONTACT_VERTICES);
                    if (r == 1) {
                        // TriangleNormal::GetNormal(index[, corrected_matrix]) (Triangle.cpp:180-195)
                        const float3 nk = k == 0 ? n3[0] : (k == 1 ? n3[1] : n3[2]);
                        const float3 nn = side ? normalize3(mul3(N, nk)) : normalize3(nk);
                        ro_ = k == 0 ? p[0] : (k == 1 ? p[1] : p[2]);
                        rd = neg3(nn);
                        ray = vertex = true;
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
                    ro_ = avg;
                    rd = neg3(nn);
                    ray = true;
                }
            }
        }
        __syncwarp();
        unsigned vo, ro;
        warp_append2(&P.ctr->n_vertices, vertex ? 1u : 0u, ray ? 1u : 0u, &vo, &ro);
        if (ray) {
            if (vertex) P.vocc[vo] = vs;  // never more entries than the set's slots
            if (ro < P.max_rays) {
                cg_ray r;
                r.query = q;
                r.side = side;
                r.origin[0] = ro_.x;
                r.origin[1] = ro_.y;
                r.origin[2] = ro_.z;
                r.direction[0] = rd.x;
                r.direction[1] = rd.y;
                r.direction[2] = rd.z;
                P.rays[ro] = r;
            } else {
                atomicOr(&P.ctr->c_overflow, CONTACT_RAYS);
            }
            double* sum = P.sums + 8ull * q + 4ull * side;
            atomicAdd(sum + 0, double(ro_.x));
            atomicAdd(sum + 1, double(ro_.y));
            atomicAdd(sum + 2, double(ro_.z));
            atomicAdd(sum + 3, 1.0);
        }
    }

    // The last block to finish: per-query mean origins, from the sums every
    // block has completed (each block publishes its atomics before it counts
    // itself done).
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last_block = atomicAdd(&P.ctr->emit_done, 1u) == gridDim.x - 1u;
    }
    __syncthreads();
    if (!last_block) return;
    __threadfence();
    for (uint32_t i = threadIdx.x; i < P.n_queries; i += blockDim.x) {
        const double* s = P.sums + 8ull * i;
        float3 avg[2];
        float cnt[2];
        for (int side = 0; side < 2; ++side) {
            const float3 sum = make_float3(float(__ldcg(s + 4 * side)), float(__ldcg(s + 4 * side + 1)),
                                           float(__ldcg(s + 4 * side + 2)));
            cnt[side] = float(__ldcg(s + 4 * side + 3));
            avg[side] = divs3(sum, cnt[side]);
        }
        const float3 back = xform(inverse4(query_mat(P.q + i)), avg[1], 1.0f);
        cg_ray_average a;
        a.first[0] = avg[0].x;
        a.first[1] = avg[0].y;
        a.first[2] = avg[0].z;
        a.second[0] = back.x;
        a.second[1] = back.y;
        a.second[2] = back.z;
        a.rays_first = uint32_t(cnt[0]);
        a.rays_second = uint32_t(cnt[1]);
        P.averages[i] = a;
    }
}

__global__ void init_tables_kernel(ContactSlot* table, uint32_t n_slots, unsigned long long* vkeys, uint32_t n_vslots) {
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
}

cudaError_t init_contact_tables(ContactSlot* table, uint32_t n_slots, unsigned long long* vkeys, uint32_t n_vslots,
                                cudaStream_t s) {
    init_tables_kernel<<<1024, 256, 0, s>>>(table, n_slots, vkeys, n_vslots);
    return cudaGetLastError();
}

// Copies the step's results to the caller's host buffers (written through the
// device's mapping of them) as 16-byte words: colliding pairs (36-byte
// records; the last words of an odd count as 4-byte words), rays and
// per-query averages. Counts from the
// step's counters, capped by what the device buffers and the host buffers hold.
__global__ void __launch_bounds__(256) copy_out_kernel(const CopyOutParams P) {
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long i0 = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const Counters& C = *P.ctr;
    if (P.host_pairs) {
        // 36-byte records: whole 16-byte words, then the last 4-byte words
        const unsigned long long n = min(min(C.n_pairs, P.pairs_avail), P.host_pairs_cap);
        const unsigned long long words = 9ull * n, quads = words >> 2;
        const uint4* src4 = reinterpret_cast<const uint4*>(P.pairs);
        uint4* dst4 = reinterpret_cast<uint4*>(P.host_pairs);
        for (unsigned long long w = i0; w < quads; w += stride) dst4[w] = __ldg(src4 + w);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(P.pairs);
        uint32_t* dst = reinterpret_cast<uint32_t*>(P.host_pairs);
        for (unsigned long long w = 4ull * quads + i0; w < words; w += stride) dst[w] = __ldg(src + w);
    }
    if (P.host_rays) {
        const unsigned long long n = min(min((unsigned long long)C.n_rays, P.rays_avail), P.host_rays_cap);
        const uint4* src = reinterpret_cast<const uint4*>(P.rays);
        uint4* dst = reinterpret_cast<uint4*>(P.host_rays);
        for (unsigned long long w = i0; w < 2ull * n; w += stride) dst[w] = __ldg(src + w);
    }
    if (P.host_averages) {
        const unsigned long long n = min((unsigned long long)C.n_queries, P.host_averages_cap);
        const uint4* src = reinterpret_cast<const uint4*>(P.averages);
        uint4* dst = reinterpret_cast<uint4*>(P.host_averages);
        for (unsigned long long w = i0; w < 2ull * n; w += stride) dst[w] = __ldg(src + w);
    }
}

cudaError_t launch_copy_out(const CopyOutParams& p, uint32_t blocks, cudaStream_t s) {
    copy_out_kernel<<<blocks, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t contacts_occupancy(int* accumulate_blocks_per_sm, int* emit_blocks_per_sm) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(accumulate_blocks_per_sm, contacts_accumulate_kernel,
                                                                  256, 0);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(emit_blocks_per_sm, contacts_emit_kernel, 256, 0);
}

cudaError_t launch_contacts(const ContactParams& p, uint32_t accumulate_grid, uint32_t emit_grid, cudaStream_t s) {
    contacts_accumulate_kernel<<<accumulate_grid, 256, 0, s>>>(p);
    contacts_emit_kernel<<<emit_grid, 256, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace cg
