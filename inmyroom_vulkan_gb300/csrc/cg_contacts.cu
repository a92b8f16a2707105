// Contacts and uncollide rays on the device: the part of
// CreateUncollideRays::ExecuteCreateUncollideRays
// (src/CollisionDetection/CreateUncollideRays.cpp:60-201) that follows the
// triangle-pair tests, for every query of a launch at once, with the
// reference's results bit for bit.
//
// What the reference's results depend on, and how each is reproduced:
// * Per triangle and leaf pair it folds the colliding pairs' weighted
//   midpoints and weights in float, starting from zero, in its pair loop's
//   order (:79-113), then merges the records of non-zero weight into a map, in
//   the order of the candidate leaf pairs (:117-127). All leaf pairs that hold
//   one triangle share its leaf, and in the descent's depth-first order they
//   come in the order of the other leaf's first triangle; within a leaf pair
//   the fold runs over the other triangle's index. So both folds follow from
//   sorting a triangle's colliding pairs by the other triangle: no global
//   order is needed for the sums.
// * Its rays come out of a std::unordered_map<uint32_t, ...> in the map's
//   iteration order (:138), and the per-query mean origin folds them in that
//   order (:185-196). With GCC's libstdc++ that order is a function of the
//   insertion order of the keys and of the sizes at which the table grows:
//   after every growth the table lists its buckets most recently started
//   first, each bucket's keys most recently placed first, where a growth
//   re-places the keys in the order the table held them. The growth sizes are
//   read from the host's own std::unordered_map (cg_api.cu); the insertion
//   order is the order of the triangles' first leaf pairs of non-zero weight
//   in the descent, then the triangle index.
// * The descent's order of two leaf pairs is the order of their paths from
//   the root pair (one bit per split, OBBtree.cpp:414-476). A contact's path
//   is found again by walking from the roots to its leaf pair, taking the
//   reference's split decision at every node pair (the larger surface, the
//   second tree's box as transformed, ties to the first tree) and the child
//   that holds the leaf.
//
// Kernels (one launch each, in this order):
//   contacts_pairs    thread per colliding pair: planes (Plane.cpp:5-28),
//                     weight, weighted midpoint, vertex bits; the two
//                     triangles' slots in the contact table, a place in each
//                     slot's list; its leaf pair listed once; empties the
//                     previous launch's global vertex set
//   contacts_alloc    each slot's place in the contribution list (one atomic
//                     per 32 slots), the slots of more than kFoldThread
//                     contributions listed; the first block: the maps'
//                     offsets
//   contacts_scatter  thread per pair: both contributions into their lists
//   contacts_paths    (on a branch beside alloc and scatter) lane pair per
//                     listed leaf pair: the two trees' ways down walked side
//                     by side, merged into its descent path
//   contacts_fold     thread per slot (a warp per listed large slot): the
//                     list sorted by the other triangle, the reference's two
//                     folds, the path of the first leaf pair of non-zero
//                     weight; the triangle into its map. Its last block
//                     ranks the maps, largest first
//   contacts_order    persistent, a block per map in that order: the
//                     insertion order (sort by path, triangle, in registers
//                     on the narrowest exact key), the iteration order (the
//                     growth steps: by one warp up to 32 keys, else counting
//                     passes), the rays (find_rays_lambda,
//                     CreateUncollideRays.cpp:131-178: one per vertex index,
//                     at its first corner in iteration order, else from the
//                     weighted average; the vertex set in shared memory when
//                     it fits), the mean origin in ray order. Its last block
//                     places each map's first record and ray
//   contacts_emit     block per map: records and rays to their places;
//                     empties the table slots, leaf-pair marks and map
//                     counters it used
// Geometry uses the reference's arithmetic (no contraction, IEEE division and
// square root).
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

// Everything the contact step needs of one colliding pair.
struct PairGeom {
    uint32_t q, tri_a, tri_b;  // query, tree-local triangles
    float w;
    float3 mid;
    unsigned mask_a, mask_b;
};

// CreateUncollideRays.cpp:87-112 for pair i: the second triangle is moved
// into the first tree's space, each triangle's vertices are tested against
// the other's plane, w = |source - target| and mid = w * (source + target) / 2.
__device__ PairGeom pair_geom(const ContactParams& P, unsigned long long i) {
    const cg_tri_pair r = P.pairs[i];
    const uint4 x = P.pair_aux[i];
    PairGeom g;
    g.q = x.w;
    g.tri_a = r.tri_a;
    g.tri_b = r.tri_b;
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

__device__ __forceinline__ int insert(const Probe& T, unsigned long long key, uint32_t* slot) {
    const uint32_t h = T.home(key);
    return finish_insert(T, key, atomicCAS(T.at(h), kEmptyKey, key), h, slot);
}

constexpr uint32_t kSlotWords = sizeof(ContactSlot) / sizeof(unsigned long long);
static_assert(sizeof(ContactSlot) % sizeof(unsigned long long) == 0, "contact slots hold whole key words");

__device__ __forceinline__ Probe contact_table(const ContactParams& P) {
    return Probe{&P.table->key, kSlotWords, P.table_mask};
}

__device__ __forceinline__ unsigned long long n_written_pairs(const ContactParams& P) {
    const unsigned long long n = P.ctr->n_pairs;
    return n < P.pairs_cap ? n : P.pairs_cap;
}

__device__ __forceinline__ uint32_t n_slots(const ContactParams& P) {
    const uint32_t n = *reinterpret_cast<const volatile unsigned*>(&P.ctr->n_contacts);
    return n < P.table_mask + 1u ? n : P.table_mask + 1u;
}

// Exclusive scans by one block (blockDim.x a multiple of 32, at most 1024) of
// get1(0..n1-1) and get2(0..n2-1) side by side: each thread takes a
// contiguous run of each, the runs' sums are scanned with warp shuffles, every
// warp adds up the partial sums of the warps before it, put(i, prefix) is
// called in order within each run. Two barriers; the totals go to every
// thread. `part` holds 64 words. get must return the same value twice.
template <class Get1, class Put1, class Get2, class Put2>
__device__ void block_scan2(uint32_t n1, uint32_t n2, uint32_t* part, Get1 get1, Put1 put1, Get2 get2, Put2 put2,
                            uint32_t& total1, uint32_t& total2) {
    const uint32_t T = blockDim.x, t = threadIdx.x, lane = t & 31u, warp = t >> 5, nw = T >> 5;
    const uint32_t per1 = (n1 + T - 1u) / T, a0 = min(n1, t * per1), a1 = min(n1, a0 + per1);
    const uint32_t per2 = (n2 + T - 1u) / T, c0 = min(n2, t * per2), c1 = min(n2, c0 + per2);
    uint32_t s1 = 0, s2 = 0;
    for (uint32_t i = a0; i < a1; ++i) s1 += get1(i);
    for (uint32_t i = c0; i < c1; ++i) s2 += get2(i);
    uint32_t i1 = s1, i2 = s2;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v1 = __shfl_up_sync(kFullMask, i1, o);
        const uint32_t v2 = __shfl_up_sync(kFullMask, i2, o);
        if (lane >= uint32_t(o)) {
            i1 += v1;
            i2 += v2;
        }
    }
    if (lane == 31u) {
        part[warp] = i1;
        part[32u + warp] = i2;
    }
    __syncthreads();
    uint32_t b1 = 0, b2 = 0, t1 = 0, t2 = 0;
    for (uint32_t w = 0; w < nw; ++w) {
        const uint32_t p1 = part[w], p2 = part[32u + w];
        if (w < warp) {
            b1 += p1;
            b2 += p2;
        }
        t1 += p1;
        t2 += p2;
    }
    uint32_t r1 = b1 + i1 - s1, r2 = b2 + i2 - s2;
    for (uint32_t i = a0; i < a1; ++i) {
        const uint32_t v = get1(i);
        put1(i, r1);
        r1 += v;
    }
    for (uint32_t i = c0; i < c1; ++i) {
        const uint32_t v = get2(i);
        put2(i, r2);
        r2 += v;
    }
    __syncthreads();
    total1 = t1;
    total2 = t2;
}

// One exclusive scan of get(0..n-1) (block_scan2 with an empty second).
// Returns the total.
template <class Get, class Put>
__device__ uint32_t block_scan(uint32_t n, uint32_t* part, Get get, Put put) {
    uint32_t total = 0, none = 0;
    block_scan2(
        n, 0u, part, get, put, [](uint32_t) { return 0u; }, [](uint32_t, uint32_t) {}, total, none);
    return total;
}

struct WalkRec {
    Box box;
    uint32_t ref, meta, split;
    float surf;
};

__device__ __forceinline__ WalkRec walk_rec(const float4* recs, uint32_t r) {
    const float4* p = recs + 4ull * r;
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    WalkRec R;
    R.box.c = make_float3(a.x, a.y, a.z);
    R.box.u = make_float3(a.w, b.x, b.y);
    R.box.v = make_float3(b.z, b.w, c.x);
    R.box.w = make_float3(c.y, c.z, c.w);
    R.ref = __float_as_uint(d.x);
    R.meta = __float_as_uint(d.y);
    R.surf = d.z;
    R.split = __float_as_uint(d.w);
    return R;
}

// A path of `depth` splits (1 <= depth < 128) held in the low bits of
// (hi, lo), moved to the top (left-aligned in 128 bits).
__device__ __forceinline__ void align_path(unsigned long long& hi, unsigned long long& lo, uint32_t depth) {
    if (depth == 0u || depth >= 128u) return;
    const uint32_t s = 128u - depth;
    if (s >= 64u) {
        hi = lo << (s - 64u);
        lo = 0ull;
    } else {
        hi = (hi << s) | (lo >> (64u - s));
        lo <<= s;
    }
}

// The path of the simultaneous descent (OBBtree::IntersectOBBtreesRecursive,
// src/Geometry/OBBtree.cpp:414-476) from the root pair to leaf pair lp
// (query, first triangle a, first triangle b, counts; arena indices): at every
// node pair the reference's split decision (two inner boxes: the first tree's
// when its surface is at least the second's as transformed; else the inner
// one), then the child whose subtree holds the leaf's first triangle (bit 0
// left, 1 right, from the record's split word). A step on the first tree
// reads the child's link word only; one on the second tree reads the child's
// box to transform it. The way down each tree is fixed by the leaf alone, so
// each tree's next node is loaded one step ahead: a split of the other tree
// finds it there. Left-aligned in 128 bits; *depth = splits.
__device__ void descent_path(const PackedQuery* queries, const DevTree* trees, const float4* recs, uint4 lp,
                             unsigned long long& hi, unsigned long long& lo, uint32_t& depth) {
    const PackedQuery* Q = queries + lp.x;
    const uint32_t base_a = trees[__ldg(&Q->tree_a)].rec_base;
    const uint32_t base_b = trees[__ldg(&Q->tree_b)].rec_base;
    const Mat4 M = query_mat(Q);
    // (ref, meta, surface, split) of the first tree's node
    auto a_leaf = [](float4 a) { return (__float_as_uint(a.y) & kLeafFlag) != 0u; };
    auto a_next = [&](float4 a) {
        return a_leaf(a) ? a : __ldg(recs + 4ull * (__float_as_uint(a.x) + (lp.y >= __float_as_uint(a.w))) + 3);
    };
    auto b_next = [&](const WalkRec& b) {
        return (b.meta & kLeafFlag) != 0u ? b : walk_rec(recs, b.ref + (lp.z >= b.split ? 1u : 0u));
    };
    float4 A = __ldg(recs + 4ull * (base_a + 1u) + 3);
    WalkRec B = walk_rec(recs, base_b + 1u);
    float4 An = a_next(A);
    WalkRec Bn = b_next(B);
    float sb = surface(xform_box(M, B.box));
    hi = lo = 0ull;
    depth = 0;
    for (;;) {
        const bool la = a_leaf(A), lb = (B.meta & kLeafFlag) != 0u;
        if ((la && lb) || depth > 128u) break;
        const bool split_a = (!la && !lb) ? (A.z >= sb) : !la;
        uint32_t bit;
        if (split_a) {
            bit = lp.y >= __float_as_uint(A.w) ? 1u : 0u;
            A = An;
            An = a_next(A);
        } else {
            bit = lp.z >= B.split ? 1u : 0u;
            B = Bn;
            Bn = b_next(B);
            sb = surface(xform_box(M, B.box));
        }
        hi = (hi << 1) | (lo >> 63);
        lo = (lo << 1) | bit;
        ++depth;
    }
    align_path(hi, lo, depth);
}

constexpr uint32_t kWayLevels = 64;  // levels of one tree's way a lane stages (deeper: descent_path)
constexpr uint32_t kPathWarps = 4;   // warps of a paths block

// descent_path for 16 leaf pairs per warp (all lanes call it; `valid`: this
// lane pair has leaf pair lp), with the two trees' ways down walked side by
// side: the way to a leaf is fixed by the leaf alone, so lane 2i follows the
// first tree to the pair's first leaf and lane 2i + 1 the second tree to its
// second leaf, both chains of dependent loads in flight together; each lane
// stages per level its node's surface (the second tree's box as transformed)
// in its row of `way` and keeps the child taken in `bits`. Lane 2i then
// merges the two ways by the reference's split rule into the path (its hi,
// lo, depth; the other lanes' are zero). A way of more than kWayLevels
// levels falls back to descent_path.
__device__ void paired_path(const PackedQuery* queries, const DevTree* trees, const float4* recs, uint4 lp, bool valid,
                            float (*way)[kWayLevels + 1], unsigned long long& hi, unsigned long long& lo,
                            uint32_t& depth) {
    const uint32_t lane = threadIdx.x & 31u;
    const bool second = (lane & 1u) != 0u;
    uint32_t d = 0;
    unsigned long long bits = 0ull;
    bool deep = false;
    if (valid) {
        const PackedQuery* Q = queries + lp.x;
        const uint32_t base = trees[second ? __ldg(&Q->tree_b) : __ldg(&Q->tree_a)].rec_base;
        const uint32_t target = second ? lp.z : lp.y;
        const Mat4 M = query_mat(Q);
        float* row = way[lane];
        uint32_t node = base + 1u;
        for (;;) {
            const WalkRec R = walk_rec(recs, node);
            if (R.meta & kLeafFlag) break;
            if (d == kWayLevels) {
                deep = true;
                break;
            }
            row[d] = second ? surface(xform_box(M, R.box)) : R.surf;
            const uint32_t bit = target >= R.split ? 1u : 0u;
            bits |= (unsigned long long)bit << d;
            node = R.ref + bit;
            ++d;
        }
    }
    __syncwarp();
    const uint32_t d2 = __shfl_down_sync(kFullMask, d, 1);
    const unsigned long long bits2 = __shfl_down_sync(kFullMask, bits, 1);
    const bool deep2 = __shfl_down_sync(kFullMask, deep ? 1u : 0u, 1) != 0u;
    hi = lo = 0ull;
    depth = 0u;
    if (second || !valid) return;
    if (deep || deep2) {
        descent_path(queries, trees, recs, lp, hi, lo, depth);
        return;
    }
    const float* SA = way[lane];
    const float* SB = way[lane + 1u];
    uint32_t i = 0, j = 0;
    while (i < d || j < d2) {
        const bool la = i == d, lb = j == d2;
        const bool split_a = (!la && !lb) ? (SA[i] >= SB[j]) : !la;
        const uint32_t bit = split_a ? uint32_t(bits >> i) & 1u : uint32_t(bits2 >> j) & 1u;
        hi = (hi << 1) | (lo >> 63);
        lo = (lo << 1) | bit;
        if (split_a)
            ++i;
        else
            ++j;
        ++depth;
    }
    align_path(hi, lo, depth);
}

// Ascending bitonic sort of n2 (a power of two) entries by the whole block.
template <class K, class Less>
__device__ void bitonic(K* a, uint32_t n2, Less less) {
    for (uint32_t k = 2; k <= n2; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < n2; i += blockDim.x) {
                const uint32_t l = i ^ j;
                if (l > i) {
                    const K x = a[i], y = a[l];
                    const bool swap = (i & k) == 0u ? less(y, x) : less(x, y);
                    if (swap) {
                        a[i] = y;
                        a[l] = x;
                    }
                }
            }
            __syncthreads();
        }
}

struct SortKey {
    unsigned long long hi, lo;
    uint32_t tri, idx;
};

// Insertion-order keys held in registers, each the narrowest exact form of
// (first leaf pair's path, triangle) with the element index as payload: K1
// when every path of the map has at most 32 splits (path's top 32 bits <<
// 32 | triangle), K2 at most 64 (path's high word, triangle << 32 |
// element), K3 any (high word, low word, triangle << 32 | element).
struct K1 {
    unsigned long long k;
    uint32_t idx;
    __device__ __forceinline__ static bool less(const K1& a, const K1& b) { return a.k < b.k; }
    __device__ __forceinline__ K1 xor_lane(uint32_t j) const {
        return K1{__shfl_xor_sync(kFullMask, k, j), __shfl_xor_sync(kFullMask, idx, j)};
    }
    __device__ __forceinline__ static K1 make(unsigned long long hi, unsigned long long, uint32_t tri, uint32_t i) {
        return K1{(hi & 0xffffffff00000000ull) | tri, i};
    }
    __device__ __forceinline__ static K1 pad() { return K1{~0ull, ~0u}; }
    __device__ __forceinline__ uint32_t tri() const { return uint32_t(k); }
    __device__ __forceinline__ uint32_t elem() const { return idx; }
};
struct K2 {
    unsigned long long hi, ti;
    __device__ __forceinline__ static bool less(const K2& a, const K2& b) {
        return a.hi != b.hi ? a.hi < b.hi : a.ti < b.ti;
    }
    __device__ __forceinline__ K2 xor_lane(uint32_t j) const {
        return K2{__shfl_xor_sync(kFullMask, hi, j), __shfl_xor_sync(kFullMask, ti, j)};
    }
    __device__ __forceinline__ static K2 make(unsigned long long hi, unsigned long long, uint32_t tri, uint32_t i) {
        return K2{hi, (unsigned long long)tri << 32 | i};
    }
    __device__ __forceinline__ static K2 pad() { return K2{~0ull, ~0ull}; }
    __device__ __forceinline__ uint32_t tri() const { return uint32_t(ti >> 32); }
    __device__ __forceinline__ uint32_t elem() const { return uint32_t(ti); }
};
struct K3 {
    unsigned long long hi, lo, ti;
    __device__ __forceinline__ static bool less(const K3& a, const K3& b) {
        return a.hi != b.hi ? a.hi < b.hi : (a.lo != b.lo ? a.lo < b.lo : a.ti < b.ti);
    }
    __device__ __forceinline__ K3 xor_lane(uint32_t j) const {
        return K3{__shfl_xor_sync(kFullMask, hi, j), __shfl_xor_sync(kFullMask, lo, j),
                  __shfl_xor_sync(kFullMask, ti, j)};
    }
    __device__ __forceinline__ static K3 make(unsigned long long hi, unsigned long long lo, uint32_t tri, uint32_t i) {
        return K3{hi, lo, (unsigned long long)tri << 32 | i};
    }
    __device__ __forceinline__ static K3 pad() { return K3{~0ull, ~0ull, ~0ull}; }
    __device__ __forceinline__ uint32_t tri() const { return uint32_t(ti >> 32); }
    __device__ __forceinline__ uint32_t elem() const { return uint32_t(ti); }
};

// x becomes the smaller (keep_min) or the larger of x and y (keys are
// distinct but for the padding, whose order does not matter).
template <class K>
__device__ __forceinline__ void k_keep(K& x, const K& y, bool keep_min) {
    if (K::less(y, x) == keep_min) x = y;
}

constexpr uint32_t kSortThreads = 256;               // the order kernel's block
constexpr uint32_t kRegSortMax = 4u * kSortThreads;  // keys the block sorts in registers

// Ascending bitonic sort by the block (kSortThreads threads) of n2 keys (a
// power of two, 32 <= n2 <= E * kSortThreads, E = 1, 2 or 4); thread t holds
// keys t + 256 e: exchanges within a warp by shuffles, across warps through
// xchg (n2 keys of shared memory, two barriers), between a thread's own keys
// in registers.
template <class K, int E>
__device__ __forceinline__ void block_sort_regs(K (&x)[E], uint32_t n2, K* xchg) {
    const uint32_t t = threadIdx.x;
    const bool active = t < n2;  // warp-uniform: n2 is a multiple of 32
    for (uint32_t k = 2; k <= n2; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            if (j >= kSortThreads) {
                // a thread's own keys e and e ^ (j / 256); the lower one keeps
                // the minimum when ascending
                const uint32_t jj = j / kSortThreads;
#pragma unroll
                for (int e = 0; e < E; ++e)
#pragma unroll
                    for (int f = e + 1; f < E; ++f)
                        if (uint32_t(e ^ f) == jj) {
                            const bool asc = ((t + kSortThreads * uint32_t(e)) & k) == 0u;
                            const K lo = x[e], hi = x[f];
                            const bool sw = K::less(hi, lo) == asc;
                            x[e] = sw ? hi : lo;
                            x[f] = sw ? lo : hi;
                        }
            } else if (j >= 32u) {
                if (active) {
#pragma unroll
                    for (int e = 0; e < E; ++e) xchg[t + kSortThreads * e] = x[e];
                }
                __syncthreads();
                if (active) {
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                        const uint32_t i = t + kSortThreads * e;
                        k_keep(x[e], xchg[i ^ j], ((i & j) == 0u) == ((i & k) == 0u));
                    }
                }
                __syncthreads();
            } else if (active) {
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const uint32_t i = t + kSortThreads * e;
                    k_keep(x[e], x[e].xor_lane(j), ((i & j) == 0u) == ((i & k) == 0u));
                }
            }
        }
    }
}

// The insertion order of the map's n elements El (n2 = pow2 >= max(n, 32),
// n2 <= E * kSortThreads): keys from the elements' paths and triangles,
// sorted, then per insertion index its triangle and element.
template <class K, int E>
__device__ __forceinline__ void insertion_order(const ContactElem* El, uint32_t n, uint32_t n2, void* xchg,
                                                uint32_t* ins_tri, uint32_t* ins_elem) {
    const uint32_t t = threadIdx.x;
    K x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t i = t + kSortThreads * e;
        x[e] = i < n ? K::make(El[i].key_hi, El[i].key_lo, El[i].tri, i) : K::pad();
    }
    block_sort_regs<K, E>(x, n2, reinterpret_cast<K*>(xchg));
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t i = t + kSortThreads * e;
        if (i < n) {
            ins_tri[i] = x[e].tri();
            ins_elem[i] = x[e].elem();
        }
    }
}

__device__ __forceinline__ uint32_t pow2_ceil(uint32_t n) {
    uint32_t p = 1;
    while (p < n) p <<= 1;
    return p;
}

// Bucket count of the table while element n - 1 is inserted.
__device__ __forceinline__ uint32_t buckets_at(const ContactParams& P, uint32_t n) {
    uint32_t b = P.sched_buckets[0];
    for (uint32_t e = 1; e < P.n_sched && P.sched_start[e] < n; ++e) b = P.sched_buckets[e];
    return b;
}

// Working memory of the order kernel for a map of n triangles (words): per
// insertion index its triangle and element, per element its corner mask;
// then either the insertion sort's keys, or for the growth steps two orders
// (the table's, the next), each place's bucket, its place in the bucket's
// member list, the run starts, the member lists, and per bucket its first
// place and count (two sets: this step's and the next's) and member offset;
// the ray phase keeps the order and reuses the rest.
struct OrderLayout {
    uint32_t nr, n2, nb, words;
};
__device__ __forceinline__ OrderLayout order_layout(const ContactParams& P, uint32_t n) {
    OrderLayout L;
    L.nr = (n + 1u) & ~1u;
    L.n2 = pow2_ceil(n > 32u ? n : 32u);
    L.nb = buckets_at(P, n);
    const uint32_t sort_w = 6u * L.n2;
    const uint32_t epoch_w = 6u * L.nr + 5u * (L.nb + 1u);
    L.words = 3u * L.nr + (sort_w > epoch_w ? sort_w : epoch_w);
    return L;
}

}  // namespace

__global__ void __launch_bounds__(256) contacts_pairs_kernel(const ContactParams P) {
    const unsigned long long tid = blockIdx.x * 1ull * blockDim.x + threadIdx.x;
    const unsigned long long stride = 1ull * gridDim.x * blockDim.x;
    // the vertex set of the previous contacts launch
    const uint32_t nv = P.ctr->prev_vertices;
    for (unsigned long long j = tid; j < nv; j += stride) {
        const uint32_t s = P.vocc[j];
        P.vkeys[s] = kEmptyKey;
        P.vval[s] = ~0u;
    }
    const unsigned long long n = n_written_pairs(P);
    const unsigned long long warp0 = tid & ~31ull;  // warp-uniform loop: warp_append needs all lanes
    for (unsigned long long base = warp0; base < n; base += stride) {
        const unsigned long long i = base + (threadIdx.x & 31u);
        int ra = -2, rb = -2;  // -2: no slot wanted, else the insert's result
        uint32_t sa = 0, sb = 0, leaf = 0;
        bool new_leaf = false;
        if (i < n) {
            const PairGeom g = pair_geom(P, i);
            const Probe T = contact_table(P);
            const unsigned long long ka = make_key(0u, g.q, g.tri_a), kb = make_key(1u, g.q, g.tri_b);
            const uint32_t ha = T.home(ka), hb = T.home(kb);
            const unsigned long long ca = atomicCAS(T.at(ha), kEmptyKey, ka);
            const unsigned long long cb = atomicCAS(T.at(hb), kEmptyKey, kb);
            ra = finish_insert(T, ka, ca, ha, &sa);
            rb = finish_insert(T, kb, cb, hb, &sb);
            // a slot taken counts in its map whatever happens to the pair
            if (ra == 1) atomicAdd(P.map_cnt + 2u * g.q, 1u);
            if (rb == 1) atomicAdd(P.map_cnt + 2u * g.q + 1u, 1u);
            uint4 link = make_uint4(~0u, ~0u, 0u, 0u);
            if (ra < 0 || rb < 0) {
                atomicOr(&P.ctr->c_overflow, CONTACT_TABLE);
            } else {
                // a place in each slot's contribution list
                link = make_uint4(sa, sb, atomicAdd(&P.table[sa].count, 1u), atomicAdd(&P.table[sb].count, 1u));
                // the leaf pair has colliding pairs: its descent path is needed
                leaf = __ldg(&P.pair_aux[i].z);
                new_leaf = atomicCAS(P.leaf_mark + leaf, 0u, 1u) == 0u;
            }
            P.pg_geom[i] = make_float4(g.mid.x, g.mid.y, g.mid.z, g.w);
            P.pg_link[i] = link;
            P.pg_mask[i] = g.mask_a | (g.mask_b << 3);
        }
        __syncwarp();
        const unsigned new_a = ra == 1, new_b = rb == 1;
        const unsigned o = warp_append(&P.ctr->n_contacts, new_a + new_b);
        if (new_a) P.occupied[o] = sa;  // one entry per slot: the list never outgrows the table
        if (new_b) P.occupied[o + new_a] = sb;
        const unsigned k = warp_append(&P.ctr->n_kleaf, new_leaf ? 1u : 0u);
        if (new_leaf) {
            if (k < P.kleaf_cap) {
                P.kleaf[k] = leaf;
                P.leaf_mark[leaf] = 1u + k;
            } else {
                atomicOr(&P.ctr->c_overflow, CONTACT_TABLE);
            }
        }
    }
}

// Each slot's place in the contribution list (one atomic per warp of 32
// slots), the list of slots for the fold's warps, and, in the first block,
// the maps' element offsets.
__global__ void __launch_bounds__(256) contacts_alloc_kernel(const ContactParams P) {
    __shared__ uint32_t part[64];
    const uint32_t ns = n_slots(P);
    if (blockIdx.x == 0 && threadIdx.x == 0 && ns > P.max_contacts) atomicOr(&P.ctr->c_overflow, CONTACT_TABLE);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; j0 < ns; j0 += stride) {
        const uint32_t j = j0 + (threadIdx.x & 31u);
        ContactSlot* sl = j < ns ? P.table + P.occupied[j] : nullptr;
        const ContactSlot v = sl ? *sl : ContactSlot{kEmptyKey, 0u, 0u};
        const uint32_t off = warp_append(&P.ctr->contrib_used, v.count);
        const unsigned big = v.count > kFoldThread ? 1u : 0u;
        const uint32_t bi = warp_append(&P.ctr->n_big, big);
        if (sl) {
            sl->offset = off;
            P.slot_info[j] = make_uint4(uint32_t(v.key), uint32_t(v.key >> 32), off, v.count);
        }
        if (big) P.big_slots[bi] = j;  // at most one entry per slot: the list never outgrows the table
    }
    if (blockIdx.x == 0)
        block_scan(
            2u * P.n_queries, part, [&](uint32_t i) { return P.map_cnt[i]; },
            [&](uint32_t i, uint32_t v) { P.map_off[i] = v; });
}

// Both contributions of every pair into their slots' lists.
__global__ void __launch_bounds__(256) contacts_scatter_kernel(const ContactParams P) {
    const unsigned long long n = n_written_pairs(P);
    for (unsigned long long i = blockIdx.x * 1ull * blockDim.x + threadIdx.x; i < n;
         i += 1ull * gridDim.x * blockDim.x) {
        const uint4 link = P.pg_link[i];
        if (link.x == ~0u) continue;
        const uint4 aux = P.pair_aux[i];
        const unsigned long long c = (unsigned long long)i << 1;
        P.contrib[P.table[link.x].offset + link.z] = ((unsigned long long)aux.y << 32) | c;
        P.contrib[P.table[link.y].offset + link.w] = ((unsigned long long)aux.x << 32) | c | 1ull;
    }
}

// The descent path of every listed leaf pair (those with colliding pairs).
__global__ void __launch_bounds__(kPathWarps * 32) contacts_paths_kernel(const ContactParams P) {
    __shared__ float way[kPathWarps][32][kWayLevels + 1];
    const uint32_t nk = min(*reinterpret_cast<const volatile unsigned*>(&P.ctr->n_kleaf), P.kleaf_cap);
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    for (uint32_t b = (blockIdx.x * kPathWarps + wib) * 16u; b < nk; b += gridDim.x * kPathWarps * 16u) {
        const uint32_t j = b + (lane >> 1);
        const bool valid = j < nk;
        const uint4 lp = valid ? P.leaf_list[P.kleaf[j]] : make_uint4(0u, 0u, 0u, 0u);
        unsigned long long hi, lo;
        uint32_t depth;
        paired_path(P.q, P.trees, P.recs, lp, valid, way[wib], hi, lo, depth);
        if (!(lane & 1u) && valid) {
            if (depth >= 128u) atomicOr(&P.ctr->c_overflow, CONTACT_ORDER);
            P.kpath[j] = make_ulonglong2(hi, lo);
        }
        __syncwarp();  // the rows are the next round's
    }
}

// The reference's two folds over one triangle's colliding pairs in the
// order of the other triangle (CreateUncollideRays.cpp:79-100, 117-127): a
// fold per leaf pair from zero, merged in leaf-pair order when its weight is
// not zero; the first leaf pair merged is kept for the insertion order.
struct TriFold {
    bool have = false;
    float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
    unsigned am = 7u;
    uint32_t first_leaf = 0u, cur = ~0u;
    float px = 0.f, py = 0.f, pz = 0.f, pw = 0.f;
    unsigned pm = 7u;
    __device__ __forceinline__ void close() {
        if (pw == 0.0f) return;
        if (!have) {
            have = true;
            first_leaf = cur;
            ax = px, ay = py, az = pz, aw = pw;
            am = pm;
        } else {
            am &= pm;
            ax = ax + px;
            ay = ay + py;
            az = az + pz;
            aw = aw + pw;
        }
    }
    __device__ __forceinline__ void add(uint32_t leaf, float4 g, unsigned mk) {
        if (leaf != cur) {
            if (cur != ~0u) close();
            cur = leaf;
            px = py = pz = pw = 0.0f;
            pm = 7u;
        }
        px = px + g.x;
        py = py + g.y;
        pz = pz + g.z;
        pw = pw + g.w;
        pm &= mk;
    }
    __device__ __forceinline__ void finish() {
        if (cur != ~0u) close();
    }
};

// The triangle of slot key `key` into its map, with the path of its first
// leaf pair of non-zero weight; nothing when every pair had zero length
// (IsNull).
__device__ __forceinline__ void put_elem(const ContactParams& P, unsigned long long key, const TriFold& F) {
    if (!F.have) return;
    const uint32_t side = uint32_t(key >> 63);
    const uint32_t q = uint32_t(key >> 32) & 0x7fffffffu;
    const uint32_t mark = P.leaf_mark[F.first_leaf];
    const ulonglong2 path =
        mark > 0u && mark - 1u < P.kleaf_cap ? P.kpath[mark - 1u] : make_ulonglong2(~0ull, ~0ull);
    ContactElem E;
    E.key_hi = path.x;
    E.key_lo = path.y;
    E.depth = 0u;
    E.sx = F.ax;
    E.sy = F.ay;
    E.sz = F.az;
    E.w = F.aw;
    E.tri = uint32_t(key);
    E.mask = F.am;
    E.pad = 0u;
    const uint32_t map = 2u * q + side;
    const uint32_t idx = P.map_off[map] + atomicAdd(P.map_fill + map, 1u);
    if (idx < P.max_contacts) P.elems[idx] = E;
}

// One slot of at most kFoldThread contributions by its own thread: the
// contributions sorted in registers, their pairs' data loaded together, the
// folds.
__device__ __forceinline__ void fold_thread(const ContactParams& P, unsigned long long key, uint32_t off, uint32_t c,
                                            TriFold& F) {
    const uint32_t side = uint32_t(key >> 63);
    unsigned long long v[kFoldThread];
#pragma unroll
    for (uint32_t a = 0; a < kFoldThread; ++a) v[a] = a < c ? P.contrib[off + a] : ~0ull;
    if (c > 1u) {
        // odd-even transposition sort: kFoldThread rounds sort kFoldThread values
#pragma unroll
        for (uint32_t r = 0; r < kFoldThread; ++r)
#pragma unroll
            for (uint32_t a = r & 1u; a + 1u < kFoldThread; a += 2u) {
                const unsigned long long x = v[a], y = v[a + 1u];
                v[a] = x < y ? x : y;
                v[a + 1u] = x < y ? y : x;
            }
    }
    uint32_t leaf[kFoldThread];
    float4 g[kFoldThread];
    unsigned mk[kFoldThread];
#pragma unroll
    for (uint32_t a = 0; a < kFoldThread; ++a) {
        if (a < c) {
            const uint32_t pid = uint32_t(v[a]) >> 1;
            leaf[a] = __ldg(&P.pair_aux[pid].z);
            g[a] = __ldg(P.pg_geom + pid);
            mk[a] = (__ldg(P.pg_mask + pid) >> (3u * side)) & 7u;
        }
    }
#pragma unroll
    for (uint32_t a = 0; a < kFoldThread; ++a)
        if (a < c) F.add(leaf[a], g[a], mk[a]);
    F.finish();
}

// A contribution's pair data staged for the folding lane.
struct FoldItem {
    float4 g;
    uint32_t leaf, mk;
};

// Ascending bitonic sort by one warp of n2 (32, 64 or 128) values, four per
// lane (value i = lane + 32 r in v[r]): between a lane's own values in
// registers, within a row by shuffles.
__device__ __forceinline__ void warp_sort128(unsigned long long (&v)[4], uint32_t n2) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t k = 2; k <= n2; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32u) {
                const uint32_t jj = j >> 5;
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int f = r + 1; f < 4; ++f)
                        if (uint32_t(r ^ f) == jj) {
                            const bool asc = ((lane + 32u * uint32_t(r)) & k) == 0u;
                            const unsigned long long lo = v[r], hi = v[f];
                            const bool sw = (hi < lo) == asc;
                            v[r] = sw ? hi : lo;
                            v[f] = sw ? lo : hi;
                        }
            } else {
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    if (32u * uint32_t(r) < n2) {
                        const uint32_t i = lane + 32u * uint32_t(r);
                        const unsigned long long o = __shfl_xor_sync(kFullMask, v[r], j);
                        const bool keep_min = ((i & j) == 0u) == ((i & k) == 0u);
                        v[r] = keep_min ? (o < v[r] ? o : v[r]) : (o > v[r] ? o : v[r]);
                    }
                }
            }
        }
}

constexpr uint32_t kFoldStage = 128;  // contributions a fold warp sorts in registers and stages at once
constexpr uint32_t kFoldSort = kFoldStage * sizeof(FoldItem) / sizeof(unsigned long long);  // ... sorts in its staging buffer

// Ascending sort of a[0..c-1] by one warp (all lanes call it): a bitonic
// network whose comparators all put the smaller value first (the first step
// of each merge compares mirrored places), so that the places past c, the
// network's padding, are +infinity that never moves: a comparison with a
// place past c is skipped. __syncwarp orders the lanes' accesses between
// steps (shared or global memory).
__device__ void warp_sort_any(unsigned long long* a, uint32_t c) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t n2 = 1;
    while (n2 < c) n2 <<= 1;
    auto cmpx = [&](uint32_t i, uint32_t l) {
        if (l < c) {
            const unsigned long long x = a[i], y = a[l];
            if (y < x) {
                a[i] = y;
                a[l] = x;
            }
        }
    };
    for (uint32_t k = 2; k <= n2; k <<= 1) {
        const uint32_t h = k >> 1;
#pragma unroll 4
        for (uint32_t t = lane; t < (n2 >> 1); t += 32u) {
            const uint32_t base = (t / h) * k, off = t % h;
            cmpx(base + off, base + k - 1u - off);
        }
        __syncwarp();
        for (uint32_t j = k >> 2; j > 0; j >>= 1) {
#pragma unroll 4
            for (uint32_t t = lane; t < (n2 >> 1); t += 32u) {
                const uint32_t i = (t / j) * 2u * j + t % j;
                cmpx(i, i + j);
            }
            __syncwarp();
        }
    }
}

// One slot of more than kFoldThread contributions by the whole warp (all
// lanes call it): sorted in registers (<= kFoldStage), in the warp's staging
// buffer (<= kFoldSort) or in place in global memory; kFoldStage at a time,
// every lane stages its contributions' pair data in `stage` (all loads in
// flight together) and lane 0 folds them in order (F is lane 0's).
__device__ void fold_warp(const ContactParams& P, unsigned long long key, uint32_t off, uint32_t c,
                          FoldItem* stage, TriFold& F) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t side = uint32_t(key >> 63);
    unsigned long long v[4];
    const unsigned long long* S = nullptr;
    if (c <= kFoldStage) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t i = lane + 32u * uint32_t(r);
            v[r] = i < c ? P.contrib[off + i] : ~0ull;
        }
        warp_sort128(v, c <= 32u ? 32u : (c <= 64u ? 64u : 128u));
    } else {
        unsigned long long* G = P.contrib + off;
        if (c <= kFoldSort) {
            unsigned long long* sh = reinterpret_cast<unsigned long long*>(stage);
            for (uint32_t i = lane; i < c; i += 32u) sh[i] = G[i];
            __syncwarp();
            warp_sort_any(sh, c);
            for (uint32_t i = lane; i < c; i += 32u) G[i] = sh[i];
        } else {
            warp_sort_any(G, c);
        }
        __syncwarp();
        S = G;
    }
    for (uint32_t a0 = 0; a0 < c; a0 += kFoldStage) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t a = a0 + lane + 32u * uint32_t(r);
            if (a < c) {
                const unsigned long long x = S ? S[a] : v[r];
                const uint32_t pid = uint32_t(x) >> 1;
                FoldItem it;
                it.leaf = __ldg(&P.pair_aux[pid].z);
                it.g = __ldg(P.pg_geom + pid);
                it.mk = (__ldg(P.pg_mask + pid) >> (3u * side)) & 7u;
                stage[a - a0] = it;
            }
        }
        __syncwarp();
        if (lane == 0) {
            const uint32_t m = c - a0 < kFoldStage ? c - a0 : kFoldStage;
            for (uint32_t k = 0; k < m; ++k) F.add(stage[k].leaf, stage[k].g, stage[k].mk);
        }
        __syncwarp();
    }
    if (lane == 0) F.finish();
}

// The maps, largest first (by size class: the bit length of the triangle
// count), for the order kernel's blocks to take in that order; by one block.
__device__ void rank_maps(const ContactParams& P) {
    __shared__ uint32_t count[33], start[33];
    const uint32_t m = 2u * P.n_queries;
    if (threadIdx.x < 33u) count[threadIdx.x] = 0u;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const uint32_t n = P.map_fill[i];
        atomicAdd(count + (n ? 32u - __clz(n) : 0u), 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t off = 0;
        for (int c = 32; c >= 0; --c) {
            start[c] = off;
            off += count[c];
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const uint32_t n = P.map_fill[i];
        P.map_order[atomicAdd(start + (n ? 32u - __clz(n) : 0u), 1u)] = i;
    }
}

// Each map's first record and ray in the outputs, the counts; by one block.
__device__ void place_maps(const ContactParams& P, uint32_t* part) {
    const uint32_t m = 2u * P.n_queries;
    const uint32_t nc = block_scan(
        m, part, [&](uint32_t i) { return P.map_fill[i]; }, [&](uint32_t i, uint32_t v) { P.map_coff[i] = v; });
    const uint32_t nr = block_scan(
        m, part, [&](uint32_t i) { return P.map_nr[i]; }, [&](uint32_t i, uint32_t v) { P.map_roff[i] = v; });
    if (threadIdx.x == 0) {
        P.ctr->n_elems = nc;
        P.ctr->n_rays = nr;
        P.ctr->prev_vertices = 0u;  // the pairs kernel emptied them
    }
}

// True in the block that finishes last of the grid (counted on `done`); its
// threads then see every other block's writes.
__device__ bool last_block(unsigned* done) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1u;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// A thread per slot: the triangle's contributions sorted by the other
// triangle (a triangle's pairs within a leaf pair come in the other
// triangle's order, and its leaf pairs in the order of the other leaf's first
// triangle), the reference's folds in that order, the path of the first leaf
// pair of non-zero weight; the triangle into its map. A slot of more than
// kFoldThread contributions is folded by a warp of its own, the listed slots
// taken from the grid's last warp down (one resident wave: those warps have
// few or no slots of their own).
constexpr uint32_t kFoldWarps = 8;

__global__ void __launch_bounds__(256, 3) contacts_fold_kernel(const ContactParams P) {
    __shared__ FoldItem stage[kFoldWarps][kFoldStage];
    const uint32_t ns = n_slots(P);
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; j0 < ns; j0 += stride) {
        const uint32_t j = j0 + lane;
        const uint4 si = j < ns ? P.slot_info[j] : make_uint4(0u, 0u, 0u, 0u);
        const unsigned long long key = (unsigned long long)si.y << 32 | si.x;
        if (si.w <= kFoldThread) {
            TriFold F;
            fold_thread(P, key, si.z, si.w, F);
            put_elem(P, key, F);
        }
    }
    const uint32_t n_warps = gridDim.x * kFoldWarps;
    const uint32_t gw = blockIdx.x * kFoldWarps + wib;
    const uint32_t nb = *reinterpret_cast<const volatile unsigned*>(&P.ctr->n_big);
    for (uint32_t b = n_warps - 1u - gw; b < nb; b += n_warps) {
        const uint4 si = P.slot_info[P.big_slots[b]];
        const unsigned long long key = (unsigned long long)si.y << 32 | si.x;
        TriFold F;
        fold_warp(P, key, si.z, si.w, stage[wib], F);
        if (lane == 0) put_elem(P, key, F);
    }
    if (last_block(&P.ctr->fold_done)) rank_maps(P);
}

// A ray of find_rays_lambda (CreateUncollideRays.cpp:140-173) for contact
// element E of (query, side): the vertex ray of corner k, or (k < 0) the ray
// from the weighted average with the barycentric-interpolated normal.
__device__ cg_ray contact_ray(const ContactParams& P, uint32_t q, uint32_t side, const ContactElem& E, int k) {
    const PackedQuery* Q = P.q + q;
    const float* nrm = P.trees[side ? __ldg(&Q->tree_b) : __ldg(&Q->tree_a)].nrm;
    const Mat4 M = query_mat(Q);
    float3 p[3], n3[3];
    uint32_t vi[3];
    tri_at(P.tris, (side ? __ldg(&Q->tri_base_b) : __ldg(&Q->tri_base_a)) + E.tri, p, vi);
    if (nrm) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* np = nrm + 9ull * E.tri + 3 * c;
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
    float3 o, d;
    if (k >= 0) {
        // TriangleNormal::GetNormal(index[, corrected_matrix]) (Triangle.cpp:180-195)
        const float3 nk = k == 0 ? n3[0] : (k == 1 ? n3[1] : n3[2]);
        d = neg3(side ? normalize3(mul3(N, nk)) : normalize3(nk));
        o = k == 0 ? p[0] : (k == 1 ? p[1] : p[2]);
    } else {
        // TriangleCandidateRays::GetWeightedAvg, TrianglePosition::GetBarycentricOfPoint
        // (Triangle.cpp:148-163), TriangleNormal::GetNormal(bary[, corrected_matrix]) (:197-212)
        const float3 avg = divs3(make_float3(E.sx, E.sy, E.sz), E.w);
        const float3 v0 = sub3(p[1], p[0]), v1 = sub3(p[2], p[0]), v2 = sub3(avg, p[0]);
        const float d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1);
        const float d20 = dot3(v2, v0), d21 = dot3(v2, v1);
        const float den = d00 * d11 - d01 * d01;
        const float bx = (d11 * d20 - d01 * d21) / den;
        const float by = (d00 * d21 - d01 * d20) / den;
        const float b0 = 1.f - bx - by;
        const float3 in = add3(add3(scale3(b0, n3[0]), scale3(bx, n3[1])), scale3(by, n3[2]));
        d = neg3(side ? normalize3(mul3(N, in)) : normalize3(in));
        o = avg;
    }
    cg_ray r;
    r.query = q;
    r.side = side;
    r.origin[0] = o.x;
    r.origin[1] = o.y;
    r.origin[2] = o.z;
    r.direction[0] = d.x;
    r.direction[1] = d.y;
    r.direction[2] = d.z;
    return r;
}

// The vertex set of one map (CreateUncollideRays.cpp:148-161, the
// emplaced_point_indices set): each vertex index of a corner that may make a
// ray, with the place code (place * 4 + corner) of its first such corner in
// iteration order. In shared memory (keys: vertex indices, ~0u empty; `mask`
// + 1 slots, a power of two, hashed by the top bits of a multiplicative
// hash) when `keys` is set, else the launch's global set keyed by (side,
// query, vertex index).
struct VSet {
    uint32_t* keys;
    uint32_t* vals;
    uint32_t mask, shift;
};

__device__ __forceinline__ int smem_insert(const VSet& V, uint32_t key, uint32_t* slot) {
    uint32_t s = (key * 0x9E3779B1u) >> V.shift;
    for (uint32_t probe = 0; probe <= V.mask; ++probe) {
        const uint32_t cur = atomicCAS(V.keys + s, ~0u, key);
        if (cur == ~0u || cur == key) {
            *slot = s;
            return cur == ~0u ? 1 : 0;
        }
        s = (s + 1u) & V.mask;
    }
    return -1;
}

// The corners of a contact element (mask bits, vertex indices vi) whose
// vertex ray this map makes (bit k): a corner whose bit is set makes the ray
// of its vertex index when it is that index's first corner in iteration
// order; an earlier corner of the same triangle with the same index makes it
// instead. kRecord: record this element's codes first (place `pos`).
template <bool kRecord>
__device__ unsigned vertex_corners(const ContactParams& P, const VSet& V, uint32_t q, uint32_t side, uint32_t mask,
                                   const uint32_t vi[3], uint32_t pos) {
    unsigned out = 0u;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (!((mask >> k) & 1u)) continue;
        bool dup = false;
#pragma unroll
        for (int j = 0; j < k; ++j) dup |= ((mask >> j) & 1u) && vi[j] == vi[k];
        if (dup) continue;
        uint32_t slot = 0;
        uint32_t* val;
        int r;
        if (V.keys) {
            r = smem_insert(V, vi[k], &slot);
            val = V.vals + slot;
        } else {
            r = insert(Probe{P.vkeys, 1u, P.vtable_mask}, make_key(side, q, vi[k]), &slot);
            val = P.vval + slot;
            if (kRecord && r == 1) P.vocc[atomicAdd(&P.ctr->n_vertices, 1u)] = slot;
        }
        if (r < 0) {
            atomicOr(&P.ctr->c_overflow, CONTACT_VERTICES);
            continue;
        }
        const uint32_t code = pos * 4u + uint32_t(k);
        if (kRecord)
            atomicMin(val, code);
        else if ((V.keys ? *val : atomicOr(val, 0u)) == code)
            out |= 1u << k;
    }
    return out;
}

// Keys in the table at the end of growth step e of a map of n keys.
__device__ __forceinline__ uint32_t step_end(const ContactParams& P, uint32_t e, uint32_t n) {
    return (e + 1u < P.n_sched && P.sched_start[e + 1u] < n) ? P.sched_start[e + 1u] : n;
}

// The growth steps of a map of n keys that end with at most 32 keys.
__device__ __forceinline__ uint32_t warp_step_count(const ContactParams& P, uint32_t n) {
    uint32_t e = 0;
    while (e < P.n_sched && P.sched_start[e] < n && step_end(P, e, n) <= 32u) ++e;
    return e;
}

// Growth steps 0..steps-1 (at most 32 keys each) by one warp, a key per
// lane: a bucket's keys are the lanes that match its index, its first place
// the lowest of them; a key goes after the keys of the buckets whose first
// place is later and after the later keys of its own bucket.
__device__ void warp_steps(const ContactParams& P, uint32_t n, uint32_t steps, const uint32_t* ins_tri,
                           uint32_t* ord) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t e = 0; e < steps; ++e) {
        const uint32_t st = P.sched_start[e];
        const uint32_t m = step_end(P, e, n);
        const uint32_t nb = P.sched_buckets[e];
        const uint32_t x = lane < m ? (lane < st ? ord[lane] : lane) : ~0u;
        const uint32_t b = lane < m ? ins_tri[x] % nb : ~0u;
        const unsigned same = __match_any_sync(kFullMask, b);
        const uint32_t first = uint32_t(__ffs(same)) - 1u;
        const uint32_t c = lane < m && lane == first ? uint32_t(__popc(same)) : 0u;
        uint32_t after = c;  // keys of the buckets first placed at this lane or later
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_down_sync(kFullMask, after, o);
            if (lane + uint32_t(o) < 32u) after += v;
        }
        after -= c;
        const uint32_t before_bucket = __shfl_sync(kFullMask, after, first);
        const uint32_t later = lane < 31u ? uint32_t(__popc(same >> (lane + 1u))) : 0u;
        __syncwarp();
        if (lane < m) ord[before_bucket + later] = x;
        __syncwarp();
    }
}

// One map (query, side) by the whole block: its triangles in the reference's
// iteration order, their contact records and rays in that order, and the
// map's mean ray origin.
__device__ void order_map(const ContactParams& P, uint32_t map, uint32_t* smem, uint32_t* part, float* fold) {
    const uint32_t q = map >> 1, side = map & 1u;
    const uint32_t n = P.map_fill[map];
    const uint32_t base = P.map_off[map];
    const uint32_t T = blockDim.x, t = threadIdx.x;
    uint32_t n_rays = 0;
    bool ok = n > 0u && base + n <= P.max_contacts;
    OrderLayout L{};
    uint32_t* W = smem;
    VSet V{nullptr, nullptr, 0u, 0u};
    if (ok) {
        L = order_layout(P, n);
        // the vertex set: at most 3 n keys, at most three quarters full
        const uint32_t hs = pow2_ceil(4u * n);
        uint32_t used = L.words;
        if (L.words + 2u * hs > kOrderSmemWords) {
            // this map's part of the global working memory: kOrderWords per
            // element from its first element (base + n <= max_contacts)
            W = P.work + size_t(kOrderWords) * base;
            ok = L.words <= kOrderWords * n;
            if (!ok && t == 0u) atomicOr(&P.ctr->c_overflow, CONTACT_ORDER);
            used = 0u;
        }
        if (used + 2u * hs <= kOrderSmemWords) {
            V.keys = smem + used;
            V.vals = V.keys + hs;
            V.mask = hs - 1u;
            V.shift = 33u - uint32_t(__ffs(hs));
            for (uint32_t i = t; i < hs; i += T) {
                V.keys[i] = ~0u;
                V.vals[i] = ~0u;
            }
        }
    }
    cg_ray* R = P.rtmp + 3ull * base;
    if (ok) {
        const ContactElem* El = P.elems + base;
        const PackedQuery* Q = P.q + q;
        const uint32_t tri_base = side ? __ldg(&Q->tri_base_b) : __ldg(&Q->tri_base_a);
        uint32_t* ins_tri = W;
        uint32_t* ins_elem = W + L.nr;
        uint32_t* mask_of = W + 2u * L.nr;
        uint32_t* B0 = W + 3u * L.nr;
        // 1. insertion order: the first leaf pair's path, then the triangle
        if (L.n2 <= kRegSortMax) {
            bool wide = false, mid = false;  // a path with low-word bits; with bits in the high word's low half
            for (uint32_t i = t; i < n; i += T) {
                const ContactElem& E = El[i];
                mask_of[i] = E.mask;
                wide |= E.key_lo != 0ull;
                mid |= (E.key_hi & 0xffffffffull) != 0ull;
            }
            wide = __syncthreads_or(wide) != 0;
            mid = __syncthreads_or(mid) != 0;
            const uint32_t E = L.n2 <= kSortThreads ? 1u : (L.n2 <= 2u * kSortThreads ? 2u : 4u);
            if (!wide && !mid) {
                if (E == 1u) insertion_order<K1, 1>(El, n, L.n2, B0, ins_tri, ins_elem);
                else if (E == 2u) insertion_order<K1, 2>(El, n, L.n2, B0, ins_tri, ins_elem);
                else insertion_order<K1, 4>(El, n, L.n2, B0, ins_tri, ins_elem);
            } else if (!wide) {
                if (E == 1u) insertion_order<K2, 1>(El, n, L.n2, B0, ins_tri, ins_elem);
                else if (E == 2u) insertion_order<K2, 2>(El, n, L.n2, B0, ins_tri, ins_elem);
                else insertion_order<K2, 4>(El, n, L.n2, B0, ins_tri, ins_elem);
            } else {
                if (E == 1u) insertion_order<K3, 1>(El, n, L.n2, B0, ins_tri, ins_elem);
                else if (E == 2u) insertion_order<K3, 2>(El, n, L.n2, B0, ins_tri, ins_elem);
                else insertion_order<K3, 4>(El, n, L.n2, B0, ins_tri, ins_elem);
            }
        } else {
            SortKey* sk = reinterpret_cast<SortKey*>(B0);
            for (uint32_t i = t; i < L.n2; i += T) {
                SortKey k;
                if (i < n) {
                    const ContactElem& E = El[i];
                    k.hi = E.key_hi;
                    k.lo = E.key_lo;
                    k.tri = E.tri;
                    k.idx = i;
                    mask_of[i] = E.mask;
                } else {
                    k.hi = k.lo = ~0ull;
                    k.tri = k.idx = ~0u;
                }
                sk[i] = k;
            }
            __syncthreads();
            bitonic(sk, L.n2, [](const SortKey& a, const SortKey& b) {
                return a.hi != b.hi ? a.hi < b.hi : (a.lo != b.lo ? a.lo < b.lo : a.tri < b.tri);
            });
            for (uint32_t i = t; i < n; i += T) {
                ins_tri[i] = sk[i].tri;
                ins_elem[i] = sk[i].idx;
            }
        }
        __syncthreads();
        // 2. the table's order (insertion indices) after each growth: its
        // buckets in the order of their first place, latest first, each
        // bucket's keys latest first, where a growth places the table's keys
        // in the order it held them and then the new keys in insertion order
        uint32_t* ord = B0;
        uint32_t* nord = B0 + L.nr;
        uint32_t* bs = B0 + 2u * L.nr;    // per place: its bucket
        uint32_t* kb = B0 + 3u * L.nr;    // per place: its place in the bucket's member list
        uint32_t* run = B0 + 4u * L.nr;   // per place: keys of the buckets first placed later
        uint32_t* mem = B0 + 5u * L.nr;   // the buckets' member lists (places)
        uint32_t* first = B0 + 6u * L.nr;
        uint32_t* cnt = first + L.nb + 1u;
        uint32_t* first2 = cnt + L.nb + 1u;
        uint32_t* cnt2 = first2 + L.nb + 1u;
        uint32_t* boff = cnt2 + L.nb + 1u;
        // the steps of up to 32 keys by warp 0, meanwhile the first larger
        // step's buckets start empty
        uint32_t e = warp_step_count(P, n);
        if (t < 32u && e > 0u) warp_steps(P, n, e, ins_tri, ord);
        const uint32_t nb0 = e < P.n_sched && P.sched_start[e] < n ? P.sched_buckets[e] : 0u;
        for (uint32_t b = t; b < nb0; b += T) {
            first[b] = ~0u;
            cnt[b] = 0u;
        }
        __syncthreads();
        for (; e < P.n_sched && P.sched_start[e] < n; ++e) {
            const uint32_t st = P.sched_start[e];  // keys in the table when it grows
            const uint32_t m = step_end(P, e, n);
            const uint32_t nb = P.sched_buckets[e];
            for (uint32_t s = t; s < m; s += T) {
                const uint32_t x = s < st ? ord[s] : s;
                const uint32_t b = ins_tri[x] % nb;
                bs[s] = b;
                kb[s] = atomicAdd(cnt + b, 1u);
                atomicMin(first + b, s);
            }
            __syncthreads();
            // the member lists' offsets, and the run starts (the keys of the
            // buckets whose first place is later)
            uint32_t total = 0, none = 0;
            block_scan2(
                nb, m, part, [&](uint32_t b) { return cnt[b]; }, [&](uint32_t b, uint32_t v) { boff[b] = v; },
                [&](uint32_t i) {
                    const uint32_t s = m - 1u - i, b = bs[s];
                    return first[b] == s ? cnt[b] : 0u;
                },
                [&](uint32_t i, uint32_t v) { run[m - 1u - i] = v; }, total, none);
            for (uint32_t s = t; s < m; s += T) mem[boff[bs[s]] + kb[s]] = s;
            if (t == 0u) boff[nb] = total;
            __syncthreads();
            // the next step's buckets start empty
            const bool more = e + 1u < P.n_sched && P.sched_start[e + 1u] < n;
            const uint32_t nb2 = more ? P.sched_buckets[e + 1u] : 0u;
            for (uint32_t b = t; b < nb2; b += T) {
                first2[b] = ~0u;
                cnt2[b] = 0u;
            }
            for (uint32_t s = t; s < m; s += T) {
                const uint32_t b = bs[s];
                uint32_t later = 0;
                for (uint32_t k = boff[b]; k < boff[b + 1u]; ++k) later += mem[k] > s ? 1u : 0u;
                nord[run[first[b]] + later] = s < st ? ord[s] : s;
            }
            __syncthreads();
            uint32_t* sw = ord;
            ord = nord;
            nord = sw;
            sw = first;
            first = first2;
            first2 = sw;
            sw = cnt;
            cnt = cnt2;
            cnt2 = sw;
        }
        // 3. rays: the vertex set keeps each vertex index's first corner. Per
        // place: mask then vertex-ray corners (rb), rays (rc), its corners'
        // vertex indices (vi0..2); the order stays where the last step left it
        uint32_t* rb = B0 + 2u * L.nr;
        uint32_t* rc = B0 + 3u * L.nr;
        uint32_t* vi0 = B0 + 4u * L.nr;
        uint32_t* vi1 = B0 + 5u * L.nr;
        uint32_t* vi2 = B0 + 6u * L.nr;
        for (uint32_t p = t; p < n; p += T) {
            const uint32_t x = ord[p];
            const uint32_t mask = mask_of[ins_elem[x]];
            uint32_t vi[3] = {0u, 0u, 0u};
            if (mask) {
                const float4* tv = P.tris + 3ull * (tri_base + ins_tri[x]);
#pragma unroll
                for (int k = 0; k < 3; ++k) vi[k] = __float_as_uint(__ldg(&tv[k].w));
                vertex_corners<true>(P, V, q, side, mask, vi, p);
            }
            rb[p] = mask;
            vi0[p] = vi[0];
            vi1[p] = vi[1];
            vi2[p] = vi[2];
        }
        __syncthreads();
        for (uint32_t p = t; p < n; p += T) {
            const uint32_t mask = rb[p];
            const uint32_t vi[3] = {vi0[p], vi1[p], vi2[p]};
            const unsigned bits = mask ? vertex_corners<false>(P, V, q, side, mask, vi, p) : 0u;
            rb[p] = bits;
            rc[p] = mask ? __popc(bits) : 1u;
        }
        __syncthreads();
        n_rays = block_scan(
            n, part, [&](uint32_t i) { return rc[i]; }, [&](uint32_t i, uint32_t v) { rc[i] = v; });
        // a thread per ray: its place is the last one whose first ray is at
        // or before it (a place without rays shares its first ray with the
        // next place)
        for (uint32_t r = t; r < n_rays; r += T) {
            uint32_t a = 0, b = n - 1u;
            while (a < b) {
                const uint32_t mid = (a + b + 1u) >> 1;
                if (rc[mid] <= r)
                    a = mid;
                else
                    b = mid - 1u;
            }
            const ContactElem& E = El[ins_elem[ord[a]]];
            int corner = -1;
            if (E.mask) {
                uint32_t left = r - rc[a];  // the ray's rank among the place's vertex rays
                const uint32_t bits = rb[a];
                for (int k = 0; k < 3; ++k)
                    if ((bits >> k) & 1u) {
                        if (left == 0u) {
                            corner = k;
                            break;
                        }
                        --left;
                    }
            }
            R[r] = contact_ray(P, q, side, E, corner);
        }
        for (uint32_t p = t; p < n; p += T) {
            const ContactElem& E = El[ins_elem[ord[p]]];
            cg_contact c;
            c.query = q;
            c.side = side;
            c.tri = E.tri;
            c.mask = E.mask;
            const float3 avg = divs3(make_float3(E.sx, E.sy, E.sz), E.w);
            c.weighted_avg[0] = avg.x;
            c.weighted_avg[1] = avg.y;
            c.weighted_avg[2] = avg.z;
            c.weight = E.w;
            P.ctmp[base + p] = c;
        }
        __syncthreads();
    }
    // the mean origin: std::accumulate over the rays in order, one coordinate
    // per lane, from shared memory a chunk of rays at a time
    {
        constexpr uint32_t kStageRays = kOrderSmemWords / 3u;
        float* stage = reinterpret_cast<float*>(smem);
        float acc = 0.0f;
        for (uint32_t r0 = 0; r0 < n_rays; r0 += kStageRays) {
            const uint32_t m = n_rays - r0 < kStageRays ? n_rays - r0 : kStageRays;
            for (uint32_t i = t; i < 3u * m; i += T) stage[i] = R[r0 + i / 3u].origin[i % 3u];
            __syncthreads();
            if (t < 3u) {
#pragma unroll 8
                for (uint32_t r = 0; r < m; ++r) acc = acc + stage[3u * r + t];
            }
            __syncthreads();
        }
        if (t < 3u) fold[t] = acc;
    }
    __syncthreads();
    if (t == 0u) {
        // CreateUncollideRays.cpp:185-198: the sum over the count (0 / 0 for
        // a side without rays), the second side's moved back to its space
        const float cnt_f = float(n_rays);
        float3 avg = divs3(make_float3(fold[0], fold[1], fold[2]), cnt_f);
        if (side) avg = xform(inverse4(query_mat(P.q + q)), avg, 1.0f);
        for (int copy = 0; copy < 2; ++copy) {  // the device's averages, then the host buffer's
            cg_ray_average* A = copy ? (q < P.host_averages_cap ? P.host_averages + q : nullptr) : P.averages + q;
            if (!A) break;
            if (side) {
                A->second[0] = avg.x;
                A->second[1] = avg.y;
                A->second[2] = avg.z;
                A->rays_second = n_rays;
            } else {
                A->first[0] = avg.x;
                A->first[1] = avg.y;
                A->first[2] = avg.z;
                A->rays_first = n_rays;
            }
        }
        P.map_nr[map] = n_rays;
        if (!ok) P.map_fill[map] = 0u;  // a map that did not fit makes no records
    }
}

// Persistent: each block takes the next map of the largest-first list.
__global__ void __launch_bounds__(256, 2) contacts_order_kernel(const ContactParams P) {
    extern __shared__ __align__(16) uint32_t smem_order[];
    __shared__ uint32_t part[64];
    __shared__ float fold[3];
    __shared__ uint32_t next_map;
    const uint32_t n_maps = 2u * P.n_queries;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t i = atomicAdd(&P.ctr->order_ticket, 1u);
            next_map = i < n_maps ? P.map_order[i] : ~0u;
        }
        __syncthreads();
        const uint32_t map = next_map;
        if (map == ~0u) break;
        order_map(P, map, smem_order, part, fold);
        __syncthreads();
    }
    if (last_block(&P.ctr->order_done)) place_maps(P, part);
}

__global__ void __launch_bounds__(256) contacts_emit_kernel(const ContactParams P) {
    const uint32_t m = 2u * P.n_queries;
    for (uint32_t map = blockIdx.x; map < m; map += gridDim.x) {
        const uint32_t n = P.map_fill[map], base = P.map_off[map];
        const uint32_t co = P.map_coff[map], nr = P.map_nr[map], ro = P.map_roff[map];
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
            if (co + i < P.max_contacts) P.contacts[co + i] = P.ctmp[base + i];
        for (uint32_t r = threadIdx.x; r < nr; r += blockDim.x)
            if (ro + r < P.max_rays) {
                const cg_ray ray = P.rtmp[3ull * base + r];
                P.rays[ro + r] = ray;
                if (ro + r < P.host_rays_cap) P.host_rays[ro + r] = ray;
            }
        __syncthreads();
        if (threadIdx.x == 0) {
            P.map_cnt[map] = 0u;
            P.map_fill[map] = 0u;
        }
    }
    // the table slots and leaf-pair marks this launch took
    const uint32_t ns = n_slots(P);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < ns; j += gridDim.x * blockDim.x) {
        ContactSlot e;
        e.key = kEmptyKey;
        e.count = 0u;
        e.offset = 0u;
        P.table[P.occupied[j]] = e;
    }
    const uint32_t nk = min(P.ctr->n_kleaf, P.kleaf_cap);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nk; j += gridDim.x * blockDim.x)
        P.leaf_mark[P.kleaf[j]] = 0u;
}

__global__ void init_tables_kernel(ContactSlot* table, uint32_t n_slots, unsigned long long* vkeys, uint32_t* vval,
                                   uint32_t n_vslots) {
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t i = i0; i < n_slots; i += stride) {
        ContactSlot s;
        s.key = kEmptyKey;
        s.count = 0u;
        s.offset = 0u;
        table[i] = s;
    }
    for (uint32_t i = i0; i < n_vslots; i += stride) {
        vkeys[i] = kEmptyKey;
        vval[i] = ~0u;
    }
}

cudaError_t init_contact_tables(ContactSlot* table, uint32_t n_slots, unsigned long long* vkeys, uint32_t* vval,
                                uint32_t n_vslots, cudaStream_t s) {
    init_tables_kernel<<<1024, 256, 0, s>>>(table, n_slots, vkeys, vval, n_vslots);
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

// The descent path of every stored candidate leaf pair (CG_DFS_ORDER), for
// reading them back in the reference's depth-first order: keys[i] = (path
// high 64 bits, path low 64 bits) of leaf pair i; ERR_DEEP in *error when a
// path has 128 or more splits.
__global__ void __launch_bounds__(kPathWarps * 32) leaf_keys_kernel(const LeafKeyParams P) {
    __shared__ float way[kPathWarps][32][kWayLevels + 1];
    const unsigned long long n_all = *reinterpret_cast<const volatile unsigned long long*>(P.n_leafs);
    const uint32_t n = uint32_t(n_all < P.leaf_cap ? n_all : P.leaf_cap);
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    for (uint32_t b = (blockIdx.x * kPathWarps + wib) * 16u; b < n; b += gridDim.x * kPathWarps * 16u) {
        const uint32_t i = b + (lane >> 1);
        const bool valid = i < n;
        const uint4 lp = valid ? P.leaf_list[i] : make_uint4(0u, 0u, 0u, 0u);
        unsigned long long hi, lo;
        uint32_t depth;
        paired_path(P.q, P.trees, P.recs, lp, valid, way[wib], hi, lo, depth);
        if (!(lane & 1u) && valid) {
            if (depth >= 128u) atomicOr(P.error, ERR_DEEP);
            P.keys[i] = make_ulonglong2(hi, lo);
        }
        __syncwarp();
    }
}

cudaError_t launch_leaf_keys(const LeafKeyParams& p, uint32_t grid, cudaStream_t s) {
    leaf_keys_kernel<<<2u * grid, kPathWarps * 32, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t contacts_order_occupancy(int* blocks_per_sm) {
    const int smem = int(kOrderSmemWords * sizeof(uint32_t));
    cudaError_t e = cudaFuncSetAttribute(contacts_order_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, contacts_order_kernel, 256, smem);
}

cudaError_t contacts_fold_occupancy(int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, contacts_fold_kernel, 256, 0);
}

cudaError_t launch_contacts(const ContactParams& p, uint32_t grid, uint32_t fold_grid, uint32_t order_grid,
                            cudaStream_t s, cudaStream_t branch, cudaEvent_t ev_fork, cudaEvent_t ev_join) {
    if (!p.n_queries) return cudaSuccess;
    const uint32_t maps = 2u * p.n_queries;
    contacts_pairs_kernel<<<grid, 256, 0, s>>>(p);
    // the descent paths need only the listed leaf pairs: a branch beside the
    // contribution lists, joined before the fold
    cudaError_t e = cudaEventRecord(ev_fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(branch, ev_fork, 0);
    if (e != cudaSuccess) return e;
    contacts_paths_kernel<<<2u * grid, kPathWarps * 32, 0, branch>>>(p);
    e = cudaEventRecord(ev_join, branch);
    if (e != cudaSuccess) return e;
    contacts_alloc_kernel<<<grid, 256, 0, s>>>(p);
    contacts_scatter_kernel<<<grid, 256, 0, s>>>(p);
    e = cudaStreamWaitEvent(s, ev_join, 0);
    if (e != cudaSuccess) return e;
    contacts_fold_kernel<<<fold_grid, 256, 0, s>>>(p);
    contacts_order_kernel<<<maps < order_grid ? maps : order_grid, 256, kOrderSmemWords * sizeof(uint32_t), s>>>(p);
    contacts_emit_kernel<<<maps < grid ? maps : grid, 256, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace cg
