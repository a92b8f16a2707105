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
//                     slot's list; empties the previous launch's vertex set
//   contacts_scan     one block: the slots' list offsets, the maps' offsets
//   contacts_scatter  thread per pair: both contributions into their lists
//   contacts_fold     thread per slot: the list sorted by the other triangle,
//                     the reference's two folds, the path of the first leaf
//                     pair of non-zero weight; the triangle into its map
//   contacts_order    block per map (query, side): the insertion order (sort
//                     by path, triangle), the iteration order (one reordering
//                     per growth), the rays (find_rays_lambda,
//                     CreateUncollideRays.cpp:131-178: one per vertex index,
//                     at its first corner in iteration order, else from the
//                     weighted average), the mean origin in ray order
//   contacts_offsets  one block: each map's first record and ray
//   contacts_emit     block per map: records and rays to their places;
//                     empties the table slots and map counters it used
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

// Exclusive scan of get(0..n-1) by one block (blockDim.x <= 1024): each
// thread takes a contiguous run, the runs' sums are scanned in shared memory,
// put(i, prefix) is called in order within each run. Returns the total.
template <class Get, class Put>
__device__ uint32_t block_scan(uint32_t n, uint32_t* part, Get get, Put put) {
    const uint32_t T = blockDim.x, t = threadIdx.x;
    const uint32_t per = (n + T - 1u) / T;
    const uint32_t b0 = min(n, t * per), b1 = min(n, b0 + per);
    uint32_t sum = 0;
    for (uint32_t i = b0; i < b1; ++i) sum += get(i);
    part[t] = sum;
    __syncthreads();
    for (uint32_t o = 1; o < T; o <<= 1) {
        const uint32_t v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;
    const uint32_t total = part[T - 1u];
    for (uint32_t i = b0; i < b1; ++i) {
        const uint32_t v = get(i);
        put(i, run);
        run += v;
    }
    __syncthreads();
    return total;
}

struct WalkRec {
    Box box;
    uint32_t ref, meta;
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
    return R;
}

// The path of the simultaneous descent (OBBtree::IntersectOBBtreesRecursive,
// src/Geometry/OBBtree.cpp:414-476) from the root pair to leaf pair `leaf_i`
// of the list: at every node pair the reference's split decision (two inner
// boxes: the first tree's when its surface is at least the second's as
// transformed; else the inner one), then the child whose subtree holds the
// leaf (bit 0 left, 1 right). Left-aligned in 128 bits; *depth = splits.
__device__ void descent_path(const PackedQuery* queries, const DevTree* trees, const float4* recs, uint4 lp,
                             unsigned long long& hi, unsigned long long& lo, uint32_t& depth) {
    // lp: (query, first triangle a, first triangle b, counts), arena indices
    const PackedQuery* Q = queries + lp.x;
    const DevTree* TA = trees + __ldg(&Q->tree_a);
    const DevTree* TB = trees + __ldg(&Q->tree_b);
    const uint32_t base_a = TA->rec_base, base_b = TB->rec_base;
    const uint2* rg_a = TA->ranges;
    const uint2* rg_b = TB->ranges;
    const uint32_t ta = lp.y - TA->tri_base, tb = lp.z - TB->tri_base;
    const Mat4 M = query_mat(Q);
    WalkRec A = walk_rec(recs, base_a + 1u);
    WalkRec B = walk_rec(recs, base_b + 1u);
    float sb = surface(xform_box(M, B.box));
    hi = lo = 0ull;
    depth = 0;
    for (;;) {
        const bool la = (A.meta & kLeafFlag) != 0u, lb = (B.meta & kLeafFlag) != 0u;
        if ((la && lb) || depth > 128u) break;
        const bool split_a = (!la && !lb) ? (A.surf >= sb) : !la;
        const uint32_t left = split_a ? A.ref : B.ref;
        const uint2 rg = split_a ? __ldg(rg_a + (left - base_a)) : __ldg(rg_b + (left - base_b));
        const uint32_t target = split_a ? ta : tb;
        const uint32_t bit = target >= rg.x + rg.y ? 1u : 0u;
        hi = (hi << 1) | (lo >> 63);
        lo = (lo << 1) | bit;
        ++depth;
        if (split_a) {
            A = walk_rec(recs, left + bit);
        } else {
            B = walk_rec(recs, left + bit);
            sb = surface(xform_box(M, B.box));
        }
    }
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

// Working memory of the order kernel for a map of n triangles (words):
// insertion order (triangle, element), then the sort keys, or the iteration
// order, the growth step's sort keys, their values and the buckets' first
// places; later the rays' counts and places.
struct OrderLayout {
    uint32_t nr, n2, words;
};
__device__ __forceinline__ OrderLayout order_layout(const ContactParams& P, uint32_t n) {
    OrderLayout L;
    L.nr = (n + 1u) & ~1u;
    L.n2 = pow2_ceil(n);
    const uint32_t sort_w = 6u * L.n2;
    const uint32_t epoch_w = 2u * L.nr + 2u * L.n2 + buckets_at(P, n);
    L.words = 2u * L.nr + (sort_w > epoch_w ? sort_w : epoch_w);
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
        uint32_t sa = 0, sb = 0;
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
                const uint32_t xa = atomicAdd(&P.table[sa].count, 1u);
                const uint32_t xb = atomicAdd(&P.table[sb].count, 1u);
                link = make_uint4(sa, sb, xa, xb);
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
    }
}

__global__ void __launch_bounds__(1024) contacts_scan_kernel(const ContactParams P) {
    __shared__ uint32_t part[1024];
    const uint32_t ns = n_slots(P);
    if (threadIdx.x == 0 && ns > P.max_contacts) atomicOr(&P.ctr->c_overflow, CONTACT_TABLE);
    block_scan(
        ns, part, [&](uint32_t i) { return P.table[P.occupied[i]].count; },
        [&](uint32_t i, uint32_t v) { P.table[P.occupied[i]].offset = v; });
    block_scan(
        2u * P.n_queries, part, [&](uint32_t i) { return P.map_cnt[i]; }, [&](uint32_t i, uint32_t v) { P.map_off[i] = v; });
}

__global__ void __launch_bounds__(256) contacts_scatter_kernel(const ContactParams P) {
    const unsigned long long n = n_written_pairs(P);
    for (unsigned long long i = blockIdx.x * 1ull * blockDim.x + threadIdx.x; i < n;
         i += 1ull * gridDim.x * blockDim.x) {
        const uint4 link = P.pg_link[i];
        if (link.x == ~0u) continue;
        const uint4 aux = P.pair_aux[i];
        const unsigned long long pid = (unsigned long long)i << 1;
        P.contrib[P.table[link.x].offset + link.z] = ((unsigned long long)aux.y << 32) | pid;
        P.contrib[P.table[link.y].offset + link.w] = ((unsigned long long)aux.x << 32) | pid | 1ull;
    }
}

__global__ void __launch_bounds__(256) contacts_fold_kernel(const ContactParams P) {
    const uint32_t ns = n_slots(P);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < ns; j += gridDim.x * blockDim.x) {
        const ContactSlot sl = P.table[P.occupied[j]];
        const uint32_t side = uint32_t(sl.key >> 63);
        const uint32_t q = uint32_t(sl.key >> 32) & 0x7fffffffu;
        const uint32_t c = sl.count;
        unsigned long long* L = P.contrib + sl.offset;
        // the triangle's colliding pairs by the other triangle (a handful)
        for (uint32_t a = 1; a < c; ++a) {
            const unsigned long long x = L[a];
            uint32_t b = a;
            while (b > 0u && L[b - 1u] > x) {
                L[b] = L[b - 1u];
                --b;
            }
            L[b] = x;
        }
        // CreateUncollideRays.cpp:96-100, 117-127: a fold per leaf pair from
        // zero, merged in leaf-pair order when its weight is not zero
        bool have = false;
        float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
        unsigned am = 7u;
        uint32_t first_leaf = 0u, cur = ~0u;
        float px = 0.f, py = 0.f, pz = 0.f, pw = 0.f;
        unsigned pm = 7u;
        auto close = [&]() {
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
        };
        for (uint32_t a = 0; a < c; ++a) {
            const uint32_t pid = uint32_t(L[a]) >> 1;
            const uint32_t leaf = __ldg(&P.pair_aux[pid].z);
            if (leaf != cur) {
                if (cur != ~0u) close();
                cur = leaf;
                px = py = pz = pw = 0.0f;
                pm = 7u;
            }
            const float4 g = P.pg_geom[pid];
            px = px + g.x;
            py = py + g.y;
            pz = pz + g.z;
            pw = pw + g.w;
            pm &= (P.pg_mask[pid] >> (3u * side)) & 7u;
        }
        if (cur != ~0u) close();
        if (!have) continue;  // only pairs of zero length: no record (IsNull)
        ContactElem E;
        descent_path(P.q, P.trees, P.recs, P.leaf_list[first_leaf], E.key_hi, E.key_lo, E.depth);
        if (E.depth >= 128u) atomicOr(&P.ctr->c_overflow, CONTACT_ORDER);
        E.sx = ax;
        E.sy = ay;
        E.sz = az;
        E.w = aw;
        E.tri = uint32_t(sl.key);
        E.mask = am;
        E.pad = 0u;
        const uint32_t map = 2u * q + side;
        const uint32_t idx = P.map_off[map] + atomicAdd(P.map_fill + map, 1u);
        if (idx < P.max_contacts) P.elems[idx] = E;
    }
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

// The corners of element E whose vertex ray this map makes (bit k), given
// each corner's place code (pos * 4 + k) in the vertex set: a corner whose
// bit is set makes the ray of its vertex index when it is that index's first
// corner in iteration order (CreateUncollideRays.cpp:148-161, the
// emplaced_point_indices set). insert_codes: record this element's codes
// first.
__device__ unsigned vertex_corners(const ContactParams& P, uint32_t q, uint32_t side, const ContactElem& E,
                                   uint32_t pos, bool insert_codes) {
    const PackedQuery* Q = P.q + q;
    const float4* t = P.tris + 3ull * ((side ? __ldg(&Q->tri_base_b) : __ldg(&Q->tri_base_a)) + E.tri);
    uint32_t vi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) vi[k] = __float_as_uint(__ldg(&t[k].w));
    const Probe V{P.vkeys, 1u, P.vtable_mask};
    unsigned out = 0u;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (!((E.mask >> k) & 1u)) continue;
        bool dup = false;  // an earlier corner of the same triangle with the same vertex index
#pragma unroll
        for (int j = 0; j < k; ++j) dup |= ((E.mask >> j) & 1u) && vi[j] == vi[k];
        if (dup) continue;
        uint32_t slot = 0;
        const int r = insert(V, make_key(side, q, vi[k]), &slot);
        if (r < 0) {
            atomicOr(&P.ctr->c_overflow, CONTACT_VERTICES);
            continue;
        }
        const uint32_t code = pos * 4u + uint32_t(k);
        if (insert_codes) {
            if (r == 1) P.vocc[atomicAdd(&P.ctr->n_vertices, 1u)] = slot;
            atomicMin(P.vval + slot, code);
        } else if (atomicOr(P.vval + slot, 0u) == code) {
            out |= 1u << k;
        }
    }
    return out;
}

__global__ void __launch_bounds__(256) contacts_order_kernel(const ContactParams P) {
    extern __shared__ __align__(16) uint32_t smem_order[];
    __shared__ uint32_t part[256];
    __shared__ float fold[3];
    const uint32_t map = blockIdx.x;
    const uint32_t q = map >> 1, side = map & 1u;
    const uint32_t n = P.map_fill[map];
    const uint32_t base = P.map_off[map];
    const uint32_t T = blockDim.x, t = threadIdx.x;
    uint32_t n_rays = 0;
    bool ok = n > 0u && base + n <= P.max_contacts;
    OrderLayout L{};
    uint32_t* W = smem_order;
    if (ok) {
        L = order_layout(P, n);
        if (L.words > kOrderSmem * 8u) {
            // this map's part of the global working memory: kOrderWords per
            // element from its first element (base + n <= max_contacts)
            W = P.work + size_t(kOrderWords) * base;
            ok = L.words <= kOrderWords * n;
            if (!ok && t == 0u) atomicOr(&P.ctr->c_overflow, CONTACT_ORDER);
        }
    }
    if (ok) {
        const ContactElem* El = P.elems + base;
        uint32_t* ins_tri = W;
        uint32_t* ins_elem = W + L.nr;
        uint32_t* B0 = W + 2u * L.nr;
        // 1. insertion order: the first leaf pair's path, then the triangle
        SortKey* sk = reinterpret_cast<SortKey*>(B0);
        for (uint32_t i = t; i < L.n2; i += T) {
            SortKey k;
            if (i < n) {
                const ContactElem& E = El[i];
                k.hi = E.key_hi;
                k.lo = E.key_lo;
                k.tri = E.tri;
                k.idx = i;
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
        __syncthreads();
        // 2. iteration order after each growth of the table: its buckets most
        // recently started first, each bucket's keys most recently placed
        // first; `ord` is the table's order (insertion indices)
        uint32_t* ord = B0;
        unsigned long long* k64 = reinterpret_cast<unsigned long long*>(B0 + L.nr);
        uint32_t* val = B0 + L.nr + 2u * L.n2;
        uint32_t* first = val + L.nr;
        for (uint32_t e = 0; e < P.n_sched && P.sched_start[e] < n; ++e) {
            const uint32_t st = P.sched_start[e];  // keys in the table when it grows
            const uint32_t m = (e + 1u < P.n_sched && P.sched_start[e + 1u] < n) ? P.sched_start[e + 1u] : n;
            const uint32_t nb = P.sched_buckets[e];
            const uint32_t m2 = pow2_ceil(m);
            for (uint32_t b = t; b < nb; b += T) first[b] = ~0u;
            __syncthreads();
            // place s: the key the growth re-places s-th (the table's order),
            // then the keys inserted before the next growth
            for (uint32_t s = t; s < m; s += T) {
                const uint32_t x = s < st ? ord[s] : s;
                atomicMin(first + ins_tri[x] % nb, s);
            }
            __syncthreads();
            for (uint32_t s = t; s < m2; s += T) {
                unsigned long long k = ~0ull;
                if (s < m) {
                    const uint32_t x = s < st ? ord[s] : s;
                    k = ((unsigned long long)(~first[ins_tri[x] % nb]) << 32) | (~s);
                }
                k64[s] = k;
            }
            __syncthreads();
            bitonic(k64, m2, [](unsigned long long a, unsigned long long b) { return a < b; });
            for (uint32_t p = t; p < m; p += T) {
                const uint32_t s = ~uint32_t(k64[p]);
                val[p] = s < st ? ord[s] : s;
            }
            __syncthreads();
            for (uint32_t p = t; p < m; p += T) ord[p] = val[p];
            __syncthreads();
        }
        // 3. rays: the vertex set keeps each vertex index's first corner
        uint32_t* rc = B0 + L.nr;  // per place: rays
        uint32_t* rb = val;        // per place: vertex corners that make a ray
        for (uint32_t p = t; p < n; p += T) {
            const ContactElem& E = El[ins_elem[ord[p]]];
            if (E.mask) vertex_corners(P, q, side, E, p, true);
        }
        __syncthreads();
        for (uint32_t p = t; p < n; p += T) {
            const ContactElem& E = El[ins_elem[ord[p]]];
            const unsigned bits = E.mask ? vertex_corners(P, q, side, E, p, false) : 0u;
            rb[p] = bits;
            rc[p] = E.mask ? __popc(bits) : 1u;
        }
        __syncthreads();
        n_rays = block_scan(
            n, part, [&](uint32_t i) { return rc[i]; }, [&](uint32_t i, uint32_t v) { rc[i] = v; });
        cg_ray* R = P.rtmp + 3ull * base;
        for (uint32_t p = t; p < n; p += T) {
            const ContactElem& E = El[ins_elem[ord[p]]];
            uint32_t o = rc[p];
            if (E.mask) {
                for (int k = 0; k < 3; ++k)
                    if ((rb[p] >> k) & 1u) R[o++] = contact_ray(P, q, side, E, k);
            } else {
                R[o] = contact_ray(P, q, side, E, -1);
            }
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
        // the mean origin: std::accumulate over the rays in order, one
        // coordinate per lane
        if (t < 3u) {
            float s = 0.0f;
            for (uint32_t r = 0; r < n_rays; ++r) s = s + R[r].origin[t];
            fold[t] = s;
        }
    } else if (t < 3u) {
        fold[t] = 0.0f;
    }
    __syncthreads();
    if (t == 0u) {
        // CreateUncollideRays.cpp:185-198: the sum over the count (0 / 0 for
        // a side without rays), the second side's moved back to its space
        const float cnt = float(n_rays);
        float3 avg = divs3(make_float3(fold[0], fold[1], fold[2]), cnt);
        cg_ray_average* A = P.averages + q;
        if (side) {
            avg = xform(inverse4(query_mat(P.q + q)), avg, 1.0f);
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
        P.map_nr[map] = n_rays;
        if (!ok) P.map_fill[map] = 0u;  // a map that did not fit makes no records
    }
}

__global__ void __launch_bounds__(1024) contacts_offsets_kernel(const ContactParams P) {
    __shared__ uint32_t part[1024];
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

__global__ void __launch_bounds__(256) contacts_emit_kernel(const ContactParams P) {
    const uint32_t m = 2u * P.n_queries;
    for (uint32_t map = blockIdx.x; map < m; map += gridDim.x) {
        const uint32_t n = P.map_fill[map], base = P.map_off[map];
        const uint32_t co = P.map_coff[map], nr = P.map_nr[map], ro = P.map_roff[map];
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
            if (co + i < P.max_contacts) P.contacts[co + i] = P.ctmp[base + i];
        for (uint32_t r = threadIdx.x; r < nr; r += blockDim.x)
            if (ro + r < P.max_rays) P.rays[ro + r] = P.rtmp[3ull * base + r];
        __syncthreads();
        if (threadIdx.x == 0) {
            P.map_cnt[map] = 0u;
            P.map_fill[map] = 0u;
        }
    }
    // the table slots this launch took
    const uint32_t ns = n_slots(P);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < ns; j += gridDim.x * blockDim.x) {
        ContactSlot e;
        e.key = kEmptyKey;
        e.count = 0u;
        e.offset = 0u;
        P.table[P.occupied[j]] = e;
    }
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
__global__ void __launch_bounds__(256) leaf_keys_kernel(const LeafKeyParams P) {
    const unsigned long long n_all = *reinterpret_cast<const volatile unsigned long long*>(P.n_leafs);
    const uint32_t n = uint32_t(n_all < P.leaf_cap ? n_all : P.leaf_cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned long long hi, lo;
        uint32_t depth;
        descent_path(P.q, P.trees, P.recs, P.leaf_list[i], hi, lo, depth);
        if (depth >= 128u) atomicOr(P.error, ERR_DEEP);
        P.keys[i] = make_ulonglong2(hi, lo);
    }
}

cudaError_t launch_leaf_keys(const LeafKeyParams& p, uint32_t grid, cudaStream_t s) {
    leaf_keys_kernel<<<grid, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_contacts(const ContactParams& p, uint32_t grid, cudaStream_t s) {
    if (!p.n_queries) return cudaSuccess;
    const uint32_t maps = 2u * p.n_queries;
    contacts_pairs_kernel<<<grid, 256, 0, s>>>(p);
    contacts_scan_kernel<<<1, 1024, 0, s>>>(p);
    contacts_scatter_kernel<<<grid, 256, 0, s>>>(p);
    contacts_fold_kernel<<<grid, 256, 0, s>>>(p);
    contacts_order_kernel<<<maps, 256, kOrderSmem * 8u * sizeof(uint32_t), s>>>(p);
    contacts_offsets_kernel<<<1, 1024, 0, s>>>(p);
    contacts_emit_kernel<<<maps < grid ? maps : grid, 256, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace cg
