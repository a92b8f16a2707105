// Collision kernels for sm_103a: query packing, counter reset, record surfaces
// and the persistent warp-cooperative OBB-tree traversal with the fused
// triangle-pair (Moller) narrow phase.
//
// Traversal design. Each warp owns a node-pair deque in shared memory and
// advances up to 32 node pairs per step, one per lane: load both child-box
// records (four 16-byte loads each), move B's box into A's space, run the
// 15-axis SAT, and apply the reference's descent rule
// (OBBtree::IntersectOBBtreesRecursive, src/Geometry/OBBtree.cpp:414-476):
// two inner nodes -> split the one with the larger surface, ties to the first
// tree; one leaf -> split the other; two leaves -> a candidate leaf pair.
// Surviving child pairs are pushed with __ballot_sync/__popc compaction, and
// leaf pairs are buffered per warp; once leaf_flush of them are buffered the
// warp runs their triangle pairs, one pair per lane. Load balance across warps
// uses a global task queue: root pairs of all queries are the first slots, and
// a warp with surplus work gives the bottom (shallowest) entries of its deque
// to warps that are waiting. Every wait is bounded by wait_ns (globaltimer),
// after which the kernel records ERR_TIMEOUT and returns.
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint4 ld_relaxed4(const uint4* p) {
    uint4 v;
    asm volatile("ld.relaxed.gpu.global.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
}
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

struct Rec {
    Box box;
    uint32_t ref;
    uint32_t meta;
    float surf;
};

__device__ __forceinline__ Rec load_rec(const float4* recs, uint32_t r) {
    const float4* p = recs + 4ull * r;
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    Rec R;
    R.box.c = make_float3(a.x, a.y, a.z);
    R.box.u = make_float3(a.w, b.x, b.y);
    R.box.v = make_float3(b.z, b.w, c.x);
    R.box.w = make_float3(c.y, c.z, c.w);
    R.ref = __float_as_uint(d.x);
    R.meta = __float_as_uint(d.y);
    R.surf = d.z;
    return R;
}

__device__ __forceinline__ Mat4 load_mat(const PackedQuery* Q) {
    Mat4 M;
    M.c0 = __ldg(&Q->m[0]);
    M.c1 = __ldg(&Q->m[1]);
    M.c2 = __ldg(&Q->m[2]);
    M.c3 = __ldg(&Q->m[3]);
    return M;
}

__device__ __forceinline__ void load_tri(const float4* tris, uint32_t i, float3& p0, float3& p1, float3& p2) {
    const float4* p = tris + 3ull * i;
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    p0 = make_float3(a.x, a.y, a.z);
    p1 = make_float3(b.x, b.y, b.z);
    p2 = make_float3(c.x, c.y, c.z);
}

// Claims the next queue slot (lane 0 only). Root slots are immediate; a
// donated slot is waited for until it is published, all work is finished, an
// error is raised, or the wait limit passes.
__device__ int acquire(const TraverseParams& P, uint32_t& q, uint32_t& a, uint32_t& b) {
    const unsigned slot = atomicAdd(&P.ctr->head, 1u);
    if (slot < P.n_queries) {
        q = slot;
        a = 1;
        b = 1;
        return 1;
    }
    const unsigned idx = slot - P.n_queries;
    if (idx >= P.task_slots) {
        // Only reachable if more warps wait than the slack allows; nothing
        // can ever be published there, so wait for the end of all work.
        const unsigned long long t0 = gtimer();
        while (ld_relaxed(&P.ctr->work) != 0 && ld_relaxed(&P.ctr->error) == 0) {
            if (gtimer() - t0 > P.wait_ns) {
                atomicOr(&P.ctr->error, ERR_TIMEOUT);
                break;
            }
            __nanosleep(1024);
        }
        return 0;
    }
    const unsigned long long t0 = gtimer();
    unsigned ns = 32;
    for (;;) {
        if (ld_acquire(P.ready + idx)) {
            const uint4 t = ld_relaxed4(P.tasks + idx);
            q = t.x;
            a = t.y;
            b = t.z;
            return 1;
        }
        if (ld_relaxed(&P.ctr->work) == 0) return 0;
        if (ld_relaxed(&P.ctr->error) != 0) return 0;
        if (gtimer() - t0 > P.wait_ns) {
            atomicOr(&P.ctr->error, ERR_TIMEOUT);
            return 0;
        }
        __nanosleep(ns);
        if (ns < 1024) ns <<= 1;
    }
}

struct LeafBuf {
    uint32_t* q;
    uint32_t* oa;
    uint32_t* ob;
    uint32_t* cn;  // count_a | count_b << 16
    uint32_t* pre; // kLeafCap + 1 exclusive prefix sums of count_a * count_b
};

// Runs every triangle pair of the buffered leaf pairs, one pair per lane, in
// the order of the reference's pair loop per leaf pair
// (CreateUncollideRays.cpp:139-148): B's triangle is moved into A's space with
// TrianglePosition::MultiplyBy4x4Matrix arithmetic, then tested.
__device__ void flush_leafs(const TraverseParams& P, const LeafBuf& L, uint32_t nl, int lane,
                            unsigned long long& tests, unsigned long long& fragile) {
    uint32_t c0 = 0, c1 = 0;
    if (uint32_t(lane) < nl) {
        const uint32_t cn = L.cn[lane];
        c0 = (cn & 0xffffu) * (cn >> 16);
    }
    if (uint32_t(lane) + 32 < nl) {
        const uint32_t cn = L.cn[lane + 32];
        c1 = (cn & 0xffffu) * (cn >> 16);
    }
    uint32_t s0 = c0, s1 = c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t0 = __shfl_up_sync(kFull, s0, o);
        const uint32_t t1 = __shfl_up_sync(kFull, s1, o);
        if (lane >= o) {
            s0 += t0;
            s1 += t1;
        }
    }
    const uint32_t tot0 = __shfl_sync(kFull, s0, 31);
    const uint32_t total = tot0 + __shfl_sync(kFull, s1, 31);
    L.pre[lane] = s0 - c0;
    L.pre[lane + 32] = tot0 + s1 - c1;
    if (lane == 0) L.pre[kLeafCap] = total;

    if (P.flags & CG_KEEP_LEAF_PAIRS) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&P.ctr->n_leafs, (unsigned long long)nl);
        base = __shfl_sync(kFull, base, 0);
        for (uint32_t e = lane; e < nl; e += 32) {
            if (base + e < P.leafs_cap) {
                cg_leaf_pair lp;
                lp.query = L.q[e];
                lp.offset_a = L.oa[e];
                lp.offset_b = L.ob[e];
                lp.count_a = uint16_t(L.cn[e] & 0xffffu);
                lp.count_b = uint16_t(L.cn[e] >> 16);
                P.leafs[base + e] = lp;
            }
        }
    } else {
        if (lane == 0) atomicAdd(&P.ctr->n_leafs, (unsigned long long)nl);
    }
    __syncwarp();

    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t t = base + lane;
        int res = TT_MISS;
        uint32_t q = 0, ia = 0, ib = 0;
        float3 src = make_float3(0.f, 0.f, 0.f), tgt = src;
        if (t < total) {
            int lo = 0, hi = int(nl) - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (L.pre[mid] <= t)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const uint32_t local = t - L.pre[lo];
            const uint32_t cn = L.cn[lo];
            const uint32_t cb = cn >> 16;
            const uint32_t i = local / cb;
            const uint32_t j = local - i * cb;
            q = L.q[lo];
            ia = L.oa[lo] + i;
            ib = L.ob[lo] + j;
            const PackedQuery* Q = P.q + q;
            const Mat4 M = load_mat(Q);
            const float4* tris_a = reinterpret_cast<const float4*>(__ldg(reinterpret_cast<const unsigned long long*>(&Q->tris_a)));
            const float4* tris_b = reinterpret_cast<const float4*>(__ldg(reinterpret_cast<const unsigned long long*>(&Q->tris_b)));
            float3 a0, a1, a2, b0, b1, b2;
            load_tri(tris_a, ia, a0, a1, a2);
            load_tri(tris_b, ib, b0, b1, b2);
            b0 = xform(M, b0, 1.0f);
            b1 = xform(M, b1, 1.0f);
            b2 = xform(M, b2, 1.0f);
            res = tri_tri(a0, a1, a2, b0, b1, b2, src, tgt);
        }
        const unsigned hitmask = __ballot_sync(kFull, res == TT_HIT);
        const unsigned fragmask = __ballot_sync(kFull, res == TT_FRAGILE);
        if (hitmask) {
            unsigned long long obase = 0;
            if (lane == 0) obase = atomicAdd(&P.ctr->n_pairs, (unsigned long long)__popc(hitmask));
            obase = __shfl_sync(kFull, obase, 0);
            if (res == TT_HIT && !(P.flags & CG_NO_TRI_PAIRS)) {
                const unsigned long long o = obase + __popc(hitmask & lanemask_lt());
                if (o < P.pairs_cap) {
                    cg_tri_pair r;
                    r.query = q;
                    r.tri_a = ia;
                    r.tri_b = ib;
                    r.source[0] = src.x;
                    r.source[1] = src.y;
                    r.source[2] = src.z;
                    r.target[0] = tgt.x;
                    r.target[1] = tgt.y;
                    r.target[2] = tgt.z;
                    P.pairs[o] = r;
                }
            }
        }
        if (lane == 0) fragile += __popc(fragmask);
    }
    if (lane == 0) tests += total;
    __syncwarp();
}

}  // namespace

__global__ void __launch_bounds__(512) traverse_kernel(const TraverseParams P) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const uint32_t S = P.stack_cap;
    const uint32_t MASK = S - 1u;
    uint32_t* sq = smem + size_t(warp) * warp_smem_words(S);
    uint32_t* sa = sq + S;
    uint32_t* sb = sa + S;
    LeafBuf L;
    L.q = sb + S;
    L.oa = L.q + kLeafCap;
    L.ob = L.oa + kLeafCap;
    L.cn = L.ob + kLeafCap;
    L.pre = L.cn + kLeafCap;

    uint32_t top = 0, bot = 0, nl = 0;
    unsigned long long st_nodes = 0, st_tests = 0, st_frag = 0, st_don = 0;

    for (;;) {
        if (top == bot) {
            uint32_t tq = 0, ta = 0, tb = 0;
            int got = 0;
            if (lane == 0) got = acquire(P, tq, ta, tb);
            got = __shfl_sync(kFull, got, 0);
            if (!got) break;
            tq = __shfl_sync(kFull, tq, 0);
            ta = __shfl_sync(kFull, ta, 0);
            tb = __shfl_sync(kFull, tb, 0);
            if (lane == 0) {
                sq[top & MASK] = tq;
                sa[top & MASK] = ta;
                sb[top & MASK] = tb;
            }
            ++top;
            __syncwarp();
        }

        // ---- one step over up to 32 node pairs from the top of the deque
        const uint32_t size = top - bot;
        const uint32_t n = size < 32u ? size : 32u;
        const bool active = uint32_t(lane) < n;
        uint32_t q = 0, ra = 0, rb = 0;
        if (active) {
            const uint32_t pos = (top - n + lane) & MASK;
            q = sq[pos];
            ra = sa[pos];
            rb = sb[pos];
        }
        top -= n;
        __syncwarp();

        int act = 0;  // 1: split A, 2: split B, 3: leaf pair
        uint32_t child = 0, offA = 0, offB = 0, cnt = 0;
        if (active) {
            const PackedQuery* Q = P.q + q;
            const float4* recs_a = reinterpret_cast<const float4*>(__ldg(reinterpret_cast<const unsigned long long*>(&Q->recs_a)));
            const float4* recs_b = reinterpret_cast<const float4*>(__ldg(reinterpret_cast<const unsigned long long*>(&Q->recs_b)));
            if (recs_a != nullptr && recs_b != nullptr) {
                const Mat4 M = load_mat(Q);
                const Rec A = load_rec(recs_a, ra);
                const Rec B = load_rec(recs_b, rb);
                const Box bb = xform_box(M, B.box);
                if (sat(A.box, bb)) {
                    const bool la = (A.meta & kLeafFlag) != 0;
                    const bool lb = (B.meta & kLeafFlag) != 0;
                    if (!la && !lb)
                        act = (A.surf >= surface(bb)) ? 1 : 2;
                    else if (la && !lb)
                        act = 2;
                    else if (!la && lb)
                        act = 1;
                    else
                        act = 3;
                    child = act == 1 ? A.ref : B.ref;
                    offA = A.ref;
                    offB = B.ref;
                    cnt = (A.meta & 0xffffu) | ((B.meta & 0xffffu) << 16);
                }
            }
        }

        const unsigned pushmask = __ballot_sync(kFull, act == 1 || act == 2);
        if (act == 1 || act == 2) {
            const uint32_t r = __popc(pushmask & lanemask_lt());
            const uint32_t p0 = (top + 2u * r) & MASK;
            const uint32_t p1 = (top + 2u * r + 1u) & MASK;
            const uint32_t c_left = 2u * child + 2u, c_right = 2u * child + 3u;
            sq[p0] = q;
            sq[p1] = q;
            if (act == 1) {
                sa[p0] = c_right;
                sb[p0] = rb;
                sa[p1] = c_left;
                sb[p1] = rb;
            } else {
                sa[p0] = ra;
                sb[p0] = c_right;
                sa[p1] = ra;
                sb[p1] = c_left;
            }
        }
        top += 2u * __popc(pushmask);

        const unsigned leafmask = __ballot_sync(kFull, act == 3);
        if (act == 3) {
            const uint32_t slot = nl + __popc(leafmask & lanemask_lt());
            L.q[slot] = q;
            L.oa[slot] = offA;
            L.ob[slot] = offB;
            L.cn[slot] = cnt;
        }
        nl += __popc(leafmask);
        if (lane == 0) st_nodes += n;
        __syncwarp();

        if (nl >= P.leaf_flush || (top == bot && nl > 0)) {
            flush_leafs(P, L, nl, lane, st_tests, st_frag);
            nl = 0;
        }

        // ---- give the bottom of the deque away: when it is nearly full
        // (forced), or when other warps wait for work.
        const uint32_t held = top - bot;
        if (held >= P.donate_min) {
            const bool forced = held + 64u > S;
            int give = 0;
            if (lane == 0) {
                const unsigned tail = ld_relaxed(&P.ctr->tail);
                const unsigned head = ld_relaxed(&P.ctr->head);
                const bool waiting = int(tail - head) < 0;
                const uint32_t k = min(32u, held - 32u);
                if ((forced || waiting) && tail - P.n_queries + k <= P.task_cap) {
                    atomicAdd(&P.ctr->work, k);
                    give = int(atomicAdd(&P.ctr->tail, k) - P.n_queries);
                    give = give + 1;  // 0 means "no donation"
                }
            }
            give = __shfl_sync(kFull, give, 0);
            const uint32_t k = min(32u, held - 32u);
            if (give > 0) {
                const uint32_t idx = uint32_t(give - 1) + lane;
                if (uint32_t(lane) < k) {
                    const uint32_t pos = (bot + lane) & MASK;
                    P.tasks[idx] = make_uint4(sq[pos], sa[pos], sb[pos], 0u);
                    st_release(P.ready + idx, 1u);
                }
                bot += k;
                if (lane == 0) st_don += k;
                __syncwarp();
            } else if (forced) {
                if (lane == 0) atomicOr(&P.ctr->error, ERR_QUEUE);
                break;
            }
        }

        if (top == bot && lane == 0) atomicSub(&P.ctr->work, 1u);
    }

    if (lane == 0) {
        atomicAdd(&P.ctr->node_pairs, st_nodes);
        atomicAdd(&P.ctr->tri_tests, st_tests);
        atomicAdd(&P.ctr->fragile, st_frag);
        atomicAdd(&P.ctr->donations, st_don);
    }
}

__global__ void pack_kernel(const cg_query* in, uint32_t n, const DevTree* trees, uint32_t n_trees, PackedQuery* out,
                            Counters* ctr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cg_query Q = in[i];
    PackedQuery p;
    p.m[0] = make_float4(Q.relative[0], Q.relative[1], Q.relative[2], Q.relative[3]);
    p.m[1] = make_float4(Q.relative[4], Q.relative[5], Q.relative[6], Q.relative[7]);
    p.m[2] = make_float4(Q.relative[8], Q.relative[9], Q.relative[10], Q.relative[11]);
    p.m[3] = make_float4(Q.relative[12], Q.relative[13], Q.relative[14], Q.relative[15]);
    const bool ok = Q.tree_a < n_trees && Q.tree_b < n_trees && trees[Q.tree_a].recs != nullptr &&
                    trees[Q.tree_b].recs != nullptr;
    if (ok) {
        p.recs_a = trees[Q.tree_a].recs;
        p.recs_b = trees[Q.tree_b].recs;
        p.tris_a = trees[Q.tree_a].tris;
        p.tris_b = trees[Q.tree_b].tris;
    } else {
        p.recs_a = p.recs_b = p.tris_a = p.tris_b = nullptr;
        atomicOr(&ctr->error, ERR_BAD_QUERY);
    }
    out[i] = p;
}

__global__ void init_kernel(Counters* ctr, uint32_t n_queries) {
    Counters c = {};
    c.tail = n_queries;
    c.work = n_queries;
    *ctr = c;
}

// Paralgram::GetSurface of every record, written into q3.z.
__global__ void surfaces_kernel(float4* recs, uint32_t n_recs) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_recs) return;
    float4* p = recs + 4ull * r;
    const float4 a = p[0], b = p[1], c = p[2];
    Box box;
    box.c = make_float3(a.x, a.y, a.z);
    box.u = make_float3(a.w, b.x, b.y);
    box.v = make_float3(b.z, b.w, c.x);
    box.w = make_float3(c.y, c.z, c.w);
    p[3].z = surface(box);
}

cudaError_t launch_pack(const cg_query* in, uint32_t n, const DevTree* trees, uint32_t n_trees, PackedQuery* out,
                        Counters* ctr, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    pack_kernel<<<(n + 255) / 256, 256, 0, s>>>(in, n, trees, n_trees, out, ctr);
    return cudaGetLastError();
}

cudaError_t launch_init(Counters* ctr, uint32_t n_queries, cudaStream_t s) {
    init_kernel<<<1, 1, 0, s>>>(ctr, n_queries);
    return cudaGetLastError();
}

cudaError_t launch_surfaces(float4* recs, uint32_t n_recs, cudaStream_t s) {
    if (n_recs == 0) return cudaSuccess;
    surfaces_kernel<<<(n_recs + 255) / 256, 256, 0, s>>>(recs, n_recs);
    return cudaGetLastError();
}

cudaError_t traverse_occupancy(uint32_t warps_per_block, uint32_t stack_cap, int* blocks_per_sm) {
    const size_t smem = size_t(warps_per_block) * warp_smem_words(stack_cap) * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(traverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, traverse_kernel, int(32 * warps_per_block),
                                                         smem);
}

cudaError_t launch_traverse(const TraverseParams& p, uint32_t blocks, uint32_t warps_per_block, cudaStream_t s) {
    const size_t smem = size_t(warps_per_block) * warp_smem_words(p.stack_cap) * sizeof(uint32_t);
    traverse_kernel<<<blocks, 32 * warps_per_block, smem, s>>>(p);
    return cudaGetLastError();
}

}  // namespace cg
