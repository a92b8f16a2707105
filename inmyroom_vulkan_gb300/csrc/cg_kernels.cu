// Collision kernels for sm_103a: query packing, counter reset, record surfaces
// and the persistent warp-cooperative OBB-tree traversal with the fused
// triangle-pair (Moller) narrow phase.
//
// Traversal design. Each warp owns a node-pair deque in shared memory and
// advances up to 32 node pairs per step, one per lane: load both box records
// (four 16-byte loads each), move B's box into A's space, run the 15-axis SAT,
// and apply the reference's descent rule (OBBtree::IntersectOBBtreesRecursive,
// src/Geometry/OBBtree.cpp:414-476): two inner nodes -> split the one with the
// larger surface, ties to the first tree; one leaf -> split the other; two
// leaves -> a candidate leaf pair. Surviving child pairs are pushed with
// __ballot_sync/__popc compaction; leaf pairs are buffered per warp, and once
// leaf_flush of them are buffered the warp runs their triangle pairs, one pair
// per lane.
//
// Load balance uses a global task queue. Tasks are chunks of up to 32 node
// pairs in a pool; the root pairs of all queries are the first slots. A warp
// whose deque runs dry claims the next slot and waits for it; a warp with
// fewer than 32 node pairs tops up with already published slots without
// waiting; a warp with surplus gives half of the bottom (shallowest) part of
// its deque to waiting warps. Every wait is bounded by wait_ns (globaltimer),
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
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
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
__device__ __forceinline__ uint2 ld_relaxed2(const uint2* p) {
    uint2 v;
    asm volatile("ld.relaxed.gpu.global.v2.u32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// head in the low 32 bits, tail in the high 32 bits of Counters::ht.
__device__ __forceinline__ unsigned long long* ht_of(Counters* c) {
    return reinterpret_cast<unsigned long long*>(&c->head);
}
__device__ __forceinline__ uint32_t ht_head(unsigned long long v) { return uint32_t(v); }
__device__ __forceinline__ uint32_t ht_tail(unsigned long long v) { return uint32_t(v >> 32); }

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

// The same 15 axes in the same order as cg::sat, as loops (a's then b's face
// normals, then a_i x b_j) to keep the traversal kernel's code small.
__device__ __forceinline__ bool sat_rolled(const Box& a, const Box& b) {
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
        const float3 u = s ? b.u : a.u;
        const float3 v = s ? b.v : a.v;
        const float3 w = s ? b.w : a.w;
        if (!overlap_on(a, b, cross3(v, w))) return false;
        if (!overlap_on(a, b, cross3(u, w))) return false;
        if (!overlap_on(a, b, cross3(u, v))) return false;
    }
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        const float3 e = i == 0 ? a.u : (i == 1 ? a.v : a.w);
        if (!overlap_on(a, b, cross3(e, b.u))) return false;
        if (!overlap_on(a, b, cross3(e, b.v))) return false;
        if (!overlap_on(a, b, cross3(e, b.w))) return false;
    }
    return true;
}

struct Deque {
    uint32_t* q;
    uint32_t* a;
    uint32_t* b;
    uint32_t mask;
};

struct LeafBuf {
    uint32_t* q;
    uint32_t* oa;
    uint32_t* ob;
    uint32_t* cn;  // count_a | count_b << 16
    uint32_t* pre; // kLeafCap + 1 exclusive prefix sums of count_a * count_b
};

// Reads the chunk of slot `slot` (already published) into the deque at `top`;
// returns its size (uniform over the warp).
__device__ uint32_t take_chunk(const TraverseParams& P, uint32_t slot, const Deque& D, uint32_t top, int lane) {
    uint32_t off = 0, cnt = 1;
    // Lane 0 observed the slot's release (wait_ready); the barrier orders the
    // other lanes' pool reads after that acquire.
    __syncwarp();
    if (slot >= P.n_queries) {
        if (lane == 0) {
            const uint2 c = ld_relaxed2(P.slots + (slot - P.n_queries));
            off = c.x;
            cnt = c.y;
        }
        off = __shfl_sync(kFull, off, 0);
        cnt = __shfl_sync(kFull, cnt, 0);
        if (uint32_t(lane) < cnt) {
            const uint4 e = ld_relaxed4(P.pool + off + lane);
            const uint32_t pos = (top + lane) & D.mask;
            D.q[pos] = e.x;
            D.a[pos] = e.y;
            D.b[pos] = e.z;
        }
    } else {
        // root pair of query `slot`; an invalid query (root 0) has no work
        uint32_t ra = 0, rb = 0;
        if (lane == 0) {
            const PackedQuery* Q = P.q + slot;
            ra = __ldg(&Q->root_a);
            rb = __ldg(&Q->root_b);
            if (ra != 0u) {
                const uint32_t pos = top & D.mask;
                D.q[pos] = slot;
                D.a[pos] = ra;
                D.b[pos] = rb;
            }
        }
        cnt = __shfl_sync(kFull, ra != 0u ? 1u : 0u, 0);
    }
    __syncwarp();
    return cnt;
}

// Lane 0: waits until donated slot `slot` is published. Returns 0 when all
// work finished, an error was raised, or the wait limit passed.
__device__ int wait_ready(const TraverseParams& P, uint32_t slot) {
    if (slot < P.n_queries) return 1;
    const uint32_t idx = slot - P.n_queries;
    const unsigned long long t0 = gtimer();
    if (idx >= P.slot_alloc) {
        // Past every slot a donor could publish: only the end of the work or
        // an error can release this warp.
        while (ld_relaxed(&P.ctr->work) != 0 && ld_relaxed(&P.ctr->error) == 0) {
            if (gtimer() - t0 > P.wait_ns) {
                atomicOr(&P.ctr->error, ERR_TIMEOUT);
                break;
            }
            __nanosleep(1024);
        }
        return 0;
    }
    unsigned ns = 32;
    for (;;) {
        if (ld_acquire(P.ready + idx)) return 1;
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

// Lane 0: claims a slot below the tail without waiting for new donations.
// A claimed slot below the tail is published promptly by its donor.
__device__ int try_claim(const TraverseParams& P, unsigned long long ht, uint32_t& slot) {
    unsigned long long* w = ht_of(P.ctr);
    for (int tries = 0; tries < 4; ++tries) {
        if (int(ht_tail(ht) - ht_head(ht)) <= 0) return 0;
        const unsigned long long prev = atomicCAS(w, ht, ht + 1ull);
        if (prev == ht) {
            slot = ht_head(ht);
            return 1;
        }
        ht = prev;
    }
    return 0;
}

// Runs every triangle pair of the buffered leaf pairs, one pair per lane, in
// the order of the reference's pair loop per leaf pair
// (CreateUncollideRays.cpp:139-148): B's triangle is moved into A's space with
// TrianglePosition::MultiplyBy4x4Matrix arithmetic, then tested.
__device__ void flush_leafs(const TraverseParams& P, const LeafBuf& L, uint32_t nl, int lane,
                            unsigned long long& tests, unsigned long long& fragile, unsigned long long t_base) {
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

    unsigned long long lbase = 0;
    if (lane == 0) lbase = atomicAdd(&P.ctr->n_leafs, (unsigned long long)nl);
    if (P.flags & CG_KEEP_LEAF_PAIRS) {
        lbase = __shfl_sync(kFull, lbase, 0);
        for (uint32_t e = lane; e < nl; e += 32) {
            if (lbase + e < P.leafs_cap) {
                const PackedQuery* Q = P.q + L.q[e];
                cg_leaf_pair lp;
                lp.query = L.q[e];
                lp.offset_a = L.oa[e] - __ldg(&Q->tri_base_a);
                lp.offset_b = L.ob[e] - __ldg(&Q->tri_base_b);
                lp.count_a = uint16_t(L.cn[e] & 0xffffu);
                lp.count_b = uint16_t(L.cn[e] >> 16);
                P.leafs[lbase + e] = lp;
            }
        }
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
            float3 a0, a1, a2, b0, b1, b2;
            load_tri(P.tris, ia, a0, a1, a2);
            load_tri(P.tris, ib, b0, b1, b2);
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
                    const PackedQuery* Q = P.q + q;
                    cg_tri_pair r;
                    r.query = q;
                    r.tri_a = ia - __ldg(&Q->tri_base_a);
                    r.tri_b = ib - __ldg(&Q->tri_base_b);
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
        if (lane == 0) {
            fragile += __popc(fragmask);
            if (P.trace) {
                const unsigned long long b = (gtimer() - t_base) / P.trace_ns;
                if (b < kTraceBuckets) {
                    atomicAdd(P.trace + 4 * b + 2, min(32u, total - base));
                    atomicAdd(P.trace + 4 * b + 3, 1u);
                }
            }
        }
    }
    if (lane == 0) tests += total;
    __syncwarp();
}

}  // namespace

__global__ void __launch_bounds__(256, 3) traverse_kernel(const TraverseParams P) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const uint32_t S = P.stack_cap;
    Deque D;
    D.q = smem + size_t(warp) * warp_smem_words(S);
    D.a = D.q + S;
    D.b = D.a + S;
    D.mask = S - 1u;
    LeafBuf L;
    L.q = D.b + S;
    L.oa = L.q + kLeafCap;
    L.ob = L.oa + kLeafCap;
    L.cn = L.ob + kLeafCap;
    L.pre = L.cn + kLeafCap;
    unsigned long long* ht = ht_of(P.ctr);

    uint32_t top = 0, bot = 0, nl = 0, held_tasks = 0;
    unsigned long long st_nodes = 0, st_tests = 0, st_frag = 0, st_don = 0, st_steps = 0;
    unsigned long long t_base = 0;
    if (P.trace && lane == 0) {
        const unsigned long long now = gtimer();
        const unsigned long long old = atomicCAS(&P.ctr->t_start, 0ull, now);
        t_base = old ? old : now;
    }

    for (;;) {
        if (top == bot) {
            // Out of work: claim the next slot and wait for it.
            uint32_t slot = 0;
            int got = 0;
            if (lane == 0) {
                slot = ht_head(atomicAdd(ht, 1ull));
                got = wait_ready(P, slot);
            }
            got = __shfl_sync(kFull, got, 0);
            if (!got) break;
            slot = __shfl_sync(kFull, slot, 0);
            top += take_chunk(P, slot, D, top, lane);
            held_tasks = 1;
        }

        // Queue state, read early so its latency overlaps the step's loads.
        unsigned long long qs = 0;
        if (lane == 0) qs = ld_relaxed64(ht);

        // ---- one step over up to 32 node pairs from the top of the deque
        const uint32_t size = top - bot;
        const uint32_t n = size < 32u ? size : 32u;
        const bool active = uint32_t(lane) < n;
        uint32_t q = 0, ra = 0, rb = 0;
        if (active) {
            const uint32_t pos = (top - n + lane) & D.mask;
            q = D.q[pos];
            ra = D.a[pos];
            rb = D.b[pos];
        }
        top -= n;
        __syncwarp();

        int act = 0;  // 1: split A, 2: split B, 3: leaf pair
        uint32_t child = 0, offA = 0, offB = 0, cnt = 0;
        if (active) {
            const Mat4 M = load_mat(P.q + q);
            const Rec A = load_rec(P.recs, ra);
            const Rec B = load_rec(P.recs, rb);
            {
                const Box bb = xform_box(M, B.box);
                if (sat_rolled(A.box, bb)) {
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
            const uint32_t p0 = (top + 2u * r) & D.mask;
            const uint32_t p1 = (top + 2u * r + 1u) & D.mask;
            const uint32_t c_left = child, c_right = child + 1u;
            D.q[p0] = q;
            D.q[p1] = q;
            if (act == 1) {
                D.a[p0] = c_right;
                D.b[p0] = rb;
                D.a[p1] = c_left;
                D.b[p1] = rb;
            } else {
                D.a[p0] = ra;
                D.b[p0] = c_right;
                D.a[p1] = ra;
                D.b[p1] = c_left;
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
        if (lane == 0) {
            st_nodes += n;
            ++st_steps;
            if (P.trace) {
                const unsigned long long b = (gtimer() - t_base) / P.trace_ns;
                if (b < kTraceBuckets) {
                    atomicAdd(P.trace + 4 * b, n);
                    atomicAdd(P.trace + 4 * b + 1, 1u);
                }
            }
        }
        __syncwarp();

        if (nl >= P.leaf_flush || (top == bot && nl > 0)) {
            flush_leafs(P, L, nl, lane, st_tests, st_frag, t_base);
            nl = 0;
        }

        // ---- balance: give half of the bottom of the deque to waiting warps
        // (all of a chunk when the deque is nearly full), or top up from
        // published chunks when fewer than 32 node pairs are left.
        const uint32_t held = top - bot;
        const bool forced = held + 64u > S;
        int mode = 0;  // 1: donate k, 2: top up from slot
        uint32_t k = 0, base = 0, slot = 0;
        if (lane == 0) {
            const bool waiting = int(ht_tail(qs) - ht_head(qs)) < 0;
            if (forced || (waiting && held >= P.donate_min)) {
                k = forced ? 32u : min(32u, held >> 1);
                const unsigned pt = ld_relaxed(&P.ctr->pool_tail);
                if (pt + k <= P.pool_cap && ht_tail(qs) - P.n_queries < P.slot_cap) {
                    atomicAdd(&P.ctr->work, 1u);
                    base = atomicAdd(&P.ctr->pool_tail, k);
                    slot = ht_tail(atomicAdd(ht, 1ull << 32));
                    mode = 1;
                } else if (forced) {
                    atomicOr(&P.ctr->error, ERR_QUEUE);
                    mode = -1;
                }
            } else if (held < 32u && held > 0u && !waiting) {
                if (try_claim(P, qs, slot)) mode = wait_ready(P, slot) ? 2 : -1;
            }
        }
        mode = __shfl_sync(kFull, mode, 0);
        if (mode == -1) break;
        if (mode == 1) {
            k = __shfl_sync(kFull, k, 0);
            base = __shfl_sync(kFull, base, 0);
            slot = __shfl_sync(kFull, slot, 0);
            if (uint32_t(lane) < k) {
                const uint32_t pos = (bot + lane) & D.mask;
                P.pool[base + lane] = make_uint4(D.q[pos], D.a[pos], D.b[pos], 0u);
            }
            __threadfence();
            __syncwarp();
            if (lane == 0) {
                P.slots[slot - P.n_queries] = make_uint2(base, k);
                st_release(P.ready + (slot - P.n_queries), 1u);
                st_don += k;
            }
            bot += k;
            __syncwarp();
        } else if (mode == 2) {
            slot = __shfl_sync(kFull, slot, 0);
            top += take_chunk(P, slot, D, top, lane);
            ++held_tasks;
        }

        if (top == bot) {
            if (lane == 0) atomicSub(&P.ctr->work, held_tasks);
            held_tasks = 0;
        }
    }

    if (lane == 0) {
        atomicAdd(&P.ctr->node_pairs, st_nodes);
        atomicAdd(&P.ctr->tri_tests, st_tests);
        atomicAdd(&P.ctr->fragile, st_frag);
        atomicAdd(&P.ctr->donations, st_don);
        atomicAdd(&P.ctr->warp_steps, st_steps);
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
    const bool ok = Q.tree_a < n_trees && Q.tree_b < n_trees && trees[Q.tree_a].live && trees[Q.tree_b].live;
    if (ok) {
        p.root_a = trees[Q.tree_a].rec_base + 1u;
        p.root_b = trees[Q.tree_b].rec_base + 1u;
        p.tri_base_a = trees[Q.tree_a].tri_base;
        p.tri_base_b = trees[Q.tree_b].tri_base;
    } else {
        p.root_a = p.root_b = p.tri_base_a = p.tri_base_b = 0u;
        atomicOr(&ctr->error, ERR_BAD_QUERY);
    }
    out[i] = p;
}

// Resets the counters for a launch over n_queries and clears the ready flags
// of the slots the previous launch published (their count is still in the
// counters).
__global__ void init_kernel(Counters* ctr, unsigned int* ready, uint32_t slot_alloc, uint32_t n_queries,
                            unsigned int* trace) {
    __shared__ uint32_t used;
    if (threadIdx.x == 0) {
        const unsigned long long ht = *reinterpret_cast<unsigned long long*>(&ctr->head);
        const uint32_t tail = uint32_t(ht >> 32);
        const uint32_t prev_n = ctr->n_queries;
        used = tail > prev_n ? min(tail - prev_n, slot_alloc) : 0u;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < used; i += blockDim.x) ready[i] = 0u;
    if (trace)
        for (uint32_t i = threadIdx.x; i < 4u * kTraceBuckets; i += blockDim.x) trace[i] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
        Counters c = {};
        c.tail = n_queries;
        c.work = n_queries;
        c.n_queries = n_queries;
        *ctr = c;
    }
}

// Paralgram::GetSurface of records [first, first + n_recs), written into q3.z.
__global__ void surfaces_kernel(float4* recs, uint32_t first, uint32_t n_recs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_recs) return;
    const uint32_t r = first + i;
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

cudaError_t launch_init(Counters* ctr, unsigned int* ready, uint32_t slot_alloc, uint32_t n_queries,
                        unsigned int* trace, cudaStream_t s) {
    init_kernel<<<1, 1024, 0, s>>>(ctr, ready, slot_alloc, n_queries, trace);
    return cudaGetLastError();
}

cudaError_t launch_surfaces(float4* recs, uint32_t first, uint32_t n_recs, cudaStream_t s) {
    if (n_recs == 0) return cudaSuccess;
    surfaces_kernel<<<(n_recs + 255) / 256, 256, 0, s>>>(recs, first, n_recs);
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
