// Collision kernels for sm_103a: query packing, counter reset, record surfaces,
// the persistent warp-cooperative OBB-tree traversal, and the persistent
// triangle-pair (Moller) narrow phase.
//
// Traversal. Each warp owns a node-pair deque in shared memory and advances up
// to 32 node pairs per step, one per lane: load both box records (four
// 16-byte loads each) and the query's matrix in parallel, move B's box into
// A's space, run the 15-axis SAT (three independent axes at a time), and apply
// the reference's descent rule (OBBtree::IntersectOBBtreesRecursive,
// src/Geometry/OBBtree.cpp:414-476): two inner nodes -> split the one with the
// larger surface, ties to the first tree; one leaf -> split the other; two
// leaves -> a candidate leaf pair. Surviving child pairs are pushed with
// __ballot_sync/__popc compaction; candidate leaf pairs are buffered per warp
// and appended to a global list in batches.
//
// Load balance uses a global task queue. Tasks are chunks of up to 32 node
// pairs; the root pairs of all queries are the first slots. A warp whose deque
// runs dry claims the next slot and waits for it; a warp with fewer than 32
// node pairs tops up with already reserved slots; a warp with surplus gives
// half of the bottom (shallowest) part of its deque to waiting warps, with one
// atomic per donation. Every wait is bounded by wait_ns (globaltimer), after
// which the kernel records ERR_TIMEOUT and returns.
//
// Narrow phase. Each warp takes 32 leaf pairs of the list at a time and runs
// their triangle pairs, one pair per lane.
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned kPollSleepMaxNs = 256;  // longest sleep of a waiting warp between two looks at its slot

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
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// head in the low 32 bits, tail in the high 32 bits.
__device__ __forceinline__ unsigned long long* ht_of(Counters* c) {
    return reinterpret_cast<unsigned long long*>(&c->head);
}
__device__ __forceinline__ uint32_t ht_head(unsigned long long v) { return uint32_t(v); }
__device__ __forceinline__ uint32_t ht_tail(unsigned long long v) { return uint32_t(v >> 32); }

// True once every reserved task has finished. `done` is read (acquire)
// before the tail: done(t1) == tail(t2) with t1 < t2 implies no task was
// running at t1 and none could be reserved afterwards.
__device__ __forceinline__ bool all_done(Counters* c) {
    const unsigned d = ld_acquire(&c->done);
    return d == ht_tail(ld_relaxed64(ht_of(c)));
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

// Round g of the 15 axes of cg::sat (same axes, same order, same arithmetic):
// g = 0 a's faces, 1 b's faces, 2..4 a_u|a_v|a_w x b_u, b_v, b_w.
__device__ __forceinline__ bool sat_round(const Box& a, const Box& b, int g) {
    float3 x0, y0, x1, y1, x2, y2;
    if (g < 2) {
        const float3 u = g ? b.u : a.u;
        const float3 v = g ? b.v : a.v;
        const float3 w = g ? b.w : a.w;
        x0 = v;
        y0 = w;
        x1 = u;
        y1 = w;
        x2 = u;
        y2 = v;
    } else {
        const float3 e = g == 2 ? a.u : (g == 3 ? a.v : a.w);
        x0 = e;
        y0 = b.u;
        x1 = e;
        y1 = b.v;
        x2 = e;
        y2 = b.w;
    }
    const bool ok0 = overlap_on(a, b, cross3(x0, y0));
    const bool ok1 = overlap_on(a, b, cross3(x1, y1));
    const bool ok2 = overlap_on(a, b, cross3(x2, y2));
    return ok0 & ok1 & ok2;
}

// Two box-pair SATs side by side, round by round, for instruction-level
// parallelism; each verdict is the conjunction of its 15 axes, identical to
// cg::sat.
__device__ __forceinline__ void sat_two(const Box& a0, const Box& b0, const Box& a1, const Box& b1, bool& ok0,
                                        bool& ok1) {
    bool al0 = ok0, al1 = ok1;
#pragma unroll 1
    for (int g = 0; g < 5 && (al0 | al1); ++g) {
        const bool r0 = sat_round(a0, b0, g);
        const bool r1 = sat_round(a1, b1, g);
        al0 = al0 & r0;
        al1 = al1 & r1;
    }
    ok0 = al0;
    ok1 = al1;
}

// Axis k (0..14) of the SAT in the reference's order: a's face normals
// (v x w, u x w, u x v), b's, then a_i x b_j; true when the boxes overlap on
// it. The SAT verdict is the conjunction over k, whatever lanes compute it.
__device__ __forceinline__ bool sat_axis(const Box& a, const Box& b, uint32_t k) {
    float3 x, y;
    if (k < 6u) {
        const bool onA = k < 3u;
        const uint32_t f = onA ? k : k - 3u;
        const float3 u = onA ? a.u : b.u, v = onA ? a.v : b.v, w = onA ? a.w : b.w;
        x = f == 0u ? v : u;
        y = f == 2u ? v : w;
    } else {
        const uint32_t i = (k - 6u) / 3u, j = (k - 6u) % 3u;
        x = i == 0u ? a.u : (i == 1u ? a.v : a.w);
        y = j == 0u ? b.u : (j == 1u ? b.v : b.w);
    }
    return overlap_on(a, b, cross3(x, y));
}

// The reference descent rule (OBBtree.cpp:414-476) for a child pair whose
// boxes overlap: split the inner node with the larger box surface (the first
// tree's on ties), else the inner one, or report a leaf pair. C is the child
// record (record rc) of the split node, O the other box (record io), bx the
// child pair's box of the second tree as transformed for the SAT.
__device__ __forceinline__ void descend(const TraverseParams& P, bool sideB, const Rec& O, const Rec& C, uint32_t rc,
                                        uint32_t io, uint32_t qi, const Box& bx, bool& item, bool& leaf,
                                        uint32_t& out_q, uint32_t& out_s, uint32_t& out_o) {
    const uint32_t a_ref = sideB ? O.ref : C.ref;
    const uint32_t a_meta = sideB ? O.meta : C.meta;
    const float a_surf = sideB ? O.surf : C.surf;
    const uint32_t b_ref = sideB ? C.ref : O.ref;
    const uint32_t b_meta = sideB ? C.meta : O.meta;
    const uint32_t ra = sideB ? io : rc;
    const uint32_t rb = sideB ? rc : io;
    const bool la = (a_meta & kLeafFlag) != 0;
    const bool lb = (b_meta & kLeafFlag) != 0;
    int act;  // 1: split A, 2: split B, 3: leaf pair
    if (!la && !lb)
        act = (a_surf >= surface(bx)) ? 1 : 2;
    else if (la && !lb)
        act = 2;
    else if (!la && lb)
        act = 1;
    else
        act = 3;
    if (act == 3) {
        // leaf pair: first triangles of both leaves, counts packed
        leaf = true;
        out_s = a_ref;
        out_o = b_ref;
        out_q = (a_meta & 0xffffu) | ((b_meta & 0xffffu) << 16);
    } else {
        item = true;
        const uint32_t split = act == 1 ? a_ref : b_ref;
        out_q = act == 1 ? qi : (qi | kItemSideB);
        out_s = split;
        out_o = act == 1 ? rb : ra;
        // the split node's two child records share one 128-byte line: fetch
        // it into L1 for the step that tests them
        asm volatile("prefetch.global.L1 [%0];" ::"l"(P.recs + 4ull * split));
    }
}

struct Deque {
    uint32_t* q;
    uint32_t* a;
    uint32_t* b;
    uint32_t mask;
};

// Lane 0: one look at slot `slot`: 1 with r = its chunk size + 1 (2 for a
// root slot) when it can be read, 0 with r = 0
// when all work finished, an error was raised or the wait limit (counted
// from t0) passed, -1 when it is not ready yet.
__device__ int poll_ready(const TraverseParams& P, uint32_t slot, unsigned long long t0, unsigned& r) {
    r = 0;
    if (slot < P.n_queries) {
        r = 2u;
        return 1;
    }
    const uint32_t idx = slot - P.n_queries;
    if (idx < P.slot_alloc) {
        r = ld_acquire(P.ready + idx);
        if (r) return 1;
    }
    // past every slot a donor could publish, only the end of the work or an
    // error releases the warp
    if (all_done(P.ctr) || ld_relaxed(&P.ctr->error) != 0) return 0;
    if (gtimer() - t0 > P.wait_ns) {
        atomicOr(&P.ctr->error, ERR_TIMEOUT);
        return 0;
    }
    return -1;
}

// Copies the chunk of slot `slot` into the deque at `top` (all lanes); `r` is
// poll_ready's value. Returns the number of node pairs added.
__device__ uint32_t take_chunk(const TraverseParams& P, uint32_t slot, unsigned r, const Deque& D, uint32_t top,
                               int lane) {
    // Lane 0 observed the slot's release; the barrier orders the other lanes'
    // pool reads after that acquire.
    __syncwarp();
    uint32_t cnt = 0;
    if (slot >= P.n_queries) {
        cnt = r - 1u;
        if (uint32_t(lane) < cnt) {
            const uint4 e = ld_relaxed4(P.pool + size_t(kChunk) * (slot - P.n_queries) + lane);
            const uint32_t pos = (top + lane) & D.mask;
            D.q[pos] = e.x;
            D.a[pos] = e.y;
            D.b[pos] = e.z;
        }
    } else {
        // the first item of query `slot`, made by the pack kernel
        uint32_t iq = kNoItem;
        if (lane == 0) {
            const PackedQuery* Q = P.q + slot;
            iq = __ldg(&Q->item_q);
            if (iq != kNoItem) {
                const uint32_t pos = top & D.mask;
                D.q[pos] = iq;
                D.a[pos] = __ldg(&Q->item_split);
                D.b[pos] = __ldg(&Q->item_other);
            }
        }
        cnt = __shfl_sync(kFull, iq != kNoItem ? 1u : 0u, 0);
    }
    __syncwarp();
    return cnt;
}

__device__ __forceinline__ void trace_add(unsigned int* trace, uint32_t trace_ns, unsigned long long t_base, int field,
                                          unsigned v) {
    const unsigned long long b = (gtimer() - t_base) / trace_ns;
    if (b < kTraceBuckets) {
        atomicAdd(trace + 4 * b + field, v);
        atomicAdd(trace + 4 * b + field + 1, 1u);
    }
}

__device__ __forceinline__ unsigned long long trace_base(Counters* ctr) {
    const unsigned long long now = gtimer();
    const unsigned long long old = atomicCAS(&ctr->t_start, 0ull, now);
    return old ? old : now;
}

// The narrow phase of leaf pairs [first, first + nl) of the list (nl <= 32),
// staged in `stage` (kNarrowWarpWords words); all 32 lanes call it. The
// entries must be visible to the calling warp.
template <int kMode>
__device__ __forceinline__ void narrow_block(const NarrowParams& P, uint32_t* stage, uint32_t first, uint32_t nl,
                                             int lane, unsigned long long& tests, unsigned long long& fragile,
                                             unsigned long long& rechecked, unsigned long long& disagree,
                                             unsigned long long t_base) {
    uint32_t* lq = stage;
    uint32_t* loa = lq + 32;
    uint32_t* lob = loa + 32;
    uint32_t* lcn = lob + 32;
    uint32_t* lrc = lcn + 32;  // ceil(2^16 / count_b), or 0 where the division is done in full
    uint32_t* pre = lrc + 32;  // 33 entries
    uint32_t c0 = 0;
    if (uint32_t(lane) < nl) {
        const uint4 e = P.leaf_list[first + lane];
        lq[lane] = e.x;
        loa[lane] = e.y;
        lob[lane] = e.z;
        lcn[lane] = e.w;
        const uint32_t cb = e.w >> 16;
        c0 = (e.w & 0xffffu) * cb;
        // local / cb == (local * ceil(2^16 / cb)) >> 16 for local < 256, cb <= 16
        lrc[lane] = (cb <= 16u && c0 < 256u) ? (65536u + cb - 1u) / cb : 0u;
        if ((P.flags & CG_KEEP_LEAF_PAIRS) && first + lane < P.leafs_cap) {
            const PackedQuery* Q = P.q + e.x;
            cg_leaf_pair lp;
            lp.query = e.x;
            lp.offset_a = e.y - __ldg(&Q->tri_base_a);
            lp.offset_b = e.z - __ldg(&Q->tri_base_b);
            lp.count_a = uint16_t(e.w & 0xffffu);
            lp.count_b = uint16_t(e.w >> 16);
            P.leafs[first + lane] = lp;
        }
    }
    uint32_t s0 = c0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t0 = __shfl_up_sync(kFull, s0, o);
        if (lane >= o) s0 += t0;
    }
    const uint32_t total = (P.flags & CG_MID_ONLY) ? 0u : __shfl_sync(kFull, s0, 31);
    const uint32_t my_pre = s0 - c0;  // first test of this lane's leaf pair
    pre[lane] = my_pre;
    if (lane == 0) pre[32] = total;
    __syncwarp();

    // The leaf pair of test t: each round, the leaf pairs that start inside
    // the round's 32 tests set their bit, and a lane counts the starts at or
    // below it from the leaf pair that holds the round's first test. A leaf
    // pair without tests (an empty leaf) starts where the next one does; a
    // block with one looks the leaf pair up by binary search instead.
    const bool counted = __all_sync(kFull, uint32_t(lane) >= nl || c0 != 0u);
    uint32_t own0 = 0;
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t t = base + lane;
        const int d = int(my_pre) - int(base);
        const bool mine = uint32_t(lane) < nl;
        const unsigned starts = __reduce_or_sync(kFull, (mine && d >= 1 && d <= 31) ? (1u << d) : 0u);
        const bool next_at_32 = __any_sync(kFull, mine && d == 32);
        uint32_t lo = own0 + __popc(starts & ((2u << lane) - 1u));
        own0 += __popc(starts) + (next_at_32 ? 1u : 0u);
        int res = TT_MISS;
        uint32_t q = 0, ia = 0, ib = 0, leaf_i = 0;
        float3 src = make_float3(0.f, 0.f, 0.f), tgt = src;
        Recheck rck;
        if (t < total) {
            if (!counted) {
                int l = 0, h = int(nl) - 1;
                while (l < h) {
                    const int mid = (l + h + 1) >> 1;
                    if (pre[mid] <= t)
                        l = mid;
                    else
                        h = mid - 1;
                }
                lo = uint32_t(l);
            }
            const uint32_t local = t - pre[lo];
            const uint32_t cn = lcn[lo];
            const uint32_t cb = cn >> 16;
            const uint32_t rc = lrc[lo];
            const uint32_t i = rc ? (local * rc) >> 16 : local / cb;
            const uint32_t j = local - i * cb;
            q = lq[lo];
            leaf_i = first + uint32_t(lo);
            ia = loa[lo] + i;
            ib = lob[lo] + j;
            const Mat4 M = load_mat(P.q + q);
            float3 a0, a1, a2, b0, b1, b2;
            load_tri(P.tris, ia, a0, a1, a2);
            load_tri(P.tris, ib, b0, b1, b2);
            b0 = xform(M, b0, 1.0f);
            b1 = xform(M, b1, 1.0f);
            b2 = xform(M, b2, 1.0f);
            res = tri_tri_mode<kMode>(a0, a1, a2, b0, b1, b2, src, tgt, rck);
        }
        const unsigned hitmask = __ballot_sync(kFull, res == TT_HIT);
        const unsigned fragmask = __ballot_sync(kFull, res == TT_FRAGILE);
        if (kMode != 0) {
            const unsigned nchk = __reduce_add_sync(kFull, rck.checked);
            const unsigned ndis = __popc(__ballot_sync(kFull, rck.disagree));
            if (lane == 0) {
                rechecked += nchk;
                disagree += ndis;
            }
        }
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
                    if (P.pair_aux) P.pair_aux[o] = make_uint4(ia, ib, leaf_i, q);
                }
            }
        }
        if (lane == 0) {
            fragile += __popc(fragmask);
            if (P.trace) trace_add(P.trace, P.trace_ns, t_base, 2, min(32u, total - base));
        }
    }
    if (lane == 0) tests += total;
    __syncwarp();
}

// Appends the warp's buffered leaf pairs to the list.
__device__ __forceinline__ void flush_leafs(const TraverseParams& P, const uint32_t* lq, const uint32_t* loa,
                                            const uint32_t* lob, const uint32_t* lcn, uint32_t nl, int lane) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&P.ctr->n_leafs, (unsigned long long)nl);
    base = __shfl_sync(kFull, base, 0);
    for (uint32_t e = lane; e < nl; e += 32)
        if (base + e < P.leaf_cap) P.leaf_list[base + e] = make_uint4(lq[e], loa[e], lob[e], lcn[e]);
    __syncwarp();
}

}  // namespace

__global__ void __launch_bounds__(256, 2) traverse_kernel(const TraverseParams P) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const uint32_t S = P.stack_cap;
    Deque D;
    D.q = smem + size_t(warp) * warp_smem_words(S);
    D.a = D.q + S;
    D.b = D.a + S;
    D.mask = S - 1u;
    uint32_t* lq = D.b + S;
    uint32_t* loa = lq + kLeafCap;
    uint32_t* lob = loa + kLeafCap;
    uint32_t* lcn = lob + kLeafCap;
    unsigned long long* ht = ht_of(P.ctr);

    uint32_t top = 0, bot = 0, nl = 0, held_tasks = 0;
    unsigned long long st_nodes = 0, st_don = 0, st_steps = 0;
    unsigned long long t_base = 0;
    if (P.trace && lane == 0) t_base = trace_base(P.ctr);

    for (;;) {
        if (top == bot) {
            // Out of work: claim the next slot and wait for it (the whole
            // warp polls; lane 0 looks and sleeps between looks).
            uint32_t slot = 0;
            if (lane == 0) slot = ht_head(atomicAdd(ht, 1ull));
            slot = __shfl_sync(kFull, slot, 0);
            unsigned r = 0;
            unsigned long long t0 = 0;
            unsigned ns = 32;
            for (;;) {
                int st = 0;
                if (lane == 0) {
                    if (!t0) t0 = gtimer();
                    st = poll_ready(P, slot, t0, r);
                }
                st = __shfl_sync(kFull, st, 0);
                if (st >= 0) break;
                if (lane == 0) {
                    __nanosleep(ns);
                    if (ns < kPollSleepMaxNs) ns <<= 1;
                }
                __syncwarp();
            }
            r = __shfl_sync(kFull, r, 0);
            if (!r) break;
            top += take_chunk(P, slot, r, D, top, lane);
            held_tasks = 1;
        }

        // Queue state, read early so its latency overlaps the step's loads.
        unsigned long long qs = 0;
        if (lane == 0) qs = ld_relaxed64(ht);

        // ---- one step over up to 32 items from the top of the deque. An item
        // tests both children of a split node against the other box: the
        // other record is loaded (and, for the second tree, transformed) once,
        // the two child records come from one 128-byte line. With more than
        // 16 items a lane runs an item's two SATs side by side; with fewer,
        // 2 L lanes share an item, L per child (L = 1, 2, 4, 8, 16 for 9-16,
        // 5-8, 3-4, 2 and 1 items), each taking every L-th of the child's 15
        // axes, so that a step with few items (the ramp and the tail of a
        // launch, where the deepest queries' chains of dependent steps set
        // the time) takes less time. Every verdict is the conjunction of the
        // same 15 axes.
        const uint32_t size = top - bot;
        const uint32_t n = size < 32u ? size : 32u;
        // log2 of lanes per item
        const uint32_t lg = n <= 1u ? 5u : (n <= 2u ? 4u : (n <= 4u ? 3u : (n <= 8u ? 2u : (n <= 16u ? 1u : 0u))));
        const uint32_t slot_i = uint32_t(lane) >> lg;
        const uint32_t sub = uint32_t(lane) & ((1u << lg) - 1u);
        const bool active = slot_i < n;
        uint32_t iq = 0, is = 0, io = 0;
        if (active) {
            const uint32_t pos = (top - n + slot_i) & D.mask;
            iq = D.q[pos];
            is = D.a[pos];
            io = D.b[pos];
        }
        top -= n;
        __syncwarp();

        // Per lane, per child k: a new item (split node, other record, query
        // word) or a candidate leaf pair (triangle offsets and counts).
        bool item[2] = {false, false}, leaf[2] = {false, false};
        uint32_t out_q[2] = {0, 0}, out_s[2] = {0, 0}, out_o[2] = {0, 0};
        const uint32_t qi = iq & ~kItemSideB;
        const bool sideB = (iq & kItemSideB) != 0;
        if (lg == 0u) {
            if (active) {
                const Mat4 M = load_mat(P.q + qi);
                const Rec O = load_rec(P.recs, io);
                const Rec C0 = load_rec(P.recs, is);
                const Rec C1 = load_rec(P.recs, is + 1u);
                Box a0, a1, b0, b1;
                if (sideB) {
                    a0 = O.box;
                    a1 = O.box;
                    b0 = xform_box(M, C0.box);
                    b1 = xform_box(M, C1.box);
                } else {
                    a0 = C0.box;
                    a1 = C1.box;
                    b0 = xform_box(M, O.box);
                    b1 = b0;
                }
                bool ok[2] = {true, true};
                sat_two(a0, b0, a1, b1, ok[0], ok[1]);
                if (ok[0]) descend(P, sideB, O, C0, is, io, qi, b0, item[0], leaf[0], out_q[0], out_s[0], out_o[0]);
                if (ok[1]) descend(P, sideB, O, C1, is + 1u, io, qi, b1, item[1], leaf[1], out_q[1], out_s[1], out_o[1]);
            }
        } else {
            const uint32_t lc = lg - 1u;               // log2 of lanes per child
            const uint32_t kc = sub >> lc;             // the child this lane tests
            const uint32_t ax0 = sub & ((1u << lc) - 1u);  // its first axis; it takes every (1 << lc)-th
            bool ok = true;
            Rec O, C;
            Box bx;
            if (active) {
                const Mat4 M = load_mat(P.q + qi);
                O = load_rec(P.recs, io);
                C = load_rec(P.recs, is + kc);
                const Box ax = sideB ? O.box : C.box;
                bx = xform_box(M, sideB ? C.box : O.box);
#pragma unroll 1
                for (uint32_t k = ax0; k < 15u && ok; k += 1u << lc) ok = sat_axis(ax, bx, k);
            }
            // the child's verdict: no lane of its group found a separating axis
            const unsigned fail = __ballot_sync(kFull, !ok);
            const unsigned group = (lc == 4u ? 0xffffu : ((1u << (1u << lc)) - 1u)) << (uint32_t(lane) & ~((1u << lc) - 1u));
            ok = (fail & group) == 0u;
            if (active && ok && ax0 == 0u)
                descend(P, sideB, O, C, is + kc, io, qi, bx, item[0], leaf[0], out_q[0], out_s[0], out_o[0]);
        }

        const unsigned i0 = __ballot_sync(kFull, item[0]), i1 = __ballot_sync(kFull, item[1]);
        {
            const unsigned lt = lanemask_lt();
            uint32_t r = __popc(i0 & lt) + __popc(i1 & lt);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (item[k]) {
                    const uint32_t p = (top + r) & D.mask;
                    D.q[p] = out_q[k];
                    D.a[p] = out_s[k];
                    D.b[p] = out_o[k];
                    ++r;
                }
            }
        }
        top += __popc(i0) + __popc(i1);

        const unsigned l0 = __ballot_sync(kFull, leaf[0]), l1 = __ballot_sync(kFull, leaf[1]);
        {
            const unsigned lt = lanemask_lt();
            uint32_t r = nl + __popc(l0 & lt) + __popc(l1 & lt);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (leaf[k]) {
                    lq[r] = qi;
                    loa[r] = out_s[k];
                    lob[r] = out_o[k];
                    lcn[r] = out_q[k];
                    ++r;
                }
            }
        }
        nl += __popc(l0) + __popc(l1);
        if (lane == 0) {
            st_nodes += 2u * n;
            ++st_steps;
            if (P.trace) trace_add(P.trace, P.trace_ns, t_base, 0, n);
        }
        __syncwarp();

        if (nl >= P.leaf_flush) {
            flush_leafs(P, lq, loa, lob, lcn, nl, lane);
            nl = 0;
        }

        // ---- balance: give chunks from the bottom of the deque to the warps
        // that wait (one chunk per waiting warp, up to 8, keeping at least a
        // chunk; a full chunk when the deque is nearly full). A warp does not
        // take queued chunks while it has work: that costs a contended atomic
        // per step and measured slower.
        const uint32_t held = top - bot;
        const bool forced = held + 64u > S;
        int mode = 0;  // 1: donate nch chunks of c
        uint32_t c = 0, nch = 0, slot = 0;
        if (lane == 0) {
            const int waiting = int(ht_head(qs) - ht_tail(qs));
            if (forced || (waiting > 0 && held >= P.donate_min)) {
                c = held >= 2u * kChunk ? uint32_t(kChunk) : (held >> 1);
                nch = min(uint32_t(waiting > 0 ? waiting : 1), min(held / c - 1u, 8u));
                if (nch == 0) nch = 1;
                if (ht_tail(qs) - P.n_queries + nch <= P.slot_cap) {
                    slot = ht_tail(atomicAdd(ht, (unsigned long long)nch << 32));
                    mode = 1;
                } else if (forced) {
                    atomicOr(&P.ctr->error, ERR_QUEUE);
                    mode = -1;
                }
            }
        }
        mode = __shfl_sync(kFull, mode, 0);
        if (mode == -1) break;
        if (mode == 1) {
            c = __shfl_sync(kFull, c, 0);
            nch = __shfl_sync(kFull, nch, 0);
            slot = __shfl_sync(kFull, slot, 0);
            const uint32_t idx0 = slot - P.n_queries;
            for (uint32_t ch = 0; ch < nch; ++ch) {
                if (uint32_t(lane) < c) {
                    const uint32_t pos = (bot + ch * c + lane) & D.mask;
                    P.pool[size_t(kChunk) * (idx0 + ch) + lane] = make_uint4(D.q[pos], D.a[pos], D.b[pos], 0u);
                }
            }
            __threadfence();
            __syncwarp();
            if (uint32_t(lane) < nch) st_release(P.ready + idx0 + lane, c + 1u);
            if (lane == 0) st_don += c * nch;
            bot += c * nch;
            __syncwarp();
        }

        if (top == bot) {
            if (lane == 0) atomicAdd(&P.ctr->done, held_tasks);
            held_tasks = 0;
        }
    }

    // remaining buffered leaf pairs
    if (nl) flush_leafs(P, lq, loa, lob, lcn, nl, lane);
    if (lane == 0) {
        if (st_nodes) atomicAdd(&P.ctr->node_pairs, st_nodes);
        if (st_don) atomicAdd(&P.ctr->donations, st_don);
        if (st_steps) atomicAdd(&P.ctr->warp_steps, st_steps);
    }
}

// Runs the triangle pairs of the leaf-pair list, 32 leaf pairs per warp and
// one triangle pair per lane, in the order of the reference's pair loop per
// leaf pair (CreateUncollideRays.cpp:78-86): B's triangle is moved into A's
// space with TrianglePosition::MultiplyBy4x4Matrix arithmetic, then tested.
template <int kMode>
__global__ void __launch_bounds__(256, 3) narrow_kernel(const NarrowParams P) {
    __shared__ uint32_t sm[8 * kNarrowWarpWords];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    uint32_t* stage = sm + warp * kNarrowWarpWords;

    const unsigned long long n_all = *reinterpret_cast<volatile unsigned long long*>(&P.ctr->n_leafs);
    const uint32_t n = uint32_t(n_all < P.leaf_cap ? n_all : P.leaf_cap);
    unsigned long long tests = 0, fragile = 0, rechecked = 0, disagree = 0;
    unsigned long long t_base = 0;
    if (P.trace && lane == 0) t_base = trace_base(P.ctr);

    // Each warp's first `per` leaf pairs are fixed by its index; later ones
    // come from the shared counter, past all first rounds. A small list
    // costs no atomic to the warps it does not reach, and is spread over all
    // warps (per < 32 leaf pairs each) so that its rounds run side by side.
    const uint32_t n_warps = gridDim.x * (blockDim.x >> 5);
    const uint32_t per = n >= 32u * n_warps ? 32u : max(1u, (n + n_warps - 1u) / n_warps);
    uint32_t first = per * (blockIdx.x * (blockDim.x >> 5) + uint32_t(warp));
    while (first < n) {
        const uint32_t nl = min(per, n - first);
        narrow_block<kMode>(P, stage, first, nl, lane, tests, fragile, rechecked, disagree, t_base);
        uint32_t next = 0;
        if (lane == 0) next = per * n_warps + atomicAdd(&P.ctr->narrow_lp, per);
        first = __shfl_sync(kFull, next, 0);
    }
    if (lane == 0) {
        if (tests) atomicAdd(&P.ctr->tri_tests, tests);
        if (fragile) atomicAdd(&P.ctr->fragile, fragile);
        if (kMode != 0) {
            if (rechecked) atomicAdd(&P.ctr->rechecked, rechecked);
            if (disagree) atomicAdd(&P.ctr->disagreements, disagree);
        }
    }
}

// One thread per query: packs the relative matrix and runs the root pair the
// way the traversal runs every pair (SAT, then the descent rule), so that the
// query enters the work queue as its first item; a leaf-leaf root goes
// straight to the leaf-pair list.
__global__ void pack_kernel(const cg_query* in, uint32_t n, const DevTree* trees, uint32_t n_trees,
                            const float4* recs, PackedQuery* out, Counters* ctr, uint4* leaf_list, uint32_t leaf_cap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cg_query Q = in[i];
    PackedQuery p;
    p.m[0] = make_float4(Q.relative[0], Q.relative[1], Q.relative[2], Q.relative[3]);
    p.m[1] = make_float4(Q.relative[4], Q.relative[5], Q.relative[6], Q.relative[7]);
    p.m[2] = make_float4(Q.relative[8], Q.relative[9], Q.relative[10], Q.relative[11]);
    p.m[3] = make_float4(Q.relative[12], Q.relative[13], Q.relative[14], Q.relative[15]);
    p.item_q = kNoItem;
    p.item_split = p.item_other = p.pad = 0u;
    p.tri_base_a = p.tri_base_b = 0u;
    p.tree_a = Q.tree_a;
    p.tree_b = Q.tree_b;
    const bool ok = Q.tree_a < n_trees && Q.tree_b < n_trees && trees[Q.tree_a].live && trees[Q.tree_b].live;
    if (!ok) {
        atomicOr(&ctr->error, ERR_BAD_QUERY);
        out[i] = p;
        return;
    }
    p.tri_base_a = trees[Q.tree_a].tri_base;
    p.tri_base_b = trees[Q.tree_b].tri_base;
    const uint32_t ra = trees[Q.tree_a].rec_base + 1u;
    const uint32_t rb = trees[Q.tree_b].rec_base + 1u;
    const Mat4 M{p.m[0], p.m[1], p.m[2], p.m[3]};
    const Rec A = load_rec(recs, ra);
    const Rec B = load_rec(recs, rb);
    const Box bb = xform_box(M, B.box);
    {
        // one atomic per group of converged lanes
        const unsigned m = __activemask();
        if ((threadIdx.x & 31u) == unsigned(__ffs(m) - 1)) atomicAdd(&ctr->node_pairs, (unsigned long long)__popc(m));
    }
    if (sat(A.box, bb)) {
        const bool la = (A.meta & kLeafFlag) != 0;
        const bool lb = (B.meta & kLeafFlag) != 0;
        if (la && lb) {
            const unsigned long long idx = atomicAdd(&ctr->n_leafs, 1ull);
            if (idx < leaf_cap) leaf_list[idx] = make_uint4(i, A.ref, B.ref, (A.meta & 0xffffu) | ((B.meta & 0xffffu) << 16));
        } else {
            const bool split_a = (!la && !lb) ? (A.surf >= surface(bb)) : !la;
            p.item_q = split_a ? i : (i | kItemSideB);
            p.item_split = split_a ? A.ref : B.ref;
            p.item_other = split_a ? rb : ra;
        }
    }
    out[i] = p;
}

// Resets the counters for a launch over n_queries and clears the ready flags
// of the slots the previous launch reserved (their count is still in the
// counters), and the trace when it is kept.
__global__ void init_kernel(Counters* ctr, unsigned int* ready, uint32_t slot_alloc, uint32_t n_queries,
                            unsigned int* trace) {
    __shared__ uint32_t used;
    if (threadIdx.x == 0) {
        const uint32_t tail = ctr->tail;
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
        c.n_queries = n_queries;
        // vertex-set slots stay taken until a contacts launch empties them
        c.prev_vertices = ctr->prev_vertices + ctr->n_vertices;
        *ctr = c;
    }
}

// Paralgram::GetSurface of records [first, first + n_recs), written into q3.z.
__global__ void surfaces_kernel(float4* recs, uint32_t first, uint32_t n_recs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_recs) return;
    float4* p = recs + 4ull * (first + i);
    const float4 a = p[0], b = p[1], c = p[2];
    Box box;
    box.c = make_float3(a.x, a.y, a.z);
    box.u = make_float3(a.w, b.x, b.y);
    box.v = make_float3(b.z, b.w, c.x);
    box.w = make_float3(c.y, c.z, c.w);
    p[3].z = surface(box);
}

cudaError_t launch_pack(const cg_query* in, uint32_t n, const DevTree* trees, uint32_t n_trees, const float4* recs,
                        PackedQuery* out, Counters* ctr, uint4* leaf_list, uint32_t leaf_cap, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    pack_kernel<<<(n + 127) / 128, 128, 0, s>>>(in, n, trees, n_trees, recs, out, ctr, leaf_list, leaf_cap);
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

cudaError_t narrow_occupancy(uint32_t warps_per_block, int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, narrow_kernel<0>, int(32 * warps_per_block), 0);
}

cudaError_t launch_traverse(const TraverseParams& p, uint32_t blocks, uint32_t warps_per_block, cudaStream_t s) {
    const size_t smem = size_t(warps_per_block) * warp_smem_words(p.stack_cap) * sizeof(uint32_t);
    traverse_kernel<<<blocks, 32 * warps_per_block, smem, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_narrow(const NarrowParams& p, uint32_t blocks, uint32_t warps_per_block, cudaStream_t s) {
    if (p.flags & CG_ROBUST)
        narrow_kernel<2><<<blocks, 32 * warps_per_block, 0, s>>>(p);
    else if (p.flags & CG_RECHECK)
        narrow_kernel<1><<<blocks, 32 * warps_per_block, 0, s>>>(p);
    else
        narrow_kernel<0><<<blocks, 32 * warps_per_block, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace cg
