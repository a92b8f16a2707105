// OBB-tree construction: OBBtree::OBBtree(vector<Triangle>&&)
// (src/Geometry/OBBtree.cpp:321-358) for a batch of meshes on the device, one
// tree level per round of launches, every node of every tree of the level at
// once.
//
// A node is a range of a triangle permutation; a split partitions its range
// in place (stably, as the reference's push_backs keep order), so every node's
// triangles stay in the reference's order. The box of a node is
// OBB::CreateOBBfromTriangles / CreateOBBfromPoints / CreateAABBfromPoints
// (src/Geometry/OBB.cpp:33-166). Its FP64 sums are sequential in the
// reference (std::accumulate, std::inner_product), so each is one thread's
// chain here; the FP64 pipe of this part is narrow, so everything around the
// chains runs a thread per corner on every SM:
//   build_points  a thread per triangle position: its corners as doubles
//   build_sums    a thread per node and coordinate: the sum in corner order,
//                 the mean
//   build_terms   a thread per triangle position: the six centred products
//                 of its corners
//   build_cov     a thread per node and product: the covariance sum in
//                 corner order (build_cov_big: a warp per node of more
//                 than kBuildBig triangles)
//   build_eig     a thread per node: eig3 of the covariance in FP64; the
//                 box axes are the rows of the eigenvector matrix
//   build_proj    a thread per triangle position: its corners' FP64
//                 projections on its node's axes
//   build_fit     a warp per node of more than 16 triangles (build_fit_small:
//                 a thread per smaller node; build_fit_big: a block per node
//                 of more than kBuildBig): fewer than two distinct corners
//                 give the empty or point box; else the min/max projections
//                 (integer keys of the doubles; equal values: the later
//                 corner, as the sequential std::min / std::max keep) and the
//                 box; then, for a node of more than 4 triangles,
//                 OBBtreeSplitBuildNode::SplitOBBandCreateChildren
//                 (OBBtree.cpp:43-108): axes by half-length, longest first
//                 (equal lengths keep u, v, w order); left when the mean of a
//                 triangle's projection interval is <= the centre's
//                 projection; the first axis leaving both sides non-empty,
//                 else halves by position; the two children appended to the
//                 node table for the next level
// Built with no contraction, IEEE division and square root, the boxes are the
// reference builder's bits. Then the trees' pre-order layout
// (OBBtree.cpp:179-233, 385-394), the larger-surface child first
// (OBBtree.cpp:100-106), goes straight into the context's arenas:
//   build_inner   bottom-up by level: the inner nodes of each subtree
//   build_order   top-down by level: each node's pre-order index, first
//                 triangle, leaf ordinal and record
//   build_emit    a thread per node: its record (box, links), subtree range,
//                 parent and leaf-list entry; a thread per triangle: the
//                 triangle (and its corner normals) at its leaf's place
// The meshes' triangles are gathered from their vertex and index buffers on
// the device (build_gather) before the first level.
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include "cg_device.cuh"
#include "cg_eig.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr unsigned kAll = 0xffffffffu;
constexpr uint32_t kLeafMax = 4;  // OBBtree.h:49 maxNumberOfTriangles
constexpr uint32_t kBigWarps = 16;  // warps of the block that handles one node of more than kBuildBig triangles

__device__ __forceinline__ float3 corner(const float* P, uint32_t t, uint32_t k) {
    const float* q = P + 9ull * t + 3u * k;
    return make_float3(q[0], q[1], q[2]);
}

// An order-preserving integer key of a double for min/max on the integer
// pipe (this part's FP64 pipe is narrow); both zeros key 0, as they compare
// equal.
__device__ __forceinline__ long long dkey(double x) {
    const long long b = __double_as_longlong(x);
    return (b & 0x7fffffffffffffffll) == 0 ? 0ll : (b >= 0 ? b : b ^ 0x7fffffffffffffffll);
}

// One projection extreme: its key, value and corner position.
struct Ext {
    long long k;
    double v;
    uint32_t j;
};

// std::min(pr, lo) / std::max(pr, hi) as the sequential scan applies them:
// an equal value replaces (the later corner is kept).
__device__ __forceinline__ void take_lo(Ext& e, long long k, double v, uint32_t j) {
    if (k <= e.k) e = Ext{k, v, j};
}
__device__ __forceinline__ void take_hi(Ext& e, long long k, double v, uint32_t j) {
    if (k >= e.k) e = Ext{k, v, j};
}

// The warp's extreme: the smaller key (lo) or the larger (hi); of equal keys
// the later corner.
__device__ __forceinline__ void warp_extreme(Ext& e, bool lo) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const long long ok = __shfl_xor_sync(kAll, e.k, o);
        const double ov = __shfl_xor_sync(kAll, e.v, o);
        const uint32_t oj = __shfl_xor_sync(kAll, e.j, o);
        if ((lo ? ok < e.k : ok > e.k) || (ok == e.k && oj > e.j)) e = Ext{ok, ov, oj};
    }
}

// The corners of the level's triangles at their triangle's position: as
// doubles by coordinate, and as floats by position (so that a node reads its
// corners contiguously); a thread per position (positions of earlier levels'
// leaves are skipped).
__global__ void build_points_kernel(const BuildParams B) {
    const uint64_t n3 = 3ull * B.T;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < B.T; t += gridDim.x * blockDim.x) {
        const uint32_t o = B.own[t];
        if (o < B.lo || o >= B.hi) continue;
        const float* q = B.P + 9ull * B.perm[t];
        float* pp = B.Pp + 9ull * t;
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                B.D[c * n3 + 3ull * t + k] = double(q[3 * k + c]);
                pp[3 * k + c] = q[3 * k + c];
            }
    }
}

// Sum of x[0..n-1] in order, in FP64: the reference's std::accumulate. The
// adds are one dependent chain, and on this part each FP64 instruction holds
// the sub-partition's FP64 pipe for about 64 cycles, so the chain's pace is
// one add per FP64 instruction time if its terms are at hand: they are loaded
// 16 bytes (two terms) at a time, in blocks of kChainBlock, the next block in
// flight while the current one is added (a chain that starts off a 16-byte
// boundary takes its first term alone); then the tail, in order. Only the
// reference's terms are added (adding a 0 could turn a -0 into +0).
constexpr uint32_t kChainBlock = 64;
__device__ __forceinline__ double chain_sum(const double* x, uint32_t n) {
    double s = 0.0;
    if (n && (reinterpret_cast<uintptr_t>(x) & 15u)) {
        s = s + x[0];
        ++x;
        --n;
    }
    constexpr uint32_t H = kChainBlock / 2;
    const double2* x2 = reinterpret_cast<const double2*>(x);
    const uint32_t nb = n / kChainBlock;  // full blocks
    double2 a[H], b[H];
    if (nb > 0) {
#pragma unroll
        for (uint32_t k = 0; k < H; ++k) a[k] = __ldg(x2 + k);
    }
    uint32_t blk = 0;
    for (; blk + 2u <= nb; blk += 2u) {
        const double2* xb = x2 + size_t(blk) * H;
        // blocks four and five ahead into L2 (four 128-byte lines each): the
        // terms come from DRAM when a level's arrays outgrow L2
        if (blk + 6u <= nb) {
#pragma unroll
            for (uint32_t k = 0; k < 8u; ++k) asm volatile("prefetch.global.L2 [%0];" ::"l"(xb + 4u * H + 8u * k));
        }
#pragma unroll
        for (uint32_t k = 0; k < H; ++k) b[k] = __ldg(xb + H + k);
#pragma unroll
        for (uint32_t k = 0; k < H; ++k) {
            s = s + a[k].x;
            s = s + a[k].y;
        }
        if (blk + 2u < nb) {
#pragma unroll
            for (uint32_t k = 0; k < H; ++k) a[k] = __ldg(xb + 2u * H + k);
        }
#pragma unroll
        for (uint32_t k = 0; k < H; ++k) {
            s = s + b[k].x;
            s = s + b[k].y;
        }
    }
    if (blk < nb) {
#pragma unroll
        for (uint32_t k = 0; k < H; ++k) {
            s = s + a[k].x;
            s = s + a[k].y;
        }
        ++blk;
    }
    for (uint32_t j = blk * kChainBlock; j < n; ++j) s = s + x[j];
    return s;
}

// A thread per node and coordinate: the coordinate's sum over the node's
// corners in order (std::accumulate, OBB.cpp:53-55), then the mean.
__global__ void build_sums_kernel(const BuildParams B) {
    const uint64_t n3 = 3ull * B.T;
    const uint32_t total = 3u * (B.hi - B.lo);
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const uint32_t node = B.lo + g / 3u, c = g % 3u;
        const BuildNode& N = B.nodes[node];
        if (N.count > kBuildBig) continue;  // build_sums_big
        const uint32_t np = 3u * N.count;
        const double s = chain_sum(B.D + c * n3 + 3ull * N.begin, np);
        B.mom[9ull * (node - B.lo) + c] = np ? s / double(np) : 0.0;
    }
}

// The corner's coordinate (a float as a double, finite) as an integer count of
// 2^q, q at most its float ulp's exponent: exact (the shifted-out bits are
// zero) while the count fits 64 bits.
__device__ __forceinline__ long long units_of(double x, int q) {
    const long long b = __double_as_longlong(x);
    if ((b & 0x7fffffffffffffffll) == 0) return 0;
    const int sh = int((b >> 52) & 0x7ff) - 1023 - 52 - q;
    const long long m = (b & 0xfffffffffffffll) | (1ll << 52);
    const long long v = sh >= 0 ? (m << sh) : (m >> -sh);
    return b < 0 ? -v : v;
}

// Block-wide sum of a 64-bit value per thread; every thread gets the total,
// and `before` the sum over the threads before it.
template <uint32_t kWarps>
__device__ __forceinline__ long long block_scan_ll(long long v, long long* sh, long long& before) {
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(kAll, inc, o);
        if (lane >= uint32_t(o)) inc += t;
    }
    if (lane == 31u) sh[w] = inc;
    __syncthreads();
    long long wb = 0, total = 0;
    for (uint32_t k = 0; k < kWarps; ++k) {
        const long long t = sh[k];
        if (k < w) wb += t;
        total += t;
    }
    __syncthreads();
    before = wb + inc - v;
    return total;
}

// A NaN payload that no sum produces: the mean is left to a chain.
constexpr long long kChainDue = 0x7ff4c4a1d0e00000ll;

// Whether count * 2^q is a double: its significant bits span at most 53.
__device__ __forceinline__ bool fits_double(long long count) {
    if (count == 0) return true;
    const unsigned long long m = count < 0 ? 0ull - (unsigned long long)count : (unsigned long long)count;
    return (64 - __clzll((long long)m)) - (__ffsll((long long)m) - 1) <= 53;
}

// count rounded to a double's 53 significant bits, to nearest, ties to even
// (the sequential sum's add; count * 2^q stays in the normal range).
__device__ __forceinline__ long long round_double(long long count) {
    if (fits_double(count)) return count;
    const bool neg = count < 0;
    const unsigned long long m = neg ? 0ull - (unsigned long long)count : (unsigned long long)count;
    const int d = (64 - __clzll((long long)m)) - 53;
    unsigned long long k = m >> d;
    const unsigned long long rem = m & ((1ull << d) - 1ull), half = 1ull << (d - 1);
    if (rem > half || (rem == half && (k & 1ull))) ++k;
    const long long r = (long long)(k << d);
    return neg ? -r : r;
}

constexpr uint32_t kSumChunk = 32;   // consecutive terms a thread adds up at a time
constexpr uint32_t kSumRounds = 64;  // roundings replayed before a sum is left to the chain

// A block per node of the level's list of nodes of more than kBuildBig
// triangles: the coordinate sums of build_sums_kernel without the chain. The
// terms are floats, integer multiples of 2^q (q the smallest exponent of
// their ulps), so the sequential sum is replayed exactly in 64-bit integer
// counts of 2^q (the terms are bounded so that no running sum can overflow):
// the running sums from a start are computed in parallel, a tile of 32-term
// chunks at a time (chunk sums, their exclusive scan in shared memory, then
// each chunk's running sums term by term), up to the first one that is not a
// double. That add is the first that rounds; its rounded value is the next
// start. A sum that rounds more than kSumRounds times, or holds a non-finite
// term, is marked due (kChainDue) and summed by build_sums_due's chain.
__global__ void __launch_bounds__(kBigWarps * 32) build_sums_big_kernel(const BuildParams B) {
    constexpr uint32_t NT = kBigWarps * 32u;
    __shared__ int s_q[kBigWarps][3], s_e[kBigWarps][3];
    __shared__ long long s_sc[kBigWarps];
    __shared__ long long s_chunk[NT];
    __shared__ unsigned s_hit;
    __shared__ long long s_start;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    const uint64_t n3 = 3ull * B.T;
    for (uint32_t i = blockIdx.x; i < B.n_big; i += gridDim.x) {
        const uint32_t id = B.big[i];
        const BuildNode& N = B.nodes[id];
        const uint32_t np = 3u * N.count;
        const double* x0 = B.D + 3ull * N.begin;
        // the smallest ulp exponent and the largest exponent of the non-zero terms
        int q[3], e[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) q[c] = INT_MAX, e[c] = INT_MIN;
        for (uint32_t j = tid; j < np; j += NT)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const long long b = __double_as_longlong(x0[c * n3 + j]);
                if ((b & 0x7fffffffffffffffll) == 0) continue;
                const int E = int((b >> 52) & 0x7ff) - 1023;
                q[c] = min(q[c], max(E, -126) - 23);
                e[c] = max(e[c], E);
            }
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                q[c] = min(q[c], __shfl_xor_sync(kAll, q[c], o));
                e[c] = max(e[c], __shfl_xor_sync(kAll, e[c], o));
            }
        if (lane == 0u)
#pragma unroll
            for (int c = 0; c < 3; ++c) s_q[w][c] = q[c], s_e[w][c] = e[c];
        __syncthreads();
        const int lg = 32 - __clz(np - 1u);  // ceil(log2(np)), np > 1
        const uint32_t n_chunks = (np + kSumChunk - 1u) / kSumChunk;
        for (int c = 0; c < 3; ++c) {
            int qc = INT_MAX, ec = INT_MIN;
            for (uint32_t k = 0; k < kBigWarps; ++k) qc = min(qc, s_q[k][c]), ec = max(ec, s_e[k][c]);
            double m = 0.0;  // every term a zero: +0, as the chain from +0 gives
            // |term| < 2^(e + 1), so |count| < 2^(e + 1 - q); np of them, and
            // the drift of the replayed roundings, < 2^63
            if (ec != INT_MIN && !(ec < 1024 && lg + ec + 1 - qc <= 62)) {
                m = __longlong_as_double(kChainDue);
            } else if (ec != INT_MIN) {
                const double* x = x0 + c * n3;
                long long start = 0;  // the sequential sum before term k0, in counts of 2^q
                uint32_t k0 = 0, rounds = 0;
                bool due = false;
                while (k0 < np) {
                    // running sums from (k0, start), a tile of chunks at a time,
                    // up to the first that is not a double
                    uint32_t c0 = k0 / kSumChunk, hit = 0xffffffffu;
                    long long carry = start;
                    for (;;) {
                        const uint32_t ch = c0 + tid;
                        const uint32_t j0 = max(k0, ch * kSumChunk), j1 = min(np, ch * kSumChunk + kSumChunk);
                        long long sum = 0;
                        if (ch < n_chunks) {
#pragma unroll 8
                            for (uint32_t j = j0; j < j1; ++j) sum += units_of(x[j], qc);
                        }
                        long long before;
                        const long long tile = block_scan_ll<kBigWarps>(sum, s_sc, before);
                        if (tid == 0u) s_hit = 0xffffffffu;
                        __syncthreads();
                        if (ch < n_chunks) {
                            long long r = carry + before;
#pragma unroll 8
                            for (uint32_t j = j0; j < j1; ++j) {
                                r += units_of(x[j], qc);
                                if (!fits_double(r)) {
                                    atomicMin(&s_hit, j);
                                    break;
                                }
                            }
                            s_chunk[tid] = carry + before;
                        }
                        __syncthreads();
                        hit = s_hit;
                        if (hit != 0xffffffffu || c0 + NT >= n_chunks) {
                            if (hit == 0xffffffffu) start = carry + tile;
                            break;
                        }
                        carry += tile;
                        c0 += NT;
                        __syncthreads();  // s_hit and s_chunk are rewritten by the next tile
                    }
                    if (hit == 0xffffffffu) break;  // no add rounds from k0 on: start is the sum
                    if (tid == 0u) {  // the add of term hit rounds: the sum so far, rounded
                        const uint32_t ch = hit / kSumChunk;
                        long long r = s_chunk[ch - c0];
                        for (uint32_t j = max(k0, ch * kSumChunk); j <= hit; ++j) r += units_of(x[j], qc);
                        s_start = round_double(r);
                    }
                    __syncthreads();
                    start = s_start;
                    k0 = hit + 1u;
                    __syncthreads();  // s_start, s_hit and s_chunk are rewritten by the next round
                    if (++rounds > kSumRounds) {
                        due = true;
                        break;
                    }
                }
                // exact: start * 2^q, q >= -149
                m = due ? __longlong_as_double(kChainDue)
                        : __ll2double_rn(start) * __longlong_as_double((long long)(qc + 1023) << 52) / double(np);
            }
            if (tid == 0u) B.mom[9ull * (id - B.lo) + c] = m;
            __syncthreads();  // shared memory is reused by the next coordinate
        }
    }
}

// A thread per coordinate of the list's nodes: the chain of each sum that
// build_sums_big left due.
__global__ void build_sums_due_kernel(const BuildParams B) {
    const uint64_t n3 = 3ull * B.T;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < 3u * B.n_big; g += gridDim.x * blockDim.x) {
        const uint32_t id = B.big[g / 3u], c = g % 3u;
        double* m = B.mom + 9ull * (id - B.lo) + c;
        if (__double_as_longlong(*m) != kChainDue) continue;
        const BuildNode& N = B.nodes[id];
        const uint32_t np = 3u * N.count;
        *m = chain_sum(B.D + c * n3 + 3ull * N.begin, np) / double(np);
    }
}

// The centred products of every corner of the level, a thread per position:
// xx, yy, zz, xy, xz, yz (OBB.cpp:57-74).
__global__ void build_terms_kernel(const BuildParams B) {
    const uint64_t n3 = 3ull * B.T;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < B.T; t += gridDim.x * blockDim.x) {
        const uint32_t o = B.own[t];
        if (o < B.lo || o >= B.hi) continue;
        const double* m = B.mom + 9ull * (o - B.lo);
        const double mx = m[0], my = m[1], mz = m[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint64_t j = 3ull * t + k;
            const double dx = B.D[j] - mx, dy = B.D[n3 + j] - my, dz = B.D[2 * n3 + j] - mz;
            B.Tm[j] = dx * dx;
            B.Tm[n3 + j] = dy * dy;
            B.Tm[2 * n3 + j] = dz * dz;
            B.Tm[3 * n3 + j] = dx * dy;
            B.Tm[4 * n3 + j] = dx * dz;
            B.Tm[5 * n3 + j] = dy * dz;
        }
    }
}

// A thread per node and product: the covariance sum over the node's corners
// in order (std::inner_product, OBB.cpp:57-74).
__global__ void build_cov_kernel(const BuildParams B) {
    const uint64_t n3 = 3ull * B.T;
    const uint32_t total = 6u * (B.hi - B.lo);
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const uint32_t node = B.lo + g / 6u, q = g % 6u;
        const BuildNode& N = B.nodes[node];
        if (N.count > kBuildBig) continue;  // build_cov_big
        B.mom[9ull * (node - B.lo) + 3u + q] = chain_sum(B.Tm + q * n3 + 3ull * N.begin, 3u * N.count);
    }
}

// The same for the list's nodes of more than kBuildBig triangles, a
// one-warp block each (lanes 0-5 its six chains): a large node's chains
// share their warp's FP64 instructions and loads with no other node's.
__global__ void __launch_bounds__(32) build_cov_big_kernel(const BuildParams B) {
    const uint64_t n3 = 3ull * B.T;
    const uint32_t q = threadIdx.x;
    if (q >= 6u) return;
    for (uint32_t i = blockIdx.x; i < B.n_big; i += gridDim.x) {
        const uint32_t id = B.big[i];
        const BuildNode& N = B.nodes[id];
        B.mom[9ull * (id - B.lo) + 3u + q] = chain_sum(B.Tm + q * n3 + 3ull * N.begin, 3u * N.count);
    }
}

// A thread per node of the level: eig3 of its covariance (OBB.cpp:76-86) in
// FP64; the box axes (the rows of the eigenvector matrix) replace the node's
// moments.
__global__ void build_eig_kernel(const BuildParams B) {
    for (uint32_t node = B.lo + blockIdx.x * blockDim.x + threadIdx.x; node < B.hi; node += gridDim.x * blockDim.x) {
        double* m = B.mom + 9ull * (node - B.lo);
        if (B.nodes[node].count == 0u) continue;  // an empty mesh: the empty box, no axes
        const double dn = double(3u * B.nodes[node].count);
        const double cxx = m[3], cyy = m[4], czz = m[5], cxy = m[6], cxz = m[7], cyz = m[8];
        double v[3][3] = {{cxx / dn, cxy / dn, cxz / dn}, {cxy / dn, cyy / dn, cyz / dn}, {cxz / dn, cyz / dn, czz / dn}};
        double d[3], off[3];
        tridiagonalize(v, d, off);
        ql_sort(v, d, off, 2.220446049250313e-16);  // 2^-52
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) m[3 * r + c] = v[r][c];
    }
}

// The projections of every corner of the level on its node's three axes
// (the dot products of OBB.cpp:117, 136, 155), a thread per triangle
// position, into the products' buffer (free once the covariances are
// summed): [axis][corner].
__global__ void build_proj_kernel(const BuildParams B) {
    const uint64_t n3 = 3ull * B.T;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < B.T; t += gridDim.x * blockDim.x) {
        const uint32_t o = B.own[t];
        if (o < B.lo || o >= B.hi) continue;
        const double* ax = B.mom + 9ull * (o - B.lo);
        double a[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) a[k] = ax[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint64_t j = 3ull * t + k;
            const double px = B.D[j], py = B.D[n3 + j], pz = B.D[2 * n3 + j];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                double pr = a[3 * r] * px;
                pr = pr + a[3 * r + 1] * py;
                pr = pr + a[3 * r + 2] * pz;
                B.Tm[r * n3 + j] = pr;
            }
        }
    }
}

__device__ __forceinline__ Box empty_box() {  // OBB::EmptyOBB (OBB.cpp:168-178)
    const float e = FLT_EPSILON;
    return Box{make_float3(0.f, 0.f, 0.f), make_float3(e, 0.f, 0.f), make_float3(0.f, e, 0.f),
               make_float3(0.f, 0.f, e)};
}

// Corner j's projections (from build_proj) into the extremes.
__device__ __forceinline__ void extend3(const double* pr, uint64_t n3, uint32_t j, Ext* lo, Ext* hi) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double v = pr[a * n3 + j];
        const long long k = dkey(v);
        take_lo(lo[a], k, v, j);
        take_hi(hi[a], k, v, j);
    }
}

__device__ __forceinline__ void init_ext(Ext* lo, Ext* hi) {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = Ext{dkey(inf), inf, 0u};
        hi[a] = Ext{dkey(-inf), -inf, 0u};
    }
}

// OBB::CreateAABBfromPoints (OBB.cpp:105-166) from the extremes.
__device__ Box box_from(const double* ax, const Ext* lo, const Ext* hi) {
    const double pad = 2.0 * double(FLT_EPSILON);
    double cx = 0.0, cy = 0.0, cz = 0.0;
    float3 half[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double delta = (hi[a].v - lo[a].v) + pad;
        const double mid = (hi[a].v + lo[a].v) / 2.0;
        cx = cx + mid * ax[3 * a];
        cy = cy + mid * ax[3 * a + 1];
        cz = cz + mid * ax[3 * a + 2];
        const double h = delta / 2.0;
        half[a] = make_float3(float(h * ax[3 * a]), float(h * ax[3 * a + 1]), float(h * ax[3 * a + 2]));
    }
    return Box{make_float3(float(cx), float(cy), float(cz)), half[0], half[1], half[2]};
}

__device__ __forceinline__ bool same_point(float3 p, float3 q) { return p.x == q.x && p.y == q.y && p.z == q.z; }

// The node's box (OBB::CreateOBBfromPoints, OBB.cpp:33-89) by a warp.
__device__ Box fit_warp(const BuildParams& B, uint32_t begin, uint32_t n, const double* ax, uint32_t lane) {
    if (n == 0u) return empty_box();
    const float* pn = B.Pp + 9ull * begin;
    const uint32_t np = 3u * n;
    const float3 p0 = corner(pn, 0, 0);
    bool differ = false;
    for (uint32_t j = lane; j < np; j += 32u) differ |= !same_point(corner(pn, j / 3u, j % 3u), p0);
    if (!__any_sync(kAll, differ)) {  // one distinct point
        Box b = empty_box();
        b.c = p0;
        return b;
    }
    double a[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = ax[k];
    Ext lo[3], hi[3];
    init_ext(lo, hi);
    const uint64_t n3 = 3ull * B.T;
    const double* pr = B.Tm + 3ull * begin;
    for (uint32_t j = lane; j < np; j += 32u) extend3(pr, n3, j, lo, hi);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        warp_extreme(lo[k], true);
        warp_extreme(hi[k], false);
    }
    return box_from(a, lo, hi);
}

// The same by one thread (a small node).
__device__ Box fit_thread(const BuildParams& B, uint32_t begin, uint32_t n, const double* ax) {
    if (n == 0u) return empty_box();
    const float* pn = B.Pp + 9ull * begin;
    const uint32_t np = 3u * n;
    const float3 p0 = corner(pn, 0, 0);
    bool differ = false;
    for (uint32_t j = 1; j < np && !differ; ++j) differ = !same_point(corner(pn, j / 3u, j % 3u), p0);
    if (!differ) {
        Box b = empty_box();
        b.c = p0;
        return b;
    }
    double a[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = ax[k];
    Ext lo[3], hi[3];
    init_ext(lo, hi);
    const uint64_t n3 = 3ull * B.T;
    const double* pr = B.Tm + 3ull * begin;
    for (uint32_t j = 0; j < np; ++j) extend3(pr, n3, j, lo, hi);
    return box_from(a, lo, hi);
}

// TrianglePosition::GetMinMaxProjectionToAxis (Triangle.cpp:113-138), then the
// split test of OBBtree.cpp:70-74.
__device__ __forceinline__ bool goes_left(const float* P, uint32_t t, float3 axis, float cp) {
    float lo = __int_as_float(0x7f800000), hi = -lo;
#pragma unroll
    for (uint32_t k = 0; k < 3u; ++k) {
        const float pr = dot3(axis, corner(P, t, k));
        if (pr < lo) lo = pr;
        if (pr > hi) hi = pr;
    }
    const float mid = (lo + hi) / 2.0f;
    return mid <= cp;
}

__device__ __forceinline__ void split_axes(const Box& b, float3* dir, int* ord);

// Splits the node's range (perm, n > kLeafMax; P its corners by position) in
// place and returns the left child's size.
__device__ uint32_t split_node(const float* P, uint32_t* perm, uint32_t* scratch, uint32_t n, const Box& b,
                               uint32_t lane) {
    float3 dir[3];
    int ord[3];
    split_axes(b, dir, ord);
    bool chosen = false;
    uint32_t nl = n / 2u;
    float3 axis = dir[ord[0]];
    float cp = 0.f;
    for (int k = 0; k < 3 && !chosen; ++k) {
        const float3 a = dir[ord[k]];
        const float c = dot3(b.c, a);
        uint32_t cnt = 0;
        for (uint32_t base = 0; base < n; base += 32u) {
            const uint32_t t = base + lane;
            const bool left = t < n && goes_left(P, t, a, c);
            cnt += __popc(__ballot_sync(kAll, left));
        }
        if (cnt > 0u && cnt < n) {
            chosen = true;
            nl = cnt;
            axis = a;
            cp = c;
        }
    }
    uint32_t lb = 0, rb = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (uint32_t base = 0; base < n; base += 32u) {
        const uint32_t t = base + lane;
        const bool valid = t < n;
        uint32_t id = 0;
        bool left = false;
        if (valid) {
            id = perm[t];
            left = chosen ? goes_left(P, t, axis, cp) : (t < nl);
        }
        const unsigned ml = __ballot_sync(kAll, left), mv = __ballot_sync(kAll, valid);
        if (valid) scratch[left ? lb + __popc(ml & lt) : nl + rb + __popc(mv & ~ml & lt)] = id;
        lb += __popc(ml);
        rb += __popc(mv & ~ml);
    }
    __syncwarp();
    for (uint32_t t = lane; t < n; t += 32u) perm[t] = scratch[t];
    __syncwarp();
    return nl;
}

// The split's axes in order (OBBtree.cpp:45-53): by half-length, longest
// first; equal lengths keep u, v, w order (std::sort of three is an
// insertion sort).
__device__ __forceinline__ void split_axes(const Box& b, float3* dir, int* ord) {
    const float len[3] = {length3(b.u), length3(b.v), length3(b.w)};
    dir[0] = normalize3(b.u);
    dir[1] = normalize3(b.v);
    dir[2] = normalize3(b.w);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int r = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j)
            r += (len[j] > len[k]) || (j < k && !(len[j] > len[k]) && !(len[k] > len[j]));
        ord[r] = k;
    }
}

// The same split by one thread (a small node).
__device__ uint32_t split_thread(const float* P, uint32_t* perm, uint32_t* scratch, uint32_t n, const Box& b) {
    float3 dir[3];
    int ord[3];
    split_axes(b, dir, ord);
    bool chosen = false;
    uint32_t nl = n / 2u;
    float3 axis = dir[ord[0]];
    float cp = 0.f;
    for (int k = 0; k < 3 && !chosen; ++k) {
        const float3 a = dir[ord[k]];
        const float c = dot3(b.c, a);
        uint32_t cnt = 0;
        for (uint32_t t = 0; t < n; ++t) cnt += goes_left(P, t, a, c) ? 1u : 0u;
        if (cnt > 0u && cnt < n) {
            chosen = true;
            nl = cnt;
            axis = a;
            cp = c;
        }
    }
    uint32_t lb = 0, rb = nl;
    for (uint32_t t = 0; t < n; ++t) {
        const uint32_t id = perm[t];
        const bool left = chosen ? goes_left(P, t, axis, cp) : (t < nl);
        scratch[left ? lb++ : rb++] = id;
    }
    for (uint32_t t = 0; t < n; ++t) perm[t] = scratch[t];
    return nl;
}

__device__ __forceinline__ void store_box(BuildNode& N, const Box& box) {
    float* o = N.box;
    o[0] = box.c.x, o[1] = box.c.y, o[2] = box.c.z;
    o[3] = box.u.x, o[4] = box.u.y, o[5] = box.u.z;
    o[6] = box.v.x, o[7] = box.v.y, o[8] = box.v.z;
    o[9] = box.w.x, o[10] = box.w.y, o[11] = box.w.z;
}

// Appends the two children of a split node (its first nl triangles, the
// rest) and returns the first's id, or kNoKid when the table is full.
__device__ __forceinline__ uint32_t add_children(const BuildParams& B, BuildNode& N, uint32_t nl) {
    const uint32_t k = atomicAdd(B.node_ctr, 2u);
    if (k + 2u > B.node_cap) {
        atomicOr(B.error, 1u);
        return kNoKid;
    }
    BuildNode& L = B.nodes[k];
    BuildNode& R = B.nodes[k + 1u];
    L.begin = N.begin, L.count = nl, L.kid = kNoKid, L.tree = N.tree;
    R.begin = N.begin + nl, R.count = N.count - nl, R.kid = kNoKid, R.tree = N.tree;
    N.kid = k;
    return k;
}

constexpr uint32_t kSmall = 16;  // nodes of at most this many triangles: a thread each

// A warp per node of the level with more than kSmall and at most kBuildBig
// triangles: the box, the split, the children's positions.
__global__ void __launch_bounds__(128) build_fit_kernel(const BuildParams B) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t id = B.lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); id < B.hi; id += warps) {
        BuildNode& N = B.nodes[id];
        const uint32_t begin = N.begin, n = N.count;
        if (n <= kSmall || n > kBuildBig) continue;
        const Box box = fit_warp(B, begin, n, B.mom + 9ull * (id - B.lo), lane);
        const uint32_t nl = split_node(B.Pp + 9ull * begin, B.perm + begin, B.scratch + begin, n, box, lane);
        uint32_t k = 0;
        if (lane == 0u) {
            store_box(N, box);
            N.kid = kNoKid;
            k = add_children(B, N, nl);
        }
        k = __shfl_sync(kAll, k, 0);
        if (k == kNoKid) continue;
        for (uint32_t t = lane; t < n; t += 32u) B.own[begin + t] = t < nl ? k : k + 1u;
    }
}

// Of two extremes with keys k (smaller wins for lo, larger for hi), the one
// the sequential scan keeps: on equal keys the later corner.
__device__ __forceinline__ void merge_ext(Ext& e, const Ext& o, bool lo) {
    if ((lo ? o.k < e.k : o.k > e.k) || (o.k == e.k && o.j > e.j)) e = o;
}

// A block per node of the level's list of nodes of more than kBuildBig
// triangles (the top levels of the large meshes, where one warp's walk of the
// range set the level's time): the box and split of build_fit_kernel, the
// corners shared out by thread, the split's counts and partition by warp over
// consecutive segments of the range (each warp's lefts and rights go after
// those of the segments before it, so the partition stays stable). Children
// of more than kBuildBig triangles go to the next level's list.
__global__ void __launch_bounds__(kBigWarps * 32) build_fit_big_kernel(const BuildParams B) {
    constexpr uint32_t NT = kBigWarps * 32u;
    __shared__ Ext s_lo[kBigWarps][3], s_hi[kBigWarps][3];
    __shared__ uint32_t s_cnt[kBigWarps], s_sel[kBigWarps];
    __shared__ Box s_box;
    __shared__ uint32_t s_kid;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    for (uint32_t i = blockIdx.x; i < B.n_big; i += gridDim.x) {
        const uint32_t id = B.big[i];
        BuildNode& N = B.nodes[id];
        const uint32_t begin = N.begin, n = N.count;
        const float* pn = B.Pp + 9ull * begin;
        const uint32_t np = 3u * n;
        const float3 p0 = corner(pn, 0, 0);
        bool differ = false;
        for (uint32_t j = tid; j < np; j += NT) differ |= !same_point(corner(pn, j / 3u, j % 3u), p0);
        const bool distinct = __syncthreads_or(differ) != 0;
        if (distinct) {
            Ext lo[3], hi[3];
            init_ext(lo, hi);
            const uint64_t n3 = 3ull * B.T;
            const double* pr = B.Tm + 3ull * begin;
            for (uint32_t j = tid; j < np; j += NT) extend3(pr, n3, j, lo, hi);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                warp_extreme(lo[k], true);
                warp_extreme(hi[k], false);
            }
            if (lane == 0u)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    s_lo[w][k] = lo[k];
                    s_hi[w][k] = hi[k];
                }
        }
        __syncthreads();
        if (tid == 0u) {
            Box box;
            if (distinct) {
                Ext lo[3], hi[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    lo[k] = s_lo[0][k];
                    hi[k] = s_hi[0][k];
                }
                for (uint32_t v = 1; v < kBigWarps; ++v)
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        merge_ext(lo[k], s_lo[v][k], true);
                        merge_ext(hi[k], s_hi[v][k], false);
                    }
                double a[9];
                const double* ax = B.mom + 9ull * (id - B.lo);
#pragma unroll
                for (int k = 0; k < 9; ++k) a[k] = ax[k];
                box = box_from(a, lo, hi);
            } else {  // one distinct point
                box = empty_box();
                box.c = p0;
            }
            s_box = box;
        }
        __syncthreads();
        const Box box = s_box;

        // the split (split_node's rule), this warp over positions [sb, se)
        float3 dir[3];
        int ord[3];
        split_axes(box, dir, ord);
        const uint32_t seg = (n + kBigWarps - 1u) / kBigWarps;
        const uint32_t sb = min(n, w * seg), se = min(n, sb + seg);
        bool chosen = false;
        uint32_t nl = n / 2u;
        float3 axis = dir[ord[0]];
        float cp = 0.f;
        for (int k = 0; k < 3 && !chosen; ++k) {
            const float3 a = dir[ord[k]];
            const float c = dot3(box.c, a);
            uint32_t cnt = 0;
            for (uint32_t base = sb; base < se; base += 32u) {
                const uint32_t t = base + lane;
                cnt += __popc(__ballot_sync(kAll, t < se && goes_left(pn, t, a, c)));
            }
            if (lane == 0u) s_cnt[w] = cnt;
            __syncthreads();
            uint32_t total = 0;
            for (uint32_t v = 0; v < kBigWarps; ++v) total += s_cnt[v];
            if (total > 0u && total < n) {
                chosen = true;
                nl = total;
                axis = a;
                cp = c;
                if (tid < kBigWarps) s_sel[tid] = s_cnt[tid];
            }
            __syncthreads();
        }
        uint32_t lb = 0;  // left positions before this warp's segment
        if (chosen)
            for (uint32_t v = 0; v < w; ++v) lb += s_sel[v];
        else
            lb = min(sb, nl);
        uint32_t rb = sb - lb;
        uint32_t* perm = B.perm + begin;
        uint32_t* scr = B.scratch + begin;
        for (uint32_t base = sb; base < se; base += 32u) {
            const uint32_t t = base + lane;
            const bool valid = t < se;
            uint32_t tri = 0;
            bool left = false;
            if (valid) {
                tri = perm[t];
                left = chosen ? goes_left(pn, t, axis, cp) : (t < nl);
            }
            const unsigned ml = __ballot_sync(kAll, left), mv = __ballot_sync(kAll, valid);
            if (valid) scr[left ? lb + __popc(ml & lt) : nl + rb + __popc(mv & ~ml & lt)] = tri;
            lb += __popc(ml);
            rb += __popc(mv & ~ml);
        }
        __syncthreads();
        for (uint32_t t = tid; t < n; t += NT) perm[t] = scr[t];
        if (tid == 0u) {
            store_box(N, box);
            N.kid = kNoKid;
            const uint32_t k = add_children(B, N, nl);
            if (k != kNoKid) {
                if (nl > kBuildBig) B.big_out[atomicAdd(B.n_big_out, 1u)] = k;
                if (n - nl > kBuildBig) B.big_out[atomicAdd(B.n_big_out, 1u)] = k + 1u;
            }
            s_kid = k;
        }
        __syncthreads();
        const uint32_t k = s_kid;
        if (k != kNoKid)
            for (uint32_t t = tid; t < n; t += NT) B.own[begin + t] = t < nl ? k : k + 1u;
        __syncthreads();  // shared memory is reused by the next node
    }
}

// A thread per node of the level with at most kSmall triangles.
__global__ void __launch_bounds__(128) build_fit_small_kernel(const BuildParams B) {
    for (uint32_t id = B.lo + blockIdx.x * blockDim.x + threadIdx.x; id < B.hi; id += gridDim.x * blockDim.x) {
        BuildNode& N = B.nodes[id];
        const uint32_t begin = N.begin, n = N.count;
        if (n > kSmall) continue;
        const Box box = fit_thread(B, begin, n, B.mom + 9ull * (id - B.lo));
        store_box(N, box);
        N.kid = kNoKid;
        if (n <= kLeafMax) continue;
        const uint32_t nl = split_thread(B.Pp + 9ull * begin, B.perm + begin, B.scratch + begin, n, box);
        const uint32_t k = add_children(B, N, nl);
        if (k == kNoKid) continue;
        for (uint32_t t = 0; t < n; ++t) B.own[begin + t] = t < nl ? k : k + 1u;
    }
}

// The meshes' triangles from their vertex and index buffers: a thread per
// triangle (its mesh is its root node, the owner of every position before
// the first split).
// A thread per triangle position: its mesh (the last mesh whose first
// triangle is at or before it; empty meshes share the next one's start).
__global__ void build_owner_kernel(const BuildParams B, const BuildInput I, uint32_t n_meshes) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < B.T; t += gridDim.x * blockDim.x) {
        uint32_t a = 0, b = n_meshes - 1u;
        while (a < b) {
            const uint32_t m = (a + b + 1u) >> 1;
            if (I.meshes[m].tbase <= t)
                a = m;
            else
                b = m - 1u;
        }
        B.own[t] = a;
    }
}

// A vertex index out of its mesh's range is recorded (the smallest mesh, then
// index position, in I.bad) and its corner read as vertex 0, or as zeros for
// a mesh without vertices; the host then fails the build.
__global__ void build_gather_kernel(const BuildParams B, const BuildInput I) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < B.T; g += gridDim.x * blockDim.x) {
        const uint32_t m = B.own[g];
        const BuildMesh M = I.meshes[m];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            uint32_t vi = I.indices[3ull * g + k];
            if (vi >= M.n_vertices) {
                atomicMin(I.bad, (unsigned long long)m << 32 | (3ull * (g - M.tbase) + k));
                vi = 0;
            }
            float* o = I.P + 9ull * g + 3 * k;
            float* on = M.has_normals ? I.corner_normals + 9ull * g + 3 * k : nullptr;
            if (M.n_vertices == 0u) {
                o[0] = o[1] = o[2] = 0.f;
                if (on) on[0] = on[1] = on[2] = 0.f;
                continue;
            }
            const float* v = I.vertices + 3ull * (M.vbase + vi);
            o[0] = v[0], o[1] = v[1], o[2] = v[2];
            if (on) {
                const float* nv = I.normals + 3ull * (M.vbase + vi);
                on[0] = nv[0], on[1] = nv[1], on[2] = nv[2];
            }
        }
        B.perm[g] = g;
    }
}

// The meshes' host arrays into the build's input buffers, read by the device
// (pageable host memory, where the device reads it): block (x, y) copies
// words [x kPullWords, (x + 1) kPullWords) of segment y, each thread's loads
// issued before its stores.
constexpr uint32_t kPullThreads = 256, kPullPer = 16, kPullWords = kPullThreads * kPullPer;
__global__ void __launch_bounds__(kPullThreads) build_pull_kernel(const PullSeg* segs) {
    const PullSeg S = segs[blockIdx.y];
    const uint64_t base = uint64_t(blockIdx.x) * kPullWords;
    if (base >= S.n) return;
    uint32_t v[kPullPer];
#pragma unroll
    for (uint32_t k = 0; k < kPullPer; ++k) {
        const uint64_t w = base + k * kPullThreads + threadIdx.x;
        if (w < S.n) v[k] = S.src[w];
    }
#pragma unroll
    for (uint32_t k = 0; k < kPullPer; ++k) {
        const uint64_t w = base + k * kPullThreads + threadIdx.x;
        if (w < S.n) S.dst[w] = v[k];
    }
}

// Bottom-up, a level at a time from the deepest: the inner nodes of each
// node's subtree.
__global__ void build_inner_kernel(const BuildParams B, BuildFlat* flat) {
    for (uint32_t id = B.lo + blockIdx.x * blockDim.x + threadIdx.x; id < B.hi; id += gridDim.x * blockDim.x) {
        const uint32_t k = B.nodes[id].kid;
        flat[id].inner = k == kNoKid ? 0u : 1u + flat[k].inner + flat[k + 1u].inner;
    }
}

__device__ __forceinline__ float node_surface(const BuildNode& N) {  // Paralgram::GetSurface (Paralgram.cpp:203-210)
    const float* b = N.box;
    const float3 u = make_float3(b[3], b[4], b[5]), v = make_float3(b[6], b[7], b[8]), w = make_float3(b[9], b[10], b[11]);
    const float uv = length3(cross3(u, v)), uw = length3(cross3(u, w)), vw = length3(cross3(v, w));
    return 2.0f * (uv + uw + vw);
}

// Top-down, a level at a time from the roots: each node's place in its tree's
// pre-order layout (OBBtree.cpp:179-233, 385-394): the larger-surface child
// first (OBBtree.cpp:100-106), inner nodes numbered in pre-order, leaves'
// triangles appended in pre-order; the children's records follow their
// parent's index (records 2k + 2 and 2k + 3 of inner node k, the root's 1).
__global__ void build_order_kernel(const BuildParams B, BuildFlat* flat, uint32_t n_roots) {
    for (uint32_t id = B.lo + blockIdx.x * blockDim.x + threadIdx.x; id < B.hi; id += gridDim.x * blockDim.x) {
        BuildFlat X = flat[id];
        if (id < n_roots) {
            X.index = 0u, X.tri_off = 0u, X.leaf_off = 0u, X.rec = 1u, X.prec = kNoKid;
            flat[id] = X;
        }
        const BuildNode& N = B.nodes[id];
        if (N.kid == kNoKid) continue;
        uint32_t f = N.kid, s = N.kid + 1u;
        if (node_surface(B.nodes[s]) > node_surface(B.nodes[f])) {
            const uint32_t t = f;
            f = s;
            s = t;
        }
        BuildFlat& F = flat[f];
        BuildFlat& S = flat[s];
        flat[id].split_off = X.tri_off + B.nodes[f].count;
        F.index = X.index + 1u;
        S.index = X.index + 1u + F.inner;
        F.tri_off = X.tri_off;
        S.tri_off = X.tri_off + B.nodes[f].count;
        F.leaf_off = X.leaf_off;
        S.leaf_off = X.leaf_off + F.inner + 1u;
        F.rec = 2u * X.index + 2u;
        S.rec = 2u * X.index + 3u;
        F.prec = S.prec = X.rec;
    }
}

// A thread per node of the batch: its record in its tree's arena range (box,
// link word: first child record or first triangle, leaf word), its subtree's
// triangle range, its parent record and, for a leaf, its place in the leaf
// list; a root also writes its tree's unused record 0.
__global__ void build_emit_nodes_kernel(const BuildParams B, const BuildFlat* flat, const BuildEmit* emit,
                                        float4* recs, uint32_t n_nodes, uint32_t n_roots) {
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n_nodes; id += gridDim.x * blockDim.x) {
        const BuildNode& N = B.nodes[id];
        const BuildFlat& X = flat[id];
        const BuildEmit& E = emit[N.tree];
        const bool leaf = N.kid == kNoKid;
        const uint32_t ref = leaf ? E.tri_base + X.tri_off : E.rec_base + 2u * X.index + 2u;
        const uint32_t meta = leaf ? (kLeafFlag | (N.count & 0xffffu)) : 0u;
        const float* b = N.box;
        float4* r = recs + 4ull * (E.rec_base + X.rec);
        r[0] = make_float4(b[0], b[1], b[2], b[3]);
        r[1] = make_float4(b[4], b[5], b[6], b[7]);
        r[2] = make_float4(b[8], b[9], b[10], b[11]);
        r[3] = make_float4(__uint_as_float(ref), __uint_as_float(meta), node_surface(N),
                           __uint_as_float(leaf ? 0u : E.tri_base + X.split_off));
        E.ranges[X.rec] = make_uint2(X.tri_off, N.count);
        E.topo[X.rec] = X.prec;
        if (leaf) E.topo[E.n_recs + X.leaf_off] = X.rec;
        if (id < n_roots) {
            float4* z = recs + 4ull * E.rec_base;
            z[0] = z[1] = z[2] = z[3] = make_float4(0.f, 0.f, 0.f, 0.f);
            E.ranges[0] = make_uint2(0u, ~0u);
            E.topo[0] = kNoKid;
        }
    }
}

// A thread per triangle position: the triangle into its tree's arena range at
// its leaf's place (corners, vertex indices in the w words), with its corner
// normals when the mesh has them.
__global__ void build_emit_tris_kernel(const BuildParams B, const BuildInput I, const BuildFlat* flat,
                                       const BuildEmit* emit, float4* tris) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < B.T; p += gridDim.x * blockDim.x) {
        const uint32_t leaf = B.own[p];
        const BuildNode& N = B.nodes[leaf];
        const BuildEmit& E = emit[N.tree];
        const uint32_t local = flat[leaf].tri_off + (p - N.begin);
        const uint32_t g = B.perm[p];
        const float* c = I.P + 9ull * g;
        float4* o = tris + 3ull * (E.tri_base + local);
#pragma unroll
        for (int k = 0; k < 3; ++k) o[k] = make_float4(c[3 * k], c[3 * k + 1], c[3 * k + 2], __uint_as_float(I.indices[3ull * g + k]));
        if (E.nrm) {
            const float* n = I.corner_normals + 9ull * g;
            float* on = E.nrm + 9ull * local;
#pragma unroll
            for (int k = 0; k < 9; ++k) on[k] = n[k];
        }
    }
}

}  // namespace

cudaError_t launch_build_level(const BuildParams& p, uint32_t sm_count, cudaStream_t s) {
    if (p.hi <= p.lo) return cudaSuccess;
    const uint32_t width = p.hi - p.lo;
    const uint32_t wide = sm_count * 8u;  // blocks of the per-position kernels
    auto grid = [&](uint64_t threads) {
        const uint64_t b = (threads + 127u) / 128u;
        return uint32_t(b < wide ? (b ? b : 1u) : wide);
    };
    build_points_kernel<<<grid(p.T), 128, 0, s>>>(p);
    build_sums_kernel<<<grid(3ull * width), 128, 0, s>>>(p);
    if (p.n_big) {
        build_sums_big_kernel<<<p.n_big < 65535u ? p.n_big : 65535u, kBigWarps * 32u, 0, s>>>(p);
        build_sums_due_kernel<<<grid(3ull * p.n_big), 128, 0, s>>>(p);
    }
    build_terms_kernel<<<grid(p.T), 128, 0, s>>>(p);
    build_cov_kernel<<<grid(6ull * width), 128, 0, s>>>(p);
    if (p.n_big) build_cov_big_kernel<<<p.n_big < 65535u ? p.n_big : 65535u, 32, 0, s>>>(p);
    build_eig_kernel<<<grid(width), 128, 0, s>>>(p);
    build_proj_kernel<<<grid(p.T), 128, 0, s>>>(p);
    if (p.n_big) build_fit_big_kernel<<<p.n_big < 65535u ? p.n_big : 65535u, kBigWarps * 32u, 0, s>>>(p);
    const uint32_t blocks = (width + 3u) / 4u;
    build_fit_kernel<<<blocks < 65535u ? blocks : 65535u, 128, 0, s>>>(p);
    build_fit_small_kernel<<<grid(width), 128, 0, s>>>(p);
    return cudaGetLastError();
}

namespace {
uint32_t grid_of(uint64_t threads, uint32_t sm_count) {
    const uint64_t b = (threads + 127u) / 128u, cap = uint64_t(sm_count) * 8u;
    return uint32_t(b < cap ? (b ? b : 1u) : cap);
}
}  // namespace

cudaError_t launch_build_gather(const BuildParams& p, const BuildInput& in, uint32_t n_meshes, uint32_t sm_count,
                                cudaStream_t s) {
    if (p.T && n_meshes) build_owner_kernel<<<grid_of(p.T, sm_count), 128, 0, s>>>(p, in, n_meshes);
    if (p.T) build_gather_kernel<<<grid_of(p.T, sm_count), 128, 0, s>>>(p, in);
    return cudaGetLastError();
}

cudaError_t launch_build_pull(const PullSeg* segs, uint32_t n_segs, uint64_t max_words, cudaStream_t s) {
    if (!n_segs || !max_words) return cudaSuccess;
    const uint64_t gx = (max_words + kPullWords - 1u) / kPullWords;
    if (gx > 0x7fffffffull) return cudaErrorInvalidValue;
    for (uint32_t first = 0; first < n_segs; first += 65535u) {  // the grid's y extent
        const uint32_t ny = n_segs - first < 65535u ? n_segs - first : 65535u;
        build_pull_kernel<<<dim3(uint32_t(gx), ny), kPullThreads, 0, s>>>(segs + first);
    }
    return cudaGetLastError();
}

cudaError_t launch_build_inner(const BuildParams& p, BuildFlat* flat, uint32_t sm_count, cudaStream_t s) {
    if (p.hi > p.lo) build_inner_kernel<<<grid_of(p.hi - p.lo, sm_count), 128, 0, s>>>(p, flat);
    return cudaGetLastError();
}

cudaError_t launch_build_order(const BuildParams& p, BuildFlat* flat, uint32_t n_roots, uint32_t sm_count,
                               cudaStream_t s) {
    if (p.hi > p.lo) build_order_kernel<<<grid_of(p.hi - p.lo, sm_count), 128, 0, s>>>(p, flat, n_roots);
    return cudaGetLastError();
}

cudaError_t launch_build_emit(const BuildParams& p, const BuildInput& in, const BuildFlat* flat,
                              const BuildEmit* emit, float4* recs, float4* tris, uint32_t n_nodes, uint32_t n_roots,
                              uint32_t sm_count, cudaStream_t s) {
    if (n_nodes) build_emit_nodes_kernel<<<grid_of(n_nodes, sm_count), 128, 0, s>>>(p, flat, emit, recs, n_nodes, n_roots);
    if (p.T) build_emit_tris_kernel<<<grid_of(p.T, sm_count), 128, 0, s>>>(p, in, flat, emit, tris);
    return cudaGetLastError();
}

}  // namespace cg
