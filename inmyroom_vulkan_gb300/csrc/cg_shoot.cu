// Uncollide-ray shooting: ShootUncollideRays::ExecuteShootUncollideRays
// (src/CollisionDetection/ShootUncollideRays.cpp:14-180) for a batch of entity
// pairs, over Ray::IntersectOBBtree closest-hit traversals
// (src/Geometry/Ray.cpp:36-237).
//
//   shoot_ray_kernel    four lanes per ray: the Hermann pass of the ray (the
//                       closest hit on the other tree, a back face, no nearer
//                       hit on its own tree from the origin moved by 4 ulps;
//                       the two traversals side by side, each kept by a lane
//                       pair), and when it succeeds the pass of its
//                       reflection back; each success as (signed force
//                       response, signed ray response)
//   shoot_query_kernel  a warp per pair: the force responses summed in the
//                       reference's order (rays from the first entity, each
//                       followed by its reflection, then those from the
//                       second), FindResponse's maximum over the ray
//                       responses (order-free), the delta in world space
// Every step rounds where the reference rounds (built without contraction,
// IEEE division and square root), so the deltas are the reference's bits for
// the same rays in the same order. The ray/triangle test is the one the glm
// shim states for the reference's glm fork (Moller-Trumbore, two-sided, back
// face = negative determinant).
//
// The traversal keeps the recursion's order with an explicit stack: of two
// children whose slabs the ray enters, the nearer entry first (ties: the
// right child), each visited only if its entry is before the best hit so far
// (checked when it is taken from the stack, as the recursion checks the
// second child after the first's subtree) and its exit is not behind the ray.
#include <cuda_runtime.h>

#include <cfloat>

#include "cg_device.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr uint32_t kShootStack = 96;  // deferred boxes per ray (a tree deeper than this reports ERR_QUEUE)

struct Slab {
    bool hit;
    float tmin, tmax;
};

// Ray::IntersectParalgram (Ray.cpp:36-133) for a ray from the origin.
__device__ __forceinline__ Slab ray_box(const Box& b, float3 dir) {
    float mn = -__int_as_float(0x7f800000), mx = __int_as_float(0x7f800000);
    const float3 ro = sub3(make_float3(0.f, 0.f, 0.f), b.c);
    const float3 fa[3] = {b.v, b.w, b.u}, fb[3] = {b.w, b.u, b.v}, side[3] = {b.u, b.v, b.w};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float3 pd = normalize3(cross3(fa[k], fb[k]));
        const float d = -fabsf(dot3(pd, side[k]));
        const float pc = dot3(pd, ro);
        const float n1 = pc + d;
        const float n2 = -pc + d;
        const float vd = dot3(pd, dir);
        if (fabsf(vd) >= FLT_EPSILON) {
            const float inv = 1.f / vd;
            float t1 = -n1 * inv;
            float t2 = n2 * inv;
            if (t1 > t2) {
                const float t = t1;
                t1 = t2;
                t2 = t;
            }
            mn = (t1 < mn) ? mn : t1;
            mx = (mx < t2) ? mx : t2;
            if (mn > mx || mx < 0.f) return Slab{false, 0.f, 0.f};
        } else if (n1 > 0.f || n2 > 0.f) {
            return Slab{false, 0.f, 0.f};
        }
    }
    return Slab{true, mn, mx};
}

// The glm fork's intersectRayTriangle as the shim states it (Ray.cpp:22-33).
__device__ __forceinline__ bool ray_tri(float3 orig, float3 dir, float3 v0, float3 v1, float3 v2, float& bx,
                                        float& by, float& t, bool& back) {
    const float3 e1 = sub3(v1, v0), e2 = sub3(v2, v0);
    const float3 p = cross3(dir, e2);
    const float det = dot3(e1, p);
    back = det < 0.f;
    if (fabsf(det) <= FLT_EPSILON) return false;
    const float inv = 1.f / det;
    const float3 s0 = sub3(orig, v0);
    const float u = dot3(s0, p) * inv;
    if (u < 0.f || u > 1.f) return false;
    const float3 q = cross3(s0, e1);
    const float v = dot3(dir, q) * inv;
    if (v < 0.f || u + v > 1.f) return false;
    const float tt = dot3(e2, q) * inv;
    if (tt < 0.f) return false;
    bx = u;
    by = v;
    t = tt;
    return true;
}

struct TreeHit {
    bool hit, back;
    float dist;
    uint32_t tri;  // arena index
    float bx, by;
};

__device__ __forceinline__ void rec_box(const float4* recs, uint32_t r, Box& b, uint32_t& ref, uint32_t& meta) {
    const float4* p = recs + 4ull * r;
    const float4 a = __ldg(p), c1 = __ldg(p + 1), c2 = __ldg(p + 2), d = __ldg(p + 3);
    b.c = make_float3(a.x, a.y, a.z);
    b.u = make_float3(a.w, c1.x, c1.y);
    b.v = make_float3(c1.z, c1.w, c2.x);
    b.w = make_float3(c2.y, c2.z, c2.w);
    ref = __float_as_uint(d.x);
    meta = __float_as_uint(d.y);
}

// Ray::IntersectOBBtree (Ray.cpp:135-237) on the tree rooted at record root,
// by a lane pair (c = 0, 1; pm = the pair's mask) that keeps one traversal in
// step: both lanes hold the same stack; at an inner node lane c tests child
// c's box and the pair swaps the results, at a leaf lane c tests every other
// triangle and the pair keeps the nearer hit (equal distances: the lower
// triangle, as the one-lane scan keeps the first). A stack entry carries the
// child's own link word and leaf word, read when its box was tested.
__device__ __noinline__ TreeHit ray_tree(const float4* recs, const float4* tris, uint32_t root, const Mat4& matrix,
                                         float3 origin, float3 dir, unsigned* error, uint32_t c, unsigned pm) {
    Mat4 cm = matrix;
    if (!(origin.x == 0.f && origin.y == 0.f && origin.z == 0.f))
        cm.c3 = make_float4(matrix.c3.x - origin.x, matrix.c3.y - origin.y, matrix.c3.z - origin.z, matrix.c3.w - 0.f);
    TreeHit best{false, false, __int_as_float(0x7f800000), 0xffffffffu, 0.f, 0.f};
    uint32_t st_ref[kShootStack], st_meta[kShootStack];
    float st_min[kShootStack];
    uint32_t sp = 0;
    {
        Box b;
        uint32_t ref, meta;
        rec_box(recs, root, b, ref, meta);
        const Slab h = ray_box(xform_box(cm, b), dir);
        if (h.hit && h.tmax >= 0.f) {
            st_ref[0] = ref;
            st_meta[0] = meta;
            st_min[0] = -__int_as_float(0x7f800000);  // the root is entered without the distance check
            sp = 1;
        }
    }
    const float3 zero = make_float3(0.f, 0.f, 0.f);
    while (sp) {
        --sp;
        const uint32_t ref = st_ref[sp], meta = st_meta[sp];
        if (!(st_min[sp] < best.dist)) continue;
        if (!(meta & kLeafFlag)) {
            Box b;
            uint32_t cref, cmeta;
            rec_box(recs, ref + c, b, cref, cmeta);
            const Slab h = ray_box(xform_box(cm, b), dir);
            const int ohit = __shfl_xor_sync(pm, int(h.hit), 1);
            const float omin = __shfl_xor_sync(pm, h.tmin, 1), omax = __shfl_xor_sync(pm, h.tmax, 1);
            const uint32_t oref = __shfl_xor_sync(pm, cref, 1), ometa = __shfl_xor_sync(pm, cmeta, 1);
            const Slab other{ohit != 0, omin, omax};
            const Slab hl = c ? other : h, hr = c ? h : other;
            const uint32_t lref = c ? oref : cref, lmeta = c ? ometa : cmeta;
            const uint32_t rref = c ? cref : oref, rmeta = c ? cmeta : ometa;
            auto push = [&](uint32_t r, uint32_t m, const Slab& s) {
                if (s.tmax < 0.f) return;  // the box is behind the ray
                if (sp < kShootStack) {
                    st_ref[sp] = r;
                    st_meta[sp] = m;
                    st_min[sp] = s.tmin;
                    ++sp;
                } else {
                    atomicOr(error, ERR_QUEUE);
                }
            };
            if (hl.hit && hr.hit) {
                // the later one first, so that the nearer one is taken next
                if (hl.tmin < hr.tmin) {
                    push(rref, rmeta, hr);
                    push(lref, lmeta, hl);
                } else {
                    push(lref, lmeta, hl);
                    push(rref, rmeta, hr);
                }
            } else if (hl.hit) {
                push(lref, lmeta, hl);
            } else if (hr.hit) {
                push(rref, rmeta, hr);
            }
            continue;
        }
        const uint32_t n = meta & 0xffffu;
        TreeHit mine = best;
        for (uint32_t i = ref + c; i < ref + n; i += 2u) {
            const float4* t4 = tris + 3ull * i;
            const float4 q0 = __ldg(t4), q1 = __ldg(t4 + 1), q2 = __ldg(t4 + 2);
            const float3 p0 = xform(cm, make_float3(q0.x, q0.y, q0.z), 1.0f);
            const float3 p1 = xform(cm, make_float3(q1.x, q1.y, q1.z), 1.0f);
            const float3 p2 = xform(cm, make_float3(q2.x, q2.y, q2.z), 1.0f);
            float bx = 0.f, by = 0.f, t = 0.f;
            bool back = false;
            const bool hit = ray_tri(zero, dir, p0, p1, p2, bx, by, t, back);
            if (hit && t > 0.f && t < mine.dist) {
                mine.hit = true;
                mine.back = back;
                mine.dist = t;
                mine.tri = i;
                mine.bx = bx;
                mine.by = by;
            }
        }
        TreeHit oth;
        const int flags = __shfl_xor_sync(pm, int(mine.hit) | (int(mine.back) << 1), 1);
        oth.hit = (flags & 1) != 0;
        oth.back = (flags & 2) != 0;
        oth.dist = __shfl_xor_sync(pm, mine.dist, 1);
        oth.tri = __shfl_xor_sync(pm, mine.tri, 1);
        oth.bx = __shfl_xor_sync(pm, mine.bx, 1);
        oth.by = __shfl_xor_sync(pm, mine.by, 1);
        const bool take = oth.dist < mine.dist || (!(mine.dist < oth.dist) && oth.tri < mine.tri);
        best = take ? oth : mine;
    }
    return best;
}

struct Mat3s {
    float3 c0, c1, c2;
};
__device__ __forceinline__ Mat3s cofactor(const Mat4& M) {
    const float m00 = M.c0.x, m01 = M.c0.y, m02 = M.c0.z;  // m<column><row>
    const float m10 = M.c1.x, m11 = M.c1.y, m12 = M.c1.z;
    const float m20 = M.c2.x, m21 = M.c2.y, m22 = M.c2.z;
    Mat3s R;
    R.c0 = make_float3(m11 * m22 - m21 * m12, m20 * m12 - m10 * m22, m10 * m21 - m20 * m11);
    R.c1 = make_float3(m21 * m02 - m01 * m22, m00 * m22 - m20 * m02, m20 * m01 - m00 * m21);
    R.c2 = make_float3(m01 * m12 - m11 * m02, m10 * m02 - m00 * m12, m00 * m11 - m10 * m01);
    return R;
}
__device__ __forceinline__ float3 mul3s(const Mat3s& N, float3 v) {
    return make_float3((N.c0.x * v.x + N.c1.x * v.y) + N.c2.x * v.z, (N.c0.y * v.x + N.c1.y * v.y) + N.c2.y * v.z,
                       (N.c0.z * v.x + N.c1.z * v.y) + N.c2.z * v.z);
}

__device__ __forceinline__ float3 add3s(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 scale3s(float s, float3 v) { return make_float3(s * v.x, s * v.y, s * v.z); }
__device__ __forceinline__ float3 neg3(float3 v) { return make_float3(-v.x, -v.y, -v.z); }

struct Side {
    uint32_t root;      // root record
    uint32_t tri_base;
    const float* nrm;   // per-vertex normals [n_tris][9], or null (face normal)
    Mat4 m;
};

struct Pass {
    bool ok;
    float3 response, normal;
};

// The lanes of a ray: a quad; lanes 0-1 and 2-3 are the pairs of the two
// traversals of a pass.
struct Quad {
    uint32_t q;     // lane within the quad
    uint32_t base;  // the quad's first lane in the warp
    unsigned qm;    // the quad's mask
    unsigned pm;    // the lane pair's mask
};

__device__ __forceinline__ TreeHit shfl_hit(const TreeHit& h, uint32_t src, unsigned m) {
    TreeHit o;
    const int f = __shfl_sync(m, int(h.hit) | (int(h.back) << 1), src);
    o.hit = (f & 1) != 0;
    o.back = (f & 2) != 0;
    o.dist = __shfl_sync(m, h.dist, src);
    o.tri = __shfl_sync(m, h.tri, src);
    o.bx = __shfl_sync(m, h.bx, src);
    o.by = __shfl_sync(m, h.by, src);
    return o;
}

// ShootUncollideRays::HermannPass (ShootUncollideRays.cpp:127-158). Its two
// traversals (the closest hit on B from the origin, on A from the origin moved
// by 4 ulps) do not depend on each other: lane pair 0 runs the first, pair 1
// the second (which the reference skips when the first fails; its result is
// then unused), and the quad shares both.
__device__ Pass hermann(const ShootParams& P, const Side& A, const Side& B, const Mat3s& nb, float3 o, float3 d,
                        const Quad& L) {
    Pass r{false, make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f)};
    // Ray::MoveOriginEpsilonTowardsDirection(4) (Ray.cpp:13-20)
    const float big = fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
    const float eps = big * FLT_EPSILON;
    const float3 moved = add3s(o, scale3s(4.f * eps, d));
    const float eps_dist = length3(sub3(moved, o));
    const bool own = (L.q >> 1) != 0u;
    const TreeHit h = ray_tree(P.recs, P.tris, own ? A.root : B.root, own ? A.m : B.m, own ? moved : o, d, P.error,
                               L.q & 1u, L.pm);
    const TreeHit p2 = shfl_hit(h, L.base, L.qm);
    const TreeHit p3 = shfl_hit(h, L.base + 2u, L.qm);
    if (!(p2.hit && p2.back)) return r;
    if (p2.dist <= p3.dist + eps_dist) {
        r.ok = true;
        r.response = scale3s(p2.dist, d);
        // TriangleNormal::GetNormal(bary, matrix) (Triangle.cpp:197-204)
        float3 n0, n1, n2;
        const uint32_t local = p2.tri - B.tri_base;
        if (B.nrm) {
            const float* nn = B.nrm + 9ull * local;
            n0 = make_float3(nn[0], nn[1], nn[2]);
            n1 = make_float3(nn[3], nn[4], nn[5]);
            n2 = make_float3(nn[6], nn[7], nn[8]);
        } else {
            const float4* t4 = P.tris + 3ull * p2.tri;
            const float4 a = __ldg(t4), b = __ldg(t4 + 1), c = __ldg(t4 + 2);
            n0 = n1 = n2 = normalize3(cross3(sub3(make_float3(b.x, b.y, b.z), make_float3(a.x, a.y, a.z)),
                                             sub3(make_float3(c.x, c.y, c.z), make_float3(a.x, a.y, a.z))));
        }
        const float b0 = (1.f - p2.bx) - p2.by;
        const float3 n = add3s(add3s(scale3s(b0, n0), scale3s(p2.bx, n1)), scale3s(p2.by, n2));
        r.normal = normalize3(mul3s(nb, n));
    }
    return r;
}

// ShootUncollideRays::CalcForceResponse (ShootUncollideRays.cpp:116-125).
__device__ __forceinline__ float3 force_response(const Pass& h) {
    const float3 dir = normalize3(h.response);
    const float len = length3(h.response);
    const float c = dot3(h.normal, dir);
    return scale3s(c * c * len, dir);
}

__device__ __forceinline__ void put3(float* p, float3 v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
__device__ __forceinline__ float3 get3(const float* p) { return make_float3(p[0], p[1], p[2]); }

__device__ __forceinline__ Mat4 mat_of(const float* m) {
    return Mat4{make_float4(m[0], m[1], m[2], m[3]), make_float4(m[4], m[5], m[6], m[7]),
                make_float4(m[8], m[9], m[10], m[11]), make_float4(m[12], m[13], m[14], m[15])};
}

// Four lanes per ray (a quad), the rays strided over the grid.
__global__ void __launch_bounds__(128, 6) shoot_ray_kernel(const ShootParams P) {
    uint32_t nr = P.n_rays;
    if (P.n_rays_dev) {
        const uint32_t v = *P.n_rays_dev;
        nr = v < nr ? v : nr;
    }
    Quad L;
    const uint32_t lane = threadIdx.x & 31u;
    L.q = lane & 3u;
    L.base = lane & ~3u;
    L.qm = 0xfu << L.base;
    L.pm = 0x3u << (lane & ~1u);
    const uint32_t stride = (gridDim.x * blockDim.x) >> 2;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; i < nr; i += stride) {
        const uint32_t tag = P.ray_query[i];
        const uint32_t qi = tag & 0x7fffffffu;
        const bool from_second = (tag >> 31) != 0;
        const ShootQuery& Q = P.q[qi];
        if (!Q.pad[0]) {  // a pair that is not shot
            if (L.q == 0u) {
                ShootRayOut none;
                none.ok1 = none.ok2 = 0u;
                P.out[i] = none;
            }
            continue;
        }
        const DevTree& TA = P.trees[Q.tree_a];
        const DevTree& TB = P.trees[Q.tree_b];
        const Mat4 M = mat_of(Q.relative);
        const Mat4 I = Mat4{make_float4(1.f, 0.f, 0.f, 0.f), make_float4(0.f, 1.f, 0.f, 0.f),
                            make_float4(0.f, 0.f, 1.f, 0.f), make_float4(0.f, 0.f, 0.f, 1.f)};
        const Mat3s N = cofactor(M);
        const Mat3s I3 = Mat3s{make_float3(1.f, 0.f, 0.f), make_float3(0.f, 1.f, 0.f), make_float3(0.f, 0.f, 1.f)};
        const Side first{TA.rec_base + 1u, TA.tri_base, TA.nrm, I};
        const Side second{TB.rec_base + 1u, TB.tri_base, TB.nrm, M};
        const float* ray = P.rays + 6ull * i;
        const float3 o = get3(ray), d = get3(ray + 3);
        // The ray's pass, then (when it succeeds) its reflection's pass back, in
        // one loop so that the traversal code exists once. First to second: the
        // pass against the second entity (force subtracted, response negated);
        // second to first: against the first entity.
        float3 res[4];  // f1, r1, f2, r2
        uint32_t ok = 0;
        float3 po = o, pd = d;
        bool to_first = from_second;
#pragma unroll 1
        for (uint32_t k = 0; k < 2u; ++k) {
            const Pass h = hermann(P, to_first ? second : first, to_first ? first : second, to_first ? I3 : N, po, pd,
                                   L);
            if (!h.ok) break;
            const float3 fr = force_response(h);
            res[2 * k] = to_first ? fr : neg3(fr);
            res[2 * k + 1] = to_first ? h.response : neg3(h.response);
            ok = k + 1u;
            // ShootUncollideRays::ReflectHermannResult (ShootUncollideRays.cpp:100-106)
            po = add3s(o, h.response);
            pd = neg3(h.normal);
            to_first = !to_first;
        }
        if (L.q == 0u) {
            ShootRayOut out;
            out.ok1 = ok >= 1u ? 1u : 0u;
            out.ok2 = ok >= 2u ? 1u : 0u;
            if (ok >= 1u) put3(out.f1, res[0]), put3(out.r1, res[1]);
            if (ok >= 2u) put3(out.f2, res[2]), put3(out.r2, res[3]);
            P.out[i] = out;
        }
    }
}

// ShootUncollideRays::SmootherStep (ShootUncollideRays.cpp:175-179).
__device__ __forceinline__ float smoother_step(float a, float b, float x) {
    float v = (x - a) / (b - a);
    v = (v < 0.f) ? 0.f : ((1.f < v) ? 1.f : v);
    return v * v * v * (v * (v * 6.f - 15.f) + 10.f);
}

// A warp per pair: the force responses summed in the reference's order (a
// float sum is order-dependent), FindResponse's maximum over the ray
// responses split over the lanes (a maximum is not), then the delta.
__global__ void __launch_bounds__(128) shoot_query_kernel(const ShootParams P) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t qi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; qi < P.n_queries; qi += warps) {
        const ShootQuery& Q = P.q[qi];
        const uint32_t r0 = Q.ray_first, r1 = Q.ray_first + Q.n_first + Q.n_second;
        // the lanes load 32 rays' responses at a time; every lane then adds
        // them in ray order from the shuffles (the same sum on all lanes)
        float3 avg = make_float3(0.f, 0.f, 0.f);
        for (uint32_t base = r0; base < r1; base += 32u) {
            const uint32_t i = base + lane;
            uint32_t ok = 0u;
            float3 f1 = make_float3(0.f, 0.f, 0.f), f2 = f1;
            if (i < r1) {
                const ShootRayOut& o = P.out[i];
                ok = (o.ok1 ? 1u : 0u) | (o.ok2 ? 2u : 0u);
                if (ok & 1u) f1 = get3(o.f1);
                if (ok & 2u) f2 = get3(o.f2);
            }
            const uint32_t m = (r1 - base) < 32u ? (r1 - base) : 32u;
            for (uint32_t j = 0; j < m; ++j) {
                const uint32_t k = __shfl_sync(0xffffffffu, ok, j);
                const float3 a = make_float3(__shfl_sync(0xffffffffu, f1.x, j), __shfl_sync(0xffffffffu, f1.y, j),
                                             __shfl_sync(0xffffffffu, f1.z, j));
                const float3 b = make_float3(__shfl_sync(0xffffffffu, f2.x, j), __shfl_sync(0xffffffffu, f2.y, j),
                                             __shfl_sync(0xffffffffu, f2.z, j));
                if (k & 1u) avg = add3s(avg, a);
                if (k & 2u) avg = add3s(avg, b);
            }
        }
        float3 delta = make_float3(0.f, 0.f, 0.f);
        if (avg.x != 0.f || avg.y != 0.f || avg.z != 0.f) {
            const float3 nf = normalize3(avg);
            float max_len = 0.f;
            auto one = [&](float3 r) {
                const float3 nr = normalize3(r);
                const float dt = dot3(nr, nf);
                const float len = length3(r);
                const float need = len / dt;
                const float x = smoother_step(P.cos_finish, P.cos_start, dt) * need;
                max_len = (max_len < x) ? x : max_len;
            };
            for (uint32_t i = r0 + lane; i < r1; i += 32u) {
                const ShootRayOut& o = P.out[i];
                if (o.ok1) one(get3(o.r1));
                if (o.ok2) one(get3(o.r2));
            }
#pragma unroll
            for (int w = 16; w; w >>= 1) {
                const float x = __shfl_xor_sync(0xffffffffu, max_len, w);
                max_len = (max_len < x) ? x : max_len;
            }
            const float3 local = scale3s(P.bias, scale3s(max_len, nf));
            delta = xform(mat_of(Q.first_global), local, 0.f);
        }
        if (lane == 0u) put3(P.deltas + 3ull * qi, delta);
    }
}

}  // namespace

cudaError_t launch_shoot(const ShootParams& p, cudaStream_t s) {
    if (p.n_rays) {
        const uint64_t blocks = (4ull * p.n_rays + 127u) / 128u;  // a quad per ray, strided beyond 8192 blocks
        shoot_ray_kernel<<<uint32_t(blocks < 8192u ? blocks : 8192u), 128, 0, s>>>(p);
    }
    if (p.n_queries) {
        const uint32_t blocks = (p.n_queries + 3u) / 4u;  // a warp per pair
        shoot_query_kernel<<<blocks < 65535u ? blocks : 65535u, 128, 0, s>>>(p);
    }
    return cudaGetLastError();
}

}  // namespace cg
