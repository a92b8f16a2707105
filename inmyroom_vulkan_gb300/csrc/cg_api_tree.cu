// The C ABI's trees built on the device (cg_tree_build: the build kernels of
// cg_build.cu, then the layout written into the arenas), their flat layout
// read back (cg_tree_info, cg_tree_export) and the tree cache file
// (cg_tree_save, cg_tree_load).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "cg_ctx.h"

using namespace cg_host;

namespace {
inline uint32_t bits_of(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
}  // namespace

namespace {
constexpr char kCacheMagic[8] = {'C', 'G', 'T', 'R', 'E', 'E', '0', '1'};

uint64_t fnv1a(const unsigned char* p, size_t n, uint64_t h = 1469598103934665603ull) {
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}
}  // namespace

int cg_tree_build(cg_ctx* c, const cg_mesh_view* meshes, uint32_t n, uint32_t* tree_ids) {
    if (!c || (n && (!meshes || !tree_ids))) return CG_ERR_INVALID_ARGUMENT;
    if (n == 0) return CG_OK;
    std::vector<uint64_t> base(n + 1, 0), vbase(n + 1, 0);
    bool any_normals = false;
    for (uint32_t i = 0; i < n; ++i) {
        const cg_mesh_view& m = meshes[i];
        if (m.n_triangles && (!m.positions || !m.indices))
            return fail(c, CG_ERR_INVALID_ARGUMENT, "mesh %u has null positions or indices", i);
        // vertex indices are checked on the device, as the triangles are gathered
        any_normals |= m.normals != nullptr && m.n_triangles;
        base[i + 1] = base[i] + m.n_triangles;
        vbase[i + 1] = vbase[i] + (m.n_triangles ? m.n_vertices : 0u);
    }
    const uint64_t total = base[n], nv = vbase[n];
    if (total > 0x3fffffffull || nv > 0xffffffffull)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "%llu triangles in one build", (unsigned long long)total);
    const uint64_t T = std::max<uint64_t>(total, 1);
    const uint32_t cap = uint32_t(2 * total + n);
    // the scratch: carved in 256-byte steps
    auto up = [](size_t x) { return (x + 255u) & ~size_t(255); };
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += up(bytes);
        return o;
    };
    const size_t oP = take(sizeof(float) * 9 * T), oPp = take(sizeof(float) * 9 * T);
    const size_t oCN = take(any_normals ? sizeof(float) * 9 * T : 0);
    const size_t oPerm = take(4 * T), oScr = take(4 * T), oOwn = take(4 * T);
    const size_t oD = take(sizeof(double) * 9 * T), oTm = take(sizeof(double) * 18 * T);
    const size_t oMom = take(sizeof(double) * 9 * std::max<uint64_t>(T, n));  // a level: one node per triangle, or the roots
    // counters: next node, error, large nodes by level parity; then the first bad vertex index
    struct LevelState {
        uint32_t ctr[4];
        unsigned long long bad;
    };
    const size_t oNodes = take(sizeof(BuildNode) * cap), oFlat = take(sizeof(BuildFlat) * cap),
                 oCtr = take(sizeof(LevelState));
    const size_t oSegs = take(sizeof(PullSeg) * 3 * n);
    // a level's nodes of more than kBuildBig triangles: the roots, or disjoint
    // ranges of more than kBuildBig triangles each
    const uint64_t big_cap = n + T / (kBuildBig + 1) + 1;
    const size_t oBig = take(sizeof(uint32_t) * 2 * big_cap);
    const size_t oV = take(sizeof(float) * 3 * std::max<uint64_t>(nv, 1));
    const size_t oNV = take(any_normals ? sizeof(float) * 3 * std::max<uint64_t>(nv, 1) : 0);
    const size_t oIdx = take(sizeof(uint32_t) * 3 * T), oMesh = take(sizeof(BuildMesh) * n);
    const size_t oEmit = take(sizeof(BuildEmit) * n);
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    if (off > c->build_cap) {
        CG_CUDA(cudaStreamSynchronize(s), "build scratch");
        cudaFree(c->build);
        c->build = nullptr;
        c->build_cap = 0;
        CG_CUDA(cudaMalloc(&c->build, off), "alloc build scratch");
        c->build_cap = off;
    }
    char* mem = static_cast<char*>(c->build);
    BuildParams bp{};
    BuildInput in{};
    in.P = reinterpret_cast<float*>(mem + oP);
    in.corner_normals = any_normals ? reinterpret_cast<float*>(mem + oCN) : nullptr;
    bp.P = in.P;
    bp.Pp = reinterpret_cast<float*>(mem + oPp);
    bp.perm = reinterpret_cast<uint32_t*>(mem + oPerm);
    bp.scratch = reinterpret_cast<uint32_t*>(mem + oScr);
    bp.own = reinterpret_cast<uint32_t*>(mem + oOwn);
    bp.D = reinterpret_cast<double*>(mem + oD);
    bp.Tm = reinterpret_cast<double*>(mem + oTm);
    bp.mom = reinterpret_cast<double*>(mem + oMom);
    bp.nodes = reinterpret_cast<BuildNode*>(mem + oNodes);
    BuildFlat* flat = reinterpret_cast<BuildFlat*>(mem + oFlat);
    bp.node_ctr = reinterpret_cast<uint32_t*>(mem + oCtr);
    bp.error = bp.node_ctr + 1;
    in.bad = reinterpret_cast<unsigned long long*>(mem + oCtr + offsetof(LevelState, bad));
    bp.node_cap = cap;
    bp.T = uint32_t(total);
    uint32_t* big_list[2] = {reinterpret_cast<uint32_t*>(mem + oBig), reinterpret_cast<uint32_t*>(mem + oBig) + big_cap};
    float* d_V = reinterpret_cast<float*>(mem + oV);
    float* d_NV = any_normals ? reinterpret_cast<float*>(mem + oNV) : nullptr;
    uint32_t* d_idx = reinterpret_cast<uint32_t*>(mem + oIdx);
    BuildMesh* d_mesh = reinterpret_cast<BuildMesh*>(mem + oMesh);
    BuildEmit* d_emit = reinterpret_cast<BuildEmit*>(mem + oEmit);
    in.meshes = d_mesh;
    in.vertices = d_V;
    in.normals = d_NV;
    in.indices = d_idx;
    // the meshes' buffers, one after another: pulled by the device from the
    // caller's arrays where it reads pageable host memory, else copied
    std::vector<BuildMesh> mt(n);
    std::vector<BuildNode> roots(n);
    std::vector<PullSeg> segs;
    uint64_t seg_max = 0;
    auto pull = [&](const void* src, void* dst, uint64_t words) {
        segs.push_back(PullSeg{static_cast<const uint32_t*>(src), static_cast<uint32_t*>(dst), words});
        seg_max = std::max(seg_max, words);
    };
    for (uint32_t i = 0; i < n; ++i) {
        const cg_mesh_view& m = meshes[i];
        mt[i] = BuildMesh{uint32_t(vbase[i]), (m.normals && m.n_triangles) ? 1u : 0u, uint32_t(base[i]),
                          m.n_triangles ? m.n_vertices : 0u};
        roots[i] = BuildNode{};
        roots[i].begin = uint32_t(base[i]);
        roots[i].count = m.n_triangles;
        roots[i].kid = kNoKid;
        roots[i].tree = i;
        if (!m.n_triangles) continue;
        // the device's 4-byte loads need 4-byte aligned arrays; others are copied
        auto word_aligned = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) == 0; };
        if (c->pageable_access && word_aligned(m.positions) && word_aligned(m.normals) && word_aligned(m.indices)) {
            if (m.n_vertices) pull(m.positions, d_V + 3 * vbase[i], 3ull * m.n_vertices);
            if (m.normals && m.n_vertices) pull(m.normals, d_NV + 3 * vbase[i], 3ull * m.n_vertices);
            pull(m.indices, d_idx + 3 * base[i], 3ull * m.n_triangles);
            continue;
        }
        CG_CUDA(cudaMemcpyAsync(d_V + 3 * vbase[i], m.positions, sizeof(float) * 3 * m.n_vertices,
                                cudaMemcpyHostToDevice, s),
                "upload vertices");
        if (m.normals)
            CG_CUDA(cudaMemcpyAsync(d_NV + 3 * vbase[i], m.normals, sizeof(float) * 3 * m.n_vertices,
                                    cudaMemcpyHostToDevice, s),
                    "upload normals");
        CG_CUDA(cudaMemcpyAsync(d_idx + 3 * base[i], m.indices, sizeof(uint32_t) * 3 * m.n_triangles,
                                cudaMemcpyHostToDevice, s),
                "upload indices");
    }
    if (!segs.empty()) {
        PullSeg* d_segs = reinterpret_cast<PullSeg*>(mem + oSegs);
        CG_CUDA(cudaMemcpyAsync(d_segs, segs.data(), sizeof(PullSeg) * segs.size(), cudaMemcpyHostToDevice, s),
                "upload mesh table");
        CG_CUDA(launch_build_pull(d_segs, uint32_t(segs.size()), seg_max, s), "pull meshes");
    }
    const LevelState st0{{n, 0u, 0u, 0u}, ~0ull};
    std::vector<uint32_t> big_roots;
    for (uint32_t i = 0; i < n; ++i)
        if (roots[i].count > kBuildBig) big_roots.push_back(i);
    CG_CUDA(cudaMemcpyAsync(d_mesh, mt.data(), sizeof(BuildMesh) * n, cudaMemcpyHostToDevice, s), "upload meshes");
    CG_CUDA(cudaMemcpyAsync(bp.nodes, roots.data(), sizeof(BuildNode) * n, cudaMemcpyHostToDevice, s), "upload roots");
    CG_CUDA(cudaMemcpyAsync(bp.node_ctr, &st0, sizeof(st0), cudaMemcpyHostToDevice, s), "upload counter");
    if (!big_roots.empty())
        CG_CUDA(cudaMemcpyAsync(big_list[0], big_roots.data(), sizeof(uint32_t) * big_roots.size(),
                                cudaMemcpyHostToDevice, s),
                "upload large roots");
    const uint32_t sms = uint32_t(c->sm_count);
    CG_CUDA(launch_build_gather(bp, in, n, sms, s), "gather kernel");
    // one level per round of launches; the splits' children are the next level
    std::vector<std::pair<uint32_t, uint32_t>> levels;
    uint32_t lo = 0, hi = n, n_big = uint32_t(big_roots.size());
    for (uint32_t level = 0; lo < hi; ++level) {
        const uint32_t in = level & 1u, out = in ^ 1u;
        bp.lo = lo;
        bp.hi = hi;
        bp.big = big_list[in];
        bp.n_big = n_big;
        bp.big_out = big_list[out];
        bp.n_big_out = bp.node_ctr + 2 + out;
        levels.emplace_back(lo, hi);
        CG_CUDA(cudaMemsetAsync(bp.n_big_out, 0, sizeof(uint32_t), s), "clear large node count");
        CG_CUDA(launch_build_level(bp, sms, s), "build level kernels");
        LevelState st;
        CG_CUDA(cudaMemcpyAsync(&st, bp.node_ctr, sizeof(st), cudaMemcpyDeviceToHost, s), "read node count");
        CG_CUDA(cudaStreamSynchronize(s), "build level");
        if (st.bad != ~0ull) {
            const uint32_t i = uint32_t(st.bad >> 32);
            const uint64_t k = st.bad & 0xffffffffull;
            return fail(c, CG_ERR_BAD_TREE, "mesh %u index %llu is vertex %u of %u", i, (unsigned long long)k,
                        meshes[i].indices[k], meshes[i].n_vertices);
        }
        if (st.ctr[1]) return fail(c, CG_ERR_OUT_OF_MEMORY, "tree build ran out of node slots");
        lo = hi;
        hi = std::min(st.ctr[0], cap);
        n_big = st.ctr[2 + out];
    }
    const uint32_t n_nodes = hi;
    // the pre-order layout: subtree sizes bottom-up, places top-down
    for (size_t l = levels.size(); l-- > 0;) {
        bp.lo = levels[l].first;
        bp.hi = levels[l].second;
        CG_CUDA(launch_build_inner(bp, flat, sms, s), "layout kernel");
    }
    for (const auto& lv : levels) {
        bp.lo = lv.first;
        bp.hi = lv.second;
        CG_CUDA(launch_build_order(bp, flat, n, sms, s), "layout kernel");
    }
    std::vector<BuildFlat> rootflat(n);
    CG_CUDA(cudaMemcpyAsync(rootflat.data(), flat, sizeof(BuildFlat) * n, cudaMemcpyDeviceToHost, s), "read layout");
    CG_CUDA(cudaStreamSynchronize(s), "tree layout");
    // arena places and the trees' side arrays (one block for the batch)
    struct Place {
        uint64_t rpair, n_recs, tb, n_tris, nrm, ranges, topo;
        uint32_t n_leaves;
    };
    std::vector<Place> pl(n);
    size_t aux = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint64_t N = rootflat[i].inner, Ti = meshes[i].n_triangles;
        Place& p = pl[i];
        p.n_recs = 2 * N + 2;
        p.n_tris = std::max<uint64_t>(Ti, 1);
        p.n_leaves = uint32_t(N + 1);
        p.nrm = mt[i].has_normals ? aux : ~0ull;
        if (mt[i].has_normals) aux += up(sizeof(float) * 9 * Ti);
        p.ranges = aux;
        aux += up(sizeof(uint2) * p.n_recs);
        p.topo = aux;
        aux += up(sizeof(uint32_t) * (p.n_recs + p.n_leaves));
    }
    void* block = nullptr;
    CG_CUDA(cudaMalloc(&block, aux), "alloc tree side arrays");
    std::shared_ptr<void> pool(block, [](void* q) { cudaFree(q); });
    uint32_t done = 0;
    auto undo = [&]() {
        for (uint32_t j = 0; j < done; ++j) {
            c->recs.release(pl[j].rpair, pl[j].n_recs / 2);
            c->tris.release(pl[j].tb, pl[j].n_tris);
        }
    };
    for (; done < n; ++done) {
        Place& p = pl[done];
        cudaError_t e = c->recs.alloc(p.n_recs / 2, &p.rpair, s);
        if (e != cudaSuccess) {
            undo();
            return cuda_fail(c, e, "record arena");
        }
        e = c->tris.alloc(p.n_tris, &p.tb, s);
        if (e != cudaSuccess) {
            c->recs.release(p.rpair, p.n_recs / 2);
            undo();
            return cuda_fail(c, e, "triangle arena");
        }
        if (2 * p.rpair + p.n_recs > 0xffffffffull || p.tb + p.n_tris > 0x7fffffffull) {
            c->recs.release(p.rpair, p.n_recs / 2);
            c->tris.release(p.tb, p.n_tris);
            undo();
            return fail(c, CG_ERR_OUT_OF_MEMORY, "arena index space exhausted");
        }
    }
    char* ab = static_cast<char*>(block);
    std::vector<BuildEmit> em(n);
    for (uint32_t i = 0; i < n; ++i) {
        const Place& p = pl[i];
        em[i] = BuildEmit{uint32_t(2 * p.rpair), uint32_t(p.tb), uint32_t(p.n_recs), 0u,
                          p.nrm == ~0ull ? nullptr : reinterpret_cast<float*>(ab + p.nrm),
                          reinterpret_cast<uint2*>(ab + p.ranges), reinterpret_cast<uint32_t*>(ab + p.topo)};
    }
    // from here on a failure gives the arena places back
    cudaError_t e = cudaMemcpyAsync(d_emit, em.data(), sizeof(BuildEmit) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_build_emit(bp, in, flat, d_emit, c->recs.ptr, c->tris.ptr, n_nodes, n, sms, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        undo();
        return cuda_fail(c, e, "tree layout kernels");
    }
    for (uint32_t i = 0; i < n; ++i) {
        cg_ctx::Slot slot;
        slot.rec_base = em[i].rec_base;
        slot.n_recs = pl[i].n_recs;
        slot.tri_base = pl[i].tb;
        slot.n_tris = pl[i].n_tris;
        slot.n_tri_used = meshes[i].n_triangles;
        slot.nrm = em[i].nrm;
        slot.ranges = em[i].ranges;
        slot.topo = em[i].topo;
        slot.n_leaves = pl[i].n_leaves;
        slot.pool = pool;
        slot.live = true;
        uint32_t id = uint32_t(c->trees.size());
        for (uint32_t k = 0; k < c->trees.size(); ++k)
            if (!c->trees[k].live) {
                id = k;
                break;
            }
        if (id == c->trees.size())
            c->trees.push_back(slot);
        else
            c->trees[id] = slot;
        tree_ids[i] = id;
    }
    return sync_tree_table(c);
}

int cg_tree_info(cg_ctx* c, uint32_t id, uint32_t* node_count, uint32_t* triangle_count, uint32_t* has_normals) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (id >= c->trees.size() || !c->trees[id].live) return fail(c, CG_ERR_NOT_FOUND, "tree %u", id);
    const auto& t = c->trees[id];
    if (node_count) *node_count = uint32_t((t.n_recs - 2) / 2);
    if (triangle_count) *triangle_count = t.n_tri_used;
    if (has_normals) *has_normals = t.nrm ? 1u : 0u;
    return CG_OK;
}

int cg_tree_export(cg_ctx* c, uint32_t id, cg_obb* root, cg_obb* node_obbs, uint32_t* node_ref,
                   uint32_t* node_tri_count, float* triangles_position, float* triangles_normal,
                   uint32_t* triangles_indices) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (id >= c->trees.size() || !c->trees[id].live) return fail(c, CG_ERR_NOT_FOUND, "tree %u", id);
    const auto& t = c->trees[id];
    const uint32_t N = uint32_t((t.n_recs - 2) / 2), T = t.n_tri_used;
    cudaSetDevice(c->device);
    CG_CUDA(cudaStreamSynchronize(c->stream), "export tree");
    std::vector<float4> recs(4ull * t.n_recs);
    CG_CUDA(cudaMemcpy(recs.data(), c->recs.ptr + 4 * t.rec_base, sizeof(float4) * recs.size(), cudaMemcpyDeviceToHost),
            "read records");
    auto unbox = [](const float4* r, cg_obb* b) {
        b->center[0] = r[0].x, b->center[1] = r[0].y, b->center[2] = r[0].z;
        b->u[0] = r[0].w, b->u[1] = r[1].x, b->u[2] = r[1].y;
        b->v[0] = r[1].z, b->v[1] = r[1].w, b->v[2] = r[2].x;
        b->w[0] = r[2].y, b->w[1] = r[2].z, b->w[2] = r[2].w;
    };
    if (root) unbox(&recs[4], root);
    for (uint32_t r = 2; r < t.n_recs; ++r) {
        const float4* q = &recs[4ull * r];
        if (node_obbs) unbox(q, node_obbs + (r - 2));
        const uint32_t ref = bits_of(q[3].x), meta = bits_of(q[3].y);
        const bool leaf = (meta & kLeafFlag) != 0u;
        if (node_ref) node_ref[r - 2] = leaf ? uint32_t(ref - t.tri_base) : uint32_t((ref - t.rec_base - 2) / 2);
        if (node_tri_count) node_tri_count[r - 2] = leaf ? (meta & 0xffffu) : 0u;
    }
    if (T && (triangles_position || triangles_indices)) {
        std::vector<float4> tris(3ull * T);
        CG_CUDA(cudaMemcpy(tris.data(), c->tris.ptr + 3 * t.tri_base, sizeof(float4) * tris.size(),
                           cudaMemcpyDeviceToHost),
                "read triangles");
        for (size_t k = 0; k < tris.size(); ++k) {
            if (triangles_position) {
                triangles_position[3 * k] = tris[k].x;
                triangles_position[3 * k + 1] = tris[k].y;
                triangles_position[3 * k + 2] = tris[k].z;
            }
            if (triangles_indices) triangles_indices[k] = bits_of(tris[k].w);
        }
    }
    if (T && triangles_normal && t.nrm)
        CG_CUDA(cudaMemcpy(triangles_normal, t.nrm, sizeof(float) * 9ull * T, cudaMemcpyDeviceToHost), "read normals");
    return CG_OK;
}

int cg_tree_save(cg_ctx* c, uint32_t id, const char* path) {
    if (!c || !path) return CG_ERR_INVALID_ARGUMENT;
    uint32_t N = 0, T = 0, has_nrm = 0;
    int rc = cg_tree_info(c, id, &N, &T, &has_nrm);
    if (rc != CG_OK) return rc;
    cg_obb root;
    std::vector<cg_obb> obbs(2ull * N);
    std::vector<uint32_t> ref(2ull * N), cnt(2ull * N), idx(3ull * T);
    std::vector<float> pos(9ull * T), nrm(has_nrm ? 9ull * T : 0);
    rc = cg_tree_export(c, id, &root, obbs.data(), ref.data(), cnt.data(), pos.data(), has_nrm ? nrm.data() : nullptr,
                        idx.data());
    if (rc != CG_OK) return rc;
    std::vector<unsigned char> buf;
    auto put = [&](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        buf.insert(buf.end(), b, b + n);
    };
    const uint32_t head[3] = {N, T, has_nrm ? 1u : 0u};
    put(kCacheMagic, 8);
    put(head, sizeof(head));
    put(&root, sizeof(root));
    put(obbs.data(), sizeof(cg_obb) * obbs.size());
    put(ref.data(), 4 * ref.size());
    put(cnt.data(), 4 * cnt.size());
    put(pos.data(), 4 * pos.size());
    put(nrm.data(), 4 * nrm.size());
    put(idx.data(), 4 * idx.size());
    const uint64_t h = fnv1a(buf.data(), buf.size());
    put(&h, 8);
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(c, CG_ERR_INVALID_ARGUMENT, "cannot write %s", path);
    const size_t w = std::fwrite(buf.data(), 1, buf.size(), f);
    const int closed = std::fclose(f);
    if (w != buf.size() || closed != 0) return fail(c, CG_ERR_INVALID_ARGUMENT, "short write to %s", path);
    return CG_OK;
}

int cg_tree_load(cg_ctx* c, const char* path, uint32_t* tree_id) {
    if (!c || !path || !tree_id) return CG_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(c, CG_ERR_NOT_FOUND, "cannot read %s", path);
    std::vector<unsigned char> buf;
    unsigned char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    std::fclose(f);
    const size_t fixed = 8 + 12 + sizeof(cg_obb) + 8;
    if (buf.size() < fixed || std::memcmp(buf.data(), kCacheMagic, 8) != 0)
        return fail(c, CG_ERR_BAD_TREE, "%s is not a tree cache file", path);
    uint32_t head[3];
    std::memcpy(head, buf.data() + 8, sizeof(head));
    const uint64_t N = head[0], T = head[1];
    const bool has_nrm = (head[2] & 1u) != 0;
    const uint64_t need = fixed + N * (2 * sizeof(cg_obb) + 16) + T * (36 + (has_nrm ? 36 : 0) + 12);
    if (buf.size() != need) return fail(c, CG_ERR_BAD_TREE, "%s: %zu bytes, its header says %llu", path, buf.size(),
                                        (unsigned long long)need);
    uint64_t h;
    std::memcpy(&h, buf.data() + need - 8, 8);
    if (h != fnv1a(buf.data(), need - 8)) return fail(c, CG_ERR_BAD_TREE, "%s: checksum mismatch", path);
    const unsigned char* p = buf.data() + 20;
    cg_obb root;
    std::memcpy(&root, p, sizeof(root));
    p += sizeof(root);
    std::vector<cg_obb> obbs(2 * N);
    std::vector<uint32_t> ref(2 * N), cnt(2 * N), idx(3 * T);
    std::vector<float> pos(9 * T), nrm(has_nrm ? 9 * T : 0);
    auto get = [&](void* d, size_t n) {
        if (n) std::memcpy(d, p, n);
        p += n;
    };
    get(obbs.data(), sizeof(cg_obb) * obbs.size());
    get(ref.data(), 4 * ref.size());
    get(cnt.data(), 4 * cnt.size());
    get(pos.data(), 4 * pos.size());
    get(nrm.data(), 4 * nrm.size());
    get(idx.data(), 4 * idx.size());
    cg_tree_view v{};
    v.root_obb = root;
    v.node_count = uint32_t(N);
    v.node_obbs = obbs.data();
    v.node_ref = ref.data();
    v.node_tri_count = cnt.data();
    v.triangle_count = uint32_t(T);
    v.triangles_position = pos.data();
    v.triangles_normal = has_nrm ? nrm.data() : nullptr;
    v.triangles_indices = idx.data();
    return cg_tree_upload(c, &v, tree_id);
}
