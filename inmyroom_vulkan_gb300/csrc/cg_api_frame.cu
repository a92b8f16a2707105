// The C ABI's steps either side of the collide step: the broad phase
// (cg_broad_phase), the shooting of uncollide rays (cg_shoot_rays), one whole
// collision frame (cg_collision_frame) and the fan-out of its results to the
// entities' ancestors (cg_frame_callbacks).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "cg_ctx.h"

using namespace cg_host;

int cg_broad_phase(cg_ctx* c, const uint32_t* tree_ids, const float* globals, const uint8_t* callback, uint32_t n,
                   const float* axes, cg_entity_pair* pairs, uint64_t cap, uint64_t* n_pairs) {
    if (!c || !n_pairs || (n && (!tree_ids || !globals)) || (cap && !pairs)) return CG_ERR_INVALID_ARGUMENT;
    *n_pairs = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (tree_ids[i] >= c->trees.size() || !c->trees[tree_ids[i]].live)
            return fail(c, CG_ERR_NOT_FOUND, "entity %u names tree %u", i, tree_ids[i]);
    if (n < 2) return CG_OK;
    float ax[9];
    if (axes)
        std::memcpy(ax, axes, sizeof(ax));
    else
        engine_axes(ax);
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    auto up = [](size_t x) { return (x + 255u) & ~size_t(255); };
    const uint64_t pair_cap = std::max<uint64_t>(cap, 1);
    const size_t b_id = up(sizeof(uint32_t) * n), b_g = up(sizeof(float) * 16 * n), b_cb = up(n),
                 b_p = up(sizeof(float) * 6 * n), b_out = up(sizeof(uint2) * pair_cap), b_cnt = 256;
    const size_t need = b_id + b_g + b_cb + b_p + b_out + b_cnt;
    if (need > c->broad_cap) {
        CG_CUDA(cudaStreamSynchronize(s), "broad-phase buffers");
        cudaFree(c->broad);
        c->broad = nullptr;
        c->broad_cap = 0;
        CG_CUDA(cudaMalloc(&c->broad, need), "alloc broad-phase buffers");
        c->broad_cap = need;
    }
    char* base = static_cast<char*>(c->broad);
    BroadParams p{};
    uint32_t* d_ids = reinterpret_cast<uint32_t*>(base);
    float* d_g = reinterpret_cast<float*>(base + b_id);
    uint8_t* d_cb = reinterpret_cast<uint8_t*>(base + b_id + b_g);
    p.proj = reinterpret_cast<float*>(base + b_id + b_g + b_cb);
    p.pairs = reinterpret_cast<uint2*>(base + b_id + b_g + b_cb + b_p);
    p.count = reinterpret_cast<unsigned long long*>(base + b_id + b_g + b_cb + b_p + b_out);
    CG_CUDA(cudaMemcpyAsync(d_ids, tree_ids, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s), "upload ids");
    CG_CUDA(cudaMemcpyAsync(d_g, globals, sizeof(float) * 16 * n, cudaMemcpyHostToDevice, s), "upload matrices");
    if (callback) CG_CUDA(cudaMemcpyAsync(d_cb, callback, n, cudaMemcpyHostToDevice, s), "upload callbacks");
    CG_CUDA(cudaMemsetAsync(p.count, 0, sizeof(unsigned long long), s), "clear count");
    p.tree_ids = d_ids;
    p.trees = c->d_trees;
    p.recs = c->recs.ptr;
    p.globals = d_g;
    p.callback = callback ? d_cb : nullptr;
    p.n = n;
    for (int k = 0; k < 3; ++k) p.axes[k] = make_float3(ax[3 * k], ax[3 * k + 1], ax[3 * k + 2]);
    p.cap = cap;
    CG_CUDA(launch_broad(p, s), "broad-phase kernels");
    unsigned long long cnt = 0;
    CG_CUDA(cudaMemcpyAsync(&cnt, p.count, sizeof(cnt), cudaMemcpyDeviceToHost, s), "read count");
    CG_CUDA(cudaStreamSynchronize(s), "broad phase");
    *n_pairs = cnt;
    const uint64_t m = std::min<uint64_t>(cnt, cap);
    if (m) CG_CUDA(cudaMemcpy(pairs, p.pairs, sizeof(uint2) * m, cudaMemcpyDeviceToHost), "read pairs");
    return cnt > cap ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
}

int cg_collision_frame(cg_ctx* c, const cg_frame_entity* entities, uint32_t n, const cg_shoot_params* params,
                       cg_frame_result* results, uint64_t cap, uint64_t* n_results) {
    if (!c || !n_results || (n && !entities) || (cap && !results)) return CG_ERR_INVALID_ARGUMENT;
    *n_results = 0;
    if (!c->cfg.max_contacts || !c->cfg.max_tri_pairs)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "a collision frame needs max_contacts and max_tri_pairs > 0");
    for (uint32_t i = 0; i < n; ++i)
        if (entities[i].tree >= c->trees.size() || !c->trees[entities[i].tree].live)
            return fail(c, CG_ERR_NOT_FOUND, "entity %u names tree %u", i, entities[i].tree);
    if (n < 2) return CG_OK;  // CollisionDetection.cpp:40
    cg_shoot_params pr;
    cg_shoot_params_default(&pr);
    if (params) pr = *params;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    // broad phase, on the device
    std::vector<uint32_t> ids(n);
    std::vector<float> globals(16ull * n);
    std::vector<uint8_t> cbs(n);
    for (uint32_t i = 0; i < n; ++i) {
        ids[i] = entities[i].tree;
        std::memcpy(globals.data() + 16ull * i, entities[i].current_global, 16 * sizeof(float));
        cbs[i] = entities[i].should_callback ? 1u : 0u;
    }
    const uint32_t max_pairs = c->cfg.max_queries;
    const uint32_t max_rays = c->ct.max_rays;
    auto up = [](size_t x) { return (x + 255u) & ~size_t(255); };
    const size_t b_ent = up(sizeof(cg_frame_entity) * n), b_id = up(sizeof(uint32_t) * n),
                 b_g = up(sizeof(float) * 16 * n), b_cb = up(n), b_proj = up(sizeof(float) * 6 * n),
                 b_pairs = up(sizeof(uint2) * max_pairs), b_cnt = 256,
                 b_grp = up(sizeof(float) * 6 * max_rays), b_tag = up(sizeof(uint32_t) * max_rays),
                 b_sq = up(sizeof(ShootQuery) * max_pairs), b_so = up(sizeof(ShootRayOut) * max_rays),
                 b_dl = up(sizeof(float) * 3 * max_pairs), b_res = up(sizeof(cg_frame_result) * max_pairs);
    const size_t need = b_ent + b_id + b_g + b_cb + b_proj + b_pairs + b_cnt + b_grp + b_tag + b_sq + b_so +
                        b_dl + b_res + b_cnt;
    if (need > c->frame_cap) {
        CG_CUDA(cudaStreamSynchronize(s), "frame buffers");
        cudaFree(c->frame);
        c->frame = nullptr;
        c->frame_cap = 0;
        CG_CUDA(cudaMalloc(&c->frame, need), "alloc frame buffers");
        c->frame_cap = need;
    }
    char* p0 = static_cast<char*>(c->frame);
    auto take = [&](size_t b) {
        char* r = p0;
        p0 += b;
        return r;
    };
    cg_frame_entity* d_ent = reinterpret_cast<cg_frame_entity*>(take(b_ent));
    uint32_t* d_ids = reinterpret_cast<uint32_t*>(take(b_id));
    float* d_g = reinterpret_cast<float*>(take(b_g));
    uint8_t* d_cb = reinterpret_cast<uint8_t*>(take(b_cb));
    float* d_proj = reinterpret_cast<float*>(take(b_proj));
    uint2* d_pairs = reinterpret_cast<uint2*>(take(b_pairs));
    unsigned long long* d_npairs = reinterpret_cast<unsigned long long*>(take(b_cnt));
    float* d_grp = reinterpret_cast<float*>(take(b_grp));
    uint32_t* d_tag = reinterpret_cast<uint32_t*>(take(b_tag));
    ShootQuery* d_sq = reinterpret_cast<ShootQuery*>(take(b_sq));
    ShootRayOut* d_so = reinterpret_cast<ShootRayOut*>(take(b_so));
    float* d_dl = reinterpret_cast<float*>(take(b_dl));
    cg_frame_result* d_res = reinterpret_cast<cg_frame_result*>(take(b_res));
    unsigned long long* d_nres = reinterpret_cast<unsigned long long*>(take(b_cnt));
    CG_CUDA(cudaMemcpyAsync(d_ent, entities, sizeof(cg_frame_entity) * n, cudaMemcpyHostToDevice, s), "upload entities");
    CG_CUDA(cudaMemcpyAsync(d_ids, ids.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s), "upload ids");
    CG_CUDA(cudaMemcpyAsync(d_g, globals.data(), sizeof(float) * 16 * n, cudaMemcpyHostToDevice, s), "upload matrices");
    CG_CUDA(cudaMemcpyAsync(d_cb, cbs.data(), n, cudaMemcpyHostToDevice, s), "upload callbacks");
    CG_CUDA(cudaMemsetAsync(d_npairs, 0, sizeof(unsigned long long), s), "clear count");
    BroadParams bp{};
    bp.tree_ids = d_ids;
    bp.trees = c->d_trees;
    bp.recs = c->recs.ptr;
    bp.globals = d_g;
    bp.callback = d_cb;
    bp.n = n;
    float ax[9];
    engine_axes(ax);
    for (int k = 0; k < 3; ++k) bp.axes[k] = make_float3(ax[3 * k], ax[3 * k + 1], ax[3 * k + 2]);
    bp.proj = d_proj;
    bp.pairs = d_pairs;
    bp.cap = max_pairs;
    bp.count = d_npairs;
    CG_CUDA(launch_broad(bp, s), "broad-phase kernels");
    unsigned long long np = 0;
    CG_CUDA(cudaMemcpyAsync(&np, d_npairs, sizeof(np), cudaMemcpyDeviceToHost, s), "read pair count");
    CG_CUDA(cudaStreamSynchronize(s), "broad phase");
    if (np > max_pairs)
        return fail(c, CG_ERR_OUTPUT_OVERFLOW, "%llu broad-phase pairs > max_queries %u", np, max_pairs);
    if (np == 0) {
        c->last_flags = 0;  // no collide step in this frame: nothing to read
        return CG_OK;
    }
    // collide every broad pair with contacts and rays
    FrameParams fp{};
    fp.entities = d_ent;
    fp.pairs = d_pairs;
    fp.n_pairs = uint32_t(np);
    fp.max_rays = max_rays;
    fp.queries = c->d_queries;
    fp.rays = c->ct.rays;
    fp.n_rays = &c->d_ctr->n_rays;
    fp.counts = c->ct.maps + 3 * 2ull * c->cfg.max_queries;   // the contact step's rays per map
    fp.offsets = c->ct.maps + 5 * 2ull * c->cfg.max_queries;  // and their first ray
    fp.grouped = d_grp;
    fp.tags = d_tag;
    fp.shoot = d_sq;
    fp.deltas = d_dl;
    fp.averages = c->ct.averages;
    fp.results = d_res;
    fp.results_cap = max_pairs;
    fp.n_results = d_nres;
    CG_CUDA(launch_frame_queries(fp, s), "frame query kernel");
    c->last_flags = CG_CONTACTS;
    int rc = enqueue_step(c, c->d_queries, uint32_t(np), CG_CONTACTS, s);
    if (rc != CG_OK) return rc;
    // rays per pair, shooting, the delta split
    CG_CUDA(cudaMemsetAsync(d_nres, 0, sizeof(unsigned long long), s), "clear result count");
    CG_CUDA(launch_frame_rays(fp, uint32_t(4 * c->sm_count), s), "frame ray kernels");
    ShootParams sp{};
    sp.q = d_sq;
    sp.n_queries = uint32_t(np);
    sp.n_rays = max_rays;
    sp.n_rays_dev = fp.n_rays;
    sp.trees = c->d_trees;
    sp.recs = c->recs.ptr;
    sp.tris = c->tris.ptr;
    sp.rays = d_grp;
    sp.ray_query = d_tag;
    sp.out = d_so;
    sp.cos_start = std::cos(pr.smoothstep_start);
    sp.cos_finish = std::cos(pr.smoothstep_finish);
    sp.bias = pr.distance_bias;
    sp.deltas = d_dl;
    unsigned* d_err = reinterpret_cast<unsigned*>(d_npairs);  // the pair count is read: its word is free now
    CG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(unsigned), s), "clear flag");
    sp.error = d_err;
    CG_CUDA(launch_shoot(sp, s), "shoot kernels");
    CG_CUDA(launch_frame_split(fp, s), "frame split kernel");
    unsigned long long nres = 0;
    unsigned err = 0;
    CG_CUDA(cudaMemcpyAsync(&nres, d_nres, sizeof(nres), cudaMemcpyDeviceToHost, s), "read result count");
    CG_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(err), cudaMemcpyDeviceToHost, s), "read flag");
    CG_CUDA(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s), "read counters");
    CG_CUDA(cudaStreamSynchronize(s), "collision frame");
    cg_stats st{};
    rc = stats_from(c, *c->h_ctr, &st);
    if (rc != CG_OK) return rc;
    if (err) return fail(c, CG_ERR_QUEUE_OVERFLOW, "a tree is deeper than the ray traversal's stack");
    *n_results = nres;
    const uint64_t m = std::min<uint64_t>(nres, cap);
    if (m) CG_CUDA(cudaMemcpy(results, d_res, sizeof(cg_frame_result) * m, cudaMemcpyDeviceToHost), "read results");
    return nres > cap ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
}

int cg_frame_callbacks(const cg_frame_result* results, uint64_t n_results, const uint32_t* entity_ids,
                       uint32_t n_entities, const uint32_t* parent, uint32_t n_ids, cg_frame_callback* out,
                       uint64_t cap, uint64_t* n_out) {
    if (!n_out || (n_results && (!results || !entity_ids || !parent)) || (cap && !out)) return CG_ERR_INVALID_ARGUMENT;
    *n_out = 0;
    // EntitiesHandler::GetEntityAncestors (EntitiesHandler.cpp:186-204): the
    // chain up to the root (entity 0), reversed
    auto ancestors = [&](uint32_t e, std::vector<uint32_t>& a) {
        a.clear();
        for (;;) {
            if (e >= n_ids || a.size() > n_ids) return false;  // out of range, or a cycle
            a.push_back(e);
            if (e == 0) break;
            e = parent[e];
        }
        std::reverse(a.begin(), a.end());
        return true;
    };
    std::vector<cg_frame_callback> cb;
    std::vector<uint32_t> fa, sa;
    for (uint64_t k = 0; k < n_results; ++k) {
        const cg_frame_result& r = results[k];
        if (r.first >= n_entities || r.second >= n_entities) return CG_ERR_INVALID_ARGUMENT;
        const uint32_t f = entity_ids[r.first], s = entity_ids[r.second];
        if (!ancestors(f, fa) || !ancestors(s, sa)) return CG_ERR_INVALID_ARGUMENT;
        auto emit = [&](const std::vector<uint32_t>& mine, const std::vector<uint32_t>& other, uint32_t fam,
                        uint32_t with, const float* d) {
            for (size_t i = 0; i < mine.size(); ++i)
                if (i >= other.size() || mine[i] != other[i])
                    cb.push_back(cg_frame_callback{mine[i], fam, with, {d[0], d[1], d[2]}});
        };
        emit(fa, sa, f, s, r.first_delta);   // CollisionDetection.cpp:109-116
        emit(sa, fa, s, f, r.second_delta);  // :118-124
    }
    std::stable_sort(cb.begin(), cb.end(),
                     [](const cg_frame_callback& a, const cg_frame_callback& b) { return a.receiver < b.receiver; });
    *n_out = cb.size();
    const uint64_t m = std::min<uint64_t>(cb.size(), cap);
    if (m) std::memcpy(out, cb.data(), sizeof(cg_frame_callback) * m);
    return cb.size() > cap ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
}

void cg_shoot_params_default(cg_shoot_params* p) {
    if (!p) return;
    const float deg = 0.01745329251994329576923690768489f;  // glm::radians
    p->smoothstep_start = 40.f * deg;
    p->smoothstep_finish = 65.f * deg;
    p->distance_bias = 1.01f;
}

int cg_shoot_rays(cg_ctx* c, const cg_shoot_query* queries, uint32_t n, const float* rays, uint64_t n_rays,
                  const cg_shoot_params* params, float* deltas) {
    if (!c || (n && (!queries || !deltas)) || (n_rays && !rays)) return CG_ERR_INVALID_ARGUMENT;
    if (n_rays > 0x7fffffffull) return fail(c, CG_ERR_INVALID_ARGUMENT, "more than 2^31 rays");
    if (n > 0x7fffffffu) return fail(c, CG_ERR_INVALID_ARGUMENT, "more than 2^31 queries");
    cg_shoot_params pr;
    cg_shoot_params_default(&pr);
    if (params) pr = *params;
    std::vector<ShootQuery> table(n);
    std::vector<uint32_t> tags(n_rays);
    uint64_t next = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const cg_shoot_query& q = queries[i];
        if (q.tree_a >= c->trees.size() || !c->trees[q.tree_a].live || q.tree_b >= c->trees.size() ||
            !c->trees[q.tree_b].live)
            return fail(c, CG_ERR_NOT_FOUND, "shoot query %u names tree %u / %u", i, q.tree_a, q.tree_b);
        const uint64_t cnt = uint64_t(q.n_first) + q.n_second;
        if (next + cnt > n_rays)
            return fail(c, CG_ERR_INVALID_ARGUMENT, "the queries' ray counts exceed n_rays (%llu)",
                        (unsigned long long)n_rays);
        ShootQuery& t = table[i];
        float inv[16];
        mat_inverse(q.first_global, inv);
        mat_mul(inv, q.second_global, t.relative);  // OBBtreesCollision.cpp:15 / ShootUncollideRays.cpp:16-17
        std::memcpy(t.first_global, q.first_global, sizeof(t.first_global));
        t.tree_a = q.tree_a;
        t.tree_b = q.tree_b;
        t.ray_first = uint32_t(next);
        t.n_first = q.n_first;
        t.n_second = q.n_second;
        t.pad[0] = 1u;
        t.pad[1] = t.pad[2] = 0u;
        for (uint64_t k = 0; k < cnt; ++k) tags[next + k] = i | (k >= q.n_first ? 0x80000000u : 0u);
        next += cnt;
    }
    if (next != n_rays)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "the queries' ray counts (%llu) differ from n_rays (%llu)",
                    (unsigned long long)next, (unsigned long long)n_rays);
    if (n == 0) return CG_OK;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    auto up = [](size_t x) { return (x + 255u) & ~size_t(255); };
    const size_t b_q = up(sizeof(ShootQuery) * n), b_r = up(sizeof(float) * 6 * n_rays), b_t = up(sizeof(uint32_t) * n_rays),
                 b_o = up(sizeof(ShootRayOut) * n_rays), b_d = up(sizeof(float) * 3 * n), b_e = 256;
    const size_t need = b_q + b_r + b_t + b_o + b_d + b_e;
    if (need > c->shoot_cap) {
        CG_CUDA(cudaStreamSynchronize(s), "shoot buffers");
        cudaFree(c->shoot);
        c->shoot = nullptr;
        c->shoot_cap = 0;
        CG_CUDA(cudaMalloc(&c->shoot, need), "alloc shoot buffers");
        c->shoot_cap = need;
    }
    char* base = static_cast<char*>(c->shoot);
    ShootQuery* d_q = reinterpret_cast<ShootQuery*>(base);
    float* d_rays = reinterpret_cast<float*>(base + b_q);
    uint32_t* d_tags = reinterpret_cast<uint32_t*>(base + b_q + b_r);
    ShootRayOut* d_out = reinterpret_cast<ShootRayOut*>(base + b_q + b_r + b_t);
    float* d_deltas = reinterpret_cast<float*>(base + b_q + b_r + b_t + b_o);
    unsigned* d_err = reinterpret_cast<unsigned*>(base + b_q + b_r + b_t + b_o + b_d);
    CG_CUDA(cudaMemcpyAsync(d_q, table.data(), sizeof(ShootQuery) * n, cudaMemcpyHostToDevice, s), "upload queries");
    if (n_rays) {
        CG_CUDA(cudaMemcpyAsync(d_rays, rays, sizeof(float) * 6 * n_rays, cudaMemcpyHostToDevice, s), "upload rays");
        CG_CUDA(cudaMemcpyAsync(d_tags, tags.data(), sizeof(uint32_t) * n_rays, cudaMemcpyHostToDevice, s),
                "upload ray tags");
    }
    CG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(unsigned), s), "clear flag");
    ShootParams p{};
    p.q = d_q;
    p.n_queries = n;
    p.n_rays = uint32_t(n_rays);
    p.trees = c->d_trees;
    p.recs = c->recs.ptr;
    p.tris = c->tris.ptr;
    p.rays = d_rays;
    p.ray_query = d_tags;
    p.out = d_out;
    p.cos_start = std::cos(pr.smoothstep_start);  // the constructor's cosines (ShootUncollideRays.cpp:4-11)
    p.cos_finish = std::cos(pr.smoothstep_finish);
    p.bias = pr.distance_bias;
    p.deltas = d_deltas;
    p.error = d_err;
    CG_CUDA(launch_shoot(p, s), "shoot kernels");
    unsigned err = 0;
    CG_CUDA(cudaMemcpyAsync(deltas, d_deltas, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s), "read deltas");
    CG_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read flag");
    CG_CUDA(cudaStreamSynchronize(s), "shoot");
    if (err) return fail(c, CG_ERR_QUEUE_OVERFLOW, "a tree is deeper than the ray traversal's stack");
    return CG_OK;
}
