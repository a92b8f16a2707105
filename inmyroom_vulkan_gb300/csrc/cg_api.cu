// Host side of the C ABI declared in include/collide_gpu.h: context and
// buffers, tree arenas with upload validation, launches, result read-back,
// the CUDA graph of one collide step, deformation, refit and the
// differentiable energy. Tree build and the tree cache are in cg_api_tree.cu,
// the broad phase, shooting and the collision frame in cg_api_frame.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "cg_ctx.h"

namespace cg_host {

int fail(cg_ctx* c, int code, const char* fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

int cuda_fail(cg_ctx* c, cudaError_t e, const char* what) {
    const int code = (e == cudaErrorMemoryAllocation) ? CG_ERR_OUT_OF_MEMORY : CG_ERR_CUDA;
    return fail(c, code, "%s: %s", what, cudaGetErrorString(e));
}


bool pow2(uint32_t x) { return x && !(x & (x - 1)); }

// Changes whenever a device address that a captured graph holds changes.
uint64_t arena_gen(const cg_ctx* c) { return (c->recs.gen * 1000003ull + c->tris.gen) * 1000003ull + c->table_gen; }

void free_buffers(cg_ctx* c) {
    cudaFree(c->d_queries);
    cudaFree(c->d_packed);
    cudaFree(c->d_ctr);
    cudaFree(c->d_pool);
    cudaFree(c->d_leaf_list);
    cudaFree(c->d_ready);
    cudaFree(c->d_pairs);
    cudaFree(c->d_leafs);
    cudaFree(c->d_leaf_keys);
    c->d_leaf_keys = nullptr;
    cudaFree(c->d_trace);
    auto& t = c->ct;
    for (void* p : {(void*)t.pair_aux, (void*)t.table, (void*)t.occupied, (void*)t.slot_info, (void*)t.big_slots, (void*)t.pg_geom, (void*)t.pg_link,
                    (void*)t.pg_mask, (void*)t.contrib, (void*)t.leaf_mark, (void*)t.kleaf, (void*)t.kpath,
                    (void*)t.maps, (void*)t.elems, (void*)t.work, (void*)t.vkeys,
                    (void*)t.vval, (void*)t.vocc, (void*)t.ctmp, (void*)t.rtmp, (void*)t.contacts, (void*)t.rays,
                    (void*)t.averages})
        cudaFree(p);
    t = cg_ctx::Contacts{};
    cudaFreeHost(c->h_queries);
    cudaFreeHost(c->h_ctr);
    c->d_queries = nullptr;
    c->d_packed = nullptr;
    c->d_ctr = nullptr;
    c->d_pool = nullptr;
    c->d_leaf_list = nullptr;
    c->d_ready = nullptr;
    c->d_pairs = nullptr;
    c->d_leafs = nullptr;
    c->d_trace = nullptr;
    c->h_queries = nullptr;
    c->h_ctr = nullptr;
}

// Device copy of a batch table; uploaded (after the stream's earlier work,
// which may still read the old one) only when its contents changed.
int stage_table(cg_ctx* c, cg_ctx::Table& t, const void* data, size_t bytes, cudaStream_t s, const void** dev) {
    if (bytes == t.host.size() && std::memcmp(t.host.data(), data, bytes) == 0) {
        *dev = t.dev;
        return CG_OK;
    }
    CG_CUDA(cudaStreamSynchronize(s), "batch table");
    if (bytes > t.cap) {
        cudaFree(t.dev);
        t.dev = nullptr;
        t.cap = 0;
        CG_CUDA(cudaMalloc(&t.dev, bytes), "alloc batch table");
        t.cap = bytes;
    }
    CG_CUDA(cudaMemcpy(t.dev, data, bytes, cudaMemcpyHostToDevice), "upload batch table");
    t.host.assign(static_cast<const char*>(data), static_cast<const char*>(data) + bytes);
    *dev = t.dev;
    return CG_OK;
}

bool aligned_to(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

// A cg_deform_view checked and turned into the kernels' form; `out` is
// required when want_out is set.
int deform_params(cg_ctx* c, const cg_deform_view* v, float* out, bool want_out, uint32_t i, DeformParams* p) {
    if (v->n_vertices && (!v->vertices || (want_out && !out) || (v->n_targets && !v->morph_weights) ||
                          (v->n_groups && (!v->joints || !v->weights || !v->joint_matrices || !v->inverse_bind))))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "deform view %u has null arrays", i);
    if (!aligned_to(v->vertices, 16) || !aligned_to(out, 16) ||
        (v->n_groups && (!aligned_to(v->weights, 16) || !aligned_to(v->joints, 8))))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "deform view %u: arrays must be 16-byte (joints 8-byte) aligned", i);
    if (v->n_joints > kMaxJoints) return fail(c, CG_ERR_INVALID_ARGUMENT, "n_joints %u > %u", v->n_joints, kMaxJoints);
    p->n_vertices = v->n_vertices;
    p->n_targets = v->n_targets;
    p->n_groups = v->n_groups;
    p->n_joints = v->n_groups ? v->n_joints : 0u;
    p->vertices = v->vertices;
    p->morph_weights = v->morph_weights;
    p->joints = v->joints;
    p->weights = v->weights;
    p->joint_matrices = v->joint_matrices;
    p->inverse_bind = v->inverse_bind;
    p->out = out;
    return CG_OK;
}

// The skeleton of cg_pose / cg_pose_backward checked and staged in device
// memory: parents (int32), then offsets (3 floats) from a 16-byte boundary.
int pose_params(cg_ctx* c, const cg_skeleton_view* sk, uint32_t n_poses, cudaStream_t s, PoseParams* p) {
    const uint32_t nb = sk->n_bones;
    if (nb == 0 || nb > kMaxJoints || !sk->parent || !sk->offsets)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "skeleton: n_bones %u (1..%u) and both arrays are required", nb,
                    kMaxJoints);
    for (uint32_t j = 0; j < nb; ++j)
        if (sk->parent[j] < -1 || sk->parent[j] >= int32_t(j))
            return fail(c, CG_ERR_INVALID_ARGUMENT, "skeleton: parent of bone %u is %d (must be -1 or < %u)", j,
                        sk->parent[j], j);
    const size_t off = (sizeof(int32_t) * nb + 15u) & ~size_t(15);
    std::vector<char> blob(off + sizeof(float) * 3u * nb, 0);
    std::memcpy(blob.data(), sk->parent, sizeof(int32_t) * nb);
    std::memcpy(blob.data() + off, sk->offsets, sizeof(float) * 3u * nb);
    const void* d = nullptr;
    const int rc = stage_table(c, c->skeleton_table, blob.data(), blob.size(), s, &d);
    if (rc != CG_OK) return rc;
    p->n_poses = n_poses;
    p->n_bones = nb;
    p->parent = static_cast<const int32_t*>(d);
    p->offsets = reinterpret_cast<const float*>(static_cast<const char*>(d) + off);
    return CG_OK;
}

// The last collide step stored its colliding pairs.
int energy_ready(cg_ctx* c) {
    if (!c->cfg.max_tri_pairs || (c->last_flags & (CG_NO_TRI_PAIRS | CG_MID_ONLY)))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "the energy needs the colliding pairs of the last collide step");
    return CG_OK;
}

EnergyParams energy_params(cg_ctx* c) {
    EnergyParams p{};
    p.q = c->d_packed;
    p.n_queries = c->last_n;
    p.tris = c->tris.ptr;
    p.pairs = c->d_pairs;
    p.ctr = c->d_ctr;
    p.pairs_cap = c->cfg.max_tri_pairs;
    return p;
}

// The engine's broad-phase axes U, V, W (CollisionDetection.cpp:9-13) in
// glm-convention arithmetic.
void engine_axes(float* ax) {
    auto norm = [](float x, float y, float z, float* o) {
        const float inv = 1.0f / std::sqrt((x * x + y * y) + z * z);
        o[0] = x * inv, o[1] = y * inv, o[2] = z * inv;
    };
    auto cross = [](const float* a, const float* b, float* o) {
        o[0] = a[1] * b[2] - b[1] * a[2];
        o[1] = a[2] * b[0] - b[2] * a[0];
        o[2] = a[0] * b[1] - b[0] * a[1];
    };
    float t[3];
    const float down[3] = {0.f, -1.f, 0.f};
    norm(0.8f, -0.2f, 0.f, ax);
    cross(ax, down, t);
    norm(t[0], t[1], t[2], ax + 6);
    cross(ax + 6, ax, t);
    norm(t[0], t[1], t[2], ax + 3);
}

void drop_graph(cg_ctx* c) {
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    if (c->host_graph.exec) cudaGraphExecDestroy(c->host_graph.exec);
    c->graph_exec = nullptr;
    c->graph = nullptr;
    c->host_graph.exec = nullptr;
}

int check_config(cg_ctx* c, const cg_config* cfg) {
    if (cfg->max_queries == 0) return fail(c, CG_ERR_INVALID_ARGUMENT, "max_queries must be > 0");
    if (!pow2(cfg->stack_entries) || cfg->stack_entries < 256 || cfg->stack_entries > 4096)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "stack_entries must be a power of two in [256, 4096]");
    if (cfg->warps_per_block == 0 || cfg->warps_per_block > 8)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "warps_per_block must be in [1, 8]");
    if (cfg->leaf_flush == 0 || cfg->leaf_flush > uint32_t(kLeafCap - 63))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "leaf_flush must be in [1, %d]", kLeafCap - 63);
    if (cfg->max_queries >= kItemSideB) return fail(c, CG_ERR_INVALID_ARGUMENT, "max_queries must be < 2^31");
    if (cfg->queue_capacity < 1024) return fail(c, CG_ERR_INVALID_ARGUMENT, "queue_capacity must be >= 1024");
    if (cfg->wait_limit_ms == 0) return fail(c, CG_ERR_INVALID_ARGUMENT, "wait_limit_ms must be > 0");
    if (cfg->max_leaf_pairs >= (1ull << 31)) return fail(c, CG_ERR_INVALID_ARGUMENT, "max_leaf_pairs must be < 2^31");
    if (cfg->max_contacts > (1ull << 22)) return fail(c, CG_ERR_INVALID_ARGUMENT, "max_contacts must be <= 2^22");
    if (cfg->max_contacts && (cfg->max_tri_pairs == 0 || cfg->max_tri_pairs >= (1ull << 31)))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "contacts need 0 < max_tri_pairs < 2^31");
    return CG_OK;
}

// The sizes at which std::unordered_map<uint32_t, T> grows, read from the
// host's own library (the one the engine links): keys are inserted one at a
// time and every change of bucket_count() is recorded, as (insertion index,
// new bucket count). The reference's per-triangle maps list their keys in an
// order that follows from these sizes (cg_contacts.cu). Computed once per
// process up to the largest size asked for.
bool growth_schedule(uint32_t max_elems, uint32_t* start, uint32_t* buckets, uint32_t* n) {
    static std::mutex mu;
    static std::vector<std::pair<uint32_t, uint32_t>> sched;
    static uint64_t covered = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (covered <= max_elems) {
        sched.clear();
        std::unordered_map<uint32_t, char> m;
        size_t prev = m.bucket_count();
        // one growth past max_elems, so that the last entry covers every size up to it
        uint64_t i = 0;
        for (;; ++i) {
            m.emplace(uint32_t(i), 0);
            if (m.bucket_count() != prev) {
                prev = m.bucket_count();
                sched.emplace_back(uint32_t(i), uint32_t(prev));
                if (i > max_elems) break;
            }
        }
        covered = i;
    }
    if (sched.size() > kMaxSchedule) return false;
    *n = uint32_t(sched.size());
    for (size_t k = 0; k < sched.size(); ++k) {
        start[k] = sched[k].first;
        buckets[k] = sched[k].second;
    }
    return true;
}

int alloc_buffers(cg_ctx* c) {
    const cg_config& g = c->cfg;
    int occ = 0;
    CG_CUDA(traverse_occupancy(g.warps_per_block, g.stack_entries, &occ), "occupancy");
    if (occ < 1)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "traversal kernel does not fit: %u warps x %u stack entries",
                    g.warps_per_block, g.stack_entries);
    const int per_sm = g.blocks_per_sm ? std::min<int>(occ, int(g.blocks_per_sm)) : occ;
    c->blocks = uint32_t(per_sm * c->sm_count);
    const uint32_t warps = c->blocks * g.warps_per_block;
    c->slot_cap = std::max<uint32_t>(g.queue_capacity / uint32_t(kChunk), 64u);
    c->slot_alloc = c->slot_cap + 9u * warps + 64u;
    int nocc = 0;
    CG_CUDA(narrow_occupancy(8, &nocc), "occupancy");
    c->narrow_blocks = uint32_t(std::max(nocc, 1) * c->sm_count);
    c->contact_blocks = uint32_t(8 * c->sm_count);  // 2048 threads per SM of 256-thread blocks
    int oocc = 0;
    CG_CUDA(contacts_order_occupancy(&oocc), "occupancy");
    c->order_blocks = uint32_t(std::max(oocc, 1) * c->sm_count);
    int focc = 0;
    CG_CUDA(contacts_fold_occupancy(&focc), "occupancy");
    c->fold_blocks = uint32_t(std::max(focc, 1) * c->sm_count);
    CG_CUDA(deform_smem_limit(), "deform kernel shared memory");
    c->copy_blocks = uint32_t(4 * c->sm_count);
    int gocc = 0;
    CG_CUDA(energy_occupancy(&gocc), "occupancy");
    c->energy_blocks = uint32_t(std::max(gocc, 1) * c->sm_count);

    CG_CUDA(cudaMalloc(&c->d_queries, sizeof(cg_query) * g.max_queries), "alloc queries");
    CG_CUDA(cudaMalloc(&c->d_packed, sizeof(PackedQuery) * g.max_queries), "alloc packed queries");
    CG_CUDA(cudaMalloc(&c->d_ctr, sizeof(Counters)), "alloc counters");
    CG_CUDA(cudaMemset(c->d_ctr, 0, sizeof(Counters)), "zero counters");
    CG_CUDA(cudaMalloc(&c->d_pool, sizeof(uint4) * size_t(kChunk) * c->slot_alloc), "alloc task pool");
    CG_CUDA(cudaMalloc(&c->d_leaf_list, sizeof(uint4) * std::max<uint64_t>(g.max_leaf_pairs, 1)), "alloc leaf-pair list");
    CG_CUDA(cudaMalloc(&c->d_ready, sizeof(unsigned int) * c->slot_alloc), "alloc task flags");
    CG_CUDA(cudaMemset(c->d_ready, 0, sizeof(unsigned int) * c->slot_alloc), "zero task flags");
    if (g.max_tri_pairs) CG_CUDA(cudaMalloc(&c->d_pairs, sizeof(cg_tri_pair) * g.max_tri_pairs), "alloc pair output");
    if (g.max_leaf_pairs)
        CG_CUDA(cudaMalloc(&c->d_leafs, sizeof(cg_leaf_pair) * g.max_leaf_pairs), "alloc leaf-pair output");
    if (g.max_contacts) {
        // Hash tables at most half full: contact slots, vertices with a ray
        // (3 per contact at most).
        auto pow2_at_least = [](uint64_t x) {
            uint64_t p = 1024;
            while (p < x) p <<= 1;
            return uint32_t(p);
        };
        auto& t = c->ct;
        const uint64_t mc = g.max_contacts, mp = g.max_tri_pairs, mq = g.max_queries;
        t.table_slots = pow2_at_least(2 * mc);
        t.vslots = pow2_at_least(6 * mc);
        t.max_rays = uint32_t(3 * mc);
        CG_CUDA(cudaMalloc(&t.pair_aux, sizeof(uint4) * mp), "alloc pair side records");
        CG_CUDA(cudaMalloc(&t.table, sizeof(ContactSlot) * t.table_slots), "alloc contact table");
        CG_CUDA(cudaMalloc(&t.occupied, sizeof(uint32_t) * t.table_slots), "alloc contact list");
        CG_CUDA(cudaMalloc(&t.slot_info, sizeof(uint4) * t.table_slots), "alloc contact slot list");
        CG_CUDA(cudaMalloc(&t.big_slots, sizeof(uint32_t) * t.table_slots), "alloc contact slot list");
        CG_CUDA(cudaMalloc(&t.pg_geom, sizeof(float4) * mp), "alloc pair geometry");
        CG_CUDA(cudaMalloc(&t.pg_link, sizeof(uint4) * mp), "alloc pair links");
        CG_CUDA(cudaMalloc(&t.pg_mask, sizeof(uint32_t) * mp), "alloc pair masks");
        CG_CUDA(cudaMalloc(&t.contrib, sizeof(unsigned long long) * 2 * mp), "alloc contributions");
        CG_CUDA(cudaMalloc(&t.maps, sizeof(uint32_t) * 7 * 2 * mq), "alloc contact maps");
        CG_CUDA(cudaMemset(t.maps, 0, sizeof(uint32_t) * 7 * 2 * mq), "zero contact maps");
        const uint64_t ml = std::max<uint64_t>(g.max_leaf_pairs, 1);
        CG_CUDA(cudaMalloc(&t.leaf_mark, sizeof(uint32_t) * ml), "alloc leaf-pair marks");
        CG_CUDA(cudaMemset(t.leaf_mark, 0, sizeof(uint32_t) * ml), "zero leaf-pair marks");
        t.kleaf_cap = t.table_slots;
        CG_CUDA(cudaMalloc(&t.kleaf, sizeof(uint32_t) * t.kleaf_cap), "alloc contact leaf pairs");
        CG_CUDA(cudaMalloc(&t.kpath, sizeof(ulonglong2) * t.kleaf_cap), "alloc contact leaf-pair paths");
        CG_CUDA(cudaMalloc(&t.elems, sizeof(ContactElem) * mc), "alloc contact elements");
        CG_CUDA(cudaMalloc(&t.work, sizeof(uint32_t) * kOrderWords * mc), "alloc contact order memory");
        CG_CUDA(cudaMalloc(&t.vkeys, sizeof(unsigned long long) * t.vslots), "alloc vertex set");
        CG_CUDA(cudaMalloc(&t.vval, sizeof(uint32_t) * t.vslots), "alloc vertex set");
        CG_CUDA(cudaMalloc(&t.vocc, sizeof(uint32_t) * t.vslots), "alloc vertex list");
        CG_CUDA(cudaMalloc(&t.ctmp, sizeof(cg_contact) * mc), "alloc contact staging");
        CG_CUDA(cudaMalloc(&t.rtmp, sizeof(cg_ray) * t.max_rays), "alloc ray staging");
        CG_CUDA(cudaMalloc(&t.contacts, sizeof(cg_contact) * mc), "alloc contacts");
        CG_CUDA(cudaMalloc(&t.rays, sizeof(cg_ray) * t.max_rays), "alloc rays");
        CG_CUDA(cudaMalloc(&t.averages, sizeof(cg_ray_average) * mq), "alloc ray averages");
        CG_CUDA(init_contact_tables(t.table, t.table_slots, t.vkeys, t.vval, t.vslots, c->stream),
                "init contact tables");
        CG_CUDA(cudaStreamSynchronize(c->stream), "init contact tables");
        if (!growth_schedule(uint32_t(mc), c->sched_start, c->sched_buckets, &c->n_sched))
            return fail(c, CG_ERR_INVALID_ARGUMENT, "the host's unordered_map grows more than %u times up to %llu "
                        "elements", kMaxSchedule, (unsigned long long)mc);
    }
    CG_CUDA(cudaMallocHost(&c->h_queries, sizeof(cg_query) * g.max_queries), "alloc pinned queries");
    CG_CUDA(cudaMallocHost(&c->h_ctr, sizeof(Counters)), "alloc pinned counters");
    std::memset(c->h_ctr, 0, sizeof(Counters));
    return CG_OK;
}

int sync_tree_table(cg_ctx* c) {
    const uint32_t n = uint32_t(c->trees.size());
    if (n > c->d_trees_cap) {
        cudaFree(c->d_trees);
        c->d_trees = nullptr;
        const uint32_t cap = std::max<uint32_t>(64, n * 2);
        CG_CUDA(cudaMalloc(&c->d_trees, sizeof(DevTree) * cap), "alloc tree table");
        c->d_trees_cap = cap;
        ++c->table_gen;
    }
    std::vector<DevTree> host(n);
    for (uint32_t i = 0; i < n; ++i) {
        const auto& s = c->trees[i];
        host[i] = DevTree{uint32_t(s.rec_base), uint32_t(s.tri_base), uint32_t(s.n_recs), uint32_t(s.n_tris),
                          s.live ? 1u : 0u, 0u, s.nrm};
    }
    if (n) CG_CUDA(cudaMemcpy(c->d_trees, host.data(), sizeof(DevTree) * n, cudaMemcpyHostToDevice), "upload tree table");
    return CG_OK;
}

void put_box(float4* rec, const cg_obb& b, uint32_t ref, uint32_t meta, uint32_t split) {
    rec[0] = make_float4(b.center[0], b.center[1], b.center[2], b.u[0]);
    rec[1] = make_float4(b.u[1], b.u[2], b.v[0], b.v[1]);
    rec[2] = make_float4(b.v[2], b.w[0], b.w[1], b.w[2]);
    float r, m, sp;
    std::memcpy(&r, &ref, 4);
    std::memcpy(&m, &meta, 4);
    std::memcpy(&sp, &split, 4);
    rec[3] = make_float4(r, m, 0.f, sp);
}

// Enqueues counter reset, packing, the traversal and the narrow phase on `s`.
// pairs_copy: with the step's colliding pairs final (after the narrow phase),
// copy them out on a branch that runs beside the contact kernels.
int enqueue_step(cg_ctx* c, const cg_query* d_queries, uint32_t n, uint32_t flags, cudaStream_t s,
                 const CopyOutParams* pairs_copy, const CopyOutParams* results_copy) {
    c->last_n = n;
    unsigned int* trace = (flags & CG_TRACE) ? c->d_trace : nullptr;
    const uint32_t trace_ns = c->trace_ns ? c->trace_ns : 1000u;
    CG_CUDA(launch_init(c->d_ctr, c->d_ready, c->slot_alloc, n, trace, s), "init kernel");
    const uint32_t leaf_cap = uint32_t(std::min<uint64_t>(c->cfg.max_leaf_pairs, 0xffffffffull));
    CG_CUDA(launch_pack(d_queries, n, c->d_trees, uint32_t(c->trees.size()), c->recs.ptr, c->d_packed, c->d_ctr,
                        c->d_leaf_list, leaf_cap, s),
            "pack kernel");
    TraverseParams p{};
    p.q = c->d_packed;
    p.n_queries = n;
    p.recs = c->recs.ptr;
    p.pool = c->d_pool;
    p.ready = c->d_ready;
    p.slot_cap = c->slot_cap;
    p.slot_alloc = c->slot_alloc;
    p.ctr = c->d_ctr;
    p.leaf_list = c->d_leaf_list;
    p.leaf_cap = uint32_t(std::min<uint64_t>(c->cfg.max_leaf_pairs, 0xffffffffull));
    p.trace = trace;
    p.trace_ns = trace_ns;
    p.stack_cap = c->cfg.stack_entries;
    p.donate_min = std::min(std::max(c->cfg.donate_min, 2u), c->cfg.stack_entries - 63u);
    p.leaf_flush = c->cfg.leaf_flush;
    p.wait_ns = (unsigned long long)c->cfg.wait_limit_ms * 1000000ull;
    NarrowParams np{};
    np.q = c->d_packed;
    np.tris = c->tris.ptr;
    np.leaf_list = c->d_leaf_list;
    np.leaf_cap = p.leaf_cap;
    np.ctr = c->d_ctr;
    np.pairs = c->d_pairs;
    np.pair_aux = (flags & CG_CONTACTS) ? c->ct.pair_aux : nullptr;
    np.pairs_cap = c->d_pairs ? c->cfg.max_tri_pairs : 0;
    np.leafs = c->d_leafs;
    np.leafs_cap = c->d_leafs ? c->cfg.max_leaf_pairs : 0;
    np.flags = flags;
    np.trace = trace;
    np.trace_ns = trace_ns;
    const unsigned rec_flags = c->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    CG_CUDA(cudaEventRecordWithFlags(c->ev_t0, s, rec_flags), "timing event");
    if (n) CG_CUDA(launch_traverse(p, c->blocks, c->cfg.warps_per_block, s), "traversal kernel");
    CG_CUDA(cudaEventRecordWithFlags(c->ev_t1, s, rec_flags), "timing event");
    if (n) CG_CUDA(launch_narrow(np, c->narrow_blocks, 8, s), "narrow-phase kernel");
    CG_CUDA(cudaEventRecordWithFlags(c->ev_t2, s, rec_flags), "timing event");
    if ((flags & CG_DFS_ORDER) && n) {
        LeafKeyParams kp{};
        kp.q = c->d_packed;
        kp.trees = c->d_trees;
        kp.recs = c->recs.ptr;
        kp.leaf_list = c->d_leaf_list;
        kp.n_leafs = &c->d_ctr->n_leafs;
        kp.leaf_cap = p.leaf_cap;
        kp.error = &c->d_ctr->error;
        kp.keys = c->d_leaf_keys;
        CG_CUDA(launch_leaf_keys(kp, c->contact_blocks, s), "leaf-pair key kernel");
    }
    if (pairs_copy) {
        CG_CUDA(cudaEventRecord(c->ev_fork, s), "fork event");
        CG_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0), "fork");
        CG_CUDA(launch_copy_out(*pairs_copy, c->copy_blocks, c->side), "copy kernel");
        CG_CUDA(cudaEventRecord(c->ev_joined, c->side), "join event");
    }
    if ((flags & CG_CONTACTS) && n) {
        const auto& t = c->ct;
        ContactParams cp{};
        cp.q = c->d_packed;
        cp.n_queries = n;
        cp.n_sched = c->n_sched;
        cp.tris = c->tris.ptr;
        cp.recs = c->recs.ptr;
        cp.trees = c->d_trees;
        cp.pairs = c->d_pairs;
        cp.pair_aux = t.pair_aux;
        cp.leaf_list = c->d_leaf_list;
        cp.pairs_cap = c->cfg.max_tri_pairs;
        cp.table = t.table;
        cp.table_mask = t.table_slots - 1u;
        cp.max_contacts = uint32_t(c->cfg.max_contacts);
        cp.occupied = t.occupied;
        cp.slot_info = t.slot_info;
        cp.big_slots = t.big_slots;
        cp.pg_geom = t.pg_geom;
        cp.pg_link = t.pg_link;
        cp.pg_mask = t.pg_mask;
        cp.contrib = t.contrib;
        const size_t mq2 = 2ull * c->cfg.max_queries;
        cp.map_cnt = t.maps;
        cp.map_off = t.maps + mq2;
        cp.map_fill = t.maps + 2 * mq2;
        cp.map_nr = t.maps + 3 * mq2;
        cp.map_coff = t.maps + 4 * mq2;
        cp.map_roff = t.maps + 5 * mq2;
        cp.map_order = t.maps + 6 * mq2;
        cp.leaf_mark = t.leaf_mark;
        cp.kleaf = t.kleaf;
        cp.kpath = t.kpath;
        cp.kleaf_cap = t.kleaf_cap;
        cp.elems = t.elems;
        cp.work = t.work;
        cp.vkeys = t.vkeys;
        cp.vval = t.vval;
        cp.vtable_mask = t.vslots - 1u;
        cp.vocc = t.vocc;
        cp.ctmp = t.ctmp;
        cp.rtmp = t.rtmp;
        cp.contacts = t.contacts;
        cp.rays = t.rays;
        cp.max_rays = t.max_rays;
        cp.averages = t.averages;
        if (results_copy) {  // a null buffer takes nothing
            cp.host_rays = results_copy->host_rays;
            cp.host_rays_cap = cp.host_rays ? results_copy->host_rays_cap : 0;
            cp.host_averages = results_copy->host_averages;
            cp.host_averages_cap = cp.host_averages ? results_copy->host_averages_cap : 0;
        }
        cp.ctr = c->d_ctr;
        for (uint32_t k = 0; k < c->n_sched; ++k) {
            cp.sched_start[k] = c->sched_start[k];
            cp.sched_buckets[k] = c->sched_buckets[k];
        }
        CG_CUDA(launch_contacts(cp, c->contact_blocks, c->fold_blocks, c->order_blocks, s, c->branch,
                                c->ev_branch, c->ev_branched), "contact kernels");
    }
    if (pairs_copy) CG_CUDA(cudaStreamWaitEvent(s, c->ev_joined, 0), "join");
    return CG_OK;
}

int stats_from(cg_ctx* c, const Counters& k, cg_stats* st) {
    cg_stats s{};
    s.node_pairs = k.node_pairs;
    s.leaf_pairs = k.n_leafs;
    s.tri_tests = k.tri_tests;
    s.tri_pairs = k.n_pairs;
    s.fragile = k.fragile;
    s.donations = k.donations;
    s.warp_steps = k.warp_steps;
    s.contacts = k.n_elems;
    s.rays = k.n_rays;
    s.rechecked = k.rechecked;
    s.disagreements = k.disagreements;
    int status = CG_OK;
    if (k.error & ERR_TIMEOUT)
        status = fail(c, CG_ERR_TIMEOUT, "a device-side wait exceeded %u ms", c->cfg.wait_limit_ms);
    else if (k.error & ERR_QUEUE)
        status = fail(c, CG_ERR_QUEUE_OVERFLOW, "node-pair queue full (queue_capacity %u)", c->cfg.queue_capacity);
    else if (k.error & ERR_BAD_QUERY)
        status = fail(c, CG_ERR_INVALID_ARGUMENT, "a query names an unknown tree");
    else if (k.error & ERR_DEEP)
        status = fail(c, CG_ERR_OUTPUT_OVERFLOW, "CG_DFS_ORDER: a leaf pair deeper than 127 splits of the "
                      "simultaneous descent");
    else if (k.n_leafs > c->cfg.max_leaf_pairs)
        status = fail(c, CG_ERR_OUTPUT_OVERFLOW, "%llu candidate leaf pairs, max_leaf_pairs %llu: triangle tests "
                      "incomplete", (unsigned long long)k.n_leafs, (unsigned long long)c->cfg.max_leaf_pairs);
    else if (!(c->last_flags & CG_NO_TRI_PAIRS) && k.n_pairs > (c->d_pairs ? c->cfg.max_tri_pairs : 0))
        status = fail(c, CG_ERR_OUTPUT_OVERFLOW, "%llu colliding pairs, capacity %llu", (unsigned long long)k.n_pairs,
                      (unsigned long long)c->cfg.max_tri_pairs);
    else if ((c->last_flags & CG_KEEP_LEAF_PAIRS) && k.n_leafs > (c->d_leafs ? c->cfg.max_leaf_pairs : 0))
        status = fail(c, CG_ERR_OUTPUT_OVERFLOW, "%llu leaf pairs, capacity %llu", (unsigned long long)k.n_leafs,
                      (unsigned long long)c->cfg.max_leaf_pairs);
    else if ((c->last_flags & CG_CONTACTS) &&
             (k.c_overflow || k.n_contacts > c->cfg.max_contacts || k.n_rays > c->ct.max_rays)) {
        if (k.c_overflow & CONTACT_ORDER)
            status = fail(c, CG_ERR_OUTPUT_OVERFLOW, "contact order: a leaf pair deeper than 127 splits of the "
                          "simultaneous descent");
        else
            status = fail(c, CG_ERR_OUTPUT_OVERFLOW, "%u triangles with colliding pairs, %u rays (max_contacts %llu, "
                          "flags %u): raise max_contacts", k.n_contacts, k.n_rays,
                          (unsigned long long)c->cfg.max_contacts, k.c_overflow);
    }
    s.status = status;
    if (st) *st = s;
    return status;
}

int check_flags(cg_ctx* c, uint32_t flags) {
    if (flags & CG_DFS_ORDER) {
        if (!(flags & CG_KEEP_LEAF_PAIRS) || !c->d_leafs)
            return fail(c, CG_ERR_INVALID_ARGUMENT, "CG_DFS_ORDER orders the kept leaf pairs: it needs "
                        "CG_KEEP_LEAF_PAIRS and max_leaf_pairs > 0");
        if (!c->d_leaf_keys)
            CG_CUDA(cudaMalloc(&c->d_leaf_keys, sizeof(ulonglong2) * c->cfg.max_leaf_pairs), "alloc leaf-pair keys");
    }
    if (!(flags & CG_CONTACTS)) return CG_OK;
    if (!c->cfg.max_contacts) return fail(c, CG_ERR_INVALID_ARGUMENT, "CG_CONTACTS needs max_contacts > 0");
    if (flags & (CG_NO_TRI_PAIRS | CG_MID_ONLY))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "CG_CONTACTS needs the colliding pairs (no CG_NO_TRI_PAIRS, CG_MID_ONLY)");
    return CG_OK;
}

int join_stream(cg_ctx* c, cudaStream_t s) {
    if (s == c->stream) return CG_OK;
    // later reads on the context stream wait for work enqueued on s
    CG_CUDA(cudaEventRecord(c->ev_join, s), "event record");
    CG_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "stream wait");
    return CG_OK;
}

// glm-convention 4x4 product and inverse (column-major); see cg_relative_matrix.
void mat_mul(const float* A, const float* B, float* R) {
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k) {
            float acc = A[0 + k] * B[4 * j + 0];
            acc = acc + A[4 + k] * B[4 * j + 1];
            acc = acc + A[8 + k] * B[4 * j + 2];
            acc = acc + A[12 + k] * B[4 * j + 3];
            R[4 * j + k] = acc;
        }
}

void mat_inverse(const float* M, float* R) {
    auto a = [&](int r, int c) { return M[4 * c + r]; };
    const float s01 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1);
    const float s02 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2);
    const float s03 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3);
    const float s12 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2);
    const float s13 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3);
    const float s23 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
    const float q01 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
    const float q02 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2);
    const float q03 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3);
    const float q12 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2);
    const float q13 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3);
    const float q23 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3);
    const float det = s01 * q23 - s02 * q13 + s03 * q12 + s12 * q03 - s13 * q02 + s23 * q01;
    const float inv = 1.0f / det;
    float b[4][4];
    b[0][0] = (a(1, 1) * q23 - a(1, 2) * q13 + a(1, 3) * q12) * inv;
    b[0][1] = (-a(0, 1) * q23 + a(0, 2) * q13 - a(0, 3) * q12) * inv;
    b[0][2] = (a(3, 1) * s23 - a(3, 2) * s13 + a(3, 3) * s12) * inv;
    b[0][3] = (-a(2, 1) * s23 + a(2, 2) * s13 - a(2, 3) * s12) * inv;
    b[1][0] = (-a(1, 0) * q23 + a(1, 2) * q03 - a(1, 3) * q02) * inv;
    b[1][1] = (a(0, 0) * q23 - a(0, 2) * q03 + a(0, 3) * q02) * inv;
    b[1][2] = (-a(3, 0) * s23 + a(3, 2) * s03 - a(3, 3) * s02) * inv;
    b[1][3] = (a(2, 0) * s23 - a(2, 2) * s03 + a(2, 3) * s02) * inv;
    b[2][0] = (a(1, 0) * q13 - a(1, 1) * q03 + a(1, 3) * q01) * inv;
    b[2][1] = (-a(0, 0) * q13 + a(0, 1) * q03 - a(0, 3) * q01) * inv;
    b[2][2] = (a(3, 0) * s13 - a(3, 1) * s03 + a(3, 3) * s01) * inv;
    b[2][3] = (-a(2, 0) * s13 + a(2, 1) * s03 - a(2, 3) * s01) * inv;
    b[3][0] = (-a(1, 0) * q12 + a(1, 1) * q02 - a(1, 2) * q01) * inv;
    b[3][1] = (a(0, 0) * q12 - a(0, 1) * q02 + a(0, 2) * q01) * inv;
    b[3][2] = (-a(3, 0) * s12 + a(3, 1) * s02 - a(3, 2) * s01) * inv;
    b[3][3] = (a(2, 0) * s12 - a(2, 1) * s02 + a(2, 2) * s01) * inv;
    for (int col = 0; col < 4; ++col)
        for (int r = 0; r < 4; ++r) R[4 * col + r] = b[r][col];
}

}  // namespace cg_host

using namespace cg_host;

extern "C" {

void cg_config_default(cg_config* cfg) {
    if (!cfg) return;
    cfg->device = 0;
    cfg->max_queries = 1u << 16;
    cfg->max_tri_pairs = 1ull << 23;
    cfg->max_leaf_pairs = 1ull << 22;
    cfg->queue_capacity = 1u << 20;
    cfg->warps_per_block = 4;
    cfg->blocks_per_sm = 2;
    cfg->stack_entries = 512;
    cfg->donate_min = 32;
    cfg->leaf_flush = 32;
    cfg->wait_limit_ms = 2000;
    cfg->pad = 0;
    cfg->max_contacts = 1ull << 18;
}

const char* cg_status_string(int s) {
    switch (s) {
        case CG_OK: return "ok";
        case CG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case CG_ERR_CUDA: return "CUDA error";
        case CG_ERR_OUT_OF_MEMORY: return "out of device memory";
        case CG_ERR_QUEUE_OVERFLOW: return "work queue overflow";
        case CG_ERR_OUTPUT_OVERFLOW: return "output overflow";
        case CG_ERR_TIMEOUT: return "device wait timed out";
        case CG_ERR_BAD_TREE: return "malformed tree";
        case CG_ERR_NOT_FOUND: return "unknown tree id";
        default: return "unknown status";
    }
}

int cg_last_error(const cg_ctx* c, char* buf, size_t len) {
    if (!c || !buf || len == 0) return CG_ERR_INVALID_ARGUMENT;
    std::snprintf(buf, len, "%s", c->err.c_str());
    return CG_OK;
}

int cg_create(const cg_config* cfg_in, cg_ctx** out) {
    if (!out) return CG_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cg_config cfg;
    if (cfg_in)
        cfg = *cfg_in;
    else
        cg_config_default(&cfg);
    auto* c = new cg_ctx;
    c->cfg = cfg;
    c->recs.width = 8;  // units of two records: every tree starts on a 128-byte line
    c->tris.width = 3;
    int rc = check_config(c, &cfg);
    if (rc != CG_OK) {
        delete c;
        return rc;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0 || cfg.device < 0 || cfg.device >= ndev) {
        delete c;
        return CG_ERR_CUDA;
    }
    c->device = cfg.device;
    if (cudaSetDevice(c->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev_t0) != cudaSuccess || cudaEventCreate(&c->ev_t1) != cudaSuccess ||
        cudaEventCreate(&c->ev_t2) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_joined, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->branch, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_branch, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_branched, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&c->d_trace, sizeof(unsigned int) * 4 * kTraceBuckets) != cudaSuccess) {
        delete c;
        return CG_ERR_CUDA;
    }
    // where the device reads pageable host memory (Grace), the tree build
    // pulls the meshes itself; CG_PAGEABLE_ACCESS=0 keeps the copies
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c->device) != cudaSuccess) pageable = 0;
    const char* pa = std::getenv("CG_PAGEABLE_ACCESS");
    c->pageable_access = pageable && !(pa && pa[0] == '0');
    rc = alloc_buffers(c);
    if (rc != CG_OK) {
        free_buffers(c);
        cudaStreamDestroy(c->stream);
        delete c;
        return rc;
    }
    *out = c;
    return CG_OK;
}

int cg_destroy(cg_ctx* c) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    for (auto& s : c->trees) {
        if (!s.pool) {
            cudaFree(s.nrm);
            cudaFree(s.ranges);
            cudaFree(s.topo);
        }
        s = cg_ctx::Slot{};
    }
    c->recs.destroy();
    c->tris.destroy();
    cudaFree(c->d_trees);
    cudaFree(c->deform_table.dev);
    cudaFree(c->refit_table.dev);
    cudaFree(c->refit_scratch);
    cudaFree(c->skeleton_table.dev);
    cudaFree(c->energy_table.dev);
    cudaFree(c->pose_scratch);
    cudaFree(c->vgrad);
    cudaFree(c->shoot);
    cudaFree(c->broad);
    cudaFree(c->frame);
    cudaFree(c->build);
    free_buffers(c);
    cudaEventDestroy(c->ev_t0);
    cudaEventDestroy(c->ev_t1);
    cudaEventDestroy(c->ev_t2);
    cudaEventDestroy(c->ev_join);
    cudaEventDestroy(c->ev_fork);
    cudaEventDestroy(c->ev_joined);
    cudaStreamDestroy(c->side);
    cudaEventDestroy(c->ev_branch);
    cudaEventDestroy(c->ev_branched);
    cudaStreamDestroy(c->branch);
    cudaStreamDestroy(c->stream);
    delete c;
    return CG_OK;
}

int cg_get_config(const cg_ctx* c, cg_config* out) {
    if (!c || !out) return CG_ERR_INVALID_ARGUMENT;
    *out = c->cfg;
    return CG_OK;
}

int cg_reconfigure(cg_ctx* c, const cg_config* cfg) {
    if (!c || !cfg) return CG_ERR_INVALID_ARGUMENT;
    if (cfg->device != c->device) return fail(c, CG_ERR_INVALID_ARGUMENT, "cannot change device");
    int rc = check_config(c, cfg);
    if (rc != CG_OK) return rc;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    free_buffers(c);
    c->cfg = *cfg;
    CG_CUDA(cudaMalloc(&c->d_trace, sizeof(unsigned int) * 4 * kTraceBuckets), "alloc trace");
    return alloc_buffers(c);
}

int cg_relative_matrix(const float a[16], const float b[16], float out[16]) {
    if (!a || !b || !out) return CG_ERR_INVALID_ARGUMENT;
    float inv[16];
    mat_inverse(a, inv);
    mat_mul(inv, b, out);
    return CG_OK;
}

int cg_tree_upload(cg_ctx* c, const cg_tree_view* v, uint32_t* tree_id) {
    if (!c || !v || !tree_id) return CG_ERR_INVALID_ARGUMENT;
    const uint32_t N = v->node_count, T = v->triangle_count;
    if ((N && (!v->node_obbs || !v->node_ref || !v->node_tri_count)) || (T && !v->triangles_position))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "tree view has null arrays");
    if (N > (0x7fffffffu - 4u) / 2u) return fail(c, CG_ERR_BAD_TREE, "too many nodes");
    // Validation: children of node k are nodes > k (pre-order) and < N; leaf
    // ranges lie inside the triangle array; counts fit 16 bits.
    for (uint32_t k = 0; k < N; ++k)
        for (int s = 0; s < 2; ++s) {
            const uint32_t ref = v->node_ref[2 * k + s], cnt = v->node_tri_count[2 * k + s];
            if (cnt == 0) {
                if (ref <= k || ref >= N) return fail(c, CG_ERR_BAD_TREE, "node %u child %d -> %u", k, s, ref);
            } else {
                if (cnt > 0xffffu || uint64_t(ref) + cnt > T)
                    return fail(c, CG_ERR_BAD_TREE, "node %u leaf %d range [%u, +%u) outside %u triangles", k, s, ref,
                                cnt, T);
            }
        }
    if (N == 0 && T > 0xffffu) return fail(c, CG_ERR_BAD_TREE, "leaf root with %u triangles", T);
    cudaSetDevice(c->device);

    const uint64_t n_recs = 2ull * N + 2ull;  // even: whole 128-byte record pairs
    const uint64_t n_tris = std::max<uint64_t>(T, 1);
    uint64_t rpair = 0, tb = 0;
    CG_CUDA(c->recs.alloc(n_recs / 2, &rpair, c->stream), "record arena");
    const uint64_t rb = 2 * rpair;
    cudaError_t e = c->tris.alloc(n_tris, &tb, c->stream);
    if (e != cudaSuccess) {
        c->recs.release(rpair, n_recs / 2);
        return cuda_fail(c, e, "triangle arena");
    }
    if (rb + n_recs > 0xffffffffull || tb + n_tris > 0x7fffffffull) {
        c->recs.release(rpair, n_recs / 2);
        c->tris.release(tb, n_tris);
        return fail(c, CG_ERR_OUT_OF_MEMORY, "arena index space exhausted");
    }

    // subtree triangle range of every record (the root, then both children of
    // each node; children come after their parent, so a backward pass over
    // the nodes sees each inner child's range before its parent needs it)
    std::vector<uint2> rg(n_recs, make_uint2(0u, ~0u));
    std::vector<uint2> node_rg(N);
    for (uint32_t k = N; k-- > 0;) {
        uint32_t lo = 0xffffffffu, hi = 0;
        for (int s2 = 0; s2 < 2; ++s2) {
            const uint32_t ref = v->node_ref[2 * k + s2], cnt = v->node_tri_count[2 * k + s2];
            const uint2 crg = cnt ? make_uint2(ref, cnt) : node_rg[ref];
            rg[2ull * k + 2 + s2] = crg;
            if (crg.y) {
                lo = std::min(lo, crg.x);
                hi = std::max(hi, crg.x + crg.y);
            }
        }
        node_rg[k] = lo <= hi ? make_uint2(lo, hi - lo) : make_uint2(0u, 0u);
    }
    rg[1] = N ? node_rg[0] : make_uint2(0u, T);
    // an inner box's split word: the first triangle of node k's right child
    auto split_of = [&](uint32_t k) { return uint32_t(tb + rg[2ull * k + 3].x); };

    std::vector<float4> recs(4ull * n_recs, make_float4(0, 0, 0, 0));
    put_box(&recs[4], v->root_obb, N ? uint32_t(rb + 2) : uint32_t(tb), N ? 0u : (kLeafFlag | T), N ? split_of(0) : 0u);
    for (uint32_t k = 0; k < N; ++k)
        for (int s = 0; s < 2; ++s) {
            const uint64_t r = 2ull * k + 2 + s;
            const uint32_t ref = v->node_ref[2 * k + s];
            const uint32_t cnt = v->node_tri_count[2 * k + s];
            const uint32_t abs_ref = cnt ? uint32_t(tb + ref) : uint32_t(rb + 2ull * ref + 2);
            put_box(&recs[4 * r], v->node_obbs[2 * k + s], abs_ref, cnt ? (kLeafFlag | cnt) : 0u,
                    cnt ? 0u : split_of(ref));
        }
    std::vector<float4> tris(3ull * n_tris, make_float4(0, 0, 0, 0));
    for (uint32_t t = 0; t < T; ++t)
        for (int k = 0; k < 3; ++k) {
            const float* p = v->triangles_position + 9ull * t + 3 * k;
            const uint32_t vi = v->triangles_indices ? v->triangles_indices[3ull * t + k] : 3u * t + k;
            float w;
            std::memcpy(&w, &vi, 4);
            tris[3ull * t + k] = make_float4(p[0], p[1], p[2], w);
        }

    cg_ctx::Slot slot;
    slot.rec_base = rb;
    slot.n_recs = n_recs;
    slot.tri_base = tb;
    slot.n_tris = n_tris;
    CG_CUDA(cudaMemcpyAsync(c->recs.ptr + 4 * rb, recs.data(), sizeof(float4) * recs.size(), cudaMemcpyHostToDevice,
                            c->stream),
            "upload records");
    CG_CUDA(cudaMemcpyAsync(c->tris.ptr + 3 * tb, tris.data(), sizeof(float4) * tris.size(), cudaMemcpyHostToDevice,
                            c->stream),
            "upload triangles");
    if (v->triangles_normal && T) {
        CG_CUDA(cudaMalloc(&slot.nrm, sizeof(float) * 9ull * T), "alloc normals");
        CG_CUDA(cudaMemcpyAsync(slot.nrm, v->triangles_normal, sizeof(float) * 9ull * T, cudaMemcpyHostToDevice,
                                c->stream),
                "upload normals");
    }
    {
        CG_CUDA(cudaMalloc(&slot.ranges, sizeof(uint2) * n_recs), "alloc record ranges");
        CG_CUDA(cudaMemcpyAsync(slot.ranges, rg.data(), sizeof(uint2) * n_recs, cudaMemcpyHostToDevice, c->stream),
                "upload record ranges");
        // the refit's view of the topology: the parent box of every record and
        // the list of leaf boxes in tree order (a node's record is known
        // before its children's: pre-order)
        std::vector<uint32_t> topo(n_recs, ~0u), rec_of_node(N, ~0u), leaves;
        uint32_t* parent = topo.data();
        if (N) rec_of_node[0] = 1;
        for (uint32_t k = 0; k < N; ++k)
            for (int s2 = 0; s2 < 2; ++s2) {
                const uint32_t r = 2u * k + 2u + uint32_t(s2);
                const uint32_t ref = v->node_ref[2 * k + s2], cnt = v->node_tri_count[2 * k + s2];
                parent[r] = rec_of_node[k];
                if (!cnt)
                    rec_of_node[ref] = r;
                else
                    leaves.push_back(r);
            }
        if (!N) leaves.push_back(1u);
        topo.insert(topo.end(), leaves.begin(), leaves.end());
        slot.n_leaves = uint32_t(leaves.size());
        CG_CUDA(cudaMalloc(&slot.topo, sizeof(uint32_t) * topo.size()), "alloc refit topology");
        CG_CUDA(cudaMemcpyAsync(slot.topo, topo.data(), sizeof(uint32_t) * topo.size(), cudaMemcpyHostToDevice,
                                c->stream),
                "upload refit topology");
        CG_CUDA(cudaStreamSynchronize(c->stream), "upload record ranges");
    }
    slot.n_tri_used = T;
    CG_CUDA(launch_surfaces(c->recs.ptr, uint32_t(rb), uint32_t(n_recs), c->stream), "surface kernel");
    CG_CUDA(cudaStreamSynchronize(c->stream), "tree upload");
    slot.live = true;

    uint32_t id = uint32_t(c->trees.size());
    for (uint32_t i = 0; i < c->trees.size(); ++i)
        if (!c->trees[i].live) {
            id = i;
            break;
        }
    if (id == c->trees.size())
        c->trees.push_back(slot);
    else
        c->trees[id] = slot;
    int rc = sync_tree_table(c);
    if (rc != CG_OK) return rc;
    *tree_id = id;
    return CG_OK;
}

int cg_tree_free(cg_ctx* c, uint32_t id) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (id >= c->trees.size() || !c->trees[id].live) return fail(c, CG_ERR_NOT_FOUND, "tree %u", id);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    auto& s = c->trees[id];
    c->recs.release(s.rec_base / 2, s.n_recs / 2);
    c->tris.release(s.tri_base, s.n_tris);
    if (!s.pool) {
        cudaFree(s.nrm);
        cudaFree(s.ranges);
        cudaFree(s.topo);
    }
    s = cg_ctx::Slot{};
    return sync_tree_table(c);
}

int cg_collide_async(cg_ctx* c, const cg_query* d_queries, uint32_t n, uint32_t flags, void* stream) {
    if (!c || (n && !d_queries)) return CG_ERR_INVALID_ARGUMENT;
    if (n > c->cfg.max_queries)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "%u queries > max_queries %u", n, c->cfg.max_queries);
    int frc = check_flags(c, flags);
    if (frc != CG_OK) return frc;
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    c->last_flags = flags;
    c->last_n = n;
    int rc = enqueue_step(c, d_queries, n, flags, s);
    if (rc != CG_OK) return rc;
    return join_stream(c, s);
}

int cg_sync_stats(cg_ctx* c, cg_stats* st) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    CG_CUDA(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "read counters");
    CG_CUDA(cudaStreamSynchronize(c->stream), "collide");
    return stats_from(c, *c->h_ctr, st);
}

int cg_collide(cg_ctx* c, const cg_query* queries, uint32_t n, uint32_t flags, cg_stats* st) {
    if (!c || (n && !queries)) return CG_ERR_INVALID_ARGUMENT;
    if (n > c->cfg.max_queries)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "%u queries > max_queries %u", n, c->cfg.max_queries);
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t a = queries[i].tree_a, b = queries[i].tree_b;
        if (a >= c->trees.size() || !c->trees[a].live || b >= c->trees.size() || !c->trees[b].live)
            return fail(c, CG_ERR_NOT_FOUND, "query %u names tree %u / %u", i, a, b);
    }
    int frc = check_flags(c, flags);
    if (frc != CG_OK) return frc;
    cudaSetDevice(c->device);
    if (n) std::memcpy(c->h_queries, queries, sizeof(cg_query) * n);
    c->last_flags = flags;
    c->last_n = n;
    // The whole step (kernels, counter read-back) is one CUDA graph, captured
    // once per (n, flags) and tree-storage generation and replayed; the pack
    // kernel reads the queries from the pinned staging buffer through the
    // device's mapping of it.
    auto& G = c->host_graph;
    if (!G.exec || G.n != n || G.flags != flags || G.gen != arena_gen(c) ||
        G.out_gen != c->host_out.gen) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        G.exec = nullptr;
        CG_CUDA(cudaStreamSynchronize(c->stream), "sync before capture");
        CG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        c->capturing = true;
        void* q_dev = nullptr;
        cudaError_t e = cudaHostGetDevicePointer(&q_dev, c->h_queries, 0);
        // results to the host buffers: the pairs on a branch beside the
        // contact kernels, the rays and averages by the contact kernels that
        // make them
        CopyOutParams pc{}, rc2{};
        pc.ctr = rc2.ctr = c->d_ctr;
        pc.pairs = c->d_pairs;
        pc.pairs_avail = c->d_pairs ? c->cfg.max_tri_pairs : 0;
        pc.host_pairs = (flags & (CG_NO_TRI_PAIRS | CG_MID_ONLY)) ? nullptr : c->host_out.pairs;
        pc.host_pairs_cap = c->host_out.pairs_cap;
        const bool contacts = (flags & CG_CONTACTS) != 0;
        rc2.rays = c->ct.rays;
        rc2.rays_avail = c->ct.max_rays;
        rc2.host_rays = contacts ? c->host_out.rays : nullptr;
        rc2.host_rays_cap = c->host_out.rays_cap;
        rc2.averages = c->ct.averages;
        rc2.host_averages = contacts ? c->host_out.averages : nullptr;
        rc2.host_averages_cap = c->host_out.averages_cap;
        int rc = e == cudaSuccess ? enqueue_step(c, static_cast<const cg_query*>(q_dev), n, flags, c->stream,
                                                 pc.host_pairs ? &pc : nullptr, &rc2)
                                  : CG_ERR_CUDA;
        if (rc == CG_OK && e == cudaSuccess)
            e = cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream);
        c->capturing = false;
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
        if (rc != CG_OK || e != cudaSuccess || ee != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return rc != CG_OK ? rc : cuda_fail(c, e != cudaSuccess ? e : ee, "capture collide step");
        }
        e = cudaGraphInstantiate(&G.exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(c, e, "instantiate collide step");
        G.n = n;
        G.flags = flags;
        G.gen = arena_gen(c);
        G.out_gen = c->host_out.gen;
    }
    CG_CUDA(cudaGraphLaunch(G.exec, c->stream), "collide step");
    CG_CUDA(cudaStreamSynchronize(c->stream), "collide");
    return stats_from(c, *c->h_ctr, st);
}

int cg_read_tri_pairs(cg_ctx* c, cg_tri_pair* out, uint64_t cap, uint64_t* n) {
    if (!c || !n || (cap && !out)) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    CG_CUDA(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "read counters");
    CG_CUDA(cudaStreamSynchronize(c->stream), "read counters");
    const uint64_t avail = std::min<uint64_t>(c->h_ctr->n_pairs, c->d_pairs ? c->cfg.max_tri_pairs : 0);
    *n = c->h_ctr->n_pairs;
    const uint64_t m = std::min(avail, cap);
    if (m) CG_CUDA(cudaMemcpy(out, c->d_pairs, sizeof(cg_tri_pair) * m, cudaMemcpyDeviceToHost), "read pairs");
    return c->h_ctr->n_pairs > avail ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
}

int cg_set_host_outputs(cg_ctx* c, cg_tri_pair* pairs, uint64_t pairs_cap, cg_ray* rays, uint64_t rays_cap,
                        cg_ray_average* averages, uint64_t averages_cap) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    // the device's address of a host buffer it can write (null: none)
    auto alias = [&](void* h, uint64_t cap, uintptr_t align, const char* what, void** d) -> int {
        *d = nullptr;
        if (!h || !cap) return CG_OK;
        if (!aligned_to(h, align))
            return fail(c, CG_ERR_INVALID_ARGUMENT, "host %s buffer must be %u-byte aligned", what, unsigned(align));
        const cudaError_t e = cudaHostGetDevicePointer(d, h, 0);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(c, CG_ERR_INVALID_ARGUMENT, "the device cannot write the host %s buffer (%s)", what,
                        cudaGetErrorString(e));
        }
        return CG_OK;
    };
    void *dp = nullptr, *dr = nullptr, *da = nullptr;
    int rc = alias(pairs, pairs_cap, 16, "pair", &dp);
    if (rc == CG_OK) rc = alias(rays, rays_cap, 16, "ray", &dr);
    if (rc == CG_OK) rc = alias(averages, averages_cap, 16, "ray-average", &da);
    if (rc != CG_OK) return rc;
    auto& H = c->host_out;
    H.pairs = static_cast<cg_tri_pair*>(dp);
    H.pairs_cap = dp ? pairs_cap : 0;
    H.rays = static_cast<cg_ray*>(dr);
    H.rays_cap = dr ? rays_cap : 0;
    H.averages = static_cast<cg_ray_average*>(da);
    H.averages_cap = da ? averages_cap : 0;
    ++H.gen;
    return CG_OK;
}

int cg_read_leaf_pairs(cg_ctx* c, cg_leaf_pair* out, uint64_t cap, uint64_t* n) {
    if (!c || !n || (cap && !out)) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    CG_CUDA(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "read counters");
    CG_CUDA(cudaStreamSynchronize(c->stream), "read counters");
    const uint64_t avail = std::min<uint64_t>(c->h_ctr->n_leafs, c->d_leafs ? c->cfg.max_leaf_pairs : 0);
    *n = c->h_ctr->n_leafs;
    const uint64_t m = std::min(avail, cap);
    if (m && (c->last_flags & CG_DFS_ORDER)) {
        // grouped by query, each query's in the order of its descent path
        std::vector<cg_leaf_pair> all(avail);
        std::vector<ulonglong2> keys(avail);
        CG_CUDA(cudaMemcpy(all.data(), c->d_leafs, sizeof(cg_leaf_pair) * avail, cudaMemcpyDeviceToHost),
                "read leaf pairs");
        CG_CUDA(cudaMemcpy(keys.data(), c->d_leaf_keys, sizeof(ulonglong2) * avail, cudaMemcpyDeviceToHost),
                "read leaf-pair keys");
        std::vector<uint32_t> order(avail);
        for (uint32_t i = 0; i < avail; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
            if (all[x].query != all[y].query) return all[x].query < all[y].query;
            if (keys[x].x != keys[y].x) return keys[x].x < keys[y].x;
            return keys[x].y < keys[y].y;
        });
        for (uint64_t i = 0; i < m; ++i) out[i] = all[order[i]];
    } else if (m) {
        CG_CUDA(cudaMemcpy(out, c->d_leafs, sizeof(cg_leaf_pair) * m, cudaMemcpyDeviceToHost), "read leaf pairs");
    }
    return c->h_ctr->n_leafs > avail ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
}

namespace {
// Counters of the last launch, which must have been made with CG_CONTACTS.
int contact_counters(cg_ctx* c) {
    if (!(c->last_flags & CG_CONTACTS)) return fail(c, CG_ERR_INVALID_ARGUMENT, "the last launch had no CG_CONTACTS");
    cudaSetDevice(c->device);
    CG_CUDA(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "read counters");
    CG_CUDA(cudaStreamSynchronize(c->stream), "read counters");
    return CG_OK;
}
}  // namespace

int cg_read_contacts(cg_ctx* c, cg_contact* out, uint64_t cap, uint64_t* n) {
    if (!c || !n || (cap && !out)) return CG_ERR_INVALID_ARGUMENT;
    int rc = contact_counters(c);
    if (rc != CG_OK) return rc;
    const uint64_t total = c->h_ctr->n_elems;
    const uint64_t avail = std::min<uint64_t>(total, c->cfg.max_contacts);
    *n = total;
    const uint64_t m = std::min(avail, cap);
    if (m) CG_CUDA(cudaMemcpy(out, c->ct.contacts, sizeof(cg_contact) * m, cudaMemcpyDeviceToHost), "read contacts");
    return (total > avail || c->h_ctr->c_overflow) ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
}

int cg_read_rays(cg_ctx* c, cg_ray* out, uint64_t cap, uint64_t* n) {
    if (!c || !n || (cap && !out)) return CG_ERR_INVALID_ARGUMENT;
    int rc = contact_counters(c);
    if (rc != CG_OK) return rc;
    const uint64_t total = c->h_ctr->n_rays;
    const uint64_t avail = std::min<uint64_t>(total, c->ct.max_rays);
    *n = total;
    const uint64_t m = std::min(avail, cap);
    if (m) CG_CUDA(cudaMemcpy(out, c->ct.rays, sizeof(cg_ray) * m, cudaMemcpyDeviceToHost), "read rays");
    return (total > avail || c->h_ctr->c_overflow) ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
}

int cg_read_ray_averages(cg_ctx* c, cg_ray_average* out, uint64_t cap, uint64_t* n) {
    if (!c || !n || (cap && !out)) return CG_ERR_INVALID_ARGUMENT;
    int rc = contact_counters(c);
    if (rc != CG_OK) return rc;
    const uint64_t total = c->h_ctr->n_queries;
    *n = total;
    const uint64_t m = std::min(total, cap);
    if (m)
        CG_CUDA(cudaMemcpy(out, c->ct.averages, sizeof(cg_ray_average) * m, cudaMemcpyDeviceToHost), "read averages");
    return c->h_ctr->c_overflow ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
}

int cg_device_results(cg_ctx* c, const cg_tri_pair** pairs, const unsigned long long** pair_count) {
    if (!c || !pairs || !pair_count) return CG_ERR_INVALID_ARGUMENT;
    *pairs = c->d_pairs;
    *pair_count = &c->d_ctr->n_pairs;
    return CG_OK;
}

int cg_traversal_time_ms(cg_ctx* c, float* ms) {
    if (!c || !ms) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    CG_CUDA(cudaEventSynchronize(c->ev_t1), "timing event");
    CG_CUDA(cudaEventElapsedTime(ms, c->ev_t0, c->ev_t1), "timing");
    return CG_OK;
}

int cg_narrow_time_ms(cg_ctx* c, float* ms) {
    if (!c || !ms) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    CG_CUDA(cudaEventSynchronize(c->ev_t2), "timing event");
    CG_CUDA(cudaEventElapsedTime(ms, c->ev_t1, c->ev_t2), "timing");
    return CG_OK;
}

int cg_read_trace(cg_ctx* c, uint32_t bucket_ns, uint32_t* out, uint32_t n_buckets) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (bucket_ns) c->trace_ns = bucket_ns;
    if (!out || !n_buckets) return CG_OK;
    const uint32_t m = std::min<uint32_t>(n_buckets, kTraceBuckets);
    CG_CUDA(cudaStreamSynchronize(c->stream), "trace");
    CG_CUDA(cudaMemcpy(out, c->d_trace, sizeof(uint32_t) * 4 * m, cudaMemcpyDeviceToHost), "read trace");
    return CG_OK;
}

int cg_tree_download(cg_ctx* c, uint32_t id, cg_obb* root, cg_obb* node_obbs, uint32_t node_count,
                     float* triangles_position, uint32_t triangle_count) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (id >= c->trees.size() || !c->trees[id].live) return fail(c, CG_ERR_NOT_FOUND, "tree %u", id);
    const auto& t = c->trees[id];
    const uint32_t N = uint32_t((t.n_recs - 2) / 2);
    if ((node_count && node_count != N) || (triangle_count && triangle_count != t.n_tri_used))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "tree %u has %u nodes and %u triangles", id, N, t.n_tri_used);
    cudaSetDevice(c->device);
    CG_CUDA(cudaStreamSynchronize(c->stream), "download tree");
    auto unbox = [](const float4* r, cg_obb* b) {
        b->center[0] = r[0].x, b->center[1] = r[0].y, b->center[2] = r[0].z;
        b->u[0] = r[0].w, b->u[1] = r[1].x, b->u[2] = r[1].y;
        b->v[0] = r[1].z, b->v[1] = r[1].w, b->v[2] = r[2].x;
        b->w[0] = r[2].y, b->w[1] = r[2].z, b->w[2] = r[2].w;
    };
    if (root || (node_obbs && node_count)) {
        std::vector<float4> recs(4ull * t.n_recs);
        CG_CUDA(cudaMemcpy(recs.data(), c->recs.ptr + 4 * t.rec_base, sizeof(float4) * recs.size(),
                           cudaMemcpyDeviceToHost),
                "download records");
        if (root) unbox(&recs[4], root);
        if (node_obbs)
            for (uint32_t r = 2; r < t.n_recs; ++r) unbox(&recs[4ull * r], node_obbs + (r - 2));
    }
    if (triangles_position && triangle_count) {
        std::vector<float4> tris(3ull * triangle_count);
        CG_CUDA(cudaMemcpy(tris.data(), c->tris.ptr + 3 * t.tri_base, sizeof(float4) * tris.size(),
                           cudaMemcpyDeviceToHost),
                "download triangles");
        for (size_t k = 0; k < tris.size(); ++k) {
            triangles_position[3 * k] = tris[k].x;
            triangles_position[3 * k + 1] = tris[k].y;
            triangles_position[3 * k + 2] = tris[k].z;
        }
    }
    return CG_OK;
}

int cg_tree_refit_batch(cg_ctx* c, const uint32_t* tree_ids, const float* const* positions,
                        const uint32_t* n_positions, uint32_t n, void* stream) {
    if (!c || (n && (!tree_ids || !positions || !n_positions))) return CG_ERR_INVALID_ARGUMENT;
    if (n == 0) return CG_OK;
    std::vector<RefitTree> table(n);
    uint32_t max_tris = 0, max_recs = 0, total_recs = 0, max_leaves = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t id = tree_ids[i];
        if (id >= c->trees.size() || !c->trees[id].live) return fail(c, CG_ERR_NOT_FOUND, "tree %u", id);
        if ((!positions[i] && n_positions[i]) || (reinterpret_cast<uintptr_t>(positions[i]) & 15u))
            return fail(c, CG_ERR_INVALID_ARGUMENT, "positions %u must be 16-byte aligned device memory", i);
        const auto& t = c->trees[id];
        table[i] = RefitTree{uint32_t(t.rec_base), uint32_t(t.n_recs), uint32_t(t.tri_base), t.n_tri_used, t.ranges,
                             reinterpret_cast<const float4*>(positions[i]), n_positions[i], total_recs,
                             t.topo, t.topo + t.n_recs, t.n_leaves, 0u};
        max_leaves = std::max(max_leaves, t.n_leaves);
        total_recs += uint32_t(t.n_recs);
        max_tris = std::max(max_tris, t.n_tri_used);
        max_recs = std::max(max_recs, uint32_t(t.n_recs));
    }
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    const void* d_table = nullptr;
    int rc = stage_table(c, c->refit_table, table.data(), sizeof(RefitTree) * n, s, &d_table);
    if (rc != CG_OK) return rc;
    if (total_recs > c->refit_scratch_cap) {
        CG_CUDA(cudaStreamSynchronize(s), "refit scratch");
        cudaFree(c->refit_scratch);
        c->refit_scratch = nullptr;
        c->refit_scratch_cap = 0;
        CG_CUDA(cudaMalloc(&c->refit_scratch, refit_bytes(total_recs)), "alloc refit scratch");
        c->refit_scratch_cap = total_recs;
        CG_CUDA(init_refit_scratch(refit_bufs(c->refit_scratch, total_recs), total_recs, s), "clear refit scratch");
    }
    CG_CUDA(launch_refit(c->recs.ptr, c->tris.ptr, static_cast<const RefitTree*>(d_table), n, max_tris, max_recs,
                         max_leaves, refit_bufs(c->refit_scratch, c->refit_scratch_cap), s),
            "refit kernels");
    return CG_OK;
}

int cg_tree_refit(cg_ctx* c, uint32_t id, const float* positions, uint32_t n_positions, void* stream) {
    return cg_tree_refit_batch(c, &id, &positions, &n_positions, 1, stream);
}

int cg_deform_batch(cg_ctx* c, const cg_deform_view* views, float* const* outs, uint32_t n, void* stream) {
    if (!c || (n && (!views || !outs))) return CG_ERR_INVALID_ARGUMENT;
    std::vector<DeformParams> table(n);
    uint32_t max_vertices = 0, max_joints = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const int rc = deform_params(c, views + i, outs[i], true, i, &table[i]);
        if (rc != CG_OK) return rc;
        max_vertices = std::max(max_vertices, table[i].n_vertices);
        max_joints = std::max(max_joints, table[i].n_joints);
    }
    if (n == 0 || max_vertices == 0) return CG_OK;
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    const void* d_table = nullptr;
    int rc = stage_table(c, c->deform_table, table.data(), sizeof(DeformParams) * n, s, &d_table);
    if (rc != CG_OK) return rc;
    CG_CUDA(launch_deform(static_cast<const DeformParams*>(d_table), n, max_vertices, max_joints, s), "deform kernel");
    return CG_OK;
}

int cg_deform(cg_ctx* c, const cg_deform_view* v, float* out, void* stream) {
    return cg_deform_batch(c, v, &out, 1, stream);
}

int cg_pose(cg_ctx* c, const cg_skeleton_view* sk, const float* d_axis_angles, uint32_t n_poses,
            float* d_joint_matrices, void* stream) {
    if (!c || !sk || (n_poses && (!d_axis_angles || !d_joint_matrices))) return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    PoseParams p{};
    int rc = pose_params(c, sk, n_poses, s, &p);
    if (rc != CG_OK) return rc;
    p.axis_angles = d_axis_angles;
    p.joint_matrices = d_joint_matrices;
    CG_CUDA(launch_pose(p, s), "pose kernel");
    return CG_OK;
}

int cg_pose_backward(cg_ctx* c, const cg_skeleton_view* sk, const float* d_axis_angles, const float* d_joint_matrices,
                     const float* d_grad_joint_matrices, uint32_t n_poses, float* d_grad_axis_angles, void* stream) {
    if (!c || !sk || (n_poses && (!d_axis_angles || !d_joint_matrices || !d_grad_joint_matrices || !d_grad_axis_angles)))
        return CG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    PoseParams p{};
    int rc = pose_params(c, sk, n_poses, s, &p);
    if (rc != CG_OK) return rc;
    const uint64_t need = uint64_t(n_poses) * p.n_bones * 37u;  // dE/dG, local matrices, dE/dR per bone
    if (need > c->pose_scratch_cap) {
        CG_CUDA(cudaStreamSynchronize(s), "pose scratch");
        cudaFree(c->pose_scratch);
        c->pose_scratch = nullptr;
        c->pose_scratch_cap = 0;
        CG_CUDA(cudaMalloc(&c->pose_scratch, sizeof(float) * need), "alloc pose scratch");
        c->pose_scratch_cap = need;
    }
    p.axis_angles = d_axis_angles;
    p.joint_matrices = const_cast<float*>(d_joint_matrices);  // read only in the adjoint
    p.grad_joint = d_grad_joint_matrices;
    p.grad_acc = c->pose_scratch;
    p.grad_axis_angles = d_grad_axis_angles;
    CG_CUDA(launch_pose_backward(p, s), "pose adjoint kernel");
    return CG_OK;
}

int cg_energy(cg_ctx* c, double* d_energy, void* stream) {
    if (!c || !d_energy) return CG_ERR_INVALID_ARGUMENT;
    int rc = energy_ready(c);
    if (rc != CG_OK) return rc;
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    EnergyParams p = energy_params(c);
    p.energy = d_energy;
    CG_CUDA(cudaMemsetAsync(d_energy, 0, sizeof(double), s), "clear energy");
    CG_CUDA(launch_energy(p, c->energy_blocks, s), "energy kernel");
    return CG_OK;
}

int cg_energy_backward(cg_ctx* c, const double* d_grad_energy, const cg_energy_side* side_a,
                       const cg_energy_side* side_b, void* stream) {
    if (!c || !d_grad_energy) return CG_ERR_INVALID_ARGUMENT;
    int rc = energy_ready(c);
    if (rc != CG_OK) return rc;
    const uint32_t n = c->last_n;
    std::vector<EnergySide> sides(2ull * n);
    std::vector<uint32_t> deforming;
    uint64_t total = 0;
    uint32_t max_vertices = 0, max_joints = 0, max_targets = 0;
    const cg_energy_side* both[2] = {side_a, side_b};
    for (uint32_t k = 0; k < 2; ++k) {
        const cg_energy_side* sd = both[k];
        if (!sd || !sd->views) continue;
        for (uint32_t q = 0; q < n; ++q) {
            const cg_deform_view* v = sd->views + q;
            if (!v->n_vertices) continue;
            if (!sd->grad_joint_matrices || (sd->target_stride && !sd->grad_morph_weights))
                return fail(c, CG_ERR_INVALID_ARGUMENT, "energy side %u: null gradient arrays", k);
            EnergySide& e = sides[size_t(k) * n + q];
            rc = deform_params(c, v, nullptr, false, q, &e.d);
            if (rc != CG_OK) return rc;
            if (e.d.n_joints > sd->joint_stride || v->n_targets > sd->target_stride || v->n_targets > 256u)
                return fail(c, CG_ERR_INVALID_ARGUMENT,
                            "energy side %u view %u: %u joints / %u targets over the strides %u / %u (targets <= 256)",
                            k, q, e.d.n_joints, v->n_targets, sd->joint_stride, sd->target_stride);
            if (total + v->n_vertices > 0xffffffffull)
                return fail(c, CG_ERR_INVALID_ARGUMENT, "more than 2^32 deforming vertices");
            e.grad_base = uint32_t(total);
            total += v->n_vertices;
            e.grad_joint = sd->grad_joint_matrices + size_t(q) * sd->joint_stride * 16u;
            e.grad_morph = sd->grad_morph_weights ? sd->grad_morph_weights + size_t(q) * sd->target_stride : nullptr;
            deforming.push_back(k * n + q);
            max_vertices = std::max(max_vertices, e.d.n_vertices);
            max_joints = std::max(max_joints, e.d.n_joints);
            max_targets = std::max(max_targets, e.d.n_targets);
        }
    }
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    for (uint32_t k = 0; k < 2; ++k) {
        const cg_energy_side* sd = both[k];
        if (!sd || !sd->views || !n) continue;
        if (sd->grad_joint_matrices && sd->joint_stride)
            CG_CUDA(cudaMemsetAsync(sd->grad_joint_matrices, 0, sizeof(float) * 16u * sd->joint_stride * n, s),
                    "clear joint gradients");
        if (sd->grad_morph_weights && sd->target_stride)
            CG_CUDA(cudaMemsetAsync(sd->grad_morph_weights, 0, sizeof(float) * sd->target_stride * n, s),
                    "clear morph-weight gradients");
    }
    if (deforming.empty()) return CG_OK;
    if (3u * total > c->vgrad_cap) {
        CG_CUDA(cudaStreamSynchronize(s), "vertex gradient buffer");
        cudaFree(c->vgrad);
        c->vgrad = nullptr;
        c->vgrad_cap = 0;
        CG_CUDA(cudaMalloc(&c->vgrad, sizeof(float) * 3u * total), "alloc vertex gradients");
        CG_CUDA(cudaMemset(c->vgrad, 0, sizeof(float) * 3u * total), "zero vertex gradients");
        c->vgrad_cap = 3u * total;
    }
    std::vector<char> blob(sizeof(EnergySide) * sides.size() + sizeof(uint32_t) * deforming.size());
    std::memcpy(blob.data(), sides.data(), sizeof(EnergySide) * sides.size());
    std::memcpy(blob.data() + sizeof(EnergySide) * sides.size(), deforming.data(), sizeof(uint32_t) * deforming.size());
    const void* d_blob = nullptr;
    rc = stage_table(c, c->energy_table, blob.data(), blob.size(), s, &d_blob);
    if (rc != CG_OK) return rc;
    EnergyParams p = energy_params(c);
    p.grad_energy = d_grad_energy;
    p.sides = static_cast<const EnergySide*>(d_blob);
    p.deforming = reinterpret_cast<const uint32_t*>(static_cast<const char*>(d_blob) + sizeof(EnergySide) * sides.size());
    p.n_deforming = uint32_t(deforming.size());
    p.vgrad = c->vgrad;
    p.max_joints = max_joints;
    p.max_targets = max_targets;
    CG_CUDA(launch_energy_backward(p, c->energy_blocks, max_vertices, s), "energy adjoint kernels");
    return CG_OK;
}

int cg_graph_capture(cg_ctx* c, const cg_query* d_queries, uint32_t n, uint32_t flags) {
    if (!c || (n && !d_queries)) return CG_ERR_INVALID_ARGUMENT;
    if (n > c->cfg.max_queries)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "%u queries > max_queries %u", n, c->cfg.max_queries);
    int frc = check_flags(c, flags);
    if (frc != CG_OK) return frc;
    cudaSetDevice(c->device);
    CG_CUDA(cudaStreamSynchronize(c->stream), "sync before capture");
    drop_graph(c);
    CG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    c->capturing = true;
    const int rc = enqueue_step(c, d_queries, n, flags, c->stream);
    c->capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc != CG_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    c->graph = g;
    CG_CUDA(cudaGraphInstantiate(&c->graph_exec, g, 0), "instantiate graph");
    c->graph_gen = arena_gen(c);
    c->graph_n = n;
    c->graph_flags = flags;
    c->last_flags = flags;
    c->last_n = n;
    return CG_OK;
}

int cg_graph_launch(cg_ctx* c, void* stream) {
    if (!c || !c->graph_exec) return fail(c, CG_ERR_INVALID_ARGUMENT, "no captured graph");
    if (c->graph_gen != arena_gen(c))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "tree storage moved since the capture: capture the graph again");
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    CG_CUDA(cudaGraphLaunch(c->graph_exec, s), "graph launch");
    c->last_flags = c->graph_flags;
    c->last_n = c->graph_n;
    return join_stream(c, s);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// cg_collide_static: the collide step with its per-launch scratch in one
// static device array (no allocation on the call's path).
namespace {

constexpr uint32_t kStaticSlots = 65536;      // work-queue chunk slots (ready flags + pool)
constexpr uint32_t kStaticMinChunks = 32768;  // donated chunks a launch may always reserve: cg_collide's default
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffReady = align256(sizeof(Counters));
constexpr size_t kOffPool = kOffReady + align256(sizeof(unsigned int) * kStaticSlots);
constexpr size_t kOffLeaf = kOffPool + align256(sizeof(uint4) * kChunk * kStaticSlots);
constexpr size_t kOffPacked = kOffLeaf + align256(sizeof(uint4) * CG_STATIC_MAX_LEAF_PAIRS);
constexpr size_t kStaticBytes = kOffPacked + align256(sizeof(PackedQuery) * CG_STATIC_MAX_QUERIES);
static_assert(kStaticBytes == CG_STATIC_SCRATCH_BYTES, "CG_STATIC_SCRATCH_BYTES is the static scratch size");

// Counters | ready flags | node-pair pool | leaf-pair list | packed queries
static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

constexpr int kStaticMaxDevices = 64;
unsigned char* g_static_base[kStaticMaxDevices];  // device address of the scratch, per device once set up
std::mutex g_static_mu;

// Once per device, with that device current: the scratch's address, and the
// counters and ready flags (which must start at zero) cleared.
int static_scratch(cg_ctx* c, cudaStream_t s, unsigned char** out) {
    if (c->device < 0 || c->device >= kStaticMaxDevices)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "device %d beyond the static scratch table", c->device);
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_base[c->device]) {
        void* p = nullptr;
        CG_CUDA(cudaGetSymbolAddress(&p, g_static_scratch), "static scratch address");
        CG_CUDA(cudaMemsetAsync(p, 0, kOffPool, s), "clear static scratch");
        CG_CUDA(cudaStreamSynchronize(s), "clear static scratch");
        g_static_base[c->device] = static_cast<unsigned char*>(p);
    }
    *out = g_static_base[c->device];
    return CG_OK;
}

__global__ void static_counts_kernel(const Counters* k, uint64_t pairs_cap, cg_static_counts* out) {
    cg_static_counts r;
    r.tri_pairs = k->n_pairs;
    r.tri_tests = k->tri_tests;
    r.leaf_pairs = k->n_leafs;
    r.pad = 0;
    if (k->error & ERR_TIMEOUT)
        r.status = CG_ERR_TIMEOUT;
    else if (k->error & ERR_QUEUE)
        r.status = CG_ERR_QUEUE_OVERFLOW;
    else if (k->error & ERR_BAD_QUERY)
        r.status = CG_ERR_INVALID_ARGUMENT;
    else if (k->n_leafs > CG_STATIC_MAX_LEAF_PAIRS || (pairs_cap && k->n_pairs > pairs_cap))
        r.status = CG_ERR_OUTPUT_OVERFLOW;  // a count-only call (no pair buffer) is not an overflow
    else
        r.status = CG_OK;
    *out = r;
}

}  // namespace

extern "C" int cg_collide_static(cg_ctx* c, const cg_query* d_queries, uint32_t n, cg_tri_pair* d_pairs,
                                 uint64_t pairs_cap, cg_static_counts* d_counts, void* stream) {
    if (!c || (n && !d_queries) || (pairs_cap && !d_pairs) || !d_counts) return CG_ERR_INVALID_ARGUMENT;
    if (n > CG_STATIC_MAX_QUERIES)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "%u queries > CG_STATIC_MAX_QUERIES (%u)", n, CG_STATIC_MAX_QUERIES);
    CG_CUDA(cudaSetDevice(c->device), "set device");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    unsigned char* base = nullptr;
    int rc = static_scratch(c, s, &base);
    if (rc != CG_OK) return rc;
    auto* ctr = reinterpret_cast<Counters*>(base);
    auto* ready = reinterpret_cast<unsigned int*>(base + kOffReady);
    auto* pool = reinterpret_cast<uint4*>(base + kOffPool);
    auto* leaf_list = reinterpret_cast<uint4*>(base + kOffLeaf);
    auto* packed = reinterpret_cast<PackedQuery*>(base + kOffPacked);

    // The traversal grid is the context's, made smaller if its waiting warps
    // would leave fewer than kStaticMinChunks slots for donations (the
    // default grids leave more).
    const uint32_t wpb = c->cfg.warps_per_block;
    const uint32_t max_blocks = (kStaticSlots - kStaticMinChunks - 64u) / (9u * wpb);
    const uint32_t blocks = std::min(c->blocks, max_blocks);

    CG_CUDA(launch_init(ctr, ready, kStaticSlots, n, nullptr, s), "init kernel");
    CG_CUDA(launch_pack(d_queries, n, c->d_trees, uint32_t(c->trees.size()), c->recs.ptr, packed, ctr, leaf_list,
                        CG_STATIC_MAX_LEAF_PAIRS, s),
            "pack kernel");
    TraverseParams p{};
    p.q = packed;
    p.n_queries = n;
    p.recs = c->recs.ptr;
    p.pool = pool;
    p.ready = ready;
    p.slot_cap = kStaticSlots - 9u * blocks * wpb - 64u;
    p.slot_alloc = kStaticSlots;
    p.ctr = ctr;
    p.leaf_list = leaf_list;
    p.leaf_cap = CG_STATIC_MAX_LEAF_PAIRS;
    p.trace = nullptr;
    p.trace_ns = 1000u;
    p.stack_cap = c->cfg.stack_entries;
    p.donate_min = std::min(std::max(c->cfg.donate_min, 2u), c->cfg.stack_entries - 63u);
    p.leaf_flush = c->cfg.leaf_flush;
    p.wait_ns = (unsigned long long)c->cfg.wait_limit_ms * 1000000ull;
    NarrowParams np{};
    np.q = packed;
    np.tris = c->tris.ptr;
    np.leaf_list = leaf_list;
    np.leaf_cap = CG_STATIC_MAX_LEAF_PAIRS;
    np.ctr = ctr;
    np.pairs = d_pairs;
    np.pair_aux = nullptr;
    np.pairs_cap = d_pairs ? pairs_cap : 0;
    np.leafs = nullptr;
    np.leafs_cap = 0;
    np.flags = 0;
    np.trace = nullptr;
    np.trace_ns = 1000u;
    if (n) CG_CUDA(launch_traverse(p, blocks, wpb, s), "traversal kernel");
    if (n) CG_CUDA(launch_narrow(np, c->narrow_blocks, 8, s), "narrow-phase kernel");
    static_counts_kernel<<<1, 1, 0, s>>>(ctr, np.pairs_cap, d_counts);
    CG_CUDA(cudaGetLastError(), "counts kernel");
    return CG_OK;
}
