// Host side of the C ABI declared in include/collide_gpu.h: context and
// buffers, tree arenas with upload validation, launches, result read-back and
// the CUDA graph of one collide step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "cg_internal.h"
#include "collide_gpu.h"

using namespace cg;

namespace {

// A growable device array of fixed-size units (a unit is `width` float4s)
// with first-fit reuse of released ranges. Growth copies the contents to a
// larger allocation at the same offsets, so indices stay valid; the base
// pointer changes and `gen` counts those changes.
struct Arena {
    float4* ptr = nullptr;
    uint32_t width = 1;
    uint64_t cap = 0;
    uint64_t used = 0;
    uint64_t gen = 0;
    std::vector<std::pair<uint64_t, uint64_t>> free_list;  // (offset, units), sorted by offset

    cudaError_t alloc(uint64_t n, uint64_t* off, cudaStream_t s) {
        for (size_t i = 0; i < free_list.size(); ++i) {
            if (free_list[i].second >= n) {
                *off = free_list[i].first;
                free_list[i].first += n;
                free_list[i].second -= n;
                if (free_list[i].second == 0) free_list.erase(free_list.begin() + long(i));
                return cudaSuccess;
            }
        }
        if (used + n > cap) {
            uint64_t ncap = std::max<uint64_t>(std::max<uint64_t>(cap * 2, used + n), 1u << 14);
            float4* np = nullptr;
            cudaError_t e = cudaMalloc(&np, sizeof(float4) * width * ncap);
            if (e != cudaSuccess) return e;
            if (used) {
                e = cudaStreamSynchronize(s);
                if (e == cudaSuccess)
                    e = cudaMemcpy(np, ptr, sizeof(float4) * width * used, cudaMemcpyDeviceToDevice);
                if (e != cudaSuccess) {
                    cudaFree(np);
                    return e;
                }
            }
            cudaFree(ptr);
            ptr = np;
            cap = ncap;
            ++gen;
        }
        *off = used;
        used += n;
        return cudaSuccess;
    }

    void release(uint64_t off, uint64_t n) {
        if (n == 0) return;
        auto it = std::lower_bound(free_list.begin(), free_list.end(), std::make_pair(off, uint64_t(0)));
        it = free_list.insert(it, {off, n});
        size_t i = size_t(it - free_list.begin());
        if (i + 1 < free_list.size() && free_list[i].first + free_list[i].second == free_list[i + 1].first) {
            free_list[i].second += free_list[i + 1].second;
            free_list.erase(free_list.begin() + long(i + 1));
        }
        if (i > 0 && free_list[i - 1].first + free_list[i - 1].second == free_list[i].first) {
            free_list[i - 1].second += free_list[i].second;
            free_list.erase(free_list.begin() + long(i));
            --i;
        }
        if (free_list[i].first + free_list[i].second == used) {
            used = free_list[i].first;
            free_list.erase(free_list.begin() + long(i));
        }
    }

    void destroy() {
        cudaFree(ptr);
        ptr = nullptr;
        cap = used = 0;
        free_list.clear();
    }
};

}  // namespace

struct cg_ctx {
    cg_config cfg{};
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    uint32_t blocks = 0;         // persistent traversal grid
    uint32_t narrow_blocks = 0;  // persistent narrow-phase grid
    uint32_t accumulate_blocks = 0, emit_blocks = 0;  // contact kernels: one resident wave
    uint32_t energy_blocks = 0;                        // energy kernels: one resident wave

    // trees
    struct Slot {
        uint64_t rec_base = 0, n_recs = 0, tri_base = 0, n_tris = 0;
        uint32_t n_tri_used = 0;  // the tree's triangle count (n_tris is at least 1)
        float* nrm = nullptr;
        uint2* ranges = nullptr;  // per record: first triangle and count of its subtree (refit)
        uint32_t* topo = nullptr;  // refit: parent per record, then the leaf records
        uint32_t n_leaves = 0;
        std::shared_ptr<void> pool;  // the block that holds nrm, ranges and topo when the tree was built here
        bool live = false;
    };
    std::vector<Slot> trees;
    Arena recs, tris;
    DevTree* d_trees = nullptr;
    uint32_t d_trees_cap = 0;
    uint64_t table_gen = 0;         // reallocations of d_trees

    // per-launch buffers
    cg_query* d_queries = nullptr;  // staging for host queries
    PackedQuery* d_packed = nullptr;
    Counters* d_ctr = nullptr;
    uint4* d_pool = nullptr;        // donated node-pair entries
    unsigned int* d_ready = nullptr;
    uint32_t slot_cap = 0;          // chunk slots donors may reserve
    uint32_t slot_alloc = 0;        // allocated, with slack for concurrent reservations and waiters
    uint4* d_leaf_list = nullptr;   // candidate leaf pairs between the two kernels
    cg_tri_pair* d_pairs = nullptr;
    cg_leaf_pair* d_leafs = nullptr;
    unsigned int* d_trace = nullptr;
    uint32_t trace_ns = 0;

    // contacts and rays (CG_CONTACTS), allocated when max_contacts > 0
    struct Contacts {
        uint4* pair_aux = nullptr;
        ContactSlot* table = nullptr;
        uint32_t table_slots = 0;
        uint32_t* occupied = nullptr;
        unsigned long long* vkeys = nullptr;
        uint32_t vslots = 0;
        uint32_t* vocc = nullptr;
        cg_contact* contacts = nullptr;
        cg_ray* rays = nullptr;
        uint32_t max_rays = 0;
        double* sums = nullptr;
        cg_ray_average* averages = nullptr;
    } ct;

    cg_query* h_queries = nullptr;  // pinned
    Counters* h_ctr = nullptr;      // pinned

    uint32_t last_flags = 0;
    uint32_t last_n = 0;            // queries of the last collide step enqueued

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_gen = 0;         // arena generations the graph was captured with
    uint32_t graph_n = 0, graph_flags = 0;
    struct HostGraph {              // cg_collide's own graph of a whole step
        cudaGraphExec_t exec = nullptr;
        uint32_t n = 0, flags = 0;
        uint64_t gen = 0, out_gen = 0;
    } host_graph;
    bool capturing = false;
    // cg_set_host_outputs: page-locked host destinations of cg_collide's
    // results (device aliases), written by the step graph itself
    struct HostOut {
        cg_tri_pair* pairs = nullptr;
        uint64_t pairs_cap = 0;
        cg_ray* rays = nullptr;
        uint64_t rays_cap = 0;
        cg_ray_average* averages = nullptr;
        uint64_t averages_cap = 0;
        uint64_t gen = 0;  // settings changes (the step graph is captured again)
    } host_out;
    uint32_t copy_blocks = 0;
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr, ev_t2 = nullptr;  // traversal start, end; narrow end
    cudaEvent_t ev_join = nullptr;  // joins an external launch stream to the context stream
    cudaStream_t side = nullptr;    // a branch of cg_collide's step graph (host copy of the pairs)
    cudaEvent_t ev_fork = nullptr, ev_joined = nullptr;

    // batch tables of cg_deform_batch / cg_tree_refit_batch in device memory,
    // uploaded when their contents change
    struct Table {
        std::vector<char> host;
        void* dev = nullptr;
        size_t cap = 0;
    } deform_table, refit_table, skeleton_table, energy_table;
    void* refit_scratch = nullptr;          // RefitBufs for this many records of a refit batch
    uint32_t refit_scratch_cap = 0;
    float* pose_scratch = nullptr;          // pose adjoint: dE/dG accumulated per bone
    uint64_t pose_scratch_cap = 0;
    float* vgrad = nullptr;                 // energy adjoint: per-vertex gradient, zero between calls
    uint64_t vgrad_cap = 0;
    void* shoot = nullptr;                  // cg_shoot_rays: queries, rays, tags, per-ray results, deltas, flag
    size_t shoot_cap = 0;
    void* broad = nullptr;                  // cg_broad_phase: ids, globals, callbacks, projections, pairs, count
    size_t broad_cap = 0;
    void* frame = nullptr;                  // cg_collision_frame's buffers
    size_t frame_cap = 0;
    void* build = nullptr;                  // cg_tree_build's scratch
    size_t build_cap = 0;

    std::string err;
};

namespace {

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

#define CG_CUDA(call, what)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)

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
    cudaFree(c->d_trace);
    auto& t = c->ct;
    cudaFree(t.pair_aux);
    cudaFree(t.table);
    cudaFree(t.occupied);
    cudaFree(t.vkeys);
    cudaFree(t.vocc);
    cudaFree(t.contacts);
    cudaFree(t.rays);
    cudaFree(t.sums);
    cudaFree(t.averages);
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
    if (cfg->max_contacts > (1ull << 28)) return fail(c, CG_ERR_INVALID_ARGUMENT, "max_contacts must be <= 2^28");
    if (cfg->max_contacts && (cfg->max_tri_pairs == 0 || cfg->max_tri_pairs >= (1ull << 32)))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "contacts need 0 < max_tri_pairs < 2^32");
    return CG_OK;
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
    int aocc = 0, eocc = 0;
    CG_CUDA(contacts_occupancy(&aocc, &eocc), "occupancy");
    c->accumulate_blocks = uint32_t(std::max(aocc, 1) * c->sm_count);
    c->emit_blocks = uint32_t(std::max(eocc, 1) * c->sm_count);
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
        // Hash tables at most half full: contacts, vertices with a ray (3 per
        // contact at most).
        auto pow2_at_least = [](uint64_t x) {
            uint64_t p = 1024;
            while (p < x) p <<= 1;
            return uint32_t(p);
        };
        auto& t = c->ct;
        t.table_slots = pow2_at_least(2 * g.max_contacts);
        t.vslots = pow2_at_least(6 * g.max_contacts);
        t.max_rays = uint32_t(3 * g.max_contacts);
        CG_CUDA(cudaMalloc(&t.pair_aux, sizeof(uint4) * g.max_tri_pairs), "alloc pair side records");
        CG_CUDA(cudaMalloc(&t.table, sizeof(ContactSlot) * t.table_slots), "alloc contact table");
        CG_CUDA(cudaMalloc(&t.occupied, sizeof(uint32_t) * t.table_slots), "alloc contact list");
        CG_CUDA(cudaMalloc(&t.vkeys, sizeof(unsigned long long) * t.vslots), "alloc vertex set");
        CG_CUDA(cudaMalloc(&t.vocc, sizeof(uint32_t) * t.vslots), "alloc vertex list");
        CG_CUDA(cudaMalloc(&t.contacts, sizeof(cg_contact) * g.max_contacts), "alloc contacts");
        CG_CUDA(cudaMalloc(&t.rays, sizeof(cg_ray) * t.max_rays), "alloc rays");
        CG_CUDA(cudaMalloc(&t.sums, sizeof(double) * 8 * g.max_queries), "alloc ray sums");
        CG_CUDA(cudaMalloc(&t.averages, sizeof(cg_ray_average) * g.max_queries), "alloc ray averages");
        CG_CUDA(init_contact_tables(t.table, t.table_slots, t.vkeys, t.vslots, c->stream), "init contact tables");
        CG_CUDA(cudaStreamSynchronize(c->stream), "init contact tables");
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

void put_box(float4* rec, const cg_obb& b, uint32_t ref, uint32_t meta) {
    rec[0] = make_float4(b.center[0], b.center[1], b.center[2], b.u[0]);
    rec[1] = make_float4(b.u[1], b.u[2], b.v[0], b.v[1]);
    rec[2] = make_float4(b.v[2], b.w[0], b.w[1], b.w[2]);
    float r, m;
    std::memcpy(&r, &ref, 4);
    std::memcpy(&m, &meta, 4);
    rec[3] = make_float4(r, m, 0.f, 0.f);
}

// Enqueues counter reset, packing, the traversal and the narrow phase on `s`.
// pairs_copy: with the step's colliding pairs final (after the narrow phase),
// copy them out on a branch that runs beside the contact kernels.
int enqueue_step(cg_ctx* c, const cg_query* d_queries, uint32_t n, uint32_t flags, cudaStream_t s,
                 const CopyOutParams* pairs_copy = nullptr) {
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
        cp.tris = c->tris.ptr;
        cp.trees = c->d_trees;
        cp.pairs = c->d_pairs;
        cp.pair_aux = t.pair_aux;
        cp.leaf_list = c->d_leaf_list;
        cp.pairs_cap = c->cfg.max_tri_pairs;
        cp.table = t.table;
        cp.table_mask = t.table_slots - 1u;
        cp.occupied = t.occupied;
        cp.vkeys = t.vkeys;
        cp.vtable_mask = t.vslots - 1u;
        cp.vocc = t.vocc;
        cp.max_contacts = uint32_t(c->cfg.max_contacts);
        cp.contacts = t.contacts;
        cp.rays = t.rays;
        cp.max_rays = t.max_rays;
        cp.sums = t.sums;
        cp.averages = t.averages;
        cp.ctr = c->d_ctr;
        CG_CUDA(launch_contacts(cp, c->accumulate_blocks, c->emit_blocks, s), "contact kernels");
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
    s.contacts = k.n_contacts;
    s.rays = k.n_rays;
    int status = CG_OK;
    if (k.error & ERR_TIMEOUT)
        status = fail(c, CG_ERR_TIMEOUT, "a device-side wait exceeded %u ms", c->cfg.wait_limit_ms);
    else if (k.error & ERR_QUEUE)
        status = fail(c, CG_ERR_QUEUE_OVERFLOW, "node-pair queue full (queue_capacity %u)", c->cfg.queue_capacity);
    else if (k.error & ERR_BAD_QUERY)
        status = fail(c, CG_ERR_INVALID_ARGUMENT, "a query names an unknown tree");
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
             (k.c_overflow || k.n_contacts > c->cfg.max_contacts || k.n_rays > c->ct.max_rays))
        status = fail(c, CG_ERR_OUTPUT_OVERFLOW, "%u contacts, %u rays (max_contacts %llu, flags %u): raise max_contacts",
                      k.n_contacts, k.n_rays, (unsigned long long)c->cfg.max_contacts, k.c_overflow);
    s.status = status;
    if (st) *st = s;
    return status;
}

int check_flags(cg_ctx* c, uint32_t flags) {
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

}  // namespace

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
        cudaMalloc(&c->d_trace, sizeof(unsigned int) * 4 * kTraceBuckets) != cudaSuccess) {
        delete c;
        return CG_ERR_CUDA;
    }
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

    std::vector<float4> recs(4ull * n_recs, make_float4(0, 0, 0, 0));
    put_box(&recs[4], v->root_obb, N ? uint32_t(rb + 2) : uint32_t(tb), N ? 0u : (kLeafFlag | T));
    for (uint32_t k = 0; k < N; ++k)
        for (int s = 0; s < 2; ++s) {
            const uint64_t r = 2ull * k + 2 + s;
            const uint32_t ref = v->node_ref[2 * k + s];
            const uint32_t cnt = v->node_tri_count[2 * k + s];
            const uint32_t abs_ref = cnt ? uint32_t(tb + ref) : uint32_t(rb + 2ull * ref + 2);
            put_box(&recs[4 * r], v->node_obbs[2 * k + s], abs_ref, cnt ? (kLeafFlag | cnt) : 0u);
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
    // subtree triangle range of every record (the root, then both children of
    // each node; children come after their parent, so a backward pass over
    // the nodes sees each inner child's range before its parent needs it)
    {
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

namespace {
inline uint32_t bits_of(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
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
        for (uint64_t k = 0; k < 3ull * m.n_triangles; ++k)
            if (m.indices[k] >= m.n_vertices)
                return fail(c, CG_ERR_BAD_TREE, "mesh %u index %llu is vertex %u of %u", i, (unsigned long long)k,
                            m.indices[k], m.n_vertices);
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
    const size_t oNodes = take(sizeof(BuildNode) * cap), oFlat = take(sizeof(BuildFlat) * cap), oCtr = take(8);
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
    bp.node_cap = cap;
    bp.T = uint32_t(total);
    float* d_V = reinterpret_cast<float*>(mem + oV);
    float* d_NV = any_normals ? reinterpret_cast<float*>(mem + oNV) : nullptr;
    uint32_t* d_idx = reinterpret_cast<uint32_t*>(mem + oIdx);
    BuildMesh* d_mesh = reinterpret_cast<BuildMesh*>(mem + oMesh);
    BuildEmit* d_emit = reinterpret_cast<BuildEmit*>(mem + oEmit);
    in.meshes = d_mesh;
    in.vertices = d_V;
    in.normals = d_NV;
    in.indices = d_idx;
    // the meshes' buffers, one after another
    std::vector<BuildMesh> mt(n);
    std::vector<BuildNode> roots(n);
    std::vector<uint32_t> own(T, 0u);
    for (uint32_t i = 0; i < n; ++i) {
        const cg_mesh_view& m = meshes[i];
        mt[i] = BuildMesh{uint32_t(vbase[i]), (m.normals && m.n_triangles) ? 1u : 0u};
        roots[i] = BuildNode{};
        roots[i].begin = uint32_t(base[i]);
        roots[i].count = m.n_triangles;
        roots[i].kid = kNoKid;
        roots[i].tree = i;
        std::fill(own.begin() + long(base[i]), own.begin() + long(base[i + 1]), i);
        if (!m.n_triangles) continue;
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
    const uint32_t ctr0[2] = {n, 0u};
    CG_CUDA(cudaMemcpyAsync(d_mesh, mt.data(), sizeof(BuildMesh) * n, cudaMemcpyHostToDevice, s), "upload meshes");
    CG_CUDA(cudaMemcpyAsync(bp.own, own.data(), sizeof(uint32_t) * T, cudaMemcpyHostToDevice, s), "upload owners");
    CG_CUDA(cudaMemcpyAsync(bp.nodes, roots.data(), sizeof(BuildNode) * n, cudaMemcpyHostToDevice, s), "upload roots");
    CG_CUDA(cudaMemcpyAsync(bp.node_ctr, ctr0, sizeof(ctr0), cudaMemcpyHostToDevice, s), "upload counter");
    const uint32_t sms = uint32_t(c->sm_count);
    CG_CUDA(launch_build_gather(bp, in, sms, s), "gather kernel");
    // one level per round of launches; the splits' children are the next level
    std::vector<std::pair<uint32_t, uint32_t>> levels;
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        bp.lo = lo;
        bp.hi = hi;
        levels.emplace_back(lo, hi);
        CG_CUDA(launch_build_level(bp, sms, s), "build level kernels");
        uint32_t ctr[2];
        CG_CUDA(cudaMemcpyAsync(ctr, bp.node_ctr, sizeof(ctr), cudaMemcpyDeviceToHost, s), "read node count");
        CG_CUDA(cudaStreamSynchronize(s), "build level");
        if (ctr[1]) return fail(c, CG_ERR_OUT_OF_MEMORY, "tree build ran out of node slots");
        lo = hi;
        hi = std::min(ctr[0], cap);
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
    for (uint32_t i = 0; i < n && e == cudaSuccess; ++i) e = launch_surfaces(c->recs.ptr, em[i].rec_base, em[i].n_recs, s);
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
    // The whole step (query upload from the pinned staging buffer, kernels,
    // counter read-back) is one CUDA graph, captured once per (n, flags) and
    // tree-storage generation and replayed.
    auto& G = c->host_graph;
    if (!G.exec || G.n != n || G.flags != flags || G.gen != arena_gen(c) ||
        G.out_gen != c->host_out.gen) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        G.exec = nullptr;
        CG_CUDA(cudaStreamSynchronize(c->stream), "sync before capture");
        CG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        c->capturing = true;
        cudaError_t e = cudaSuccess;
        if (n)
            e = cudaMemcpyAsync(c->d_queries, c->h_queries, sizeof(cg_query) * n, cudaMemcpyHostToDevice, c->stream);
        // results to the host buffers: the pairs on a branch beside the
        // contact kernels, the rays and averages after them
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
        int rc = e == cudaSuccess ? enqueue_step(c, c->d_queries, n, flags, c->stream, pc.host_pairs ? &pc : nullptr)
                                  : CG_ERR_CUDA;
        if (rc == CG_OK && (rc2.host_rays || rc2.host_averages)) e = launch_copy_out(rc2, c->copy_blocks, c->stream);
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
    if (m) CG_CUDA(cudaMemcpy(out, c->d_leafs, sizeof(cg_leaf_pair) * m, cudaMemcpyDeviceToHost), "read leaf pairs");
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
    const uint64_t total = c->h_ctr->n_contacts;
    const uint64_t avail = std::min<uint64_t>(total, c->cfg.max_contacts);
    *n = total;
    const uint64_t m = std::min(avail, cap);
    if (m) CG_CUDA(cudaMemcpy(out, c->ct.contacts, sizeof(cg_contact) * m, cudaMemcpyDeviceToHost), "read contacts");
    return (total > avail || (c->h_ctr->c_overflow & CONTACT_TABLE)) ? CG_ERR_OUTPUT_OVERFLOW : CG_OK;
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
                 b_pairs = up(sizeof(uint2) * max_pairs), b_cnt = 256, b_c3 = up(3 * sizeof(uint32_t) * 2 * max_pairs),
                 b_grp = up(sizeof(float) * 6 * max_rays), b_tag = up(sizeof(uint32_t) * max_rays),
                 b_sq = up(sizeof(ShootQuery) * max_pairs), b_so = up(sizeof(ShootRayOut) * max_rays),
                 b_dl = up(sizeof(float) * 3 * max_pairs), b_res = up(sizeof(cg_frame_result) * max_pairs);
    const size_t need = b_ent + b_id + b_g + b_cb + b_proj + b_pairs + b_cnt + b_c3 + b_grp + b_tag + b_sq + b_so +
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
    uint32_t* d_c3 = reinterpret_cast<uint32_t*>(take(b_c3));
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
    fp.counts = d_c3;
    fp.offsets = d_c3 + 2 * max_pairs;
    fp.cursor = d_c3 + 4 * max_pairs;
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
    CG_CUDA(cudaMemsetAsync(fp.counts, 0, sizeof(uint32_t) * 2 * np, s), "clear ray counts");
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

constexpr uint32_t kStaticSlots = 16384;     // work-queue chunk slots (ready flags + pool)
constexpr uint32_t kStaticMinChunks = 1024;  // donated chunks a launch may always reserve
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
    else if (k->n_leafs > CG_STATIC_MAX_LEAF_PAIRS || k->n_pairs > pairs_cap)
        r.status = CG_ERR_OUTPUT_OVERFLOW;
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
    // would leave fewer than kStaticMinChunks slots for donations.
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
