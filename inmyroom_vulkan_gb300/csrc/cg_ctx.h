// The context behind the C ABI of include/collide_gpu.h and the host helpers
// that its implementation files (cg_api.cu: context, collide steps, reads,
// graphs, deformation, energy; cg_api_tree.cu: tree build, export and cache;
// cg_api_frame.cu: broad phase, shooting, the collision frame) share.
// Internal: included by those files only.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "cg_internal.h"
#include "collide_gpu.h"

using namespace cg;

namespace cg_host {

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

}  // namespace cg_host

struct cg_ctx {
    cg_config cfg{};
    int device = 0;
    int sm_count = 0;
    int pageable_access = 0;     // the device reads pageable host memory (cudaDevAttrPageableMemoryAccess)
    cudaStream_t stream = nullptr;
    uint32_t blocks = 0;         // persistent traversal grid
    uint32_t narrow_blocks = 0;  // persistent narrow-phase grid
    uint32_t contact_blocks = 0;                       // contact kernels: one resident wave
    uint32_t fold_blocks = 0;                          // the contact fold kernel: one resident wave
    uint32_t order_blocks = 0;                         // the persistent contact order kernel
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
    cg_host::Arena recs, tris;
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
    ulonglong2* d_leaf_keys = nullptr;  // CG_DFS_ORDER: each leaf pair's descent path (allocated on first use)
    unsigned int* d_trace = nullptr;
    uint32_t trace_ns = 0;

    // contacts and rays (CG_CONTACTS), allocated when max_contacts > 0
    struct Contacts {
        uint4* pair_aux = nullptr;
        ContactSlot* table = nullptr;
        uint32_t table_slots = 0;
        uint32_t* occupied = nullptr;
        uint4* slot_info = nullptr;
        uint32_t* big_slots = nullptr;
        float4* pg_geom = nullptr;
        uint4* pg_link = nullptr;
        uint32_t* pg_mask = nullptr;
        unsigned long long* contrib = nullptr;
        uint32_t* leaf_mark = nullptr;  // per leaf-list entry, zero between launches
        uint32_t* kleaf = nullptr;
        ulonglong2* kpath = nullptr;
        uint32_t kleaf_cap = 0;
        uint32_t* maps = nullptr;  // 7 arrays of 2 max_queries: count, offset, fill, rays, record and ray
                                   // offsets, the largest-first order
        ContactElem* elems = nullptr;
        uint32_t* work = nullptr;
        unsigned long long* vkeys = nullptr;
        uint32_t* vval = nullptr;
        uint32_t vslots = 0;
        uint32_t* vocc = nullptr;
        cg_contact* ctmp = nullptr;
        cg_ray* rtmp = nullptr;
        cg_contact* contacts = nullptr;
        cg_ray* rays = nullptr;
        uint32_t max_rays = 0;
        cg_ray_average* averages = nullptr;
    } ct;
    // growth sizes of the host's std::unordered_map<uint32_t, T> (the
    // reference's per-triangle maps), up to max_contacts elements
    uint32_t n_sched = 0;
    uint32_t sched_start[kMaxSchedule] = {};
    uint32_t sched_buckets[kMaxSchedule] = {};

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
    cudaStream_t branch = nullptr;  // a branch of the contact kernels (the descent paths)
    cudaEvent_t ev_branch = nullptr, ev_branched = nullptr;

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

namespace cg_host {

int fail(cg_ctx* c, int code, const char* fmt, ...);
int cuda_fail(cg_ctx* c, cudaError_t e, const char* what);
bool pow2(uint32_t x);
uint64_t arena_gen(const cg_ctx* c);
void free_buffers(cg_ctx* c);
int stage_table(cg_ctx* c, cg_ctx::Table& t, const void* data, size_t bytes, cudaStream_t s, const void** dev);
bool aligned_to(const void* p, uintptr_t a);
int deform_params(cg_ctx* c, const cg_deform_view* v, float* out, bool want_out, uint32_t i, DeformParams* p);
int pose_params(cg_ctx* c, const cg_skeleton_view* sk, uint32_t n_poses, cudaStream_t s, PoseParams* p);
int energy_ready(cg_ctx* c);
EnergyParams energy_params(cg_ctx* c);
void engine_axes(float* ax);
void drop_graph(cg_ctx* c);
int check_config(cg_ctx* c, const cg_config* cfg);
int alloc_buffers(cg_ctx* c);
bool growth_schedule(uint32_t max_elems, uint32_t* start, uint32_t* buckets, uint32_t* n);
int sync_tree_table(cg_ctx* c);
void put_box(float4* rec, const cg_obb& b, uint32_t ref, uint32_t meta, uint32_t split);
int enqueue_step(cg_ctx* c, const cg_query* d_queries, uint32_t n, uint32_t flags, cudaStream_t s,
                 const CopyOutParams* pairs_copy = nullptr, const CopyOutParams* results_copy = nullptr);
int stats_from(cg_ctx* c, const Counters& k, cg_stats* st);
int check_flags(cg_ctx* c, uint32_t flags);
int join_stream(cg_ctx* c, cudaStream_t s);
void mat_mul(const float* A, const float* B, float* R);
void mat_inverse(const float* M, float* R);

}  // namespace cg_host

// Returns the CUDA failure of `call` (with `what`) from the enclosing
// function, whose context is `c`.
#define CG_CUDA(call, what)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)
