// Shared between the host side of the C ABI and the collision kernels.
//
// Device layout (HBM). All trees of a context live in two arenas, addressed by
// absolute indices so that a traversal step needs no per-tree pointer:
//   records  : float4[4 * n], one 64-byte record per box. A tree occupies a
//              block of 2*node_count + 2 records starting at rec_base: record
//              rec_base + 1 is the root, and the two child boxes of inner node
//              k are records rec_base + 2k + 2 (left) and + 2k + 3 (right), so
//              one node's children share a 128-byte line.
//              q0 = (c.x, c.y, c.z, u.x)  q1 = (u.y, u.z, v.x, v.y)
//              q2 = (v.z, w.x, w.y, w.z)  q3 = (ref, meta, surface, split)
//              ref  = absolute record index of the left child (inner box), or
//                     absolute index of the leaf's first triangle
//              meta = triangle count | 0x80000000 for a leaf
//              surface = Paralgram::GetSurface of the box, precomputed
//              split = absolute index of the right child's first triangle
//                      (inner box; 0 for a leaf): a triangle t of the subtree
//                      lies under the right child when t >= split
//   triangles: float4[3 * n], 48 bytes per triangle in leaf (DFS) order,
//              (p_k.xyz, vertex index k as bits) for k = 0, 1, 2; a tree's
//              triangles start at tri_base.
//   normals  : float[9 * n_tris] per tree (uncollide rays), optional.
//
// A collide step runs two persistent kernels: the traversal writes candidate
// leaf pairs to a list, and the narrow phase runs the triangle pairs of that
// list, 32 leaf pairs per warp.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "collide_gpu.h"

namespace cg {

constexpr uint32_t kLeafFlag = 0x80000000u;
constexpr int kLeafCap = 96;        // buffered leaf pairs per traversal warp (a step adds up to 64)
constexpr int kChunk = 32;          // node pairs per donated task slot
constexpr int kTraceBuckets = 512;  // utilisation trace: counters per time bucket

struct DevTree {
    uint32_t rec_base;  // first record of the tree (its root is rec_base + 1)
    uint32_t tri_base;  // first triangle of the tree
    uint32_t n_recs;
    uint32_t n_tris;
    uint32_t live;
    uint32_t pad;
    const float* nrm;
};

// A query as the kernels read it: relative matrix columns, the first
// traversal item (made by the pack kernel from the root pair) and the
// triangle bases (to report tree-local triangle indices).
//
// Traversal item (query word, split record, other record): the node being
// split has its two child boxes at records split and split + 1; `other` is
// the box of the other tree they are tested against. kItemSideB in the query
// word marks children of the second tree. A query word of kNoItem means the
// query has no item (invalid query, roots disjoint, or roots both leaves).
constexpr uint32_t kItemSideB = 0x80000000u;
constexpr uint32_t kNoItem = 0xffffffffu;

struct alignas(16) PackedQuery {
    float4 m[4];
    uint32_t item_q, item_split, item_other, pad;
    uint32_t tri_base_a, tri_base_b, tree_a, tree_b;
};

struct Counters {
    unsigned int head;        // next task slot to claim (slots < n_queries are the root tasks)
    unsigned int tail;        // one past the last reserved task slot
    unsigned int done;        // finished tasks; all work is done when done == tail
    unsigned int error;       // ERR_* bits
    unsigned int n_queries;   // queries of the launch (the next launch clears the slots it published)
    unsigned int narrow_lp;   // next leaf pair for the narrow phase
    unsigned long long n_pairs;
    unsigned long long n_leafs;
    unsigned long long node_pairs;
    unsigned long long tri_tests;
    unsigned long long fragile;
    unsigned long long rechecked;      // plane distances recomputed in FP64 (CG_RECHECK, CG_ROBUST)
    unsigned long long disagreements;  // triangle-pair tests where one changed class
    unsigned long long donations;  // node pairs handed to other warps
    unsigned long long warp_steps; // traversal steps (node_pairs / warp_steps = lanes busy per step)
    unsigned long long t_start;    // globaltimer at the first warp's start (trace only)
    // contacts (CG_CONTACTS)
    unsigned int n_vertices;     // vertex-set slots taken by this launch (emptied by the next contacts launch)
    unsigned int n_rays;         // uncollide rays
    unsigned int n_contacts;     // contact slots taken: (side, query, triangle) with a colliding pair
    unsigned int c_overflow;     // CONTACT_* bits
    unsigned int n_elems;        // triangles with contacts (non-zero weight): the contact records
    unsigned int prev_vertices;  // vertex-set slots earlier launches took and no launch emptied yet
    unsigned int n_kleaf;        // leaf pairs with colliding pairs (listed for their descent paths)
    unsigned int contrib_used;   // contribution-list entries given to slots
    unsigned int order_ticket;   // maps taken by the order kernel's blocks
    unsigned int n_big;          // contact slots of more than kFoldThread contributions (listed for the fold)
    unsigned int fold_done;      // fold blocks finished (the last one ranks the maps)
    unsigned int order_done;     // order blocks finished (the last one places the maps' records and rays)
};

enum : unsigned int { CONTACT_TABLE = 1u, CONTACT_VERTICES = 2u, CONTACT_RAYS = 4u, CONTACT_ORDER = 8u };

enum : unsigned int { ERR_TIMEOUT = 1u, ERR_QUEUE = 2u, ERR_BAD_QUERY = 4u, ERR_DEEP = 8u };

// Contacts and rays (cg_contacts.cu). A slot of the contact table names one
// triangle of one side of one query that has colliding pairs; its pairs'
// contributions are listed together and folded in the reference's order.
constexpr unsigned long long kEmptyKey = ~0ull;

struct ContactSlot {
    unsigned long long key;  // side << 63 | query << 32 | tree-local triangle, or kEmptyKey
    uint32_t count;          // colliding pairs of the triangle
    uint32_t offset;         // first entry of its contributions in the contribution list
};

// A triangle with contacts (the merged TriangleCandidateRays of a non-zero
// weight), the element of its (query, side) map. key: the path of the
// simultaneous descent to the first leaf pair that gave it weight, one bit per
// split (left 0, right 1), left-aligned in 128 bits; in the engine's
// unordered_map it was inserted in that leaf pair's turn.
struct alignas(16) ContactElem {
    unsigned long long key_hi, key_lo;
    float sx, sy, sz, w;  // weighted midpoint sum and weight: the reference's float folds
    uint32_t tri, mask, depth, pad;
};

// std::unordered_map<uint32_t, T> grows at fixed sizes: the elements with
// insertion index in [start[e], start[e + 1]) are inserted with bucket count
// buckets[e] (the whole table is rehashed into it when start[e] is inserted).
constexpr uint32_t kMaxSchedule = 40;

// Order kernel working memory: a map whose working set and vertex set fit
// kOrderSmemWords words (every map of up to 1,024 triangles) is ordered in
// shared memory, larger ones in global memory (kOrderWords words per
// element).
constexpr uint32_t kOrderSmemWords = 24576;
constexpr uint32_t kOrderWords = 24;
constexpr uint32_t kFoldThread = 8;  // contributions a slot's own thread folds (more: its warp)

struct ContactParams {
    const PackedQuery* q;
    uint32_t n_queries;
    uint32_t n_sched;           // entries of the growth schedule
    const float4* tris;
    const float4* recs;
    const DevTree* trees;
    const cg_tri_pair* pairs;
    const uint4* pair_aux;      // per pair: (first triangle, second triangle, leaf-list index, query), arena indices
    const uint4* leaf_list;     // the launch's candidate leaf pairs
    unsigned long long pairs_cap;
    ContactSlot* table;
    uint32_t table_mask;
    uint32_t max_contacts;      // contact slots (and records) a launch can hold
    uint32_t* occupied;         // slots taken this launch, in the order they were taken
    uint4* slot_info;           // per entry of occupied: its key (low, high word), first contribution, count
    uint32_t* big_slots;        // entries of occupied with more than kFoldThread contributions
    float4* pg_geom;            // per pair: weight * midpoint, weight
    uint4* pg_link;             // per pair: both triangles' slots and places in their slots' lists
    uint32_t* pg_mask;          // per pair: "not outside" bits of the first triangle | the second's << 3
    unsigned long long* contrib;// contributions by slot: (other triangle << 32) | (pair << 1) | side
    uint32_t* leaf_mark;        // per leaf pair of the list: 0, or 1 + its place in kleaf once listed
    uint32_t* kleaf;            // leaf pairs with colliding pairs, listed once each
    ulonglong2* kpath;          // their descent paths (high, low)
    uint32_t kleaf_cap;
    uint32_t* map_order;        // the maps, largest first
    uint32_t* map_cnt;          // per map (2 query + side): slots; then per map element offsets
    uint32_t* map_off;
    uint32_t* map_fill;         // elements (triangles with contacts)
    uint32_t* map_nr;           // rays
    uint32_t* map_coff;         // first contact record and first ray of each map in the outputs
    uint32_t* map_roff;
    ContactElem* elems;         // per map from map_off
    uint32_t* work;             // order kernel: global working memory of large maps
    unsigned long long* vkeys;  // set of (side, query, vertex index) with their first corner in map order
    uint32_t* vval;
    uint32_t vtable_mask;
    uint32_t* vocc;             // vertex-set slots taken, in order
    cg_contact* ctmp;           // per map from map_off: the map's records in iteration order
    cg_ray* rtmp;               // per map from 3 map_off: its rays in order
    cg_contact* contacts;
    cg_ray* rays;
    uint32_t max_rays;
    cg_ray_average* averages;
    cg_ray* host_rays;                  // device alias of the caller's host buffers, or null: the
    unsigned long long host_rays_cap;   // rays and averages written there too, as the kernels
    cg_ray_average* host_averages;      // write them
    unsigned long long host_averages_cap;
    Counters* ctr;
    uint32_t sched_start[kMaxSchedule];
    uint32_t sched_buckets[kMaxSchedule];
};

cudaError_t launch_contacts(const ContactParams& p, uint32_t grid, uint32_t fold_grid, uint32_t order_grid,
                            cudaStream_t s, cudaStream_t branch, cudaEvent_t ev_fork, cudaEvent_t ev_join);
cudaError_t contacts_order_occupancy(int* blocks_per_sm);
cudaError_t contacts_fold_occupancy(int* blocks_per_sm);

// Descent paths of the stored candidate leaf pairs (CG_DFS_ORDER).
struct LeafKeyParams {
    const PackedQuery* q;
    const DevTree* trees;
    const float4* recs;
    const uint4* leaf_list;
    const unsigned long long* n_leafs;  // the launch's count (device)
    uint32_t leaf_cap;
    unsigned* error;                    // ERR_DEEP when a path is too deep for 128 bits
    ulonglong2* keys;                   // per leaf pair: path high, low
};
cudaError_t launch_leaf_keys(const LeafKeyParams& p, uint32_t grid, cudaStream_t s);

// Results of a step written to host buffers (cg_set_host_outputs).
struct CopyOutParams {
    const Counters* ctr;
    const cg_tri_pair* pairs;
    unsigned long long pairs_avail;  // records the device buffer holds
    cg_tri_pair* host_pairs;         // device alias of the host buffer, or null
    unsigned long long host_pairs_cap;
    const cg_ray* rays;
    unsigned long long rays_avail;
    cg_ray* host_rays;
    unsigned long long host_rays_cap;
    const cg_ray_average* averages;
    cg_ray_average* host_averages;
    unsigned long long host_averages_cap;
};
cudaError_t launch_copy_out(const CopyOutParams& p, uint32_t blocks, cudaStream_t s);
cudaError_t init_contact_tables(ContactSlot* table, uint32_t n_slots, unsigned long long* vkeys, uint32_t* vval,
                                uint32_t n_vslots, cudaStream_t s);

struct NarrowParams {
    const PackedQuery* q;
    const float4* tris;   // triangle arena
    const uint4* leaf_list;
    uint32_t leaf_cap;
    Counters* ctr;
    cg_tri_pair* pairs;
    uint4* pair_aux;      // per written pair (contacts): arena triangles, leaf-list index, query; or null
    unsigned long long pairs_cap;
    cg_leaf_pair* leafs;  // the public copy of the leaf pairs (CG_KEEP_LEAF_PAIRS)
    unsigned long long leafs_cap;
    uint32_t flags;
    unsigned int* trace;
    uint32_t trace_ns;
};

// Work queue. A task is a chunk of up to kChunk node pairs: donated slot
// s >= n_queries holds its chunk at pool[kChunk * (s - n_queries)], and
// ready[s - n_queries] becomes count + 1 when it is published. Slot
// s < n_queries is the root pair of query s.
struct TraverseParams {
    const PackedQuery* q;
    uint32_t n_queries;
    const float4* recs;   // record arena
    uint4* pool;          // node-pair entries (query, record a, record b, 0)
    unsigned int* ready;  // per donated slot
    uint32_t slot_cap;    // donated slots donors may reserve
    uint32_t slot_alloc;  // allocated slots (slot_cap plus room for warps waiting past it)
    Counters* ctr;
    uint4* leaf_list;     // (query, first triangle a, first triangle b, count_a | count_b << 16)
    uint32_t leaf_cap;
    unsigned int* trace;  // kTraceBuckets x 4 or null
    uint32_t trace_ns;    // trace bucket width
    uint32_t stack_cap;   // power of two
    uint32_t donate_min;
    uint32_t leaf_flush;  // leaf pairs buffered before they are appended to the list
    unsigned long long wait_ns;
};


__host__ __device__ inline uint32_t warp_smem_words(uint32_t stack_cap) { return 3u * stack_cap + 4u * kLeafCap; }
constexpr uint32_t kNarrowWarpWords = 6u * 32u + 1u;  // a narrow block: 32 leaf pairs + prefix sums

// Morph and skinning (cg_deform.cu); the arrays are those of cg_deform_view.
struct DeformParams {
    uint32_t n_vertices, n_targets, n_groups, n_joints;
    const float* vertices;
    const float* morph_weights;
    const uint16_t* joints;
    const float* weights;
    const float* joint_matrices;
    const float* inverse_bind;
    float* out;
};
constexpr uint32_t kMaxJoints = 2048;  // joint products staged in shared memory (128 KB)
// One launch for a batch of meshes (grid.y = mesh); the parameters are in
// device memory.
cudaError_t launch_deform(const DeformParams* d_meshes, uint32_t n_meshes, uint32_t max_vertices, uint32_t max_joints,
                          cudaStream_t s);
cudaError_t deform_smem_limit();

// Refit (cg_refit.cu): new corner positions of a tree's triangles from a
// vertex array, then every record's box from its triangle range (x first, y
// count; y = ~0 marks the unused record). One launch per kernel for a batch
// of trees (grid.y = tree); the table is in device memory, the scratch holds
// one entry per record of the batch (tree i's from scratch_base).
struct RefitTree {
    uint32_t rec_base, n_recs, tri_base, n_tris;
    const uint2* ranges;
    const float4* positions;
    uint32_t n_positions, scratch_base;
    const uint32_t* parent;       // per record: the record of its parent box, or ~0 (root, unused)
    const uint32_t* leaves;       // the leaf records, in tree order
    uint32_t n_leaves, pad;
};
enum : uint32_t { kRefitSkip = 0, kRefitEmpty = 1, kRefitPoint = 2, kRefitBox = 3 };
constexpr int kExtLo = 0x7f800000;           // order key of +inf
constexpr int kExtHi = int(0x807fffffu);     // order key of -inf
struct alignas(16) RefitMom {  // count, mean, centred second moments, first point, largest |x| + |y| + |z|
    uint32_t n, kind;
    float mean[3];
    float m2[6];  // xx, yy, zz, xy, xz, yz
    float p0[3];
    float mabs;
    float pad;
};
static_assert(sizeof(RefitMom) == 64, "RefitMom is read as four 16-byte words");
// Refit scratch, one entry per record of a batch (tree i's from scratch_base),
// in separate arrays so that each kernel reads only what it needs.
struct RefitBufs {
    RefitMom* mom;
    float4* axes;       // [3] per record: axis rows (xyz); w of the first is 1 for a box
    int4* ext;          // [2] per record: order keys of the min and max projections (xyz); kExtLo / kExtHi between refits
    uint32_t* arrive;   // children that finished their moments; 0 between refits
};
// bytes of the scratch for cap records: each array starts on a 256-byte boundary
inline size_t refit_bytes(uint32_t cap) {
    auto up = [](size_t x) { return (x + 255u) & ~size_t(255); };
    return up(sizeof(RefitMom) * size_t(cap)) + up(3 * sizeof(float4) * size_t(cap)) +
           up(2 * sizeof(int4) * size_t(cap)) + up(sizeof(uint32_t) * size_t(cap));
}
inline RefitBufs refit_bufs(void* base, uint32_t cap) {
    auto up = [](size_t x) { return (x + 255u) & ~size_t(255); };
    char* p = static_cast<char*>(base);
    RefitBufs b;
    b.mom = reinterpret_cast<RefitMom*>(p);
    p += up(sizeof(RefitMom) * size_t(cap));
    b.axes = reinterpret_cast<float4*>(p);
    p += up(3 * sizeof(float4) * size_t(cap));
    b.ext = reinterpret_cast<int4*>(p);
    p += up(2 * sizeof(int4) * size_t(cap));
    b.arrive = reinterpret_cast<uint32_t*>(p);
    return b;
}
cudaError_t init_refit_scratch(const RefitBufs& b, uint32_t n, cudaStream_t s);
cudaError_t launch_refit(float4* recs, float4* tris, const RefitTree* d_trees, uint32_t n_trees, uint32_t max_tris,
                         uint32_t max_recs, uint32_t max_leaves, const RefitBufs& scratch, cudaStream_t s);

// Axis-angle posing of a skeleton and its adjoint (cg_energy.cu): bone j's
// world matrix is G_parent(j) * T(offset_j) * R(axis_angle_j).
struct PoseParams {
    uint32_t n_poses, n_bones;
    uint32_t per_block, staged;     // set by the launchers
    const int32_t* parent;          // [n_bones], < j or -1
    const float* offsets;           // [n_bones][3]
    const float* axis_angles;       // [n_poses][n_bones][3]
    float* joint_matrices;          // forward out / backward in: [n_poses][n_bones][16]
    const float* grad_joint;        // backward in: [n_poses][n_bones][16]
    float* grad_acc;                // backward scratch: [n_poses][n_bones][37] (used when not staged)
    float* grad_axis_angles;        // backward out: [n_poses][n_bones][3]
};
cudaError_t launch_pose(const PoseParams& p, cudaStream_t s);
cudaError_t launch_pose_backward(const PoseParams& p, cudaStream_t s);

// Penetration energy over the colliding pairs of the last collide and its
// adjoint (cg_energy.cu). One side of a query deforms when its view has
// vertices; then its vertices are recomputed from the view (cg_skin.cuh) and
// its gradient lands in grad_joint / grad_morph.
struct EnergySide {
    DeformParams d;      // d.n_vertices == 0: the side is static
    uint32_t grad_base;  // first vertex of this side in the vertex-gradient buffer
    uint32_t pad;
    float* grad_joint;   // [joint_stride][16], rows 0-2 written
    float* grad_morph;   // [n_targets]
};
struct EnergyParams {
    const PackedQuery* q;
    uint32_t n_queries;
    uint32_t n_deforming;         // entries of `deforming`
    const float4* tris;           // triangle arena
    const cg_tri_pair* pairs;
    const Counters* ctr;          // n_pairs of the collide
    unsigned long long pairs_cap;
    double* energy;               // forward out
    const double* grad_energy;    // backward in (dL/dE)
    const EnergySide* sides;      // [2 * n_queries]: side A of every query, then side B
    const uint32_t* deforming;    // indices into sides of the deforming ones
    float* vgrad;                 // [sum of deforming sides' n_vertices][3], zero between calls
    uint32_t max_joints, max_targets;
    uint32_t skin_in_smem;        // set by the launcher
};
cudaError_t launch_energy(const EnergyParams& p, uint32_t blocks, cudaStream_t s);
cudaError_t launch_energy_backward(const EnergyParams& p, uint32_t blocks, uint32_t max_vertices, cudaStream_t s);
cudaError_t energy_occupancy(int* blocks_per_sm);

// Broad phase (cg_broad.cu).
struct BroadParams {
    const uint32_t* tree_ids;  // per entity
    const DevTree* trees;
    const float4* recs;
    const float* globals;      // [n][16] world matrices
    const uint8_t* callback;   // per entity, or null: all call back
    uint32_t n;
    float3 axes[3];            // U, V, W
    float* proj;               // [n][6] scratch: min/max on U, V, W
    uint2* pairs;
    unsigned long long cap;
    unsigned long long* count;
};
cudaError_t launch_broad(const BroadParams& p, cudaStream_t s);

// Uncollide-ray shooting (cg_shoot.cu).
struct ShootQuery {
    float relative[16];      // second entity's model space to the first's
    float first_global[16];  // the first entity's world matrix (the delta's frame)
    uint32_t tree_a, tree_b;
    uint32_t ray_first, n_first, n_second;  // rays [ray_first, + n_first) from the first, then n_second
    uint32_t pad[3];                        // pad[0]: shoot this pair's rays (0: skip them)
};
struct ShootRayOut {  // a ray's pass and its reflection's: signed force and ray responses
    float f1[3], r1[3], f2[3], r2[3];
    uint32_t ok1, ok2;
};
struct ShootParams {
    const ShootQuery* q;
    uint32_t n_queries, n_rays;
    const DevTree* trees;
    const float4* recs;
    const float4* tris;
    const float* rays;          // [n_rays][6] origin, direction (the first entity's space)
    const uint32_t* ray_query;  // per ray: query | (from the second entity) << 31
    ShootRayOut* out;
    float cos_start, cos_finish, bias;
    float* deltas;              // [n_queries][3]
    unsigned* error;            // ERR_QUEUE when a tree is deeper than the traversal stack
    const unsigned* n_rays_dev; // or null: the rays' count in device memory (at most n_rays)
};
cudaError_t launch_shoot(const ShootParams& p, cudaStream_t s);

// OBB-tree construction (cg_build.cu).
constexpr uint32_t kNoKid = 0xffffffffu;
struct BuildNode {           // 64 bytes
    uint32_t begin, count;   // the node's triangles: perm[begin, begin + count)
    uint32_t kid;            // its children at kid, kid + 1 (as split: left, right), or kNoKid
    uint32_t tree;
    float box[12];           // centre, u, v, w
};
static_assert(sizeof(BuildNode) == 64, "BuildNode layout");
struct BuildParams {
    const float* P;          // [triangles][3][3] corners, the meshes one after another
    float* Pp;               // [triangles][3][3] the same at each triangle's position in the permutation
    uint32_t* perm;          // [triangles] triangle ids, each node's range partitioned in place
    uint32_t* scratch;       // [triangles]
    uint32_t* own;           // [triangles] the node that holds each position (its level's or a leaf's)
    double* D;               // [3][3 triangles] the corners' coordinates at their position, by coordinate
    double* Tm;              // [6][3 triangles] the corners' centred products
    double* mom;             // [level width][9] mean, then the six covariance sums
    BuildNode* nodes;
    uint32_t T;              // triangles
    uint32_t lo, hi;         // this level's nodes
    uint32_t* node_ctr;      // [0] next free node, [1] error, [2 + parity] nodes in big_out
    uint32_t node_cap;
    unsigned* error;
    const uint32_t* big;     // this level's nodes of more than kBuildBig triangles (a block fits each)
    uint32_t n_big;
    uint32_t* big_out;       // the next level's, appended by the splits of this level's
    uint32_t* n_big_out;
};
constexpr uint32_t kBuildBig = 256;  // nodes of more than this many triangles are fitted by a block
cudaError_t launch_build_level(const BuildParams& p, uint32_t sm_count, cudaStream_t s);
struct BuildMesh {
    uint32_t vbase;          // first vertex in BuildInput::vertices / normals
    uint32_t has_normals;
    uint32_t tbase;          // first triangle position
    uint32_t n_vertices;
};
struct BuildInput {
    const BuildMesh* meshes;
    const float* vertices;   // [all meshes' vertices][3]
    const float* normals;    // [all meshes' vertices][3] (rows of meshes without normals unused)
    const uint32_t* indices; // [triangles][3] mesh-local vertex indices
    float* P;                // [triangles][3][3] out: corners
    float* corner_normals;   // [triangles][3][3] out: corner normals
    unsigned long long* bad; // out: the smallest (mesh << 32 | index position) whose vertex index is out of range
};
// One host array copied into the build's input buffers by the device itself
// (where it reads pageable host memory): n 4-byte words from src to dst.
struct PullSeg {
    const uint32_t* src;
    uint32_t* dst;
    uint64_t n;
};
cudaError_t launch_build_pull(const PullSeg* segs, uint32_t n_segs, uint64_t max_words, cudaStream_t s);
struct BuildFlat {           // a node's place in its tree's layout
    uint32_t inner;          // inner nodes of its subtree
    uint32_t index;          // pre-order index (inner nodes)
    uint32_t tri_off;        // first triangle of its subtree
    uint32_t leaf_off;       // leaves before it in pre-order
    uint32_t rec;            // its record (tree-local)
    uint32_t prec;           // its parent's record
    uint32_t split_off;      // first triangle of its second (right) child's subtree (inner nodes)
};
struct BuildEmit {           // a built tree's arena places
    uint32_t rec_base, tri_base, n_recs, pad;
    float* nrm;              // [triangles][9] or null
    uint2* ranges;           // [n_recs]
    uint32_t* topo;          // [n_recs] parents, then the leaf records
};
cudaError_t launch_build_gather(const BuildParams& p, const BuildInput& in, uint32_t n_meshes, uint32_t sm_count,
                                cudaStream_t s);
cudaError_t launch_build_inner(const BuildParams& p, BuildFlat* flat, uint32_t sm_count, cudaStream_t s);
cudaError_t launch_build_order(const BuildParams& p, BuildFlat* flat, uint32_t n_roots, uint32_t sm_count,
                               cudaStream_t s);
cudaError_t launch_build_emit(const BuildParams& p, const BuildInput& in, const BuildFlat* flat,
                              const BuildEmit* emit, float4* recs, float4* tris, uint32_t n_nodes, uint32_t n_roots,
                              uint32_t sm_count, cudaStream_t s);

// A collision frame (cg_frame.cu).
struct FrameParams {
    const cg_frame_entity* entities;
    const uint2* pairs;          // broad-phase pairs (first, second)
    uint32_t n_pairs;
    uint32_t max_rays;
    cg_query* queries;           // [n_pairs] collide queries
    const cg_ray* rays;          // the collide step's rays
    const unsigned* n_rays;      // their count (device)
    const uint32_t* counts;      // [2 n_pairs] rays per pair and side (the contact step's)
    const uint32_t* offsets;     // [2 n_pairs] first ray of each pair and side
    float* grouped;              // [max_rays][6] the rays as origin, direction
    uint32_t* tags;              // [max_rays] pair | (from the second entity) << 31
    ShootQuery* shoot;           // [n_pairs]; pad[0]: an entity moved
    const float* deltas;         // [n_pairs][3]
    const cg_ray_average* averages;
    cg_frame_result* results;
    unsigned long long results_cap;
    unsigned long long* n_results;
};
cudaError_t launch_frame_queries(const FrameParams& p, cudaStream_t s);
cudaError_t launch_frame_rays(const FrameParams& p, uint32_t blocks, cudaStream_t s);
cudaError_t launch_frame_split(const FrameParams& p, cudaStream_t s);

// Kernel launchers (cg_kernels.cu).
cudaError_t launch_pack(const cg_query* in, uint32_t n, const DevTree* trees, uint32_t n_trees, const float4* recs,
                        PackedQuery* out, Counters* ctr, uint4* leaf_list, uint32_t leaf_cap, cudaStream_t s);
cudaError_t launch_init(Counters* ctr, unsigned int* ready, uint32_t slot_alloc, uint32_t n_queries,
                        unsigned int* trace, cudaStream_t s);
cudaError_t launch_traverse(const TraverseParams& p, uint32_t blocks, uint32_t warps_per_block, cudaStream_t s);
cudaError_t launch_narrow(const NarrowParams& p, uint32_t blocks, uint32_t warps_per_block, cudaStream_t s);
cudaError_t traverse_occupancy(uint32_t warps_per_block, uint32_t stack_cap, int* blocks_per_sm);
cudaError_t narrow_occupancy(uint32_t warps_per_block, int* blocks_per_sm);
cudaError_t launch_surfaces(float4* recs, uint32_t first, uint32_t n_recs, cudaStream_t s);

}  // namespace cg
