/*
 * collide_gpu.h — C ABI of the GB300 (sm_103a) collision-detection library.
 *
 * Drop-in boundary for the CPU collision path of the inMyRoom_vulkan engine.
 * The reference runs, per pair of CollisionDetectionEntry, a mid phase
 *   OBBtreesCollision::ExecuteOBBtreesCollision
 *     (inMyRoom_vulkan/include/CollisionDetection/OBBtreesCollision.h:14-20,
 *      src/CollisionDetection/OBBtreesCollision.cpp:7-18)
 * and a narrow phase
 *   CreateUncollideRays::ExecuteCreateUncollideRays
 *     (include/CollisionDetection/CreateUncollideRays.h:16-23,
 *      src/CollisionDetection/CreateUncollideRays.cpp:60-201)
 * on OBB trees built by OBBtree::OBBtree (src/Geometry/OBBtree.cpp:321-358).
 * This ABI replaces those calls for a whole batch of pairs at once: trees are
 * uploaded once (cg_tree_upload), a batch of queries is resolved in one
 * persistent launch (cg_collide / cg_collide_async / cg_graph_launch), and the
 * candidate leaf pairs, colliding triangle pairs, per-triangle contacts and
 * uncollide rays are read back.
 *
 * Conventions: every function returns CG_OK (0) or a negative CG_ERR_* code;
 * matrices are 4x4 column-major float[16] (glm::mat4 memory layout); triangle
 * indices are positions in the tree's leaf (DFS) order, exactly the indices
 * OBBtree::GetTrianglePosition takes. One context is used by one host thread
 * at a time. There is no CPU fallback: without a usable CUDA device every call
 * that needs one fails with CG_ERR_CUDA.
 */
#ifndef COLLIDE_GPU_H
#define COLLIDE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum cg_status {
    CG_OK = 0,
    CG_ERR_INVALID_ARGUMENT = -1,
    CG_ERR_CUDA = -2,
    CG_ERR_OUT_OF_MEMORY = -3,
    CG_ERR_QUEUE_OVERFLOW = -4,  /* the node-pair work queue filled up: raise cg_config.queue_capacity */
    CG_ERR_OUTPUT_OVERFLOW = -5, /* more results than capacity; counts are exact, raise the capacity */
    CG_ERR_TIMEOUT = -6,         /* a bounded device-side wait ran out (cg_config.wait_limit_ms) */
    CG_ERR_BAD_TREE = -7,        /* tree view fails validation (index out of range, non-forward child) */
    CG_ERR_NOT_FOUND = -8,       /* unknown tree id */
};

typedef struct cg_ctx cg_ctx;

/* Launch and capacity settings. cg_config_default fills every field. */
typedef struct cg_config {
    int32_t device;            /* CUDA device ordinal */
    uint32_t max_queries;      /* queries per launch */
    uint64_t max_tri_pairs;    /* colliding triangle pairs kept per launch */
    uint64_t max_leaf_pairs;   /* candidate leaf pairs per launch (the list between traversal and narrow phase) */
    uint32_t queue_capacity;   /* node pairs the global work queue can hold (in chunks of 32) */
    uint32_t warps_per_block;  /* persistent traversal kernel shape; 0 = tuned default */
    uint32_t blocks_per_sm;    /* 0 = as many as fit */
    uint32_t stack_entries;    /* per-warp shared-memory node-pair stack, power of two (256..4096) */
    uint32_t donate_min;       /* a warp donates work to idle warps only above this stack size */
    uint32_t leaf_flush;       /* leaf pairs a traversal warp buffers before appending them to the list (1..33) */
    uint32_t wait_limit_ms;    /* limit of every device-side wait */
    uint32_t pad;
    uint64_t max_contacts;     /* triangles with contacts per launch (CG_CONTACTS); rays <= 3x this */
} cg_config;

void cg_config_default(cg_config* cfg);

int cg_create(const cg_config* cfg, cg_ctx** out);
int cg_destroy(cg_ctx* ctx);
int cg_reconfigure(cg_ctx* ctx, const cg_config* cfg); /* resizes buffers / launch shape */
int cg_get_config(const cg_ctx* ctx, cg_config* out);
const char* cg_status_string(int status);
/* Copies the last error message of the context (NUL-terminated). */
int cg_last_error(const cg_ctx* ctx, char* buf, size_t len);

/* ---- trees ------------------------------------------------------------ */

/* Paralgram / OBB: center and three half-extent vectors
 * (include/Geometry/Paralgram.h:28-35), 48 bytes. */
typedef struct cg_obb {
    float center[3];
    float u[3];
    float v[3];
    float w[3];
} cg_obb;

/* A flat OBB tree in the reference's layout (include/Geometry/OBBtree.h:61-75,
 * 129-134): inner node k holds both child boxes and, per child, either an inner
 * node index (count 0) or a triangle offset and count; node 0 is the root's
 * node; the root box is separate; triangles are in leaf (DFS) order. A tree
 * whose root is a leaf has node_count 0. Export it from an OBBtree through the
 * public OBBtree::OBBtreeTraveler walk (inner nodes in pre-order). */
typedef struct cg_tree_view {
    cg_obb root_obb;
    uint32_t node_count;
    const cg_obb* node_obbs;          /* [node_count][2] left, right */
    const uint32_t* node_ref;         /* [node_count][2] child node index or triangle offset */
    const uint32_t* node_tri_count;   /* [node_count][2] triangle count, 0 = inner child */
    uint32_t triangle_count;
    const float* triangles_position;  /* [triangle_count][3][3] */
    const float* triangles_normal;    /* [triangle_count][3][3], may be NULL (rays then use the face normal) */
    const uint32_t* triangles_indices;/* [triangle_count][3] vertex indices, may be NULL */
} cg_tree_view;

/* Replaces building/holding OBBtree objects for the GPU: copies the tree to
 * device memory and returns its id. */
int cg_tree_upload(cg_ctx* ctx, const cg_tree_view* view, uint32_t* tree_id);
int cg_tree_free(cg_ctx* ctx, uint32_t tree_id);

/* An indexed triangle mesh: the vertex and index buffers the engine reads
 * its collision triangles from (one Triangle per index triple, with the
 * vertices' positions, normals and indices). */
typedef struct cg_mesh_view {
    const float* positions;   /* [n_vertices][3] */
    const float* normals;     /* [n_vertices][3], or NULL (rays then use the face normal) */
    const uint32_t* indices;  /* [n_triangles][3], each < n_vertices */
    uint32_t n_vertices;
    uint32_t n_triangles;
} cg_mesh_view;

/* OBBtree::OBBtree(std::vector<Triangle>&&) (src/Geometry/OBBtree.cpp:321-358)
 * for n meshes on the device: the PCA-fitted boxes (FP64 covariance and eig3,
 * OBB.cpp:33-166), the centre splits of at most 4 triangles per leaf
 * (OBBtree.cpp:43-108) and the pre-order layout, bit-identical to the
 * reference builder's tree; then each tree is uploaded as by cg_tree_upload.
 * tree_ids[n] out. CG_ERR_BAD_TREE for an index outside its mesh's vertices
 * (the first by mesh, then index position; checked on the device). Where the
 * device reads pageable host memory (Grace), it reads the meshes' arrays
 * itself (a mesh whose arrays are not 4-byte aligned is copied); else they
 * are copied. Either way each array must hold what its counts say
 * (n_vertices x 3 floats, n_triangles x 3 indices).
 * The environment variable CG_PAGEABLE_ACCESS=0, read when a context is
 * created, makes the context copy them. Synchronous. */
int cg_tree_build(cg_ctx* ctx, const cg_mesh_view* meshes, uint32_t n, uint32_t* tree_ids);

/* A tree's sizes, and its whole flat layout back in the form of
 * cg_tree_view (the tree cache's content): root box, node_obbs[node_count][2],
 * node_ref and node_tri_count [node_count][2], triangles_position and
 * triangles_normal [triangle_count][3][3], triangles_indices [triangle_count][3]
 * (a tree uploaded without indices gives 3t + k). Any pointer may be NULL;
 * the arrays must hold the sizes cg_tree_info gives. Normals exist when
 * has_normals is 1. Waits for the context's stream. */
int cg_tree_info(cg_ctx* ctx, uint32_t tree_id, uint32_t* node_count, uint32_t* triangle_count,
                 uint32_t* has_normals);
int cg_tree_export(cg_ctx* ctx, uint32_t tree_id, cg_obb* root, cg_obb* node_obbs, uint32_t* node_ref,
                   uint32_t* node_tri_count, float* triangles_position, float* triangles_normal,
                   uint32_t* triangles_indices);

/* The tree cache: a tree's flat layout in a file, loaded again without a
 * build. Little-endian: "CGTREE01", uint32 node_count, triangle_count, flags
 * (1: normals), then the root box, node_obbs, node_ref, node_tri_count,
 * triangles_position, triangles_normal (if flagged), triangles_indices, and a
 * 64-bit FNV-1a of everything before it. cg_tree_load checks the sizes and
 * the checksum (CG_ERR_BAD_TREE) and uploads as cg_tree_upload. */
int cg_tree_save(cg_ctx* ctx, uint32_t tree_id, const char* path);
int cg_tree_load(cg_ctx* ctx, const char* path, uint32_t* tree_id);

/* ---- queries ---------------------------------------------------------- */

/* One entity pair, the unit of OBBtreesCollision::ExecuteOBBtreesCollision.
 * relative = inverse(first.currentGlobalMatrix) * second.currentGlobalMatrix
 * (OBBtreesCollision.cpp:15), computed on the host by the caller's math
 * library so that it is bit-identical to the reference. 72 bytes. */
typedef struct cg_query {
    uint32_t tree_a;
    uint32_t tree_b;
    float relative[16];
} cg_query;

/* inverse(a) * b with the operation order of the glm-compatible convention
 * this library is validated against (for callers without glm). */
int cg_relative_matrix(const float a[16], const float b[16], float out[16]);

/* One candidate leaf pair: OBBtreesIntersectInfo::CandidateTriangleRangeCombination
 * (include/Geometry/OBBtree.h:8-19) tagged with its query. 16 bytes. */
typedef struct cg_leaf_pair {
    uint32_t query;
    uint32_t offset_a;
    uint32_t offset_b;
    uint16_t count_a;
    uint16_t count_b;
} cg_leaf_pair;

/* One colliding triangle pair (TrianglesIntersectionInfo with doIntersept &&
 * !areCoplanar, include/Geometry/Triangle.h:12-18): tree-order triangle indices
 * and the intersection segment in the first tree's model space. 36 bytes. */
typedef struct cg_tri_pair {
    uint32_t query;
    uint32_t tri_a;
    uint32_t tri_b;
    float source[3];
    float target[3];
} cg_tri_pair;

typedef struct cg_stats {
    uint64_t node_pairs;  /* box pairs tested (SAT) */
    uint64_t leaf_pairs;  /* candidate leaf pairs */
    uint64_t tri_tests;   /* triangle-pair tests (Moller calls) */
    uint64_t tri_pairs;   /* colliding triangle pairs (may exceed max_tri_pairs) */
    uint64_t fragile;     /* pairs whose second interval degenerated (see docs) */
    uint64_t donations;   /* node pairs handed from busy to waiting warps */
    uint64_t warp_steps;  /* traversal steps; node_pairs / warp_steps = busy lanes per step */
    uint64_t contacts;    /* triangles with contacts (CG_CONTACTS) */
    uint64_t rays;        /* uncollide rays (CG_CONTACTS) */
    int32_t status;       /* CG_OK or the error the launch raised */
    int32_t pad;
    uint64_t rechecked;      /* plane distances recomputed in FP64 (CG_RECHECK / CG_ROBUST) */
    uint64_t disagreements;  /* triangle-pair tests where a recomputed distance changed class */
} cg_stats;

#define CG_KEEP_LEAF_PAIRS 1u /* also write the candidate leaf pairs */
#define CG_NO_TRI_PAIRS 2u    /* count triangle tests and hits but do not write pairs */
#define CG_TRACE 4u           /* record a utilisation timeline (see cg_read_trace) */
#define CG_MID_ONLY 8u        /* mid phase only: candidate leaf pairs, no triangle tests */
#define CG_CONTACTS 16u       /* also per-triangle contacts, uncollide rays and their averages */
/* FP64 recheck of the triangle tests' orientation determinants. The Moller
 * test (Triangle.cpp:866-1003) classifies the six plane distances
 * d = n . p + d0 of each pair (FP32, as the reference computes them) as zero
 * (|d| < 1e-6), positive or negative. A distance whose FP32 magnitude lies
 * within the filter bound B = 32 u C |e1|_1 |e2|_1 of 0 or of 1e-6 (u = 2^-24;
 * e1, e2 the plane's triangle edges; C the largest coordinate magnitude of
 * its first corner and the three tested corners; twice the forward error of
 * the FP32 value against the exact determinant) is recomputed in FP64 as
 * det[e1, e2, p - a0] and classified again.
 * CG_RECHECK: the verdicts stay the reference's; cg_stats.rechecked counts
 * the recomputed distances and cg_stats.disagreements the tests in which one
 * changed class. CG_ROBUST: the same, and the test goes on with the FP64
 * classes (and the FP64 values, rounded to FP32, of the nonzero ones): a
 * robust verdict that can differ from the reference's on those tests. */
#define CG_RECHECK 32u
#define CG_ROBUST 64u
/* With CG_KEEP_LEAF_PAIRS: cg_read_leaf_pairs returns the candidate leaf pairs
 * grouped by query and, within a query, in the order the reference's
 * recursion emits them (OBBtree::IntersectOBBtreesRecursive,
 * src/Geometry/OBBtree.cpp:414-476: the order of their paths from the root
 * pair, left before right), the exact vector ExecuteOBBtreesCollision
 * returns. Each leaf pair's path is found on the device; a path of 128 or
 * more splits makes the launch CG_ERR_OUTPUT_OVERFLOW. */
#define CG_DFS_ORDER 128u

/* Per-triangle contact record, the TriangleCandidateRays of
 * CreateUncollideRays.cpp:14-58 after the merge: bit k of mask set = vertex k
 * of the triangle is not outside the other triangles' planes; weighted_avg =
 * length-weighted mean of the intersection-segment midpoints (the first
 * tree's model space); weight = total segment length. side 0 = first tree,
 * 1 = second tree; tri is the tree-order index. 32 bytes. */
typedef struct cg_contact {
    uint32_t query;
    uint32_t side;
    uint32_t tri;
    uint32_t mask;
    float weighted_avg[3];
    float weight;
} cg_contact;

/* One uncollide ray (CreateUncollideRays.cpp:131-178) in the first tree's
 * model space: from a "not outside" vertex (once per vertex index) along the
 * negated vertex normal, or from the weighted contact average along the
 * negated interpolated normal. side as in cg_contact. 32 bytes. */
typedef struct cg_ray {
    uint32_t query;
    uint32_t side;
    float origin[3];
    float direction[3];
} cg_ray;

/* Per query: average_point_first_modelspace and
 * average_point_second_modelspace of CDentriesUncollideRays
 * (CreateUncollideRays.cpp:183-198) and the ray counts. 32 bytes. */
typedef struct cg_ray_average {
    float first[3];
    float second[3];
    uint32_t rays_first;
    uint32_t rays_second;
} cg_ray_average;

/* Host queries in, stats out; synchronous. Results stay on the device until read. */
int cg_collide(cg_ctx* ctx, const cg_query* queries, uint32_t n, uint32_t flags, cg_stats* stats);
/* Queries already in device memory; enqueued on `stream` (cudaStream_t, NULL =
 * the context's stream); no host synchronisation. */
int cg_collide_async(cg_ctx* ctx, const cg_query* d_queries, uint32_t n, uint32_t flags, void* stream);
/* Waits for the last launch and reads its statistics. */
int cg_sync_stats(cg_ctx* ctx, cg_stats* stats);
int cg_read_tri_pairs(cg_ctx* ctx, cg_tri_pair* out, uint64_t cap, uint64_t* n);
/* Candidate leaf pairs of the last launch made with CG_KEEP_LEAF_PAIRS: in no
 * fixed order, or in the reference's order with CG_DFS_ORDER. */
int cg_read_leaf_pairs(cg_ctx* ctx, cg_leaf_pair* out, uint64_t cap, uint64_t* n);
/* Device pointers to the last launch's results (valid until the next launch). */
int cg_device_results(cg_ctx* ctx, const cg_tri_pair** pairs, const unsigned long long** pair_count);

/* Results of a launch made with CG_CONTACTS. Contacts and rays come grouped by
 * query, then side (first tree, second tree); within a group in the order the
 * reference makes them: the iteration order of its per-triangle
 * std::unordered_map<uint32_t, ...> (CreateUncollideRays.cpp:70-71, 138) as
 * GCC's libstdc++ lays it out, reproduced from the library's own growth
 * sizes read on the host. So rays_from_first_to_second of query q is the run
 * of rays with (query q, side 0), bit for bit and in order. Read the averages
 * with cap >= the launch's query count. */
int cg_read_contacts(cg_ctx* ctx, cg_contact* out, uint64_t cap, uint64_t* n);
int cg_read_rays(cg_ctx* ctx, cg_ray* out, uint64_t cap, uint64_t* n);
int cg_read_ray_averages(cg_ctx* ctx, cg_ray_average* out, uint64_t cap, uint64_t* n);

/* Host destinations of cg_collide's results, so that one cg_collide call
 * returns them (no read calls, one synchronisation): with these set, every
 * cg_collide step also writes its colliding pairs (the first pairs_cap), and
 * for CG_CONTACTS steps its uncollide rays (the first rays_cap) and per-query
 * ray averages (the first averages_cap), straight into these buffers, as part
 * of the step's own launch sequence. The counts are the step's cg_stats
 * (tri_pairs, rays; averages: one per query). The buffers must be host memory
 * the device can write: page-locked (cudaHostAlloc, cudaHostRegister), or any
 * host memory where the device accesses pageable memory (Grace); 16-byte
 * aligned; valid until replaced. The pairs are copied while the contact
 * kernels run; the rays and averages are written by the contact kernels that
 * make them. A NULL pointer
 * or zero capacity leaves that result on the device only. Results are still
 * readable with the cg_read_* calls. Does not apply to cg_collide_async and
 * cg_graph_launch. */
int cg_set_host_outputs(cg_ctx* ctx, cg_tri_pair* pairs, uint64_t pairs_cap, cg_ray* rays, uint64_t rays_cap,
                        cg_ray_average* averages, uint64_t averages_cap);

/* Device times of the last step's two main kernels, the OBB-tree traversal
 * (emits candidate leaf pairs) and the narrow phase (triangle-pair tests),
 * from CUDA events recorded around their launches; each waits for its kernel. */
int cg_traversal_time_ms(cg_ctx* ctx, float* ms);
int cg_narrow_time_ms(cg_ctx* ctx, float* ms);

/* Utilisation timeline of the last launch made with CG_TRACE: per time bucket
 * of bucket_ns nanoseconds since the traversal started, four counters (busy
 * lanes summed over traversal steps, traversal steps, triangle tests, triangle
 * passes). bucket_ns (if non-zero) sets the width for later launches; out
 * receives n_buckets x 4 values (at most 512 buckets). */
int cg_read_trace(cg_ctx* ctx, uint32_t bucket_ns, uint32_t* out, uint32_t n_buckets);

/* CUDA graph of one whole collide step over device-resident queries
 * (counter reset, query packing, persistent traversal + narrow phase). */
int cg_graph_capture(cg_ctx* ctx, const cg_query* d_queries, uint32_t n, uint32_t flags);
int cg_graph_launch(cg_ctx* ctx, void* stream);

/* ---- deforming meshes ------------------------------------------------- */

/* Morph targets, then linear-blend skinning, of a vertex array: the position
 * path of the engine's skinning compute shader
 * (shaders/dynamicMeshShader_glsl.comp:78-145, which replaces vertex data the
 * engine's CPU collision path then uses). All arrays are device memory:
 *   vertices       n_vertices x (1 + n_targets) x float4: per vertex the base
 *                  position (w = 1) then the morph target offsets (w = 0), the
 *                  shader's interleaved layout; 16-byte aligned
 *   morph_weights  n_targets floats
 *   joints         n_vertices x n_groups x 4 uint16 (8-byte aligned); a joint
 *                  index >= n_joints makes that vertex NaN
 *   weights        n_vertices x n_groups x float4 (16-byte aligned)
 *   joint_matrices n_joints x 16 floats, column-major: the shader's
 *                  modelMatrices[matrixOffset + 1 + j]
 *   inverse_bind   n_joints x 16 floats: inverseModelMatrices[inverseMatricesOffset + j]
 * out receives n_vertices x float4 (16-byte aligned). n_groups = 0 skips the
 * skin. n_joints <= 2048. Enqueued on `stream` (NULL = the context's). */
typedef struct cg_deform_view {
    uint32_t n_vertices;
    uint32_t n_targets;
    uint32_t n_groups;
    uint32_t n_joints;
    const float* vertices;
    const float* morph_weights;
    const uint16_t* joints;
    const float* weights;
    const float* joint_matrices;
    const float* inverse_bind;
} cg_deform_view;

int cg_deform(cg_ctx* ctx, const cg_deform_view* view, float* out, void* stream);
/* n meshes in one launch: views[i] into outs[i]. The table of views goes to
 * device memory when it differs from the previous call's (that upload waits
 * for the stream, so make the first call of a new table outside stream
 * capture); repeating the same batch costs one kernel launch. */
int cg_deform_batch(cg_ctx* ctx, const cg_deform_view* views, float* const* outs, uint32_t n, void* stream);

/* Refits an uploaded tree to new vertex positions (device, n_positions x
 * float4, 16-byte aligned, indexed by the triangles' vertex indices given at
 * upload, e.g. cg_deform's output): the topology stays; every box is fitted
 * again with OBB::CreateOBBfromPoints (src/Geometry/OBB.cpp:33-89) to the
 * corners of its subtree's triangles, taken in the tree's leaf (DFS) order.
 * A vertex index >= n_positions makes its corner NaN. Enqueued on `stream`
 * (NULL = the context's); a collide launched after it on the same stream sees
 * the new boxes. */
int cg_tree_refit(cg_ctx* ctx, uint32_t tree_id, const float* positions, uint32_t n_positions, void* stream);
/* n trees in one launch of each refit kernel (the table is handled as in
 * cg_deform_batch). */
int cg_tree_refit_batch(cg_ctx* ctx, const uint32_t* tree_ids, const float* const* positions,
                        const uint32_t* n_positions, uint32_t n, void* stream);

/* Copies an uploaded (or refitted) tree's boxes and triangle positions back:
 * root box, node_obbs[node_count][2] (left, right) and
 * triangles_position[triangle_count][3][3], in the layout of cg_tree_view; any
 * pointer may be NULL. node_count and triangle_count must be the tree's (or
 * 0 for an array not wanted). Waits for the context's stream. */
int cg_tree_download(cg_ctx* ctx, uint32_t tree_id, cg_obb* root, cg_obb* node_obbs, uint32_t node_count,
                     float* triangles_position, uint32_t triangle_count);

/* ---- Differentiable penetration energy (no reference counterpart: the
 * engine does not differentiate its collision response) ----
 *
 * Skeleton posing from per-bone axis-angle rotations: bone j's world matrix is
 * G_j = G_parent(j) * T(offset_j) * R(a_j) (G of a root = T(offset_j) * R(a_j)),
 * R(a) the rotation by |a| about a / |a|. The matrices feed
 * cg_deform_view.joint_matrices, as the skin's joint nodes' world matrices
 * do in the engine (shaders/dynamicMeshShader_glsl.comp:41-44, 78-83). */
typedef struct cg_skeleton_view {
    uint32_t n_bones;       /* 1 .. CG_MAX_JOINTS */
    const int32_t* parent;  /* host [n_bones]: parent(j) < j, or -1 */
    const float* offsets;   /* host [n_bones][3]: translation from the parent */
} cg_skeleton_view;
#define CG_MAX_JOINTS 2048u

/* d_axis_angles [n_poses][n_bones][3] -> d_joint_matrices
 * [n_poses][n_bones][16] (column-major), device memory, on `stream`. */
int cg_pose(cg_ctx* ctx, const cg_skeleton_view* skeleton, const float* d_axis_angles, uint32_t n_poses,
            float* d_joint_matrices, void* stream);
/* Adjoint of cg_pose: d_grad_joint_matrices (dE/dG, same layout as the
 * matrices) -> d_grad_axis_angles (dE/da, overwritten). d_joint_matrices is
 * cg_pose's output for the same angles. */
int cg_pose_backward(cg_ctx* ctx, const cg_skeleton_view* skeleton, const float* d_axis_angles,
                     const float* d_joint_matrices, const float* d_grad_joint_matrices, uint32_t n_poses,
                     float* d_grad_axis_angles, void* stream);

/* Penetration energy of the colliding triangle pairs of the context's last
 * collide step (cg_collide, cg_collide_async or cg_graph_launch, with the
 * pairs stored: no CG_NO_TRI_PAIRS / CG_MID_ONLY), into *d_energy (device):
 *   E = sum over pairs, both directions of the vertex-vs-plane test of
 *       src/CollisionDetection/CreateUncollideRays.cpp:102-112, of min(0, s)^2,
 *       s = n . (p - p0): the depth of the vertex p below the other triangle's
 *       plane (unit face normal n through its first vertex p0, Plane.cpp:14-20),
 * in the first tree's space. FP32 terms, FP64 sum. Pairs beyond max_tri_pairs
 * (reported by the collide's stats) are not in the sum. Enqueue it on the
 * collide's stream. */
int cg_energy(cg_ctx* ctx, double* d_energy, void* stream);

/* One side (first or second tree) of every query of that collide step, for
 * the adjoint. views[q] describes how tree q's vertices were made (the
 * cg_deform view its refit positions came from, read again now: deformed
 * vertices are recomputed, not kept); a view with n_vertices = 0, or
 * views = NULL, marks a static side. Gradients are written (overwritten) to
 *   grad_joint_matrices [n_queries][joint_stride][16] dE/d joint_matrices
 *                       (column-major; row 3 is zero),
 *   grad_morph_weights  [n_queries][target_stride]   dE/d morph_weights,
 * device memory. n_targets <= 256 per view. */
typedef struct cg_energy_side {
    const cg_deform_view* views;
    uint32_t joint_stride;
    uint32_t target_stride;
    float* grad_joint_matrices;
    float* grad_morph_weights;
} cg_energy_side;

/* Adjoint of cg_energy for the same collide step: *d_grad_energy (device,
 * dL/dE) -> dL/d joint_matrices and dL/d morph_weights of both sides (either
 * may be NULL: static). Joint matrices and morph weights must still hold the
 * forward's values. */
int cg_energy_backward(cg_ctx* ctx, const double* d_grad_energy, const cg_energy_side* side_a,
                       const cg_energy_side* side_b, void* stream);

/* ---- Broad phase ----
 *
 * SweepAndPrune::ExecuteSweepAndPrune (src/CollisionDetection/SweepAndPrune.cpp:
 * 15-88) for n entities: the pairs whose world root boxes
 * (global * root OBB) project onto each of the three axes as overlapping
 * closed intervals, where at least one entity calls back, as (the entity
 * whose projection starts earlier on U, the other; equal starts: the lower
 * index first). axes: U, V, W (9 floats) or NULL for the engine's
 * (CollisionDetection.cpp:9-13). Host arrays; callback may be NULL (all call
 * back); synchronous. Pairs beyond cap are counted in *n_pairs, not written
 * (then CG_ERR_OUTPUT_OVERFLOW). */
typedef struct cg_entity_pair {
    uint32_t first, second;
} cg_entity_pair;

int cg_broad_phase(cg_ctx* ctx, const uint32_t* tree_ids, const float* globals, const uint8_t* callback, uint32_t n,
                   const float* axes, cg_entity_pair* pairs, uint64_t cap, uint64_t* n_pairs);

/* ---- Uncollide-ray shooting ----
 *
 * ShootUncollideRays::ExecuteShootUncollideRays
 * (src/CollisionDetection/ShootUncollideRays.cpp:14-98) for a batch of entity
 * pairs: each ray's Hermann pass (closest hit on the other entity's tree with
 * Ray::IntersectOBBtree, Ray.cpp:135-237; a back face; nothing nearer on its
 * own tree) and its reflection's, the force responses summed in the
 * reference's order, FindResponse, and the first entity's world-space delta.
 * Bit for bit the reference's result for the same rays in the same order; the
 * ray/triangle test is Moller-Trumbore, two-sided, back face = negative
 * determinant (the reference's glm fork is not public). */
typedef struct cg_shoot_params {
    float smoothstep_start;   /* radians; the engine: 40 degrees (CollisionDetection.cpp:22-24) */
    float smoothstep_finish;  /* radians; the engine: 65 degrees */
    float distance_bias;      /* the engine: 1.01 */
} cg_shoot_params;
void cg_shoot_params_default(cg_shoot_params* params);

/* One entity pair. Its rays are consecutive in the ray array: n_first from
 * the first entity (CDentriesUncollideRays::rays_from_first_to_second), then
 * n_second from the second (rays_from_second_to_first), all in the first
 * entity's model space, as CreateUncollideRays makes them (cg_read_rays gives
 * them per query and side). 144 bytes. */
typedef struct cg_shoot_query {
    uint32_t tree_a, tree_b;
    float first_global[16];   /* firstEntry.currentGlobalMatrix */
    float second_global[16];  /* secondEntry.currentGlobalMatrix */
    uint32_t n_first, n_second;
} cg_shoot_query;

/* n pairs, rays (host, [n_rays][6]: origin, direction; n_rays the sum of the
 * queries' counts) -> deltas (host, [n][3]). params NULL: the engine's.
 * Synchronous. CG_ERR_QUEUE_OVERFLOW if a tree is deeper than the traversal's
 * stack (96 levels). */
int cg_shoot_rays(cg_ctx* ctx, const cg_shoot_query* queries, uint32_t n, const float* rays, uint64_t n_rays,
                  const cg_shoot_params* params, float* deltas);

/* ---- A collision frame ----
 *
 * CollisionDetection::ExecuteCollisionDetection
 * (src/CollisionDetection/CollisionDetection.cpp:38-129) for n entities on the
 * device: broad phase (cg_broad_phase), the collide step of every broad pair
 * with contacts and uncollide rays, shooting (cg_shoot_rays, for pairs where an
 * entity moved, :80-82) and the delta split by each entity's movement of its
 * mean ray origin (:84-103). One result per pair with rays (:62-66), the
 * pair as the broad phase orients it; the fan-out of each result to the
 * entities' ancestors (:106-124) needs the engine's entity tree and is the
 * caller's. The pairs are the reference's. The deltas follow the
 * reference's arithmetic on the step's rays, which match the reference's up to
 * the last bits of the rays that start at a contact's weighted average point
 * (summed in another order); a few deltas per frame can differ from the
 * reference's by up to a percent where such a ray grazes a triangle's edge or
 * sets the shooting's maximum. After the call, cg_read_rays and
 * cg_read_ray_averages give the frame's collide step, whose query index is a
 * result's `query`. The broad pairs must fit in max_queries. Synchronous. */
typedef struct cg_frame_entity {
    uint32_t tree;
    uint32_t should_callback;
    float current_global[16];
    float previous_global[16];
} cg_frame_entity;

typedef struct cg_frame_result {
    uint32_t first, second;   /* entity indices */
    float first_delta[3];     /* CollisionCallbackData::deltaVector of the first entity */
    float second_delta[3];    /* and of the second */
    uint32_t query;           /* the pair's query index in the frame's collide step */
    uint32_t reserved;
} cg_frame_result;

int cg_collision_frame(cg_ctx* ctx, const cg_frame_entity* entities, uint32_t n, const cg_shoot_params* params,
                       cg_frame_result* results, uint64_t cap, uint64_t* n_results);

/* The fan-out of a frame's results to the entities' ancestors
 * (CollisionDetection.cpp:104-124, host only, no device): result k gives
 * CollisionCallbackData{first, second, first_delta} to every ancestor of
 * `first` (the root, entity 0, down to `first` itself,
 * EntitiesHandler::GetEntityAncestors) that is not the second's ancestor at
 * the same depth, and {second, first, second_delta} likewise. entity_ids maps
 * the frame's entity indices to the engine's entities; parent[e] is entity
 * e's parent (parent of the root unused). The callbacks come grouped by
 * receiver, each receiver's in result order (the reference's map of vectors,
 * flattened). CG_ERR_OUTPUT_OVERFLOW with the exact count when cap is short;
 * CG_ERR_INVALID_ARGUMENT for an id out of range or a parent cycle. */
typedef struct cg_frame_callback {
    uint32_t receiver;       /* the entity whose components get the callback */
    uint32_t family_entity;  /* CollisionCallbackData::familyEntity */
    uint32_t collide_with;   /* CollisionCallbackData::collideWithEntity */
    float delta[3];          /* CollisionCallbackData::deltaVector */
} cg_frame_callback;

int cg_frame_callbacks(const cg_frame_result* results, uint64_t n_results, const uint32_t* entity_ids,
                       uint32_t n_entities, const uint32_t* parent, uint32_t n_ids, cg_frame_callback* out,
                       uint64_t cap, uint64_t* n_out);

/* ---- No-allocation collide step (no reference counterpart) ----
 *
 * The collide step of cg_collide_async (same kernels, same colliding pairs)
 * for callers that must not allocate device memory on the call's path: a
 * frame loop that is being captured into a CUDA graph in global capture mode
 * (where cudaMalloc is refused and cudaFree would synchronise the device), or
 * an engine whose device memory comes from its own fixed budget. The call
 * makes no cudaMalloc, cudaFree or other allocating call: its per-launch
 * scratch (counters, work queue, candidate leaf pairs, packed queries) is one
 * static device array of CG_STATIC_SCRATCH_BYTES inside the library, and the
 * results go to caller-owned device memory. Trees come from `ctx`
 * (cg_tree_upload, done beforehand).
 *
 * The first call on a device sets the scratch up (looks up its address and
 * clears the counters and work-queue flags, then waits for that clear): make
 * it before any stream capture. The scratch is one per device and process,
 * so calls whose work overlaps on the device (any context, any stream) race:
 * order them on one stream or wait for one before launching the next.
 *
 * The set-up is per process and device: a cudaDeviceReset, which ends every
 * context of this library anyway, also ends it, and the entry point is not
 * usable in that process afterwards.
 *
 * Limits: n <= CG_STATIC_MAX_QUERIES (else CG_ERR_INVALID_ARGUMENT, nothing
 * launched); at most CG_STATIC_MAX_LEAF_PAIRS candidate leaf pairs per call
 * (else counts->status = CG_ERR_OUTPUT_OVERFLOW); a work queue of at least
 * 32,768 donated chunks of node pairs, as many as cg_collide's default
 * queue_capacity (the traversal grid is narrowed when the context's would
 * leave fewer), else counts->status = CG_ERR_QUEUE_OVERFLOW. Enqueued on
 * `stream` (NULL = the context's stream), no host synchronisation: *d_counts
 * (device memory) is valid once the stream reaches that point. Pairs beyond
 * pairs_cap are counted, not written, and make the status
 * CG_ERR_OUTPUT_OVERFLOW; a count-only call (d_pairs NULL, pairs_cap 0)
 * reports the count with CG_OK. */
#define CG_STATIC_MAX_QUERIES 1024u
#define CG_STATIC_MAX_LEAF_PAIRS 131072u
#define CG_STATIC_SCRATCH_BYTES 36012288u /* about 34.3 MiB */

typedef struct cg_static_counts {
    uint64_t tri_pairs;  /* colliding triangle pairs found */
    uint64_t tri_tests;  /* triangle-pair tests */
    uint64_t leaf_pairs; /* candidate leaf pairs */
    int32_t status;      /* CG_OK or the CG_ERR_* of the launch */
    int32_t pad;
} cg_static_counts;

int cg_collide_static(cg_ctx* ctx, const cg_query* d_queries, uint32_t n, cg_tri_pair* d_pairs, uint64_t pairs_cap,
                      cg_static_counts* d_counts, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* COLLIDE_GPU_H */
