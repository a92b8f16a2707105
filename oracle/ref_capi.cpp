// Oracle test infrastructure (reference build): a C ABI over the reference's own
// collision classes, compiled together with the reference sources
// (inMyRoom_vulkan/src/Geometry/*.cpp, src/CollisionDetection/*.cpp,
// eig3/eig3.cpp) against the glm shim. Tests use it to pin the C++ restatement
// in oracle/port and to make golden fixtures; it only exists where the
// reference sources are present.
#include <atomic>
#include <algorithm>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "CollisionDetection/CreateUncollideRays.h"
#include "CollisionDetection/OBBtreesCollision.h"
#include "CollisionDetection/ShootUncollideRays.h"
#include "CollisionDetection/SweepAndPrune.h"
#include "Geometry/OBBtree.h"
#include "Geometry/Paralgram.h"
#include "Geometry/Triangle.h"
#include "eig3.h"

namespace {

// Paralgram keeps its fields protected; a derived view reads and writes them.
struct BoxAccess : public OBB {
    static OBB Make(const float* b) {
        BoxAccess o;
        o.center = glm::vec3(b[0], b[1], b[2]);
        o.sideDirections.u = glm::vec3(b[3], b[4], b[5]);
        o.sideDirections.v = glm::vec3(b[6], b[7], b[8]);
        o.sideDirections.w = glm::vec3(b[9], b[10], b[11]);
        return o;
    }
};

void put_box(const Paralgram& p, float* out) {
    glm::vec3 c = p.GetCenter(), u = p.GetSideDirectionU(), v = p.GetSideDirectionV(), w = p.GetSideDirectionW();
    const float vals[12] = {c.x, c.y, c.z, u.x, u.y, u.z, v.x, v.y, v.z, w.x, w.y, w.z};
    std::memcpy(out, vals, sizeof(vals));
}

glm::mat4 load_mat(const float* m) {
    glm::mat4 r;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) r[c][k] = m[4 * c + k];
    return r;
}

void put_vec(const glm::vec3& v, float* out) {
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
}

struct MidResult {
    CDentriesPairTrianglesPairs pairs;
};

// Walks the tree in pre-order through the public traveler (OBBtree.h:78-101),
// giving inner nodes the indices the flattener assigned them
// (OBBtree.cpp:179-233, 385-394: inner nodes are appended in pre-order).
void export_walk(const OBBtree::OBBtreeTraveler& t, size_t& next_index, float* node_obbs, uint32_t* node_ref,
                 uint32_t* node_cnt) {
    size_t me = next_index++;
    OBBtree::OBBtreeTraveler kids[2] = {t.GetLeftChildTraveler(), t.GetRightChildTraveler()};
    for (int s = 0; s < 2; ++s) {
        put_box(kids[s].GetOBB(), node_obbs + (me * 2 + s) * 12);
        if (kids[s].IsLeaf()) {
            node_ref[me * 2 + s] = uint32_t(kids[s].GetTrianglesOffset());
            node_cnt[me * 2 + s] = uint32_t(kids[s].GetTrianglesCount());
        } else {
            node_ref[me * 2 + s] = uint32_t(next_index);
            node_cnt[me * 2 + s] = 0;
            export_walk(kids[s], next_index, node_obbs, node_ref, node_cnt);
        }
    }
}

size_t count_inner(const OBBtree::OBBtreeTraveler& t) {
    if (t.IsLeaf()) return 0;
    return 1 + count_inner(t.GetLeftChildTraveler()) + count_inner(t.GetRightChildTraveler());
}

}  // namespace

extern "C" {

// Builds a tree the way PrimitivesOfMeshes::GetOBBtreeAndReset does
// (inMyRoom_vulkan/src/Graphics/Meshes/PrimitivesOfMeshes.cpp:840-863) for one
// glTF "triangles" primitive.
void* ref_tree_build(const float* points, size_t n_points, const float* normals, const uint32_t* indices,
                     size_t n_indices) {
    std::vector<glm::vec3> pts(n_points), nrm;
    for (size_t i = 0; i < n_points; ++i) pts[i] = glm::vec3(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
    if (normals) {
        nrm.resize(n_points);
        for (size_t i = 0; i < n_points; ++i)
            nrm[i] = glm::vec3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
    }
    std::vector<uint32_t> idx(indices, indices + n_indices);
    std::vector<Triangle> tris = Triangle::CreateTriangleList(pts, nrm, idx, glTFmode::triangles);
    return new OBBtree(std::move(tris));
}

void ref_tree_free(void* t) { delete static_cast<OBBtree*>(t); }

void ref_tree_sizes(void* tp, size_t* n_nodes, size_t* n_tris) {
    const OBBtree* t = static_cast<const OBBtree*>(tp);
    *n_nodes = count_inner(t->GetRootTraveler());
    OBBtree::OBBtreeTraveler root = t->GetRootTraveler();
    size_t n = 0;
    if (root.IsLeaf()) {
        n = root.GetTrianglesCount();
    } else {
        // Triangles are stored contiguously in leaf order; the largest
        // offset+count over leaves is their number.
        std::vector<OBBtree::OBBtreeTraveler> stack;
        stack.push_back(root);
        while (!stack.empty()) {
            OBBtree::OBBtreeTraveler cur = stack.back();
            stack.pop_back();
            if (cur.IsLeaf()) {
                n = std::max(n, cur.GetTrianglesOffset() + cur.GetTrianglesCount());
            } else {
                stack.push_back(cur.GetLeftChildTraveler());
                stack.push_back(cur.GetRightChildTraveler());
            }
        }
    }
    *n_tris = n;
}

// node_obbs: [n_nodes][2][12]; node_ref/node_cnt: [n_nodes][2];
// tri_pos/tri_nrm: [n_tris][9]; tri_idx: [n_tris][3].
void ref_tree_export(void* tp, float* root12, float* node_obbs, uint32_t* node_ref, uint32_t* node_cnt,
                     float* tri_pos, float* tri_nrm, uint32_t* tri_idx) {
    const OBBtree* t = static_cast<const OBBtree*>(tp);
    put_box(t->GetRootOBB(), root12);
    OBBtree::OBBtreeTraveler root = t->GetRootTraveler();
    if (!root.IsLeaf()) {
        size_t next = 0;
        export_walk(root, next, node_obbs, node_ref, node_cnt);
    }
    size_t n_nodes, n_tris;
    ref_tree_sizes(tp, &n_nodes, &n_tris);
    for (size_t i = 0; i < n_tris; ++i) {
        TrianglePosition p = t->GetTrianglePosition(i);
        TriangleNormal nn = t->GetTriangleNormal(i);
        TriangleIndices ii = t->GetTriangleIndices(i);
        for (int k = 0; k < 3; ++k) {
            put_vec(p.GetP(k), tri_pos + 9 * i + 3 * k);
            put_vec(nn.GetN(k), tri_nrm + 9 * i + 3 * k);
            tri_idx[3 * i + k] = ii.GetI(k);
        }
    }
}

void ref_relative_matrix(const float* a16, const float* b16, float* out16) {
    glm::mat4 r = glm::inverse(load_mat(a16)) * load_mat(b16);
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) out16[4 * c + k] = r[c][k];
}

// Mid phase exactly as the engine calls it (CollisionDetection.cpp:49-56).
void* ref_mid_phase(void* ta, void* tb, const float* a16, const float* b16) {
    std::pair<CollisionDetectionEntry, CollisionDetectionEntry> p;
    p.first.currentGlobalMatrix = load_mat(a16);
    p.first.previousGlobalMatrix = load_mat(a16);
    p.first.OBBtree_ptr = static_cast<const OBBtree*>(ta);
    p.first.shouldCallback = true;
    p.first.entity = 0;
    p.second.currentGlobalMatrix = load_mat(b16);
    p.second.previousGlobalMatrix = load_mat(b16);
    p.second.OBBtree_ptr = static_cast<const OBBtree*>(tb);
    p.second.shouldCallback = true;
    p.second.entity = 1;
    auto* r = new MidResult;
    r->pairs = OBBtreesCollision().ExecuteOBBtreesCollision(p);
    return r;
}

void ref_mid_free(void* r) { delete static_cast<MidResult*>(r); }

size_t ref_mid_count(void* rp) {
    return static_cast<MidResult*>(rp)->pairs.OBBtreesIntersectInfoObj.candidateTriangleRangeCombinations.size();
}

// out: [n][4] = first offset, first count, second offset, second count.
void ref_mid_get(void* rp, uint32_t* out) {
    const auto& v = static_cast<MidResult*>(rp)->pairs.OBBtreesIntersectInfoObj.candidateTriangleRangeCombinations;
    for (size_t i = 0; i < v.size(); ++i) {
        out[4 * i + 0] = uint32_t(v[i].first_obbtree_offset);
        out[4 * i + 1] = uint32_t(v[i].first_obbtree_count);
        out[4 * i + 2] = uint32_t(v[i].second_obbtree_offset);
        out[4 * i + 3] = uint32_t(v[i].second_obbtree_count);
    }
}

// The narrow-phase pair loop of CreateUncollideRays.cpp:74-115, calling the
// reference's own transform and Moller test per pair, collecting the pairs
// that count as colliding (doIntersept && !areCoplanar) with their segment.
// Returns the number of colliding pairs (writes at most cap); *tests receives
// the number of triangle-pair tests.
size_t ref_narrow(void* rp, uint32_t* pair_out, float* seg_out, size_t cap, uint64_t* tests) {
    const CDentriesPairTrianglesPairs& e = static_cast<MidResult*>(rp)->pairs;
    const glm::mat4 m = glm::inverse(e.firstEntry.currentGlobalMatrix) * e.secondEntry.currentGlobalMatrix;
    const OBBtree* A = e.firstEntry.OBBtree_ptr;
    const OBBtree* B = e.secondEntry.OBBtree_ptr;
    size_t n = 0;
    uint64_t t = 0;
    for (const auto& lp : e.OBBtreesIntersectInfoObj.candidateTriangleRangeCombinations) {
        for (size_t i = 0; i != lp.first_obbtree_count; ++i) {
            for (size_t j = 0; j != lp.second_obbtree_count; ++j) {
                TrianglePosition ta = A->GetTrianglePosition(i + lp.first_obbtree_offset);
                TrianglePosition tb = m * B->GetTrianglePosition(j + lp.second_obbtree_offset);
                TrianglesIntersectionInfo info = Triangle::IntersectTriangles(ta, tb);
                ++t;
                if (info.doIntersept && !info.areCoplanar) {
                    if (n < cap) {
                        pair_out[2 * n] = uint32_t(i + lp.first_obbtree_offset);
                        pair_out[2 * n + 1] = uint32_t(j + lp.second_obbtree_offset);
                        put_vec(info.source, seg_out + 6 * n);
                        put_vec(info.target, seg_out + 6 * n + 3);
                    }
                    ++n;
                }
            }
        }
    }
    if (tests) *tests = t;
    return n;
}

// CreateUncollideRays::ExecuteCreateUncollideRays (CreateUncollideRays.cpp:60-201).
// rays: [n][6] = origin, direction. counts[0..1] = rays first->second,
// second->first; both arrays must hold the returned sizes (call with cap 0
// first to size them). avg: [6] = average points first and second.
void ref_rays(void* rp, float* rays_a, float* rays_b, size_t cap_a, size_t cap_b, size_t* counts, float* avg) {
    const CDentriesPairTrianglesPairs& e = static_cast<MidResult*>(rp)->pairs;
    CDentriesUncollideRays r = CreateUncollideRays().ExecuteCreateUncollideRays(e);
    counts[0] = r.rays_from_first_to_second.size();
    counts[1] = r.rays_from_second_to_first.size();
    for (size_t i = 0; i < counts[0] && i < cap_a; ++i) {
        put_vec(r.rays_from_first_to_second[i].GetOrigin(), rays_a + 6 * i);
        put_vec(r.rays_from_first_to_second[i].GetDirection(), rays_a + 6 * i + 3);
    }
    for (size_t i = 0; i < counts[1] && i < cap_b; ++i) {
        put_vec(r.rays_from_second_to_first[i].GetOrigin(), rays_b + 6 * i);
        put_vec(r.rays_from_second_to_first[i].GetDirection(), rays_b + 6 * i + 3);
    }
    if (avg) {
        put_vec(r.average_point_first_modelspace, avg);
        put_vec(r.average_point_second_modelspace, avg + 3);
    }
}

int ref_tri_tri(const float* a9, const float* b9, int* coplanar, float* src3, float* tgt3) {
    TrianglePosition a(glm::vec3(a9[0], a9[1], a9[2]), glm::vec3(a9[3], a9[4], a9[5]), glm::vec3(a9[6], a9[7], a9[8]));
    TrianglePosition b(glm::vec3(b9[0], b9[1], b9[2]), glm::vec3(b9[3], b9[4], b9[5]), glm::vec3(b9[6], b9[7], b9[8]));
    TrianglesIntersectionInfo info = Triangle::IntersectTriangles(a, b);
    *coplanar = info.areCoplanar ? 1 : 0;
    if (info.doIntersept && !info.areCoplanar) {
        put_vec(info.source, src3);
        put_vec(info.target, tgt3);
    }
    return info.doIntersept ? 1 : 0;
}

void ref_transform_tri(const float* m16, const float* a9, float* out9) {
    TrianglePosition a(glm::vec3(a9[0], a9[1], a9[2]), glm::vec3(a9[3], a9[4], a9[5]), glm::vec3(a9[6], a9[7], a9[8]));
    TrianglePosition r = load_mat(m16) * a;
    for (int k = 0; k < 3; ++k) put_vec(r.GetP(k), out9 + 3 * k);
}

int ref_sat(const float* a12, const float* b12) {
    return Paralgram::IntersectParalgramsBoolean(BoxAccess::Make(a12), BoxAccess::Make(b12)) ? 1 : 0;
}

float ref_surface(const float* a12) { return BoxAccess::Make(a12).GetSurface(); }

void ref_transform_box(const float* m16, const float* a12, float* out12) {
    put_box(load_mat(m16) * static_cast<const Paralgram&>(BoxAccess::Make(a12)), out12);
}

void ref_obb_from_points(const float* pts, size_t n, float* out12) {
    std::vector<glm::vec3> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = glm::vec3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    put_box(OBB::CreateOBBfromPoints(v), out12);
}

void ref_eig3(const double* a9, double* v9, double* d3) {
    double A[3][3], V[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = a9[3 * i + j];
    eigen_decomposition(A, V, d3);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) v9[3 * i + j] = V[i][j];
}

// The engine's per-pair mid + narrow calls (CollisionDetection.cpp:49-67) over
// a batch of queries, split over `threads` host threads by query. Returns the
// number of triangle-pair tests the narrow phase ran (sum of leaf-pair count
// products); *n_rays receives the total number of uncollide rays.
uint64_t ref_collide_batch(void* const* trees_a, void* const* trees_b, const float* mats_a, const float* mats_b,
                           size_t n, int threads, uint64_t* n_rays, const uint64_t* order) {
    threads = std::max(1, threads);
    std::vector<uint64_t> tests(threads, 0), rays(threads, 0);
    // Each thread takes the next query of `order` (the caller's: largest
    // first) from a shared counter: the cost of a query varies by orders of
    // magnitude, so a fixed split of the list leaves threads idle while one
    // finishes its share.
    std::atomic<size_t> next{0};
    auto work = [&](int tid) {
        OBBtreesCollision mid;
        CreateUncollideRays narrow;
        for (size_t k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
            const size_t q = order ? size_t(order[k]) : k;
            std::pair<CollisionDetectionEntry, CollisionDetectionEntry> p;
            p.first.currentGlobalMatrix = p.first.previousGlobalMatrix = load_mat(mats_a + 16 * q);
            p.first.OBBtree_ptr = static_cast<const OBBtree*>(trees_a[q]);
            p.first.shouldCallback = true;
            p.first.entity = 0;
            p.second.currentGlobalMatrix = p.second.previousGlobalMatrix = load_mat(mats_b + 16 * q);
            p.second.OBBtree_ptr = static_cast<const OBBtree*>(trees_b[q]);
            p.second.shouldCallback = true;
            p.second.entity = 1;
            CDentriesPairTrianglesPairs r = mid.ExecuteOBBtreesCollision(p);
            const auto& lps = r.OBBtreesIntersectInfoObj.candidateTriangleRangeCombinations;
            if (lps.empty()) continue;
            for (const auto& lp : lps) tests[tid] += uint64_t(lp.first_obbtree_count) * lp.second_obbtree_count;
            CDentriesUncollideRays u = narrow.ExecuteCreateUncollideRays(r);
            rays[tid] += u.rays_from_first_to_second.size() + u.rays_from_second_to_first.size();
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
    uint64_t total = 0, total_rays = 0;
    for (int t = 0; t < threads; ++t) {
        total += tests[t];
        total_rays += rays[t];
    }
    if (n_rays) *n_rays = total_rays;
    return total;
}

// ShootUncollideRays::ExecuteShootUncollideRays for one entity pair, built
// with the engine's settings (CollisionDetection.cpp:22-24) or params (start
// and finish angle in radians, bias); rays as (origin, direction) sextuples.
void ref_shoot_rays(void* ta, void* tb, const float* ga16, const float* gb16, const float* rays_a, size_t n_a,
                    const float* rays_b, size_t n_b, const float* params, float* out3) {
    CDentriesUncollideRays u;
    u.firstEntry.currentGlobalMatrix = u.firstEntry.previousGlobalMatrix = load_mat(ga16);
    u.firstEntry.OBBtree_ptr = static_cast<const OBBtree*>(ta);
    u.firstEntry.shouldCallback = true;
    u.firstEntry.entity = 0;
    u.secondEntry.currentGlobalMatrix = u.secondEntry.previousGlobalMatrix = load_mat(gb16);
    u.secondEntry.OBBtree_ptr = static_cast<const OBBtree*>(tb);
    u.secondEntry.shouldCallback = true;
    u.secondEntry.entity = 1;
    auto load = [](const float* r, size_t n, std::vector<Ray>& out) {
        for (size_t i = 0; i < n; ++i)
            out.emplace_back(glm::vec3(r[6 * i], r[6 * i + 1], r[6 * i + 2]),
                             glm::vec3(r[6 * i + 3], r[6 * i + 4], r[6 * i + 5]));
    };
    load(rays_a, n_a, u.rays_from_first_to_second);
    load(rays_b, n_b, u.rays_from_second_to_first);
    const ShootUncollideRays shooter = params ? ShootUncollideRays(params[0], params[1], params[2])
                                              : ShootUncollideRays(glm::radians(40.f), glm::radians(65.f), 1.01f);
    put_vec(shooter.ExecuteShootUncollideRays(u), out3);
}

// SweepAndPrune::ExecuteSweepAndPrune with the engine's axes
// (CollisionDetection.cpp:9-13) or axes9 (U, V, W): the pairs as
// (first entity, second entity) in the order produced; returns their count
// (pairs beyond cap are counted, not written).
size_t ref_sweep_and_prune(void* const* trees, const float* globals, const uint8_t* callback, size_t n,
                           const float* axes9, uint32_t* out_pairs, size_t cap) {
    glm::vec3 U, V, W;
    if (axes9) {
        U = glm::vec3(axes9[0], axes9[1], axes9[2]);
        V = glm::vec3(axes9[3], axes9[4], axes9[5]);
        W = glm::vec3(axes9[6], axes9[7], axes9[8]);
    } else {
        U = glm::normalize(glm::vec3(0.8f, -0.2f, 0.f));
        W = glm::normalize(glm::cross(U, glm::vec3(0.f, -1.f, 0.f)));
        V = glm::normalize(glm::cross(W, U));
    }
    SweepAndPrune sap(U, V, W);
    std::vector<CollisionDetectionEntry> entries(n);
    for (size_t i = 0; i < n; ++i) {
        entries[i].currentGlobalMatrix = entries[i].previousGlobalMatrix = load_mat(globals + 16 * i);
        entries[i].OBBtree_ptr = static_cast<const OBBtree*>(trees[i]);
        entries[i].shouldCallback = callback[i] != 0;
        entries[i].entity = Entity(i);
    }
    const auto pairs = sap.ExecuteSweepAndPrune(entries);
    for (size_t k = 0; k < pairs.size() && k < cap; ++k) {
        out_pairs[2 * k] = pairs[k].first.entity;
        out_pairs[2 * k + 1] = pairs[k].second.entity;
    }
    return pairs.size();
}

}  // extern "C"
