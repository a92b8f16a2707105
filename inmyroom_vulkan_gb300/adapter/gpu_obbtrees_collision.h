// Drop-in GPU mid phase for the inMyRoom_vulkan engine, header-only C++ over
// the C ABI of include/collide_gpu.h. It is compiled inside the engine (it
// uses the engine's OBBtree, CollisionDetectionEntry and glm types) and sits
// beside OBBtreesCollision (include/CollisionDetection/OBBtreesCollision.h):
//
//   OBBtreesCollision::ExecuteOBBtreesCollision(pair)      (CPU, one pair)
//   GpuOBBtreesCollision::ExecuteOBBtreesCollision(pair)   (GPU, same result)
//   GpuOBBtreesCollision::ExecuteOBBtreesCollisionBatch(pairs)
//                                   (GPU, every pair of a frame in one launch)
//
// The candidate leaf pairs are the same set as the CPU call returns; within a
// pair's vector they are sorted by (first offset, second offset) instead of
// the CPU recursion order. Trees are uploaded on first use, keyed by the
// OBBtree pointer; call ForgetTree when an OBBtree is destroyed.
#pragma once

#include <algorithm>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "CollisionDetection/OBBtreesCollision.h"
#include "Geometry/OBBtree.h"
#include "collide_gpu.h"
#include "glm/gtc/type_ptr.hpp"

class GpuOBBtreesCollision {
public:
    explicit GpuOBBtreesCollision(const cg_config* cfg = nullptr) {
        const int rc = cg_create(cfg, &ctx_);
        if (rc != CG_OK) throw std::runtime_error(std::string("cg_create: ") + cg_status_string(rc));
    }
    ~GpuOBBtreesCollision() { cg_destroy(ctx_); }
    GpuOBBtreesCollision(const GpuOBBtreesCollision&) = delete;
    GpuOBBtreesCollision& operator=(const GpuOBBtreesCollision&) = delete;

    // Same signature and result as OBBtreesCollision::ExecuteOBBtreesCollision.
    CDentriesPairTrianglesPairs ExecuteOBBtreesCollision(
        const std::pair<CollisionDetectionEntry, CollisionDetectionEntry>& entries) const {
        return ExecuteOBBtreesCollisionBatch({entries}).front();
    }

    std::vector<CDentriesPairTrianglesPairs> ExecuteOBBtreesCollisionBatch(
        const std::vector<std::pair<CollisionDetectionEntry, CollisionDetectionEntry>>& pairs) const {
        std::vector<cg_query> queries(pairs.size());
        for (size_t i = 0; i < pairs.size(); ++i) {
            queries[i].tree_a = TreeId(pairs[i].first.OBBtree_ptr);
            queries[i].tree_b = TreeId(pairs[i].second.OBBtree_ptr);
            // the relative matrix of OBBtreesCollision.cpp:15, with the engine's glm
            const glm::mat4 rel =
                glm::inverse(pairs[i].first.currentGlobalMatrix) * pairs[i].second.currentGlobalMatrix;
            std::copy(glm::value_ptr(rel), glm::value_ptr(rel) + 16, queries[i].relative);
        }
        cg_stats st;
        Check(cg_collide(ctx_, queries.data(), uint32_t(queries.size()), CG_KEEP_LEAF_PAIRS | CG_MID_ONLY, &st));
        std::vector<cg_leaf_pair> leafs(st.leaf_pairs);
        uint64_t n = 0;
        Check(cg_read_leaf_pairs(ctx_, leafs.data(), leafs.size(), &n));
        std::sort(leafs.begin(), leafs.end(), [](const cg_leaf_pair& a, const cg_leaf_pair& b) {
            return a.query != b.query ? a.query < b.query
                                      : (a.offset_a != b.offset_a ? a.offset_a < b.offset_a : a.offset_b < b.offset_b);
        });
        std::vector<CDentriesPairTrianglesPairs> out(pairs.size());
        for (size_t i = 0; i < pairs.size(); ++i) {
            out[i].firstEntry = pairs[i].first;
            out[i].secondEntry = pairs[i].second;
        }
        for (const cg_leaf_pair& lp : leafs)
            out[lp.query].OBBtreesIntersectInfoObj.candidateTriangleRangeCombinations.push_back(
                {size_t(lp.offset_a), size_t(lp.count_a), size_t(lp.offset_b), size_t(lp.count_b)});
        return out;
    }

    void ForgetTree(const OBBtree* tree) {
        auto it = ids_.find(tree);
        if (it != ids_.end()) {
            cg_tree_free(ctx_, it->second);
            ids_.erase(it);
        }
    }

    cg_ctx* Context() const { return ctx_; }

    // Uploads `tree` (once) and returns its id. The flat view is exported
    // through the public OBBtreeTraveler walk: inner nodes in pre-order get
    // the indices OBBtree::ConstructDFSrecursive gave them.
    uint32_t TreeId(const OBBtree* tree) const {
        auto it = ids_.find(tree);
        if (it != ids_.end()) return it->second;
        std::vector<cg_obb> obbs;
        std::vector<uint32_t> refs, counts;
        size_t n_tris = 0;
        OBBtree::OBBtreeTraveler root = tree->GetRootTraveler();
        if (root.IsLeaf()) {
            n_tris = root.GetTrianglesCount();
        } else {
            Walk(root, obbs, refs, counts, n_tris);
        }
        std::vector<float> pos(9 * n_tris), nrm(9 * n_tris);
        std::vector<uint32_t> idx(3 * n_tris);
        for (size_t t = 0; t < n_tris; ++t) {
            const TrianglePosition p = tree->GetTrianglePosition(t);
            const TriangleNormal nn = tree->GetTriangleNormal(t);
            const TriangleIndices ii = tree->GetTriangleIndices(t);
            for (int k = 0; k < 3; ++k) {
                const glm::vec3 v = p.GetP(k), w = nn.GetN(k);
                pos[9 * t + 3 * k] = v.x, pos[9 * t + 3 * k + 1] = v.y, pos[9 * t + 3 * k + 2] = v.z;
                nrm[9 * t + 3 * k] = w.x, nrm[9 * t + 3 * k + 1] = w.y, nrm[9 * t + 3 * k + 2] = w.z;
                idx[3 * t + k] = ii.GetI(k);
            }
        }
        cg_tree_view view{};
        view.root_obb = Box(tree->GetRootOBB());
        view.node_count = uint32_t(obbs.size() / 2);
        view.node_obbs = obbs.data();
        view.node_ref = refs.data();
        view.node_tri_count = counts.data();
        view.triangle_count = uint32_t(n_tris);
        view.triangles_position = pos.data();
        view.triangles_normal = nrm.data();
        view.triangles_indices = idx.data();
        uint32_t id = 0;
        Check(cg_tree_upload(ctx_, &view, &id));
        ids_.emplace(tree, id);
        return id;
    }

private:
    static cg_obb Box(const Paralgram& p) {
        cg_obb b;
        const glm::vec3 c = p.GetCenter(), u = p.GetSideDirectionU(), v = p.GetSideDirectionV(),
                        w = p.GetSideDirectionW();
        const float vals[12] = {c.x, c.y, c.z, u.x, u.y, u.z, v.x, v.y, v.z, w.x, w.y, w.z};
        std::copy(vals, vals + 3, b.center);
        std::copy(vals + 3, vals + 6, b.u);
        std::copy(vals + 6, vals + 9, b.v);
        std::copy(vals + 9, vals + 12, b.w);
        return b;
    }

    // Pre-order walk of the inner nodes (OBBtree.cpp:179-233, 385-394).
    static void Walk(const OBBtree::OBBtreeTraveler& t, std::vector<cg_obb>& obbs, std::vector<uint32_t>& refs,
                     std::vector<uint32_t>& counts, size_t& n_tris) {
        const size_t me = obbs.size() / 2;
        obbs.resize(obbs.size() + 2);
        refs.resize(refs.size() + 2);
        counts.resize(counts.size() + 2);
        const OBBtree::OBBtreeTraveler kids[2] = {t.GetLeftChildTraveler(), t.GetRightChildTraveler()};
        for (int s = 0; s < 2; ++s) {
            obbs[2 * me + s] = Box(kids[s].GetOBB());
            if (kids[s].IsLeaf()) {
                refs[2 * me + s] = uint32_t(kids[s].GetTrianglesOffset());
                counts[2 * me + s] = uint32_t(kids[s].GetTrianglesCount());
                n_tris = std::max(n_tris, kids[s].GetTrianglesOffset() + kids[s].GetTrianglesCount());
            } else {
                refs[2 * me + s] = uint32_t(obbs.size() / 2);
                counts[2 * me + s] = 0;
                Walk(kids[s], obbs, refs, counts, n_tris);
            }
        }
    }

    void Check(int rc) const {
        if (rc != CG_OK) {
            char buf[512];
            cg_last_error(ctx_, buf, sizeof(buf));
            throw std::runtime_error(std::string(cg_status_string(rc)) + ": " + buf);
        }
    }

    cg_ctx* ctx_ = nullptr;
    mutable std::unordered_map<const OBBtree*, uint32_t> ids_;
};
