// Drop-in GPU mid and narrow phase for the inMyRoom_vulkan engine, header-only
// C++ over the C ABI of include/collide_gpu.h (through cg_session.h). It is
// compiled inside the engine (it uses the engine's OBBtree,
// CollisionDetectionEntry, Ray and glm types) and sits beside the CPU classes
// that CollisionDetection owns (include/CollisionDetection/CollisionDetection.h:
// 29-32):
//
//   OBBtreesCollision::ExecuteOBBtreesCollision(pair)           (CPU, one pair)
//   GpuOBBtreesCollision::ExecuteOBBtreesCollision(pair)        (GPU, same result)
//   GpuOBBtreesCollision::ExecuteOBBtreesCollisionBatch(pairs)  (GPU, one launch)
//
//   CreateUncollideRays::ExecuteCreateUncollideRays(pair_tris)        (CPU)
//   GpuCreateUncollideRays::ExecuteCreateUncollideRays(pair_tris)     (GPU, same result)
//   GpuCreateUncollideRays::ExecuteCreateUncollideRaysBatch(...)      (GPU, one launch)
//
// Results are the CPU calls' bit for bit and in their order: the candidate
// leaf pairs in the recursion's order, the rays in the order the CPU's
// per-triangle unordered_map gives them (GCC's libstdc++), the mean origins.
// The GPU narrow phase runs the mid phase of the pair again in the same
// launch (it does not read the CDentriesPairTrianglesPairs' leaf pairs), so
// its result is the CPU's for the leaf pairs the engine passes: those of the
// pair's own mid phase in their order (CollisionDetection.cpp:49-67).
//
// Both adapters can share one GpuCollisionContext (its trees are uploaded on
// first use, keyed by the OBBtree pointer; call ForgetTree when an OBBtree is
// destroyed).
#pragma once

#include <algorithm>
#include <memory>
#include <unordered_map>
#include <utility>
#include <vector>

#include "CollisionDetection/CreateUncollideRays.h"
#include "CollisionDetection/OBBtreesCollision.h"
#include "Geometry/OBBtree.h"
#include "Geometry/Ray.h"
#include "cg_session.h"
#include "collide_gpu.h"
#include "glm/gtc/type_ptr.hpp"

class GpuCollisionContext {
public:
    explicit GpuCollisionContext(const cg_config* cfg = nullptr) : session_(cfg) {}

    const cg_adapter::Session& Session() const { return session_; }

    // The query of an entity pair: both trees' ids and the relative matrix of
    // OBBtreesCollision.cpp:15 / CreateUncollideRays.cpp:62-63, with the
    // engine's glm.
    cg_query Query(const CollisionDetectionEntry& first, const CollisionDetectionEntry& second) const {
        cg_query q;
        q.tree_a = TreeId(first.OBBtree_ptr);
        q.tree_b = TreeId(second.OBBtree_ptr);
        const glm::mat4 rel = glm::inverse(first.currentGlobalMatrix) * second.currentGlobalMatrix;
        std::copy(glm::value_ptr(rel), glm::value_ptr(rel) + 16, q.relative);
        return q;
    }

    void ForgetTree(const OBBtree* tree) {
        auto it = ids_.find(tree);
        if (it != ids_.end()) {
            session_.Free(it->second);
            ids_.erase(it);
        }
    }

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
        const uint32_t id = session_.Upload(view);
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

    cg_adapter::Session session_;
    mutable std::unordered_map<const OBBtree*, uint32_t> ids_;
};

class GpuOBBtreesCollision {
public:
    explicit GpuOBBtreesCollision(const cg_config* cfg = nullptr)
        : ctx_(std::make_shared<GpuCollisionContext>(cfg)) {}
    explicit GpuOBBtreesCollision(std::shared_ptr<GpuCollisionContext> ctx) : ctx_(std::move(ctx)) {}

    // Same signature and result as OBBtreesCollision::ExecuteOBBtreesCollision.
    CDentriesPairTrianglesPairs ExecuteOBBtreesCollision(
        const std::pair<CollisionDetectionEntry, CollisionDetectionEntry>& entries) const {
        return ExecuteOBBtreesCollisionBatch({entries}).front();
    }

    std::vector<CDentriesPairTrianglesPairs> ExecuteOBBtreesCollisionBatch(
        const std::vector<std::pair<CollisionDetectionEntry, CollisionDetectionEntry>>& pairs) const {
        std::vector<cg_query> queries(pairs.size());
        for (size_t i = 0; i < pairs.size(); ++i) queries[i] = ctx_->Query(pairs[i].first, pairs[i].second);
        const std::vector<std::vector<cg_leaf_pair>> leafs = ctx_->Session().MidPhase(queries);
        std::vector<CDentriesPairTrianglesPairs> out(pairs.size());
        for (size_t i = 0; i < pairs.size(); ++i) {
            out[i].firstEntry = pairs[i].first;
            out[i].secondEntry = pairs[i].second;
            auto& v = out[i].OBBtreesIntersectInfoObj.candidateTriangleRangeCombinations;
            for (const cg_leaf_pair& lp : leafs[i])
                v.push_back({size_t(lp.offset_a), size_t(lp.count_a), size_t(lp.offset_b), size_t(lp.count_b)});
        }
        return out;
    }

    void ForgetTree(const OBBtree* tree) { ctx_->ForgetTree(tree); }
    cg_ctx* Context() const { return ctx_->Session().Context(); }
    const std::shared_ptr<GpuCollisionContext>& Shared() const { return ctx_; }

private:
    std::shared_ptr<GpuCollisionContext> ctx_;
};

class GpuCreateUncollideRays {
public:
    explicit GpuCreateUncollideRays(const cg_config* cfg = nullptr)
        : ctx_(std::make_shared<GpuCollisionContext>(cfg)) {}
    explicit GpuCreateUncollideRays(std::shared_ptr<GpuCollisionContext> ctx) : ctx_(std::move(ctx)) {}

    // Same signature and result as CreateUncollideRays::ExecuteCreateUncollideRays.
    CDentriesUncollideRays ExecuteCreateUncollideRays(const CDentriesPairTrianglesPairs& pair_tris) const {
        return ExecuteCreateUncollideRaysBatch({pair_tris}).front();
    }

    std::vector<CDentriesUncollideRays> ExecuteCreateUncollideRaysBatch(
        const std::vector<CDentriesPairTrianglesPairs>& batch) const {
        std::vector<cg_query> queries(batch.size());
        for (size_t i = 0; i < batch.size(); ++i) queries[i] = ctx_->Query(batch[i].firstEntry, batch[i].secondEntry);
        const std::vector<cg_adapter::QueryRays> rays = ctx_->Session().UncollideRays(queries);
        std::vector<CDentriesUncollideRays> out(batch.size());
        auto vec = [](const float* p) { return glm::vec3(p[0], p[1], p[2]); };
        for (size_t i = 0; i < batch.size(); ++i) {
            out[i].firstEntry = batch[i].firstEntry;
            out[i].secondEntry = batch[i].secondEntry;
            for (const cg_ray& r : rays[i].first) out[i].rays_from_first_to_second.emplace_back(vec(r.origin), vec(r.direction));
            for (const cg_ray& r : rays[i].second) out[i].rays_from_second_to_first.emplace_back(vec(r.origin), vec(r.direction));
            out[i].average_point_first_modelspace = vec(rays[i].average_first);
            out[i].average_point_second_modelspace = vec(rays[i].average_second);
        }
        return out;
    }

    void ForgetTree(const OBBtree* tree) { ctx_->ForgetTree(tree); }
    const std::shared_ptr<GpuCollisionContext>& Shared() const { return ctx_; }

private:
    std::shared_ptr<GpuCollisionContext> ctx_;
};
