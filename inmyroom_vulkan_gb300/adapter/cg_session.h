// The engine-independent core of the C++ drop-in adapters: one collision
// context, the trees uploaded into it, and the two batch calls the engine's
// collision step makes per frame, with their results in the reference's
// containers and order:
//
//   MidPhase       per query, the candidate leaf pairs in the order of
//                  OBBtree::IntersectOBBtreesRecursive
//                  (src/Geometry/OBBtree.cpp:414-476), the vector
//                  OBBtreesCollision::ExecuteOBBtreesCollision returns
//   UncollideRays  per query, the uncollide rays of both sides in the order
//                  CreateUncollideRays::ExecuteCreateUncollideRays makes them
//                  (its unordered_map's iteration order, CreateUncollideRays.cpp:
//                  131-178) and the two mean origins (:183-198)
//
// Only the C ABI of include/collide_gpu.h and the standard library are used,
// so the core builds without the engine's headers (the engine adapters in
// gpu_obbtrees_collision.h wrap it with the engine's types). Errors throw
// std::runtime_error with the library's message.
#pragma once

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "collide_gpu.h"

namespace cg_adapter {

// The rays and mean origins of one query (CDentriesUncollideRays without its
// entries): rays from the first tree to the second, then the other way, all
// in the first tree's model space; the second mean origin in the second
// tree's model space.
struct QueryRays {
    std::vector<cg_ray> first, second;
    float average_first[3] = {0.f, 0.f, 0.f};
    float average_second[3] = {0.f, 0.f, 0.f};
};

class Session {
public:
    explicit Session(const cg_config* cfg = nullptr) { Check(cg_create(cfg, &ctx_)); }
    ~Session() { cg_destroy(ctx_); }
    Session(const Session&) = delete;
    Session& operator=(const Session&) = delete;

    cg_ctx* Context() const { return ctx_; }

    uint32_t Upload(const cg_tree_view& view) const {
        uint32_t id = 0;
        Check(cg_tree_upload(ctx_, &view, &id));
        return id;
    }
    void Free(uint32_t tree_id) const { cg_tree_free(ctx_, tree_id); }

    // Per query, its candidate leaf pairs in the reference's order (one
    // launch for the batch: mid phase only).
    std::vector<std::vector<cg_leaf_pair>> MidPhase(const std::vector<cg_query>& queries) const {
        std::vector<std::vector<cg_leaf_pair>> out(queries.size());
        if (queries.empty()) return out;
        cg_stats st;
        Check(cg_collide(ctx_, queries.data(), uint32_t(queries.size()),
                         CG_KEEP_LEAF_PAIRS | CG_DFS_ORDER | CG_MID_ONLY, &st));
        std::vector<cg_leaf_pair> all(st.leaf_pairs);
        uint64_t n = 0;
        Check(cg_read_leaf_pairs(ctx_, all.data(), all.size(), &n));
        for (const cg_leaf_pair& lp : all) out[lp.query].push_back(lp);  // grouped and ordered already
        return out;
    }

    // Per query, its uncollide rays and mean origins (one launch for the
    // batch: mid phase, triangle tests, contacts and rays).
    std::vector<QueryRays> UncollideRays(const std::vector<cg_query>& queries) const {
        std::vector<QueryRays> out(queries.size());
        if (queries.empty()) return out;
        cg_stats st;
        Check(cg_collide(ctx_, queries.data(), uint32_t(queries.size()), CG_CONTACTS, &st));
        std::vector<cg_ray> rays(st.rays);
        std::vector<cg_ray_average> avg(queries.size());
        uint64_t n = 0;
        Check(cg_read_rays(ctx_, rays.data(), rays.size(), &n));
        Check(cg_read_ray_averages(ctx_, avg.data(), avg.size(), &n));
        for (const cg_ray& r : rays) (r.side ? out[r.query].second : out[r.query].first).push_back(r);
        for (size_t q = 0; q < queries.size(); ++q) {
            std::copy(avg[q].first, avg[q].first + 3, out[q].average_first);
            std::copy(avg[q].second, avg[q].second + 3, out[q].average_second);
        }
        return out;
    }

    void Check(int rc) const {
        if (rc != CG_OK) {
            char buf[512] = {0};
            if (ctx_) cg_last_error(ctx_, buf, sizeof(buf));
            throw std::runtime_error(std::string(cg_status_string(rc)) + ": " + buf);
        }
    }

private:
    cg_ctx* ctx_ = nullptr;
};

}  // namespace cg_adapter
