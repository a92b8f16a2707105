// The C++ adapters' core (inmyroom_vulkan_gb300/adapter/cg_session.h) driven
// the way the engine adapters drive it, checked against the oracle: built by
// tests/test_gpu_adapter_session.py against libcollide_gpu.so and the oracle's
// restatement (liboracle_port.so, its C functions declared below).
//
// Input (binary, little-endian): uint32 n_meshes; per mesh uint32 n_points,
// n_indices, has_normals, then the points, the normals (if any) and the
// indices; uint32 n_queries; per query uint32 mesh_a, mesh_b and two 16-float
// world matrices. For every query it compares, bit for bit and in order:
//   Session::MidPhase       with the oracle's recursion's leaf pairs
//   Session::UncollideRays  with the oracle's rays of both sides and mean origins
// and prints "ok <queries> <leaf pairs> <rays>", or the first difference and
// exits 1.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "cg_session.h"

extern "C" {
void* port_tree_build(const float* points, size_t n_points, const float* normals, const uint32_t* indices,
                      size_t n_indices);
void port_tree_free(void* t);
void port_tree_sizes(void* t, size_t* n_nodes, size_t* n_tris);
void port_tree_export(void* t, float* root12, float* node_obbs, uint32_t* node_ref, uint32_t* node_cnt,
                      float* tri_pos, float* tri_nrm, uint32_t* tri_idx);
void port_relative_matrix(const float* a16, const float* b16, float* out16);
void* port_mid_phase(void* ta, void* tb, const float* a16, const float* b16);
void port_mid_free(void* r);
size_t port_mid_count(void* r);
void port_mid_get(void* r, uint32_t* out);
void port_rays(void* r, float* rays_a, float* rays_b, size_t cap_a, size_t cap_b, size_t* counts, float* avg);
}

namespace {

bool read_u32(FILE* f, uint32_t* v) { return std::fread(v, 4, 1, f) == 1; }
template <class T>
bool read_n(FILE* f, std::vector<T>& v, size_t n) {
    v.resize(n);
    return n == 0 || std::fread(v.data(), sizeof(T), n, f) == n;
}

bool same_bits(const float* a, const float* b, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        if (std::isnan(a[i]) && std::isnan(b[i])) continue;  // 0 / 0 of a side without rays
        if (std::memcmp(a + i, b + i, 4) != 0) return false;
    }
    return true;
}

int fail(const char* what, size_t q) {
    std::printf("mismatch: %s, query %zu\n", what, q);
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    uint32_t n_meshes = 0;
    if (!read_u32(f, &n_meshes)) return 2;
    cg_adapter::Session session;
    std::vector<void*> port_trees(n_meshes);
    std::vector<uint32_t> ids(n_meshes);
    for (uint32_t m = 0; m < n_meshes; ++m) {
        uint32_t np = 0, ni = 0, hn = 0;
        std::vector<float> pts, nrm;
        std::vector<uint32_t> idx;
        if (!read_u32(f, &np) || !read_u32(f, &ni) || !read_u32(f, &hn) || !read_n(f, pts, 3ull * np) ||
            (hn && !read_n(f, nrm, 3ull * np)) || !read_n(f, idx, ni))
            return 2;
        port_trees[m] = port_tree_build(pts.data(), np, hn ? nrm.data() : nullptr, idx.data(), ni);
        // the flat tree the engine adapter would export from an OBBtree
        size_t nn = 0, nt = 0;
        port_tree_sizes(port_trees[m], &nn, &nt);
        std::vector<float> root(12), obbs(24 * nn), pos(9 * nt), tn(9 * nt);
        std::vector<uint32_t> ref(2 * nn), cnt(2 * nn), ti(3 * nt);
        port_tree_export(port_trees[m], root.data(), obbs.data(), ref.data(), cnt.data(), pos.data(), tn.data(),
                         ti.data());
        cg_tree_view v{};
        std::memcpy(&v.root_obb, root.data(), sizeof(cg_obb));
        v.node_count = uint32_t(nn);
        v.node_obbs = reinterpret_cast<const cg_obb*>(obbs.data());
        v.node_ref = ref.data();
        v.node_tri_count = cnt.data();
        v.triangle_count = uint32_t(nt);
        v.triangles_position = pos.data();
        v.triangles_normal = tn.data();
        v.triangles_indices = ti.data();
        ids[m] = session.Upload(v);
    }
    uint32_t nq = 0;
    if (!read_u32(f, &nq)) return 2;
    std::vector<uint32_t> qa(nq), qb(nq);
    std::vector<float> ma(16ull * nq), mb(16ull * nq);
    std::vector<cg_query> queries(nq);
    for (uint32_t q = 0; q < nq; ++q) {
        if (!read_u32(f, &qa[q]) || !read_u32(f, &qb[q]) || std::fread(&ma[16 * q], 4, 16, f) != 16 ||
            std::fread(&mb[16 * q], 4, 16, f) != 16)
            return 2;
        queries[q].tree_a = ids[qa[q]];
        queries[q].tree_b = ids[qb[q]];
        port_relative_matrix(&ma[16 * q], &mb[16 * q], queries[q].relative);
    }
    std::fclose(f);

    const auto leafs = session.MidPhase(queries);
    const auto rays = session.UncollideRays(queries);
    size_t n_leaf = 0, n_rays = 0;
    for (uint32_t q = 0; q < nq; ++q) {
        void* mid = port_mid_phase(port_trees[qa[q]], port_trees[qb[q]], &ma[16 * q], &mb[16 * q]);
        const size_t nl = port_mid_count(mid);
        std::vector<uint32_t> want(4 * nl + 4);
        port_mid_get(mid, want.data());
        if (leafs[q].size() != nl) return fail("leaf-pair count", q);
        for (size_t i = 0; i < nl; ++i) {
            const cg_leaf_pair& g = leafs[q][i];
            if (g.offset_a != want[4 * i] || g.count_a != want[4 * i + 1] || g.offset_b != want[4 * i + 2] ||
                g.count_b != want[4 * i + 3])
                return fail("leaf pair", q);
        }
        size_t counts[2] = {0, 0};
        float avg[6];
        port_rays(mid, nullptr, nullptr, 0, 0, counts, avg);
        std::vector<float> ra(6 * counts[0] + 6), rb(6 * counts[1] + 6);
        port_rays(mid, ra.data(), rb.data(), counts[0], counts[1], counts, avg);
        const std::vector<cg_ray>* got[2] = {&rays[q].first, &rays[q].second};
        const std::vector<float>* exp[2] = {&ra, &rb};
        for (int s = 0; s < 2; ++s) {
            if (got[s]->size() != counts[s]) return fail("ray count", q);
            for (size_t i = 0; i < counts[s]; ++i) {
                const cg_ray& r = (*got[s])[i];
                if (!same_bits(r.origin, exp[s]->data() + 6 * i, 3) || !same_bits(r.direction, exp[s]->data() + 6 * i + 3, 3))
                    return fail("ray", q);
            }
        }
        if (!same_bits(rays[q].average_first, avg, 3) || !same_bits(rays[q].average_second, avg + 3, 3))
            return fail("mean origin", q);
        port_mid_free(mid);
        n_leaf += nl;
        n_rays += counts[0] + counts[1];
    }
    for (void* t : port_trees) port_tree_free(t);
    std::printf("ok %u %zu %zu\n", nq, n_leaf, n_rays);
    return 0;
}
