// Oracle test infrastructure: a C++ restatement of the reference engine's CPU
// collision path (inMyRoom_vulkan), used only by tests and by the CPU baseline
// timing. It is never linked into the GPU library.
//
// Each function follows the reference function cited beside it, step for step
// and in the same floating-point operation order (built with
// -ffp-contract=off), so that its trees, candidate leaf pairs, colliding
// triangle pairs and segments are bit-identical to the reference compiled
// against the same glm-convention shim. The C ABI mirrors oracle/ref_capi.cpp
// with a port_ prefix.
#include <atomic>
#include <algorithm>
#include <array>
#include <cstring>
#include <memory>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

#include "eig3x3.h"
#include "vecmath.h"

namespace port {

// ---------------------------------------------------------------- boxes ----
// Paralgram = center plus three half-extent vectors
// (inMyRoom_vulkan/include/Geometry/Paralgram.h:28-35).
struct Box {
    V3 c, u, v, w;
};

// Paralgram::MultiplyBy4x4Matrix (src/Geometry/Paralgram.cpp:4-15).
inline Box xform_box(const M4& M, const Box& b) {
    return Box{xform(M, b.c, 1.0f), xform(M, b.u, 0.0f), xform(M, b.v, 0.0f), xform(M, b.w, 0.0f)};
}

// Paralgram::GetMinMaxProjectionToAxis / GetCenterProjectionToAxis
// (Paralgram.cpp:175-196).
inline void project(const Box& b, V3 axis, float& lo, float& hi) {
    float cp = dot(b.c, axis);
    float eu = std::abs(dot(axis, b.u));
    float ev = std::abs(dot(axis, b.v));
    float ew = std::abs(dot(axis, b.w));
    float e = eu + ev + ew;
    lo = cp - e;
    hi = cp + e;
}

// One separating-axis check (Paralgram.cpp:198-201): true when the
// projections overlap on this axis.
inline bool overlap_on(const Box& a, const Box& b, V3 axis) {
    float alo, ahi, blo, bhi;
    project(a, axis, alo, ahi);
    project(b, axis, blo, bhi);
    return (ahi >= blo) && (bhi >= alo);
}

// Paralgram::IntersectParalgramsBoolean (Paralgram.cpp:17-173): the face
// normals of a, then of b, then the nine edge crosses a_i x b_j, unnormalised,
// in the reference's order.
inline bool sat(const Box& a, const Box& b) {
    if (!overlap_on(a, b, cross(a.v, a.w))) return false;
    if (!overlap_on(a, b, cross(a.u, a.w))) return false;
    if (!overlap_on(a, b, cross(a.u, a.v))) return false;
    if (!overlap_on(a, b, cross(b.v, b.w))) return false;
    if (!overlap_on(a, b, cross(b.u, b.w))) return false;
    if (!overlap_on(a, b, cross(b.u, b.v))) return false;
    const V3 ea[3] = {a.u, a.v, a.w};
    const V3 eb[3] = {b.u, b.v, b.w};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (!overlap_on(a, b, cross(ea[i], eb[j]))) return false;
    return true;
}

// Paralgram::GetSurface (Paralgram.cpp:203-210).
inline float surface(const Box& b) {
    float uv = length(cross(b.u, b.v));
    float uw = length(cross(b.u, b.w));
    float vw = length(cross(b.v, b.w));
    return 2.0f * (uv + uw + vw);
}

// ------------------------------------------------------------ triangles ----
struct Tri {
    V3 p[3];
    V3 n[3];
    uint32_t i[3];
};

// TrianglePosition::GetTriangleFaceNormal (src/Geometry/Triangle.cpp:140-146).
inline V3 face_normal(const V3 p[3]) { return normalize(cross(sub(p[1], p[0]), sub(p[2], p[0]))); }

// TrianglePosition::GetMinMaxProjectionToAxis (Triangle.cpp:113-138).
inline void tri_project(const Tri& t, V3 axis, float& lo, float& hi) {
    lo = std::numeric_limits<float>::infinity();
    hi = -std::numeric_limits<float>::infinity();
    for (int k = 0; k < 3; ++k) {
        float pr = dot(axis, t.p[k]);
        if (pr < lo) lo = pr;
        if (pr > hi) hi = pr;
    }
}

// ----------------------------------------------------------------- OBBs ----
// OBB::EmptyOBB (src/Geometry/OBB.cpp:168-178).
inline Box empty_box() {
    const float e = std::numeric_limits<float>::epsilon();
    return Box{V3{0, 0, 0}, V3{e, 0, 0}, V3{0, e, 0}, V3{0, 0, e}};
}

// OBB::CreateAABBfromPoints (OBB.cpp:105-166): FP64 projections on each axis,
// extents padded by 2*FLT_EPSILON, centre and half-extents cast to float.
inline Box box_on_axes(const std::vector<V3>& pts, const D3 axes[3]) {
    D3 center{0.0, 0.0, 0.0};
    V3 half[3];
    const double pad = 2.0 * double(std::numeric_limits<float>::epsilon());
    for (int a = 0; a < 3; ++a) {
        double lo = std::numeric_limits<double>::infinity();
        double hi = -std::numeric_limits<double>::infinity();
        for (const V3& p : pts) {
            double pr = dotd(axes[a], D3{double(p.x), double(p.y), double(p.z)});
            lo = (lo < pr) ? lo : pr;  // std::min(pr, lo)
            hi = (pr < hi) ? hi : pr;  // std::max(pr, hi)
        }
        double delta = (hi - lo) + pad;
        double mid = (hi + lo) / 2.0;
        center.x = center.x + mid * axes[a].x;
        center.y = center.y + mid * axes[a].y;
        center.z = center.z + mid * axes[a].z;
        double h = delta / 2.0;
        half[a] = V3{float(h * axes[a].x), float(h * axes[a].y), float(h * axes[a].z)};
    }
    return Box{V3{float(center.x), float(center.y), float(center.z)}, half[0], half[1], half[2]};
}

// OBB::CreateOBBfromPoints (OBB.cpp:33-89). Fewer than two distinct points
// give the empty or point box; otherwise the FP64 mean and covariance are
// accumulated sequentially, eig3 is applied, and the box axes are the ROWS of
// eig3's eigenvector matrix (the glm column-major view of its output).
inline Box fit_box(const std::vector<V3>& pts) {
    if (pts.empty()) return empty_box();
    bool all_same = true;
    for (size_t k = 1; k < pts.size() && all_same; ++k)
        if (!eq(pts[k], pts[0])) all_same = false;
    if (all_same) {
        Box b = empty_box();
        b.c = pts[0];
        return b;
    }
    const double n = double(pts.size());
    D3 sum{0.0, 0.0, 0.0};
    for (const V3& p : pts) {
        sum.x = sum.x + double(p.x);
        sum.y = sum.y + double(p.y);
        sum.z = sum.z + double(p.z);
    }
    const D3 mean{sum.x / n, sum.y / n, sum.z / n};
    double cxx = 0, cyy = 0, czz = 0, cxy = 0, cxz = 0, cyz = 0;
    for (const V3& p : pts) cxx = cxx + (p.x - mean.x) * (p.x - mean.x);
    for (const V3& p : pts) cyy = cyy + (p.y - mean.y) * (p.y - mean.y);
    for (const V3& p : pts) czz = czz + (p.z - mean.z) * (p.z - mean.z);
    for (const V3& p : pts) cxy = cxy + (p.x - mean.x) * (p.y - mean.y);
    for (const V3& p : pts) cxz = cxz + (p.x - mean.x) * (p.z - mean.z);
    for (const V3& p : pts) cyz = cyz + (p.y - mean.y) * (p.z - mean.z);
    const double a[3][3] = {{cxx / n, cxy / n, cxz / n}, {cxy / n, cyy / n, cyz / n}, {cxz / n, cyz / n, czz / n}};
    double vecs[3][3], vals[3];
    eigen_sym3(a, vecs, vals);
    const D3 axes[3] = {D3{vecs[0][0], vecs[0][1], vecs[0][2]}, D3{vecs[1][0], vecs[1][1], vecs[1][2]},
                        D3{vecs[2][0], vecs[2][1], vecs[2][2]}};
    return box_on_axes(pts, axes);
}

// OBB::CreateOBBfromTriangles (OBB.cpp:91-103).
inline Box fit_tris(const std::vector<Tri>& tris) {
    std::vector<V3> pts;
    pts.reserve(tris.size() * 3);
    for (const Tri& t : tris)
        for (int k = 0; k < 3; ++k) pts.push_back(t.p[k]);
    return fit_box(pts);
}

// ----------------------------------------------------------------- tree ----
constexpr size_t kLeafMax = 4;  // OBBtree.h:49 maxNumberOfTriangles

struct BuildNode {
    Box box;
    bool leaf = true;
    bool right = false;
    std::unique_ptr<BuildNode> kid[2];
    std::vector<Tri> tris;
    size_t index = size_t(-1);
};

std::unique_ptr<BuildNode> build_node(std::vector<Tri> tris, bool is_right);

// OBBtreeSplitBuildNode::SplitOBBandCreateChildren (OBBtree.cpp:43-108):
// axes by half-length, longest first (ties keep u,v,w order); a triangle goes
// left when the mean of its projection interval is <= the box centre's
// projection; the first axis that leaves both sides non-empty wins, else the
// list is halved by index; the child with the larger surface goes left.
void split(BuildNode& nd) {
    struct AxisLen {
        float len;
        V3 dir;
    };
    AxisLen ax[3] = {{length(nd.box.u), normalize(nd.box.u)},
                     {length(nd.box.v), normalize(nd.box.v)},
                     {length(nd.box.w), normalize(nd.box.w)}};
    std::stable_sort(ax, ax + 3, [](const AxisLen& a, const AxisLen& b) { return a.len > b.len; });

    std::vector<Tri> left, right;
    size_t k = 0;
    do {
        left.clear();
        right.clear();
        const V3 axis = ax[k].dir;
        const float cp = dot(nd.box.c, axis);
        for (const Tri& t : nd.tris) {
            float lo, hi;
            tri_project(t, axis, lo, hi);
            float mid = (lo + hi) / 2.0f;
            if (mid <= cp)
                left.push_back(t);
            else
                right.push_back(t);
        }
        ++k;
    } while ((left.empty() || right.empty()) && k < 3);

    if (left.empty() || right.empty()) {
        left.clear();
        right.clear();
        const size_t half = nd.tris.size() / 2;
        for (size_t i = 0; i < nd.tris.size(); ++i) (i < half ? left : right).push_back(nd.tris[i]);
    }
    nd.tris.clear();
    nd.leaf = false;
    nd.kid[0] = build_node(std::move(left), false);
    nd.kid[1] = build_node(std::move(right), true);
    if (surface(nd.kid[1]->box) > surface(nd.kid[0]->box)) {
        std::swap(nd.kid[0], nd.kid[1]);
        nd.kid[1]->right = true;
        nd.kid[0]->right = false;
    }
}

// OBBtreeSplitBuildNode constructor (OBBtree.cpp:8-18).
std::unique_ptr<BuildNode> build_node(std::vector<Tri> tris, bool is_right) {
    auto nd = std::make_unique<BuildNode>();
    nd->right = is_right;
    nd->tris = std::move(tris);
    nd->box = fit_tris(nd->tris);
    if (nd->tris.size() > kLeafMax) split(*nd);
    return nd;
}

// Flat tree (OBBtree.h:61-75, 129-134): each inner node holds both child boxes
// and, per child, an inner-node index (count 0) or a triangle offset and count.
struct Node {
    Box box[2];
    uint32_t ref[2];
    uint32_t cnt[2];
};

struct Tree {
    Box root;
    std::vector<Node> nodes;
    std::vector<Tri> tris;  // leaf (DFS) order
};

// OBBtreeNode::InitializeTreeBuildNode + OBBtree::ConstructDFSrecursive
// (OBBtree.cpp:179-233, 385-394): pre-order, inner nodes appended, leaf
// triangles appended in visit order.
void flatten(BuildNode* nd, BuildNode* parent, Tree& t) {
    const int slot = nd->right ? 1 : 0;
    if (!nd->leaf) {
        nd->index = t.nodes.size();
        t.nodes.push_back(Node{});
        Node& p = t.nodes[parent->index];
        p.ref[slot] = uint32_t(nd->index);
        p.cnt[slot] = 0;
        p.box[slot] = nd->box;
    } else {
        const uint32_t off = uint32_t(t.tris.size());
        for (const Tri& tr : nd->tris) t.tris.push_back(tr);
        Node& p = t.nodes[parent->index];
        p.ref[slot] = off;
        p.cnt[slot] = uint32_t(uint16_t(nd->tris.size()));
        p.box[slot] = nd->box;
    }
    if (!nd->leaf) {
        flatten(nd->kid[0].get(), nd, t);
        flatten(nd->kid[1].get(), nd, t);
    }
}

// OBBtree::OBBtree(vector<Triangle>&&) (OBBtree.cpp:321-358).
Tree* build_tree(std::vector<Tri> tris) {
    auto* t = new Tree;
    std::vector<Tri> copy = tris;  // the reference keeps its input for the leaf-root case
    auto root = build_node(std::move(tris), false);
    t->root = root->box;
    if (!root->leaf) {
        root->index = 0;
        t->nodes.push_back(Node{});
        flatten(root->kid[0].get(), root.get(), *t);
        flatten(root->kid[1].get(), root.get(), *t);
    } else {
        t->tris = std::move(copy);
    }
    return t;
}

// --------------------------------------------------------- traversal ----
// OBBtree::OBBtreeTraveler (OBBtree.cpp:235-319): a box plus either an inner
// node or a triangle range.
struct Traveler {
    const Box* box;
    bool leaf;
    uint32_t node;
    uint32_t off, cnt;
};

inline Traveler root_traveler(const Tree& t) {
    if (!t.nodes.empty()) return Traveler{&t.root, false, 0, 0, 0};
    return Traveler{&t.root, true, 0, 0, uint32_t(t.tris.size())};
}
inline Traveler child(const Tree& t, const Traveler& tr, int s) {
    const Node& n = t.nodes[tr.node];
    if (n.cnt[s] == 0) return Traveler{&n.box[s], false, n.ref[s], 0, 0};
    return Traveler{&n.box[s], true, 0, n.ref[s], n.cnt[s]};
}

struct LeafPair {
    uint32_t off_a, cnt_a, off_b, cnt_b;
};

// OBBtree::IntersectOBBtreesRecursive (OBBtree.cpp:414-476).
void traverse(const Tree& A, const Tree& B, const Traveler& ta, const Traveler& tb, const M4& M,
              std::vector<LeafPair>& out) {
    const Box& a = *ta.box;
    const Box b = xform_box(M, *tb.box);
    if (!sat(a, b)) return;
    if (!ta.leaf && !tb.leaf) {
        if (surface(a) >= surface(b)) {
            traverse(A, B, child(A, ta, 0), tb, M, out);
            traverse(A, B, child(A, ta, 1), tb, M, out);
        } else {
            traverse(A, B, ta, child(B, tb, 0), M, out);
            traverse(A, B, ta, child(B, tb, 1), M, out);
        }
    } else if (ta.leaf && !tb.leaf) {
        traverse(A, B, ta, child(B, tb, 0), M, out);
        traverse(A, B, ta, child(B, tb, 1), M, out);
    } else if (!ta.leaf && tb.leaf) {
        traverse(A, B, child(A, ta, 0), tb, M, out);
        traverse(A, B, child(A, ta, 1), tb, M, out);
    } else {
        out.push_back(LeafPair{ta.off, ta.cnt, tb.off, tb.cnt});
    }
}

// ------------------------------------------------------ Moller 1997 ----
// Triangle/triangle test with intersection segment, restated from T. Moller,
// "A Fast Triangle-Triangle Intersection Test", JGT 2(2) 1997 (2001 revision
// with the intersection line), as the reference uses it
// (src/Geometry/Triangle.cpp:325-1003): absolute epsilon 1e-6 compared in
// double, coplanar pairs go to the 2-D edge tests.
namespace moller {

// |x| < 1e-6 evaluated as the reference does: the float promoted to double.
inline bool tiny(float x) { return double(std::fabs(x)) < 0.000001; }

inline bool edge_hits(const float* a0, const float* b0, const float* b1, float ax, float ay, int i0, int i1) {
    const float bx = b0[i0] - b1[i0];
    const float by = b0[i1] - b1[i1];
    const float cx = a0[i0] - b0[i0];
    const float cy = a0[i1] - b0[i1];
    const float f = ay * bx - ax * by;
    const float d = by * cx - bx * cy;
    if ((f > 0 && d >= 0 && d <= f) || (f < 0 && d <= 0 && d >= f)) {
        const float e = ax * cy - ay * cx;
        if (f > 0) {
            if (e >= 0 && e <= f) return true;
        } else {
            if (e <= 0 && e >= f) return true;
        }
    }
    return false;
}

inline bool edge_vs_tri(const float* a0, const float* a1, const float* u0, const float* u1, const float* u2,
                        int i0, int i1) {
    const float ax = a1[i0] - a0[i0];
    const float ay = a1[i1] - a0[i1];
    return edge_hits(a0, u0, u1, ax, ay, i0, i1) || edge_hits(a0, u1, u2, ax, ay, i0, i1) ||
           edge_hits(a0, u2, u0, ax, ay, i0, i1);
}

inline bool point_in_tri(const float* p, const float* u0, const float* u1, const float* u2, int i0, int i1) {
    float a = u1[i1] - u0[i1];
    float b = -(u1[i0] - u0[i0]);
    float c = -a * u0[i0] - b * u0[i1];
    const float d0 = a * p[i0] + b * p[i1] + c;
    a = u2[i1] - u1[i1];
    b = -(u2[i0] - u1[i0]);
    c = -a * u1[i0] - b * u1[i1];
    const float d1 = a * p[i0] + b * p[i1] + c;
    a = u0[i1] - u2[i1];
    b = -(u0[i0] - u2[i0]);
    c = -a * u2[i0] - b * u2[i1];
    const float d2 = a * p[i0] + b * p[i1] + c;
    if (d0 * d1 > 0.0f) {
        if (d0 * d2 > 0.0f) return true;
    }
    return false;
}

// coplanar_tri_tri (Triangle.cpp:460-507).
inline int coplanar(const float* n, const float* v0, const float* v1, const float* v2, const float* u0,
                    const float* u1, const float* u2) {
    const float a0 = std::fabs(n[0]), a1 = std::fabs(n[1]), a2 = std::fabs(n[2]);
    int i0, i1;
    if (a0 > a1) {
        if (a0 > a2) {
            i0 = 1;
            i1 = 2;
        } else {
            i0 = 0;
            i1 = 1;
        }
    } else {
        if (a2 > a1) {
            i0 = 0;
            i1 = 1;
        } else {
            i0 = 0;
            i1 = 2;
        }
    }
    if (edge_vs_tri(v0, v1, u0, u1, u2, i0, i1)) return 1;
    if (edge_vs_tri(v1, v2, u0, u1, u2, i0, i1)) return 1;
    if (edge_vs_tri(v2, v0, u0, u1, u2, i0, i1)) return 1;
    if (point_in_tri(v0, u0, u1, u2, i0, i1)) return 1;
    if (point_in_tri(u0, v0, v1, v2, i0, i1)) return 1;
    return 0;
}

// isect2 (Triangle.cpp:764-778): interval end points on the line and the
// corresponding points on the triangle's edges.
inline void edge_points(const float* x0, const float* x1, const float* x2, float p0, float p1, float p2, float d0,
                        float d1, float d2, float* t0, float* t1, float* q0, float* q1) {
    float s = d0 / (d0 - d1);
    *t0 = p0 + (p1 - p0) * s;
    for (int k = 0; k < 3; ++k) q0[k] = s * (x1[k] - x0[k]) + x0[k];
    s = d0 / (d0 - d2);
    *t1 = p0 + (p2 - p0) * s;
    for (int k = 0; k < 3; ++k) q1[k] = x0[k] + s * (x2[k] - x0[k]);
}

// compute_intervals_isectline (Triangle.cpp:795-830): picks the vertex alone
// on its side of the other plane. Returns 1 for "coplanar" (all distances 0).
inline int interval(const float* x0, const float* x1, const float* x2, float p0, float p1, float p2, float d0,
                    float d1, float d2, float d0d1, float d0d2, float* t0, float* t1, float* q0, float* q1) {
    if (d0d1 > 0.0f)
        edge_points(x2, x0, x1, p2, p0, p1, d2, d0, d1, t0, t1, q0, q1);
    else if (d0d2 > 0.0f)
        edge_points(x1, x0, x2, p1, p0, p2, d1, d0, d2, t0, t1, q0, q1);
    else if (d1 * d2 > 0.0f || d0 != 0.0f)
        edge_points(x0, x1, x2, p0, p1, p2, d0, d1, d2, t0, t1, q0, q1);
    else if (d1 != 0.0f)
        edge_points(x1, x0, x2, p1, p0, p2, d1, d0, d2, t0, t1, q0, q1);
    else if (d2 != 0.0f)
        edge_points(x2, x0, x1, p2, p0, p1, d2, d0, d1, t0, t1, q0, q1);
    else
        return 1;
    return 0;
}

struct Result {
    int hit;
    int coplanar;
    int fragile;  // the second interval saw all-zero distances (reference reads uninitialised values)
    float src[3], tgt[3];
};

// FP64 recheck of the six plane distances: the GPU library's CG_RECHECK /
// CG_ROBUST, which the reference does not have, restated here as its checker.
// A distance d (FP32, the reference's arithmetic) is uncertain when |d| lies
// within B = 32 u C |e1|_1 |e2|_1 of 0 or of 1e-6 (u = 2^-24, e1, e2 the
// plane triangle's edges, C the largest coordinate magnitude of its first
// corner and the three tested corners); then det[e1, e2, p - a0] is computed
// in FP64 and classified (zero below 1e-6, else by sign). mode 1 counts,
// mode 2 also goes on with the FP64 classes (nonzero ones as the FP64 value
// rounded to FP32).
struct Recheck {
    uint64_t checked = 0;
    int disagree = 0;
};
inline float amax3(const float* p) { return std::fmax(std::fmax(std::fabs(p[0]), std::fabs(p[1])), std::fabs(p[2])); }
inline float norm1(const float* p) { return (std::fabs(p[0]) + std::fabs(p[1])) + std::fabs(p[2]); }
inline int class32(float d) { return tiny(d) ? 0 : (d > 0.0f ? 1 : -1); }
inline int class64(double d) { return std::fabs(d) < 1e-6 ? 0 : (d > 0.0 ? 1 : -1); }
inline double orient64(const float* a0, const float* a1, const float* a2, const float* p) {
    const double e1x = double(a1[0]) - double(a0[0]), e1y = double(a1[1]) - double(a0[1]), e1z = double(a1[2]) - double(a0[2]);
    const double e2x = double(a2[0]) - double(a0[0]), e2y = double(a2[1]) - double(a0[1]), e2z = double(a2[2]) - double(a0[2]);
    const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    return (nx * (double(p[0]) - double(a0[0])) + ny * (double(p[1]) - double(a0[1]))) +
           nz * (double(p[2]) - double(a0[2]));
}
// The snap of three distances (Triangle.cpp:898-915) with the recheck.
inline void snap3(int mode, const float* a0, const float* a1, const float* a2, const float* e1, const float* e2,
                  const float* const p[3], float d[3], Recheck* rc) {
    bool unc[3] = {false, false, false};
    if (mode != 0) {
        const float C = std::fmax(std::fmax(amax3(a0), amax3(p[0])), std::fmax(amax3(p[1]), amax3(p[2])));
        const float B = (32.0f * 0x1p-24f) * C * norm1(e1) * norm1(e2);
        for (int k = 0; k < 3; ++k) {
            const float a = std::fabs(d[k]);
            unc[k] = a < B || std::fabs(a - 1e-6f) < B;
        }
        for (int k = 0; k < 3; ++k) {
            if (!unc[k]) continue;
            const double x = orient64(a0, a1, a2, p[k]);
            const int c = class64(x);
            ++rc->checked;
            if (c != class32(d[k])) rc->disagree = 1;
            if (mode == 2) d[k] = c == 0 ? 0.0f : float(x);
        }
    }
    for (int k = 0; k < 3; ++k)
        if (!(mode == 2 && unc[k]) && tiny(d[k])) d[k] = 0.0f;
}

// tri_tri_intersect_with_isectline (Triangle.cpp:866-1003) as called through
// TrianglePosition::IntersectTriangles (Triangle.cpp:85-110).
inline Result test(const float* V0, const float* V1, const float* V2, const float* U0, const float* U1,
                   const float* U2, int mode = 0, Recheck* rc = nullptr) {
    Result r{};
    Recheck scratch;
    if (!rc) rc = &scratch;
    float e1[3], e2[3], n1[3], n2[3], dd[3];
    for (int k = 0; k < 3; ++k) {
        e1[k] = V1[k] - V0[k];
        e2[k] = V2[k] - V0[k];
    }
    n1[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n1[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n1[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const float d1 = -(n1[0] * V0[0] + n1[1] * V0[1] + n1[2] * V0[2]);
    float du[3];
    du[0] = (n1[0] * U0[0] + n1[1] * U0[1] + n1[2] * U0[2]) + d1;
    du[1] = (n1[0] * U1[0] + n1[1] * U1[1] + n1[2] * U1[2]) + d1;
    du[2] = (n1[0] * U2[0] + n1[1] * U2[1] + n1[2] * U2[2]) + d1;
    {
        const float* const Up[3] = {U0, U1, U2};
        snap3(mode, V0, V1, V2, e1, e2, Up, du, rc);
    }
    const float du0 = du[0], du1 = du[1], du2 = du[2];
    const float du0du1 = du0 * du1;
    const float du0du2 = du0 * du2;
    if (du0du1 > 0.0f && du0du2 > 0.0f) return r;

    for (int k = 0; k < 3; ++k) {
        e1[k] = U1[k] - U0[k];
        e2[k] = U2[k] - U0[k];
    }
    n2[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n2[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n2[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const float d2 = -(n2[0] * U0[0] + n2[1] * U0[1] + n2[2] * U0[2]);
    float dv[3];
    dv[0] = (n2[0] * V0[0] + n2[1] * V0[1] + n2[2] * V0[2]) + d2;
    dv[1] = (n2[0] * V1[0] + n2[1] * V1[1] + n2[2] * V1[2]) + d2;
    dv[2] = (n2[0] * V2[0] + n2[1] * V2[1] + n2[2] * V2[2]) + d2;
    {
        const float* const Vp[3] = {V0, V1, V2};
        snap3(mode, U0, U1, U2, e1, e2, Vp, dv, rc);
    }
    const float dv0 = dv[0], dv1 = dv[1], dv2 = dv[2];
    const float dv0dv1 = dv0 * dv1;
    const float dv0dv2 = dv0 * dv2;
    if (dv0dv1 > 0.0f && dv0dv2 > 0.0f) return r;

    dd[0] = n1[1] * n2[2] - n1[2] * n2[1];
    dd[1] = n1[2] * n2[0] - n1[0] * n2[2];
    dd[2] = n1[0] * n2[1] - n1[1] * n2[0];
    float mx = std::fabs(dd[0]);
    int index = 0;
    const float b = std::fabs(dd[1]);
    const float c = std::fabs(dd[2]);
    if (b > mx) mx = b, index = 1;
    if (c > mx) mx = c, index = 2;

    const float vp0 = V0[index], vp1 = V1[index], vp2 = V2[index];
    const float up0 = U0[index], up1 = U1[index], up2 = U2[index];

    float is1[2], is2[2], pa1[3], pa2[3], pb1[3], pb2[3];
    r.coplanar = interval(V0, V1, V2, vp0, vp1, vp2, dv0, dv1, dv2, dv0dv1, dv0dv2, &is1[0], &is1[1], pa1, pa2);
    if (r.coplanar) {
        r.hit = coplanar(n1, V0, V1, V2, U0, U1, U2);
        return r;
    }
    if (interval(U0, U1, U2, up0, up1, up2, du0, du1, du2, du0du1, du0du2, &is2[0], &is2[1], pb1, pb2)) {
        // Both distances of U to V's plane vanished while V is not in U's
        // plane: the reference goes on with uninitialised interval values.
        // This restatement defines the outcome as "no intersection" and flags it.
        r.fragile = 1;
        return r;
    }

    int smallest1, smallest2;
    if (is1[0] > is1[1]) {
        std::swap(is1[0], is1[1]);
        smallest1 = 1;
    } else {
        smallest1 = 0;
    }
    if (is2[0] > is2[1]) {
        std::swap(is2[0], is2[1]);
        smallest2 = 1;
    } else {
        smallest2 = 0;
    }
    if (is1[1] < is2[0] || is2[1] < is1[0]) return r;

    r.hit = 1;
    const float *s, *t;
    if (is2[0] < is1[0]) {
        s = smallest1 == 0 ? pa1 : pa2;
        if (is2[1] < is1[1])
            t = smallest2 == 0 ? pb2 : pb1;
        else
            t = smallest1 == 0 ? pa2 : pa1;
    } else {
        s = smallest2 == 0 ? pb1 : pb2;
        if (is2[1] > is1[1])
            t = smallest1 == 0 ? pa2 : pa1;
        else
            t = smallest2 == 0 ? pb2 : pb1;
    }
    for (int k = 0; k < 3; ++k) {
        r.src[k] = s[k];
        r.tgt[k] = t[k];
    }
    return r;
}

}  // namespace moller

// ------------------------------------------------------- narrow phase ----
struct Hit {
    uint32_t ia, ib;
    float src[3], tgt[3];
};

// TrianglePosition::MultiplyBy4x4Matrix (Triangle.cpp:69-78).
inline void xform_tri(const M4& M, const Tri& t, V3 out[3]) {
    for (int k = 0; k < 3; ++k) out[k] = xform(M, t.p[k], 1.0f);
}

// Per-triangle contact record (CreateUncollideRays.cpp:14-58,
// TriangleCandidateRays): 3-bit "vertex not outside the other triangle's
// plane" mask, length-weighted sum of segment midpoints, total weight.
struct Contact {
    uint8_t mask = 7;
    V3 wsum{0.f, 0.f, 0.f};
    float weight = 0.f;
};

// Plane::Plane + CreatePlaneFromTriangle + IntersectPoint
// (src/Geometry/Plane.cpp:5-28); true when the point is OUTSIDE (s > 0).
struct Plane {
    V3 n;
    float d;
};
inline Plane plane_of(const V3 p[3]) {
    V3 fn = face_normal(p);
    float d = -dot(p[0], fn);
    float len = length(fn);
    return Plane{divs(fn, len), d / len};
}
inline bool outside(const Plane& pl, V3 p) { return dot(p, pl.n) + pl.d > 0; }

struct Narrow {
    std::vector<Hit> hits;
    uint64_t tests = 0;
    std::unordered_map<uint32_t, Contact> ca, cb;
    uint64_t fragile = 0;
    int recheck_mode = 0;         // moller::snap3's mode for every test
    uint64_t rechecked = 0;       // distances recomputed in FP64
    uint64_t disagreements = 0;   // tests where one changed class
};

// The pair loop of CreateUncollideRays::ExecuteCreateUncollideRays
// (CreateUncollideRays.cpp:74-127): every (i, j) of every candidate leaf
// pair, B's triangle re-transformed per pair; colliding = hit and not
// coplanar; contacts accumulated per leaf pair, then merged per triangle in
// leaf-pair order.
void narrow(const Tree& A, const Tree& B, const M4& M, const std::vector<LeafPair>& lps, Narrow& out,
            bool keep_hits, bool contacts) {
    for (const LeafPair& lp : lps) {
        Contact la[kLeafMax], lb[kLeafMax];
        for (uint32_t i = 0; i != lp.cnt_a; ++i) {
            for (uint32_t j = 0; j != lp.cnt_b; ++j) {
                const Tri& ta = A.tris[lp.off_a + i];
                V3 pb[3];
                xform_tri(M, B.tris[lp.off_b + j], pb);
                moller::Recheck rc;
                moller::Result r = moller::test(&ta.p[0].x, &ta.p[1].x, &ta.p[2].x, &pb[0].x, &pb[1].x, &pb[2].x,
                                                out.recheck_mode, &rc);
                ++out.tests;
                out.fragile += uint64_t(r.fragile);
                out.rechecked += rc.checked;
                out.disagreements += uint64_t(rc.disagree);
                if (!(r.hit && !r.coplanar)) continue;
                if (keep_hits) {
                    Hit h;
                    h.ia = lp.off_a + i;
                    h.ib = lp.off_b + j;
                    std::memcpy(h.src, r.src, sizeof(h.src));
                    std::memcpy(h.tgt, r.tgt, sizeof(h.tgt));
                    out.hits.push_back(h);
                }
                if (!contacts) continue;
                const Plane pla = plane_of(ta.p);
                const Plane plb = plane_of(pb);
                const V3 s = v3(r.src[0], r.src[1], r.src[2]);
                const V3 t = v3(r.tgt[0], r.tgt[1], r.tgt[2]);
                const float w = length(sub(s, t));
                const V3 mid = divs(scale(w, add(s, t)), 2.0f);
                la[i].wsum = add(la[i].wsum, mid);
                la[i].weight = la[i].weight + w;
                lb[j].wsum = add(lb[j].wsum, mid);
                lb[j].weight = lb[j].weight + w;
                for (int k = 0; k < 3; ++k) {
                    if (outside(plb, ta.p[k])) la[i].mask &= uint8_t(~(1u << k));
                    if (outside(pla, pb[k])) lb[j].mask &= uint8_t(~(1u << k));
                }
            }
        }
        if (!contacts) continue;
        auto merge = [](std::unordered_map<uint32_t, Contact>& m, uint32_t key, const Contact& c) {
            auto ins = m.emplace(key, c);
            if (!ins.second) {
                Contact& e = ins.first->second;
                e.mask &= c.mask;
                e.wsum = add(e.wsum, c.wsum);
                e.weight = e.weight + c.weight;
            }
        };
        for (uint32_t i = 0; i != lp.cnt_a; ++i)
            if (!(la[i].weight == 0.f)) merge(out.ca, lp.off_a + i, la[i]);
        for (uint32_t j = 0; j != lp.cnt_b; ++j)
            if (!(lb[j].weight == 0.f)) merge(out.cb, lp.off_b + j, lb[j]);
    }
}

struct Ray {
    V3 o, d;
};

// TrianglePosition::GetBarycentricOfPoint (Triangle.cpp:148-163).
inline void barycentric(const V3 p[3], V3 q, float& bx, float& by) {
    V3 v0 = sub(p[1], p[0]), v1 = sub(p[2], p[0]), v2 = sub(q, p[0]);
    float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    float den = d00 * d11 - d01 * d01;
    bx = (d11 * d20 - d01 * d21) / den;
    by = (d00 * d21 - d01 * d20) / den;
}

// find_rays_lambda of CreateUncollideRays.cpp:131-178: one ray per vertex
// "not outside" (deduplicated by vertex index), else one ray from the
// weighted contact average with the barycentric-interpolated normal; the
// second object's rays are moved into the first object's space.
std::vector<Ray> make_rays(const std::unordered_map<uint32_t, Contact>& cs, const Tree& T, bool second, const M4& M,
                           const M3& N) {
    std::vector<Ray> rays;
    std::unordered_set<uint32_t> seen;
    for (const auto& kv : cs) {
        const Tri& tr = T.tris[kv.first];
        V3 pos[3];
        if (second)
            xform_tri(M, tr, pos);
        else
            for (int k = 0; k < 3; ++k) pos[k] = tr.p[k];
        if (kv.second.mask != 0) {
            for (int k = 0; k < 3; ++k) {
                if (!(kv.second.mask & (1u << k))) continue;
                if (!seen.insert(tr.i[k]).second) continue;
                V3 nrm = second ? normalize(mul3(N, tr.n[k])) : normalize(tr.n[k]);
                rays.push_back(Ray{pos[k], neg(nrm)});
            }
        } else {
            V3 q = divs(kv.second.wsum, kv.second.weight);
            float bx, by;
            barycentric(pos, q, bx, by);
            float b0 = 1.f - bx - by;
            V3 n = add(add(scale(b0, tr.n[0]), scale(bx, tr.n[1])), scale(by, tr.n[2]));
            V3 nrm = second ? normalize(mul3(N, n)) : normalize(n);
            rays.push_back(Ray{q, neg(nrm)});
        }
    }
    return rays;
}

inline V3 mean_origin(const std::vector<Ray>& rays) {
    V3 s{0.f, 0.f, 0.f};
    for (const Ray& r : rays) s = add(s, r.o);
    return divs(s, float(rays.size()));
}

// Whole query as the engine runs it (CollisionDetection.cpp:49-67) with the
// relative matrix computed as OBBtreesCollision.cpp:15 does.
struct Query {
    std::vector<LeafPair> lps;
    Narrow nr;
    std::vector<Ray> ra, rb;
    V3 avg_a{}, avg_b{};
};

inline M4 relative(const M4& a, const M4& b) { return mul(inverse(a), b); }

void run_query(const Tree& A, const Tree& B, const M4& ma, const M4& mb, Query& q, bool keep_hits, bool rays,
               int recheck_mode = 0) {
    const M4 M = relative(ma, mb);
    q.nr.recheck_mode = recheck_mode;
    q.lps.clear();
    traverse(A, B, root_traveler(A), root_traveler(B), M, q.lps);
    if (q.lps.empty()) return;
    narrow(A, B, M, q.lps, q.nr, keep_hits, rays);
    if (!rays) return;
    const M3 N = cofactor3(M);
    q.ra = make_rays(q.nr.ca, A, false, M, N);
    q.avg_a = mean_origin(q.ra);
    q.rb = make_rays(q.nr.cb, B, true, M, N);
    V3 avg = mean_origin(q.rb);
    q.avg_b = xform(inverse(M), avg, 1.0f);
}

// ------------------------------------------------------ ray shooting ----
// Ray::IntersectParalgram (Ray.cpp:36-133): Haines' slab test against the
// box's three face-plane pairs, the ray starting at the origin (the tree is
// moved so, Ray.cpp:150-157).
struct Slab {
    bool hit;
    float tmin, tmax;
};
inline Slab ray_box(const Box& b, V3 dir) {
    float mn = -std::numeric_limits<float>::infinity();
    float mx = std::numeric_limits<float>::infinity();
    const V3 ro = sub(V3{0.f, 0.f, 0.f}, b.c);
    const V3 fa[3] = {b.v, b.w, b.u}, fb[3] = {b.w, b.u, b.v}, side[3] = {b.u, b.v, b.w};
    for (int k = 0; k < 3; ++k) {
        const V3 pd = normalize(cross(fa[k], fb[k]));
        const float d = -std::fabs(dot(pd, side[k]));
        const float pc = dot(pd, ro);
        const float n1 = pc + d;
        const float n2 = -pc + d;
        const float vd = dot(pd, dir);
        if (std::fabs(vd) >= std::numeric_limits<float>::epsilon()) {
            const float inv = 1.f / vd;
            float t1 = -n1 * inv;
            float t2 = n2 * inv;
            if (t1 > t2) std::swap(t1, t2);
            mn = (t1 < mn) ? mn : t1;  // std::max(t1, mn)
            mx = (mx < t2) ? mx : t2;  // std::min(t2, mx)
            if (mn > mx || mx < 0.f) return Slab{false, 0.f, 0.f};
        } else if (n1 > 0 || n2 > 0) {
            return Slab{false, 0.f, 0.f};
        }
    }
    return Slab{true, mn, mx};
}

// The ray/triangle test the reference calls through its glm fork
// (Ray.cpp:22-33), as the glm shim states it: Moller-Trumbore, two-sided,
// reporting a back-face hit (a negative determinant).
inline bool ray_tri(V3 orig, V3 dir, V3 v0, V3 v1, V3 v2, float& bx, float& by, float& t, bool& back) {
    const V3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    const V3 p = cross(dir, e2);
    const float det = dot(e1, p);
    back = det < 0.f;
    if (std::fabs(det) <= std::numeric_limits<float>::epsilon()) return false;
    const float inv = 1.f / det;
    const V3 s0 = sub(orig, v0);
    const float u = dot(s0, p) * inv;
    if (u < 0.f || u > 1.f) return false;
    const V3 q = cross(s0, e1);
    const float v = dot(dir, q) * inv;
    if (v < 0.f || u + v > 1.f) return false;
    const float tt = dot(e2, q) * inv;
    if (tt < 0.f) return false;
    bx = u;
    by = v;
    t = tt;
    return true;
}

// RayOBBtreeIntersectInfo (Ray.h:17-24).
struct TreeHit {
    bool hit = false, back = false;
    float dist = std::numeric_limits<float>::infinity();
    uint32_t tri = ~0u;
    float bx = 0.f, by = 0.f;
};

// Ray::IntersectOBBtreeRecursive (Ray.cpp:161-237): both children's slabs,
// the nearer entry first (ties: the right child first), a child visited when
// its entry is before the best hit so far and its exit not behind the ray.
void ray_tree_rec(const Tree& T, const Traveler& tr, const M4& cm, V3 dir, TreeHit& best) {
    if (!tr.leaf) {
        const Traveler L = child(T, tr, 0), R = child(T, tr, 1);
        const Slab hl = ray_box(xform_box(cm, *L.box), dir);
        const Slab hr = ray_box(xform_box(cm, *R.box), dir);
        auto visit = [&](const Traveler& c, const Slab& h) {
            if (h.tmin < best.dist && h.tmax >= 0.f) ray_tree_rec(T, c, cm, dir, best);
        };
        if (hl.hit && hr.hit) {
            if (hl.tmin < hr.tmin) {
                visit(L, hl);
                visit(R, hr);
            } else {
                visit(R, hr);
                visit(L, hl);
            }
        } else if (hl.hit) {
            visit(L, hl);
        } else if (hr.hit) {
            visit(R, hr);
        }
        return;
    }
    for (uint32_t i = tr.off; i != tr.off + tr.cnt; ++i) {
        V3 p[3];
        xform_tri(cm, T.tris[i], p);
        float bx = 0.f, by = 0.f, t = 0.f;
        bool back = false;
        const bool hit = ray_tri(V3{0.f, 0.f, 0.f}, dir, p[0], p[1], p[2], bx, by, t, back);
        if (hit && t > 0.f && t < best.dist) {
            best.hit = true;
            best.back = back;
            best.dist = t;
            best.tri = i;
            best.bx = bx;
            best.by = by;
        }
    }
}

// Ray::IntersectOBBtree (Ray.cpp:135-159): the tree moved so that the ray
// starts at the origin, then the root's slab.
TreeHit ray_tree(const Tree& T, const M4& matrix, V3 origin, V3 dir) {
    M4 cm = matrix;
    if (!(origin.x == 0.f && origin.y == 0.f && origin.z == 0.f)) {
        cm.m[12] = matrix.m[12] - origin.x;
        cm.m[13] = matrix.m[13] - origin.y;
        cm.m[14] = matrix.m[14] - origin.z;
        cm.m[15] = matrix.m[15] - 0.f;
    }
    TreeHit best;
    const Traveler root = root_traveler(T);
    const Slab h = ray_box(xform_box(cm, *root.box), dir);
    if (h.hit && h.tmax >= 0.f) ray_tree_rec(T, root, cm, dir, best);
    return best;
}

inline M4 identity4() {
    M4 m{};
    m.m[0] = m.m[5] = m.m[10] = m.m[15] = 1.f;
    return m;
}
inline M3 identity3() {
    M3 m{};
    m.m[0] = m.m[4] = m.m[8] = 1.f;
    return m;
}

// ShootUncollideRays::HermannPass (ShootUncollideRays.cpp:127-158).
struct Hermann {
    bool ok = false;
    V3 response{}, normal{};
};
Hermann hermann_pass(const Tree& A, const Tree& B, const M4& ma, const M4& mb, const M3& nb, const Ray& ray) {
    Hermann r;
    const TreeHit p2 = ray_tree(B, mb, ray.o, ray.d);
    if (!(p2.hit && p2.back)) return r;
    // Ray::MoveOriginEpsilonTowardsDirection(4) (Ray.cpp:13-20)
    const float big = std::max({std::fabs(ray.o.x), std::fabs(ray.o.y), std::fabs(ray.o.z)});
    const float eps = big * std::numeric_limits<float>::epsilon();
    const V3 moved = add(ray.o, scale(4.f * eps, ray.d));
    const float eps_dist = length(sub(moved, ray.o));
    const TreeHit p3 = ray_tree(A, ma, moved, ray.d);
    if (p2.dist <= p3.dist + eps_dist) {
        r.ok = true;
        r.response = scale(p2.dist, ray.d);
        // TriangleNormal::GetNormal(bary, matrix) (Triangle.cpp:197-204)
        const Tri& tr = B.tris[p2.tri];
        const float b0 = (1.f - p2.bx) - p2.by;
        const V3 n = add(add(scale(b0, tr.n[0]), scale(p2.bx, tr.n[1])), scale(p2.by, tr.n[2]));
        r.normal = normalize(mul3(nb, n));
    }
    return r;
}

// ShootUncollideRays::CalcForceResponse (ShootUncollideRays.cpp:116-125).
inline V3 force_response(const Hermann& h) {
    const V3 dir = normalize(h.response);
    const float len = length(h.response);
    const float c = dot(h.normal, dir);
    return scale(c * c * len, dir);
}

// ShootUncollideRays::SmootherStep (ShootUncollideRays.cpp:175-179).
inline float smoother_step(float a, float b, float x) {
    float v = (x - a) / (b - a);
    v = (v < 0.f) ? 0.f : ((1.f < v) ? 1.f : v);  // std::clamp(v, 0, 1)
    return v * v * v * (v * (v * 6 - 15) + 10);
}

struct ShootParams {
    float cos_start, cos_finish, bias;
};

// ShootUncollideRays::ExecuteShootUncollideRays (ShootUncollideRays.cpp:14-98)
// with FindResponse (:160-173): the world-space delta for the first entity.
V3 shoot(const Tree& A, const Tree& B, const M4& ga, const M4& gb, const std::vector<Ray>& rays_a,
         const std::vector<Ray>& rays_b, const ShootParams& P) {
    const M4 M = relative(ga, gb);
    const M3 N = cofactor3(M);
    const M4 I = identity4();
    const M3 I3 = identity3();
    V3 avg{0.f, 0.f, 0.f};
    std::vector<V3> responses;
    auto reflect = [](const Hermann& h, const Ray& ray) { return Ray{add(ray.o, h.response), neg(h.normal)}; };
    auto first_to_second = [&](const Ray& ray, Ray& out) {
        const Hermann h = hermann_pass(A, B, I, M, N, ray);
        if (!h.ok) return false;
        avg = sub(avg, force_response(h));
        responses.push_back(neg(h.response));
        out = reflect(h, ray);
        return true;
    };
    auto second_to_first = [&](const Ray& ray, Ray& out) {
        const Hermann h = hermann_pass(B, A, M, I, I3, ray);
        if (!h.ok) return false;
        avg = add(avg, force_response(h));
        responses.push_back(h.response);
        out = reflect(h, ray);
        return true;
    };
    Ray r1, r2;
    for (const Ray& ray : rays_a)
        if (first_to_second(ray, r1)) second_to_first(r1, r2);
    for (const Ray& ray : rays_b)
        if (second_to_first(ray, r1)) first_to_second(r1, r2);
    if (avg.x == 0.f && avg.y == 0.f && avg.z == 0.f) return V3{0.f, 0.f, 0.f};
    const V3 nf = normalize(avg);
    float max_len = 0.f;
    for (const V3& r : responses) {
        const V3 nr = normalize(r);
        const float dt = dot(nr, nf);
        const float len = length(r);
        const float need = len / dt;
        const float sm = smoother_step(P.cos_finish, P.cos_start, dt);
        const float x = sm * need;
        max_len = (max_len < x) ? x : max_len;  // std::max(max_len, x)
    }
    const V3 local = scale(P.bias, scale(max_len, nf));
    return xform(ga, local, 0.f);
}

// ------------------------------------------------------- broad phase ----
// The engine's three skewed axes (CollisionDetection.cpp:9-13).
inline void engine_axes(V3& U, V3& V, V3& W) {
    U = normalize(V3{0.8f, -0.2f, 0.f});
    W = normalize(cross(U, V3{0.f, -1.f, 0.f}));
    V = normalize(cross(W, U));
}

// SweepAndPrune::ExecuteSweepAndPrune (SweepAndPrune.cpp:15-88): each
// entity's world root box projected on U, V, W; per axis sorted by the
// projection's start and swept with an active list (an entry leaves when its
// end is before the new start); a pair found on U (at least one entity with a
// callback) is kept when V and W find it too. Pairs as (the entity earlier on
// U, the later one).
std::vector<std::pair<uint32_t, uint32_t>> sweep_and_prune(const std::vector<const Tree*>& trees,
                                                           const std::vector<M4>& globals,
                                                           const std::vector<uint8_t>& callback, V3 U, V3 V,
                                                           V3 W) {
    struct Entry {
        float lo, hi;
        uint32_t index;
        bool cb;
    };
    const size_t n = trees.size();
    std::vector<Entry> axis_entries[3];
    const V3 axes[3] = {U, V, W};
    for (size_t i = 0; i < n; ++i) {
        const Box b = xform_box(globals[i], trees[i]->root);
        for (int a = 0; a < 3; ++a) {
            Entry e{0.f, 0.f, uint32_t(i), callback[i] != 0};
            project(b, axes[a], e.lo, e.hi);
            axis_entries[a].push_back(e);
        }
    }
    for (auto& v : axis_entries)
        std::sort(v.begin(), v.end(), [](const Entry& a, const Entry& b) { return a.lo < b.lo; });
    struct Found {
        uint32_t first, second, count;
    };
    std::unordered_map<uint64_t, Found> found;  // keyed by the unordered pair
    auto key = [](uint32_t a, uint32_t b) { return (uint64_t(std::min(a, b)) << 32) | std::max(a, b); };
    for (int a = 0; a < 3; ++a) {
        std::vector<Entry> active;
        for (const Entry& e : axis_entries[a]) {
            std::vector<Entry> kept;
            for (const Entry& act : active) {
                if (act.hi < e.lo) continue;  // leaves the active list
                kept.push_back(act);
                if (!(act.cb || e.cb)) continue;
                if (a == 0) {
                    found.emplace(key(act.index, e.index), Found{act.index, e.index, 1});
                } else {
                    auto it = found.find(key(act.index, e.index));
                    if (it != found.end()) ++it->second.count;
                }
            }
            kept.push_back(e);
            active.swap(kept);
        }
    }
    std::vector<std::pair<uint32_t, uint32_t>> out;
    for (const auto& kv : found)
        if (kv.second.count == 3) out.emplace_back(kv.second.first, kv.second.second);
    return out;
}

}  // namespace port

// ================================================================ C ABI ====
using namespace port;

namespace {
V3 ld3(const float* p) { return V3{p[0], p[1], p[2]}; }
void st3(V3 v, float* p) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
Box ldbox(const float* b) { return Box{ld3(b), ld3(b + 3), ld3(b + 6), ld3(b + 9)}; }
void stbox(const Box& b, float* o) {
    st3(b.c, o);
    st3(b.u, o + 3);
    st3(b.v, o + 6);
    st3(b.w, o + 9);
}
M4 ldm(const float* m) {
    M4 r;
    std::memcpy(r.m, m, sizeof(r.m));
    return r;
}
}  // namespace

extern "C" {

// Triangle::CreateTriangleList for glTF "triangles" (Triangle.cpp:11-62,
// 214-234, 242-280): positions and indices by triplet, vertex normals when
// given, else the face normal on all three corners.
void* port_tree_build(const float* points, size_t n_points, const float* normals, const uint32_t* indices,
                      size_t n_indices) {
    (void)n_points;
    std::vector<Tri> tris(n_indices / 3);
    for (size_t t = 0; t < tris.size(); ++t) {
        Tri& tr = tris[t];
        for (int k = 0; k < 3; ++k) {
            const uint32_t vi = indices[3 * t + k];
            tr.p[k] = ld3(points + 3 * size_t(vi));
            tr.i[k] = vi;
        }
        if (normals) {
            for (int k = 0; k < 3; ++k) tr.n[k] = ld3(normals + 3 * size_t(indices[3 * t + k]));
        } else {
            V3 fn = face_normal(tr.p);
            tr.n[0] = tr.n[1] = tr.n[2] = fn;
        }
    }
    return build_tree(std::move(tris));
}

// Rebuilds a tree from its flat export (the layout of ref_tree_export).
void* port_tree_import(const float* root12, size_t n_nodes, const float* node_obbs, const uint32_t* node_ref,
                       const uint32_t* node_cnt, size_t n_tris, const float* tri_pos, const float* tri_nrm,
                       const uint32_t* tri_idx) {
    auto* t = new Tree;
    t->root = ldbox(root12);
    t->nodes.resize(n_nodes);
    for (size_t k = 0; k < n_nodes; ++k)
        for (int s = 0; s < 2; ++s) {
            t->nodes[k].box[s] = ldbox(node_obbs + (2 * k + s) * 12);
            t->nodes[k].ref[s] = node_ref[2 * k + s];
            t->nodes[k].cnt[s] = node_cnt[2 * k + s];
        }
    t->tris.resize(n_tris);
    for (size_t i = 0; i < n_tris; ++i)
        for (int k = 0; k < 3; ++k) {
            t->tris[i].p[k] = ld3(tri_pos + 9 * i + 3 * k);
            t->tris[i].n[k] = tri_nrm ? ld3(tri_nrm + 9 * i + 3 * k) : V3{0, 0, 0};
            t->tris[i].i[k] = tri_idx ? tri_idx[3 * i + k] : uint32_t(3 * i + k);
        }
    return t;
}

void port_tree_free(void* t) { delete static_cast<Tree*>(t); }

void port_tree_sizes(void* tp, size_t* n_nodes, size_t* n_tris) {
    const Tree* t = static_cast<const Tree*>(tp);
    *n_nodes = t->nodes.size();
    *n_tris = t->tris.size();
}

void port_tree_export(void* tp, float* root12, float* node_obbs, uint32_t* node_ref, uint32_t* node_cnt,
                      float* tri_pos, float* tri_nrm, uint32_t* tri_idx) {
    const Tree* t = static_cast<const Tree*>(tp);
    stbox(t->root, root12);
    for (size_t k = 0; k < t->nodes.size(); ++k)
        for (int s = 0; s < 2; ++s) {
            stbox(t->nodes[k].box[s], node_obbs + (2 * k + s) * 12);
            node_ref[2 * k + s] = t->nodes[k].ref[s];
            node_cnt[2 * k + s] = t->nodes[k].cnt[s];
        }
    for (size_t i = 0; i < t->tris.size(); ++i)
        for (int k = 0; k < 3; ++k) {
            st3(t->tris[i].p[k], tri_pos + 9 * i + 3 * k);
            st3(t->tris[i].n[k], tri_nrm + 9 * i + 3 * k);
            tri_idx[3 * i + k] = t->tris[i].i[k];
        }
}

void port_relative_matrix(const float* a16, const float* b16, float* out16) {
    M4 r = relative(ldm(a16), ldm(b16));
    std::memcpy(out16, r.m, sizeof(r.m));
}

struct MidHandle {
    Query q;
    const Tree* A;
    const Tree* B;
    M4 M;
};
static MidHandle* as_mid(void* r) { return static_cast<MidHandle*>(r); }

void* port_mid_phase(void* ta, void* tb, const float* a16, const float* b16) {
    auto* h = new MidHandle;
    h->A = static_cast<const Tree*>(ta);
    h->B = static_cast<const Tree*>(tb);
    h->M = relative(ldm(a16), ldm(b16));
    traverse(*h->A, *h->B, root_traveler(*h->A), root_traveler(*h->B), h->M, h->q.lps);
    return h;
}

void port_mid_free(void* r) { delete as_mid(r); }

size_t port_mid_count(void* r) { return as_mid(r)->q.lps.size(); }

void port_mid_get(void* r, uint32_t* out) {
    const auto& v = as_mid(r)->q.lps;
    for (size_t i = 0; i < v.size(); ++i) {
        out[4 * i + 0] = v[i].off_a;
        out[4 * i + 1] = v[i].cnt_a;
        out[4 * i + 2] = v[i].off_b;
        out[4 * i + 3] = v[i].cnt_b;
    }
}

size_t port_narrow(void* r, uint32_t* pair_out, float* seg_out, size_t cap, uint64_t* tests, uint64_t* fragile) {
    auto* h = as_mid(r);
    Narrow nr;
    narrow(*h->A, *h->B, h->M, h->q.lps, nr, true, false);
    for (size_t k = 0; k < nr.hits.size() && k < cap; ++k) {
        pair_out[2 * k] = nr.hits[k].ia;
        pair_out[2 * k + 1] = nr.hits[k].ib;
        std::memcpy(seg_out + 6 * k, nr.hits[k].src, 3 * sizeof(float));
        std::memcpy(seg_out + 6 * k + 3, nr.hits[k].tgt, 3 * sizeof(float));
    }
    if (tests) *tests = nr.tests;
    if (fragile) *fragile = nr.fragile;
    return nr.hits.size();
}

// Per-triangle contact records (the TriangleCandidateRays map contents) of
// side 0 (first tree) or 1 (second tree), sorted by triangle index:
// out_idx[n], out_mask[n], out_f[n][4] = weighted sum xyz, weight.
size_t port_contacts(void* r, int side, uint32_t* out_idx, uint32_t* out_mask, float* out_f, size_t cap) {
    auto* h = as_mid(r);
    Narrow nr;
    narrow(*h->A, *h->B, h->M, h->q.lps, nr, false, true);
    const auto& m = side == 0 ? nr.ca : nr.cb;
    std::vector<uint32_t> keys;
    for (const auto& kv : m) keys.push_back(kv.first);
    std::sort(keys.begin(), keys.end());
    for (size_t k = 0; k < keys.size() && k < cap; ++k) {
        const Contact& c = m.at(keys[k]);
        out_idx[k] = keys[k];
        out_mask[k] = c.mask;
        out_f[4 * k + 0] = c.wsum.x;
        out_f[4 * k + 1] = c.wsum.y;
        out_f[4 * k + 2] = c.wsum.z;
        out_f[4 * k + 3] = c.weight;
    }
    return keys.size();
}

// The same records in the map's own iteration order (the order of the rays
// that find_rays_lambda makes from it, CreateUncollideRays.cpp:138).
size_t port_contacts_iter(void* r, int side, uint32_t* out_idx, uint32_t* out_mask, float* out_f, size_t cap) {
    auto* h = as_mid(r);
    Narrow nr;
    narrow(*h->A, *h->B, h->M, h->q.lps, nr, false, true);
    const auto& m = side == 0 ? nr.ca : nr.cb;
    size_t k = 0;
    for (const auto& kv : m) {
        if (k < cap) {
            out_idx[k] = kv.first;
            out_mask[k] = kv.second.mask;
            out_f[4 * k + 0] = kv.second.wsum.x;
            out_f[4 * k + 1] = kv.second.wsum.y;
            out_f[4 * k + 2] = kv.second.wsum.z;
            out_f[4 * k + 3] = kv.second.weight;
        }
        ++k;
    }
    return m.size();
}

void port_rays(void* r, float* rays_a, float* rays_b, size_t cap_a, size_t cap_b, size_t* counts, float* avg) {
    auto* h = as_mid(r);
    const Tree& A = *h->A;
    const Tree& B = *h->B;
    const M4& M = h->M;
    Narrow nr;
    narrow(A, B, M, h->q.lps, nr, false, true);
    const M3 N = cofactor3(M);
    const std::vector<Ray> ra = make_rays(nr.ca, A, false, M, N);
    const std::vector<Ray> rb = make_rays(nr.cb, B, true, M, N);
    const V3 avg_a = mean_origin(ra);
    const V3 avg_b = xform(inverse(M), mean_origin(rb), 1.0f);
    counts[0] = ra.size();
    counts[1] = rb.size();
    for (size_t k = 0; k < ra.size() && k < cap_a; ++k) {
        st3(ra[k].o, rays_a + 6 * k);
        st3(ra[k].d, rays_a + 6 * k + 3);
    }
    for (size_t k = 0; k < rb.size() && k < cap_b; ++k) {
        st3(rb[k].o, rays_b + 6 * k);
        st3(rb[k].d, rays_b + 6 * k + 3);
    }
    if (avg) {
        st3(avg_a, avg);
        st3(avg_b, avg + 3);
    }
}

int port_tri_tri(const float* a9, const float* b9, int* coplanar, float* src3, float* tgt3) {
    moller::Result r = moller::test(a9, a9 + 3, a9 + 6, b9, b9 + 3, b9 + 6);
    *coplanar = r.coplanar;
    if (r.hit && !r.coplanar) {
        std::memcpy(src3, r.src, sizeof(r.src));
        std::memcpy(tgt3, r.tgt, sizeof(r.tgt));
    }
    return r.hit;
}

// Same as port_tri_tri, also reporting the "fragile" flag.
// One test with the FP64 recheck (mode 1 counted, 2 FP64 verdict); checks[0]
// distances recomputed, checks[1] 1 when one of them changed class.
int port_tri_tri_recheck(const float* a9, const float* b9, int mode, int* coplanar, int* fragile, uint32_t* checks,
                         float* src3, float* tgt3) {
    moller::Recheck rc;
    moller::Result r = moller::test(a9, a9 + 3, a9 + 6, b9, b9 + 3, b9 + 6, mode, &rc);
    *coplanar = r.coplanar;
    *fragile = r.fragile;
    checks[0] = uint32_t(rc.checked);
    checks[1] = uint32_t(rc.disagree);
    if (r.hit && !r.coplanar) {
        std::memcpy(src3, r.src, sizeof(r.src));
        std::memcpy(tgt3, r.tgt, sizeof(r.tgt));
    }
    return r.hit;
}

int port_tri_tri_ex(const float* a9, const float* b9, int* coplanar, int* fragile, float* src3, float* tgt3) {
    moller::Result r = moller::test(a9, a9 + 3, a9 + 6, b9, b9 + 3, b9 + 6);
    *coplanar = r.coplanar;
    *fragile = r.fragile;
    if (r.hit && !r.coplanar) {
        std::memcpy(src3, r.src, sizeof(r.src));
        std::memcpy(tgt3, r.tgt, sizeof(r.tgt));
    }
    return r.hit;
}

void port_transform_tri(const float* m16, const float* a9, float* out9) {
    M4 M = ldm(m16);
    for (int k = 0; k < 3; ++k) st3(xform(M, ld3(a9 + 3 * k), 1.0f), out9 + 3 * k);
}

int port_sat(const float* a12, const float* b12) { return sat(ldbox(a12), ldbox(b12)) ? 1 : 0; }

float port_surface(const float* a12) { return surface(ldbox(a12)); }

void port_transform_box(const float* m16, const float* a12, float* out12) {
    stbox(xform_box(ldm(m16), ldbox(a12)), out12);
}

void port_obb_from_points(const float* pts, size_t n, float* out12) {
    std::vector<V3> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = ld3(pts + 3 * i);
    stbox(fit_box(v), out12);
}

void port_eig3(const double* a9, double* v9, double* d3) {
    double a[3][3], v[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = a9[3 * i + j];
    eigen_sym3(a, v, d3);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) v9[3 * i + j] = v[i][j];
}

// The engine's per-pair mid + narrow phases over a batch of queries (the CPU
// baseline), split over `threads` host threads by query. Returns the number of
// triangle-pair tests; *n_hits receives the number of colliding pairs and
// *n_rays the number of uncollide rays.
uint64_t port_collide_batch(void* const* trees_a, void* const* trees_b, const float* mats_a, const float* mats_b,
                            size_t n, int threads, uint64_t* n_hits, uint64_t* n_rays, const uint64_t* order) {
    threads = std::max(1, threads);
    std::vector<uint64_t> tests(threads, 0), hits(threads, 0), rays(threads, 0);
    // Each thread takes the next query of `order` (the caller's: largest
    // first) from a shared counter (costs differ by orders of magnitude: a
    // fixed split leaves threads idle).
    std::atomic<size_t> next{0};
    auto work = [&](int tid) {
        for (size_t k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
            const size_t q = order ? size_t(order[k]) : k;
            Query qr;
            run_query(*static_cast<const Tree*>(trees_a[q]), *static_cast<const Tree*>(trees_b[q]),
                      ldm(mats_a + 16 * q), ldm(mats_b + 16 * q), qr, true, true);
            tests[tid] += qr.nr.tests;
            hits[tid] += qr.nr.hits.size();
            rays[tid] += qr.ra.size() + qr.rb.size();
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
    uint64_t tt = 0, th = 0, tr = 0;
    for (int t = 0; t < threads; ++t) {
        tt += tests[t];
        th += hits[t];
        tr += rays[t];
    }
    if (n_hits) *n_hits = th;
    if (n_rays) *n_rays = tr;
    return tt;
}

// Colliding pairs of a batch of queries: for query q, pairs are written to
// pair_out[...] as (query, ia, ib) with segments; returns total count (writes
// at most cap). Used as the parity oracle for batched GPU runs.
// The colliding pairs of a batch with the FP64 recheck in mode `mode` (0 off,
// 1 counted, 2 FP64 verdict; moller::snap3), its counts in recheck[2].
size_t port_collide_pairs_mode(void* const* trees_a, void* const* trees_b, const float* mats_a, const float* mats_b,
                               size_t n, uint32_t* pair_out, float* seg_out, size_t cap, uint64_t* tests_out,
                               uint64_t* leafpairs_out, int mode, uint64_t* recheck) {
    size_t total = 0;
    uint64_t tests = 0, lpairs = 0, checked = 0, disagree = 0;
    for (size_t q = 0; q < n; ++q) {
        Query qr;
        run_query(*static_cast<const Tree*>(trees_a[q]), *static_cast<const Tree*>(trees_b[q]),
                  ldm(mats_a + 16 * q), ldm(mats_b + 16 * q), qr, true, false, mode);
        tests += qr.nr.tests;
        lpairs += qr.lps.size();
        checked += qr.nr.rechecked;
        disagree += qr.nr.disagreements;
        for (const Hit& h : qr.nr.hits) {
            if (total < cap) {
                pair_out[3 * total + 0] = uint32_t(q);
                pair_out[3 * total + 1] = h.ia;
                pair_out[3 * total + 2] = h.ib;
                std::memcpy(seg_out + 6 * total, h.src, 3 * sizeof(float));
                std::memcpy(seg_out + 6 * total + 3, h.tgt, 3 * sizeof(float));
            }
            ++total;
        }
    }
    if (tests_out) *tests_out = tests;
    if (leafpairs_out) *leafpairs_out = lpairs;
    if (recheck) {
        recheck[0] = checked;
        recheck[1] = disagree;
    }
    return total;
}

size_t port_collide_pairs(void* const* trees_a, void* const* trees_b, const float* mats_a, const float* mats_b,
                          size_t n, uint32_t* pair_out, float* seg_out, size_t cap, uint64_t* tests_out,
                          uint64_t* leafpairs_out) {
    return port_collide_pairs_mode(trees_a, trees_b, mats_a, mats_b, n, pair_out, seg_out, cap, tests_out,
                                   leafpairs_out, 0, nullptr);
}

// Morph targets, then linear-blend skinning, of dynamicMeshShader_glsl.comp
// (shaders/dynamicMeshShader_glsl.comp:78-145; position path: no NORMALIZE,
// no ZERO_W), restated in C++ because the shader cannot run here.
// vertices: per vertex the base then n_targets target offsets, vec4 each (the
// shader's interleaved buffer); joints/weights: n_groups groups of four per
// vertex; joint_matrices[j] is the shader's modelMatrices[matrixOffset + 1 + j],
// inverse_bind[j] its inverseModelMatrices[inverseMatricesOffset + j].
// Operation order: morphed += w_i * target_i per component; each joint's
// matrix is joint_matrix * inverse_bind (glm convention), applied to the vec4
// as (c0 x + c1 y) + (c2 z + c3 w); result += weight * that, joints x, y, z, w
// in turn.
void port_deform(size_t n_vertices, size_t n_targets, size_t n_groups, size_t n_joints, const float* vertices,
                 const float* morph_weights, const uint16_t* joints, const float* weights, const float* joint_matrices,
                 const float* inverse_bind, float* out) {
    std::vector<M4> mats(n_joints);
    for (size_t j = 0; j < n_joints; ++j) {
        M4 g, ib;
        std::memcpy(g.m, joint_matrices + 16 * j, sizeof(g.m));
        std::memcpy(ib.m, inverse_bind + 16 * j, sizeof(ib.m));
        mats[j] = mul(g, ib);
    }
    for (size_t x = 0; x < n_vertices; ++x) {
        const float* vx = vertices + 4 * (n_targets + 1) * x;
        float v[4] = {vx[0], vx[1], vx[2], vx[3]};
        for (size_t i = 0; i < n_targets; ++i)
            for (int c = 0; c < 4; ++c) v[c] = v[c] + morph_weights[i] * vx[4 * (i + 1) + c];
        float r[4] = {0.f, 0.f, 0.f, 0.f};
        if (n_groups == 0)
            for (int c = 0; c < 4; ++c) r[c] = v[c];
        for (size_t g = 0; g < n_groups; ++g) {
            const float* w = weights + 4 * (n_groups * x + g);
            const uint16_t* jn = joints + 4 * (n_groups * x + g);
            for (int e = 0; e < 4; ++e) {
                const float* m = mats[jn[e]].m;
                for (int c = 0; c < 4; ++c) {
                    const float t = (m[0 + c] * v[0] + m[4 + c] * v[1]) + (m[8 + c] * v[2] + m[12 + c] * v[3]);
                    r[c] = r[c] + w[e] * t;
                }
            }
        }
        for (int c = 0; c < 4; ++c) out[4 * x + c] = r[c];
    }
}

// Refit of a flat tree to new vertex positions (n_positions x 4 floats,
// indexed by tri_idx): corner positions replaced, then every box fitted again
// with fit_box (OBB::CreateOBBfromPoints) to the corners of its subtree's
// triangles in leaf (DFS) order. Writes the new root box, node boxes and
// triangle positions.
void port_tree_refit(size_t n_nodes, const uint32_t* node_ref, const uint32_t* node_cnt, size_t n_tris,
                     const uint32_t* tri_idx, const float* positions, size_t n_positions, float* out_root12,
                     float* out_node_obbs, float* out_tri_pos) {
    std::vector<V3> pos(3 * n_tris);
    const float nan = std::numeric_limits<float>::quiet_NaN();
    for (size_t t = 0; t < n_tris; ++t)
        for (int k = 0; k < 3; ++k) {
            const uint32_t vi = tri_idx[3 * t + k];
            pos[3 * t + k] = vi < n_positions ? V3{positions[4 * vi], positions[4 * vi + 1], positions[4 * vi + 2]}
                                              : V3{nan, nan, nan};
            st3(pos[3 * t + k], out_tri_pos + 9 * t + 3 * k);
        }
    auto fit_range = [&](uint32_t first, uint32_t count) {
        std::vector<V3> pts(pos.begin() + 3 * size_t(first), pos.begin() + 3 * size_t(first + count));
        return fit_box(pts);
    };
    std::vector<std::pair<uint32_t, uint32_t>> rg(n_nodes);
    for (size_t k = n_nodes; k-- > 0;) {
        uint32_t lo = 0xffffffffu, hi = 0;
        for (int s = 0; s < 2; ++s) {
            const uint32_t ref = node_ref[2 * k + s], cnt = node_cnt[2 * k + s];
            const std::pair<uint32_t, uint32_t> c = cnt ? std::make_pair(ref, cnt) : rg[ref];
            stbox(fit_range(c.first, c.second), out_node_obbs + 24 * k + 12 * s);
            if (c.second) {
                lo = std::min(lo, c.first);
                hi = std::max(hi, c.first + c.second);
            }
        }
        rg[k] = lo <= hi ? std::make_pair(lo, hi - lo) : std::make_pair(0u, 0u);
    }
    const std::pair<uint32_t, uint32_t> root = n_nodes ? rg[0] : std::make_pair(0u, uint32_t(n_tris));
    stbox(fit_range(root.first, root.second), out_root12);
}


// ShootUncollideRays::ExecuteShootUncollideRays for one entity pair with the
// engine's settings (CollisionDetection.cpp:22-24: 40 and 65 degrees, 1.01)
// unless params (start angle, finish angle in radians, bias) is given; rays
// as (origin, direction) sextuples in the first entity's space.
void port_shoot_rays(void* ta, void* tb, const float* ga16, const float* gb16, const float* rays_a, size_t n_a,
                     const float* rays_b, size_t n_b, const float* params, float* out3) {
    auto load = [](const float* r, size_t n) {
        std::vector<Ray> v(n);
        for (size_t i = 0; i < n; ++i) v[i] = Ray{ld3(r + 6 * i), ld3(r + 6 * i + 3)};
        return v;
    };
    const float deg = 0.01745329251994329576923690768489f;
    ShootParams P;
    P.cos_start = std::cos(params ? params[0] : 40.f * deg);
    P.cos_finish = std::cos(params ? params[1] : 65.f * deg);
    P.bias = params ? params[2] : 1.01f;
    const V3 r = shoot(*static_cast<Tree*>(ta), *static_cast<Tree*>(tb), ldm(ga16), ldm(gb16), load(rays_a, n_a),
                       load(rays_b, n_b), P);
    st3(r, out3);
}

// SweepAndPrune::ExecuteSweepAndPrune with the engine's axes or axes9 (U, V,
// W); the pairs (first, second) in no particular order; returns their count.
size_t port_sweep_and_prune(void* const* trees, const float* globals, const uint8_t* callback, size_t n,
                            const float* axes9, uint32_t* out_pairs, size_t cap) {
    std::vector<const Tree*> ts(n);
    std::vector<M4> gs(n);
    std::vector<uint8_t> cb(callback, callback + n);
    for (size_t i = 0; i < n; ++i) {
        ts[i] = static_cast<const Tree*>(trees[i]);
        gs[i] = ldm(globals + 16 * i);
    }
    V3 U, V, W;
    if (axes9) {
        U = ld3(axes9);
        V = ld3(axes9 + 3);
        W = ld3(axes9 + 6);
    } else {
        engine_axes(U, V, W);
    }
    const auto pairs = sweep_and_prune(ts, gs, cb, U, V, W);
    for (size_t k = 0; k < pairs.size() && k < cap; ++k) {
        out_pairs[2 * k] = pairs[k].first;
        out_pairs[2 * k + 1] = pairs[k].second;
    }
    return pairs.size();
}

}  // extern "C"
