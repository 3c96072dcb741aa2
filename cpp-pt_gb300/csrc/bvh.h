// Host-side BVH construction.
//
// Two hierarchies are built for every scene:
//
// 1. RefTopology -- the reference's own binary BVH (BVH::build_node /
//    compute_split, src/primitive/bvh.h:57-216), rebuilt with the same bins,
//    cost, tie order and child order.  It is never traversed on the GPU.  It
//    yields, per triangle, (a) its rank = position in the order
//    BVHNode::intersect visits leaves (bvh.h:33-34, member `right` first), and
//    (b) the box of the innermost internal node above its leaf.  Those two
//    values let any traversal reproduce the reference's closest hit exactly:
//      - the reference reports the smallest t among the triangles it tests,
//        the later-visited (higher rank) one on equal t (triangle.h:55,106);
//      - it tests a triangle iff every ancestor box passes its slab test
//        (aabb.h:19-61), and that test is monotone under box inclusion
//        (every float step -- subtraction, division by the same d, min/max --
//        is monotone), so passing the innermost ancestor box implies
//        passing all of them.
//
// 2. WideBVH -- a binned-SAH BVH collapsed to 4 children per node, with
//    children boxes quantised to 8 bits relative to the node (64 bytes per
//    node), triangles reordered into its leaves as {a, b-a, c-a} + rank +
//    parent-box index + insertion index (48 bytes).  This is what the GPU
//    traverses.
#pragma once
#include <cstdint>
#include <vector>

namespace cpppt_gb300 {

struct Box3 {
    float lo[3], hi[3];
};

struct RefTopology {
    std::vector<int32_t> rank;          // per triangle (insertion index -> DFS rank)
    std::vector<int32_t> leaf_order;    // DFS order of insertion indices
    std::vector<Box3> node_box;         // internal nodes, pre-order
    std::vector<int32_t> node_parent;   // per internal node
    std::vector<int32_t> prim_parent;   // per triangle: internal node holding its leaf (-1: root is a leaf)
};

// Builds the reference topology from per-triangle vertex positions.
// tri_v: 9 floats per triangle (a, b, c).
// n_threads: 0 = all hardware threads, 1 = sequential; the result does not
// depend on it (independent subtrees are built in parallel and joined in
// the reference's pre-order).
RefTopology build_ref_topology(const float* tri_v, int n_tris, int n_threads = 0);

// Compressed 4-wide node, 64 bytes (4 x uint4 on the device):
//   w[0..2] origin p (float bits); w[3] = ex | ey<<8 | ez<<16  (biased float exponents of the
//   per-axis scale s = 2^(e-127)); w[4..7] lo_x[4] lo_y[4] lo_z[4] hi_x[4] (bytes, child c at
//   byte c); w[8..9] hi_y[4] hi_z[4]; w[10..13] child refs; w[14..15] unused.
// A child box is [p + lo*s, p + hi*s].  Empty slots have lo = 255, hi = 0.
// Child ref: bit 31 clear -> internal node index; bit 31 set -> leaf with
// (ref >> 27 & 15) + 1 triangles starting at (ref & 0x7ffffff).
struct WideNode {
    uint32_t w[16];
};

struct WideBVH {
    std::vector<WideNode> nodes;      // breadth-first order, root at 0
    std::vector<int32_t> tri_order;   // leaf order -> insertion index
    int max_depth = 0;                // in wide nodes
    int max_leaf = 0;
    float inflate = 0.0f;             // absolute box inflation used
};

// tri_v as above.  max_leaf <= 16.
WideBVH build_wide_bvh(const float* tri_v, int n_tris, int max_leaf = 4, int n_threads = 0);

constexpr uint32_t kLeafBit = 0x80000000u;
inline uint32_t make_leaf_ref(uint32_t start, uint32_t count) {
    return kLeafBit | ((count - 1u) << 27) | start;
}

}  // namespace cpppt_gb300
