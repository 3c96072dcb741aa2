// SD-tree of practical path guiding as the reference builds it
// (src/algorithms/sdtree.h:268-674, used by PPG, src/renderer/ppg.h:41-215).
//
// Host side: the tree structure and its between-iteration update
// (SDTree::update -> subdivide -> DTree::adapt_and_build_leaves), restated
// with the reference's thresholds, traversal orders and quirks:
//   - spatial binary tree split at cell midpoints, axis = depth % 3, a point
//     goes right iff coordinate > mid (sdtree.h:354-406);
//   - a spatial leaf splits when its splat count exceeds
//     12000 * int(2^(iteration/2)) (sdtree.h:460-482), int(log2(ratio))+1
//     times, and both halves copy the rebuilt directional tree;
//   - the directional quadtree over (phi in [-pi,pi], cos(theta) in [-1,1])
//     is pruned below 1% of the leaf's flux and subdivided above it
//     (sdtree.h:97-113,172-233); a leaf with zero flux keeps its old tree,
//     count and flux;
//   - sampling is uniform over the quadtree's leaves, pdf = 1/(n_leaves *
//     leaf area) (sdtree.h:408-430,525-537).
// Device side (flattened by `flatten`): lookups, sampling, pdf and atomic
// splats of max-channel radiance (sdtree.h:514-524).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

namespace cpppt_gb300 {

struct DNodeH {
    bool leaf = true;
    float value = 0.0f;
    std::unique_ptr<DNodeH> child[4];
    std::unique_ptr<DNodeH> clone() const;
};

struct DLeafRegion {
    float bx, by, sx, sy;  // begin (phi, cos theta), size
};

struct DTreeH {
    std::unique_ptr<DNodeH> root;
    int count = 0;
    float radiance = 0.0f;
    std::vector<DLeafRegion> leaves;
    DTreeH();
    std::unique_ptr<DTreeH> clone() const;
    void adapt_and_build_leaves();
};

struct SNodeH {
    std::unique_ptr<DTreeH> dtree;  // leaf when set
    std::unique_ptr<SNodeH> child[2];
};

// Flat device image of the tree.
struct SDTreeFlat {
    float lo[3], hi[3];                 // spatial bounds
    std::vector<int32_t> snode;         // 2 per spatial node: children, or (-1 - dtree, -1) for a leaf
    std::vector<int32_t> dnode;         // per quadtree node: first of 4 children, or (-1 - value slot) for a leaf
    std::vector<int32_t> dtree_root;    // per dtree: its root in dnode
    std::vector<int32_t> dtree_leaf_off, dtree_leaf_cnt;  // per dtree: range in `leaves`
    std::vector<float> leaves;          // 4 per sampling leaf: begin phi, begin cos, size phi, size cos
    int n_value_slots = 0;              // quadtree leaves (splat accumulators)
};

class SDTreeHost {
public:
    SDTreeHost(const float lo[3], const float hi[3]);
    // Folds one iteration's device accumulators (slot values in flatten()
    // order, per-dtree counts and flux) into the tree.
    void accumulate(const float* slot_values, const int32_t* counts, const float* radiance);
    void update();  // SDTree::update: subdivide(12000, iteration); iteration++
    SDTreeFlat flatten() const;
    // Host versions of the device lookups (used by the host-only checks):
    // SDTree::splat and SDTree::pdf (sdtree.h:514-537).
    void splat(float radiance, const float pos[3], const float dir[3]);
    float pdf(const float pos[3], const float dir[3]) const;
    // Sampling leaves, counts and flux of every spatial leaf, depth first.
    void dump(std::vector<DLeafRegion>* leaves, std::vector<int>* leaf_counts, std::vector<int>* counts,
              std::vector<float>* flux) const;
    int iteration() const { return iteration_; }
    int n_spatial_leaves() const;

private:
    DTreeH* find(const float pos[3]) const;
    float lo_[3], hi_[3];
    std::unique_ptr<SNodeH> root_;
    int iteration_ = 1;
    int c_ = 12000;
};

}  // namespace cpppt_gb300
