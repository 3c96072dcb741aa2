// Device build of the reference-topology BVH (gpu_bvh.cu).
#pragma once
#include <cuda_runtime.h>

#include "bvh.h"

namespace cpppt_gb300 {

struct RefBuildStats {
    int levels = 0;  // tree levels (kernel launches of the level loop)
    int nodes = 0;   // internal nodes
};

// The same RefTopology as build_ref_topology (bvh.cpp), bit for bit, built
// on the current device on stream st.  tri_v: 9 floats per triangle in host
// memory.  Synchronises st.
RefTopology build_ref_topology_device(const float* tri_v, int n_tris, cudaStream_t st, RefBuildStats* stats = nullptr);

struct WideBuildStats {
    int top_levels = 0;    // level-synchronous launches over nodes of more than 4096 triangles
    int subtrees = 0;      // CTAs that each built a subtree of at most 4096 triangles
    int binary_nodes = 0;  // nodes of the binary SAH tree
    int wide_levels = 0;   // breadth-first levels of the 4-wide tree
};

// The same WideBVH as build_wide_bvh (bvh.cpp), bit for bit (nodes, leaf
// order, depth, inflation), built on the current device on stream st
// (gpu_sah.cu).  tri_v: 9 floats per triangle in host memory.  Synchronises
// st.
WideBVH build_wide_bvh_device(const float* tri_v, int n_tris, int max_leaf, cudaStream_t st,
                              WideBuildStats* stats = nullptr);

}  // namespace cpppt_gb300
