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

}  // namespace cpppt_gb300
