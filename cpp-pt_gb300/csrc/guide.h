// Device SD-tree (flattened by SDTreeHost::flatten) and the PPG wavefront
// stages implemented in guide.cu.
#pragma once
#include <cuda_runtime.h>

#include "dev_types.h"
#include "kernels.h"

namespace cpppt_gb300 {

struct DevSDTree {
    float lo[3], hi[3];
    const int2* snode;       // children, or (-1 - dtree, -1) at a leaf
    const int* dnode;        // first of 4 children, or (-1 - value slot) at a leaf
    const int* dtree_root;
    const int* leaf_off;     // per dtree: first sampling leaf
    const int* leaf_cnt;     // per dtree: number of sampling leaves
    const float4* leaves;    // begin phi, begin cos theta, size phi, size cos theta
    float* slot_value;       // splat accumulator per quadtree leaf
    int* dtree_count;        // splats per spatial leaf
    float* dtree_rad;        // splatted flux per spatial leaf
};

// Per-path vertex records, max_depth per slot: position + direction.x,
// direction.yz + factor.xy, factor.z.
struct PPGVerts {
    float4* vp;
    float4* vd;
    float* vr;
};

void launch_init_slots(int* slot_stack, int n, cudaStream_t st);
void launch_shade_ppg(const DevScene& S, const PathBuffers& B, int cur, const RenderParams& P, WaveCounters* ctr,
                      unsigned long long* film, const DevSDTree& T, const PPGVerts& V, int* slot_stack,
                      cudaStream_t st);
void launch_generate_ppg(const DevScene& S, const PathBuffers& B, int cur, const RenderParams& P, WaveCounters* ctr,
                         const int* slot_stack, cudaStream_t st);

}  // namespace cpppt_gb300
