// Launchers of the multi-scene arena merge (batch.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dev_types.h"

namespace cpppt_gb300 {

void launch_rebase_nodes(uint4* dst, const uint4* src, int n, uint32_t node_off, uint32_t tri_off, cudaStream_t st);
void launch_rebase_tris(float4* dst, const float4* src, int n, int rbox_off, int prim_off, cudaStream_t st);
void launch_rebase_vidx(int4* dst, const int4* src, int n, int v_off, int m_off, cudaStream_t st);
void launch_offset_i32(int32_t* dst, const int32_t* src, int n, int off, cudaStream_t st);

}  // namespace cpppt_gb300
