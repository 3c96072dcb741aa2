// Multi-scene arena: copies of several scenes' device arrays merged into one
// set of arrays, with every cross-reference rebased by the scene's offsets.
// The merged arrays hold exactly the same nodes, triangles and shading data
// (same boxes, same leaf order, same reference ranks), so a ray traced from
// a scene's root inside the arena visits the same nodes and reports the same
// hit as in the scene's own copy.
#include <cuda_runtime.h>

#include "batch.h"

namespace cpppt_gb300 {

__device__ __forceinline__ uint32_t rebase_ref(uint32_t r, uint32_t node_off, uint32_t tri_off) {
    if (r == 0xffffffffu) return r;               // empty child slot
    if (r & 0x80000000u) return r + tri_off;      // leaf: start is the low 27 bits (sum checked on the host)
    return r + node_off;
}

// Wide node (4 x uint4): origin and exponents | child lo x, y, z, hi x |
// hi y, hi z, ref 0, ref 1 | ref 2, ref 3, unused: the child references are
// words 10-13.
__global__ void k_rebase_nodes(uint4* __restrict__ dst, const uint4* __restrict__ src, int n, uint32_t node_off,
                               uint32_t tri_off) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint4* s = src + 4 * (size_t)i;
        uint4* d = dst + 4 * (size_t)i;
        uint4 w2 = s[2], w3 = s[3];
        w2.z = rebase_ref(w2.z, node_off, tri_off);
        w2.w = rebase_ref(w2.w, node_off, tri_off);
        w3.x = rebase_ref(w3.x, node_off, tri_off);
        w3.y = rebase_ref(w3.y, node_off, tri_off);
        d[0] = s[0];
        d[1] = s[1];
        d[2] = w2;
        d[3] = w3;
    }
}

// Traversal triangles: {a, rank}, {b - a, parent box}, {c - a, prim}.
__global__ void k_rebase_tris(float4* __restrict__ dst, const float4* __restrict__ src, int n, int rbox_off,
                              int prim_off) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4* s = src + 3 * (size_t)i;
        float4* d = dst + 3 * (size_t)i;
        float4 e1 = s[1], e2 = s[2];
        const int parent = __float_as_int(e1.w);
        if (parent >= 0) e1.w = __int_as_float(parent + rbox_off);
        e2.w = __int_as_float(__float_as_int(e2.w) + prim_off);
        d[0] = s[0];
        d[1] = e1;
        d[2] = e2;
    }
}

__global__ void k_rebase_vidx(int4* __restrict__ dst, const int4* __restrict__ src, int n, int v_off, int m_off) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 v = src[i];
        dst[i] = make_int4(v.x + v_off, v.y + v_off, v.z + v_off, v.w + m_off);
    }
}

__global__ void k_offset_i32(int32_t* __restrict__ dst, const int32_t* __restrict__ src, int n, int off) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i] + off;
}

namespace {
int grid_for(int n) { return n <= 0 ? 0 : (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096; }
}  // namespace

void launch_rebase_nodes(uint4* dst, const uint4* src, int n, uint32_t node_off, uint32_t tri_off, cudaStream_t st) {
    if (n > 0) k_rebase_nodes<<<grid_for(n), 256, 0, st>>>(dst, src, n, node_off, tri_off);
}
void launch_rebase_tris(float4* dst, const float4* src, int n, int rbox_off, int prim_off, cudaStream_t st) {
    if (n > 0) k_rebase_tris<<<grid_for(n), 256, 0, st>>>(dst, src, n, rbox_off, prim_off);
}
void launch_rebase_vidx(int4* dst, const int4* src, int n, int v_off, int m_off, cudaStream_t st) {
    if (n > 0) k_rebase_vidx<<<grid_for(n), 256, 0, st>>>(dst, src, n, v_off, m_off);
}
void launch_offset_i32(int32_t* dst, const int32_t* src, int n, int off, cudaStream_t st) {
    if (n > 0) k_offset_i32<<<grid_for(n), 256, 0, st>>>(dst, src, n, off);
}

}  // namespace cpppt_gb300
