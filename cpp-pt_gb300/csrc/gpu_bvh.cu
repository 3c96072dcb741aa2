// Device build of the reference's binary BVH topology (BVH::build_node /
// compute_split, src/primitive/bvh.h:57-216), bit-identical to the host
// restatement build_ref_topology (bvh.cpp) and so to the reference.
//
// Level-synchronous: every node of one tree level is a segment [start,
// start + count) of the primitive array, processed by one CTA of 128
// threads, which
//   1. reduces the node's bounds and centroid bounds,
//   2. bins the centroids into 5 equal-width bins per axis (a primitive
//      joins the first bin j with c < min + (max - min) * (j + 1) / 5) and
//      reduces each bin's count and box,
//   3. evaluates the 4 splits per axis (area(L) + area(R), +inf when a side
//      is empty; first strict minimum; the reference's nested axis choice),
//   4. writes its primitives into the other buffer in the bins'
//      concatenation order (bin 0's primitives, then bin 1's, ..., each bin
//      in input order), and emits the node and its two child segments (bins
//      0..split and the rest) for the next level.
// A segment of fewer than 4 primitives is a leaf (bvh.h:152-158).  Where the
// chosen split leaves one side empty the reference recurses without end
// (bvh.h:200); like the host build, one leaf then holds them all.
//
// The reference unites boxes in the primitives' order with
// min(a, b) = a < b ? a : b (and max likewise), so among equal values the
// later primitive's value is kept (this matters for -0.0 against +0.0).
// Each min / max is therefore a reduction of a 64-bit key -- the value
// mapped to an ordered integer with -0.0 and +0.0 equal, then the position
// (ties to the later one) -- and the winner's own float is read back.
// All float arithmetic is unfused (__fadd_rn / __fmul_rn) in the
// reference's order.
//
// Nodes are created level by level in no particular order; the pre-order
// numbering of the reference (parent, then the first partition's subtree,
// then the second's) follows from the subtree sizes, computed bottom-up.
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu_bvh.h"

namespace cpppt_gb300 {

namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kBins = 5;

struct PrimG {
    float lo[3], hi[3], c[3];
    int32_t id;
};

struct SegG {
    int32_t start, count, parent, side;  // parent: node id (-1: none); side 0 = first partition
};

struct NodeG {
    float lo[3], hi[3];
    int32_t parent, side;
    int32_t child[2];  // node ids, -1 for a leaf child
};

__device__ __forceinline__ uint32_t okey(float v) {
    if (v == 0.0f) v = 0.0f;  // -0.0 and +0.0 compare equal
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
// smallest value, then the later position
__device__ __forceinline__ unsigned long long kmin(float v, uint32_t pos) {
    return ((unsigned long long)okey(v) << 32) | (unsigned long long)(0xffffffffu - pos);
}
// largest value, then the later position
__device__ __forceinline__ unsigned long long kmax(float v, uint32_t pos) {
    return ((unsigned long long)okey(v) << 32) | (unsigned long long)pos;
}
__device__ __forceinline__ uint32_t kpos_min(unsigned long long k) { return 0xffffffffu - (uint32_t)(k & 0xffffffffu); }
__device__ __forceinline__ uint32_t kpos_max(unsigned long long k) { return (uint32_t)(k & 0xffffffffu); }

__device__ __forceinline__ unsigned long long warp_min64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ unsigned long long warp_max64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// AABB::area (aabb.h:77-82): 2.0 * (|dx| dy + |dz| dy + |dx| dz), the sum in
// float, doubled in double
__device__ __forceinline__ float ref_area(const float* lo, const float* hi) {
    const float dx = fabsf(__fsub_rn(hi[0], lo[0])), dy = __fsub_rn(hi[1], lo[1]);
    const float dz = fabsf(__fsub_rn(hi[2], lo[2])), dzy = __fsub_rn(hi[2], lo[2]);
    float s = __fmul_rn(dx, dy);
    s = __fadd_rn(s, __fmul_rn(dz, dy));
    s = __fadd_rn(s, __fmul_rn(dx, dzy));
    return (float)(2.0 * (double)s);
}

// a < b ? a : b and a > b ? a : b (the later operand kept on ties)
__device__ __forceinline__ float vmin1(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float vmax1(float a, float b) { return a > b ? a : b; }

__device__ __forceinline__ int bin_of(float c, const float* thr) {
    int b = kBins - 1;
#pragma unroll
    for (int j = kBins - 2; j >= 0; j--)
        if (c < thr[j]) b = j;
    return b;
}

// Per-primitive records: Triangle::get_bounds (triangle.h:197-207) and
// AABB::center ((min + max) * 0.5, aabb.h:62-64).
__global__ void k_prims(const float* __restrict__ tv, int n, PrimG* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = tv + 9 * (size_t)i;
    PrimG p;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        p.lo[k] = vmin1(vmin1(v[k], v[3 + k]), v[6 + k]);
        p.hi[k] = vmax1(vmax1(v[k], v[3 + k]), v[6 + k]);
        p.c[k] = __fmul_rn(__fadd_rn(p.lo[k], p.hi[k]), 0.5f);
    }
    p.id = i;
    out[i] = p;
}

__global__ void __launch_bounds__(kThreads) k_level(const SegG* __restrict__ segs, const PrimG* __restrict__ pin,
                                                    PrimG* __restrict__ pout, NodeG* __restrict__ nodes,
                                                    int* __restrict__ node_count, SegG* __restrict__ next,
                                                    int* __restrict__ next_count, int32_t* __restrict__ final_id,
                                                    int32_t* __restrict__ leaf_parent) {
    __shared__ unsigned long long s_red[kWarps][12];
    __shared__ float s_bounds[12];  // lo xyz, hi xyz, centroid lo xyz, centroid hi xyz
    __shared__ unsigned long long s_bin[3][kBins][6];
    __shared__ int s_cnt[3][kBins];
    __shared__ int s_axis, s_leaf;
    __shared__ float s_thr[3][kBins - 1];
    __shared__ int s_wbin[kWarps][kBins];
    const SegG seg = segs[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const PrimG* P = pin + seg.start;
    const int n = seg.count;

    auto emit_leaf = [&]() {
        for (int i = tid; i < n; i += kThreads) {
            final_id[seg.start + i] = P[i].id;
            leaf_parent[seg.start + i] = seg.parent;
        }
    };
    if (n < 4) {  // bvh.h:152-158
        emit_leaf();
        return;
    }
    // 1. bounds and centroid bounds
    {
        unsigned long long k[12];
#pragma unroll
        for (int j = 0; j < 3; j++) { k[j] = ~0ull; k[3 + j] = 0ull; k[6 + j] = ~0ull; k[9 + j] = 0ull; }
        for (int i = tid; i < n; i += kThreads) {
            const PrimG p = P[i];
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const unsigned long long a = kmin(p.lo[j], i), b = kmax(p.hi[j], i);
                const unsigned long long c = kmin(p.c[j], i), d = kmax(p.c[j], i);
                k[j] = a < k[j] ? a : k[j];
                k[3 + j] = b > k[3 + j] ? b : k[3 + j];
                k[6 + j] = c < k[6 + j] ? c : k[6 + j];
                k[9 + j] = d > k[9 + j] ? d : k[9 + j];
            }
        }
#pragma unroll
        for (int j = 0; j < 3; j++) {
            k[j] = warp_min64(k[j]);
            k[3 + j] = warp_max64(k[3 + j]);
            k[6 + j] = warp_min64(k[6 + j]);
            k[9 + j] = warp_max64(k[9 + j]);
        }
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < 12; j++) s_red[warp][j] = k[j];
        __syncthreads();
        if (tid < 12) {
            const bool is_min = (tid < 3) || (tid >= 6 && tid < 9);
            unsigned long long r = s_red[0][tid];
            for (int w = 1; w < kWarps; w++) {
                const unsigned long long x = s_red[w][tid];
                r = is_min ? (x < r ? x : r) : (x > r ? x : r);
            }
            const uint32_t pos = is_min ? kpos_min(r) : kpos_max(r);
            const int axis = tid % 3;
            const PrimG& w = P[pos];
            s_bounds[tid] = tid < 3 ? w.lo[axis] : (tid < 6 ? w.hi[axis] : w.c[axis]);
        }
        for (int j = tid; j < 3 * kBins * 6; j += kThreads) {
            const int comp = j % 6;
            (&s_bin[0][0][0])[j] = comp < 3 ? ~0ull : 0ull;
        }
        if (tid < 3 * kBins) (&s_cnt[0][0])[tid] = 0;
        __syncthreads();
    }
    // 2. thresholds lo + (hi - lo) * float(j + 1) / 5, then the bins
    if (tid < 3 * (kBins - 1)) {
        const int axis = tid / (kBins - 1), j = tid % (kBins - 1);
        const float lo = s_bounds[6 + axis], hi = s_bounds[9 + axis];
        s_thr[axis][j] = __fadd_rn(lo, __fdiv_rn(__fmul_rn(__fsub_rn(hi, lo), (float)(j + 1)), (float)kBins));
    }
    __syncthreads();
    for (int i = tid; i < n; i += kThreads) {
        const PrimG p = P[i];
#pragma unroll
        for (int axis = 0; axis < 3; axis++) {
            const int b = bin_of(p.c[axis], s_thr[axis]);
            atomicAdd(&s_cnt[axis][b], 1);
            unsigned long long* bb = s_bin[axis][b];
#pragma unroll
            for (int j = 0; j < 3; j++) {
                atomicMin(bb + j, kmin(p.lo[j], i));
                atomicMax(bb + 3 + j, kmax(p.hi[j], i));
            }
        }
    }
    __syncthreads();
    // 3. split costs, axis (bvh.h:57-149, 179-197)
    if (tid == 0) {
        float cost[3];
        int best[3];
        for (int axis = 0; axis < 3; axis++) {
            float blo[kBins][3], bhi[kBins][3];
            for (int b = 0; b < kBins; b++)
                for (int j = 0; j < 3; j++) {
                    if (s_cnt[axis][b] > 0) {
                        blo[b][j] = P[kpos_min(s_bin[axis][b][j])].lo[j];
                        bhi[b][j] = P[kpos_max(s_bin[axis][b][3 + j])].hi[j];
                    } else {
                        blo[b][j] = __int_as_float(0x7f800000);
                        bhi[b][j] = -__int_as_float(0x7f800000);
                    }
                }
            float pc[kBins - 1];
            for (int i = 0; i < kBins - 1; i++) {
                float llo[3], lhi[3], rlo[3], rhi[3];
                for (int j = 0; j < 3; j++) {
                    llo[j] = rlo[j] = __int_as_float(0x7f800000);
                    lhi[j] = rhi[j] = -__int_as_float(0x7f800000);
                }
                int lc = 0, rc = 0;
                for (int b = 0; b < kBins; b++) {
                    const int c = s_cnt[axis][b];
                    if (b <= i) {
                        lc += c;
                        if (c)
                            for (int j = 0; j < 3; j++) { llo[j] = vmin1(llo[j], blo[b][j]); lhi[j] = vmax1(lhi[j], bhi[b][j]); }
                    } else {
                        rc += c;
                        if (c)
                            for (int j = 0; j < 3; j++) { rlo[j] = vmin1(rlo[j], blo[b][j]); rhi[j] = vmax1(rhi[j], bhi[b][j]); }
                    }
                }
                pc[i] = (lc == 0 || rc == 0) ? __int_as_float(0x7f800000)
                                             : __fadd_rn(ref_area(llo, lhi), ref_area(rlo, rhi));
            }
            int m = 0;
            float mc = pc[0];
            for (int i = 1; i < kBins - 1; i++)
                if (pc[i] < mc) { mc = pc[i]; m = i; }
            cost[axis] = mc;
            best[axis] = m;
        }
        const float c1 = cost[0], c2 = cost[1], c3 = cost[2];
        int axis;
        if (c1 < c2) axis = (c1 < c3) ? 0 : (c2 < c3 ? 1 : 2);
        else axis = (c2 < c3) ? 1 : 2;
        const int split = best[axis];
        int nl = 0;
        for (int b = 0; b <= split; b++) nl += s_cnt[axis][b];
        s_axis = axis;
        s_leaf = (nl == 0 || nl == n) ? 1 : 0;
        if (!s_leaf) {
            const int nid = atomicAdd(node_count, 1);
            NodeG nd;
            for (int j = 0; j < 3; j++) { nd.lo[j] = s_bounds[j]; nd.hi[j] = s_bounds[3 + j]; }
            nd.parent = seg.parent;
            nd.side = seg.side;
            nd.child[0] = nd.child[1] = -1;
            nodes[nid] = nd;
            if (seg.parent >= 0) nodes[seg.parent].child[seg.side] = nid;
            const int k = atomicAdd(next_count, 2);
            next[k] = SegG{seg.start, nl, nid, 0};
            next[k + 1] = SegG{seg.start + nl, n - nl, nid, 1};
        }
    }
    __syncthreads();
    if (s_leaf) {
        emit_leaf();
        return;
    }
    // 4. into pout in the bins' concatenation order (bin 0's primitives,
    // then bin 1's, ..., each bin in input order): the first partition is
    // bins 0..split, the second the rest (bvh.h:138-144)
    const int axis = s_axis;
    const float* thr = s_thr[axis];
    PrimG* Q = pout + seg.start;
    int run[kBins];
    run[0] = 0;
    for (int b = 1; b < kBins; b++) run[b] = run[b - 1] + s_cnt[axis][b - 1];
    for (int base = 0; base < n; base += kThreads) {
        const int i = base + tid;
        PrimG p;
        int mb = -1;
        if (i < n) {
            p = P[i];
            mb = bin_of(p.c[axis], thr);
        }
        unsigned bal[kBins];
#pragma unroll
        for (int b = 0; b < kBins; b++) bal[b] = __ballot_sync(0xffffffffu, mb == b);
        if (lane < kBins) s_wbin[warp][lane] = __popc(bal[lane]);
        __syncthreads();
        if (i < n) {
            int pos = run[mb] + __popc(bal[mb] & ((1u << lane) - 1u));
            for (int w = 0; w < warp; w++) pos += s_wbin[w][mb];
            Q[pos] = p;
        }
#pragma unroll
        for (int b = 0; b < kBins; b++)
            for (int w = 0; w < kWarps; w++) run[b] += s_wbin[w][b];
        __syncthreads();
    }
}

// Subtree sizes (internal nodes), one level of nodes [lo, hi), bottom-up.
__global__ void k_sizes(const NodeG* __restrict__ nodes, int lo, int hi, int32_t* __restrict__ size) {
    const int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= hi) return;
    const NodeG& nd = nodes[i];
    size[i] = 1 + (nd.child[0] >= 0 ? size[nd.child[0]] : 0) + (nd.child[1] >= 0 ? size[nd.child[1]] : 0);
}

// Pre-order numbers of the children of one level of nodes, top-down.
__global__ void k_preorder(const NodeG* __restrict__ nodes, int lo, int hi, const int32_t* __restrict__ size,
                           int32_t* __restrict__ pre) {
    const int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= hi) return;
    const NodeG& nd = nodes[i];
    const int p = pre[i];
    if (nd.child[0] >= 0) pre[nd.child[0]] = p + 1;
    if (nd.child[1] >= 0) pre[nd.child[1]] = p + 1 + (nd.child[0] >= 0 ? size[nd.child[0]] : 0);
}

__global__ void k_node_out(const NodeG* __restrict__ nodes, int n_nodes, const int32_t* __restrict__ pre,
                           float* __restrict__ box, int32_t* __restrict__ parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    const NodeG& nd = nodes[i];
    const int p = pre[i];
    for (int j = 0; j < 3; j++) {
        box[6 * (size_t)p + j] = nd.lo[j];
        box[6 * (size_t)p + 3 + j] = nd.hi[j];
    }
    parent[p] = nd.parent >= 0 ? pre[nd.parent] : -1;
}

__global__ void k_prim_out(const int32_t* __restrict__ final_id, const int32_t* __restrict__ leaf_parent, int n,
                           const int32_t* __restrict__ pre, int32_t* __restrict__ rank,
                           int32_t* __restrict__ prim_parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int id = final_id[i];
    rank[id] = i;
    const int lp = leaf_parent[i];
    prim_parent[id] = lp >= 0 ? pre[lp] : -1;
}

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string("device BVH build: ") + what + ": " + cudaGetErrorString(e));
    }
}

template <class T>
T* dmalloc(std::vector<void*>& owned, size_t n) {
    void* p = nullptr;
    ck(cudaMalloc(&p, sizeof(T) * (n ? n : 1)), "cudaMalloc");
    owned.push_back(p);
    return static_cast<T*>(p);
}

}  // namespace

RefTopology build_ref_topology_device(const float* tri_v, int n, cudaStream_t st, RefBuildStats* stats) {
    RefTopology t;
    t.rank.assign(n, 0);
    t.prim_parent.assign(n, -1);
    if (n <= 0) return t;
    std::vector<void*> owned;
    struct Free {
        std::vector<void*>& v;
        ~Free() { for (void* p : v) cudaFree(p); }
    } guard{owned};
    int* h_cnt = nullptr;  // pinned: next-level segments, nodes
    ck(cudaMallocHost(&h_cnt, 2 * sizeof(int)), "cudaMallocHost");
    struct FreeHost {
        int* p;
        ~FreeHost() { cudaFreeHost(p); }
    } hguard{h_cnt};
    float* d_tv = dmalloc<float>(owned, 9 * (size_t)n);
    ck(cudaMemcpyAsync(d_tv, tri_v, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice, st), "upload");
    PrimG* buf[2] = {dmalloc<PrimG>(owned, n), dmalloc<PrimG>(owned, n)};
    // a split leaves at least one primitive on each side, so there are fewer
    // internal nodes than primitives, and at most n segments on a level
    const int max_nodes = n;
    NodeG* nodes = dmalloc<NodeG>(owned, max_nodes);
    SegG* segs[2] = {dmalloc<SegG>(owned, n + 2), dmalloc<SegG>(owned, n + 2)};
    int* d_cnt = dmalloc<int>(owned, 2);  // [0] next-level segments, [1] nodes
    int32_t* final_id = dmalloc<int32_t>(owned, n);
    int32_t* leaf_parent = dmalloc<int32_t>(owned, n);
    k_prims<<<(n + 255) / 256, 256, 0, st>>>(d_tv, n, buf[0]);
    const SegG root{0, n, -1, 0};
    ck(cudaMemcpyAsync(segs[0], &root, sizeof(root), cudaMemcpyHostToDevice, st), "root segment");
    ck(cudaMemsetAsync(d_cnt, 0, 2 * sizeof(int), st), "memset");
    std::vector<int> level_nodes(1, 0);  // node count after each level
    int n_seg = 1, cur = 0, levels = 0;
    while (n_seg > 0) {
        ck(cudaMemsetAsync(d_cnt, 0, sizeof(int), st), "memset");
        k_level<<<n_seg, kThreads, 0, st>>>(segs[cur], buf[cur], buf[1 - cur], nodes, d_cnt + 1, segs[1 - cur], d_cnt,
                                            final_id, leaf_parent);
        ck(cudaGetLastError(), "level kernel");
        ck(cudaMemcpyAsync(h_cnt, d_cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, st), "counts");
        ck(cudaStreamSynchronize(st), "level");
        n_seg = h_cnt[0];
        level_nodes.push_back(h_cnt[1]);
        if (h_cnt[1] > max_nodes || n_seg > n + 2) throw std::runtime_error("device BVH build overflow");
        cur = 1 - cur;
        levels++;
    }
    const int n_nodes = level_nodes.back();
    int32_t* size = dmalloc<int32_t>(owned, n_nodes);
    int32_t* pre = dmalloc<int32_t>(owned, n_nodes);
    for (int L = (int)level_nodes.size() - 2; L >= 0; L--) {
        const int lo = level_nodes[L], hi = level_nodes[L + 1];
        if (hi > lo) k_sizes<<<(hi - lo + 255) / 256, 256, 0, st>>>(nodes, lo, hi, size);
    }
    if (n_nodes > 0) ck(cudaMemsetAsync(pre, 0, sizeof(int32_t), st), "root pre-order");  // node 0 is the root
    for (size_t L = 0; L + 1 < level_nodes.size(); L++) {
        const int lo = level_nodes[L], hi = level_nodes[L + 1];
        if (hi > lo) k_preorder<<<(hi - lo + 255) / 256, 256, 0, st>>>(nodes, lo, hi, size, pre);
    }
    float* d_box = dmalloc<float>(owned, 6 * (size_t)n_nodes);
    int32_t* d_parent = dmalloc<int32_t>(owned, n_nodes);
    int32_t* d_rank = dmalloc<int32_t>(owned, n);
    int32_t* d_pp = dmalloc<int32_t>(owned, n);
    if (n_nodes > 0) k_node_out<<<(n_nodes + 255) / 256, 256, 0, st>>>(nodes, n_nodes, pre, d_box, d_parent);
    k_prim_out<<<(n + 255) / 256, 256, 0, st>>>(final_id, leaf_parent, n, pre, d_rank, d_pp);
    ck(cudaGetLastError(), "outputs");
    t.leaf_order.resize(n);
    t.node_box.resize(n_nodes);
    t.node_parent.resize(n_nodes);
    std::vector<float> hbox(6 * (size_t)n_nodes);
    ck(cudaMemcpyAsync(t.leaf_order.data(), final_id, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st), "copy");
    ck(cudaMemcpyAsync(t.rank.data(), d_rank, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st), "copy");
    ck(cudaMemcpyAsync(t.prim_parent.data(), d_pp, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st), "copy");
    if (n_nodes > 0) {
        ck(cudaMemcpyAsync(hbox.data(), d_box, sizeof(float) * hbox.size(), cudaMemcpyDeviceToHost, st), "copy");
        ck(cudaMemcpyAsync(t.node_parent.data(), d_parent, sizeof(int32_t) * n_nodes, cudaMemcpyDeviceToHost, st),
           "copy");
    }
    ck(cudaStreamSynchronize(st), "outputs");
    for (int i = 0; i < n_nodes; i++)
        for (int j = 0; j < 3; j++) {
            t.node_box[i].lo[j] = hbox[6 * (size_t)i + j];
            t.node_box[i].hi[j] = hbox[6 * (size_t)i + 3 + j];
        }
    if (stats) {
        stats->levels = levels;
        stats->nodes = n_nodes;
    }
    return t;
}

}  // namespace cpppt_gb300
