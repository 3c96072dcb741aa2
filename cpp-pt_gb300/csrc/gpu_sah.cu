// Device build of the traversal tree: the binned-SAH binary BVH of
// build_wide_bvh (bvh.cpp) collapsed to 4-wide compressed nodes, bit for bit
// the host build's nodes and leaf order.
//
// The host build splits a node [start, start + count) of the primitive
// order at the first minimum of the 32-bin SAH cost over x, y, z, keeps
// both sides in their previous order (a stable partition, so every node's
// primitives stay sorted by insertion index), and falls back to halving in
// that order when no split exists (coincident centroids, or depth 56).  The
// resulting tree depends only on which primitives each node holds, so the
// device reproduces it node for node:
//
//   top levels  (nodes of more than kSmallSeg primitives): level-synchronous.
//     Every node is cut into chunks of kChunk primitives, one CTA each, that
//     bin into shared memory and merge into the node's bins with global
//     atomics (k_bin_chunks); one CTA per node picks the split from the bins
//     (k_split_big); the chunks then scatter their primitives into the other
//     order buffer, left side first, each chunk offset by the left counts of
//     the chunks before it (k_scatter_big).
//   subtrees    (nodes of at most kSmallSeg primitives): one CTA builds the
//     whole subtree depth first from a stack in shared memory
//     (k_subtree), with the same binning, decision and stable partition.
//   collapse    breadth-first, one launch set per 4-wide level: each entry
//     gathers its up-to-4 children (the child of largest SAH area opened
//     first, as the host does), an exclusive scan gives the next level's
//     queue positions, and each entry quantises its children's boxes in
//     double precision like the host (k_collapse, k_scan, k_emit).
//
// Bins hold, per axis and bin, the primitive count, the union of the boxes
// and the union of the centroids.  Unions are min / max, so their order does
// not matter; they are kept as order-preserving integer keys and combined
// with atomicMax (a minimum as the maximum of the inverted key), which makes
// every empty field zero.  No box value is -0.0: boxes are inflated by a
// positive delta (x - delta and x + delta are never -0.0 in round to
// nearest) and centroids are halves of their sums.  All float arithmetic is
// unfused (__fadd_rn and friends) in the host's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu_bvh.h"

namespace cpppt_gb300 {

namespace {

constexpr int kSahBins = 32;         // SahBuilder::kBins
constexpr int kDepthLimit = 56;      // SAH splits are tried above this depth
constexpr int kSmallSeg = 4096;      // nodes up to this size: one CTA builds the subtree
constexpr int kChunk = 4096;         // primitives per CTA in the top levels
constexpr int kThreads = 256;
constexpr int kStack = 128;          // subtree stack entries (tree depth is at most 56 + 27)
constexpr int kBinFields = 13;       // count, box lo xyz, box hi xyz, centroid lo xyz, centroid hi xyz
constexpr int kBinWords = 3 * kSahBins * kBinFields;

// status bits
constexpr int kErrStack = 1;
constexpr int kErrRange = 2;

__device__ __forceinline__ uint32_t fkey(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unkey(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// SahBuilder's AB::sah_area: dx * dy + dy * dz + dz * dx, unfused.
__device__ __forceinline__ float sah_area(const float lo[3], const float hi[3]) {
    const float dx = __fsub_rn(hi[0], lo[0]), dy = __fsub_rn(hi[1], lo[1]), dz = __fsub_rn(hi[2], lo[2]);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
}

struct Prims {
    const float4* lo;  // box lo xyz, centroid x
    const float4* hi;  // box hi xyz, centroid y
    const float* cz;   // centroid z
};

__device__ __forceinline__ float cen_axis(const Prims& P, int id, int axis) {
    return axis == 0 ? P.lo[id].w : (axis == 1 ? P.hi[id].w : P.cz[id]);
}

// A node's primitive range and bounds.  Keys: box lo / hi, centroid lo / hi
// (lo stored as the inverted key), valid when has_bounds.
struct Seg {
    int32_t start, count, node, depth;
    int32_t buf, has_bounds, pad0, pad1;
    uint32_t key[12];  // box lo xyz (~key), box hi xyz, centroid lo xyz (~key), centroid hi xyz
};

struct Node2 {
    float lo[3], hi[3];
    int32_t left, right, start, count;  // children (-1: leaf), leaf range
};

// The split of a node: axis < 0 for none (leaf or fallback).
struct Split {
    int32_t axis, bin, nleft, leaf;
    float lo, scale;
    uint32_t lkey[12], rkey[12];  // the two sides' bounds (Seg::key layout)
};

struct Chunk {
    int32_t seg, off, len, first;  // first: index of the segment's first chunk
};

__device__ __forceinline__ void seg_bounds(const uint32_t* key, float lo[3], float hi[3], float clo[3], float chi[3]) {
    for (int k = 0; k < 3; k++) {
        lo[k] = unkey(~key[k]);
        hi[k] = unkey(key[3 + k]);
        clo[k] = unkey(~key[6 + k]);
        chi[k] = unkey(key[9 + k]);
    }
}

__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
    int b = __float2int_rz(__fmul_rn(__fsub_rn(c, lo), scale));
    return b < 0 ? 0 : (b >= kSahBins ? kSahBins - 1 : b);
}

// Adds a run of primitives that share their bin on all three axes.
__device__ __forceinline__ void flush_run(uint32_t* bins, const int cur[3], uint32_t cnt, const uint32_t acc[12],
                                          const bool on[3]) {
    for (int a = 0; a < 3; a++) {
        if (!on[a]) continue;
        uint32_t* B = bins + (a * kSahBins + cur[a]) * kBinFields;
        atomicAdd(B, cnt);
        for (int f = 0; f < 12; f++) atomicMax(B + 1 + f, acc[f]);
    }
}

// Bins the primitives ord[begin, begin + len) into shared bins (zeroed by the
// caller).  Each thread takes a contiguous stretch and merges runs of
// primitives that fall into the same bins before touching shared memory.
__device__ void bin_range(const Prims& P, const int32_t* __restrict__ ord, int begin, int len, const float clo[3],
                          const float scale[3], const bool on[3], uint32_t* bins) {
    const int per = (len + blockDim.x - 1) / blockDim.x;
    const int b0 = begin + (int)threadIdx.x * per, e0 = min(b0 + per, begin + len);
    int cur[3] = {-1, -1, -1};
    uint32_t cnt = 0, acc[12];
    for (int i = b0; i < e0; i++) {
        const int id = ord[i];
        const float4 l = P.lo[id], h = P.hi[id];
        const float c[3] = {l.w, h.w, P.cz[id]};
        int b[3];
        for (int a = 0; a < 3; a++) b[a] = on[a] ? bin_of(c[a], clo[a], scale[a]) : 0;
        const uint32_t k[12] = {~fkey(l.x), ~fkey(l.y), ~fkey(l.z), fkey(h.x), fkey(h.y), fkey(h.z),
                                ~fkey(c[0]), ~fkey(c[1]), ~fkey(c[2]), fkey(c[0]), fkey(c[1]), fkey(c[2])};
        if (cnt > 0 && b[0] == cur[0] && b[1] == cur[1] && b[2] == cur[2]) {
            cnt++;
            for (int f = 0; f < 12; f++) acc[f] = max(acc[f], k[f]);
        } else {
            if (cnt > 0) flush_run(bins, cur, cnt, acc, on);
            cnt = 1;
            for (int a = 0; a < 3; a++) cur[a] = b[a];
            for (int f = 0; f < 12; f++) acc[f] = k[f];
        }
    }
    if (cnt > 0) flush_run(bins, cur, cnt, acc, on);
}

// Union of the bins below (inclusive prefix) or above (inclusive suffix) a
// lane's bin, over one warp (lane = bin).
__device__ __forceinline__ void warp_scan(uint32_t& cnt, uint32_t k[12], bool suffix) {
    const int lane = threadIdx.x & 31;
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t oc = suffix ? __shfl_down_sync(0xffffffffu, cnt, d) : __shfl_up_sync(0xffffffffu, cnt, d);
        uint32_t ok[12];
        for (int f = 0; f < 12; f++)
            ok[f] = suffix ? __shfl_down_sync(0xffffffffu, k[f], d) : __shfl_up_sync(0xffffffffu, k[f], d);
        const bool take = suffix ? lane + d < 32 : lane >= d;
        if (take) {
            cnt += oc;
            for (int f = 0; f < 12; f++) k[f] = max(k[f], ok[f]);
        }
    }
}

// The host's split decision from the bins (SahBuilder::build): warp w < 3
// evaluates axis w; the first strict minimum over (axis, bin) wins.  Writes
// *out (leaf, axis or fallback) from thread 0; the caller synchronises.
// The node's box and centroid bounds come from s.key.  All threads of the
// CTA call it (it synchronises once).
__device__ void decide(const uint32_t* bins, const Seg& s, int max_leaf, Split* out, float* s_cost, int* s_bin) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float lo[3], hi[3], clo[3], chi[3];
    seg_bounds(s.key, lo, hi, clo, chi);
    const bool try_sah = s.depth < kDepthLimit;
    if (warp < 3) {
        const int a = warp;
        float best = __int_as_float(0x7f800000);  // +inf
        int bbin = -1;
        if (try_sah && chi[a] > clo[a]) {
            const uint32_t* B = bins + (a * kSahBins + lane) * kBinFields;
            uint32_t pc = B[0], sc = B[0], pk[12], sk[12];
            for (int f = 0; f < 12; f++) pk[f] = sk[f] = B[1 + f];
            warp_scan(pc, pk, false);
            warp_scan(sc, sk, true);
            // right side of the split after bin `lane`: the suffix from lane + 1
            const uint32_t rc = __shfl_down_sync(0xffffffffu, sc, 1);
            uint32_t rk[12];
            for (int f = 0; f < 12; f++) rk[f] = __shfl_down_sync(0xffffffffu, sk[f], 1);
            float cost = __int_as_float(0x7fffffff);  // NaN: no candidate
            if (lane < kSahBins - 1 && pc != 0 && rc != 0) {
                float llo[3], lhi[3], rlo[3], rhi[3];
                for (int k = 0; k < 3; k++) {
                    llo[k] = unkey(~pk[k]);
                    lhi[k] = unkey(pk[3 + k]);
                    rlo[k] = unkey(~rk[k]);
                    rhi[k] = unkey(rk[3 + k]);
                }
                cost = __fadd_rn(__fmul_rn(sah_area(llo, lhi), __uint2float_rn(pc)),
                                 __fmul_rn(sah_area(rlo, rhi), __uint2float_rn(rc)));
            }
            // first strict minimum below +inf: the sequential scan's choice
            for (int b = 0; b < kSahBins - 1; b++) {
                const float cb = __shfl_sync(0xffffffffu, cost, b);
                if (cb < best) {
                    best = cb;
                    bbin = b;
                }
            }
        }
        if (lane == 0) {
            s_cost[a] = best;
            s_bin[a] = bbin;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float best = __int_as_float(0x7f800000);
        int axis = -1;
        for (int a = 0; a < 3; a++)
            if (s_bin[a] >= 0 && s_cost[a] < best) {
                best = s_cost[a];
                axis = a;
            }
        const float area = sah_area(lo, hi);
        const float leaf_cost = __fmul_rn(area, __int2float_rn(s.count));
        const float trav = __fmul_rn(area, 1.0f);
        out->leaf = s.count <= max_leaf && (axis < 0 || __fadd_rn(best, trav) >= leaf_cost);
        out->axis = out->leaf ? -1 : axis;
        out->bin = axis >= 0 ? s_bin[axis] : -1;
        out->nleft = 0;
        if (!out->leaf && axis >= 0) {
            out->lo = clo[axis];
            out->scale = __fdiv_rn((float)kSahBins, __fsub_rn(chi[axis], clo[axis]));
            for (int f = 0; f < 12; f++) out->lkey[f] = out->rkey[f] = 0;
            uint32_t nl = 0;
            for (int b = 0; b < kSahBins; b++) {
                const uint32_t* B = bins + (axis * kSahBins + b) * kBinFields;
                uint32_t* K = b <= out->bin ? out->lkey : out->rkey;
                if (b <= out->bin) nl += B[0];
                for (int f = 0; f < 12; f++) K[f] = max(K[f], B[1 + f]);
            }
            out->nleft = (int)nl;
        }
    }
}

// Bounds of ord[begin, begin + len) into key[12] (shared, zeroed by the caller).
__device__ void reduce_bounds(const Prims& P, const int32_t* __restrict__ ord, int begin, int len, uint32_t* key) {
    uint32_t k[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = begin + threadIdx.x; i < begin + len; i += blockDim.x) {
        const int id = ord[i];
        const float4 l = P.lo[id], h = P.hi[id];
        const float c[3] = {l.w, h.w, P.cz[id]};
        const uint32_t e[12] = {~fkey(l.x), ~fkey(l.y), ~fkey(l.z), fkey(h.x), fkey(h.y), fkey(h.z),
                                ~fkey(c[0]), ~fkey(c[1]), ~fkey(c[2]), fkey(c[0]), fkey(c[1]), fkey(c[2])};
        for (int f = 0; f < 12; f++) k[f] = max(k[f], e[f]);
    }
    for (int f = 0; f < 12; f++) {
        uint32_t v = k[f];
        for (int d = 16; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, d));
        if ((threadIdx.x & 31) == 0) atomicMax(key + f, v);
    }
}

// Stable scatter of ord[seg_start + begin, + len) (a part of a node of the
// split sp): primitives on the left side go to dst[seg_start + left rank],
// the others to dst[seg_start + nleft + right rank].  left_before: left-side
// primitives of the node before `begin`.
__device__ void scatter(const Prims& P, const int32_t* __restrict__ src, int32_t* __restrict__ dst, int seg_start,
                        int begin, int len, int left_before, const Split& sp, int* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int run = left_before;
    for (int base = 0; base < len; base += blockDim.x) {
        const int i = base + (int)threadIdx.x;
        int id = 0;
        bool left = false;
        if (i < len) {
            id = src[seg_start + begin + i];
            left = bin_of(cen_axis(P, id, sp.axis), sp.lo, sp.scale) <= sp.bin;
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, left);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < nw; w++) {
            const int c = s_warp[w];
            if (w < warp) before += c;
            total += c;
        }
        if (i < len) {
            const int lrank = run + before + __popc(bal & ((1u << lane) - 1u));  // left before i in the node
            const int pos = begin + i;                                          // position in the node
            dst[seg_start + (left ? lrank : sp.nleft + (pos - lrank))] = id;
        }
        run += total;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Primitive boxes and the root's bounds.
// ---------------------------------------------------------------------------
__global__ void k_scene_bounds(const float* __restrict__ tv, int n, uint32_t* __restrict__ key6) {
    uint32_t k[6] = {0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += gridDim.x * blockDim.x) {
        const float* v = tv + 3 * (size_t)i;
        for (int a = 0; a < 3; a++) {
            k[a] = max(k[a], ~fkey(v[a]));
            k[3 + a] = max(k[3 + a], fkey(v[a]));
        }
    }
    for (int f = 0; f < 6; f++) {
        uint32_t v = k[f];
        for (int d = 16; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, d));
        if ((threadIdx.x & 31) == 0) atomicMax(key6 + f, v);
    }
}

// Inflated boxes and centroids (build_wide_bvh), the identity order, and the
// root's bounds.  The inflation delta is computed from the scene box, as the
// host does, by every thread.
__global__ void k_prims(const float* __restrict__ tv, int n, const uint32_t* __restrict__ key6, float4* __restrict__ plo,
                        float4* __restrict__ phi, float* __restrict__ pcz, int32_t* __restrict__ ord,
                        Seg* __restrict__ root, float* __restrict__ delta_out) {
    float ext = 0.0f, mag = 0.0f;
    for (int a = 0; a < 3; a++) {
        const float lo = unkey(~key6[a]), hi = unkey(key6[3 + a]);
        ext = fmaxf(ext, __fsub_rn(hi, lo));
        mag = fmaxf(mag, fmaxf(fabsf(hi), fabsf(lo)));
    }
    const float delta = __fmul_rn(__fadd_rn(__fadd_rn(ext, mag), 1e-3f), 1.0f / 262144.0f);
    if (blockIdx.x == 0 && threadIdx.x == 0) *delta_out = delta;
    uint32_t k[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* v = tv + 9 * (size_t)i;
        float lo[3], hi[3], c[3];
        for (int a = 0; a < 3; a++) {
            // Triangle::get_bounds order: min(min(a, b), c)
            const float x0 = v[a], x1 = v[3 + a], x2 = v[6 + a];
            float mn = x0 < x1 ? x0 : x1, mx = x0 > x1 ? x0 : x1;
            mn = mn < x2 ? mn : x2;
            mx = mx > x2 ? mx : x2;
            lo[a] = __fsub_rn(mn, delta);
            hi[a] = __fadd_rn(mx, delta);
            c[a] = __fmul_rn(0.5f, __fadd_rn(lo[a], hi[a]));
        }
        plo[i] = make_float4(lo[0], lo[1], lo[2], c[0]);
        phi[i] = make_float4(hi[0], hi[1], hi[2], c[1]);
        pcz[i] = c[2];
        ord[i] = i;
        const uint32_t e[12] = {~fkey(lo[0]), ~fkey(lo[1]), ~fkey(lo[2]), fkey(hi[0]), fkey(hi[1]), fkey(hi[2]),
                                ~fkey(c[0]),  ~fkey(c[1]),  ~fkey(c[2]),  fkey(c[0]),  fkey(c[1]),  fkey(c[2])};
        for (int f = 0; f < 12; f++) k[f] = max(k[f], e[f]);
    }
    for (int f = 0; f < 12; f++) {
        uint32_t v = k[f];
        for (int d = 16; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, d));
        if ((threadIdx.x & 31) == 0) atomicMax(root->key + f, v);
    }
}

// ---------------------------------------------------------------------------
// Top levels.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_bin_chunks(Prims P, const Chunk* __restrict__ chunks,
                                                          const Seg* __restrict__ segs,
                                                          const int32_t* __restrict__ ord,
                                                          uint32_t* __restrict__ gbins,
                                                          int32_t* __restrict__ chunk_cnt) {
    __shared__ uint32_t bins[kBinWords];
    const Chunk ch = chunks[blockIdx.x];
    const Seg& s = segs[ch.seg];
    for (int i = threadIdx.x; i < kBinWords; i += blockDim.x) bins[i] = 0;
    float lo[3], hi[3], clo[3], chi[3], scale[3];
    bool on[3];
    seg_bounds(s.key, lo, hi, clo, chi);
    for (int a = 0; a < 3; a++) {
        on[a] = s.depth < kDepthLimit && chi[a] > clo[a];
        scale[a] = on[a] ? __fdiv_rn((float)kSahBins, __fsub_rn(chi[a], clo[a])) : 0.0f;
    }
    __syncthreads();
    bin_range(P, ord, s.start + ch.off, ch.len, clo, scale, on, bins);
    __syncthreads();
    uint32_t* G = gbins + (size_t)ch.seg * kBinWords;
    for (int i = threadIdx.x; i < 3 * kSahBins; i += blockDim.x) {
        const uint32_t* B = bins + i * kBinFields;
        chunk_cnt[(size_t)blockIdx.x * 3 * kSahBins + i] = (int32_t)B[0];
        if (B[0] == 0) continue;
        atomicAdd(G + i * kBinFields, B[0]);
        for (int f = 1; f < kBinFields; f++) atomicMax(G + i * kBinFields + f, B[f]);
    }
}

struct LevelOut {
    Seg* big;        // next level's large nodes
    Seg* small;      // subtree roots
    int32_t* counts;  // [0] next large nodes, [1] subtree roots, [2] node ids, [3] status
    int32_t max_big, max_small, max_nodes;
};

__device__ __forceinline__ void emit_seg(const LevelOut& L, const Seg& c) {
    if (c.count > kSmallSeg) {
        const int j = atomicAdd(L.counts + 0, 1);
        if (j < L.max_big) L.big[j] = c;
        else atomicOr(L.counts + 3, kErrRange);
    } else {
        const int j = atomicAdd(L.counts + 1, 1);
        if (j < L.max_small) L.small[j] = c;
        else atomicOr(L.counts + 3, kErrRange);
    }
}

__global__ void __launch_bounds__(kThreads) k_split_big(const Seg* __restrict__ segs, const uint32_t* __restrict__ gbins,
                                                         Split* __restrict__ splits, Node2* __restrict__ nodes,
                                                         LevelOut L, int max_leaf, int cur) {
    __shared__ uint32_t bins[kBinWords];
    __shared__ Split sp;
    __shared__ float s_cost[3];
    __shared__ int s_bin[3];
    const Seg s = segs[blockIdx.x];
    const uint32_t* G = gbins + (size_t)blockIdx.x * kBinWords;
    for (int i = threadIdx.x; i < kBinWords; i += blockDim.x) bins[i] = G[i];
    __syncthreads();
    decide(bins, s, max_leaf, &sp, s_cost, s_bin);
    __syncthreads();
    if (threadIdx.x != 0) return;
    splits[blockIdx.x] = sp;
    if (sp.axis < 0) {  // no SAH split (never a leaf at this size): the subtree kernel halves it
        Seg c = s;
        c.buf = cur;
        const int j = atomicAdd(L.counts + 1, 1);
        if (j < L.max_small) L.small[j] = c;
        else atomicOr(L.counts + 3, kErrRange);
        return;
    }
    const int id = atomicAdd(L.counts + 2, 2);
    if (id + 2 > L.max_nodes || s.node >= L.max_nodes) {
        atomicOr(L.counts + 3, kErrRange);
        return;
    }
    Node2 nd;
    float clo[3], chi[3];
    seg_bounds(s.key, nd.lo, nd.hi, clo, chi);
    nd.left = id;
    nd.right = id + 1;
    nd.start = s.start;
    nd.count = 0;
    nodes[s.node] = nd;
    Seg c{};
    c.depth = s.depth + 1;
    c.buf = 1 - cur;
    c.has_bounds = 1;
    c.start = s.start;
    c.count = sp.nleft;
    c.node = id;
    for (int f = 0; f < 12; f++) c.key[f] = sp.lkey[f];
    emit_seg(L, c);
    c.start = s.start + sp.nleft;
    c.count = s.count - sp.nleft;
    c.node = id + 1;
    for (int f = 0; f < 12; f++) c.key[f] = sp.rkey[f];
    emit_seg(L, c);
}

__global__ void __launch_bounds__(kThreads) k_scatter_big(Prims P, const Chunk* __restrict__ chunks,
                                                           const Seg* __restrict__ segs,
                                                           const Split* __restrict__ splits,
                                                           const int32_t* __restrict__ chunk_cnt,
                                                           const int32_t* __restrict__ src, int32_t* __restrict__ dst) {
    __shared__ int s_warp[kThreads / 32];
    __shared__ int s_before;
    const Chunk ch = chunks[blockIdx.x];
    const Split sp = splits[ch.seg];
    if (sp.axis < 0) return;
    if (threadIdx.x == 0) s_before = 0;
    __syncthreads();
    // left-side primitives in the segment's earlier chunks
    int mine = 0;
    for (int c = ch.first + (int)threadIdx.x; c < (int)blockIdx.x; c += blockDim.x)
        for (int b = 0; b <= sp.bin; b++) mine += chunk_cnt[(size_t)c * 3 * kSahBins + sp.axis * kSahBins + b];
    for (int d = 16; d > 0; d >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, d);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&s_before, mine);
    __syncthreads();
    scatter(P, src, dst, segs[ch.seg].start, ch.off, ch.len, s_before, sp, s_warp);
}

// ---------------------------------------------------------------------------
// Subtrees: one CTA per root, depth first.
// ---------------------------------------------------------------------------
struct SubCtx {
    Prims P;
    int32_t* ord[2];
    int32_t* out_order;
    Node2* nodes;
    int32_t* counts;  // [2] node ids, [3] status
    int32_t max_leaf, max_nodes;
};

__global__ void __launch_bounds__(kThreads) k_subtree(const Seg* __restrict__ roots, SubCtx C) {
    __shared__ uint32_t bins[kBinWords];
    __shared__ Seg stack[kStack];
    __shared__ Seg s;
    __shared__ Split sp;
    __shared__ int sp_top;
    __shared__ float s_cost[3];
    __shared__ int s_bin[3];
    __shared__ int s_warp[kThreads / 32];
    if (threadIdx.x == 0) {
        stack[0] = roots[blockIdx.x];
        sp_top = 1;
    }
    __syncthreads();
    for (;;) {
        // every thread reads the stack top before thread 0 pops it
        const int top = sp_top;
        __syncthreads();
        if (top == 0) break;
        if (threadIdx.x == 0) {
            s = stack[sp_top - 1];
            sp_top--;
            if (!s.has_bounds)
                for (int f = 0; f < 12; f++) s.key[f] = 0;
        }
        for (int i = threadIdx.x; i < kBinWords; i += blockDim.x) bins[i] = 0;
        __syncthreads();
        const int32_t* src = C.ord[s.buf];
        if (!s.has_bounds) {
            reduce_bounds(C.P, src, s.start, s.count, s.key);
            __syncthreads();
        }
        bool leaf = s.count <= 1;
        if (!leaf) {
            float lo[3], hi[3], clo[3], chi[3], scale[3];
            bool on[3];
            seg_bounds(s.key, lo, hi, clo, chi);
            for (int a = 0; a < 3; a++) {
                on[a] = s.depth < kDepthLimit && chi[a] > clo[a];
                scale[a] = on[a] ? __fdiv_rn((float)kSahBins, __fsub_rn(chi[a], clo[a])) : 0.0f;
            }
            if (on[0] || on[1] || on[2]) bin_range(C.P, src, s.start, s.count, clo, scale, on, bins);
            __syncthreads();
            decide(bins, s, C.max_leaf, &sp, s_cost, s_bin);
            __syncthreads();
            leaf = sp.leaf;
        }
        if (leaf) {
            for (int i = threadIdx.x; i < s.count; i += blockDim.x) C.out_order[s.start + i] = src[s.start + i];
            if (threadIdx.x == 0 && s.node < C.max_nodes) {
                Node2 nd;
                float clo[3], chi[3];
                seg_bounds(s.key, nd.lo, nd.hi, clo, chi);
                nd.left = nd.right = -1;
                nd.start = s.start;
                nd.count = s.count;
                C.nodes[s.node] = nd;
            }
            __syncthreads();
            continue;
        }
        if (sp.axis >= 0) scatter(C.P, src, C.ord[1 - s.buf], s.start, 0, s.count, 0, sp, s_warp);
        if (threadIdx.x == 0) {
            const int id = atomicAdd(C.counts + 2, 2);
            Node2 nd;
            float clo[3], chi[3];
            seg_bounds(s.key, nd.lo, nd.hi, clo, chi);
            nd.left = id;
            nd.right = id + 1;
            nd.start = s.start;
            nd.count = 0;
            if (s.node < C.max_nodes) C.nodes[s.node] = nd;
            if (id + 2 > C.max_nodes) {
                atomicOr(C.counts + 3, kErrRange);
                sp_top = 0;
            } else if (sp_top + 2 > kStack) {
                atomicOr(C.counts + 3, kErrStack);
                sp_top = 0;  // give up on this subtree; the host reports the error
            } else {
                Seg l{}, r{};
                l.depth = r.depth = s.depth + 1;
                l.node = id;
                r.node = id + 1;
                l.start = s.start;
                if (sp.axis >= 0) {
                    l.count = sp.nleft;
                    l.buf = r.buf = 1 - s.buf;
                    l.has_bounds = r.has_bounds = 1;
                    for (int f = 0; f < 12; f++) {
                        l.key[f] = sp.lkey[f];
                        r.key[f] = sp.rkey[f];
                    }
                } else {  // no split: halve in the current order
                    l.count = s.count / 2;
                    l.buf = r.buf = s.buf;
                    l.has_bounds = r.has_bounds = 0;
                }
                r.start = s.start + l.count;
                r.count = s.count - l.count;
                stack[sp_top] = r;
                stack[sp_top + 1] = l;
                sp_top += 2;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Collapse to 4-wide nodes, one breadth-first level at a time.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float node_area(const Node2& n) { return sah_area(n.lo, n.hi); }

__global__ void k_collapse(const int32_t* __restrict__ q, int nq, const Node2* __restrict__ nodes,
                           int4* __restrict__ ch_out, int32_t* __restrict__ nc_out, int32_t* __restrict__ nint_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const int n2 = q[i];
    int ch[4] = {-1, -1, -1, -1};
    int nc = 0;
    if (nodes[n2].left < 0) {
        ch[nc++] = n2;  // a root that is a leaf
    } else {
        ch[nc++] = nodes[n2].left;
        ch[nc++] = nodes[n2].right;
        while (nc < 4) {
            int pick = -1;
            float best = -1.0f;
            for (int k = 0; k < nc; k++)
                if (nodes[ch[k]].left >= 0 && node_area(nodes[ch[k]]) > best) {
                    best = node_area(nodes[ch[k]]);
                    pick = k;
                }
            if (pick < 0) break;
            const int c = ch[pick];
            ch[pick] = nodes[c].left;
            ch[nc++] = nodes[c].right;
        }
    }
    int nint = 0;
    for (int k = 0; k < nc; k++)
        if (nodes[ch[k]].left >= 0) nint++;
    ch_out[i] = make_int4(ch[0], ch[1], ch[2], ch[3]);
    nc_out[i] = nc;
    nint_out[i] = nint;
}

// Exclusive scan of v[0, n) in place, total to *total; one CTA of 1024.
__global__ void __launch_bounds__(1024) k_scan(int32_t* __restrict__ v, int n, int32_t* __restrict__ total) {
    __shared__ int s_warp[32];
    __shared__ int s_run;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_run = 0;
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + (int)threadIdx.x;
        const int x = i < n ? v[i] : 0;
        int inc = x;
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += y;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            int w = s_warp[lane];
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= d) w += y;
            }
            s_warp[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const int run = s_run;
        if (i < n) v[i] = run + (warp > 0 ? s_warp[warp - 1] : 0) + inc - x;
        __syncthreads();
        if (threadIdx.x == 0) s_run = run + s_warp[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = s_run;
}

__global__ void k_emit(const int32_t* __restrict__ q, int nq, int level_base, int next_base,
                       const int4* __restrict__ ch_in, const int32_t* __restrict__ nc_in,
                       const int32_t* __restrict__ offs, const Node2* __restrict__ nodes, uint4* __restrict__ out,
                       int32_t* __restrict__ q_next, int32_t* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const int4 c4 = ch_in[i];
    const int ch[4] = {c4.x, c4.y, c4.z, c4.w};
    const int nc = nc_in[i];
    float nlo[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
    float nhi[3] = {__int_as_float(0xff800000), __int_as_float(0xff800000), __int_as_float(0xff800000)};
    for (int k = 0; k < nc; k++) {
        const Node2& c = nodes[ch[k]];
        for (int a = 0; a < 3; a++) {
            nlo[a] = nlo[a] < c.lo[a] ? nlo[a] : c.lo[a];
            nhi[a] = nhi[a] > c.hi[a] ? nhi[a] : c.hi[a];
        }
    }
    uint32_t w[16];
    for (int k = 0; k < 16; k++) w[k] = 0;
    double s[3];
    uint32_t ebits[3];
    for (int a = 0; a < 3; a++) {
        const double E = __dsub_rn((double)nhi[a], (double)nlo[a]);
        double m = __ddiv_rn(E, 254.0);
        m = m > 1e-30 ? m : 1e-30;
        int e;
        frexp(m, &e);
        if (e < -126) e = -126;
        if (e > 127) {
            atomicOr(status, kErrRange);
            e = 127;
        }
        s[a] = ldexp(1.0, e);
        ebits[a] = (uint32_t)(e + 127);
        w[a] = __float_as_uint(nlo[a]);
    }
    w[3] = ebits[0] | (ebits[1] << 8) | (ebits[2] << 16);
    uint32_t qlo[3][4], qhi[3][4];
    for (int a = 0; a < 3; a++)
        for (int k = 0; k < 4; k++) {
            qlo[a][k] = 255;
            qhi[a][k] = 0;
        }
    uint32_t refs[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
    int nint = 0;
    for (int k = 0; k < nc; k++) {
        const Node2& c = nodes[ch[k]];
        for (int a = 0; a < 3; a++) {
            const double p = (double)nlo[a];
            double lo = floor(__ddiv_rn(__dsub_rn((double)c.lo[a], p), s[a]));
            double hi = ceil(__ddiv_rn(__dsub_rn((double)c.hi[a], p), s[a]));
            while (lo > 0 && __dadd_rn(p, __dmul_rn(lo, s[a])) > (double)c.lo[a]) lo -= 1;
            while (hi < 255 && __dadd_rn(p, __dmul_rn(hi, s[a])) < (double)c.hi[a]) hi += 1;
            lo = fmax(0.0, fmin(255.0, lo));
            hi = fmax(0.0, fmin(255.0, hi));
            qlo[a][k] = (uint32_t)lo;
            qhi[a][k] = (uint32_t)hi;
        }
        if (c.left < 0) {
            if (c.count > 16) atomicOr(status, kErrRange);
            refs[k] = kLeafBit | ((uint32_t)(c.count - 1) << 27) | (uint32_t)c.start;  // make_leaf_ref
        } else {
            const int j = offs[i] + nint++;
            refs[k] = (uint32_t)(next_base + j);
            q_next[j] = ch[k];
        }
    }
    for (int a = 0; a < 3; a++) {
        w[4 + a] = qlo[a][0] | (qlo[a][1] << 8) | (qlo[a][2] << 16) | (qlo[a][3] << 24);
    }
    w[7] = qhi[0][0] | (qhi[0][1] << 8) | (qhi[0][2] << 16) | (qhi[0][3] << 24);
    w[8] = qhi[1][0] | (qhi[1][1] << 8) | (qhi[1][2] << 16) | (qhi[1][3] << 24);
    w[9] = qhi[2][0] | (qhi[2][1] << 8) | (qhi[2][2] << 16) | (qhi[2][3] << 24);
    for (int k = 0; k < 4; k++) w[10 + k] = refs[k];
    uint4* o = out + 4 * (size_t)(level_base + i);
    for (int k = 0; k < 4; k++) o[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
}

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string("device SAH build: ") + what + ": " + cudaGetErrorString(e));
    }
}

template <class T>
T* dmalloc(std::vector<void*>& owned, size_t n) {
    void* p = nullptr;
    ck(cudaMalloc(&p, sizeof(T) * (n ? n : 1)), "cudaMalloc");
    owned.push_back(p);
    return static_cast<T*>(p);
}

int grid_for(int n, int threads) { return std::max(1, std::min((n + threads - 1) / threads, 152 * 8)); }

}  // namespace

WideBVH build_wide_bvh_device(const float* tri_v, int n, int max_leaf, cudaStream_t st, WideBuildStats* stats) {
    if (max_leaf < 1 || max_leaf > 16) throw std::invalid_argument("max_leaf must be in [1,16]");
    if (n <= 0) return build_wide_bvh(tri_v, n, max_leaf, 1);
    std::vector<void*> owned;
    struct Free {
        std::vector<void*>& v;
        ~Free() { for (void* p : v) cudaFree(p); }
    } guard{owned};
    int32_t* h = nullptr;  // pinned counters
    ck(cudaMallocHost(&h, 8 * sizeof(int32_t)), "cudaMallocHost");
    struct FreeHost {
        int32_t* p;
        ~FreeHost() { cudaFreeHost(p); }
    } hguard{h};

    const int max_big = n / kSmallSeg + 2;
    const int max_small = 4 * (n / kSmallSeg) + 16;
    const int max_chunks = n / kChunk + max_big + 2;
    float* d_tv = dmalloc<float>(owned, 9 * (size_t)n);
    float4* plo = dmalloc<float4>(owned, n);
    float4* phi = dmalloc<float4>(owned, n);
    float* pcz = dmalloc<float>(owned, n);
    int32_t* ord[2] = {dmalloc<int32_t>(owned, n), dmalloc<int32_t>(owned, n)};
    int32_t* out_order = dmalloc<int32_t>(owned, n);
    Node2* nodes = dmalloc<Node2>(owned, 2 * (size_t)n);
    Seg* big[2] = {dmalloc<Seg>(owned, max_big), dmalloc<Seg>(owned, max_big)};
    Seg* small = dmalloc<Seg>(owned, max_small);
    Split* splits = dmalloc<Split>(owned, max_big);
    Chunk* d_chunks = dmalloc<Chunk>(owned, max_chunks);
    int32_t* chunk_cnt = dmalloc<int32_t>(owned, (size_t)max_chunks * 3 * kSahBins);
    uint32_t* gbins = dmalloc<uint32_t>(owned, (size_t)max_big * kBinWords);
    uint32_t* key6 = dmalloc<uint32_t>(owned, 6);
    float* d_delta = dmalloc<float>(owned, 1);
    int32_t* counts = dmalloc<int32_t>(owned, 4);  // next big, small, node ids, status

    ck(cudaMemcpyAsync(d_tv, tri_v, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice, st), "upload");
    ck(cudaMemsetAsync(key6, 0, 6 * sizeof(uint32_t), st), "memset");
    // the root: node 0, bounds reduced by k_prims
    Seg root{};
    root.start = 0;
    root.count = n;
    root.node = 0;
    root.depth = 0;
    root.buf = 0;
    root.has_bounds = 1;
    Seg* d_root = n > kSmallSeg ? big[0] : small;
    ck(cudaMemcpyAsync(d_root, &root, sizeof(Seg), cudaMemcpyHostToDevice, st), "root");
    // next-level large nodes, subtree roots, node ids (the root is node 0), status
    const int32_t init[4] = {0, n > kSmallSeg ? 0 : 1, 1, 0};
    ck(cudaMemcpyAsync(counts, init, sizeof(init), cudaMemcpyHostToDevice, st), "counts");
    k_scene_bounds<<<grid_for(3 * n, 256), 256, 0, st>>>(d_tv, n, key6);
    k_prims<<<grid_for(n, 256), 256, 0, st>>>(d_tv, n, key6, plo, phi, pcz, ord[0], d_root, d_delta);
    ck(cudaGetLastError(), "primitive boxes");
    const Prims P{plo, phi, pcz};

    // top levels
    int n_big = n > kSmallSeg ? 1 : 0, cur = 0, top_levels = 0;
    std::vector<Seg> hseg;
    std::vector<Chunk> hch;
    while (n_big > 0) {
        hseg.resize(n_big);
        ck(cudaMemcpyAsync(hseg.data(), big[cur], sizeof(Seg) * n_big, cudaMemcpyDeviceToHost, st), "segments");
        ck(cudaStreamSynchronize(st), "segments");
        hch.clear();
        for (int s = 0; s < n_big; s++) {
            const int first = (int)hch.size();
            for (int off = 0; off < hseg[s].count; off += kChunk)
                hch.push_back({s, off, std::min(kChunk, hseg[s].count - off), first});
        }
        if ((int)hch.size() > max_chunks) throw std::runtime_error("device SAH build: chunk table overflow");
        ck(cudaMemcpyAsync(d_chunks, hch.data(), sizeof(Chunk) * hch.size(), cudaMemcpyHostToDevice, st), "chunks");
        ck(cudaMemsetAsync(gbins, 0, sizeof(uint32_t) * kBinWords * (size_t)n_big, st), "memset");
        ck(cudaMemsetAsync(counts, 0, sizeof(int32_t), st), "memset");
        k_bin_chunks<<<(int)hch.size(), kThreads, 0, st>>>(P, d_chunks, big[cur], ord[cur], gbins, chunk_cnt);
        LevelOut L{big[1 - cur], small, counts, max_big, max_small, 2 * n};
        k_split_big<<<n_big, kThreads, 0, st>>>(big[cur], gbins, splits, nodes, L, max_leaf, cur);
        k_scatter_big<<<(int)hch.size(), kThreads, 0, st>>>(P, d_chunks, big[cur], splits, chunk_cnt, ord[cur],
                                                            ord[1 - cur]);
        ck(cudaGetLastError(), "top level");
        ck(cudaMemcpyAsync(h, counts, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "counts");
        ck(cudaStreamSynchronize(st), "top level");
        if (h[3] != 0) throw std::runtime_error("device SAH build: top-level overflow");
        n_big = h[0];
        cur = 1 - cur;
        top_levels++;
    }
    ck(cudaMemcpyAsync(h, counts, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "counts");
    ck(cudaStreamSynchronize(st), "counts");
    const int n_small = h[1];
    SubCtx C{P, {ord[0], ord[1]}, out_order, nodes, counts, max_leaf, 2 * n};
    if (n_small > 0) k_subtree<<<n_small, kThreads, 0, st>>>(small, C);
    ck(cudaGetLastError(), "subtrees");
    ck(cudaMemcpyAsync(h, counts, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "counts");
    ck(cudaStreamSynchronize(st), "subtrees");
    if (h[3] != 0) throw std::runtime_error("device SAH build: subtree stack or node overflow");
    const int n_node2 = h[2];
    if (n_node2 < 1 || n_node2 > 2 * n - 1) throw std::runtime_error("device SAH build: node count out of range");

    // collapse, breadth first
    int32_t* q[2] = {dmalloc<int32_t>(owned, n_node2), dmalloc<int32_t>(owned, n_node2)};
    int4* chb = dmalloc<int4>(owned, n_node2);
    int32_t* ncb = dmalloc<int32_t>(owned, n_node2);
    int32_t* offs = dmalloc<int32_t>(owned, n_node2);
    uint4* wide = dmalloc<uint4>(owned, 4 * (size_t)n_node2);
    ck(cudaMemsetAsync(q[0], 0, sizeof(int32_t), st), "root queue");  // node 0
    ck(cudaMemsetAsync(counts + 3, 0, sizeof(int32_t), st), "status");
    int nq = 1, base = 0, qc = 0, depth = 0;
    while (nq > 0) {
        depth++;
        const int g = (nq + 255) / 256;
        k_collapse<<<g, 256, 0, st>>>(q[qc], nq, nodes, chb, ncb, offs);
        k_scan<<<1, 1024, 0, st>>>(offs, nq, counts);
        k_emit<<<g, 256, 0, st>>>(q[qc], nq, base, base + nq, chb, ncb, offs, nodes, wide, q[1 - qc], counts + 3);
        ck(cudaGetLastError(), "collapse");
        ck(cudaMemcpyAsync(h, counts, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "counts");
        ck(cudaStreamSynchronize(st), "collapse");
        if (h[3] != 0) throw std::runtime_error("scene coordinates out of range");
        base += nq;
        nq = h[0];
        qc = 1 - qc;
        if (base + nq > n_node2) throw std::runtime_error("device SAH build: collapse overflow");
    }
    WideBVH out;
    out.max_leaf = max_leaf;
    out.max_depth = depth;
    out.nodes.resize(base);
    out.tri_order.resize(n);
    ck(cudaMemcpyAsync(out.nodes.data(), wide, sizeof(WideNode) * (size_t)base, cudaMemcpyDeviceToHost, st), "nodes");
    ck(cudaMemcpyAsync(out.tri_order.data(), out_order, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st), "order");
    ck(cudaMemcpyAsync(&out.inflate, d_delta, sizeof(float), cudaMemcpyDeviceToHost, st), "delta");
    ck(cudaStreamSynchronize(st), "outputs");
    if (stats) {
        stats->top_levels = top_levels;
        stats->subtrees = n_small;
        stats->binary_nodes = n_node2;
        stats->wide_levels = depth;
    }
    return out;
}

}  // namespace cpppt_gb300
