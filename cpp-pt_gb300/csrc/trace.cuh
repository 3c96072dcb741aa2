// Device traversal of the compressed 4-wide BVH with the reference's exact
// closest-hit semantics (see bvh.h for why this reproduces BVH::intersect).
#pragma once
#include "dev_types.h"

namespace cpppt_gb300 {

// Launch shape of the traversal kernels (threads per CTA, resident CTAs per
// SM; the grid is the latter times the SM count) and the number of top wide
// nodes (breadth-first, so the top levels) each CTA stages in shared memory.
// Measured on the 1M-triangle soup at 1080p, 64 spp.  With the earlier node
// phase (full child sort, 64-ray chunks), staging paid: 256x4 with 256
// nodes 273.0 Mpaths/s, 512x2 with 1024 nodes 275.2, 1024x1 with 2048
// nodes 277.3, with 3072 nodes 256.7 (L1 squeezed); 5 and 6 CTAs of 256
// threads (48 and 40 registers, spilling) 264.9 and 234.5.  With the
// current node phase the whole L1 serves better: 1024x1 with 2048 nodes
// 303.1, 1536 306.2, 1024 305.9, 512 308.8, 256 310.1, 128 310.6, none
// 310.4-310.8; without staging 512x2 310.0 and 256x4 309.4.  So no nodes
// are staged (the mechanism stays for other scenes and shapes).
#ifndef CPPPT_TRACE_THREADS
#define CPPPT_TRACE_THREADS 1024
#endif
#ifndef CPPPT_TRACE_BLOCKS_PER_SM
#define CPPPT_TRACE_BLOCKS_PER_SM 1
#endif
#ifndef CPPPT_SMEM_NODES
#define CPPPT_SMEM_NODES 0
#endif
// Child slab distances two children at a time with the packed f32x2 adds
// and FMAs of sm_100 and later (1) or one at a time (0); same results
// (bit-identical images).  Measured on the 1M-triangle soup at 1080p, 64 spp:
// 280.8 against 277.5 Mpaths/s (closest-hit kernel -0.9 %, shadow -2.4 %).
#ifndef CPPPT_TRACE_F32X2
#define CPPPT_TRACE_F32X2 1
#endif
// Any-hit queries push their children in slot order without sorting (1) or
// nearest first like closest-hit queries (0).  Measured on the 1M-triangle
// soup at 1080p, 64 spp: shadow kernel 148.2 -> 137.3 ms, 281.2 -> 287.9
// Mpaths/s, bit-identical images (an occlusion answer does not depend on the
// visiting order).
#ifndef CPPPT_ANY_UNSORTED
#define CPPPT_ANY_UNSORTED 1
#endif
// Closest-hit queries: the nearest child next and the others pushed in slot
// order (1), or all pushed far to near after a full sort (0).  Measured as
// above: closest-hit kernel 258.0 -> 250.3 ms, 286.9 -> 291.8 Mpaths/s,
// bit-identical images (culling compares each popped entry with the best
// hit, so the push order changes the work, never the answer).
#ifndef CPPPT_CLOSEST_PARTIAL
#define CPPPT_CLOSEST_PARTIAL 1
#endif
// Any-hit queries keep no entry distances (an occlusion query never culls
// below its own max_t, so the distances are not needed) (1), or keep them (0).
// Measured as above: shadow kernel 137.4 -> 136.4 ms.
#ifndef CPPPT_ANY_LEAN
#define CPPPT_ANY_LEAN 1
#endif
constexpr int kTraceThreads = CPPPT_TRACE_THREADS;
constexpr int kTraceBlocksPerSM = CPPPT_TRACE_BLOCKS_PER_SM;
constexpr int kSmemNodes = CPPPT_SMEM_NODES;
constexpr size_t kSmemNodeBytes = (size_t)kSmemNodes * 64;  // dynamic shared memory of a traversal CTA
constexpr int kStackSize = kTraversalStackSize;
// Nodes whose entry distance exceeds best_t * (1 + 2^-8) are skipped.  The
// margin covers the rounding of the reference's Cramer-rule t (triangle.h:41-57)
// for every hit that is not within ~1e-4 rad of grazing the triangle.
constexpr float kCullScale = 1.00390625f;

// float(t) < 1e-4 (double) <=> t < kTriEps (triangle.h:55 compares with the double EPS)
__device__ __forceinline__ float tri_eps() { return __int_as_float(0x38d1b718); }  // nextafterf(1e-4f, inf)

struct HitRec {
    float t;
    int32_t prim;
    float beta, gamma;
    int32_t rank;
};

__device__ __forceinline__ float m3r(float a, float b, float c) { return __fmul_rn(__fmul_rn(a, b), c); }

// Triangle::intersect up to acceptance (triangle.h:18-80): Cramer's rule with
// the reference's product and sum order, no fused multiply-add, IEEE
// reciprocal for 1.0/den (1.0 / float in double rounded to float is the
// correctly rounded float reciprocal).
__device__ __forceinline__ bool tri_exact(float4 A, float4 E1, float4 E2, float3 o, float3 d, float max_t,
                                          float& t, float& beta, float& gamma) {
    const float v1x = E1.x, v1y = E1.y, v1z = E1.z;
    const float v2x = E2.x, v2y = E2.y, v2z = E2.z;
    const float v3x = -d.x, v3y = -d.y, v3z = -d.z;
    const float vsx = __fsub_rn(o.x, A.x), vsy = __fsub_rn(o.y, A.y), vsz = __fsub_rn(o.z, A.z);
    float den = m3r(v1x, v2y, v3z);
    den = __fadd_rn(den, m3r(v2x, v3y, v1z));
    den = __fadd_rn(den, m3r(v3x, v1y, v2z));
    den = __fsub_rn(den, m3r(v3x, v2y, v1z));
    den = __fsub_rn(den, m3r(v3y, v2z, v1x));
    den = __fsub_rn(den, m3r(v3z, v2x, v1y));
    const float inv = __frcp_rn(den);
    float nt = m3r(v1x, v2y, vsz);
    nt = __fadd_rn(nt, m3r(v2x, vsy, v1z));
    nt = __fadd_rn(nt, m3r(vsx, v1y, v2z));
    nt = __fsub_rn(nt, m3r(vsx, v2y, v1z));
    nt = __fsub_rn(nt, m3r(vsy, v2z, v1x));
    nt = __fsub_rn(nt, m3r(vsz, v2x, v1y));
    t = __fmul_rn(nt, inv);
    if (t < tri_eps() || t > max_t) return false;
    float nb = m3r(vsx, v2y, v3z);
    nb = __fadd_rn(nb, m3r(v2x, v3y, vsz));
    nb = __fadd_rn(nb, m3r(v3x, vsy, v2z));
    nb = __fsub_rn(nb, m3r(v3x, v2y, vsz));
    nb = __fsub_rn(nb, m3r(v3y, v2z, vsx));
    nb = __fsub_rn(nb, m3r(v3z, v2x, vsy));
    beta = __fmul_rn(nb, inv);
    float ng = m3r(v1x, vsy, v3z);
    ng = __fadd_rn(ng, m3r(vsx, v3y, v1z));
    ng = __fadd_rn(ng, m3r(v3x, v1y, vsz));
    ng = __fsub_rn(ng, m3r(v3x, vsy, v1z));
    ng = __fsub_rn(ng, m3r(v3y, vsz, v1x));
    ng = __fsub_rn(ng, m3r(v3z, vsx, v1y));
    gamma = __fmul_rn(ng, inv);
    const float alpha = __fsub_rn(1.0f, __fadd_rn(gamma, beta));
    if (alpha < 0.f || alpha > 1.f || beta < 0.f || beta > 1.f || gamma < 0.f || gamma > 1.f) return false;
    // NaN t passes the reference's checks (it then accepts a NaN hit); such
    // rays lie exactly in the triangle's plane.  They are rejected here.
    return t == t;
}

// AABB::intersect_any (aabb.h:19-61) with the reference's division, order2
// swaps and comparison sequence.  `cand_t` stands in for the ray's running
// max_t, which only matters when tmax is NaN (a -0.0 direction component
// with the origin on the box's lower x plane).
__device__ __forceinline__ bool ref_box_exact(float4 lo, float4 hi, float3 o, float3 d, float cand_t) {
    float nminx = __fdiv_rn(__fsub_rn(lo.x, o.x), d.x);
    float nminy = __fdiv_rn(__fsub_rn(lo.y, o.y), d.y);
    float nminz = __fdiv_rn(__fsub_rn(lo.z, o.z), d.z);
    float nmaxx = __fdiv_rn(__fsub_rn(hi.x, o.x), d.x);
    float nmaxy = __fdiv_rn(__fsub_rn(hi.y, o.y), d.y);
    float nmaxz = __fdiv_rn(__fsub_rn(hi.z, o.z), d.z);
    float s;
    if (!(nmaxx >= nminx)) { s = nminx; nminx = nmaxx; nmaxx = s; }
    if (!(nmaxy >= nminy)) { s = nminy; nminy = nmaxy; nmaxy = s; }
    if (!(nmaxz >= nminz)) { s = nminz; nminz = nmaxz; nmaxz = s; }
    float tmin = nminx;
    if (tmin < nminy) tmin = nminy;
    if (tmin < nminz && nminz > nminy) tmin = nminz;
    float tmax = nmaxx;
    if (tmax > nmaxy) tmax = nmaxy;
    if (tmax > nmaxz && nmaxz < nmaxy) tmax = nmaxz;
    if (tmax < tmin) return false;
    if (tmin > 0.f && (double)tmin < (double)cand_t + 1e-4) return true;
    return tmax > 0.f;
}

// byte c of w as a float: one byte permute builds 2^23 + b, one exact
// subtraction removes 2^23 (keeps the integer pipe free for the min/max)
__device__ __forceinline__ float byte_to_float(uint32_t w, int c) {
    return __uint_as_float(__byte_perm(w, 0x4b000000u, 0x7540u | (uint32_t)c)) - 8388608.0f;
}

// Packed pairs of floats (two children per instruction on sm_100 and later:
// add.f32x2 / fma.f32x2 round each half exactly as add.f32 / fma.rn.f32).
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
    f32x2 d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ void upk2(f32x2 v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// slab distances of byte children c and c + 1 of w: q B + A, with q exact
__device__ __forceinline__ void slab2(uint32_t w, int c, f32x2 B2, f32x2 A2, float& t0, float& t1) {
    const f32x2 q = pk2(__uint_as_float(__byte_perm(w, 0x4b000000u, 0x7540u | (uint32_t)c)),
                        __uint_as_float(__byte_perm(w, 0x4b000000u, 0x7540u | (uint32_t)(c + 1))));
    upk2(fma2(add2(q, pk2(-8388608.0f, -8388608.0f)), B2, A2), t0, t1);
}

// three-operand min / max (one instruction on sm_100 and later)
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Per-lane traversal state (one ray in flight).  ANY=false: closest hit in
// `best` (best.t starts at the ray's max_t).  ANY=true: finishes at the first
// hit the reference would also report.
struct TraceCount {
    uint32_t nodes, tris;  // visited wide nodes, tested triangles (counting build only)
};

constexpr uint32_t kTravDone = 0xffffffffu;  // never a valid node or leaf reference
constexpr uint32_t kLeafRef = 0x80000000u;

__device__ __forceinline__ bool is_inner(uint32_t r) { return !(r & kLeafRef); }  // kTravDone has the bit set
__device__ __forceinline__ bool is_leaf(uint32_t r) { return (r & kLeafRef) && r != kTravDone; }

struct Trav {
    float3 o, d;
    float idx, idy, idz, oix, oiy, oiz;
    float tmax0;
    uint32_t neg;   // bit k: direction component k is negative
    uint32_t cur;   // next node or leaf to visit (kTravDone: nothing left on the stack)
    float cur_t;    // entry distance of cur
    uint32_t leaf;  // leaf postponed to the warp's next leaf phase (kTravDone: none)
    int sp, steps;
    HitRec best;
};

// Traversal stack of one lane: {node reference, entry distance bits}, one
// 8-byte local-memory access per push and pop.
struct TravStack {
    uint2 e[kStackSize];
};

// root: wide-node index where the traversal starts (0 for a scene of its own;
// the scene's first node inside a merged multi-scene arena; kTravDone for a
// scene without triangles).
__device__ __forceinline__ void trav_init(Trav& T, float3 o, float3 d, float tmax0, uint32_t root) {
    T.o = o;
    T.d = d;
    T.tmax0 = tmax0;
    T.best.t = tmax0;
    T.best.prim = -1;
    T.best.rank = -1;
    T.best.beta = T.best.gamma = 0.f;
    const float tiny = 7.888609052210118e-31f;  // 2^-100 stands in for a zero component
    const float dx = d.x == 0.f ? copysignf(tiny, d.x) : d.x;
    const float dy = d.y == 0.f ? copysignf(tiny, d.y) : d.y;
    const float dz = d.z == 0.f ? copysignf(tiny, d.z) : d.z;
    T.idx = 1.0f / dx;
    T.idy = 1.0f / dy;
    T.idz = 1.0f / dz;
    T.oix = o.x * T.idx;
    T.oiy = o.y * T.idy;
    T.oiz = o.z * T.idz;
    T.neg = (T.idx < 0.f ? 1u : 0u) | (T.idy < 0.f ? 2u : 0u) | (T.idz < 0.f ? 4u : 0u);
    T.cur = root;
    T.cur_t = 0.f;
    T.leaf = kTravDone;
    T.sp = 0;
    T.steps = 0;
}

__device__ __forceinline__ float cull_dist(const Trav& T) { return T.best.t * kCullScale + 1e-6f; }

// Next stacked node that is still in front of the best hit.
__device__ __forceinline__ void trav_pop(Trav& T, const TravStack& K) {
    const float cull = cull_dist(T);
    while (T.sp > 0) {
        T.sp--;
        const uint2 e = K.e[T.sp];
        if (__uint_as_float(e.y) <= cull) {
            T.cur = e.x;
            T.cur_t = __uint_as_float(e.y);
            return;
        }
    }
    T.cur = kTravDone;
}

__device__ __forceinline__ void trav_abort(Trav& T, uint32_t* status, uint32_t bit) {
    atomicOr(status, bit);
    T.cur = kTravDone;
    T.leaf = kTravDone;
    T.sp = 0;
}

// One inner node (T.cur): the children the ray enters in front of the best
// hit, nearest first; far children are pushed.  (Any-hit rays use the same
// order: skipping the sort measured 2% slower on the bench, since near
// occluders end a shadow ray sooner.)
template <bool ANY, bool COUNT>
__device__ __forceinline__ void trav_node(Trav& T, TravStack& K, const DevScene& S, const uint4* __restrict__ snodes,
                                          uint32_t* status, TraceCount& cnt) {
    if (COUNT) cnt.nodes++;
    const uint32_t cur = T.cur;
    uint4 w0, w1, w2, w3;
    if (cur < (uint32_t)kSmemNodes) {
        w0 = snodes[4 * cur]; w1 = snodes[4 * cur + 1]; w2 = snodes[4 * cur + 2]; w3 = snodes[4 * cur + 3];
    } else {
        const uint4* np = S.nodes + 4 * (size_t)cur;
        w0 = __ldg(np); w1 = __ldg(np + 1); w2 = __ldg(np + 2); w3 = __ldg(np + 3);
    }
    const float cull = cull_dist(T);
    // slab distance of quantised coordinate q on axis k:
    //   (p + q s - o) / d = q (s/d) + (p - o)/d = q B + A
    const float ax = fmaf(__uint_as_float(w0.x), T.idx, -T.oix);
    const float ay = fmaf(__uint_as_float(w0.y), T.idy, -T.oiy);
    const float az = fmaf(__uint_as_float(w0.z), T.idz, -T.oiz);
    const float bx = __uint_as_float((w0.w & 0xffu) << 23) * T.idx;
    const float by = __uint_as_float(((w0.w >> 8) & 0xffu) << 23) * T.idy;
    const float bz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23) * T.idz;
    // words: lo_x lo_y lo_z hi_x | hi_y hi_z ref0 ref1 | ref2 ref3
    const bool nxs = T.neg & 1u, nys = T.neg & 2u, nzs = T.neg & 4u;
    const uint32_t nx = nxs ? w1.w : w1.x, fx = nxs ? w1.x : w1.w;
    const uint32_t ny = nys ? w2.x : w1.y, fy = nys ? w1.y : w2.x;
    const uint32_t nz = nzs ? w2.y : w1.z, fz = nzs ? w1.z : w2.y;
    uint32_t key[4];
#if CPPPT_TRACE_F32X2
    // children in pairs: the same roundings as the scalar form below
    const f32x2 BX = pk2(bx, bx), BY = pk2(by, by), BZ = pk2(bz, bz);
    const f32x2 AX = pk2(ax, ax), AY = pk2(ay, ay), AZ = pk2(az, az);
#pragma unroll
    for (int c = 0; c < 4; c += 2) {
        float tnx[2], tny[2], tnz[2], tfx[2], tfy[2], tfz[2];
        slab2(nx, c, BX, AX, tnx[0], tnx[1]);
        slab2(ny, c, BY, AY, tny[0], tny[1]);
        slab2(nz, c, BZ, AZ, tnz[0], tnz[1]);
        slab2(fx, c, BX, AX, tfx[0], tfx[1]);
        slab2(fy, c, BY, AY, tfy[0], tfy[1]);
        slab2(fz, c, BZ, AZ, tfz[0], tfz[1]);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float tn = fmax3(tnx[h], tny[h], fmaxf(tnz[h], 0.0f));
            const float tf = fmin3(tfx[h], tfy[h], fminf(tfz[h], cull));
            const bool hit = tn <= tf * 1.0000005f;
            if (ANY && CPPPT_ANY_LEAN) key[c + h] = hit ? 0u : 0xffffffffu;
            else key[c + h] = hit ? ((__float_as_uint(tn) & ~3u) | (uint32_t)(c + h)) : 0xffffffffu;
        }
    }
#else
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const float tnx = fmaf(byte_to_float(nx, c), bx, ax);
        const float tny = fmaf(byte_to_float(ny, c), by, ay);
        const float tnz = fmaf(byte_to_float(nz, c), bz, az);
        const float tfx = fmaf(byte_to_float(fx, c), bx, ax);
        const float tfy = fmaf(byte_to_float(fy, c), by, ay);
        const float tfz = fmaf(byte_to_float(fz, c), bz, az);
        const float tn = fmax3(tnx, tny, fmaxf(tnz, 0.0f));
        const float tf = fmin3(tfx, tfy, fminf(tfz, cull));
        const bool hit = tn <= tf * 1.0000005f;
        key[c] = hit ? ((__float_as_uint(tn) & ~3u) | (uint32_t)c) : 0xffffffffu;
    }
#endif
    const uint32_t refs[4] = {w2.z, w2.w, w3.x, w3.y};
#if CPPPT_ANY_UNSORTED
    if (ANY) {  // any hit: children in slot order, no sorting
        if (T.sp + 3 > S.stack_limit) {
            trav_abort(T, status, kStatusStackOverflow);
            return;
        }
        uint32_t nxt = kTravDone, nxt_t = 0u;
#pragma unroll
        for (int c = 3; c >= 0; c--) {
            const bool v = key[c] != 0xffffffffu;
            K.e[T.sp] = make_uint2(nxt, nxt_t);
            T.sp += (v && nxt != kTravDone) ? 1 : 0;
            nxt = v ? refs[c] : nxt;
            nxt_t = v ? (key[c] & ~3u) : nxt_t;
        }
        if (nxt == kTravDone) {
            trav_pop(T, K);
            return;
        }
        T.cur = nxt;
        T.cur_t = __uint_as_float(nxt_t);
        return;
    }
#endif
#if CPPPT_CLOSEST_PARTIAL
    if (!ANY) {  // nearest child next, the others pushed in slot order
        const uint32_t m = min(min(key[0], key[1]), min(key[2], key[3]));
        if (m == 0xffffffffu) {
            trav_pop(T, K);
            return;
        }
        if (T.sp + 3 > S.stack_limit) {
            trav_abort(T, status, kStatusStackOverflow);
            return;
        }
#pragma unroll
        for (int c = 3; c >= 0; c--)
            if (key[c] != 0xffffffffu && key[c] != m) K.e[T.sp++] = make_uint2(refs[c], key[c] & ~3u);
        T.cur = refs[m & 3u];
        T.cur_t = __uint_as_float(m & ~3u);
        return;
    }
#endif
#define CSWAP(a, b) { uint32_t lo_ = min(key[a], key[b]), hi_ = max(key[a], key[b]); key[a] = lo_; key[b] = hi_; }
    CSWAP(0, 1) CSWAP(2, 3) CSWAP(0, 2) CSWAP(1, 3) CSWAP(1, 2)
#undef CSWAP
    if (key[0] == 0xffffffffu) {
        trav_pop(T, K);
        return;
    }
    if (T.sp + 3 > S.stack_limit) {
        trav_abort(T, status, kStatusStackOverflow);
        return;
    }
    // far children first; an invalid key is written but not counted
#pragma unroll
    for (int k = 3; k >= 1; k--) {
        K.e[T.sp] = make_uint2(refs[key[k] & 3u], key[k] & ~3u);
        T.sp += (key[k] != 0xffffffffu) ? 1 : 0;
    }
    T.cur = refs[key[0] & 3u];
    T.cur_t = __uint_as_float(key[0] & ~3u);
}

// The postponed leaf T.leaf.  Returns true when an any-hit query is answered.
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool trav_leaf(Trav& T, const DevScene& S, TraceCount& cnt) {
    const uint32_t start = T.leaf & 0x7ffffffu;
    const uint32_t count = ((T.leaf >> 27) & 15u) + 1u;
    T.leaf = kTravDone;
    if (COUNT) cnt.tris += count;
    for (uint32_t k = 0; k < count; k++) {
        const float4* tp = S.tris + 3 * (size_t)(start + k);
        const float4 A = __ldg(tp), E1 = __ldg(tp + 1), E2 = __ldg(tp + 2);
        float t, beta, gamma;
        // ANY: the reference tests against the ray's own max_t
        if (!tri_exact(A, E1, E2, T.o, T.d, ANY ? T.tmax0 : T.best.t, t, beta, gamma)) continue;
        const int32_t rank = __float_as_int(A.w);
        if (!ANY && !(t < T.best.t || rank > T.best.rank)) continue;  // equal t: the later-visited wins
        const int32_t parent = __float_as_int(E1.w);
        if (parent >= 0) {
            const float4 lo = __ldg(S.ref_box + 2 * parent), hi = __ldg(S.ref_box + 2 * parent + 1);
            if (!ref_box_exact(lo, hi, T.o, T.d, t)) continue;
        }
        T.best.t = t;
        T.best.rank = rank;
        T.best.prim = __float_as_int(E2.w);
        T.best.beta = beta;
        T.best.gamma = gamma;
        if (ANY) {
            T.cur = kTravDone;
            T.sp = 0;
            return true;
        }
    }
    return false;
}

// Persistent ray loop.  Each warp takes chunks of kChunk consecutive rays
// from a global counter into a warp-private range; a lane whose ray finishes
// takes the next ray of the range at once (no waiting for the other lanes).
// load(i, o, d, tmax, root) fetches ray i; root arrives set to the scene's
// own root and may be replaced (rays of a merged multi-scene arena).
//
// Every iteration has a node phase and a leaf phase (leaves are postponed
// as in Aila and Laine 2009, "Understanding the efficiency of ray traversal
// on GPUs"): a lane that reaches a leaf parks it and keeps descending inner
// nodes; the node phase repeats until a third of the warp's active lanes
// cannot continue without their leaf, or no lane has an inner node left,
// and then the lanes with a parked leaf test its triangles together.
// Inner-node and triangle code run with most lanes converged instead of
// alternating per lane.  Measured on the 1M-triangle soup with an earlier
// node phase: a quarter 238.7 Mpaths/s against 232.5 at one half, 232.0 at
// one eighth and 215 at any waiting lane; repeating the node phase instead
// of one node step per iteration 247 against 237 (the current figures are
// below).  The result does not depend on the visiting order: the closest
// hit is the minimum over the tested triangles of (t, -rank), and a node is
// culled only when its entry distance lies behind the best hit found so far.
// Rays a warp takes from the global counter at a time, and the leaf-phase
// trigger (a leaf phase once 1/CPPPT_LEAF_WAIT_DIV of the active lanes wait
// on a parked leaf).  Measured on the 1M-triangle soup at 1080p, 64 spp, with
// the node phase above: chunk 64 / quarter 292.5 Mpaths/s, chunk 128 277.0,
// chunk 32 300.9, chunk 16 302.0; with a third: chunk 64 294.6, chunk 32
// 302.8, chunk 16 303.1; with a sixth (chunk 64) 287.7.  Smaller chunks
// balance the lanes' and warps' uneven ray lengths better, above all at
// the end of a launch.
#ifndef CPPPT_RAY_CHUNK
#define CPPPT_RAY_CHUNK 16
#endif
#ifndef CPPPT_LEAF_WAIT_DIV
#define CPPPT_LEAF_WAIT_DIV 3
#endif
// The same trigger for any-hit queries, measured apart: a half 308.7, a
// third 310.8, a fifth 310.4, an eighth 308.1 Mpaths/s.
#ifndef CPPPT_LEAF_WAIT_DIV_ANY
#define CPPPT_LEAF_WAIT_DIV_ANY CPPPT_LEAF_WAIT_DIV
#endif
constexpr int kChunk = CPPPT_RAY_CHUNK;

template <bool ANY, bool COUNT, class Load, class Store>
__device__ __forceinline__ void persistent_trace(const DevScene& S, const uint4* __restrict__ snodes, int n,
                                                 int* counter, uint32_t* status, TraceCount& cnt, Load load,
                                                 Store store) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    Trav T;
    TravStack K;
    int ray = -1;
    int pool_next = 0, pool_end = 0;  // warp-uniform
    bool exhausted = false;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, ray < 0);
        if (idle) {
            if (pool_next >= pool_end && !exhausted) {
                int base = 0;
                if (lane == 0) base = atomicAdd(counter, kChunk);
                base = __shfl_sync(0xffffffffu, base, 0);
                pool_next = base;
                pool_end = min(base + kChunk, n);
                if (base + kChunk >= n) exhausted = true;
            }
            const int avail = max(0, pool_end - pool_next);
            if (avail > 0) {
                const int r = __popc(idle & lt_mask);
                if (ray < 0 && r < avail) {
                    ray = pool_next + r;
                    float3 o, d;
                    float tmax;
                    uint32_t root = S.n_tris > 0 ? 0u : kTravDone;
                    load(ray, o, d, tmax, root);
                    trav_init(T, o, d, tmax, root);
                }
                pool_next += min(avail, __popc(idle));
            }
        }
        const bool active = ray >= 0;
        const unsigned act = __ballot_sync(0xffffffffu, active);
        if (act == 0) break;
        unsigned wait, inner;
        do {
            if (active && is_inner(T.cur)) {
                if (++T.steps > S.step_limit) trav_abort(T, status, kStatusIterLimit);
                else if (T.cur_t > cull_dist(T)) trav_pop(T, K);
                else trav_node<ANY, COUNT>(T, K, S, snodes, status, cnt);
            }
            if (active && T.leaf == kTravDone && is_leaf(T.cur)) {
                T.leaf = T.cur;
                trav_pop(T, K);
            }
            const bool waiting = active && T.leaf != kTravDone && !is_inner(T.cur);
            wait = __ballot_sync(0xffffffffu, waiting);
            inner = __ballot_sync(0xffffffffu, active && is_inner(T.cur));
        } while (inner != 0 && (ANY ? CPPPT_LEAF_WAIT_DIV_ANY : CPPPT_LEAF_WAIT_DIV) * __popc(wait) < __popc(act));
        // leaf phase (the node phase ended because enough lanes wait or none can descend)
        if (active && T.leaf != kTravDone) {
            ++T.steps;
            if (trav_leaf<ANY, COUNT>(T, S, cnt)) T.leaf = kTravDone;
        }
        if (active && T.cur == kTravDone && T.leaf == kTravDone) {
            store(ray, T.best);
            ray = -1;
        }
    }
}

}  // namespace cpppt_gb300
