// SD-tree guided path tracing on the GPU: PPG::integrate
// (src/renderer/ppg.h:41-144) in the wavefront.  The SD-tree is built and
// updated on the host (sdtree.cpp); here it is looked up, sampled and
// splatted into.
//
// PPG keeps every path's vertices until the path ends (the splat needs the
// product of the factors that follow each vertex, ppg.h:131-141), so a path
// owns a slot of max_depth vertex records for its lifetime.  Slots come from
// a free list: k_generate_ppg pops, terminating paths push.
#include <cuda_runtime.h>

#include "guide.h"
#include "shade.cuh"

namespace cpppt_gb300 {

constexpr float kPiPPG = 3.14159265358979323846f;

// SDTree::get_leaf(pt) (sdtree.h:354-406): midpoint splits, axis = depth % 3,
// right iff coordinate > mid.
__device__ __forceinline__ int sd_dtree(const DevSDTree& T, f3 p) {
    float lo[3] = {T.lo[0], T.lo[1], T.lo[2]}, hi[3] = {T.hi[0], T.hi[1], T.hi[2]};
    const float pc[3] = {p.x, p.y, p.z};
    int node = 0;
    for (int depth = 0; depth < 64; depth++) {
        const int2 n = __ldg(T.snode + node);
        if (n.x < 0) return -1 - n.x;
        const int k = depth % 3;
        const float mid = (lo[k] + hi[k]) * 0.5f;
        if (pc[k] > mid) { lo[k] = mid; node = n.y; }
        else { hi[k] = mid; node = n.x; }
    }
    return -1;
}

// DTree leaf lookup (SDTree::get_leaf / get_area, sdtree.h:277-352).
// Returns the value slot; *area = size_phi * size_cos of the leaf cell.
__device__ __forceinline__ int sd_dleaf(const DevSDTree& T, int dtree, float x, float y, float* area) {
    float lx = -kPiPPG, ly = -1.0f, hx = kPiPPG, hy = 1.0f;
    int node = __ldg(T.dtree_root + dtree);
    for (int depth = 0; depth < 48; depth++) {
        const int c = __ldg(T.dnode + node);
        if (c < 0) {
            *area = (hx - lx) * (hy - ly);
            return -1 - c;
        }
        const float mx = (lx + hx) * 0.5f, my = (ly + hy) * 0.5f;
        int child;
        if (x < mx) {
            if (y < my) { child = 0; hx = mx; hy = my; }
            else { child = 2; hx = mx; ly = my; }
        } else {
            if (y < my) { child = 1; lx = mx; hy = my; }
            else { child = 3; lx = mx; ly = my; }
        }
        node = c + child;
    }
    *area = 1.0f;
    return -1;
}

// SDTree::pdf (sdtree.h:525-537)
__device__ __forceinline__ float sd_pdf(const DevSDTree& T, f3 p, f3 dir) {
    const int t = sd_dtree(T, p);
    if (t < 0) return 0.f;
    float area;
    sd_dleaf(T, t, atan2f(dir.y, dir.x), dir.z, &area);
    return (1.0f / (float)__ldg(T.leaf_cnt + t)) * (1.0f / area);
}

// SDTree::sample -> sample_direction (sdtree.h:408-430,445-451): uniform over
// the quadtree's leaves, uniform in (phi, cos theta) inside the leaf.
__device__ __forceinline__ BSample sd_sample(const DevSDTree& T, f3 p, float u0, float u1, float u2) {
    BSample s;
    const int t = sd_dtree(T, p);
    const int sz = t >= 0 ? __ldg(T.leaf_cnt + t) : 1;
    const int i = ((int)(u0 * (float)sz)) % sz;
    const float4 L = t >= 0 ? __ldg(T.leaves + __ldg(T.leaf_off + t) + i) : make_float4(-kPiPPG, -1.f, 2.f * kPiPPG, 2.f);
    const float phi = L.x + u1 * L.z;
    const float ct = L.y + u2 * L.w;
    const float st = sqrtf(fmaxf(0.f, 1.0f - ct * ct));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    s.wi = mk(cp * st, sp * st, ct);
    s.pdf = 1.0f / ((float)sz * (L.z * L.w));
    s.delta = false;
    return s;
}

// SDTree::splat (sdtree.h:514-524)
__device__ __forceinline__ void sd_splat(const DevSDTree& T, float rad, f3 p, f3 dir) {
    const int t = sd_dtree(T, p);
    if (t < 0) return;
    float area;
    const int slot = sd_dleaf(T, t, atan2f(dir.y, dir.x), dir.z, &area);
    if (slot >= 0) atomicAdd(T.slot_value + slot, rad);
    atomicAdd(T.dtree_count + t, 1);
    atomicAdd(T.dtree_rad + t, rad);
}

__device__ __forceinline__ int warp_append_ppg(int* counter, bool pred) {
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

// Backward products and splats of a finished path (ppg.h:131-141): only when
// the last vertex carries radiance; vertex k receives max-channel of the
// product of the factors of vertices k..n-1.
__device__ __forceinline__ void splat_path(const DevSDTree& T, const PPGVerts& V, int slot, int nv, int max_depth) {
    if (nv <= 0) return;
    const size_t base = (size_t)slot * (size_t)max_depth;
    float4 b = V.vd[base + nv - 1];
    f3 acc = mk(b.z, b.w, V.vr[base + nv - 1]);
    if (!(acc.x > 0.f || acc.y > 0.f || acc.z > 0.f)) return;
    for (int k = nv - 1; k >= 0; k--) {
        const float4 a = V.vp[base + k];
        const float4 bb = V.vd[base + k];
        if (k < nv - 1) acc = acc * mk(bb.z, bb.w, V.vr[base + k]);
        const float r = fmaxf(acc.x, fmaxf(acc.y, acc.z));
        sd_splat(T, r, mk(a.x, a.y, a.z), mk(a.w, bb.x, bb.y));
    }
}

__device__ __forceinline__ void set_vertex_rad(const PPGVerts& V, int slot, int k, int max_depth, f3 r) {
    const size_t i = (size_t)slot * (size_t)max_depth + k;
    float4 b = V.vd[i];
    b.z = r.x;
    b.w = r.y;
    V.vd[i] = b;
    V.vr[i] = r.z;
}

__global__ void __launch_bounds__(256) k_shade_ppg(DevScene S, PathBuffers B, int cur, RenderParams P,
                                                   WaveCounters* ctr, unsigned long long* __restrict__ film,
                                                   DevSDTree T, PPGVerts V, int* slot_stack) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = ctr->n_cur;
    bool push_cont = false, release = false;
    float4 no, nd, nt;
    int4 ninfo;
    int slot = -1;
    if (i < n) {
        const float4 O = B.o[cur][i], D = B.d[cur][i], Tp = B.thr[cur][i];
        const int4 I = B.info[cur][i];
        const float4 H = B.hit[i];
        const int prim = __float_as_int(H.y);
        const int pixel = I.x, sample = I.y, bounce = I.z & 0xffff;
        slot = I.w;
        const int D_ = P.max_depth;
        f3 mul = mk(Tp.x, Tp.y, Tp.z);
        const f3 ro = mk(O.x, O.y, O.z), rd = mk(D.x, D.y, D.z);
        const int nv = bounce;  // vertices recorded so far, this bounce's included (bounce > 0)
        if (bounce > 0) {  // ppg.h:51-56: a vertex at the ray's origin with radiance 1
            const size_t vi = (size_t)slot * D_ + (bounce - 1);
            V.vp[vi] = make_float4(ro.x, ro.y, ro.z, rd.x);
            V.vd[vi] = make_float4(rd.y, rd.z, 1.f, 1.f);
            V.vr[vi] = 1.f;
        }
        bool done = true;
        if (prim < 0) {  // sky = 0 (ppg.h:57-63)
            if (bounce > 0) set_vertex_rad(V, slot, bounce - 1, D_, mk(0.f, 0.f, 0.f));
        } else {
            int kind;
            DevMaterial m;
            const Surf s = make_surf(S, prim, ro, rd, H.x, H.z, H.w, bounce == 0, &kind, &m);
            const f3 wo = -rd;
            if (kind == PT_MAT_EMISSIVE_) {  // ppg.h:66-73
                const f3 rad = mk(m.r, m.g, m.b);
                if (bounce > 0) set_vertex_rad(V, slot, bounce - 1, D_, rad);
                const f3 c = mul * rad;
                film_add_rgb(film, pixel, c.x, c.y, c.z, ctr);
            } else {
                const Rng4 r0 = rng4(P.seed, sample, pixel, bounce, 0);
                const Rng4 r1 = rng4(P.seed, sample, pixel, bounce, 1);
                BSample smp;
                float weight = 1.0f;
                bool ok = true;
                if (r0.v[0] > 0.5f) {  // ppg.h:76-81: BSDF sample
                    smp = bsdf_sample(m, s, wo, r0.v[1], r0.v[2]);
                    weight = smp.pdf / (smp.pdf + sd_pdf(T, s.p, smp.wi));
                } else {  // ppg.h:83-95: SD-tree sample
                    smp = sd_sample(T, s.p, r0.v[3], r1.v[0], r1.v[1]);
                    if (!same_hemisphere(s, wo, smp.wi)) ok = false;
                    else {
                        const float pb = bsdf_pdf(m, s, wo, smp.wi);
                        weight = smp.pdf / (smp.pdf + pb);
                    }
                }
                if (ok) {
                    float p = smp.pdf * 0.5f;
                    if (same_hemisphere(s, wo, smp.wi)) {  // ppg.h:105-107
                        const f3 f = bsdf_eval(m, s, wo, smp.wi);
                        bool alive = true;
                        if (bounce >= P.rr_start) {  // ppg.h:111-117
                            const float rr = russian_roulette(f);
                            if (r1.v[2] > rr) alive = false;
                            else p = p * rr;
                        }
                        if (alive) {
                            const f3 nm = f * (weight / p);
                            if (bounce > 0) set_vertex_rad(V, slot, bounce - 1, D_, nm);
                            mul = mul * nm;
                            if (bounce + 1 < P.max_depth) {
                                done = false;
                                const f3 oo = s.p + smp.wi * kEps;
                                push_cont = true;
                                no = make_float4(oo.x, oo.y, oo.z, 1.f);
                                nd = make_float4(smp.wi.x, smp.wi.y, smp.wi.z, 0.f);
                                nt = make_float4(mul.x, mul.y, mul.z, 0.f);
                                ninfo = make_int4(pixel, sample, bounce + 1, slot);
                            }
                        }
                    }
                }
            }
        }
        if (done) {
            splat_path(T, V, slot, nv, D_);
            release = true;
        }
    }
    const int jr = warp_append_ppg(&ctr->free_top, release);
    if (release) slot_stack[jr] = slot;
    const int jc = warp_append_ppg(&ctr->n_next, push_cont);
    if (push_cont) {
        const int nx = 1 - cur;
        B.o[nx][jc] = no;
        B.d[nx][jc] = nd;
        B.thr[nx][jc] = nt;
        B.info[nx][jc] = ninfo;
    }
}

// Camera paths for PPG (ppg.h:174-186: one jittered sample per pixel per
// pass, no strata), each with a vertex slot from the free list.
__global__ void __launch_bounds__(256) k_generate_ppg(DevScene S, PathBuffers B, int cur, RenderParams P,
                                                      WaveCounters* ctr, const int* slot_stack) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_next = ctr->n_next;
    const int avail = min(B.capacity - n_next, ctr->free_top);
    const unsigned long long w = ctr->work_next + (unsigned long long)t;
    if (t >= avail || w >= ctr->work_total) return;
    const unsigned long long npix = (unsigned long long)P.width * P.height;
    const int sample = (int)(w / npix);
    const int pixel = (int)(w - (unsigned long long)sample * npix);
    const int px = pixel % P.width, py = pixel / P.width;
    const Rng4 r = rng4(P.seed, sample, pixel, 0xffffu, 2);
    const float cx = (((float)px + r.v[0]) / (float)P.width) * 2.0f - 1.0f;
    const float cy = -((((float)py + r.v[1]) / (float)P.height) * 2.0f - 1.0f);
    const DevCamera& C = S.cam;
    const float dx = cx * C.tan_fovy * C.aspect, dy = cy * C.tan_fovy, dz = -1.0f;
    const f3 d = normalized(mk(C.m[0] * dx + C.m[1] * dy + C.m[2] * dz, C.m[3] * dx + C.m[4] * dy + C.m[5] * dz,
                               C.m[6] * dx + C.m[7] * dy + C.m[8] * dz));
    const int nx = 1 - cur;
    const int j = n_next + t;
    const int slot = slot_stack[ctr->free_top - 1 - t];
    B.o[nx][j] = make_float4(C.o[0], C.o[1], C.o[2], 1.0f);
    B.d[nx][j] = make_float4(d.x, d.y, d.z, 0.f);
    B.thr[nx][j] = make_float4(1.f, 1.f, 1.f, 0.f);
    B.info[nx][j] = make_int4(pixel, sample, 0, slot);
}

__global__ void k_advance_ppg(WaveCounters* ctr, int capacity) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int n_next = ctr->n_next;
    const unsigned long long left = ctr->work_total - ctr->work_next;
    unsigned long long room = (unsigned long long)(capacity - n_next);
    if ((unsigned long long)ctr->free_top < room) room = (unsigned long long)ctr->free_top;
    const unsigned long long added = left < room ? left : room;
    ctr->work_next += added;
    ctr->stat_paths += added;
    ctr->free_top -= (int)added;
    ctr->n_cur = n_next + (int)added;
    ctr->stat_closest += (unsigned long long)ctr->n_cur;
    ctr->n_next = 0;
    ctr->n_shadow = 0;
    ctr->fetch_ext = 0;
    ctr->fetch_sh = 0;
    ctr->stat_iters += 1;
}

__global__ void k_init_slots(int* slot_stack, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) slot_stack[i] = i;
}

void launch_init_slots(int* slot_stack, int n, cudaStream_t st) {
    k_init_slots<<<min((n + 255) / 256, 2048), 256, 0, st>>>(slot_stack, n);
}
void launch_shade_ppg(const DevScene& S, const PathBuffers& B, int cur, const RenderParams& P, WaveCounters* ctr,
                      unsigned long long* film, const DevSDTree& T, const PPGVerts& V, int* slot_stack,
                      cudaStream_t st) {
    k_shade_ppg<<<(B.capacity + 255) / 256, 256, 0, st>>>(S, B, cur, P, ctr, film, T, V, slot_stack);
}
void launch_generate_ppg(const DevScene& S, const PathBuffers& B, int cur, const RenderParams& P, WaveCounters* ctr,
                         const int* slot_stack, cudaStream_t st) {
    k_generate_ppg<<<(B.capacity + 255) / 256, 256, 0, st>>>(S, B, cur, P, ctr, slot_stack);
    k_advance_ppg<<<1, 32, 0, st>>>(ctr, B.capacity);
}

}  // namespace cpppt_gb300
