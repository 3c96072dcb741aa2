// CUDA kernels: ray-batch traversal and the wavefront PT+NEE+MIS integrator
// (PathtracerMIS::integrate/render, src/renderer/pathtracerMIS.h:29-167).
//
// Wavefront layout: path state lives in HBM as structure-of-arrays, two
// copies (current / next).  One iteration = extend (closest hit for every
// live path) -> shade (emission + MIS, BSDF sample, NEE shadow ray, Russian
// roulette; survivors are appended compactly to the next buffer with
// warp-aggregated atomics) -> shadow (any hit; unoccluded NEE contributions
// go to the film) -> generate (new camera paths fill the next buffer up to
// capacity from a global work counter) -> advance (one thread swaps counts).
// All sizes are read from device counters, so an iteration needs no host
// round trip and a chain of iterations is captured once in a CUDA graph.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.h"
#include "shade.cuh"
#include "trace.cuh"

namespace cpppt_gb300 {


__device__ __forceinline__ void stage_top_nodes(const DevScene& S, uint4* snodes) {
    const int n = min(S.n_nodes, kSmemNodes) * 4;
    for (int i = threadIdx.x; i < n; i += blockDim.x) snodes[i] = __ldg(S.nodes + i);
    __syncthreads();
}

// Each warp takes 32 consecutive work items at a time from a global counter
// (persistent threads); returns the first index, or >= n when done.
__device__ __forceinline__ int warp_fetch(int* counter, int n) {
    int base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(counter, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    return base;
}

// Appends from every lane with pred set; all 32 lanes must call it.
__device__ __forceinline__ int warp_append(int* counter, bool pred) {
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

// ---------------------------------------------------------------------------
// Ray batches (BVH::intersect / intersect_any on arrays of rays)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTraceThreads, kTraceBlocksPerSM) k_trace_closest(DevScene S, const float* __restrict__ rays, int n,
                                                                 float4* __restrict__ hits, int* counter,
                                                                 uint32_t* status) {
    extern __shared__ uint4 snodes[];
    stage_top_nodes(S, snodes);
    TraceCount cnt{0u, 0u};
    persistent_trace<false, false>(
        S, snodes, n, counter, status, cnt,
        [&](int i, float3& o, float3& d, float& tmax, uint32_t& root) {
            const float* r = rays + 7 * (size_t)i;
            o = make_float3(r[0], r[1], r[2]);
            d = make_float3(r[3], r[4], r[5]);
            tmax = r[6];
        },
        [&](int i, const HitRec& h) { hits[i] = make_float4(h.t, __int_as_float(h.prim), h.beta, h.gamma); });
}

__global__ void __launch_bounds__(kTraceThreads, kTraceBlocksPerSM) k_trace_any(DevScene S, const float* __restrict__ rays, int n,
                                                             uint8_t* __restrict__ occ, int* counter,
                                                             uint32_t* status) {
    extern __shared__ uint4 snodes[];
    stage_top_nodes(S, snodes);
    TraceCount cnt{0u, 0u};
    persistent_trace<true, false>(
        S, snodes, n, counter, status, cnt,
        [&](int i, float3& o, float3& d, float& tmax, uint32_t& root) {
            const float* r = rays + 7 * (size_t)i;
            o = make_float3(r[0], r[1], r[2]);
            d = make_float3(r[3], r[4], r[5]);
            tmax = r[6];
        },
        [&](int i, const HitRec& h) { occ[i] = h.prim >= 0 ? 1 : 0; });
}

void launch_trace_closest(const DevScene& S, const float* rays, int n, float4* hits, int* counter, uint32_t* status,
                          int num_sms, cudaStream_t st) {
    if (n <= 0) return;
    const int blocks = min(num_sms * kTraceBlocksPerSM, (n + kTraceThreads - 1) / kTraceThreads);
    k_trace_closest<<<blocks, kTraceThreads, kSmemNodeBytes, st>>>(S, rays, n, hits, counter, status);
}

void launch_trace_any(const DevScene& S, const float* rays, int n, uint8_t* occ, int* counter, uint32_t* status,
                      int num_sms, cudaStream_t st) {
    if (n <= 0) return;
    const int blocks = min(num_sms * kTraceBlocksPerSM, (n + kTraceThreads - 1) / kTraceThreads);
    k_trace_any<<<blocks, kTraceThreads, kSmemNodeBytes, st>>>(S, rays, n, occ, counter, status);
}

// ---------------------------------------------------------------------------
// Wavefront integrator
// ---------------------------------------------------------------------------
// Film (film_add_rgb, shade.cuh): the image does not depend on the order in
// which contributions arrive (bit-identical across schedules, batch sizes and
// launch shapes).  The final division by spp happens in FP64.
__device__ __forceinline__ void film_add(unsigned long long* film, size_t pix, float r, float g, float b,
                                         WaveCounters* ctr) {
    film_add_rgb(film, pix, r, g, b, ctr);
}

template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, kTraceBlocksPerSM) k_extend(DevScene S, PathBuffers B, int cur, WaveCounters* ctr) {
    extern __shared__ uint4 snodes[];
    const int n = ctr->n_cur;
    if (n == 0) return;  // drained wavefront: skip staging
    stage_top_nodes(S, snodes);
    const float4* __restrict__ O = B.o[cur];
    const float4* __restrict__ D = B.d[cur];
    float4* __restrict__ Hout = B.hit;
    TraceCount cnt{0u, 0u};
    persistent_trace<false, COUNT>(
        S, snodes, n, &ctr->fetch_ext, &ctr->status, cnt,
        [&](int i, float3& o, float3& d, float& tmax, uint32_t& root) {
            const float4 a = O[i], b = D[i];
            o = make_float3(a.x, a.y, a.z);
            d = make_float3(b.x, b.y, b.z);
            tmax = __int_as_float(0x7f800000);
            if (root != kTravDone) root = __float_as_uint(b.w);  // the path's scene root (0 unbatched)
        },
        [&](int i, const HitRec& h) { Hout[i] = make_float4(h.t, __int_as_float(h.prim), h.beta, h.gamma); });
    if (COUNT) {
        const unsigned nodes = __reduce_add_sync(0xffffffffu, cnt.nodes);
        const unsigned tris = __reduce_add_sync(0xffffffffu, cnt.tris);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&ctr->stat_nodes, (unsigned long long)nodes);
            atomicAdd(&ctr->stat_tris, (unsigned long long)tris);
        }
    }
}

__global__ void __launch_bounds__(kTraceThreads, kTraceBlocksPerSM) k_shadow(DevScene S, PathBuffers B, WaveCounters* ctr,
                                                          unsigned long long* __restrict__ film) {
    extern __shared__ uint4 snodes[];
    const int n = ctr->n_shadow;
    if (n == 0) return;
    stage_top_nodes(S, snodes);
    TraceCount cnt{0u, 0u};
    persistent_trace<true, false>(
        S, snodes, n, &ctr->fetch_sh, &ctr->status, cnt,
        [&](int i, float3& o, float3& d, float& tmax, uint32_t& root) {
            const float4 a = B.sh_o[i], b = B.sh_d[i];
            o = make_float3(a.x, a.y, a.z);
            d = make_float3(b.x, b.y, b.z);
            tmax = a.w;
            if (root != kTravDone) root = __float_as_uint(B.sh_c[i].w);
        },
        [&](int i, const HitRec& h) {
            if (h.prim < 0) {  // unoccluded: the NEE contribution reaches the film
                const float4 c = B.sh_c[i];
                film_add(film, (uint32_t)__float_as_int(B.sh_d[i].w), c.x, c.y, c.z, ctr);
            }
        });
}

// info.w is the path's job: its table entry holds the render parameters,
// the scene's light list inside the arena and the job's film offset.  A
// single-scene render is a table of one job (so batched and single renders
// run the same instructions and give bit-identical images).
// Resident CTAs of 256 threads per SM for the shading kernel.  Measured on
// the 1M-triangle soup at 1080p, 64 spp, 2^24 paths in flight: 2 (128
// registers) 333.4 Mpaths/s, 3 (80 registers) 341.5, 4 (64 registers, some
// spilling) 345.1.
#ifndef CPPPT_SHADE_BLOCKS
#define CPPPT_SHADE_BLOCKS 4
#endif
__global__ void __launch_bounds__(256, CPPPT_SHADE_BLOCKS) k_shade(DevScene S, PathBuffers B, int cur, WaveCounters* ctr,
                                               unsigned long long* __restrict__ film,
                                               const DevBatchJob* __restrict__ jobs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = ctr->n_cur;
    bool push_sh = false, push_cont = false;
    float4 sh_o, sh_d, sh_c, no, nd, nt;
    int4 ninfo;
    if (i < n) {
        const float4 O = B.o[cur][i], D = B.d[cur][i], T = B.thr[cur][i];
        const int4 I = B.info[cur][i];
        const float4 H = B.hit[i];
        const int prim = __float_as_int(H.y);
        const int pixel = I.x, sample = I.y, bounce = I.z & 0xffff;
        const bool sdelta = (I.z >> 16) & 1;
        const DevBatchJob* J = jobs + I.w;
        const int integrator = J->integrator;
        const uint32_t seed = J->seed;
        const int rr_start = J->rr_start, max_depth = J->max_depth;
        const size_t fpix = (size_t)(uint32_t)pixel + J->film_off;
        S.light_prim += J->light_off;
        S.light_area += J->light_off;
        S.n_lights = J->n_lights;
        float p = O.w;
        f3 mul = mk(T.x, T.y, T.z);
        const f3 ro = mk(O.x, O.y, O.z), rd = mk(D.x, D.y, D.z);
        if (prim >= 0) {  // a miss adds render_sky = 0 (pathtracerMIS.h:38-41)
            int kind;
            DevMaterial m;
            const Surf s = make_surf(S, prim, ro, rd, H.x, H.z, H.w, bounce == 0, &kind, &m);
            const f3 wo = -rd;
            if (kind == PT_MAT_EMISSIVE_) {  // pathtracerMIS.h:43-67: emitters end the path
                float w = 1.0f;
                if (!sdelta && integrator == kIntegratorNEE) {
                    w = 0.0f;  // pathtracer.h:41-46: NEE already counted this emitter
                } else if (!sdelta && integrator == kIntegratorMIS) {
                    const int4 vi = __ldg(S.tri_vidx + prim);
                    const f3 a = f3of(__ldg(S.v_pos + vi.x)), b = f3of(__ldg(S.v_pos + vi.y)),
                             c = f3of(__ldg(S.v_pos + vi.z));
                    const float area = length(cross(b - a, c - a)) * 0.5f;
                    const float pdf_l = (1.0f / (float)S.n_lights) * (1.0f / area);
                    const float r = H.x;
                    const float cos_theta = fabsf(dot(s.n, rd)) + kEps;
                    const float p_nee = pdf_l * r * r / cos_theta;
                    w = p / (p + p_nee);
                }
                film_add(film, fpix, mul.x * m.r * w, mul.y * m.g * w, mul.z * m.b * w, ctr);
            } else {
                const Rng4 r0 = rng4(seed, sample, pixel, bounce, 0);
                const Rng4 r1 = rng4(seed, sample, pixel, bounce, 1);
                const BSample bs = bsdf_sample(m, s, wo, r0.v[0], r0.v[1]);
                p = bs.pdf;
                if (!bs.delta && S.n_lights > 0 && integrator != kIntegratorPT) {  // NEE, pathtracerMIS.h:79-106
                    const LSample ls = sample_light(S, s.p, r0.v[2], r0.v[3], r1.v[0]);
                    f3 sd = ls.pos - s.p;
                    const float len = length(sd);
                    sd = sd * (1.0f / len);
                    if (same_hemisphere(s, wo, sd)) {
                        const float pb = bsdf_pdf(m, s, wo, sd);
                        const float cosl = fabsf(dot(ls.n, sd)) + kEps;
                        const float pn = ls.pdf * len * len / cosl;
                        const float w = integrator == kIntegratorMIS ? pn / (pb + pn) : 1.0f;
                        const f3 f = bsdf_eval(m, s, wo, sd);
                        const f3 c = mul * f * ls.le * (1.0f / (ls.pdf * len * len)) * w;
                        if (c.x != 0.f || c.y != 0.f || c.z != 0.f) {
                            push_sh = true;
                            const f3 so = s.p + sd * kEps;
                            sh_o = make_float4(so.x, so.y, so.z, len - 2.0f * kEps);
                            sh_d = make_float4(sd.x, sd.y, sd.z, __int_as_float((int)(uint32_t)fpix));
                            sh_c = make_float4(c.x, c.y, c.z, D.w);  // w: the scene root
                        }
                    }
                }
                if (same_hemisphere(s, wo, bs.wi)) {  // pathtracerMIS.h:112-126
                    const f3 f = bsdf_eval(m, s, wo, bs.wi);
                    bool alive = true;
                    if (bounce >= rr_start) {
                        const float rr = russian_roulette(f);
                        if (r1.v[1] > rr) alive = false;
                        else p = p * rr;
                    }
                    if (alive && bounce + 1 < max_depth) {
                        mul = mul * f * (1.0f / p);
                        const f3 oo = s.p + bs.wi * kEps;
                        push_cont = true;
                        no = make_float4(oo.x, oo.y, oo.z, p);
                        nd = make_float4(bs.wi.x, bs.wi.y, bs.wi.z, D.w);
                        nt = make_float4(mul.x, mul.y, mul.z, 0.f);
                        ninfo = make_int4(pixel, sample, (bounce + 1) | ((bs.delta ? 1 : 0) << 16), I.w);
                    }
                }
            }
        }
    }
    const int js = warp_append(&ctr->n_shadow, push_sh);
    if (push_sh) {
        B.sh_o[js] = sh_o;
        B.sh_d[js] = sh_d;
        B.sh_c[js] = sh_c;
    }
    const int jc = warp_append(&ctr->n_next, push_cont);
    if (push_cont) {
        const int nx = 1 - cur;
        B.o[nx][jc] = no;
        B.d[nx][jc] = nd;
        B.thr[nx][jc] = nt;
        B.info[nx][jc] = ninfo;
    }
}

// Index of the job whose work range holds w (job work ranges ascend).
__device__ __forceinline__ int find_job(const DevBatchJob* __restrict__ jobs, int n_jobs, unsigned long long w) {
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&jobs[mid].work_begin) <= w) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// New camera paths for the free slots of the next buffer; work index w
// (global over the jobs' pixel x sample ranges) selects job, sample, pixel.
__global__ void __launch_bounds__(256) k_generate(DevScene S, PathBuffers B, int cur, WaveCounters* ctr,
                                                  const DevBatchJob* __restrict__ jobs, int n_jobs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_next = ctr->n_next;
    const int avail = B.capacity - n_next;
    unsigned long long w = ctr->work_next + (unsigned long long)t;
    if (t >= avail || w >= ctr->work_total) return;
    const int job = n_jobs > 1 ? find_job(jobs, n_jobs, w) : 0;
    const DevBatchJob* J = jobs + job;
    w -= J->work_begin;
    const DevCamera* C = &J->cam;
    const int width = C->width, height = C->height, spp_axis = J->spp_axis;
    const uint32_t seed = J->seed, root = J->root;
    const unsigned long long npix = (unsigned long long)width * height;
    const int sample = (int)(w / npix);
    int pixel = (int)(w - (unsigned long long)sample * npix);
    {  // visit the pass in tiles (a bijection of the pixels; the RNG is keyed by pixel, not by order)
        const int tw = J->tile_w, th = J->tile_h;
        if (tw * th > 1) {
            const int tile = pixel / (tw * th), r = pixel - tile * (tw * th);
            const int tiles_x = width / tw;
            const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
            pixel = (ty * th + r / tw) * width + tx * tw + r % tw;
        }
    }
    const int px = pixel % width, py = pixel / width;
    const Rng4 r = rng4(seed, sample, pixel, 0xffffu, 2);
    float cx, cy;
    if (spp_axis > 0) {  // pathtracerMIS.h:148-153: spp x spp strata
        const int k = sample / spp_axis, l = sample - (sample / spp_axis) * spp_axis;
        cx = (((float)px + ((float)k + r.v[0]) / (float)spp_axis) / (float)width) * 2.0f - 1.0f;
        cy = -((((float)py + ((float)l + r.v[1]) / (float)spp_axis) / (float)height) * 2.0f - 1.0f);
    } else {
        cx = (((float)px + r.v[0]) / (float)width) * 2.0f - 1.0f;
        cy = -((((float)py + r.v[1]) / (float)height) * 2.0f - 1.0f);
    }
    // CameraPerspective::get_ray (camera_perspective.h:30-39)
    const float dx = cx * C->tan_fovy * C->aspect, dy = cy * C->tan_fovy, dz = -1.0f;
    const f3 d = normalized(mk(C->m[0] * dx + C->m[1] * dy + C->m[2] * dz, C->m[3] * dx + C->m[4] * dy + C->m[5] * dz,
                               C->m[6] * dx + C->m[7] * dy + C->m[8] * dz));
    const int nx = 1 - cur;
    const int j = n_next + t;
    B.o[nx][j] = make_float4(C->o[0], C->o[1], C->o[2], 1.0f);
    B.d[nx][j] = make_float4(d.x, d.y, d.z, __uint_as_float(root));
    B.thr[nx][j] = make_float4(1.f, 1.f, 1.f, 0.f);
    B.info[nx][j] = make_int4(pixel, sample, 0 | (1 << 16), job);  // sampled_delta starts true (:34)
}

__global__ void k_advance(WaveCounters* ctr, int capacity) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int n_next = ctr->n_next;
    const unsigned long long left = ctr->work_total - ctr->work_next;
    const unsigned long long room = (unsigned long long)(capacity - n_next);
    const unsigned long long added = left < room ? left : room;
    ctr->work_next += added;
    ctr->stat_paths += added;
    ctr->stat_shadow += (unsigned long long)ctr->n_shadow;
    ctr->n_cur = n_next + (int)added;
    ctr->stat_closest += (unsigned long long)ctr->n_cur;
    ctr->n_next = 0;
    ctr->n_shadow = 0;
    ctr->fetch_ext = 0;
    ctr->fetch_sh = 0;
    ctr->stat_iters += 1;
}

__global__ void k_resolve(const unsigned long long* __restrict__ film, float* __restrict__ out, int n, double scale) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (float)((double)(long long)film[i] * scale);
}

void launch_extend(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, int num_sms, cudaStream_t st,
                   bool count) {
    if (count) k_extend<true><<<num_sms * kTraceBlocksPerSM, kTraceThreads, kSmemNodeBytes, st>>>(S, B, cur, ctr);
    else k_extend<false><<<num_sms * kTraceBlocksPerSM, kTraceThreads, kSmemNodeBytes, st>>>(S, B, cur, ctr);
}
cudaError_t trace_kernels_setup() {
    const int bytes = (int)kSmemNodeBytes;
    cudaError_t e = cudaFuncSetAttribute(k_trace_closest, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_trace_any, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_extend<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_extend<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_shadow, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e;
}

void launch_shade(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, unsigned long long* film,
                  const DevBatchJob* jobs, cudaStream_t st) {
    k_shade<<<(B.capacity + 255) / 256, 256, 0, st>>>(S, B, cur, ctr, film, jobs);
}
void launch_shadow(const DevScene& S, const PathBuffers& B, WaveCounters* ctr, unsigned long long* film, int num_sms,
                   cudaStream_t st) {
    k_shadow<<<num_sms * kTraceBlocksPerSM, kTraceThreads, kSmemNodeBytes, st>>>(S, B, ctr, film);
}
void launch_generate(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, const DevBatchJob* jobs,
                     int n_jobs, cudaStream_t st) {
    k_generate<<<(B.capacity + 255) / 256, 256, 0, st>>>(S, B, cur, ctr, jobs, n_jobs);
    k_advance<<<1, 32, 0, st>>>(ctr, B.capacity);
}

// Body end of a device-driven render loop (build_render_graph).  One thread.
__global__ void k_round_control(WaveCounters* ctr, cudaGraphConditionalHandle h) {
    const uint32_t r = ctr->rounds + 1u;
    ctr->rounds = r;
    bool more = !(ctr->n_cur == 0 && ctr->work_next >= ctr->work_total) && ctr->status == 0u;
    if (more && r >= ctr->max_rounds) {
        ctr->status |= kStatusRoundLimit;
        more = false;
    }
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

cudaError_t build_render_graph(const DevScene& S, const PathBuffers& B, WaveCounters* ctr, unsigned long long* film,
                               const DevBatchJob* jobs, int n_jobs, int iters, int num_sms, cudaStream_t st,
                               cudaGraphExec_t* out) {
    *out = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h;
    e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
    cudaGraphNodeParams cp = {};
    if (e == cudaSuccess) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
    }
    if (e == cudaSuccess) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            for (int k = 0; k < iters; k++) {
                const int cur = k & 1;
                launch_extend(S, B, cur, ctr, num_sms, st);
                launch_shade(S, B, cur, ctr, film, jobs, st);
                launch_shadow(S, B, ctr, film, num_sms, st);
                launch_generate(S, B, cur, ctr, jobs, n_jobs, st);
            }
            k_round_control<<<1, 1, 0, st>>>(ctr, h);
            cudaGraph_t captured = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(st, &captured);
            e = e2 != cudaSuccess ? e2 : cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    return e;
}

DevBatchJob single_job(const DevScene& S, const RenderParams& P) {
    DevBatchJob j{};
    j.cam = S.cam;
    j.work_begin = 0;
    j.film_off = 0;
    j.root = S.n_tris > 0 ? 0u : kTravDone;
    j.light_off = 0;
    j.n_lights = S.n_lights;
    j.spp = P.spp;
    j.spp_axis = P.spp_axis;
    j.max_depth = P.max_depth;
    j.rr_start = P.rr_start;
    j.seed = P.seed;
    j.tile_w = 1;
    j.tile_h = 1;
    j.integrator = kIntegratorMIS;
    return j;
}
void launch_film_resolve(const unsigned long long* film, float* out, int n, double scale, cudaStream_t st) {
    k_resolve<<<min((n + 255) / 256, 4096), 256, 0, st>>>(film, out, n, scale * (1.0 / 4294967296.0));
}

// ---------------------------------------------------------------------------
// Unit-test kernels: the integrator's own BxDF and light-sampling functions
// (shade.cuh) on cases given by the host, one case per thread
// (pt_debug_bsdf, pt_debug_light_sample).
// ---------------------------------------------------------------------------
__global__ void k_debug_bsdf(const float* __restrict__ in, float* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* c = in + (size_t)kDebugBsdfIn * i;
    DevMaterial m{};
    m.kind = (int32_t)c[0];
    m.r = c[1];
    m.g = c[2];
    m.b = c[3];
    m.alpha = fmaxf(c[4] * c[4], 0.01f);  // glossy_bxdf.h:77-79, as the scene upload sets it
    m.delta = (double)c[4] < 0.01 ? 1 : 0;
    m.ior = c[5];
    m.tex = kNoTextures;
    // The frame make_surf builds at a path's first hit on a flat triangle
    // whose vertices carry normal N and tangent T (bitangent N x T,
    // loader.h:237), then re-orthogonalised (standard_material.h:64-71).
    Surf s;
    s.p = mk(0.f, 0.f, 0.f);
    s.mat = 0;
    s.n = normalized(mk(c[6], c[7], c[8]));
    s.ng = s.n;
    s.b = normalized(cross(s.n, mk(c[9], c[10], c[11])));
    s.t = normalized(cross(s.b, s.n));
    if (m.kind == PT_MAT_DIFFUSE_ || m.kind == PT_MAT_GGX_) s.n = normalized(s.n);
    s.b = normalized(cross(s.n, s.t));
    s.t = normalized(cross(s.b, s.n));
    const f3 wo = mk(c[12], c[13], c[14]), wi = mk(c[15], c[16], c[17]);
    const f3 ev = bsdf_eval(m, s, wo, wi);
    const BSample b = bsdf_sample(m, s, wo, c[18], c[19]);
    float* o = out + (size_t)kDebugBsdfOut * i;
    o[0] = ev.x;
    o[1] = ev.y;
    o[2] = ev.z;
    o[3] = bsdf_pdf(m, s, wo, wi);
    o[4] = same_hemisphere(s, wo, wi) ? 1.f : 0.f;
    o[5] = b.wi.x;
    o[6] = b.wi.y;
    o[7] = b.wi.z;
    o[8] = b.pdf;
    o[9] = b.delta ? 1.f : 0.f;
}

__global__ void k_debug_light(DevScene S, const float* __restrict__ in, float* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* c = in + (size_t)kDebugLightIn * i;
    const LSample l = sample_light(S, mk(c[0], c[1], c[2]), c[3], c[4], c[5]);
    float* o = out + (size_t)kDebugLightOut * i;
    o[0] = l.pos.x; o[1] = l.pos.y; o[2] = l.pos.z;
    o[3] = l.n.x; o[4] = l.n.y; o[5] = l.n.z;
    o[6] = l.le.x; o[7] = l.le.y; o[8] = l.le.z;
    o[9] = l.pdf;
}

void launch_debug_bsdf(const float* in, float* out, int n, cudaStream_t st) {
    if (n > 0) k_debug_bsdf<<<(n + 127) / 128, 128, 0, st>>>(in, out, n);
}
void launch_debug_light(const DevScene& S, const float* in, float* out, int n, cudaStream_t st) {
    if (n > 0) k_debug_light<<<(n + 127) / 128, 128, 0, st>>>(S, in, out, n);
}

// ---------------------------------------------------------------------------
// Allocation-free render (pt_render_device_noalloc)
//
// For callers that cannot allocate device memory at render time: a host
// whose device memory is reserved up front by another allocator (a caching
// allocator or an engine's memory budget), or a frame loop that must not
// enter the driver's allocation path.  The host still polls the wavefront's
// counters between rounds of iterations.  The wavefront's scratch --
// path state, queues, film and counters -- lives in one file-scope
// __device__ array instead of per-scene buffers.  The array is part of this
// module, so every GPU that loads the library holds it until the process
// exits.  Capacity: kNoAllocPaths paths in flight, at most kNoAllocMaxPixels
// pixels.  Every call shares the array and leaves its contents behind; each
// call clears the film and counters first, and calls that overlap on the GPU
// (concurrent streams or threads) race on it.
// ---------------------------------------------------------------------------
constexpr int kNoAllocPaths = 1 << 16;
constexpr int kNoAllocMaxPixels = 1 << 18;  // e.g. 512 x 512
constexpr size_t kNoAllocPathBytes = (size_t)kNoAllocPaths * 16;  // one float4 / int4 array
constexpr size_t kNoAllocFilmOffset = 12 * kNoAllocPathBytes;
constexpr size_t kNoAllocCtrOffset = kNoAllocFilmOffset + (size_t)3 * kNoAllocMaxPixels * 8;
constexpr size_t kNoAllocJobOffset = kNoAllocCtrOffset + 256;
constexpr size_t kNoAllocBytes = kNoAllocJobOffset + 256;
static_assert(sizeof(WaveCounters) <= 256 && sizeof(DevBatchJob) <= 256, "scratch slots");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[128] = {};  // per device ordinal
}  // namespace

size_t noalloc_scratch_bytes() { return kNoAllocBytes; }
int noalloc_max_pixels() { return kNoAllocMaxPixels; }
int noalloc_paths() { return kNoAllocPaths; }

// Device address of the scratch array on the current device, looked up once
// per device (the host-side symbol is not a device address).
static cudaError_t noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 128) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return cudaSuccess;
}

cudaError_t render_noalloc(const DevScene& S, const RenderParams& P, int num_sms, int max_depth, float* d_out,
                           cudaStream_t st, WaveCounters* final_counters, int* limit_hit) {
    *limit_hit = 0;
    void* base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    if (e != cudaSuccess) return e;
    unsigned char* b = static_cast<unsigned char*>(base);
    PathBuffers B;
    for (int k = 0; k < 2; k++) {
        B.o[k] = reinterpret_cast<float4*>(b + (0 + k) * kNoAllocPathBytes);
        B.d[k] = reinterpret_cast<float4*>(b + (2 + k) * kNoAllocPathBytes);
        B.thr[k] = reinterpret_cast<float4*>(b + (4 + k) * kNoAllocPathBytes);
        B.info[k] = reinterpret_cast<int4*>(b + (6 + k) * kNoAllocPathBytes);
    }
    B.hit = reinterpret_cast<float4*>(b + 8 * kNoAllocPathBytes);
    B.sh_o = reinterpret_cast<float4*>(b + 9 * kNoAllocPathBytes);
    B.sh_d = reinterpret_cast<float4*>(b + 10 * kNoAllocPathBytes);
    B.sh_c = reinterpret_cast<float4*>(b + 11 * kNoAllocPathBytes);
    B.capacity = kNoAllocPaths;
    unsigned long long* film = reinterpret_cast<unsigned long long*>(b + kNoAllocFilmOffset);
    WaveCounters* ctr = reinterpret_cast<WaveCounters*>(b + kNoAllocCtrOffset);
    DevBatchJob* job = reinterpret_cast<DevBatchJob*>(b + kNoAllocJobOffset);
    const int film_n = 3 * P.width * P.height;
    const unsigned long long total = (unsigned long long)P.width * P.height * (unsigned long long)P.spp;
    e = cudaMemsetAsync(film, 0, sizeof(unsigned long long) * film_n, st);
    if (e != cudaSuccess) return e;
    WaveCounters init{};
    init.work_total = total;
    init.film_safe = film_safe_bound((double)P.spp * (2.0 * max_depth + 2.0));
    e = cudaMemcpyAsync(ctr, &init, sizeof(init), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    const DevBatchJob hjob = single_job(S, P);
    e = cudaMemcpyAsync(job, &hjob, sizeof(hjob), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    launch_generate(S, B, 1, ctr, job, 1, st);
    const int iters = 16;
    const unsigned long long max_rounds =
        64 + (total / (unsigned long long)kNoAllocPaths + 2) * (unsigned long long)(max_depth + 2) * 4 / iters;
    WaveCounters h{};
    for (unsigned long long round = 0;; round++) {
        for (int k = 0; k < iters; k++) {
            const int cur = k & 1;
            launch_extend(S, B, cur, ctr, num_sms, st, false);
            launch_shade(S, B, cur, ctr, film, job, st);
            launch_shadow(S, B, ctr, film, num_sms, st);
            launch_generate(S, B, cur, ctr, job, 1, st);
        }
        e = cudaMemcpyAsync(&h, ctr, sizeof(h), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        if (h.status) break;
        if (h.n_cur == 0 && h.work_next >= h.work_total) break;
        if (round > max_rounds) {
            *limit_hit = 1;
            break;
        }
    }
    *final_counters = h;
    if (h.status || *limit_hit) return cudaSuccess;
    launch_film_resolve(film, d_out, film_n, 1.0 / (double)P.spp, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

}  // namespace cpppt_gb300
