// Host-side launchers of the CUDA kernels (implemented in render.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dev_types.h"

namespace cpppt_gb300 {

// Persistent-warp ray-batch kernels.  `rays` are 7 packed floats per ray;
// `counter` is one zeroed int in device memory (work queue head);
// `status` collects kStatus* bits.
void launch_trace_closest(const DevScene& S, const float* rays, int n, float4* hits, int* counter,
                          uint32_t* status, int num_sms, cudaStream_t st);
void launch_trace_any(const DevScene& S, const float* rays, int n, uint8_t* occluded, int* counter,
                      uint32_t* status, int num_sms, cudaStream_t st);

// Wavefront path state: capacity paths, structure of arrays, two copies.
struct PathBuffers {
    float4* o[2];    // origin.xyz, p (pdf of the last BSDF sample, RR scaled)
    float4* d[2];    // direction.xyz, unused
    float4* thr[2];  // throughput rgb, unused
    int4* info[2];   // pixel, sample, bounce | sampled_delta << 16, unused
    float4* hit;     // t, prim, beta, gamma of the current buffer
    float4* sh_o;    // shadow ray origin.xyz, max_t
    float4* sh_d;    // direction.xyz, pixel
    float4* sh_c;    // contribution rgb
    int capacity;
};

struct RenderParams {
    int spp;
    int spp_axis;        // >0: spp = spp_axis^2, stratified as pathtracerMIS.h:148-153
    int max_depth;
    int rr_start;
    uint32_t seed;
    int width, height;
    uint32_t flags;      // PT_FLAG_* of the render (read by the learned-guide integrator)
};

// The stages of one wavefront iteration reading path buffer `cur` (writing
// 1 - cur): extend (closest hit), shade (BSDF, NEE, MIS, RR, compaction),
// shadow (any hit + film), generate (new camera paths) + advance (counters).
void launch_extend(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, int num_sms, cudaStream_t st,
                   bool count = false);
// jobs: device table of n_jobs DevBatchJob (one entry for a single-scene
// render; several for a batch over a merged arena, ascending work ranges).
void launch_shade(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, unsigned long long* film,
                  const DevBatchJob* jobs, cudaStream_t st);
void launch_shadow(const DevScene& S, const PathBuffers& B, WaveCounters* ctr, unsigned long long* film, int num_sms,
                   cudaStream_t st);
void launch_generate(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, const DevBatchJob* jobs,
                     int n_jobs, cudaStream_t st);
// The whole wavefront loop of a plain render (PT_MODE_MIS / NEE / PT, single
// scene or batch) as one executable graph: a conditional WHILE node whose
// body runs `iters` (even) iterations and then a round-control kernel that
// ends the loop when no path is left and no work waits, or when a kernel set
// a status bit, or at ctr->max_rounds bodies (kStatusRoundLimit).  One graph
// launch renders everything after the first generate; the host reads the
// counters once, at the end.
cudaError_t build_render_graph(const DevScene& S, const PathBuffers& B, WaveCounters* ctr, unsigned long long* film,
                               const DevBatchJob* jobs, int n_jobs, int iters, int num_sms, cudaStream_t st,
                               cudaGraphExec_t* out);
// The job-table entry of a single-scene render of S with parameters P.
DevBatchJob single_job(const DevScene& S, const RenderParams& P);
constexpr int kKernelsPerIteration = 5;
// Allocation-free render: the wavefront of launch_* above with its scratch in
// a file-scope __device__ array (see render.cu).  Synchronises `st`.
// limit_hit is set when the iteration bound ran out; the kernels' status
// bits are in final_counters->status.
cudaError_t render_noalloc(const DevScene& S, const RenderParams& P, int num_sms, int max_depth, float* d_out,
                           cudaStream_t st, WaveCounters* final_counters, int* limit_hit);
size_t noalloc_scratch_bytes();
int noalloc_max_pixels();
int noalloc_paths();
// Unit-test launches of the integrator's BxDF and light sampling
// (pt_debug_bsdf / pt_debug_light_sample): floats per case in and out.
constexpr int kDebugBsdfIn = 20, kDebugBsdfOut = 10, kDebugLightIn = 6, kDebugLightOut = 10;
void launch_debug_bsdf(const float* in, float* out, int n, cudaStream_t st);
void launch_debug_light(const DevScene& S, const float* in, float* out, int n, cudaStream_t st);
// Shared-memory limits of the traversal kernels (their top-node staging may
// exceed the default 48 KB); call on each device before the first launch.
cudaError_t trace_kernels_setup();
// film: 32.32 fixed point per pixel and channel; out = film * scale / 2^32
void launch_film_resolve(const unsigned long long* film, float* out, int n, double scale, cudaStream_t st);

}  // namespace cpppt_gb300
