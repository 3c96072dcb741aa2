// Host interface of the learned guide's kernels (nn.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "dev_types.h"
#include "kernels.h"

namespace cpppt_gb300 {

struct NNWeights {
    float* master;        // FP32 weights, kNNWeights
    float* m;             // Adam first moment
    float* v;             // Adam second moment
    __nv_bfloat16* wt;    // transposed BF16 copy (forward)
    __nv_bfloat16* w;     // row-major BF16 copy (backward)
};

struct NNNorm {
    float lo[3], inv_ext[3];  // position normalisation to the scene box
    float c_lo = 0.1f, c_hi = 0.9f;  // range of the BSDF selection probability
};

struct NNTrainBuf {
    __nv_bfloat16* act;   // 4 layers x cap x 64: input activation of each layer
    __nv_bfloat16* grad;  // 4 layers x cap x 64: gradient of each layer's output
    int cap;
};

constexpr int kNNVertFloat4 = 7;  // float4 per recorded path vertex

// Per-path state of the learned-guide integrator (slot = path's free-list entry).
struct NNPathData {
    float4* vert;        // kNNVertFloat4 float4 per vertex, max_depth vertices per slot
    float4* acc;         // film total gathered by the path so far (rgb)
    int* slot_stack;     // free list of slots
    int4* fin;           // paths finished this iteration: slot, traced vertices, extra target of the last
    float4* rec;         // training records, 4 float4 each
    int rec_cap;
};

struct NNAdam {
    float lr = 1e-3f, b1 = 0.9f, b2 = 0.99f, eps = 1e-8f, clip = 10.0f;
};

size_t nn_smem_infer();
size_t nn_smem_train();
size_t nn_wcopy_elems();  // bf16 elements of one padded weight copy
cudaError_t nn_set_smem_limits();
void launch_nn_pack(const NNWeights& W, cudaStream_t st);
// status: one zeroed word; receives kStatusTensorTimeout if a wait ran out.
void launch_nn_forward_debug(const NNWeights& W, const NNNorm& N, const float* in, int n, float* out,
                             uint32_t* status, int num_sms, cudaStream_t st);
void launch_nn_infer(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, const NNWeights& W,
                     const NNNorm& N, float4* params, int num_sms, cudaStream_t st);
// grad (kNNWeights floats) receives dL/dW; loss[0] accumulates the batch
// loss and the word at loss + 2 collects status bits (kStatusTensorTimeout);
// apply: also take one Adam step (step counts from 1).
// tsum: device pointer to the batch's sum of targets T.
void launch_nn_train_step(const NNWeights& W, const NNNorm& N, const float4* rec, int n, const float* tsum,
                          const NNTrainBuf& TB, float* grad, float* loss, const NNAdam& opt, int step, int num_sms,
                          cudaStream_t st, bool apply);

void launch_nn_shade(const DevScene& S, const PathBuffers& B, int cur, const RenderParams& P, WaveCounters* ctr,
                     unsigned long long* film, const float4* params, const NNPathData& PD, bool guided,
                     cudaStream_t st);
void launch_nn_shadow(const DevScene& S, const PathBuffers& B, WaveCounters* ctr, unsigned long long* film,
                      const NNPathData& PD, int num_sms, cudaStream_t st);
void launch_nn_generate(const DevScene& S, const PathBuffers& B, int cur, const RenderParams& P, WaveCounters* ctr,
                        const NNPathData& PD, cudaStream_t st);
// Emits the training records of the paths that finished this iteration (after
// the shadow stage, so their last NEE is counted) and frees their slots.
void launch_nn_finish(const NNPathData& PD, WaveCounters* ctr, int max_depth, int capacity, cudaStream_t st);
// T -> T^2 for every record (chi-square training)
void launch_square_T(float4* rec, int n, cudaStream_t st);
void launch_sum_T(const float4* rec, int n, float* out, cudaStream_t st);

}  // namespace cpppt_gb300
