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
    int32_t encoding = 0;            // PT_NN_ENC_* (input encoding)
};

struct NNTrainBuf {
    __nv_bfloat16* act;   // 4 layers x cap x 64: input activation of each layer
    __nv_bfloat16* grad;  // 4 layers x cap x 64: gradient of each layer's output
    int cap;
};

constexpr int kNNVertFloat4 = 7;  // float4 per recorded path vertex
constexpr int kNNMixF4 = 8;       // float4 per path of the packed mixture (inference -> shading)
constexpr int kNNMaxStepsPerRound = 64;  // batches of one network between two wavefront checks
constexpr int kNNMaxPasses = 8;          // Adam steps per batch

// Per-path state of the learned-guide integrator (slot = path's free-list entry).
struct NNPathData {
    float4* vert;        // kNNVertFloat4 float4 per vertex, max_depth vertices per slot
    float4* acc;         // film total gathered by the path so far (rgb)
    int* slot_stack;     // free list of slots
    int* slot_job;       // render job of the path holding each slot
    int4* fin;           // paths finished this iteration: slot, traced vertices, recorded vertices
    int rec_cap;         // > 0: vertex records are kept and training records emitted (to DevNNJob::rec)
};

// Learned-guide data of one render job (device table, one entry per job;
// a single-scene render is a table of one).  Jobs of one scene share its
// network and record buffer.
struct DevNNJob {
    const __nv_bfloat16* wt;  // forward weights of the job's scene (W_l^T, rows padded to 72)
    float lo[3], inv_ext[3];  // position normalisation to the scene box
    float c_lo, c_hi;         // range of the BSDF selection probability
    int32_t encoding;         // PT_NN_ENC_* of the job's network
    float4* rec;              // training records of the job's scene (4 float4 each)
    int32_t rec_cap;          // capacity of rec (0: no records)
    int32_t* n_rec;           // record counter of the job's scene
    float keep = 1.0f;        // probability that a finished path leaves its records
};

// Path info word z of the slot wavefront: bounce (bits 0-15), sampled delta
// (bit 16), render job (bits 17-31).
constexpr int kNNJobShift = 17;
constexpr int kNNMaxJobs = 1 << 15;

struct NNAdam {
    float lr = 1e-3f, b1 = 0.9f, b2 = 0.99f, eps = 1e-8f, clip = 10.0f;
};

size_t nn_smem_infer();
size_t nn_smem_train();
size_t nn_wcopy_elems();  // bf16 elements of one padded weight copy
cudaError_t nn_set_smem_limits();
void launch_nn_pack(const NNWeights& W, cudaStream_t st);
// status: one zeroed word; receives kStatusTensorTimeout if a wait ran out.
// oneblob: some network of the table uses PT_NN_ENC_ONEBLOB (else the kernel
// instance with the frequency encoding alone runs).
void launch_nn_forward_debug(const DevNNJob* nnj, const float* in, int n, float* out, uint32_t* status, int num_sms,
                             cudaStream_t st, bool oneblob);
void launch_nn_infer(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, const DevNNJob* nnj,
                     float4* params, int num_sms, cudaStream_t st, bool oneblob);
// One network's part of a fused training step (device table; one launch
// per stage covers every task: several scenes' guides train together).
struct NNTrainTask {
    NNWeights W;
    NNNorm N;
    float4* rec;  // this step's records (T squared in place for chi-square)
    int32_t n;
    int32_t chi2;
    int32_t prep;  // with the launch's prep: square T (chi-square) and sum it; 0: a later pass over the same batch
    float* scal;  // [0] batch loss, [1] sum of T, [2] status bits (kStatusTensorTimeout; accumulate)
    NNTrainBuf TB;
    float* grad;  // kNNWeights floats: dL/dW of this step
    float lr, bc1, bc2;  // Adam learning rate and bias corrections 1 - b^step
};

// One training step of n_tasks networks (max_n: the largest task's record
// count).  prep: zero and compute each task's sum of T (squaring T first
// for chi-square); otherwise scal[1] holds it already.  apply: take the
// Adam step (else only the gradient).
void launch_nn_train_tasks(const NNTrainTask* tasks, int n_tasks, int max_n, int num_sms, cudaStream_t st, bool prep,
                           bool apply, bool oneblob);
// One CTA that waits on a completion barrier nothing arrives on (bounded)
// and sets kStatusTensorTimeout in *status: the tensor-core kernels' timeout
// path, exercised without a tensor-core instruction.
void launch_debug_tc_timeout(uint32_t* status, cudaStream_t st);

// The slot wavefront's stages.  jobs: the render jobs (DevBatchJob, as the
// plain wavefront; one entry for a single render); P carries the flags and
// the vertex-record stride (P.max_depth: the largest depth of the jobs).
void launch_nn_shade(const DevScene& S, const PathBuffers& B, int cur, const RenderParams& P, WaveCounters* ctr,
                     unsigned long long* film, const float4* params, const NNPathData& PD, bool guided,
                     const DevBatchJob* jobs, cudaStream_t st);
void launch_nn_shadow(const DevScene& S, const PathBuffers& B, WaveCounters* ctr, unsigned long long* film,
                      const NNPathData& PD, const DevBatchJob* jobs, int num_sms, cudaStream_t st);
void launch_nn_generate(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, const NNPathData& PD,
                        const DevBatchJob* jobs, int n_jobs, cudaStream_t st);
// Emits the training records of the paths that finished this iteration (after
// the shadow stage, so their last NEE is counted) and frees their slots.
void launch_nn_finish(const NNPathData& PD, WaveCounters* ctr, const DevNNJob* nnj, int max_depth, int capacity,
                      cudaStream_t st);

}  // namespace cpppt_gb300
