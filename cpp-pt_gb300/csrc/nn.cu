// Learned path guide on the tensor cores: fused MLP inference and training.
//
// Layout of the weights in device memory (one contiguous block per copy):
//   master  float  [kNNWeights]          layer l at nn_layer_offset(l), row-major [in][out]
//   wt      bf16   [4 layers][64][72]    transposed [out][in], rows padded to 72
//   w       bf16   [4 layers][64][72]    row-major  [in][out] padded (backward data pass)
// Inference, the training forward/backward and the weight-gradient reduction
// over the batch run on tcgen05 (MMAs issued by one thread from operands in
// shared memory, FP32 accumulators in tensor memory).
#include <cuda_runtime.h>

#include <algorithm>

#include "nn.h"
#include "nn.cuh"
#include "trace.cuh"
#include "umma.cuh"

namespace cpppt_gb300 {

constexpr int kWStride = 72;  // padded row of 64 bf16
constexpr int kWLayer = 64 * kWStride;

// Network inputs of one sample.
struct NNIn {
    f3 pn, n, wo;
};

// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores: tiles of 128 samples, one
// sample per thread.  Thread r writes its sample's 64 input features (bf16)
// as row r of the A tile; per layer one thread issues the 128 x N x 64 MMA
// chain (four K = 16 steps) into a 128 x 64 FP32 accumulator in tensor
// memory, commits it to an mbarrier, and every thread reads its row back
// (tensor-memory lane r), applies ReLU and writes the next layer's A row.
// The output row (48 floats) never leaves the thread: it is post-processed
// into the mixture parameters in registers.
// ---------------------------------------------------------------------------
constexpr int kTcRows = 128;                     // samples per tile (MMA M)
constexpr uint32_t kTcCols = 64;                 // tensor-memory columns per CTA
constexpr uint32_t kTcSBO = 8 * 128;             // K = 64: 8 core matrices per 8-row group
constexpr int kTcWLayerBytes = 64 * 64 * 2;      // W_l^T slot (N x 64 bf16)
constexpr int kTcABytes = kTcRows * 64 * 2;      // activation tile (128 x 64 bf16)

// W_l^T (N = outputs rows x K = inputs) in the canonical K-major layout, from
// the padded transposed copy wt[l][out][in].
__device__ __forceinline__ void tc_stage_weights(const NNWeights& W, unsigned char* s_w) {
    for (int c = threadIdx.x; c < kNNLayers * 64 * 8; c += blockDim.x) {
        const int l = c >> 9, rem = c & 511, nrow = rem >> 3, k8 = rem & 7;
        if (nrow >= nn_layer_out(l)) continue;
        const uint4 v = *reinterpret_cast<const uint4*>(W.wt + (size_t)l * kWLayer + nrow * kWStride + k8 * 8);
        *reinterpret_cast<uint4*>(s_w + l * kTcWLayerBytes + umma_offset(nrow, k8 * 8, 64)) = v;
    }
}

// Row `row` of a K-column A tile (K = 48 or 64) from K floats, optionally
// through ReLU.
__device__ __forceinline__ void tc_store_row(unsigned char* s_a, int row, const float* v, bool relu, int K = 64) {
#pragma unroll
    for (int g = 0; g < 8; g++) {
        if (8 * g >= K) break;
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = relu ? fmaxf(v[8 * g + j], 0.f) : v[8 * g + j];
        uint4 q;
        q.x = pack_bf16(x[0], x[1]);
        q.y = pack_bf16(x[2], x[3]);
        q.z = pack_bf16(x[4], x[5]);
        q.w = pack_bf16(x[6], x[7]);
        *reinterpret_cast<uint4*>(s_a + umma_offset(row, 8 * g, K)) = q;
    }
}

// One layer on the tensor cores: every thread's shared-memory writes are made
// visible to the async proxy, thread 0 issues D = A B^T over K (K / 16 MMAs,
// M = 128, N columns) and commits; all threads wait for the completion.
// Returns false (for every thread) when the bounded wait ran out.
__device__ __forceinline__ bool tc_layer(uint32_t tmem, uint32_t a_addr, uint32_t a_sbo, uint32_t b_addr,
                                         uint32_t b_sbo, int K, int N, uint32_t bar, uint32_t& phase) {
    fence_proxy_async_smem();
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    if (threadIdx.x == 0) {
        const uint32_t idesc = umma_idesc_bf16_f32(kTcRows, N);
        for (int ks = 0; ks < K / 16; ks++)
            umma_bf16(tmem, umma_desc(a_addr + ks * 2 * kUmmaLBO, a_sbo), umma_desc(b_addr + ks * 2 * kUmmaLBO, b_sbo),
                      idesc, ks > 0 ? 1u : 0u);
        umma_commit(bar);
    }
    const bool ok = __syncthreads_and(mbar_wait_bounded(bar, phase)) != 0;
    phase ^= 1u;
    if (ok) tc_fence_after_sync();
    return ok;
}

// Tensor memory and the completion barrier of a CTA (call with all threads).
__device__ __forceinline__ uint32_t tc_begin(uint64_t* s_bar, uint32_t* s_tmem) {
    if (threadIdx.x == 0) mbar_init(smem_u32(s_bar), 1);
    if ((threadIdx.x >> 5) == 0) tmem_alloc(s_tmem, kTcCols);
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    return *s_tmem;
}
__device__ __forceinline__ void tc_end(bool ok, uint32_t tmem, uint32_t bar, uint32_t phase, uint32_t* status) {
    if (!ok) {
        if (threadIdx.x == 0) atomicOr(status, kStatusTensorTimeout);
        mbar_wait_bounded(bar, phase ^ 1u);  // the MMAs of the timed-out phase, if they still finish
    }
    tc_fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        tc_fence_after_sync();
        tmem_dealloc(tmem, kTcCols);
    }
}

// Unit test of the bounded completion wait: the CTA allocates its tensor
// memory, waits on a completion barrier that nothing arrives on, and takes
// the timeout path of the tensor-core kernels (status bit, the second bounded
// wait, tensor memory freed).  No tensor-core instruction is ever in flight.
__global__ void __launch_bounds__(kTcRows) k_debug_tc_timeout(uint32_t* status) {
    __shared__ uint64_t s_bar;
    __shared__ uint32_t s_tmem;
    const uint32_t tmem = tc_begin(&s_bar, &s_tmem);
    uint32_t phase = 0;
    const bool ok = __syncthreads_and(mbar_wait_bounded(smem_u32(&s_bar), phase)) != 0;
    phase ^= 1u;
    tc_end(ok, tmem, smem_u32(&s_bar), phase, status);
}

void launch_debug_tc_timeout(uint32_t* status, cudaStream_t st) { k_debug_tc_timeout<<<1, kTcRows, 0, st>>>(status); }

// Inference over the paths of several render jobs (scenes with their own
// networks): each tile runs once per distinct job among its rows, staging
// that job's weights when they differ from the staged ones.  Jobs are
// rendered in order, so nearly every tile holds one job and runs once.
// Training runs on its own stream, so an Adam step may rewrite the BF16
// weights while a tile stages them; the tile then holds a mix of two
// consecutive networks, which is still one fixed network for all its paths:
// their mixtures are written once here and both sampled and evaluated from
// that copy, so the estimator stays unbiased.
constexpr int kTcInferThreads = kTcRows;
constexpr int kTcInferSmem = kNNLayers * kTcWLayerBytes + kTcABytes + 64;

// W_l^T of one network (padded transposed copy wt[l][out][in]) into the
// canonical K-major layout.
__device__ __forceinline__ void tc_stage_wt(const __nv_bfloat16* wt, unsigned char* s_w) {
    for (int c = threadIdx.x; c < kNNLayers * 64 * 8; c += blockDim.x) {
        const int l = c >> 9, rem = c & 511, nrow = rem >> 3, k8 = rem & 7;
        if (nrow >= nn_layer_out(l)) continue;
        const uint4 v = *reinterpret_cast<const uint4*>(wt + (size_t)l * kWLayer + nrow * kWStride + k8 * 8);
        *reinterpret_cast<uint4*>(s_w + l * kTcWLayerBytes + umma_offset(nrow, k8 * 8, 64)) = v;
    }
}

// get_in(i, NNIn& in, int& job) -> bool valid, with in.pn NOT yet
// normalised (world position); put(i, const float* prm41).  All kTcRows
// threads of the CTA must call it.  status: kStatusTensorTimeout when a
// completion wait runs out (the CTA then stops, frees its tensor memory and
// returns).
template <bool ONEBLOB, class GetIn, class Put>
__device__ __forceinline__ void tc_infer_loop(int n, unsigned char* smem, const DevNNJob* __restrict__ nnj,
                                              uint32_t* status, GetIn get_in, Put put) {
    unsigned char* s_w = smem;
    unsigned char* s_a = smem + kNNLayers * kTcWLayerBytes;
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_a + kTcABytes);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(s_bar + 1);
    int* s_job = reinterpret_cast<int*>(s_tmem + 1);
    const int warp = threadIdx.x >> 5;
    const int row = threadIdx.x;  // tensor-memory lane of this thread's sample
    const uint32_t tmem = tc_begin(s_bar, s_tmem);
    const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t bar = smem_u32(s_bar), a_addr = smem_u32(s_a), w_addr = smem_u32(s_w);
    uint32_t phase = 0;
    bool ok = true;
    const __nv_bfloat16* staged = nullptr;
    for (int base = blockIdx.x * kTcRows; base < n && ok; base += gridDim.x * kTcRows) {
        const int i = base + row;
        NNIn in;
        in.pn = in.n = in.wo = mk(0.f, 0.f, 0.f);
        int job = -1;
        const bool valid = i < n && get_in(i, in, job);
        bool pending = valid;
        while (ok) {
            // smallest job among the rows still waiting
            if (threadIdx.x == 0) *s_job = 0x7fffffff;
            __syncthreads();
            if (pending) atomicMin(s_job, job);
            __syncthreads();
            const int J = *s_job;
            if (J == 0x7fffffff) break;
            const DevNNJob& nj = nnj[J];
            if (nj.wt != staged) {  // all earlier MMAs have completed (their waits returned)
                tc_stage_wt(nj.wt, s_w);
                staged = nj.wt;
            }
            const bool mine = pending && job == J;
            float v[64];
            const f3 pn = mk((in.pn.x - nj.lo[0]) * nj.inv_ext[0], (in.pn.y - nj.lo[1]) * nj.inv_ext[1],
                             (in.pn.z - nj.lo[2]) * nj.inv_ext[2]);
            nn_features<ONEBLOB>(v, pn, in.n, in.wo, nj.encoding);
            if (!mine)
#pragma unroll
                for (int k = 0; k < 64; k++) v[k] = 0.f;
            tc_store_row(s_a, row, v, false);
            for (int l = 0; l < kNNLayers; l++) {
                const int nout = nn_layer_out(l);
                ok = tc_layer(tmem, a_addr, kTcSBO, w_addr + l * kTcWLayerBytes, kTcSBO, 64, nout, bar, phase);
                if (!ok) break;
#pragma unroll
                for (int c = 0; c < 64; c += 16)
                    if (c < nout) tmem_ld16(t_row + (uint32_t)c, v + c);
                if (l < kNNLayers - 1) tc_store_row(s_a, row, v, true);
            }
            if (ok && mine) {
                float prm[kNNParams];
                nn_postprocess(v, prm, nj.c_lo, nj.c_hi);
                put(i, prm);
            }
            pending = pending && !mine;
        }
    }
    tc_end(ok, tmem, bar, phase, status);
}

template <bool ONEBLOB>
__global__ void __launch_bounds__(kTcInferThreads) k_nn_forward_debug(const DevNNJob* __restrict__ nnj,
                                                                      const float* __restrict__ in, int n,
                                                                      float* __restrict__ out, uint32_t* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    tc_infer_loop<ONEBLOB>(
        n, smem, nnj, status,
        [&](int i, NNIn& v, int& job) {
            const float* p = in + 9 * (size_t)i;
            v.pn = mk(p[0], p[1], p[2]);
            v.n = mk(p[3], p[4], p[5]);
            v.wo = mk(p[6], p[7], p[8]);
            job = 0;
            return true;
        },
        [&](int i, const float* prm) {
            for (int k = 0; k < kNNParams; k++) out[kNNParams * (size_t)i + k] = prm[k];
        });
}

// Guide parameters for every live path's hit (run between extend and shade),
// each path with its job's network.
template <bool ONEBLOB>
__global__ void __launch_bounds__(kTcInferThreads) k_nn_infer(DevScene S, PathBuffers B, int cur, WaveCounters* ctr,
                                                              const DevNNJob* __restrict__ nnj,
                                                              float4* __restrict__ params) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int n = ctr->n_cur;
    if (n == 0) return;
    tc_infer_loop<ONEBLOB>(
        n, smem, nnj, &ctr->status,
        [&](int i, NNIn& v, int& job) {
            const float4 H = B.hit[i];
            const int prim = __float_as_int(H.y);
            if (prim < 0) return false;
            const int4 vi = __ldg(S.tri_vidx + prim);
            if (S.mats[vi.w].kind == PT_MAT_EMISSIVE_) return false;
            const float4 O = B.o[cur][i], D = B.d[cur][i];
            const f3 d = mk(D.x, D.y, D.z);
            const float beta = H.z, gamma = H.w, alpha = 1.0f - (gamma + beta);
            v.pn = mk(O.x, O.y, O.z) + d * H.x;
            v.n = normalized(f3of(__ldg(S.v_nrm + vi.x)) * alpha + f3of(__ldg(S.v_nrm + vi.y)) * beta +
                             f3of(__ldg(S.v_nrm + vi.z)) * gamma);
            v.wo = -d;
            job = (int)((uint32_t)B.info[cur][i].z >> kNNJobShift);
            return true;
        },
        [&](int i, const float* prm) { nn_pack_mixture(prm, params + kNNMixF4 * (size_t)i); });
}

// ---------------------------------------------------------------------------
// Training.  Records (16 floats): pos xyz, normal xyz, wo xyz, wi xyz,
// p_bsdf(wi), target weight T (>= 0), 0, 0.  Loss over a batch:
//   L = -sum_r T_r log m_r(wi_r) / sum_r T_r,  m = c p_bsdf + (1 - c) q.
// ---------------------------------------------------------------------------

// d loss / d raw outputs for one record (raw: 48 floats; returns loss term)
__device__ __forceinline__ float nn_loss_grad(const float* raw, f3 wi, float p_bsdf, float T, float c_lo, float c_hi,
                                             float* g /*48*/) {
    for (int k = 0; k < kNNOut; k++) g[k] = 0.f;
    if (!(T > 0.f)) return 0.f;
    float prm[kNNParams];
    nn_postprocess(raw, prm, c_lo, c_hi);
    float v[kNNLobes], q = 0.f;
    for (int j = 0; j < kNNLobes; j++) {
        v[j] = vmf_pdf(mk(prm[5 * j], prm[5 * j + 1], prm[5 * j + 2]), prm[5 * j + 3], wi);
        q += prm[5 * j + 4] * v[j];
    }
    const float c = prm[40];
    const float m = fmaxf(c * p_bsdf + (1.0f - c) * q, 1e-20f);
    const float dL_dm = -T / m;
    // selection: c = c_lo + (c_hi - c_lo) sigmoid(x)
    const float sg = 1.0f / (1.0f + __expf(-raw[40]));
    g[40] = dL_dm * (p_bsdf - q) * (c_hi - c_lo) * sg * (1.0f - sg);
    const float dL_dq = dL_dm * (1.0f - c);
    float gw[kNNLobes], wg = 0.f;
    for (int j = 0; j < kNNLobes; j++) {
        gw[j] = dL_dq * v[j];
        wg += prm[5 * j + 4] * gw[j];
    }
    for (int j = 0; j < kNNLobes; j++) {
        const float wj = prm[5 * j + 4];
        g[32 + j] = wj * (gw[j] - wg);  // softmax
        const float kappa = prm[5 * j + 3];
        const f3 mu = mk(prm[5 * j], prm[5 * j + 1], prm[5 * j + 2]);
        const float dv = dL_dq * wj * v[j];  // dL/d log v_j
        // kappa = softplus(x) + 0.1 (clamped at 5000)
        const float dlogv_dk = 1.0f / kappa - 2.0f / expm1f(2.0f * kappa) + (dot(mu, wi) - 1.0f);
        const float x = raw[24 + j];
        const float dk_dx = kappa >= 5000.0f ? 0.0f : 1.0f / (1.0f + __expf(-x));
        g[24 + j] = dv * dlogv_dk * dk_dx;
        // mu = r / |r|: dL/dr = (I - mu mu^T) (dL/dmu) / |r|,  dlogv/dmu = kappa wi
        const f3 r = mk(raw[3 * j], raw[3 * j + 1], raw[3 * j + 2]);
        const float len = sqrtf(dot(r, r));
        if (len > 1e-20f) {
            const f3 gm = wi * (dv * kappa);
            const f3 gr = (gm - mu * dot(mu, gm)) * (1.0f / len);
            g[3 * j] = gr.x;
            g[3 * j + 1] = gr.y;
            g[3 * j + 2] = gr.z;
        }
    }
    return -T * __logf(m);
}

// Forward + loss gradient + backward through the data on the tensor cores,
// 128 records per tile, one record per thread.  Every layer's bf16 input
// activation A_l (B x 64) and the gradient of its output dZ_l (B x out_l,
// bf16) go to TB for the weight-gradient pass; the backward pass reads the
// thread's own A_l row back for the ReLU mask.  Backward layer l is
// dH = dZ_l W_l^T: A = dZ_l (K = out_l), B = W_l as 64 inputs x out_l.
constexpr int kTcTrainSmem = 2 * kNNLayers * kTcWLayerBytes + kTcABytes + 64;

__device__ __forceinline__ void tc_stage_weights_bwd(const NNWeights& W, unsigned char* s_b) {
    for (int c = threadIdx.x; c < kNNLayers * 64 * 8; c += blockDim.x) {
        const int l = c >> 9, rem = c & 511, nrow = rem >> 3, k8 = rem & 7;
        const int K = nn_layer_out(l);
        if (8 * k8 >= K) continue;
        const uint4 v = *reinterpret_cast<const uint4*>(W.w + (size_t)l * kWLayer + nrow * kWStride + k8 * 8);
        *reinterpret_cast<uint4*>(s_b + l * kTcWLayerBytes + umma_offset(nrow, k8 * 8, K)) = v;
    }
}

// Row of K bf16 values (K = 48 or 64) to a 64-wide global row.
__device__ __forceinline__ void store_row_bf16(__nv_bfloat16* dst, const float* v, int K, bool relu) {
#pragma unroll
    for (int g = 0; g < 8; g++) {
        if (8 * g >= K) break;
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = relu ? fmaxf(v[8 * g + j], 0.f) : v[8 * g + j];
        uint4 q;
        q.x = pack_bf16(x[0], x[1]);
        q.y = pack_bf16(x[2], x[3]);
        q.z = pack_bf16(x[4], x[5]);
        q.w = pack_bf16(x[6], x[7]);
        *reinterpret_cast<uint4*>(dst + 8 * g) = q;
    }
}

constexpr int kNNThreads = 128;

// blockIdx.y: the network (task) of a fused multi-network step.
template <bool ONEBLOB>
__global__ void __launch_bounds__(kTcRows) k_nn_train_fb(const NNTrainTask* __restrict__ tasks) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const NNTrainTask& task = tasks[blockIdx.y];
    const NNWeights W = task.W;
    const NNNorm N = task.N;
    const NNTrainBuf TB = task.TB;
    const float4* __restrict__ rec = task.rec;
    const int n = task.n;
    float* loss_out = task.scal;
    uint32_t* status = reinterpret_cast<uint32_t*>(task.scal + 2);
    unsigned char* s_wf = smem;                                  // forward B tiles: W_l^T (out x in)
    unsigned char* s_wb = smem + kNNLayers * kTcWLayerBytes;     // backward B tiles: W_l (in x out)
    unsigned char* s_a = smem + 2 * kNNLayers * kTcWLayerBytes;  // A tile: activations, then output gradients
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_a + kTcABytes);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(s_bar + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = threadIdx.x;
    tc_stage_weights(W, s_wf);
    tc_stage_weights_bwd(W, s_wb);
    const uint32_t tmem = tc_begin(s_bar, s_tmem);
    const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t bar = smem_u32(s_bar), a_addr = smem_u32(s_a);
    const uint32_t wf_addr = smem_u32(s_wf), wb_addr = smem_u32(s_wb);
    uint32_t phase = 0;
    bool ok = true;
    float loss_acc = 0.f;
    const float tsum = task.scal[1];
    const float inv_tsum = tsum > 0.f ? 1.0f / tsum : 0.f;
    for (int base = blockIdx.x * kTcRows; base < n && ok; base += gridDim.x * kTcRows) {
        const int i = base + row;
        const bool valid = i < n;
        NNIn in;
        f3 wi = mk(0.f, 0.f, 1.f);
        float pb = 0.f, T = 0.f;
        if (valid) {
            const float4 r0 = rec[4 * (size_t)i], r1 = rec[4 * (size_t)i + 1], r2 = rec[4 * (size_t)i + 2],
                         r3 = rec[4 * (size_t)i + 3];
            in.pn = mk((r0.x - N.lo[0]) * N.inv_ext[0], (r0.y - N.lo[1]) * N.inv_ext[1], (r0.z - N.lo[2]) * N.inv_ext[2]);
            in.n = mk(r0.w, r1.x, r1.y);
            in.wo = mk(r1.z, r1.w, r2.x);
            wi = mk(r2.y, r2.z, r2.w);
            pb = r3.x;
            T = r3.y * inv_tsum;
        }
        float v[64];
        nn_features<ONEBLOB>(v, in.pn, in.n, in.wo, N.encoding);
        if (!valid)
#pragma unroll
            for (int j = 0; j < 64; j++) v[j] = 0.f;
        tc_store_row(s_a, row, v, false);
        if (valid) store_row_bf16(TB.act + (size_t)i * 64, v, 64, false);
        for (int l = 0; l < kNNLayers; l++) {
            const int nout = nn_layer_out(l);
            ok = tc_layer(tmem, a_addr, kTcSBO, wf_addr + l * kTcWLayerBytes, kTcSBO, 64, nout, bar, phase);
            if (!ok) break;
#pragma unroll
            for (int c = 0; c < 64; c += 16)
                if (c < nout) tmem_ld16(t_row + (uint32_t)c, v + c);
            if (l < kNNLayers - 1) {
                tc_store_row(s_a, row, v, true);
                if (valid) store_row_bf16(TB.act + ((size_t)(l + 1) * TB.cap + i) * 64, v, 64, true);
            }
        }
        if (!ok) break;
        float g[64];
#pragma unroll
        for (int k = 0; k < 64; k++) g[k] = 0.f;
        if (valid) loss_acc += nn_loss_grad(v, wi, pb, T, N.c_lo, N.c_hi, g);
        for (int l = kNNLayers - 1; l >= 0; l--) {
            const int K = nn_layer_out(l);
            if (valid) store_row_bf16(TB.grad + ((size_t)l * TB.cap + i) * 64, g, K, false);
            if (l == 0) break;
            tc_store_row(s_a, row, g, false, K);
            const uint32_t sbo = (uint32_t)(K / 8) * 128u;
            ok = tc_layer(tmem, a_addr, sbo, wb_addr + l * kTcWLayerBytes, sbo, K, 64, bar, phase);
            if (!ok) break;
            float dh[64];
#pragma unroll
            for (int c = 0; c < 64; c += 16) tmem_ld16(t_row + (uint32_t)c, dh + c);
            // dZ_{l-1} = dH where A_l > 0 (A_l = relu(Z_{l-1}), this thread's own row)
            if (valid) {
                const uint4* ar = reinterpret_cast<const uint4*>(TB.act + ((size_t)l * TB.cap + i) * 64);
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const uint4 a4 = ar[q];
                    const uint32_t w4[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
                    for (int h = 0; h < 4; h++) {
                        const __nv_bfloat162 b2 = *reinterpret_cast<const __nv_bfloat162*>(&w4[h]);
                        g[8 * q + 2 * h] = __low2float(b2) > 0.f ? dh[8 * q + 2 * h] : 0.f;
                        g[8 * q + 2 * h + 1] = __high2float(b2) > 0.f ? dh[8 * q + 2 * h + 1] : 0.f;
                    }
                }
            }
        }
    }
    tc_end(ok, tmem, bar, phase, status);
    float ls = loss_acc;
    for (int o = 16; o > 0; o >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, o);
    if (lane == 0) atomicAdd(loss_out, ls);
}

// dW_l = A_l^T dZ_l over the batch on the tensor cores.  blockIdx.y = layer,
// blockIdx.z = network (task); the CTAs of a (layer, network) share its
// records in K tiles of kWGK.  Per tile every thread takes one record and
// writes its activation row and output-gradient row transposed into the
// canonical K-major layout (A: input x record, B: output x record), then one
// thread issues the K chain of MMAs, D (+)= A B^T, into an FP32 accumulator
// in tensor memory that persists over the CTA's tiles.  M = 128 with input
// rows 64..127 of A kept zero (lane r of the accumulator = input r); N = 64
// or 48 outputs.  The CTA's sum is read back once (tcgen05.ld, inputs
// 0..63 = warps 0 and 1) and added to the FP32 gradient.
constexpr int kWGK = 128;                               // records per K tile
constexpr uint32_t kWGSbo = (kWGK / 8) * 128;           // K = 128: 16 core matrices per 8-row group
constexpr int kWGABytes = kTcRows * kWGK * 2;           // A tile: 128 x 128 bf16
constexpr int kWGBBytes = 64 * kWGK * 2;                // B tile: 64 x 128 bf16
constexpr size_t kWGSmem = kWGABytes + kWGBBytes + 16;  // + barrier, tensor-memory address

__global__ void __launch_bounds__(kTcRows) k_nn_wgrad(const NNTrainTask* __restrict__ tasks) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const NNTrainTask& task = tasks[blockIdx.z];
    const NNTrainBuf TB = task.TB;
    const int n = task.n;
    const int l = blockIdx.y;
    const int nout = nn_layer_out(l);
    uint32_t* status = reinterpret_cast<uint32_t*>(task.scal + 2);
    unsigned char* s_a = smem;
    unsigned char* s_b = smem + kWGABytes;
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_b + kWGBBytes);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(s_bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    // zero both tiles once: A's rows 64..127 and B's rows >= nout stay zero
    for (int e = tid; e < (kWGABytes + kWGBBytes) / 16; e += blockDim.x)
        reinterpret_cast<uint4*>(smem)[e] = make_uint4(0u, 0u, 0u, 0u);
    const uint32_t tmem = tc_begin(s_bar, s_tmem);  // (its barrier also orders the zeroing)
    const uint32_t bar = smem_u32(s_bar), a_addr = smem_u32(s_a), b_addr = smem_u32(s_b);
    const __nv_bfloat16* A = TB.act + (size_t)l * TB.cap * 64;
    const __nv_bfloat16* G = TB.grad + (size_t)l * TB.cap * 64;
    uint32_t phase = 0;
    bool ok = true;
    int tiles = 0;
    for (int r0 = blockIdx.x * kWGK; r0 < n && ok; r0 += gridDim.x * kWGK, tiles++) {
        const int r = r0 + tid;  // this thread's record = column k = tid of both tiles
#pragma unroll
        for (int g = 0; g < 8; g++) {
            uint4 va = make_uint4(0u, 0u, 0u, 0u), vg = make_uint4(0u, 0u, 0u, 0u);
            if (r < n) {
                va = *reinterpret_cast<const uint4*>(A + (size_t)r * 64 + 8 * g);
                if (8 * g < nout) vg = *reinterpret_cast<const uint4*>(G + (size_t)r * 64 + 8 * g);
            }
            const uint16_t* ea = reinterpret_cast<const uint16_t*>(&va);
            const uint16_t* eg = reinterpret_cast<const uint16_t*>(&vg);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                *reinterpret_cast<uint16_t*>(s_a + umma_offset(8 * g + q, tid, kWGK)) = ea[q];
                if (8 * g < nout) *reinterpret_cast<uint16_t*>(s_b + umma_offset(8 * g + q, tid, kWGK)) = eg[q];
            }
        }
        fence_proxy_async_smem();
        tc_fence_before_sync();
        __syncthreads();
        tc_fence_after_sync();
        if (tid == 0) {
            const uint32_t idesc = umma_idesc_bf16_f32(kTcRows, nout);
            for (int ks = 0; ks < kWGK / 16; ks++)
                umma_bf16(tmem, umma_desc(a_addr + ks * 2 * kUmmaLBO, kWGSbo),
                          umma_desc(b_addr + ks * 2 * kUmmaLBO, kWGSbo), idesc, (tiles > 0 || ks > 0) ? 1u : 0u);
            umma_commit(bar);
        }
        // the tiles are rewritten only after the MMAs that read them completed
        ok = __syncthreads_and(mbar_wait_bounded(bar, phase)) != 0;
        phase ^= 1u;
        if (ok) tc_fence_after_sync();
    }
    if (ok && tiles > 0 && warp < 2) {
        const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);
        float* dst = task.grad + nn_layer_offset(l) + (size_t)tid * nout;  // row = input tid
        for (int c0 = 0; c0 < nout; c0 += 16) {
            float v[16];
            tmem_ld16(t_row + (uint32_t)c0, v);
#pragma unroll
            for (int k = 0; k < 16; k++) atomicAdd(dst + c0 + k, v[k]);
        }
    }
    tc_end(ok, tmem, bar, phase, status);
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; refreshes the two
// BF16 copies the kernels read.
// blockIdx.y: the network (task); learning rate and bias corrections are the task's.
__global__ void k_nn_adam(const NNTrainTask* __restrict__ tasks, float b1, float b2, float eps, float clip) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNNWeights) return;
    const NNTrainTask& task = tasks[blockIdx.y];
    const NNWeights W = task.W;
    const float* __restrict__ grad = task.grad;
    const float lr = task.lr, bc1 = task.bc1, bc2 = task.bc2;
    float gi = grad[i];
    gi = fminf(fmaxf(gi, -clip), clip);
    const float m = b1 * W.m[i] + (1.0f - b1) * gi;
    const float v = b2 * W.v[i] + (1.0f - b2) * gi * gi;
    W.m[i] = m;
    W.v[i] = v;
    const float w = W.master[i] - lr * (m / bc1) / (sqrtf(v / bc2) + eps);
    W.master[i] = w;
    // locate (layer, in, out)
    int l = i / (64 * 64);
    if (l > kNNLayers - 1) l = kNNLayers - 1;
    const int off = i - nn_layer_offset(l), nout = nn_layer_out(l);
    const int in = off / nout, out = off - in * nout;
    W.wt[l * kWLayer + out * kWStride + in] = __float2bfloat16_rn(w);
    W.w[l * kWLayer + in * kWStride + out] = __float2bfloat16_rn(w);
}

__global__ void k_nn_pack(NNWeights W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNNWeights) return;
    int l = i / (64 * 64);
    if (l > kNNLayers - 1) l = kNNLayers - 1;
    const int off = i - nn_layer_offset(l), nout = nn_layer_out(l);
    const int in = off / nout, out = off - in * nout;
    const __nv_bfloat16 b = __float2bfloat16_rn(W.master[i]);
    W.wt[l * kWLayer + out * kWStride + in] = b;
    W.w[l * kWLayer + in * kWStride + out] = b;
}

size_t nn_smem_infer() { return (size_t)kTcInferSmem; }
size_t nn_smem_train() { return (size_t)kTcTrainSmem; }
size_t nn_wcopy_elems() { return (size_t)kNNLayers * kWLayer; }

cudaError_t nn_shadow_smem_limit();  // after k_shadow_nn below

cudaError_t nn_set_smem_limits() {
    cudaError_t es = nn_shadow_smem_limit();
    if (es != cudaSuccess) return es;
    const int si = (int)nn_smem_infer(), stn = (int)nn_smem_train();
    cudaError_t e = cudaFuncSetAttribute(k_nn_forward_debug<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, si);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_nn_forward_debug<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, si);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_nn_infer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, si);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_nn_infer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, si);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_nn_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWGSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_nn_train_fb<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, stn);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_nn_train_fb<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, stn);
    return e;
}

void launch_nn_pack(const NNWeights& W, cudaStream_t st) {
    k_nn_pack<<<(kNNWeights + 255) / 256, 256, 0, st>>>(W);
}
void launch_nn_forward_debug(const DevNNJob* nnj, const float* in, int n, float* out, uint32_t* status, int num_sms,
                             cudaStream_t st, bool oneblob) {
    const int blocks = std::max(1, std::min(num_sms * 4, (n + kTcInferThreads - 1) / kTcInferThreads));
    if (oneblob) k_nn_forward_debug<true><<<blocks, kTcInferThreads, nn_smem_infer(), st>>>(nnj, in, n, out, status);
    else k_nn_forward_debug<false><<<blocks, kTcInferThreads, nn_smem_infer(), st>>>(nnj, in, n, out, status);
}
void launch_nn_infer(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, const DevNNJob* nnj,
                     float4* params, int num_sms, cudaStream_t st, bool oneblob) {
    // four CTAs of 128 threads per SM fit in shared memory (48 KB each)
    if (oneblob) k_nn_infer<true><<<num_sms * 4, kTcInferThreads, nn_smem_infer(), st>>>(S, B, cur, ctr, nnj, params);
    else k_nn_infer<false><<<num_sms * 4, kTcInferThreads, nn_smem_infer(), st>>>(S, B, cur, ctr, nnj, params);
}
// Zeroes each task's gradient and loss (and, with prep, its T sum).
__global__ void k_nn_task_zero(const NNTrainTask* __restrict__ tasks, int prep) {
    const NNTrainTask& task = tasks[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kNNWeights) task.grad[i] = 0.f;
    if (i == 0) {
        task.scal[0] = 0.f;
        if (prep && task.prep) task.scal[1] = 0.f;
    }
}

// Chi-square targets (T squared in place) and the sum of T of each task.
__global__ void k_nn_task_T(const NNTrainTask* __restrict__ tasks) {
    const NNTrainTask& task = tasks[blockIdx.y];
    if (!task.prep) return;  // a later pass over a batch already prepared
    float4* __restrict__ rec = task.rec;
    float s = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < task.n; i += gridDim.x * blockDim.x) {
        float t = rec[4 * (size_t)i + 3].y;
        if (task.chi2) {
            t *= t;
            rec[4 * (size_t)i + 3].y = t;
        }
        s += t;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(task.scal + 1, s);
}

void launch_nn_train_tasks(const NNTrainTask* tasks, int n_tasks, int max_n, int num_sms, cudaStream_t st, bool prep,
                           bool apply, bool oneblob) {
    if (n_tasks < 1) return;
    const NNAdam opt;
    const dim3 gz((kNNWeights + 255) / 256, n_tasks);
    k_nn_task_zero<<<gz, 256, 0, st>>>(tasks, prep ? 1 : 0);
    if (prep) {
        const dim3 gt(std::max(1, std::min(std::max(1, 1024 / n_tasks), (max_n + 255) / 256)), n_tasks);
        k_nn_task_T<<<gt, 256, 0, st>>>(tasks);
    }
    // two CTAs per SM fit (80 KB of shared memory each), shared by the tasks
    const int per_task = std::max(1, (num_sms * 2 + n_tasks - 1) / n_tasks);
    const dim3 gf(std::max(1, std::min(per_task, (max_n + kTcRows - 1) / kTcRows)), n_tasks);
    if (oneblob) k_nn_train_fb<true><<<gf, kTcRows, nn_smem_train(), st>>>(tasks);
    else k_nn_train_fb<false><<<gf, kTcRows, nn_smem_train(), st>>>(tasks);
    const int per_task_w = std::max(1, (num_sms + n_tasks - 1) / n_tasks);
    const dim3 gw(std::max(1, std::min(per_task_w, (max_n + kWGK - 1) / kWGK)), kNNLayers, n_tasks);
    k_nn_wgrad<<<gw, kTcRows, kWGSmem, st>>>(tasks);
    if (apply) k_nn_adam<<<gz, 256, 0, st>>>(tasks, opt.b1, opt.b2, opt.eps, opt.clip);
}

// ===========================================================================
// Learned-guide integrator: PT + NEE + MIS where the directional sample comes
// from the one-sample mixture c * BSDF + (1 - c) * guide.  MIS weights use
// the mixture pdf; Russian roulette survival min(rr, 1) only rescales the
// throughput (unbiased; the plain tracer's PT_FLAG_UNBIASED_MIS mode is the
// same estimator with c = 1, so both converge to the same image).
// Training data: a path keeps, per surface vertex, the inputs, the sampled
// direction, its pdfs, the throughput before the bounce and the film total
// after the vertex's own NEE; when the path ends each vertex yields
// T = luminance((S_end - S_k) / throughput_k), the importance-weighted
// integrand along the sampled direction.
// ===========================================================================

__device__ __forceinline__ float luminance(f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

__device__ __forceinline__ void film_add_nn(unsigned long long* film, size_t pix, f3 c, WaveCounters* ctr) {
    film_add_rgb(film, pix, c.x, c.y, c.z, ctr);
}

__device__ __forceinline__ int warp_append_nn(int* counter, bool pred) {
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

// Vertex record k of a path slot (kNNVert float4): 0: pos xyz, n.x  1: n.yz, wo.xy
// 2: wo.z, wi xyz  3: p_bsdf(wi), throughput before the bounce (rgb)
// 4: film total after the vertex's own NEE (rgb), wi valid (non-delta)
// 5: film total before the NEE (rgb), p_bsdf(wi_nee)  6: wi_nee xyz, NEE valid.
constexpr int kNNVert = kNNVertFloat4;
__global__ void __launch_bounds__(256, 2) k_shade_nn(DevScene S, PathBuffers B, int cur, RenderParams P,
                                                  WaveCounters* ctr, unsigned long long* __restrict__ film,
                                                  const float4* __restrict__ params, NNPathData PD, int guided,
                                                  const DevBatchJob* __restrict__ jobs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = ctr->n_cur;
    bool push_sh = false, push_cont = false, release = false;
    float4 sh_o, sh_d, sh_c, no, nd, nt;
    int4 ninfo;
    int slot = -1, fin_bounce = 0, fin_nv = 0;
    if (i < n) {
        const float4 O = B.o[cur][i], D = B.d[cur][i], Tp = B.thr[cur][i];
        const int4 I = B.info[cur][i];
        const float4 H = B.hit[i];
        const int prim = __float_as_int(H.y);
        const int pixel = I.x, sample = I.y, bounce = I.z & 0xffff;
        const bool sdelta = (I.z >> 16) & 1;
        const int job = (int)((uint32_t)I.z >> kNNJobShift);
        const DevBatchJob* J = jobs + job;
        const uint32_t seed = J->seed;
        const int rr_start = J->rr_start, max_depth = J->max_depth;
        const size_t fpix = (size_t)(uint32_t)pixel + J->film_off;
        S.light_prim += J->light_off;
        S.light_area += J->light_off;
        S.n_lights = J->n_lights;
        slot = I.w;
        const size_t vbase = (size_t)slot * P.max_depth;
        const float p = O.w;
        f3 mul = mk(Tp.x, Tp.y, Tp.z);
        const f3 ro = mk(O.x, O.y, O.z), rd = mk(D.x, D.y, D.z);
        const bool train = PD.rec_cap > 0;  // vertex records and running totals only while training
        f3 Ssum = train ? f3of(PD.acc[slot]) : mk(0.f, 0.f, 0.f);
        if (train && bounce > 0) {  // the previous vertex's incident radiance is what arrives from now on
            const float w4 = PD.vert[kNNVert * (vbase + bounce - 1) + 4].w;
            PD.vert[kNNVert * (vbase + bounce - 1) + 4] = make_float4(Ssum.x, Ssum.y, Ssum.z, w4);
        }
        bool done = true;
        if (prim >= 0) {
            int kind;
            DevMaterial m;
            const Surf s = make_surf(S, prim, ro, rd, H.x, H.z, H.w, bounce == 0, &kind, &m);
            const f3 wo = -rd;
            if (kind == PT_MAT_EMISSIVE_) {
                float w = 1.0f;
                if (!sdelta) {
                    const int4 vi = __ldg(S.tri_vidx + prim);
                    const f3 a = f3of(__ldg(S.v_pos + vi.x)), b = f3of(__ldg(S.v_pos + vi.y)),
                             c = f3of(__ldg(S.v_pos + vi.z));
                    const float area = length(cross(b - a, c - a)) * 0.5f;
                    const float pdf_l = (1.0f / (float)S.n_lights) * (1.0f / area);
                    const float r = H.x;
                    const float p_nee = pdf_l * r * r / (fabsf(dot(s.n, rd)) + kEps);
                    w = p / (p + p_nee);
                }
                const f3 c = mul * mk(m.r, m.g, m.b) * w;
                film_add_nn(film, fpix, c, ctr);
                Ssum = Ssum + c;
            } else {
                const Rng4 r0 = rng4(seed, sample, pixel, bounce, 0);
                const Rng4 r1 = rng4(seed, sample, pixel, bounce, 1);
                const bool delta_mat = (m.kind == PT_MAT_DIELECTRIC_) || (m.kind == PT_MAT_GGX_ && m.delta);
                NNMixture mix;
                float c = 1.0f;
                if (guided && !delta_mat) {
                    nn_unpack_mixture(params + kNNMixF4 * (size_t)i, mix);
                    c = mix.c;
                }
                BSample bs;
                float pmix;
                if (r1.v[3] < c) {
                    bs = bsdf_sample(m, s, wo, r0.v[0], r0.v[1]);
                    pmix = (bs.delta || c >= 1.0f) ? bs.pdf : c * bs.pdf + (1.0f - c) * nn_mixture_pdf(mix, bs.wi);
                } else {
                    bs.wi = nn_mixture_sample(mix, r0.v[0], r0.v[1], r1.v[2]);
                    bs.delta = false;
                    bs.pdf = bsdf_pdf(m, s, wo, bs.wi);
                    pmix = c * bs.pdf + (1.0f - c) * nn_mixture_pdf(mix, bs.wi);
                }
                f3 nee_wi = mk(0.f, 0.f, 0.f);
                float nee_pb = 0.f, nee_ok = 0.f;
                if (!bs.delta && S.n_lights > 0) {  // NEE; the MIS weight uses the mixture pdf
                    const LSample ls = sample_light(S, s.p, r0.v[2], r0.v[3], r1.v[0]);
                    f3 sd = ls.pos - s.p;
                    const float len = length(sd);
                    sd = sd * (1.0f / len);
                    if (same_hemisphere(s, wo, sd)) {
                        float pb = bsdf_pdf(m, s, wo, sd);
                        nee_wi = sd;
                        nee_pb = pb;
                        nee_ok = 1.f;
                        if (c < 1.0f) pb = c * pb + (1.0f - c) * nn_mixture_pdf(mix, sd);
                        const float pn = ls.pdf * len * len / (fabsf(dot(ls.n, sd)) + kEps);
                        // at the last vertex no sampled direction follows, so NEE takes the full
                        // weight (the two estimators then converge to the same depth-limited image)
                        const float w = bounce + 1 < max_depth ? pn / (pb + pn) : 1.0f;
                        const f3 f = bsdf_eval(m, s, wo, sd);
                        const f3 cc = mul * f * ls.le * (1.0f / (ls.pdf * len * len)) * w;
                        if (cc.x != 0.f || cc.y != 0.f || cc.z != 0.f) {
                            push_sh = true;
                            const f3 so = s.p + sd * kEps;
                            sh_o = make_float4(so.x, so.y, so.z, len - 2.0f * kEps);
                            sh_d = make_float4(sd.x, sd.y, sd.z, __int_as_float((int)(uint32_t)fpix));
                            sh_c = make_float4(cc.x, cc.y, cc.z, __int_as_float(slot));
                        }
                    }
                }
                if (train) {  // this vertex's training records (completed when the path ends)
                    const size_t vi = kNNVert * (vbase + bounce);
                    PD.vert[vi] = make_float4(s.p.x, s.p.y, s.p.z, s.n.x);
                    PD.vert[vi + 1] = make_float4(s.n.y, s.n.z, wo.x, wo.y);
                    PD.vert[vi + 2] = make_float4(wo.z, bs.wi.x, bs.wi.y, bs.wi.z);
                    PD.vert[vi + 3] = make_float4(bs.delta ? 0.f : bs.pdf, mul.x, mul.y, mul.z);
                    PD.vert[vi + 4] = make_float4(Ssum.x, Ssum.y, Ssum.z, bs.delta ? 0.f : 1.f);
                    PD.vert[vi + 5] = make_float4(Ssum.x, Ssum.y, Ssum.z, nee_pb);
                    PD.vert[vi + 6] = make_float4(nee_wi.x, nee_wi.y, nee_wi.z, nee_ok);
                    fin_nv = bounce + 1;
                }
                if (same_hemisphere(s, wo, bs.wi) && pmix > 0.f) {
                    const f3 f = bsdf_eval(m, s, wo, bs.wi);
                    bool alive = true;
                    float surv = 1.0f;
                    if (bounce >= rr_start) {  // survival min(rr, 1): unbiased
                        if (P.flags & PT_FLAG_THROUGHPUT_RR_) {
                            const f3 mn = mul * f * (1.0f / pmix);
                            surv = fminf(1.0f, fmaxf(fmaxf(mn.x, mn.y), mn.z));
                        } else {
                            surv = fminf(russian_roulette(f), 1.0f);
                        }
                        if (r1.v[1] > surv) alive = false;
                    }
                    if (alive && bounce + 1 < max_depth) {
                        mul = mul * f * (1.0f / (pmix * surv));
                        const f3 oo = s.p + bs.wi * kEps;
                        push_cont = true;
                        done = false;
                        no = make_float4(oo.x, oo.y, oo.z, pmix);
                        nd = make_float4(bs.wi.x, bs.wi.y, bs.wi.z, D.w);  // w: the scene root
                        nt = make_float4(mul.x, mul.y, mul.z, 0.f);
                        ninfo = make_int4(pixel, sample,
                                          (bounce + 1) | ((bs.delta ? 1 : 0) << 16) | (job << kNNJobShift), slot);
                    }
                }
            }
        }
        if (train) PD.acc[slot] = make_float4(Ssum.x, Ssum.y, Ssum.z, 0.f);
        // vertices 0 .. bounce-1 had their sampled direction traced; the
        // records are emitted once this vertex's shadow ray has resolved
        fin_bounce = bounce;
        if (fin_nv < bounce) fin_nv = bounce;
        release = done;
    }
    const int js = warp_append_nn(&ctr->n_shadow, push_sh);
    if (push_sh) {
        B.sh_o[js] = sh_o;
        B.sh_d[js] = sh_d;
        B.sh_c[js] = sh_c;
    }
    const int jc = warp_append_nn(&ctr->n_next, push_cont);
    if (push_cont) {
        const int nx = 1 - cur;
        B.o[nx][jc] = no;
        B.d[nx][jc] = nd;
        B.thr[nx][jc] = nt;
        B.info[nx][jc] = ninfo;
    }
    const int jf = warp_append_nn(&ctr->n_fin, release);
    if (release) PD.fin[jf] = make_int4(slot, fin_bounce, fin_nv, 0);
}

// Finished paths.  Two records per vertex, both MIS-weighted one-sample
// estimates of f cos L_i / p along their direction (together an unbiased
// estimate of the gradient of the loss, one sample from each technique):
// * the sampled direction wi (traced for vertices 0 .. f.y-1):
//   T = lum((S_end - S_after_nee_k) / throughput_k);
// * the NEE direction, where the shadow ray was unoccluded:
//   T = lum((S_after_nee_k - S_before_nee_k) / throughput_k).
// S_after_nee of the last vertex is S_end (its shadow ray resolved before
// this kernel runs).  visit_records calls emit(vertex record, wi,
// p_bsdf(wi), T) for every record of the finished path f (slot, traced
// vertices, recorded vertices).
template <class Emit>
__device__ __forceinline__ void visit_records(const NNPathData& PD, int4 f, int max_depth, Emit emit) {
    const float4 Se = PD.acc[f.x];
    const size_t vbase = (size_t)f.x * max_depth;
    for (int k = 0; k < f.z; k++) {
        const float4* vr = PD.vert + kNNVert * (vbase + k);
        const float4 v2 = vr[2], v3 = vr[3], v4 = vr[4], v5 = vr[5], v6 = vr[6];
        const f3 inv = mk(v3.y > 0.f ? 1.0f / v3.y : 0.f, v3.z > 0.f ? 1.0f / v3.z : 0.f,
                          v3.w > 0.f ? 1.0f / v3.w : 0.f);
        const f3 after = k < f.z - 1 || k < f.y ? mk(v4.x, v4.y, v4.z) : mk(Se.x, Se.y, Se.z);
        if (v6.w != 0.f) {
            const f3 dn = mk(after.x - v5.x, after.y - v5.y, after.z - v5.z);
            const float T = luminance(mk(dn.x * inv.x, dn.y * inv.y, dn.z * inv.z));
            if (T > 0.f && isfinite(T)) emit(vr, mk(v6.x, v6.y, v6.z), v5.w, T);
        }
        if (k < f.y && v4.w != 0.f) {
            const f3 dS = mk(Se.x - after.x, Se.y - after.y, Se.z - after.z);
            const float T = luminance(mk(dS.x * inv.x, dS.y * inv.y, dS.z * inv.z));
            if (T > 0.f && isfinite(T)) emit(vr, mk(v2.y, v2.z, v2.w), v3.x, T);
        }
    }
}

// Finished paths: records are counted first, then one atomic per warp (all
// lanes of the same job; per lane otherwise) reserves room in the job's
// record buffer, then they are written (records beyond the buffer's
// capacity are dropped); the slots go back to the free list.
__global__ void __launch_bounds__(256) k_finish_nn(NNPathData PD, WaveCounters* ctr,
                                                   const DevNNJob* __restrict__ nnj, int max_depth) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = ctr->n_fin;
    const unsigned lane = threadIdx.x & 31u;
    const bool release = i < n;
    int4 f = make_int4(0, 0, 0, 0);
    if (release) f = PD.fin[i];
    bool records = release && PD.rec_cap > 0;
    const int job = records ? PD.slot_job[f.x] : -1;
    if (records) {
        // a path keeps its records with the job's probability, decided by a
        // hash of its slot and the iteration, never by its length: the
        // records of a round then sample its paths evenly (a quota filled in
        // finishing order would hold the short paths)
        const float keep = nnj[job].keep;
        if (keep < 1.0f) {
            uint32_t h = (uint32_t)f.x * 0x9E3779B1u ^ (uint32_t)ctr->stat_iters * 0x85EBCA77u;
            h ^= h >> 15;
            h *= 0x2C1B3C6Du;
            h ^= h >> 12;
            records = (float)(h >> 8) * (1.0f / 16777216.0f) < keep;
        }
    }
    int count = 0;
    if (records) visit_records(PD, f, max_depth, [&](const float4*, f3, float, float) { count++; });
    // one job for the whole warp (the usual case: jobs are rendered in order)?
    const int job0 = __shfl_sync(0xffffffffu, job, 0);
    const bool uniform = __all_sync(0xffffffffu, job == job0 || job < 0);
    int base = 0, incl = count;
    if (uniform) {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (unsigned)o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const int lead_job = __reduce_max_sync(0xffffffffu, (unsigned)(job + 1)) - 1;
        if (lane == 31 && total > 0) base = atomicAdd(nnj[lead_job].n_rec, total);
        base = __shfl_sync(0xffffffffu, base, 31) + incl - count;
    } else if (count > 0) {
        base = atomicAdd(nnj[job].n_rec, count);
    }
    if (records && count > 0) {
        const DevNNJob& Jn = nnj[job];
        int r = base;
        visit_records(PD, f, max_depth, [&](const float4* vr, f3 wi, float pb, float T) {
            if (r < Jn.rec_cap) {
                float4* o = Jn.rec + 4 * (size_t)r;
                o[0] = vr[0];
                o[1] = vr[1];
                o[2] = make_float4(vr[2].x, wi.x, wi.y, wi.z);
                o[3] = make_float4(pb, T, 0.f, 0.f);
            }
            r++;
        });
    }
    const int jr = warp_append_nn(&ctr->free_top, release);
    if (release) PD.slot_stack[jr] = f.x;
}

// NEE shadow rays of the learned-guide integrator: unoccluded contributions
// go to the film and to the owning path's running total (for its training
// targets).
__global__ void __launch_bounds__(kTraceThreads) k_shadow_nn(DevScene S, PathBuffers B, WaveCounters* ctr,
                                                   unsigned long long* __restrict__ film, NNPathData PD,
                                                   const DevBatchJob* __restrict__ jobs) {
    extern __shared__ uint4 snodes[];
    const int n = ctr->n_shadow;
    if (n == 0) return;
    const int nn = min(S.n_nodes, kSmemNodes) * 4;
    for (int k = threadIdx.x; k < nn; k += blockDim.x) snodes[k] = __ldg(S.nodes + k);
    __syncthreads();
    TraceCount cnt{0u, 0u};
    persistent_trace<true, false>(
        S, snodes, n, &ctr->fetch_sh, &ctr->status, cnt,
        [&](int i, float3& o, float3& d, float& tmax, uint32_t& root) {
            const float4 a = B.sh_o[i], b = B.sh_d[i];
            o = make_float3(a.x, a.y, a.z);
            d = make_float3(b.x, b.y, b.z);
            tmax = a.w;
            if (root != kTravDone) root = jobs[PD.slot_job[__float_as_int(B.sh_c[i].w)]].root;
        },
        [&](int i, const HitRec& h) {
            if (h.prim < 0) {
                const float4 c = B.sh_c[i];
                const f3 cc = mk(c.x, c.y, c.z);
                film_add_nn(film, (uint32_t)__float_as_int(B.sh_d[i].w), cc, ctr);
                if (PD.rec_cap > 0) {
                    const int slot = __float_as_int(c.w);
                    const float4 a = PD.acc[slot];
                    PD.acc[slot] = make_float4(a.x + cc.x, a.y + cc.y, a.z + cc.z, 0.f);
                }
            }
        });
}

cudaError_t nn_shadow_smem_limit() {
    return cudaFuncSetAttribute(k_shadow_nn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemNodeBytes);
}

// Camera paths (stratified like pathtracerMIS.h:148-153) with a vertex slot.
__global__ void __launch_bounds__(256) k_generate_nn(DevScene S, PathBuffers B, int cur, WaveCounters* ctr,
                                                     NNPathData PD, const DevBatchJob* __restrict__ jobs,
                                                     int n_jobs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_next = ctr->n_next;
    const int avail = min(B.capacity - n_next, ctr->free_top);
    unsigned long long w = ctr->work_next + (unsigned long long)t;
    if (t >= avail || w >= ctr->work_total) return;
    int job = 0;
    if (n_jobs > 1) {  // job ranges ascend (as find_job in render.cu)
        int lo = 0, hi = n_jobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&jobs[mid].work_begin) <= w) lo = mid;
            else hi = mid - 1;
        }
        job = lo;
    }
    const DevBatchJob* J = jobs + job;
    w -= J->work_begin;
    const DevCamera* C = &J->cam;
    const int width = C->width, height = C->height, spp_axis = J->spp_axis;
    const unsigned long long npix = (unsigned long long)width * height;
    const int sample = (int)(w / npix);
    int pixel = (int)(w - (unsigned long long)sample * npix);
    if (J->tile_w * J->tile_h > 1) {  // tiled pass order (a bijection of the pixels)
        const int tw = J->tile_w, th = J->tile_h;
        const int tile = pixel / (tw * th), r = pixel - tile * (tw * th);
        const int tiles_x = width / tw;
        const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
        pixel = (ty * th + r / tw) * width + tx * tw + r % tw;
    }
    const int px = pixel % width, py = pixel / width;
    const Rng4 r = rng4(J->seed, sample, pixel, 0xffffu, 2);
    float cx, cy;
    if (spp_axis > 0) {  // pathtracerMIS.h:148-153
        const int k = sample / spp_axis, l = sample - (sample / spp_axis) * spp_axis;
        cx = (((float)px + ((float)k + r.v[0]) / (float)spp_axis) / (float)width) * 2.0f - 1.0f;
        cy = -((((float)py + ((float)l + r.v[1]) / (float)spp_axis) / (float)height) * 2.0f - 1.0f);
    } else {
        cx = (((float)px + r.v[0]) / (float)width) * 2.0f - 1.0f;
        cy = -((((float)py + r.v[1]) / (float)height) * 2.0f - 1.0f);
    }
    const float dx = cx * C->tan_fovy * C->aspect, dy = cy * C->tan_fovy, dz = -1.0f;
    const f3 d = normalized(mk(C->m[0] * dx + C->m[1] * dy + C->m[2] * dz, C->m[3] * dx + C->m[4] * dy + C->m[5] * dz,
                               C->m[6] * dx + C->m[7] * dy + C->m[8] * dz));
    const int nx = 1 - cur;
    const int j = n_next + t;
    const int slot = PD.slot_stack[ctr->free_top - 1 - t];
    PD.acc[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    PD.slot_job[slot] = job;
    B.o[nx][j] = make_float4(C->o[0], C->o[1], C->o[2], 1.0f);
    B.d[nx][j] = make_float4(d.x, d.y, d.z, __uint_as_float(J->root));
    B.thr[nx][j] = make_float4(1.f, 1.f, 1.f, 0.f);
    B.info[nx][j] = make_int4(pixel, sample, (1 << 16) | (job << kNNJobShift), slot);  // sampled_delta starts true
}

__global__ void k_advance_nn(WaveCounters* ctr, int capacity) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int n_next = ctr->n_next;
    const unsigned long long left = ctr->work_total - ctr->work_next;
    unsigned long long room = (unsigned long long)(capacity - n_next);
    if ((unsigned long long)ctr->free_top < room) room = (unsigned long long)ctr->free_top;
    const unsigned long long added = left < room ? left : room;
    ctr->work_next += added;
    ctr->stat_paths += added;
    ctr->stat_shadow += (unsigned long long)ctr->n_shadow;
    ctr->free_top -= (int)added;
    ctr->n_cur = n_next + (int)added;
    ctr->stat_closest += (unsigned long long)ctr->n_cur;
    ctr->n_next = 0;
    ctr->n_shadow = 0;
    ctr->n_fin = 0;
    ctr->fetch_ext = 0;
    ctr->fetch_sh = 0;
    ctr->stat_iters += 1;
}


void launch_nn_shade(const DevScene& S, const PathBuffers& B, int cur, const RenderParams& P, WaveCounters* ctr,
                     unsigned long long* film, const float4* params, const NNPathData& PD, bool guided,
                     const DevBatchJob* jobs, cudaStream_t st) {
    k_shade_nn<<<(B.capacity + 255) / 256, 256, 0, st>>>(S, B, cur, P, ctr, film, params, PD, guided ? 1 : 0, jobs);
}
void launch_nn_shadow(const DevScene& S, const PathBuffers& B, WaveCounters* ctr, unsigned long long* film,
                      const NNPathData& PD, const DevBatchJob* jobs, int num_sms, cudaStream_t st) {
    k_shadow_nn<<<num_sms * kTraceBlocksPerSM, kTraceThreads, kSmemNodeBytes, st>>>(S, B, ctr, film, PD, jobs);
}
void launch_nn_generate(const DevScene& S, const PathBuffers& B, int cur, WaveCounters* ctr, const NNPathData& PD,
                        const DevBatchJob* jobs, int n_jobs, cudaStream_t st) {
    k_generate_nn<<<(B.capacity + 255) / 256, 256, 0, st>>>(S, B, cur, ctr, PD, jobs, n_jobs);
    k_advance_nn<<<1, 32, 0, st>>>(ctr, B.capacity);
}
void launch_nn_finish(const NNPathData& PD, WaveCounters* ctr, const DevNNJob* nnj, int max_depth, int capacity,
                      cudaStream_t st) {
    k_finish_nn<<<(capacity + 255) / 256, 256, 0, st>>>(PD, ctr, nnj, max_depth);
}

}  // namespace cpppt_gb300
