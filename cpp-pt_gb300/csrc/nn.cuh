// Learned path guide: network layout, input encoding and the von Mises-Fisher
// mixture it outputs.  (No counterpart in the reference, which has only the
// SD-tree guide; the learned guide is compared against it and against plain
// PT.)
//
// Network: 64 inputs -> 64 -> 64 -> 64 (ReLU) -> 48 outputs, no biases
// (the constant input feature acts as one), BF16 weights and activations,
// FP32 accumulation in tensor memory (tcgen05.mma kind::f16, nn.cu).
// Inputs (64): frequency encoding of the position normalised to the scene
// box (3 axes x 8 octaves x sin/cos = 48), shading normal (3), direction to
// the previous vertex wo (3), 1, zero padding.
// Outputs (48): 8 lobes x (mean direction raw xyz) = 24, 8 concentrations,
// 8 mixture logits, 1 selection logit, 7 unused.
// Mixture: lobe j has mean mu_j = normalise(raw), kappa_j = softplus(raw) +
// 0.1 (clamped to 5e3), weight w_j = softmax; the guide is chosen with
// probability 1 - c where c = c_lo + (c_hi - c_lo) sigmoid(selection logit)
// is the BSDF fraction; c_lo >= 0.1 (default range [0.1, 0.9]) keeps BSDF
// sampling at 10% or more, so the estimator stays unbiased wherever the BSDF
// is non-zero.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "nn.h"
#include "shade.cuh"

namespace cpppt_gb300 {

constexpr int kNNIn = 64;
constexpr int kNNHidden = 64;
constexpr int kNNOut = 48;
constexpr int kNNLobes = 8;
constexpr int kNNLayers = 4;  // 64x64, 64x64, 64x64, 64x48
// weights: three 64x64 matrices and one 64x48, in->out
constexpr int kNNWeights = 3 * 64 * 64 + 64 * 48;
constexpr int kNNParams = 41;  // post-processed mixture per sample: 8 x (mu xyz, kappa, w) + c

__host__ __device__ constexpr int nn_layer_out(int l) { return l == kNNLayers - 1 ? kNNOut : kNNHidden; }
__host__ __device__ constexpr int nn_layer_offset(int l) { return l * 64 * 64; }

// One-blob encoding (Mueller et al. 2019, "Neural importance sampling"):
// a scalar s in [0, 1] spread over kNNBlobBins Gaussian bins of width
// sigma = 1 / kNNBlobBins centred at (b + 1/2) / kNNBlobBins; `wrap`: s is
// periodic (an azimuth), distances are taken around the circle.
constexpr int kNNBlobBins = 6;
__device__ __forceinline__ float one_blob(float s, int b, bool wrap) {
    float d = fabsf(s - ((float)b + 0.5f) * (1.0f / kNNBlobBins));
    if (wrap) d = fminf(d, 1.0f - d);
    const float z = d * (float)kNNBlobBins;  // distance in units of sigma
    return __expf(-0.5f * z * z);
}

// Input feature j of a sample (pos already normalised to [0,1]^3) under
// encoding 1 (PT_NN_ENC_ONEBLOB): position at 6 octaves (36), one-blob
// cos theta and phi of the normal and of wo (4 x 6), 1.
__device__ __forceinline__ float nn_feature_oneblob(int j, f3 pn, f3 n, f3 wo) {
    if (j < 36) {
        const int c = j / 12, k = (j % 12) >> 1;
        const float x = c == 0 ? pn.x : (c == 1 ? pn.y : pn.z);
        const float a = x * (float)(1 << k) * kPi;
        return (j & 1) ? __cosf(a) : __sinf(a);
    }
    if (j < 36 + 4 * kNNBlobBins) {
        const int q = (j - 36) / kNNBlobBins, b = (j - 36) % kNNBlobBins;
        const f3 v = q < 2 ? n : wo;
        const float s = (q & 1) ? atan2f(v.y, v.x) * (0.5f * kInvPi) + 0.5f : 0.5f * (v.z + 1.0f);
        return one_blob(s, b, (q & 1) != 0);
    }
    return j == 36 + 4 * kNNBlobBins ? 1.0f : 0.0f;
}

// Input feature j of a sample (pos already normalised to [0,1]^3).
__device__ __forceinline__ float nn_feature(int j, f3 pn, f3 n, f3 wo, int encoding = 0) {
    if (encoding == 1) return nn_feature_oneblob(j, pn, n, wo);
    if (j < 48) {
        const int c = j >> 4, k = (j >> 1) & 7;
        const float x = c == 0 ? pn.x : (c == 1 ? pn.y : pn.z);
        const float a = x * (float)(1 << k) * kPi;
        return (j & 1) ? __cosf(a) : __sinf(a);
    }
    switch (j) {
        case 48: return n.x;
        case 49: return n.y;
        case 50: return n.z;
        case 51: return wo.x;
        case 52: return wo.y;
        case 53: return wo.z;
        case 54: return 1.0f;
        default: return 0.0f;
    }
}

// All 64 input features of a sample under encoding (the values of
// nn_feature, with the branch on the encoding taken once and the one-blob
// angles computed once per sample).
// ONEBLOB = false: a kernel instance for networks that all use the
// frequency encoding (the branch and the one-blob code compiled out).
template <bool ONEBLOB>
__device__ __forceinline__ void nn_features(float v[64], f3 pn, f3 n, f3 wo, int encoding) {
    if (ONEBLOB && encoding == 1) {
#pragma unroll
        for (int j = 0; j < 36; j++) v[j] = nn_feature_oneblob(j, pn, n, wo);
        const float s4[4] = {0.5f * (n.z + 1.0f), atan2f(n.y, n.x) * (0.5f * kInvPi) + 0.5f, 0.5f * (wo.z + 1.0f),
                             atan2f(wo.y, wo.x) * (0.5f * kInvPi) + 0.5f};
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int b = 0; b < kNNBlobBins; b++) v[36 + q * kNNBlobBins + b] = one_blob(s4[q], b, (q & 1) != 0);
#pragma unroll
        for (int j = 36 + 4 * kNNBlobBins; j < 64; j++) v[j] = j == 36 + 4 * kNNBlobBins ? 1.0f : 0.0f;
    } else {
#pragma unroll
        for (int j = 0; j < 64; j++) v[j] = nn_feature(j, pn, n, wo, 0);
    }
}

__device__ __forceinline__ float softplusf(float x) { return x > 15.f ? x : log1pf(__expf(x)); }

// vMF lobe pdf over the sphere: kappa / (2 pi (1 - e^{-2 kappa})) e^{kappa (mu.w - 1)}
__device__ __forceinline__ float vmf_pdf(f3 mu, float kappa, f3 w) {
    const float norm = kappa / (2.0f * kPi * (-expm1f(-2.0f * kappa)));
    return norm * __expf(kappa * (dot(mu, w) - 1.0f));
}

// Sampling a vMF lobe (Jakob 2012, "Numerically stable sampling of the von
// Mises-Fisher distribution on S^2"): cos = 1 + log(u1 + (1-u1) e^{-2 kappa}) / kappa.
__device__ __forceinline__ f3 vmf_sample(f3 mu, float kappa, float u1, float u2) {
    const float w = 1.0f + __logf(u1 + (1.0f - u1) * __expf(-2.0f * kappa)) / kappa;
    const float cw = fminf(1.0f, fmaxf(-1.0f, w));
    const float sw = sqrtf(fmaxf(0.0f, 1.0f - cw * cw));
    float sp, cp;
    sincosf(2.0f * kPi * u2, &sp, &cp);
    // orthonormal basis around mu (Duff et al. 2017, "Building an Orthonormal Basis, Revisited")
    const float sign = copysignf(1.0f, mu.z);
    const float a = -1.0f / (sign + mu.z);
    const float b = mu.x * mu.y * a;
    const f3 t = mk(1.0f + sign * mu.x * mu.x * a, sign * b, -sign * mu.x);
    const f3 bt = mk(b, sign + mu.y * mu.y * a, -mu.y);
    return t * (sw * cp) + bt * (sw * sp) + mu * cw;
}

// Mixture parameters of one sample, post-processed from the raw outputs.
struct NNMix {
    f3 mu[kNNLobes];
    float kappa[kNNLobes];
    float w[kNNLobes];
    float c;  // probability of sampling the BSDF
};

__device__ __forceinline__ void nn_postprocess(const float* raw, float* out /*41*/, float c_lo, float c_hi) {
    float mx = -1e30f;
    for (int j = 0; j < kNNLobes; j++) mx = fmaxf(mx, raw[32 + j]);
    float e[kNNLobes], sum = 0.f;
    for (int j = 0; j < kNNLobes; j++) { e[j] = __expf(raw[32 + j] - mx); sum += e[j]; }
    for (int j = 0; j < kNNLobes; j++) {
        f3 m = mk(raw[3 * j], raw[3 * j + 1], raw[3 * j + 2]);
        const float l = sqrtf(dot(m, m));
        m = l > 1e-20f ? m * (1.0f / l) : mk(0.f, 0.f, 1.f);
        out[5 * j] = m.x;
        out[5 * j + 1] = m.y;
        out[5 * j + 2] = m.z;
        out[5 * j + 3] = fminf(softplusf(raw[24 + j]) + 0.1f, 5000.0f);
        out[5 * j + 4] = e[j] / sum;
    }
    out[40] = c_lo + (c_hi - c_lo) / (1.0f + __expf(-raw[40]));
}

// ---- the mixture as the shading stage reads it ----
// Per path vertex, 8 x 16 B: halves 0..39 = lobe j's mean direction xyz,
// concentration and selection probability (fp16, at 5 j .. 5 j + 4), then
// eight floats a_j = (selection probability) x (vMF normaliser), then c.
// Sampling and the pdf use the same stored values: the probability of
// choosing lobe j is its stored fp16 value (the last lobe takes the rest,
// as nn_mixture_sample picks it), the normaliser is computed from the
// stored fp16 concentration, and the mean direction is renormalised after
// unpacking, so the pdf is the density of the sampler up to FP32 rounding.
struct NNMixture {
    f3 mu[kNNLobes];
    float kappa[kNNLobes];
    float w[kNNLobes];  // lobe selection probabilities (cumulated by the sampler)
    float a[kNNLobes];  // w x kappa / (2 pi (1 - e^{-2 kappa}))
    float c;            // probability of sampling the BSDF
};

__device__ __forceinline__ float vmf_norm(float kappa) { return kappa / (2.0f * kPi * (-expm1f(-2.0f * kappa))); }

// prm: the 41 post-processed parameters (nn_postprocess).
__device__ __forceinline__ void nn_pack_mixture(const float* prm, float4* out /*kNNMixF4*/) {
    __half h[40];
    float acc = 0.f, a[kNNLobes];
#pragma unroll
    for (int j = 0; j < kNNLobes; j++) {
        h[5 * j] = __float2half_rn(prm[5 * j]);
        h[5 * j + 1] = __float2half_rn(prm[5 * j + 1]);
        h[5 * j + 2] = __float2half_rn(prm[5 * j + 2]);
        h[5 * j + 3] = __float2half_rn(prm[5 * j + 3]);
        h[5 * j + 4] = __float2half_rn(prm[5 * j + 4]);
        const float wj = j < kNNLobes - 1 ? __half2float(h[5 * j + 4]) : fmaxf(0.0f, 1.0f - acc);
        acc += __half2float(h[5 * j + 4]);
        a[j] = wj * vmf_norm(__half2float(h[5 * j + 3]));
    }
    const uint32_t* hw = reinterpret_cast<const uint32_t*>(h);
#pragma unroll
    for (int k = 0; k < 5; k++)
        out[k] = make_float4(__uint_as_float(hw[4 * k]), __uint_as_float(hw[4 * k + 1]), __uint_as_float(hw[4 * k + 2]),
                             __uint_as_float(hw[4 * k + 3]));
    out[5] = make_float4(a[0], a[1], a[2], a[3]);
    out[6] = make_float4(a[4], a[5], a[6], a[7]);
    out[7] = make_float4(prm[40], 0.f, 0.f, 0.f);
}

__device__ __forceinline__ void nn_unpack_mixture(const float4* __restrict__ p, NNMixture& M) {
    uint32_t hw[20];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float4 q = p[k];
        hw[4 * k] = __float_as_uint(q.x);
        hw[4 * k + 1] = __float_as_uint(q.y);
        hw[4 * k + 2] = __float_as_uint(q.z);
        hw[4 * k + 3] = __float_as_uint(q.w);
    }
    const __half* h = reinterpret_cast<const __half*>(hw);
#pragma unroll
    for (int j = 0; j < kNNLobes; j++) {
        M.mu[j] = normalized(mk(__half2float(h[5 * j]), __half2float(h[5 * j + 1]), __half2float(h[5 * j + 2])));
        M.kappa[j] = __half2float(h[5 * j + 3]);
        M.w[j] = __half2float(h[5 * j + 4]);
    }
    const float4 a0 = p[5], a1 = p[6];
    M.a[0] = a0.x; M.a[1] = a0.y; M.a[2] = a0.z; M.a[3] = a0.w;
    M.a[4] = a1.x; M.a[5] = a1.y; M.a[6] = a1.z; M.a[7] = a1.w;
    M.c = p[7].x;
}

__device__ __forceinline__ float nn_mixture_pdf(const NNMixture& M, f3 w) {
    float pdf = 0.f;
#pragma unroll
    for (int j = 0; j < kNNLobes; j++) pdf += M.a[j] * __expf(M.kappa[j] * (dot(M.mu[j], w) - 1.0f));
    return pdf;
}

__device__ __forceinline__ f3 nn_mixture_sample(const NNMixture& M, float u0, float u1, float u2) {
    int j = kNNLobes - 1;
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < kNNLobes - 1; k++) {
        acc += M.w[k];
        if (u0 < acc && j == kNNLobes - 1) j = k;
    }
    f3 mu = M.mu[0];
    float kappa = M.kappa[0];
#pragma unroll
    for (int k = 1; k < kNNLobes; k++)
        if (k == j) { mu = M.mu[k]; kappa = M.kappa[k]; }
    return vmf_sample(mu, kappa, u1, u2);
}

// two floats as a bf16 pair (round to nearest even), low half first
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

}  // namespace cpppt_gb300
