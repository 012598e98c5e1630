// mlp.cuh -- the learned early-termination network: constants, parameter layout and the
// warp-cooperative forward pass shared by the search kernel and the training kernels.
//
// 8 standardised search-state features -> 64 -> 64 -> 1 (ReLU hidden layers, one logit).
// Packed parameters (BF16 in device memory), weight matrices input-major so that the lanes of a
// warp, which own consecutive output units, read consecutive words:
//   W1[8][64] | b1[64] | W2[64][64] | b2[64] | w3[64] | b3      (Wk[in][out])
// Standardisation block (FP32): mean[8] | inv_std[8].
#pragma once

#include <cstdint>

#include <cuda_bf16.h>

namespace qg {

constexpr int kMlpIn = 8;
constexpr int kMlpHidden = 64;
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpHidden * kMlpIn;
constexpr int kMlpW2 = kMlpB1 + kMlpHidden;
constexpr int kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpW3 = kMlpB2 + kMlpHidden;
constexpr int kMlpB3 = kMlpW3 + kMlpHidden;
constexpr int kMlpParams = kMlpB3 + 1;  // 4801

__device__ __forceinline__ float mlp_w(const uint16_t *w, int i) {
    return __bfloat162float(__ushort_as_bfloat16(w[i]));
}

// Warp-cooperative forward of one sample. `f` (standardised features) must be identical in
// all lanes. Lane l owns hidden units l and l+32. Returns the logit in every lane; optionally
// returns this lane's two hidden activations of each layer.
__device__ __forceinline__ float mlp_forward_warp(const float (&f)[kMlpIn], const uint16_t *w, int lane,
                                                  float *h1a = nullptr, float *h1b = nullptr,
                                                  float *h2a = nullptr, float *h2b = nullptr) {
    float a1[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const int j = lane + 32 * u;
        float acc = mlp_w(w, kMlpB1 + j);
#pragma unroll
        for (int i = 0; i < kMlpIn; ++i) acc = __fmaf_rn(mlp_w(w, kMlpW1 + i * kMlpHidden + j), f[i], acc);
        a1[u] = fmaxf(acc, 0.0f);
    }
    float acc2[2] = {mlp_w(w, kMlpB2 + lane), mlp_w(w, kMlpB2 + lane + 32)};
#pragma unroll 8
    for (int i = 0; i < kMlpHidden; ++i) {
        const float hi = __shfl_sync(0xffffffffu, a1[i >> 5], i & 31);
        acc2[0] = __fmaf_rn(mlp_w(w, kMlpW2 + i * kMlpHidden + lane), hi, acc2[0]);
        acc2[1] = __fmaf_rn(mlp_w(w, kMlpW2 + i * kMlpHidden + lane + 32), hi, acc2[1]);
    }
    const float a2a = fmaxf(acc2[0], 0.0f), a2b = fmaxf(acc2[1], 0.0f);
    float out = __fmaf_rn(mlp_w(w, kMlpW3 + lane), a2a, mlp_w(w, kMlpW3 + lane + 32) * a2b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) out += __shfl_xor_sync(0xffffffffu, out, o);
    if (h1a) {
        *h1a = a1[0];
        *h1b = a1[1];
        *h2a = a2a;
        *h2b = a2b;
    }
    return out + mlp_w(w, kMlpB3);
}

// Shared-memory copy for the search kernel (one per block, staged once): every word packs
// the BF16 pair (unit j, unit j+32) that lane j reads together, so a layer step is one 32-bit
// shared load per lane. Words: W1 [8][32] | b1 [32] | W2 [64][32] | b2 [32] | w3 [32] | b3.
constexpr int kMlpSmemW1 = 0;
constexpr int kMlpSmemB1 = kMlpSmemW1 + kMlpIn * 32;
constexpr int kMlpSmemW2 = kMlpSmemB1 + 32;
constexpr int kMlpSmemB2 = kMlpSmemW2 + kMlpHidden * 32;
constexpr int kMlpSmemW3 = kMlpSmemB2 + 32;
constexpr int kMlpSmemB3 = kMlpSmemW3 + 32;
constexpr int kMlpSmemWords = kMlpSmemB3 + 1;
constexpr int kMlpSmemBytes = ((kMlpSmemWords * 4 + 15) / 16) * 16;

__device__ __forceinline__ uint32_t mlp_pair(const uint16_t *w, int base, int j) {
    return static_cast<uint32_t>(w[base + j]) | (static_cast<uint32_t>(w[base + j + 32]) << 16);
}

// All threads of the block call it; the caller synchronises before use.
__device__ __forceinline__ void mlp_stage_smem(const uint16_t *w, uint32_t *s, int tid, int nthreads) {
    for (int t = tid; t < kMlpSmemWords; t += nthreads) {
        uint32_t v;
        if (t < kMlpSmemB1) v = mlp_pair(w, kMlpW1 + (t >> 5) * kMlpHidden, t & 31);
        else if (t < kMlpSmemW2) v = mlp_pair(w, kMlpB1, t - kMlpSmemB1);
        else if (t < kMlpSmemB2) v = mlp_pair(w, kMlpW2 + ((t - kMlpSmemW2) >> 5) * kMlpHidden, (t - kMlpSmemW2) & 31);
        else if (t < kMlpSmemW3) v = mlp_pair(w, kMlpB2, t - kMlpSmemB2);
        else if (t < kMlpSmemB3) v = mlp_pair(w, kMlpW3, t - kMlpSmemW3);
        else v = w[kMlpB3];
        s[t] = v;
    }
}

__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xFFFF0000u); }

// mlp_forward_warp over the shared-memory copy: the same operations in the same order.
__device__ __forceinline__ float mlp_forward_warp_smem(const float (&f)[kMlpIn], const uint32_t *s, int lane) {
    const uint32_t bb1 = s[kMlpSmemB1 + lane];
    float acc0 = bf16_lo(bb1), acc1 = bf16_hi(bb1);
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) {
        const uint32_t ww = s[kMlpSmemW1 + i * 32 + lane];
        acc0 = __fmaf_rn(bf16_lo(ww), f[i], acc0);
        acc1 = __fmaf_rn(bf16_hi(ww), f[i], acc1);
    }
    const float a1[2] = {fmaxf(acc0, 0.0f), fmaxf(acc1, 0.0f)};
    const uint32_t bb2 = s[kMlpSmemB2 + lane];
    float acc2[2] = {bf16_lo(bb2), bf16_hi(bb2)};
#pragma unroll 8
    for (int i = 0; i < kMlpHidden; ++i) {
        const float hi = __shfl_sync(0xffffffffu, a1[i >> 5], i & 31);
        const uint32_t ww = s[kMlpSmemW2 + i * 32 + lane];
        acc2[0] = __fmaf_rn(bf16_lo(ww), hi, acc2[0]);
        acc2[1] = __fmaf_rn(bf16_hi(ww), hi, acc2[1]);
    }
    const float a2a = fmaxf(acc2[0], 0.0f), a2b = fmaxf(acc2[1], 0.0f);
    const uint32_t w3 = s[kMlpSmemW3 + lane];
    float out = __fmaf_rn(bf16_lo(w3), a2a, bf16_hi(w3) * a2b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) out += __shfl_xor_sync(0xffffffffu, out, o);
    return out + bf16_lo(s[kMlpSmemB3]);
}

}  // namespace qg
