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

}  // namespace qg
