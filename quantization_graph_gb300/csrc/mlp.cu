// mlp.cu -- training and batch inference of the learned early-termination network (mlp.cuh).
// The reference has no counterpart: its search stops only at fixed L or by the kth / stall
// heuristics (ours_diskann.rs:1784-1809).
//
// Training keeps FP32 master weights; forward and backward use their BF16 rounding (the
// gradient is taken with respect to the rounded weights and applied to the masters), with FP32
// accumulation. Loss: binary cross-entropy with logits (the stop classifier) or half the
// squared error of the output (the hop budget), mean over the batch.
//
// forward:  one warp per sample (the same warp-cooperative pass the search kernel runs).
// backward: one warp per strided set of samples; each lane owns hidden units l and l+32, so its
//           gradient columns are private; they are kept in per-warp shared memory (input-major,
//           so lanes write consecutive words), summed over the block's warps and added to the
//           global gradient with one atomicAdd per parameter per block.
// adam:     one thread per parameter; refreshes the BF16 copy.
#include <cstdint>

#include <cuda_bf16.h>

#include "mlp.cuh"
#include "qg_kernels.h"

namespace qg {
namespace {

constexpr int kWarps = 2;  // 2 x 17 KB of per-warp gradients fit static shared memory

__device__ __forceinline__ void standardise(const float *x, const float *norm, float (&f)[kMlpIn]) {
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) f[i] = (x[i] - norm[i]) * norm[kMlpIn + i];
}

__global__ void __launch_bounds__(128) mlp_forward_kernel(const float *X, size_t n, const float *norm,
                                                          const uint16_t *w, float *logits) {
    const size_t s = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= n) return;
    float f[kMlpIn];
    standardise(X + s * kMlpIn, norm, f);
    const float z = mlp_forward_warp(f, w, lane);
    if (lane == 0) logits[s] = z;
}

// per-warp gradients in shared memory, in the parameter layout itself: the weight matrices are
// input-major, so lane j (output unit j) writes consecutive words
template <bool kMse>
__global__ void __launch_bounds__(kWarps * 32) mlp_backward_kernel(const float *X, const float *y, size_t n,
                                                                   const float *norm, const uint16_t *w,
                                                                   float *grad, float *loss) {
    __shared__ float g[kWarps][kMlpParams];
    __shared__ float h1s[kWarps][kMlpHidden];
    __shared__ float d2s[kWarps][kMlpHidden];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *gw = g[warp];
    for (int i = lane; i < kMlpParams; i += 32) gw[i] = 0.0f;
    __syncwarp();
    float wloss = 0.0f;
    const size_t nwarps = static_cast<size_t>(gridDim.x) * kWarps;
    const float inv_n = 1.0f / static_cast<float>(n);
    for (size_t s = static_cast<size_t>(blockIdx.x) * kWarps + warp; s < n; s += nwarps) {
        float f[kMlpIn];
        standardise(X + s * kMlpIn, norm, f);
        float h1a, h1b, h2a, h2b;
        const float z = mlp_forward_warp(f, w, lane, &h1a, &h1b, &h2a, &h2b);
        const float t = y[s];
        float dz;
        if constexpr (kMse) {
            wloss += 0.5f * (z - t) * (z - t);
            dz = (z - t) * inv_n;
        } else {
            wloss += fmaxf(z, 0.0f) - z * t + log1pf(expf(-fabsf(z)));
            dz = (1.0f / (1.0f + expf(-z)) - t) * inv_n;
        }
        h1s[warp][lane] = h1a;
        h1s[warp][lane + 32] = h1b;
        // layer 3
        gw[kMlpW3 + lane] += dz * h2a;
        gw[kMlpW3 + lane + 32] += dz * h2b;
        const float d2a = h2a > 0.0f ? dz * mlp_w(w, kMlpW3 + lane) : 0.0f;
        const float d2b = h2b > 0.0f ? dz * mlp_w(w, kMlpW3 + lane + 32) : 0.0f;
        gw[kMlpB2 + lane] += d2a;
        gw[kMlpB2 + lane + 32] += d2b;
        d2s[warp][lane] = d2a;
        d2s[warp][lane + 32] = d2b;
        __syncwarp();
        // layer 2: dW2[i][j] = h1[i] * d2[j]
        for (int i = 0; i < kMlpHidden; ++i) {
            const float hi = h1s[warp][i];
            gw[kMlpW2 + i * kMlpHidden + lane] += d2a * hi;
            gw[kMlpW2 + i * kMlpHidden + lane + 32] += d2b * hi;
        }
        // dh1[i] = sum_j d2[j] W2[j][i] for this lane's i = lane, lane + 32
        float dh[2] = {0.0f, 0.0f};
        for (int j = 0; j < kMlpHidden; ++j) {
            const float dj = d2s[warp][j];
            dh[0] = __fmaf_rn(dj, mlp_w(w, kMlpW2 + lane * kMlpHidden + j), dh[0]);
            dh[1] = __fmaf_rn(dj, mlp_w(w, kMlpW2 + (lane + 32) * kMlpHidden + j), dh[1]);
        }
        const float d1a = h1a > 0.0f ? dh[0] : 0.0f;
        const float d1b = h1b > 0.0f ? dh[1] : 0.0f;
        gw[kMlpB1 + lane] += d1a;
        gw[kMlpB1 + lane + 32] += d1b;
#pragma unroll
        for (int c = 0; c < kMlpIn; ++c) {
            gw[kMlpW1 + c * kMlpHidden + lane] += d1a * f[c];
            gw[kMlpW1 + c * kMlpHidden + lane + 32] += d1b * f[c];
        }
        if (lane == 0) gw[kMlpB3] += dz;
        __syncwarp();
    }
    __syncthreads();
    // sum the warps, one atomicAdd per parameter per block
    for (int p = threadIdx.x; p < kMlpParams; p += blockDim.x) {
        float v = 0.0f;
        for (int k = 0; k < kWarps; ++k) v += g[k][p];
        if (v != 0.0f) atomicAdd(&grad[p], v);
    }
    if (lane == 0) atomicAdd(loss, wloss * inv_n);  // the logit, hence wloss, is warp-uniform
}

__global__ void mlp_adam_kernel(float *master, uint16_t *w, const float *grad, float *m, float *v, int n,
                                float lr, float beta1, float beta2, float eps, float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = grad[i];
    const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float nw = master[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    master[i] = nw;
    w[i] = __bfloat16_as_ushort(__float2bfloat16_rn(nw));
}

}  // namespace

cudaError_t launch_mlp_forward(const float *X, size_t n, const float *norm, const uint16_t *w, float *logits,
                               cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    mlp_forward_kernel<<<static_cast<unsigned>((n * 32 + 127) / 128), 128, 0, stream>>>(X, n, norm, w, logits);
    return cudaGetLastError();
}

cudaError_t launch_mlp_backward(const float *X, const float *y, size_t n, const float *norm, const uint16_t *w,
                                float *grad, float *loss, cudaStream_t stream, bool mse) {
    cudaError_t e = cudaMemsetAsync(grad, 0, kMlpParams * sizeof(float), stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(loss, 0, sizeof(float), stream);
    if (e != cudaSuccess || n == 0) return e;
    size_t blocks = (n + kWarps * 16 - 1) / (kWarps * 16);  // ~16 samples per warp
    if (blocks > 4096) blocks = 4096;
    if (mse)
        mlp_backward_kernel<true><<<static_cast<unsigned>(blocks), kWarps * 32, 0, stream>>>(X, y, n, norm, w, grad,
                                                                                            loss);
    else
        mlp_backward_kernel<false><<<static_cast<unsigned>(blocks), kWarps * 32, 0, stream>>>(X, y, n, norm, w, grad,
                                                                                             loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float *master, uint16_t *w, const float *grad, float *m, float *v, float lr,
                            float beta1, float beta2, float eps, int step, cudaStream_t stream) {
    double p1 = 1.0, p2 = 1.0;
    for (int i = 0; i < step; ++i) {
        p1 *= beta1;
        p2 *= beta2;
    }
    mlp_adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, stream>>>(
        master, w, grad, m, v, kMlpParams, lr, beta1, beta2, eps, static_cast<float>(1.0 - p1),
        static_cast<float>(1.0 - p2));
    return cudaGetLastError();
}

}  // namespace qg
