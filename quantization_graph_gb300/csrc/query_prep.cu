// query_prep.cu -- batched INT8 query preparation (RaBitQSpace::prepare_query with the Int8
// codec: initializePreparedQuery + buildCentroidQuery, space_rabitq.h:3429-3706).
//
// One 128-thread CTA per query. The three long sequential chains of the reference run in
// separate warps so they overlap: warp 0 rotates the query (random-sign Hadamard transform
// in shared memory, the reference's butterfly order) and reduces max|q'|; warp 1 lane 0
// accumulates ||q||^2 and <q, c> as FMA chains in double; warp 2 lane 0 hashes the raw
// query bytes (FNV-1a) and seeds MT19937-64; warp 3 lane 0 forms the pairwise half sum.
// The dither stream is then produced by the whole CTA (parallel MT19937-64 twist).
#include <cstdint>

#include "qg_device.cuh"
#include "qg_kernels.h"

namespace qg {
namespace {

constexpr int kMtN = 312;
constexpr int kMtM = 156;
constexpr unsigned long long kMatrixA = 0xB5026F5AA96619E9ULL;
constexpr unsigned long long kUpper = 0xFFFFFFFF80000000ULL;
constexpr unsigned long long kLower = 0x7FFFFFFFULL;

// MT19937-64 tempering (Matsumoto & Nishimura, 2004; std::mt19937_64 parameters).
__device__ __forceinline__ unsigned long long mt_temper(unsigned long long x) {
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= (x >> 43);
    return x;
}

// generate_canonical<double, 53> over a 64-bit engine: one draw, x / 2^64 rounded once,
// clamped below 1 (libstdc++ random.tcc).
__device__ __forceinline__ double canonical_u01(unsigned long long x) {
    double u = __ull2double_rn(x) * 0x1p-64;
    if (u >= 1.0) u = 0x1.fffffffffffffp-1;
    return u;
}

// One MT19937-64 regeneration of the 312-word state, CTA-parallel: elements [0, 156) read
// only old words; elements [156, 312) read old words and the new words [0, 156).
__device__ void mt_twist(unsigned long long *mt) {
    const int t = threadIdx.x;
    unsigned long long nv[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int i = t + r * 128;
        if (i < kMtN - kMtM) {
            const unsigned long long x = (mt[i] & kUpper) | (mt[i + 1] & kLower);
            nv[r] = mt[i + kMtM] ^ (x >> 1) ^ ((x & 1ULL) ? kMatrixA : 0ULL);
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int i = t + r * 128;
        if (i < kMtN - kMtM) mt[i] = nv[r];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int i = kMtN - kMtM + t + r * 128;
        if (i < kMtN) {
            const unsigned long long nxt = (i == kMtN - 1) ? mt[0] : mt[i + 1];
            const unsigned long long x = (mt[i] & kUpper) | (nxt & kLower);
            nv[r] = mt[i + (kMtM - kMtN)] ^ (x >> 1) ^ ((x & 1ULL) ? kMatrixA : 0ULL);
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int i = kMtN - kMtM + t + r * 128;
        if (i < kMtN) mt[i] = nv[r];
    }
    __syncthreads();
}

}  // namespace

// In-place random-sign Hadamard transform of one D-vector in shared memory by one warp,
// butterfly order of RaBitQSpace::hadamard (space_rabitq.h:944-988).
__device__ void fht_warp(float *x, int D, int lane) {
    for (int step = 1; step < D; step <<= 1) {
        for (int b = lane; b < D / 2; b += 32) {
            const int block = b / step, i = b - block * step;
            const int ia = block * 2 * step + i, ib = ia + step;
            const float a = x[ia], c = x[ib];
            x[ia] = a + c;
            x[ib] = a - c;
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(128) prepare_queries_kernel(PrepArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned long long *mt = reinterpret_cast<unsigned long long *>(smem_raw);  // [312]
    float *x = reinterpret_cast<float *>(mt + kMtN);                              // [D]
    float *qs = x + a.code_dim;                                                   // [dim] raw query
    float *cs = qs + a.dim;                                                       // [dim] centre
    __shared__ double s_rqn, s_dot;
    __shared__ float s_half, s_max;
    __shared__ int s_csum_part[4];

    const int q = blockIdx.x;
    if (q >= a.nq || (a.nq_dev != nullptr && q >= *a.nq_dev)) return;
    const int D = a.code_dim, dim = a.dim;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float *gq = a.queries + static_cast<size_t>(q) * a.query_stride;
    // stage the raw query and the centre once: the sequential chains below read shared memory
    for (int i = threadIdx.x; i < dim; i += 128) {
        qs[i] = gq[i];
        cs[i] = a.center[i];
    }
    __syncthreads();
    const float *raw = qs;

    if (warp == 0) {
        for (int i = lane; i < D; i += 32) x[i] = i < dim ? raw[i] * a.signs[i] : 0.0f;
        __syncwarp();
        fht_warp(x, D, lane);
        float m = 0.0f;
        for (int i = lane; i < D; i += 32) {
            const float v = x[i] - a.rotated_center[i];
            x[i] = v;
            a.rr[static_cast<size_t>(q) * D + i] = v;
            m = fmaxf(m, fabsf(v));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) s_max = m;
    } else if (warp == 1 && lane == 0) {
        // ||q||^2 and <q, c> (space_rabitq.h:3688-3693, 3444-3450), FMA chains in double.
        double rqn = 0.0, dot = 0.0;
        for (int i = 0; i < dim; ++i) {
            const double v = static_cast<double>(raw[i]);
            rqn = __fma_rn(v, v, rqn);
            dot = __fma_rn(v, static_cast<double>(cs[i]), dot);
        }
        s_rqn = rqn;
        s_dot = dot;
    } else if (warp == 2 && lane == 0) {
        // FNV-1a over the raw query bytes, centroid-id mix (space_rabitq.h:3568-3580), then
        // the MT19937-64 seeding recurrence.
        unsigned long long h = 1469598103934665603ULL;
        const uint32_t *words = reinterpret_cast<const uint32_t *>(raw);
        for (int i = 0; i < dim; ++i) {
            const uint32_t w = words[i];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                h ^= (w >> (8 * b)) & 0xFFu;
                h *= 1099511628211ULL;
            }
        }
        h ^= 0ULL + 0x9E3779B97F4A7C15ULL + (h << 6) + (h >> 2);
        mt[0] = h;
        for (int i = 1; i < kMtN; ++i)
            mt[i] = 6364136223846793005ULL * (mt[i - 1] ^ (mt[i - 1] >> 62)) + static_cast<unsigned long long>(i);
    }
    __syncthreads();
    if (warp == 3 && lane == 0) {
        // half_sum_residual: pairwise float accumulation in pair order (space_rabitq.h:3470-3488)
        float half = 0.0f;
        for (int p = 0; p < D / 2; ++p) half += x[2 * p] + x[2 * p + 1];
        s_half = half;
    }
    __syncthreads();

    const float qn2 = fmaxf(0.0f, static_cast<float>(s_rqn + static_cast<double>(a.center_norm_sqr[0]) -
                                                      2.0 * s_dot));
    const float max_abs = s_max;
    const float scale = max_abs > 0.0f ? max_abs / 128.0f : 1.0f;
    int csum = 0;
    int8_t *codes = a.codes + static_cast<size_t>(q) * D;
    if (max_abs > 0.0f) {
        // Two draws per dimension, the first used by INT8 (space_rabitq.h:3625-3643).
        const int draws = 2 * D;
        for (int base = 0; base < draws; base += kMtN) {
            mt_twist(mt);
            for (int p = threadIdx.x; p < kMtN; p += 128) {
                const int j = base + p;
                if (j < draws && (j & 1) == 0) {
                    const int i = j >> 1;
                    const double u = canonical_u01(mt_temper(mt[p]));
                    int v = static_cast<int>(floor(static_cast<double>(x[i]) / static_cast<double>(scale) + u));
                    v = max(-128, min(127, v));
                    codes[i] = static_cast<int8_t>(v);
                    csum += v;
                }
            }
        }
    } else {
        for (int i = threadIdx.x; i < D; i += 128) codes[i] = 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) csum += __shfl_xor_sync(0xffffffffu, csum, o);
    if (lane == 0) s_csum_part[warp] = csum;
    __syncthreads();
    if (threadIdx.x == 0) {
        const long long total = static_cast<long long>(s_csum_part[0]) + s_csum_part[1] +
                                s_csum_part[2] + s_csum_part[3];
        a.scal[q] = make_float4(qn2, sqrtf(qn2), s_half * 0.5f, scale);
        a.csum[q] = total;
    }
}

// Centre setup (setCentroids, space_rabitq.h:2918-2936): rotated centre and ||c||^2 (double
// FMA chain, stored as float). One CTA.
__global__ void __launch_bounds__(128) center_setup_kernel(const float *center, const float *signs,
                                                           int dim, int D, float *rotated,
                                                           float *norm_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *x = reinterpret_cast<float *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        for (int i = lane; i < D; i += 32) x[i] = i < dim ? center[i] * signs[i] : 0.0f;
        __syncwarp();
        fht_warp(x, D, lane);
        for (int i = lane; i < D; i += 32) rotated[i] = x[i];
    } else if (warp == 1 && lane == 0) {
        double norm = 0.0;
        for (int i = 0; i < dim; ++i) norm = __fma_rn(static_cast<double>(center[i]), static_cast<double>(center[i]), norm);
        norm_out[0] = static_cast<float>(norm);
    }
}

cudaError_t launch_prepare(const PrepArgs &a, cudaStream_t stream) {
    if (a.nq == 0) return cudaSuccess;
    const size_t smem = kMtN * sizeof(unsigned long long) +
                        (static_cast<size_t>(a.code_dim) + 2 * static_cast<size_t>(a.dim)) * sizeof(float);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(prepare_queries_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    prepare_queries_kernel<<<a.nq, 128, smem, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_center_setup(const float *center, const float *signs, int dim, int D,
                                float *rotated, float *norm_out, cudaStream_t stream) {
    center_setup_kernel<<<1, 128, static_cast<size_t>(D) * sizeof(float), stream>>>(
        center, signs, dim, D, rotated, norm_out);
    return cudaGetLastError();
}

}  // namespace qg

namespace qg {

// train_global_center_matrix (diskann_runner.rs:1677-1701): f32 sum of the sampled rows in
// ascending id order, then one multiply by the f32 reciprocal of the sample count. One
// thread per column, rows visited sequentially (coalesced across columns).
__global__ void center_mean_kernel(const float *data, size_t stride, int dim, const uint32_t *rows,
                                   size_t count, float *out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= dim) return;
    float acc = 0.0f;
    for (size_t r = 0; r < count; ++r) {
        const size_t row = rows ? rows[r] : r;
        acc = acc + data[row * stride + j];
    }
    const float inv = 1.0f / static_cast<float>(count);
    out[j] = acc * inv;
}

cudaError_t launch_center_mean(const float *data, size_t stride, int dim, const uint32_t *rows,
                               size_t count, float *out, cudaStream_t stream) {
    if (count == 0 || dim == 0) return cudaErrorInvalidValue;
    center_mean_kernel<<<(dim + 127) / 128, 128, 0, stream>>>(data, stride, dim, rows, count, out);
    return cudaGetLastError();
}

}  // namespace qg
