// encode.cu -- batched GPU ExRaBitQ4 block16 encoding (RaBitQSpace::encodeVectorFullWithCentroid,
// space_rabitq.h:5845-5999, one centroid) writing compact and residual records in the
// reference layouts (copyCompactPayloadFromFull / copyResidualRecordFromFull, :6005-6029).
//
// One warp per vector. Parallel parts (rotation, code search set-up, block scales) use all
// lanes; every floating-point accumulation whose rounding depends on order (the reference
// accumulates sequentially) runs in one lane in the reference order, so codes and factors
// are bit-identical to the reference.
//
// fastQuantizeAbs (:867-942) pops (t, i) events from a min-heap; the pop order equals the
// ascending (t, i) order of all events, since every pushed event of a dimension is larger
// than the one just popped. Here the dimensions are sorted once by (|v| descending, index
// ascending); for each code level c = 1..7 the events t = c / |v_i| then appear in that
// order, and a 7-way merge by (t, i) replays the heap's pop sequence exactly.
#include <cstdint>

#include "qg_device.cuh"
#include "qg_kernels.h"

namespace qg {
namespace {

constexpr double kEps = 1e-5;

// floatToHalfScalar (space_rabitq.h:392-411): mantissa rounded with +0x1000, carry OR-ed
// into the exponent field.
__device__ __forceinline__ uint16_t float_to_half_ref(float value) {
    const uint32_t bits = __float_as_uint(value);
    const uint32_t sign = (bits >> 16) & 0x8000u;
    uint32_t mantissa = bits & 0x007FFFFFu;
    const int exponent = static_cast<int>((bits >> 23) & 0xFFu) - 127 + 15;
    if (exponent <= 0) {
        if (exponent < -10) return static_cast<uint16_t>(sign);
        mantissa = (mantissa | 0x00800000u) >> static_cast<uint32_t>(1 - exponent);
        return static_cast<uint16_t>(sign | ((mantissa + 0x00001000u) >> 13));
    }
    if (exponent >= 31) return static_cast<uint16_t>(sign | 0x7C00u);
    return static_cast<uint16_t>(sign | (static_cast<uint32_t>(exponent) << 10) |
                                 ((mantissa + 0x00001000u) >> 13));
}

// halfToFloatScalar (:413-438) is the exact half -> float conversion.
__device__ __forceinline__ float half_to_float_ref(uint16_t h) {
    return __half2float(__ushort_as_half(h));
}

__device__ __forceinline__ int round_away(double v) {  // std::round: half away from zero
    return static_cast<int>(round(v));
}

// residualMseOptimalScale, 4-bit (space_rabitq.h:748-786)
__device__ float mse_scale16(const float *e) {
    float m = 0.0f;
    for (int i = 0; i < 16; ++i) m = fmaxf(m, fabsf(e[i]));
    if (m <= 0.0f) return 0.0f;
    float scale = m / 7.0f;
    if (scale == 0.0f || !isfinite(scale)) return scale;
    for (int iter = 0; iter < 8; ++iter) {
        double n = 0.0, d = 0.0;
        for (int i = 0; i < 16; ++i) {
            const int q = max(-7, min(7, round_away(static_cast<double>(e[i]) / static_cast<double>(scale))));
            n += static_cast<double>(e[i]) * static_cast<double>(q);
            d += static_cast<double>(q) * static_cast<double>(q);
        }
        if (d <= 0.0) break;
        const float next = static_cast<float>(n / d);
        if (next <= 0.0f || !isfinite(next)) break;
        if (fabsf(next - scale) <= 1e-6f * fmaxf(1.0f, scale)) {
            scale = next;
            break;
        }
        scale = next;
    }
    return scale;
}

__device__ void bitonic_sort_warp(unsigned long long *k, int n, int lane) {
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < n / 2; t += 32) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const unsigned long long a = k[lo], b = k[hi];
                if ((a > b) == asc) {
                    k[lo] = b;
                    k[hi] = a;
                }
            }
            __syncwarp();
        }
    }
}

__device__ void fht_warp_local(float *x, int D, int lane) {
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

__device__ __forceinline__ void put_f32(uint8_t *dst, float v) {
    const uint32_t b = __float_as_uint(v);
    dst[0] = b & 0xFF;
    dst[1] = (b >> 8) & 0xFF;
    dst[2] = (b >> 16) & 0xFF;
    dst[3] = b >> 24;
}

__global__ void __launch_bounds__(32) encode_kernel(EncodeArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int D = a.code_dim, dim = a.dim, lane = threadIdx.x;
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(smem);   // [D]
    float *ru = reinterpret_cast<float *>(keys + D);                            // [D]
    unsigned char *c0 = reinterpret_cast<unsigned char *>(ru + D);              // [D] initial code / final magnitude
    signed char *rcode = reinterpret_cast<signed char *>(c0 + D);               // [D]
    float *qerr = reinterpret_cast<float *>(keys);                              // reuses keys after the scan
    __shared__ float s_rn;
    __shared__ double s_best_t, s_num2;
    __shared__ float s_sc[128];  // stored block scales (D/16 <= 128)

    const int v = blockIdx.x;
    if (v >= a.n) return;
    const float *raw = a.raw + static_cast<size_t>(v) * a.raw_stride;

    // residual and its norm: sequential float sum of r*r (no contraction, space_rabitq.h:5856-5860)
    for (int i = lane; i < D; i += 32) ru[i] = i < dim ? raw[i] - a.center[i] : 0.0f;
    __syncwarp();
    if (lane == 0) {
        float rns = 0.0f;
        for (int i = 0; i < dim; ++i) rns = rns + ru[i] * ru[i];
        s_rn = sqrtf(rns);
    }
    __syncwarp();
    const float rn = s_rn;
    if (rn > 0.0f) {
        const float inv = 1.0f / rn;
        for (int i = lane; i < dim; i += 32) ru[i] = ru[i] * inv;
    }
    __syncwarp();
    for (int i = lane; i < dim; i += 32) ru[i] = ru[i] * a.signs[i];
    __syncwarp();
    fht_warp_local(ru, D, lane);

    // ---- fastQuantizeAbs ----
    float mx = 0.0f;
    for (int i = lane; i < D; i += 32) mx = fmaxf(mx, fabsf(ru[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const double max_o = static_cast<double>(mx);
    float ip_norm = 1.0f;
    if (max_o <= kEps) {
        for (int i = lane; i < D; i += 32) c0[i] = 0;
    } else {
        const double t_start = 2.0 / max_o;
        const double t_end = 17.0 / max_o;
        for (int i = lane; i < D; i += 32) {
            const float ai = fabsf(ru[i]);
            int c = static_cast<int>(__fma_rn(t_start, static_cast<double>(ai), kEps));
            c0[i] = static_cast<unsigned char>(min(c, 7));
            keys[i] = (static_cast<unsigned long long>(0xFFFFFFFFu - __float_as_uint(ai)) << 32) |
                      static_cast<unsigned int>(i);
        }
        __syncwarp();
        bitonic_sort_warp(keys, D, lane);
        if (lane == 0) {
            double sqr_den = static_cast<double>(D) * 0.25;
            double num = 0.0;
            for (int i = 0; i < D; ++i) {
                const int c = c0[i];
                sqr_den += static_cast<double>(c * c + c);
                num += (c + 0.5) * static_cast<double>(fabsf(ru[i]));
            }
            // 7-way merge over levels c = 1..7 of the (t, i) events
            int ptr[8];
            double head_t[8];
            int head_i[8];
            auto advance = [&](int c) {
                while (ptr[c] < D) {
                    const unsigned int i = static_cast<unsigned int>(keys[ptr[c]] & 0xFFFFFFFFu);
                    const float ai = fabsf(ru[i]);
                    const int ci = c0[i];
                    if (static_cast<double>(ai) > kEps && c > ci) {
                        const double t = static_cast<double>(c) / static_cast<double>(ai);
                        if (c == ci + 1 || t < t_end) {
                            head_t[c] = t;
                            head_i[c] = static_cast<int>(i);
                            return;
                        }
                    }
                    ++ptr[c];
                }
                head_i[c] = -1;
            };
            for (int c = 1; c <= 7; ++c) {
                ptr[c] = 0;
                advance(c);
            }
            double best_t = 0.0, max_ip = 0.0;
            for (;;) {
                int bc = -1;
                for (int c = 1; c <= 7; ++c) {
                    if (head_i[c] < 0) continue;
                    if (bc < 0 || head_t[c] < head_t[bc] ||
                        (head_t[c] == head_t[bc] && head_i[c] < head_i[bc]))
                        bc = c;
                }
                if (bc < 0) break;
                const double t = head_t[bc];
                const int id = head_i[bc];
                sqr_den += 2.0 * static_cast<double>(bc);
                num += static_cast<double>(fabsf(ru[id]));
                const double ip = num / sqrt(sqr_den);
                if (ip > max_ip) {
                    max_ip = ip;
                    best_t = t;
                }
                ++ptr[bc];
                advance(bc);
            }
            s_best_t = best_t;
        }
        __syncwarp();
        const double best_t = s_best_t;
        for (int i = lane; i < D; i += 32) {
            const int c = static_cast<int>(__fma_rn(best_t, static_cast<double>(fabsf(ru[i])), kEps));
            c0[i] = static_cast<unsigned char>(min(c, 7));
        }
        __syncwarp();
        if (lane == 0) {
            double num = 0.0;
            for (int i = 0; i < D; ++i) num += (c0[i] + 0.5) * static_cast<double>(fabsf(ru[i]));
            s_num2 = num;
        }
        __syncwarp();
        const double num2 = s_num2;
        ip_norm = num2 > kEps ? static_cast<float>(1.0 / num2) : 1.0f;
        if (!isfinite(ip_norm)) ip_norm = 1.0f;
    }
    __syncwarp();
    const float long_scale = 2.0f * rn * ip_norm;
    const float norm_sqr = rn * rn;

    uint8_t *cp = a.compact + static_cast<size_t>(v) * a.compact_bytes;
    uint8_t *rp = a.residual + static_cast<size_t>(v) * a.residual_bytes;
    // 4-bit codes: positive -> 8 + m, else 7 - m; two dims per byte, low nibble first
    for (int j = lane; j < D / 2; j += 32) {
        const int i0 = 2 * j, i1 = 2 * j + 1;
        const int v0 = ru[i0] > 0.0f ? 8 + c0[i0] : 7 - c0[i0];
        const int v1 = ru[i1] > 0.0f ? 8 + c0[i1] : 7 - c0[i1];
        cp[16 + j] = static_cast<uint8_t>(v0 | (v1 << 4));
    }
    if (lane == 0) cp[16 + D / 2] = 0;  // centroid id

    // o_obar (FMA chain) and half L1 norm, sequential in dimension order (:5893-5912)
    if (lane == 0) {
        double o_obar = 0.0, half_l1 = 0.0;
        const double inv_sqrt_d = 1.0 / sqrt(static_cast<double>(D));
        for (int i = 0; i < D; ++i) {
            const double sign = ru[i] > 0.0f ? 1.0 : -1.0;
            o_obar = __fma_rn(static_cast<double>(ru[i]) * sign, inv_sqrt_d, o_obar);
            half_l1 += 0.5 * fabs(static_cast<double>(ru[i]));
        }
        float short_scale = 0.0f, error_scale = 0.0f;
        if (rn > 0.0f && half_l1 > 1e-12) {
            short_scale = static_cast<float>(2.0 * static_cast<double>(rn) / half_l1);
            if (!isfinite(o_obar)) o_obar = 0.8;
            o_obar = fmin(0.999999, fmax(1e-6, o_obar));
            const double o2 = o_obar * o_obar;
            const double fac = 0.359375 / sqrt(static_cast<double>(D));  // ldexp(5.75, -4) / sqrt(D)
            error_scale = static_cast<float>(sqrt(fmax(0.0, (1.0 - o2) / o2)) * fac * 2.0 *
                                             static_cast<double>(rn));
        }
        put_f32(cp, norm_sqr);
        put_f32(cp + 4, long_scale);
        put_f32(cp + 8, short_scale);
        put_f32(cp + 12, error_scale);
    }
    __syncwarp();

    // quantisation error of the 4-bit code (:5927-5935); products are exact
    for (int i = lane; i < D; i += 32) {
        const int code = ru[i] > 0.0f ? 8 + c0[i] : 7 - c0[i];
        const double tv = static_cast<double>(rn) * static_cast<double>(ru[i]);
        const double x4 = 0.5 * static_cast<double>(long_scale) * (static_cast<double>(code) - 7.5);
        qerr[i] = static_cast<float>(tv - x4);
    }
    __syncwarp();
    // per-block MSE scale, fp16 store/reload, residual codes (:5936-5983)
    for (int b = lane; b < D / 16; b += 32) {
        const float sc = mse_scale16(qerr + 16 * b);
        const uint16_t h = float_to_half_ref(sc);
        rp[8 + 2 * b] = static_cast<uint8_t>(h & 0xFF);
        rp[9 + 2 * b] = static_cast<uint8_t>(h >> 8);
        const float stored = half_to_float_ref(h);
        s_sc[b] = stored;
        for (int i = 16 * b; i < 16 * b + 16; ++i) {
            int q = 0;
            if (stored != 0.0f && isfinite(stored))
                q = max(-7, min(7, round_away(static_cast<double>(qerr[i]) / static_cast<double>(stored))));
            rcode[i] = static_cast<signed char>(q);
        }
    }
    __syncwarp();
    for (int j = lane; j < D / 2; j += 32) {
        const uint32_t lo = static_cast<uint32_t>(rcode[2 * j]) & 0xFu;
        const uint32_t hi = static_cast<uint32_t>(rcode[2 * j + 1]) & 0xFu;
        rp[8 + D / 8 + j] = static_cast<uint8_t>(lo | (hi << 4));
    }
    if (lane == 0) {
        double dec_norm = 0.0, x4_ip = 0.0;
        for (int i = 0; i < D; ++i) {
            const float stored = s_sc[i >> 4];
            if (stored == 0.0f || !isfinite(stored)) continue;
            const int code = ru[i] > 0.0f ? 8 + c0[i] : 7 - c0[i];
            const double dec = static_cast<double>(stored) * static_cast<double>(rcode[i]);
            const double x4 = 0.5 * static_cast<double>(long_scale) * (static_cast<double>(code) - 7.5);
            dec_norm += dec * dec;
            x4_ip += x4 * dec;
        }
        put_f32(rp, static_cast<float>(dec_norm));
        put_f32(rp + 4, static_cast<float>(x4_ip));
    }
}

}  // namespace

cudaError_t launch_encode(const EncodeArgs &a, cudaStream_t stream) {
    if (a.n == 0) return cudaSuccess;
    if (a.code_dim > 2048 || a.code_dim < 64) return cudaErrorInvalidValue;
    const size_t smem = static_cast<size_t>(a.code_dim) * (8 + 4 + 1 + 1);
    cudaError_t e = cudaFuncSetAttribute(encode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    encode_kernel<<<a.n, 32, smem, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace qg
