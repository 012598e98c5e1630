// query_prep.cu -- batched INT8 query preparation (RaBitQSpace::prepare_query with the Int8
// codec: initializePreparedQuery + buildCentroidQuery, space_rabitq.h:3429-3706).
//
// One 128-thread CTA per query; the warps work side by side: warp 0 rotates the query
// (random-sign Hadamard transform in shared memory, the reference's butterfly order) and
// reduces max|q'|; warp 1 forms ||q - c||^2 exactly from 128-bit fixed-point sums (the
// reference's double FMA chains run only when a rigorous bound cannot decide the float);
// warp 2 lane 0 hashes the raw query bytes (FNV-1a, the one long sequential chain) and seeds
// MT19937-64; warp 3 lane 0 forms the pairwise half sum. The dither stream is then produced by
// the whole CTA (parallel MT19937-64 twist) and the INT8 codes are decided in FP32 with an
// exact margin test, double arithmetic only for draws within 2^-36 of an integer.
#include <cstdint>

#include "exact_fp.cuh"
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
    for (int ls = 0; (1 << ls) < D; ++ls) {
        const int step = 1 << ls;
        for (int b = lane; b < D / 2; b += 32) {
            const int i = b & (step - 1);
            const int ia = ((b >> ls) << (ls + 1)) + i, ib = ia + step;
            const float a = x[ia], c = x[ib];
            x[ia] = a + c;
            x[ib] = a - c;
        }
        __syncwarp();
    }
}

namespace {

// ---- ||q - c||^2 without FP64 ---------------------------------------------------------
// The reference forms ||q||^2 and <q, c> as sequential FMA chains in double (each q_i * q_i
// and q_i * c_i is exact in double, so every step is one rounding of acc + p_i), then
// qn2 = max(0, float((rqn + ||c||^2) - 2 dot)) in double. FP64 is a narrow pipe on this
// part, so the chains are not run: the exact real sums A = sum q_i^2 and B = sum q_i c_i are
// formed warp-parallel in 128-bit fixed point, and the rounding error of the reference's
// sequential evaluation is bounded (Higham, Accuracy and Stability of Numerical Algorithms,
// 2nd ed., sec. 4.2: |fl(sum) - sum| <= u * sum_i |partial_i|, u = 2^-53):
//   |t2 - X| <= 2^-53 (n + 2) (A + ||c||^2 + 2 sum|q_i c_i|),  X = A + ||c||^2 - 2B.
// If every value within that bound of X rounds to the same float, that float is the
// reference's qn2; otherwise (about once in 10^5 queries) the caller runs the double chains.

// One warp. Returns true and the reference's qn2 in *out when the bound decides it.
__device__ bool exact_qn2_warp(const float *q, const float *c, int dim, float cn, int lane, float *out) {
    constexpr int kNone = -100000;
    int emax = kNone;
    bool finite = true;
    for (int i = lane; i < dim; i += 32) {
        const FloatParts a = split_float(q[i]), b = split_float(c[i]);
        finite = finite && a.finite && b.finite;
        if (a.m != 0) {
            emax = max(emax, 2 * a.e + 48);
            if (b.m != 0) emax = max(emax, a.e + b.e + 49);
        }
    }
    const FloatParts pc = split_float(cn);
    finite = finite && pc.finite;
    if (pc.m != 0) emax = max(emax, pc.e + 24);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    if (!__all_sync(0xffffffffu, finite) || emax == kNone) return false;
    const int G = emax - 100;  // grid: every term and sum below 2^112 in grid units
    __int128 A = 0, B = 0, Babs = 0;
    for (int i = lane; i < dim; i += 32) {
        const FloatParts a = split_float(q[i]), b = split_float(c[i]);
        const unsigned long long aa = static_cast<unsigned long long>(a.m * a.m);
        A += static_cast<__int128>(to_grid(aa, 2 * a.e - G));
        const long long pb = a.m * b.m;
        const __int128 t = static_cast<__int128>(to_grid(static_cast<unsigned long long>(pb < 0 ? -pb : pb),
                                                         a.e + b.e - G));
        B += pb < 0 ? -t : t;
        Babs += t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        A += shfl_xor_i128(A, o);
        B += shfl_xor_i128(B, o);
        Babs += shfl_xor_i128(Babs, o);
    }
    const __int128 C = static_cast<__int128>(to_grid(static_cast<unsigned long long>(pc.m < 0 ? -pc.m : pc.m),
                                                     pc.e - G)) * (pc.m < 0 ? -1 : 1);
    const __int128 X = A + C - 2 * B;
    const __int128 S = A + (C < 0 ? -C : C) + 2 * Babs;
    // bound in grid units: 2x the rounding bound, plus one unit per truncated term
    const __int128 base = (S >> 52) + 1;
    const __int128 n5 = static_cast<__int128>(dim + 5);
    const __int128 E = base * n5 + ((base * n5) >> 6) + 3 * static_cast<__int128>(dim) + 4;
    const __int128 lo = X - E, hi = X + E;
    if (lo <= 0) return false;
    const int mb = msb_u128(static_cast<unsigned __int128>(lo));
    if (mb != msb_u128(static_cast<unsigned __int128>(hi))) return false;
    const int sh = mb - 23;  // float significand = bits [sh, mb]
    if (sh < 1) return false;
    const __int128 half = static_cast<__int128>(1) << (sh - 1);
    const __int128 j = (X + half) >> sh;
    if (!(lo > (2 * j - 1) * half && hi < (2 * j + 1) * half)) return false;
    const int fe = sh + G;  // the float is j * 2^fe, j in [2^23, 2^24]
    if (fe + 23 < -126 || fe + 24 > 127) return false;
    const uint32_t jj = static_cast<uint32_t>(static_cast<long long>(j));
    *out = jj == (1u << 24) ? __uint_as_float(static_cast<uint32_t>(fe + 24 + 127) << 23)
                            : __uint_as_float((static_cast<uint32_t>(fe + 23 + 127) << 23) | (jj - (1u << 23)));
    return true;
}

// ---- INT8 dither without FP64 ---------------------------------------------------------
// Reference: v = floor(double(x) / double(scale) + u), u = RN53(K) * 2^-64 clamped below 1
// (K = the tempered MT19937-64 draw). Here s1 + tail approximates x/scale + K 2^-64 to
// within 2^-38.5 (remainder of the float quotient by FMA, a TwoSum of the quotient and the
// top 24 bits of K, the next 24 bits of K), and the reference's T to within 2^-44.9 of the
// same real number; the floor is decided unless T lies within 2^-36 of an integer, in which
// case `undecided` is set and the caller evaluates the double expression.
__device__ __forceinline__ int dither_floor(float x, float scale, unsigned long long K, bool &undecided) {
    const float y = __fdiv_rn(x, scale);
    const float r = __fmaf_rn(-y, scale, x);  // exact: x - y * scale
    const float c = __fdiv_rn(r, scale);
    const float uh = __uint2float_rn(static_cast<unsigned>(K >> 40)) * 0x1p-24f;
    const float ul = __uint2float_rn(static_cast<unsigned>((K >> 16) & 0xFFFFFFu)) * 0x1p-48f;
    const float s1 = __fadd_rn(y, uh);  // TwoSum(y, uh) = s1 + e1 exactly
    const float bv = __fsub_rn(s1, y);
    const float e1 = __fadd_rn(__fsub_rn(y, __fsub_rn(s1, bv)), __fsub_rn(uh, bv));
    const float tail = __fadd_rn(__fadd_rn(e1, c), ul);
    const float n = floorf(s1);
    const float d0 = __fsub_rn(s1, n);
    constexpr float kEps = 0x1p-36f;
    int v = static_cast<int>(n);
    if (d0 < 0.5f) {  // only the lower boundary n is reachable; s1 - n is exact here
        const float g = __fadd_rn(d0, tail);
        if (g < -kEps) v -= 1;
        else if (!(g > kEps)) undecided = true;
    } else {  // only n + 1 is reachable; s1 - (n + 1) is exact here
        const float g = __fadd_rn(__fsub_rn(s1, n + 1.0f), tail);
        if (g > kEps) v += 1;
        else if (!(g < -kEps)) undecided = true;
    }
    return v;
}

}  // namespace

__global__ void __launch_bounds__(128) prepare_queries_kernel(PrepArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned long long *mt = reinterpret_cast<unsigned long long *>(smem_raw);  // [312]
    float *x = reinterpret_cast<float *>(mt + kMtN);                              // [D]
    float *qs = x + a.code_dim;                                                   // [dim] raw query
    __shared__ float s_half, s_max, s_qn2;
    __shared__ int s_csum_part[4], s_need_chain;

    const int q = blockIdx.x;
    if (q >= a.nq || (a.nq_dev != nullptr && q >= *a.nq_dev)) return;
    const int D = a.code_dim, dim = a.dim;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float *gq = a.queries + static_cast<size_t>(q) * a.query_stride;
    // stage the raw query once: the FNV chain below reads it byte by byte
    for (int i = threadIdx.x; i < dim; i += 128) qs[i] = gq[i];
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
    } else if (warp == 1) {
        // ||q - c||^2 (space_rabitq.h:3688-3693, 3444-3450)
        float v = 0.0f;
        const bool ok = exact_qn2_warp(raw, a.center, dim, a.center_norm_sqr[0], lane, &v);
        if (lane == 0) {
            s_qn2 = v;
            s_need_chain = ok ? 0 : 1;
        }
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
    } else if (warp == 1 && lane == 0 && s_need_chain) {
        // the bound did not decide qn2: the reference's double FMA chains, in order
        double rqn = 0.0, dot = 0.0;
        for (int i = 0; i < dim; ++i) {
            const double v = static_cast<double>(raw[i]);
            rqn = __fma_rn(v, v, rqn);
            dot = __fma_rn(v, static_cast<double>(a.center[i]), dot);
        }
        s_qn2 = fmaxf(0.0f, static_cast<float>(rqn + static_cast<double>(a.center_norm_sqr[0]) - 2.0 * dot));
    }
    __syncthreads();

    const float qn2 = s_qn2;
    const float max_abs = s_max;
    if (a.qbits == 32) {
        // Full (space_rabitq.h:3489-3492): the FP32 residual and the scalars, no query codes
        if (threadIdx.x == 0) {
            a.scal[q] = make_float4(qn2, sqrtf(qn2), s_half * 0.5f, 1.0f);
            a.csum[q] = 0;
        }
        return;
    }
    if (a.qbits == 2) {
        // B1Main (space_rabitq.h:3493-3510): +-1 per dimension (r > 0 -> +1) as integer codes,
        // the sign sum in the code-sum slot
        int8_t *codes = a.codes + static_cast<size_t>(q) * D;
        int pos = 0;
        for (int i = threadIdx.x; i < D; i += 128) {
            const bool p = x[i] > 0.0f;
            codes[i] = p ? 1 : -1;
            pos += p ? 1 : 0;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) pos += __shfl_xor_sync(0xffffffffu, pos, o);
        if (lane == 0) s_csum_part[warp] = pos;
        __syncthreads();
        if (threadIdx.x == 0) {
            const int p = s_csum_part[0] + s_csum_part[1] + s_csum_part[2] + s_csum_part[3];
            a.scal[q] = make_float4(qn2, sqrtf(qn2), s_half * 0.5f, 1.0f);
            a.csum[q] = static_cast<long long>(2 * p - D);
        }
        return;
    }
    if (a.qbits == 1) {
        // B1 (space_rabitq.h:3493-3523): sign bits of q' into the code buffer (bit i of byte
        // i / 8), |q'| summed in dimension order on one thread, the 1-bit estimator's scales:
        // short scale in the scale slot, error scale and alpha packed in the code-sum slot.
        int8_t *bits = a.codes + static_cast<size_t>(q) * D;
        for (int b = threadIdx.x; b < D / 8; b += 128) {
            uint32_t byte = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) byte |= (x[8 * b + k] > 0.0f ? 1u : 0u) << k;
            bits[b] = static_cast<int8_t>(byte);
        }
        if (threadIdx.x == 0) {
            float abs_sum = 0.0f;
            for (int i = 0; i < D; ++i) abs_sum += fabsf(x[i]);
            const float qn = sqrtf(qn2);
            float ss = 0.0f, es = 0.0f, al = 0.0f;
            if (qn > 0.0f && abs_sum > 0.0f && D > 1) {
                const float a_q = abs_sum / qn;
                const float alpha_q = fminf(1.0f, a_q / sqrtf(static_cast<float>(D)));
                const float alpha2 = alpha_q * alpha_q;
                al = alpha_q;
                ss = 4.0f * qn / a_q;
                es = 2.0f * qn * sqrtf(fmaxf(0.0f, (1.0f - alpha2) / alpha2)) / sqrtf(static_cast<float>(D - 1));
            }
            a.scal[q] = make_float4(qn2, qn, s_half * 0.5f, ss);
            a.csum[q] = static_cast<long long>((static_cast<unsigned long long>(__float_as_uint(al)) << 32) |
                                               __float_as_uint(es));
        }
        return;
    }
    const bool int4 = a.qbits == 4;  // Int4: max/8, [-8, 7], the second draw (space_rabitq.h:3538-3655)
    const float scale = max_abs > 0.0f ? max_abs / (int4 ? 8.0f : 128.0f) : 1.0f;
    const int vlo = int4 ? -8 : -128, vhi = int4 ? 7 : 127;
    // below this the quotient's FMA remainder may underflow: take the double expression
    const bool fast = scale >= 0x1p-100f;
    int csum = 0;
    int8_t *codes = a.codes + static_cast<size_t>(q) * D;
    if (max_abs > 0.0f) {
        // Two draws per dimension, the first used by INT8, the second by INT4
        // (space_rabitq.h:3625-3655).
        const int draws = 2 * D;
        const int parity = int4 ? 1 : 0;
        for (int base = 0; base < draws; base += kMtN) {
            mt_twist(mt);
            for (int p = threadIdx.x; p < kMtN; p += 128) {
                const int j = base + p;
                if (j < draws && (j & 1) == parity) {
                    const int i = j >> 1;
                    const unsigned long long K = mt_temper(mt[p]);
                    bool undecided = !fast;
                    int v = fast ? dither_floor(x[i], scale, K, undecided) : 0;
                    if (undecided) {
                        const double u = canonical_u01(K);
                        v = static_cast<int>(floor(static_cast<double>(x[i]) / static_cast<double>(scale) + u));
                    }
                    v = max(vlo, min(vhi, v));
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
                        (static_cast<size_t>(a.code_dim) + static_cast<size_t>(a.dim)) * sizeof(float);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(prepare_queries_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    prepare_queries_kernel<<<a.nq, 128, smem, stream>>>(a);
    return cudaGetLastError();
}

// Kernel-level check of the dither decision: out[i] = floor(double(x) / double(scale) + u(K))
// (before the INT8 clamp), undecided[i] = 1 where the double expression had to be evaluated.
__global__ void dither_pairs_kernel(const float *x, const float *scale, const unsigned long long *draws, size_t n,
                                    int *out, uint8_t *undecided) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float s = scale[i];
    bool und = !(s >= 0x1p-100f);
    int v = und ? 0 : dither_floor(x[i], s, draws[i], und);
    if (und) v = static_cast<int>(floor(static_cast<double>(x[i]) / static_cast<double>(s) + canonical_u01(draws[i])));
    out[i] = v;
    if (undecided) undecided[i] = und ? 1 : 0;
}

// Kernel-level check of the residual-code rounding of the encoder: out[i] =
// clamp(round(double(x) / double(s)), -7, 7), undecided[i] = 1 where the FP32 decision fell back.
__global__ void round_quotient_kernel(const float *x, const float *s, size_t n, int *out, uint8_t *undecided) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool und = !(s[i] >= 0x1p-100f) || !isfinite(x[i]);
    int q = und ? 0 : round_away_quotient(x[i], s[i], __frcp_rn(s[i]), und);
    if (und) q = max(-7, min(7, static_cast<int>(round(static_cast<double>(x[i]) / static_cast<double>(s[i])))));
    out[i] = q;
    if (undecided) undecided[i] = und ? 1 : 0;
}

cudaError_t launch_round_quotient_pairs(const float *x, const float *s, size_t n, int *out, uint8_t *undecided,
                                        cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    round_quotient_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(x, s, n, out, undecided);
    return cudaGetLastError();
}

cudaError_t launch_dither_pairs(const float *x, const float *scale, const unsigned long long *draws, size_t n,
                                int *out, uint8_t *undecided, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    dither_pairs_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(x, scale, draws, n, out,
                                                                                     undecided);
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
