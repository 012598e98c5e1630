// encode.cu -- batched GPU ExRaBitQ4 block16 encoding (RaBitQSpace::encodeVectorFullWithCentroid,
// space_rabitq.h:5845-5999, one centroid) writing compact and residual records in the
// reference layouts (copyCompactPayloadFromFull / copyResidualRecordFromFull, :6005-6029).
//
// One warp per vector, codes and factors bit-identical to the reference. The reference
// accumulates its floating-point sums sequentially; here a sum is formed across the lanes only
// where the result provably equals the sequential one (exact in fixed point: multiples of 2^E
// whose partial sums fit 53 bits; or a float decided within a rigorous bound on the sequential
// rounding), otherwise one lane runs it in the reference order.
//
// fastQuantizeAbs (:867-942) pops (t, i) events from a min-heap; the pop order equals the
// ascending (t, i) order of all events, since every pushed event of a dimension is larger
// than the one just popped. Here the dimensions are sorted once by (|v| descending, index
// ascending); for each code level c = 1..7 the events t = c / |v_i| then appear in that
// order, and a 7-way merge by (t, i) replays the heap's pop sequence exactly.
#include <cstdint>

#include "code_search.cuh"
#include "exact_fp.cuh"
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

// residualMseOptimalScale, 4-bit (space_rabitq.h:748-786), in double as the reference does.
__device__ float mse_scale16_f64(const float *e) {
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

// The same scale with one FP64 operation per iteration. Each q = round(e / scale) is decided in
// FP32 (round_away_quotient, one reciprocal per iteration). n = sum e_i q_i is summed exactly in
// int64 on the grid 2^G of the block's smallest nonzero e (at least as fine as the grid of the
// terms the reference adds), which equals the reference's double sum whenever every partial sum
// fits 53 bits there (the products e_i q_i are exact in double): checked once per block from
// sum 7 |e_i| when that is enough, else per partial sum. n is then that double exactly, and
// next = float(n / d) is the reference's own double division and rounding. Returns false when a
// condition fails; the caller then takes mse_scale16_f64.
__device__ bool mse_scale16_exact(const float *e, float *out) {
    float m = 0.0f;
    for (int i = 0; i < 16; ++i) m = fmaxf(m, fabsf(e[i]));
    if (m <= 0.0f) {
        *out = 0.0f;
        return true;
    }
    float scale = m / 7.0f;
    if (scale == 0.0f || !isfinite(scale)) {
        *out = scale;
        return true;
    }
    constexpr long long kLim = 1LL << 53;
    // the errors as integers on the common grid: e_i = u_i 2^G
    int G = 1 << 30;
#pragma unroll
    for (int i = 0; i < 16; ++i)
        if (e[i] != 0.0f) G = min(G, split_float(e[i]).e);
    if (G < -1000) return false;
    long long u[16];
    long long mag = 0;  // sum |u_i|, bounded by 16 * 2^60 below
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        u[i] = 0;
        if (e[i] == 0.0f) continue;
        const FloatParts p = split_float(e[i]);
        const int sh = p.e - G;
        if (sh > 36) return false;  // |u_i| < 2^60
        u[i] = p.m * (1LL << sh);
        mag += u[i] < 0 ? -u[i] : u[i];
    }
    const bool safe = mag < kLim / 7;  // |q| <= 7: no partial sum can reach 2^53
    for (int iter = 0; iter < 8; ++iter) {
        if (!(scale >= 0x1p-100f)) return false;
        const float inv = __frcp_rn(scale);
        int d = 0;
        long long N = 0;
        bool ok = true;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            bool und = false;
            int q = round_away_quotient(e[i], scale, inv, und);
            if (und) q = max(-7, min(7, round_away(static_cast<double>(e[i]) / static_cast<double>(scale))));
            d += q * q;
            N += u[i] * q;  // |u_i q| < 2^63
            if (!safe) ok = ok && N < kLim && N > -kLim;
        }
        if (!ok) return false;  // a partial sum may have rounded
        if (d <= 0) break;
        if (N == 0) break;  // next = 0: the reference stops
        const double n = __ll2double_rn(N) * pow2d(G);  // exact
        const float next = __double2float_rn(__ddiv_rn(n, static_cast<double>(d)));
        if (next <= 0.0f || !isfinite(next)) break;
        if (fabsf(next - scale) <= 1e-6f * fmaxf(1.0f, scale)) {
            scale = next;
            break;
        }
        scale = next;
    }
    *out = scale;
    return true;
}

// float(double(rn) * double(r) - 0.5 * double(long_scale) * (code - 7.5)) (space_rabitq.h:5927-5935)
// from the two exact products held in integers; falls back to the double expression when the
// operands' exponents are too far apart for the 128-bit grid or the float is not normal.
__device__ __forceinline__ float quant_error(float rn, float r, float long_scale, int code) {
    const FloatParts a = split_float(rn), b = split_float(r), c = split_float(long_scale);
    const long long tv = a.m * b.m;                       // * 2^(a.e + b.e), |tv| < 2^48
    const long long x4 = c.m * static_cast<long long>(2 * code - 15);  // * 2^(c.e - 2), |x4| < 2^29
    const int et = a.e + b.e, ex = c.e - 2;
    const int G = min(et, ex);
    bool ok = a.finite && b.finite && c.finite && et - G <= 70 && ex - G <= 90;
    float out = 0.0f;
    if (ok) {
        const __int128 v = (static_cast<__int128>(tv) << (et - G)) - (static_cast<__int128>(x4) << (ex - G));
        out = float_via_double(v < 0, static_cast<unsigned __int128>(v < 0 ? -v : v), G, ok);
    }
    if (!ok) {
        const double tvd = static_cast<double>(rn) * static_cast<double>(r);
        const double x4d = 0.5 * static_cast<double>(long_scale) * (static_cast<double>(code) - 7.5);
        out = static_cast<float>(tvd - x4d);
    }
    return out;
}

__device__ void fht_warp_local(float *x, int D, int lane) {
    for (int sh = 0; (1 << sh) < D; ++sh) {
        const int step = 1 << sh;
        for (int b = lane; b < D / 2; b += 32) {
            const int ia = ((b >> sh) << (sh + 1)) + (b & (step - 1)), ib = ia + step;
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

// The rotated residual of row v into ru[0, D): the residual, its norm (a sequential float sum of
// r * r, no contraction, space_rabitq.h:5856-5860; written to *rn_out when kNorm), normalised,
// times the random signs, then the Hadamard transform. kRotated: the rotation was done elsewhere
// (the tensor-core GEMM, rotate_gemm.cu); row v of a.rotated holds it and a.norms[v] the norm.
template <bool kRotated, bool kNorm>
__device__ void rotated_row(const EncodeArgs &a, int v, float *ru, int lane, float *s_rn, float rn_known) {
    const int D = a.code_dim, dim = a.dim;
    if constexpr (kRotated) {
        const float *rot = a.rotated + static_cast<size_t>(v) * D;
        for (int i = lane; i < D; i += 32) ru[i] = rot[i];
        if (kNorm && lane == 0) *s_rn = a.norms[v];
        __syncwarp();
    } else {
        const float *raw = a.raw + static_cast<size_t>(v) * a.raw_stride;
        for (int i = lane; i < D; i += 32) ru[i] = i < dim ? raw[i] - a.center[i] : 0.0f;
        __syncwarp();
        if constexpr (kNorm) {
            if (lane == 0) {
                float rns = 0.0f;
                for (int i = 0; i < dim; ++i) rns = rns + ru[i] * ru[i];
                *s_rn = sqrtf(rns);
            }
            __syncwarp();
        }
        const float rn = kNorm ? *s_rn : rn_known;
        if (rn > 0.0f) {
            const float inv = 1.0f / rn;
            for (int i = lane; i < dim; i += 32) ru[i] = ru[i] * inv;
        }
        __syncwarp();
        for (int i = lane; i < dim; i += 32) ru[i] = ru[i] * a.signs[i];
        __syncwarp();
        fht_warp_local(ru, D, lane);
    }
}

// Shared memory, 10 bytes per dimension: an 8D-byte region that holds the rotated row (floats
// [0, D)) until the sort keys are built over it in place, the keys through the code search, then
// the rotated row again (re-derived from the input) and the quantisation errors (floats [D, 2D));
// the codes c0[D]; the residual codes rcode[D] (the code search's block prefix sums before them).
template <bool kRotated>
__global__ void __launch_bounds__(32, 10) encode_kernel(EncodeArgs a) {  // 10 per SM: the shared-memory limit at D = 2048
    extern __shared__ __align__(16) unsigned char smem[];
    const int D = a.code_dim, lane = threadIdx.x;
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(smem);   // [D]
    float *ru = reinterpret_cast<float *>(smem);                                // [D], outside the keys' lifetime
    float *qerr = ru + D;                                                       // [D], after the keys
    unsigned char *c0 = smem + 8 * static_cast<size_t>(D);                      // [D] initial code / final magnitude
    signed char *rcode = reinterpret_cast<signed char *>(c0 + D);               // [D]
    __shared__ float s_rn;
    __shared__ double s_best_t, s_num2, s_num_start;
    __shared__ float s_sc[128];  // stored block scales (D/16 <= 128)

    const int v = blockIdx.x;
    if (v >= a.n) return;
    rotated_row<kRotated, true>(a, v, ru, lane, &s_rn, 0.0f);
    const float rn = s_rn;

    // whether the encoder's double sums over |v| are exact in any order, and their unit 2^E
    int E = 0;
    const bool exact = exact_sum_unit(ru, D, lane, &E);
    long long *lblk = reinterpret_cast<long long *>(rcode);  // scratch until the residual codes

    // ---- fastQuantizeAbs ----
    float mx = 0.0f;
    for (int i = lane; i < D; i += 32) mx = fmaxf(mx, fabsf(ru[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const double max_o = static_cast<double>(mx);
    const bool search = mx > kEpsBelowF;  // else max_o <= kEps: every code is 0
    if (!search) {
        for (int i = lane; i < D; i += 32) c0[i] = 0;
    } else {
        const double t_start = 2.0 / max_o;  // t_end = 17 / max_o is applied as an exact ratio test
        {
            const float th = __double2float_rn(t_start);
            const float tl = __double2float_rn(t_start - static_cast<double>(th));
            for (int i = lane; i < D; i += 32) {
                const float ai = fabsf(ru[i]);
                bool und = false;
                int c = floor_fma_eps(th, tl, ai, und);
                if (und) c = static_cast<int>(__fma_rn(t_start, static_cast<double>(ai), kEps));
                c0[i] = static_cast<unsigned char>(min(c, 7));
            }
        }
        __syncwarp();
        if (!exact && lane == 0) s_num_start = lane0_num_start(ru, c0, D);
        // the keys over the rotated row in place, from the top: chunk [j, j + 32) is read before
        // it is written, and its keys cover floats [2j, 2j + 64), none of them below j
        for (int base = D - 32; base >= 0; base -= 32) {
            const int j = base + lane;
            const float aj = fabsf(ru[j]);
            __syncwarp();
            keys[j] = (static_cast<unsigned long long>(0xFFFFFFFFu - __float_as_uint(aj)) << 32) |
                      static_cast<unsigned int>(j);
        }
        __syncwarp();
        bitonic_sort_warp(keys, D, lane);
        if (exact) {
            double bt = 0.0;
            code_search_warp(keys, c0, D, mx, lblk, E, lane, &bt);
            if (lane == 0) s_best_t = bt;
        } else if (lane == 0) {
            s_best_t = code_search_lane0(keys, c0, D, mx, s_num_start);
        }
        __syncwarp();
        const double best_t = s_best_t;
        {
            const float th = __double2float_rn(best_t);
            const float tl = __double2float_rn(best_t - static_cast<double>(th));
            for (int p = lane; p < D; p += 32) {
                const unsigned long long k = keys[p];
                const float ai = key_a(k);
                bool und = false;
                int c = floor_fma_eps(th, tl, ai, und);
                if (und) c = static_cast<int>(__fma_rn(best_t, static_cast<double>(ai), kEps));
                c0[key_id(k)] = static_cast<unsigned char>(min(c, 7));
            }
        }
        __syncwarp();
        if (exact) {  // the same exact sum, across the lanes in units of 2^E
            long long k = 0;
            for (int p = lane; p < D; p += 32) {
                const unsigned long long kp = keys[p];
                k += static_cast<long long>(2 * c0[key_id(kp)] + 1) * (units(key_a(kp), E) >> 1);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
            if (lane == 0) s_num2 = __ll2double_rn(k) * pow2d(E);
        }
        __syncwarp();
    }
    // the rotated row again, over the keys (the same operations give the same floats)
    rotated_row<kRotated, false>(a, v, ru, lane, &s_rn, rn);
    float ip_norm = 1.0f;
    if (search) {
        if (!exact && lane == 0) {
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

    // o_obar (FMA chain) and half L1 norm, sequential in dimension order (:5893-5912). With exact
    // sums: half_l1 and S = sum|v| across the lanes; o_obar = S / sqrt(D) exactly when sqrt(D) is
    // a power of two, else the chain lies within (D + 2) 2^-53 o of RN(S / sqrt(D)) (each FMA
    // rounds once, every partial sum is at most o) and error_scale, monotone in o, is decided
    // when both ends of that interval give the same float; otherwise lane 0 runs the chain.
    {
        const double inv_sqrt_d = 1.0 / sqrt(static_cast<double>(D));
        const double fac = 0.359375 / sqrt(static_cast<double>(D));  // ldexp(5.75, -4) / sqrt(D)
        auto error_of = [&](double o) {
            if (!isfinite(o)) o = 0.8;
            o = fmin(0.999999, fmax(1e-6, o));
            const double o2 = o * o;
            return static_cast<float>(sqrt(fmax(0.0, (1.0 - o2) / o2)) * fac * 2.0 * static_cast<double>(rn));
        };
        bool done = false;
        double half_l1 = 0.0;
        float error_scale = 0.0f;
        if (exact) {
            long long k = 0;
            for (int i = lane; i < D; i += 32) k += units(fabsf(ru[i]), E);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
            const double S = __ll2double_rn(k) * pow2d(E);
            half_l1 = __ll2double_rn(k >> 1) * pow2d(E);  // k is even: |v| / 2 is a whole number of units
            const double o_par = S * inv_sqrt_d;
            if ((D & 0x55555555) != 0) {  // D = 4^j: 1 / sqrt(D) is a power of two, every step exact
                error_scale = error_of(o_par);
                done = true;
            } else {
                const double d = (static_cast<double>(D) + 4.0) * 0x1p-53 * o_par;
                const float e_lo = error_of(o_par + d), e_hi = error_of(o_par - d);
                if (e_lo == e_hi) {
                    error_scale = e_lo;
                    done = true;
                }
            }
        }
        if (lane == 0) {
            if (!done) {
                double o_obar = 0.0, hl = 0.0;
                for (int i = 0; i < D; ++i) {
                    const double sign = ru[i] > 0.0f ? 1.0 : -1.0;
                    o_obar = __fma_rn(static_cast<double>(ru[i]) * sign, inv_sqrt_d, o_obar);
                    hl += 0.5 * fabs(static_cast<double>(ru[i]));
                }
                half_l1 = hl;
                error_scale = error_of(o_obar);
            }
            float short_scale = 0.0f;
            if (rn > 0.0f && half_l1 > 1e-12) short_scale = static_cast<float>(2.0 * static_cast<double>(rn) / half_l1);
            else error_scale = 0.0f;
            put_f32(cp, norm_sqr);
            put_f32(cp + 4, long_scale);
            put_f32(cp + 8, short_scale);
            put_f32(cp + 12, error_scale);
        }
    }
    __syncwarp();

    // quantisation error of the 4-bit code (:5927-5935); products are exact
    for (int i = lane; i < D; i += 32) {
        const int code = ru[i] > 0.0f ? 8 + c0[i] : 7 - c0[i];
        qerr[i] = quant_error(rn, ru[i], long_scale, code);
    }
    __syncwarp();
    // per-block MSE scale, fp16 store/reload, residual codes (:5936-5983)
    for (int b = lane; b < D / 16; b += 32) {
        float sc;
        if (!mse_scale16_exact(qerr + 16 * b, &sc)) sc = mse_scale16_f64(qerr + 16 * b);
        const uint16_t h = float_to_half_ref(sc);
        rp[8 + 2 * b] = static_cast<uint8_t>(h & 0xFF);
        rp[9 + 2 * b] = static_cast<uint8_t>(h >> 8);
        const float stored = half_to_float_ref(h);
        s_sc[b] = stored;
        const float inv_stored = __frcp_rn(stored);
        for (int i = 16 * b; i < 16 * b + 16; ++i) {
            int q = 0;
            if (stored != 0.0f && isfinite(stored)) {
                bool und = !(stored >= 0x1p-100f) || !isfinite(qerr[i]);
                if (!und) q = round_away_quotient(qerr[i], stored, inv_stored, und);
                if (und) q = max(-7, min(7, round_away(static_cast<double>(qerr[i]) / static_cast<double>(stored))));
            }
            rcode[i] = static_cast<signed char>(q);
        }
    }
    __syncwarp();
    for (int j = lane; j < D / 2; j += 32) {
        const uint32_t lo = static_cast<uint32_t>(rcode[2 * j]) & 0xFu;
        const uint32_t hi = static_cast<uint32_t>(rcode[2 * j + 1]) & 0xFu;
        rp[8 + D / 8 + j] = static_cast<uint8_t>(lo | (hi << 4));
    }
    // the residual record's norm and inner product (:5984-5991): sums of per-dim double products,
    // sequential in dimension order, stored as floats. Across the lanes in another order: each
    // order lies within gamma_{D-1} sum|t| of the exact sum of the same rounded terms t (Higham
    // 2002, section 3.1), so the two orders differ by at most twice that, and the float is
    // decided when both ends of that interval give the same float; otherwise lane 0 runs the loop.
    {
        double s1 = 0.0, s2 = 0.0, a2 = 0.0;
        for (int i = lane; i < D; i += 32) {
            const float stored = s_sc[i >> 4];
            if (stored == 0.0f || !isfinite(stored)) continue;
            const int code = ru[i] > 0.0f ? 8 + c0[i] : 7 - c0[i];
            const double dec = static_cast<double>(stored) * static_cast<double>(rcode[i]);
            const double x4 = 0.5 * static_cast<double>(long_scale) * (static_cast<double>(code) - 7.5);
            const double t1 = dec * dec, t2 = x4 * dec;
            s1 += t1;
            s2 += t2;
            a2 += fabs(t2);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        }
        const double g = 2.0 * (static_cast<double>(D) * 0x1p-53) / (1.0 - static_cast<double>(D) * 0x1p-53) * 1.0001;
        const double d1 = g * s1 + 4.0 * 0x1p-53 * s1, d2 = g * a2 + 4.0 * 0x1p-53 * fabs(s2);
        const bool ok1 = isfinite(s1) && static_cast<float>(s1 - d1) == static_cast<float>(s1 + d1);
        const bool ok2 = isfinite(s2) && static_cast<float>(s2 - d2) == static_cast<float>(s2 + d2);
        if (lane == 0) {
            float f1 = static_cast<float>(s1), f2 = static_cast<float>(s2);
            if (!ok1 || !ok2) {
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
                f1 = static_cast<float>(dec_norm);
                f2 = static_cast<float>(x4_ip);
            }
            put_f32(rp, f1);
            put_f32(rp + 4, f2);
        }
    }
}

}  // namespace

cudaError_t launch_encode(const EncodeArgs &a, cudaStream_t stream) {
    if (a.n == 0) return cudaSuccess;
    if (a.code_dim > 2048 || a.code_dim < 64) return cudaErrorInvalidValue;
    const size_t smem = static_cast<size_t>(a.code_dim) * (8 + 1 + 1);
    if (a.rotated != nullptr) {
        cudaError_t e = cudaFuncSetAttribute(encode_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        encode_kernel<true><<<a.n, 32, smem, stream>>>(a);
        return cudaGetLastError();
    }
    cudaError_t e = cudaFuncSetAttribute(encode_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    encode_kernel<false><<<a.n, 32, smem, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace qg
