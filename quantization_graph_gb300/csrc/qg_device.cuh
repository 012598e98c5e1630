// qg_device.cuh -- device-side arithmetic of the ExRaBitQ4 / paper-prune query path.
//
// Every function restates one reference routine of Ours/core/hnswlib/space_rabitq.h as
// built by experiments/02_diskann_fair/build.rs (x86-64, -O3 -march=native): the floating
// point operation order, the lane order of its SIMD reductions and the FMA contractions
// GCC makes there are reproduced, so results are bit-identical to the reference. All
// translation units are compiled with --fmad=false; the contracted sites are explicit
// __fmaf_rn / __fma_rn calls.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "qg_types.h"

namespace qg {

constexpr float kFltMax = 3.402823466e+38f;

__device__ __forceinline__ float f_inf() { return __int_as_float(0x7f800000); }
__device__ __forceinline__ bool f_isfinite(float x) { return isfinite(x); }

// A little-endian f32 at any byte address (the reference's records are unaligned).
__device__ __forceinline__ float ld_f32(const uint8_t *p) {
    const uint32_t v = static_cast<uint32_t>(p[0]) | (static_cast<uint32_t>(p[1]) << 8) |
                       (static_cast<uint32_t>(p[2]) << 16) | (static_cast<uint32_t>(p[3]) << 24);
    return __uint_as_float(v);
}

// PaperPruneFactors (20 bytes) -> device float4 with validity folded into cross_scale and
// error_cross_scale: both NaN when the valid flag is 0. A set flag implies a finite error cross
// scale (extract_paper_prune_sidecar, space_rabitq.h:4364-4392), so a NaN there marks exactly the
// records whose flag is 0.
__device__ __forceinline__ float4 load_factors(const uint8_t *f) {
    float4 pf = make_float4(ld_f32(f), ld_f32(f + 4), ld_f32(f + 8), ld_f32(f + 12));
    if (f[16] == 0) {
        pf.z = __int_as_float(0x7fc00000);
        pf.w = __int_as_float(0x7fc00000);
    }
    return pf;
}

// _mm512_reduce_add_ps tree over the 16 lanes of a half-warp (lane t = AVX-512 lane t):
// (v[8+j] + v[j]) -> (a[4+j] + a[j]) -> (b0 + b2, b1 + b3) -> c0 + c1. Every lane of the
// half-warp must call it; lane 0 of the half-warp holds the result.
__device__ __forceinline__ float reduce16_tree(float v) {
    v = v + __shfl_down_sync(0xffffffffu, v, 8, 16);
    v = v + __shfl_down_sync(0xffffffffu, v, 4, 16);
    v = v + __shfl_down_sync(0xffffffffu, v, 2, 16);
    v = v + __shfl_down_sync(0xffffffffu, v, 1, 16);
    return v;
}

// queryDistanceLongWithIps (space_rabitq.h:1621-1632) with the reference build's two
// contractions: fma(-7, half, 8*short + rem) and fma(-long_scale, signed, norm + qn2).
__device__ __forceinline__ float finish_long(float norm_sqr, float long_scale, float short_ip,
                                             float remaining, float half_sum, float qn2) {
    const float partial = 8.0f * short_ip + remaining;
    const float signed_long_ip = __fmaf_rn(-7.0f, half_sum, partial);
    return __fmaf_rn(-long_scale, signed_long_ip, norm_sqr + qn2);
}

// Full FP32 4-bit restore, mode 0 (query_distance_batch_by_id, space_rabitq.h:4080-4202 /
// longCodeIpsAvx512 :1551-1597). Called by the 16 lanes of a half-warp for one record; `t`
// is the lane index in the half-warp. rr = rotated query residual (D floats).
template <int D>
__device__ __forceinline__ float restore_distance_hw(const uint8_t *__restrict__ code,
                                                     const float *__restrict__ rr, float norm_sqr,
                                                     float long_scale, float half_sum, float qn2,
                                                     int t) {
    constexpr int kPairs = D / 2;
    float sel = 0.0f, rem = 0.0f;
#pragma unroll 8
    for (int base = 0; base < kPairs; base += 16) {
        const int pair = base + t;
        const uint32_t packed = code[pair];
        const uint32_t lo = packed & 0x0Fu, hi = packed >> 4;
        const float2 q = *reinterpret_cast<const float2 *>(rr + 2 * pair);
        rem = __fmaf_rn(static_cast<float>(lo & 7u), q.x, rem);
        rem = __fmaf_rn(static_cast<float>(hi & 7u), q.y, rem);
        if (lo > 7u) sel = sel + q.x;
        if (hi > 7u) sel = sel + q.y;
    }
    sel = reduce16_tree(sel);
    rem = reduce16_tree(rem);
    const float short_ip = sel - half_sum;
    float out = finish_long(norm_sqr, long_scale, short_ip, rem, half_sum, qn2);
    if (!(long_scale > 0.0f) || !f_isfinite(long_scale)) out = norm_sqr + qn2;
    return out;
}

// restore_distance_hw for two records at once (r0, r1): the same operations in the same order for
// each, as two independent chains per lane.
template <int D>
__device__ __forceinline__ void restore_distance_hw2(const uint8_t *__restrict__ c0, const uint8_t *__restrict__ c1,
                                                     const float *__restrict__ rr, float4 h0, float4 h1,
                                                     float half_sum, float qn2, int t, float *d0, float *d1) {
    constexpr int kPairs = D / 2;
    float sel0 = 0.0f, rem0 = 0.0f, sel1 = 0.0f, rem1 = 0.0f;
#pragma unroll 8
    for (int base = 0; base < kPairs; base += 16) {
        const int pair = base + t;
        const uint32_t p0 = c0[pair], p1 = c1[pair];
        const float2 q = *reinterpret_cast<const float2 *>(rr + 2 * pair);
        const uint32_t lo0 = p0 & 0x0Fu, hi0 = p0 >> 4, lo1 = p1 & 0x0Fu, hi1 = p1 >> 4;
        rem0 = __fmaf_rn(static_cast<float>(lo0 & 7u), q.x, rem0);
        rem1 = __fmaf_rn(static_cast<float>(lo1 & 7u), q.x, rem1);
        rem0 = __fmaf_rn(static_cast<float>(hi0 & 7u), q.y, rem0);
        rem1 = __fmaf_rn(static_cast<float>(hi1 & 7u), q.y, rem1);
        if (lo0 > 7u) sel0 = sel0 + q.x;
        if (lo1 > 7u) sel1 = sel1 + q.x;
        if (hi0 > 7u) sel0 = sel0 + q.y;
        if (hi1 > 7u) sel1 = sel1 + q.y;
    }
    sel0 = reduce16_tree(sel0);
    rem0 = reduce16_tree(rem0);
    sel1 = reduce16_tree(sel1);
    rem1 = reduce16_tree(rem1);
    float o0 = finish_long(h0.x, h0.y, sel0 - half_sum, rem0, half_sum, qn2);
    float o1 = finish_long(h1.x, h1.y, sel1 - half_sum, rem1, half_sum, qn2);
    if (!(h0.y > 0.0f) || !f_isfinite(h0.y)) o0 = h0.x + qn2;
    if (!(h1.y > 0.0f) || !f_isfinite(h1.y)) o1 = h1.x + qn2;
    *d0 = o0;
    *d1 = o1;
}

// The Full codec's survivor distance: the restore's 16-lane sums with the gate's FP32 short ip
// reused when `reuse` (query_distance_with_paper_msb, space_rabitq.h:3961-3966, 1609-1619; its
// remaining-bit sum, dotRemainingUint8FloatAvx512 :1052-1073, has the restore's lanes and
// contractions), else the restore itself (mode 0, invalid gates). Half-warp like
// restore_distance_hw; every lane runs the same loop and shuffles whichever result is taken.
template <int D>
__device__ __forceinline__ float full_distance_hw(const uint8_t *__restrict__ code,
                                                  const float *__restrict__ rr, float norm_sqr,
                                                  float long_scale, float half_sum, float qn2, bool reuse,
                                                  float gate_short_ip, int t) {
    constexpr int kPairs = D / 2;
    float sel = 0.0f, rem = 0.0f;
#pragma unroll 8
    for (int base = 0; base < kPairs; base += 16) {
        const int pair = base + t;
        const uint32_t packed = code[pair];
        const uint32_t lo = packed & 0x0Fu, hi = packed >> 4;
        const float2 q = *reinterpret_cast<const float2 *>(rr + 2 * pair);
        rem = __fmaf_rn(static_cast<float>(lo & 7u), q.x, rem);
        rem = __fmaf_rn(static_cast<float>(hi & 7u), q.y, rem);
        if (lo > 7u) sel = sel + q.x;
        if (hi > 7u) sel = sel + q.y;
    }
    sel = reduce16_tree(sel);
    rem = reduce16_tree(rem);
    const float short_ip = reuse ? gate_short_ip : sel - half_sum;
    float out = finish_long(norm_sqr, long_scale, short_ip, rem, half_sum, qn2);
    if (!(long_scale > 0.0f) || !f_isfinite(long_scale)) out = norm_sqr + qn2;
    return out;
}

// The Full codec's gate sum (compute_full_paper_prune_estimate_batch_by_id AVX-512 path,
// space_rabitq.h:4427-4505): lane t of a half-warp adds the rotated residual of dims 16k + t whose
// MSB bit is set, then the _mm512_reduce_add_ps tree; lane 0 of the half-warp holds the sum.
template <int D>
__device__ __forceinline__ float full_gate_selected_hw(const uint8_t *__restrict__ msb,
                                                       const float *__restrict__ rr, int t) {
    float acc = 0.0f;
#pragma unroll 8
    for (int k = 0; k < D; k += 16) {
        const int i = k + t;
        acc = acc + (((static_cast<uint32_t>(msb[i >> 3]) >> (i & 7)) & 1u) ? rr[i] : 0.0f);
    }
    return reduce16_tree(acc);
}

// finishQuantizedTraversalDistance (space_rabitq.h:4342-4358); every product is exact. The
// search calls it for all survivors of a hop in one warp-wide pass, so the double latency is
// paid once per hop rather than once per group of survivors.
__device__ __forceinline__ float finish_traversal(float norm_sqr, float long_scale, float short_ip,
                                                  int64_t remaining_dot, float scale,
                                                  int64_t code_sum, float qn2) {
    if (!(long_scale > 0.0f) || !f_isfinite(long_scale)) return norm_sqr + qn2;
    const double centered = static_cast<double>(scale) *
                            (static_cast<double>(remaining_dot) - 3.5 * static_cast<double>(code_sum));
    const double signed_long = 8.0 * static_cast<double>(short_ip) + centered;
    return norm_sqr + qn2 - static_cast<float>(static_cast<double>(long_scale) * signed_long);
}

struct GateOut {
    float lower_bound;
    float short_ip;
    float ip_hat;
    float error_bound;
    bool valid;
    bool reached;  // the estimate was computed (not refused by the validity checks)
};

// compute_paper_prune_estimate_int_msb_gate + finish_paper_prune_estimate_sidecar
// (space_rabitq.h:4873-4899, 4701-4721). `pf` is the device copy of PaperPruneFactors with
// validity folded into cross_scale and error_cross_scale (both NaN when the factors are invalid).
__device__ __forceinline__ GateOut finish_gate(int32_t selected, const float4 pf, float scale,
                                               int64_t code_sum, float qn, float qn2, float eps) {
    GateOut r{0.0f, 0.0f, 0.0f, 0.0f, false, false};
    const float cross_scale = pf.z;
    if (!(cross_scale > 0.0f) || !f_isfinite(cross_scale) || qn <= 0.0f) return r;
    r.reached = true;
    const float short_ip =
        0.5f * scale * static_cast<float>(static_cast<int64_t>(2) * selected - code_sum);
    const float cross = short_ip * cross_scale;
    const float max_cross = 2.0f * pf.y * qn;
    const float up = fmaxf(-max_cross, fminf(max_cross, cross + eps * pf.w * qn));
    r.lower_bound = pf.x + qn2 - up;
    r.short_ip = short_ip;
    r.ip_hat = max_cross > 0.0f ? cross / max_cross : 0.0f;
    r.error_bound = max_cross > 0.0f ? eps * pf.w * qn / max_cross : 0.0f;
    r.valid = f_isfinite(r.lower_bound);
    return r;
}

// compute_paper_prune_estimate (space_rabitq.h:3926-3959), the gate from the encoded record
// (rabitq_paper_estimate, rabitq_paper_estimate_batch), any codec. Its short ip is the FP32
// restore's selected sum (shortCodeIpFromFullCodeAvx512, :1307-1329: 16 lanes over pairs, the
// reduce tree) minus the half sum; half-warp like restore_distance_hw, lane 0 holds the result.
template <int D>
__device__ __forceinline__ float encoded_short_ip_hw(const uint8_t *__restrict__ code, const float *__restrict__ rr,
                                                     float half_sum, int t) {
    constexpr int kPairs = D / 2;
    float sel = 0.0f;
#pragma unroll 8
    for (int base = 0; base < kPairs; base += 16) {
        const int pair = base + t;
        const uint32_t packed = code[pair];
        const float2 q = *reinterpret_cast<const float2 *>(rr + 2 * pair);
        if ((packed & 0x0Fu) > 7u) sel = sel + q.x;
        if ((packed >> 4) > 7u) sel = sel + q.y;
    }
    return reduce16_tree(sel) - half_sum;
}

// The bound of compute_paper_prune_estimate, formed on the normalised inner product; the
// reference build contracts the last line as fma(-two_norms, ip_upper, norm_sqr + qn2).
// `alpha` receives the estimate's alpha (0 when refused).
__device__ __forceinline__ GateOut finish_gate_encoded(float short_ip, float norm_sqr, float short_scale, float qn,
                                                       float qn2, float eps, int D, float *alpha) {
    GateOut r{0.0f, 0.0f, 0.0f, 0.0f, false, false};
    *alpha = 0.0f;
    if (D <= 1 || eps < 0.0f || !f_isfinite(eps) || norm_sqr <= 0.0f || qn <= 0.0f || short_scale <= 0.0f ||
        !f_isfinite(short_scale))
        return r;
    const float data_norm = sqrtf(norm_sqr);
    const float alpha_raw = 4.0f * data_norm / (short_scale * sqrtf(static_cast<float>(D)));
    if (!(alpha_raw > 0.0f) || !f_isfinite(alpha_raw)) return r;
    const float a = fminf(1.0f, alpha_raw);
    r.reached = true;
    const float cross = short_ip * short_scale;
    const float two_norms = 2.0f * data_norm * qn;
    const float ip_hat = cross / two_norms;
    const float a2 = a * a;
    const float error_bound = sqrtf(fmaxf(0.0f, (1.0f - a2) / a2)) * eps / sqrtf(static_cast<float>(D - 1));
    const float ip_upper = fmaxf(-1.0f, fminf(1.0f, ip_hat + error_bound));
    r.lower_bound = __fmaf_rn(-two_norms, ip_upper, norm_sqr + qn2);
    r.short_ip = short_ip;
    r.ip_hat = ip_hat;
    r.error_bound = error_bound;
    r.valid = f_isfinite(r.lower_bound);
    *alpha = a;
    return r;
}

// finish_paper_prune_estimate_sidecar (space_rabitq.h:4701-4721) for the Full codec's FP32 short
// ip (selected sum - half sum): only the sidecar's valid flag is checked. `pf.w` (the error cross
// scale, finite whenever that flag is set) is NaN exactly when the flag is 0.
__device__ __forceinline__ GateOut finish_gate_full(float short_ip, const float4 pf, float qn, float qn2,
                                                    float eps) {
    GateOut r{0.0f, 0.0f, 0.0f, 0.0f, false, false};
    if (!f_isfinite(pf.w)) return r;
    r.reached = true;
    const float cross = short_ip * pf.z;
    const float max_cross = 2.0f * pf.y * qn;
    const float up = fmaxf(-max_cross, fminf(max_cross, cross + eps * pf.w * qn));
    r.lower_bound = pf.x + qn2 - up;
    r.short_ip = short_ip;
    r.ip_hat = max_cross > 0.0f ? cross / max_cross : 0.0f;
    r.error_bound = max_cross > 0.0f ? eps * pf.w * qn / max_cross : 0.0f;
    r.valid = f_isfinite(r.lower_bound);
    return r;
}

// compute_b1_paper_prune_estimate_batch_by_id + finish_b1_paper_prune_estimate
// (space_rabitq.h:4607-4695, 4727-4753): the sign codes' mismatch count gives the symmetric
// 1-bit cross term; the bound adds the query's error term to the database's (the reference
// contracts the database product into the sum).
__device__ __forceinline__ GateOut finish_gate_b1(int32_t mismatches, const float4 pf, float short_scale,
                                                  float error_scale, float qn, float qn2, float eps, int D) {
    GateOut r{0.0f, 0.0f, 0.0f, 0.0f, false, false};
    const float cross_scale = pf.z;
    if (!(short_scale > 0.0f) || !f_isfinite(short_scale) || !(qn > 0.0f) || !(cross_scale > 0.0f) ||
        !f_isfinite(cross_scale) || !(pf.y > 0.0f))
        return r;
    r.reached = true;
    const float signed_dot = static_cast<float>(D) - 2.0f * static_cast<float>(mismatches);
    const float short_ip = signed_dot * short_scale / 8.0f;
    const float cross = short_ip * cross_scale;
    const float max_cross = 2.0f * pf.y * qn;
    const float err = __fmaf_rn(pf.w, qn, error_scale * pf.y);
    const float up = fmaxf(-max_cross, fminf(max_cross, cross + eps * err));
    r.lower_bound = pf.x + qn2 - up;
    r.short_ip = short_ip;
    r.ip_hat = max_cross > 0.0f ? cross / max_cross : 0.0f;
    r.error_bound = max_cross > 0.0f ? eps * err / max_cross : 0.0f;
    r.valid = f_isfinite(r.lower_bound);
    return r;
}

// query_distance_b1 (space_rabitq.h:3741-3753): dot = sum of the 4-bit codes times the query's
// +-1 signs (exact), then norm_sqr + qn2 - float(long_scale * (dot - 7.5 * sign_sum)) in double;
// a degenerate long_scale gives norm_sqr + qn2.
__device__ __forceinline__ float finish_b1main(float norm_sqr, float long_scale, int32_t dot, long long sign_sum,
                                               float qn2) {
    if (!(long_scale > 0.0f) || !f_isfinite(long_scale)) return norm_sqr + qn2;
    const double signed_long_ip =
        __dsub_rn(static_cast<double>(dot), __dmul_rn(7.5, static_cast<double>(sign_sum)));
    const double est = __dmul_rn(static_cast<double>(long_scale), signed_long_ip);
    return (norm_sqr + qn2) - __double2float_rn(est);
}

// B1 prepared scalars packed in the code-sum slot: error scale (low word), alpha (high word).
__device__ __forceinline__ float b1_error_scale(long long packed) {
    return __uint_as_float(static_cast<uint32_t>(static_cast<unsigned long long>(packed)));
}
__device__ __forceinline__ float b1_alpha(long long packed) {
    return __uint_as_float(static_cast<uint32_t>(static_cast<unsigned long long>(packed) >> 32));
}

// Residual rerank interval (compute_residual_distance_intervals_batch_by_id AVX2 path,
// space_rabitq.h:5432-5548), one thread per record: per 16-dim block, eight lanes of
// fma(hi, qo, lo*qe) summed in lane order, then ips = fma(scale, block_ip, ips).
// fused: the product order of the fused restore + residual kernel
// (compute_full_residual_distance_intervals_batch_by_id, space_rabitq.h:5700-5743),
// fma(lo, qe, hi*qo); the two orders differ by one ulp on rare records.
template <int D>
__device__ __forceinline__ void residual_interval_thread(const uint16_t *__restrict__ scales,
                                                         const uint8_t *__restrict__ codes,
                                                         const float *__restrict__ rr, float long_d,
                                                         float qn, bool fused, float *est,
                                                         float *lo_out, float *hi_out) {
    constexpr int kBlocks = D / 16;
    float ips = 0.0f;
    double err_sqr = 0.0;
    for (int b = 0; b < kBlocks; ++b) {
        const float scale = __half2float(__ushort_as_half(scales[b]));
        if (scale == 0.0f || !f_isfinite(scale)) continue;
        const uint2 packed = *reinterpret_cast<const uint2 *>(codes + 8 * b);
        const float4 *q4 = reinterpret_cast<const float4 *>(rr + 16 * b);
        float block_ip = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t word = j < 4 ? packed.x : packed.y;
            const uint32_t byte = (word >> (8 * (j & 3))) & 0xFFu;
            int lo = static_cast<int>(byte & 0x0Fu), hi = static_cast<int>(byte >> 4);
            lo -= (lo > 7) ? 16 : 0;
            hi -= (hi > 7) ? 16 : 0;
            const float4 q = q4[j >> 1];
            const float qe = (j & 1) ? q.z : q.x;
            const float qo = (j & 1) ? q.w : q.y;
            const float fl = static_cast<float>(lo), fh = static_cast<float>(hi);
            const float prod = fused ? __fmaf_rn(fl, qe, __fmul_rn(fh, qo)) : __fmaf_rn(fh, qo, __fmul_rn(fl, qe));
            block_ip = block_ip + prod;
        }
        ips = __fmaf_rn(scale, block_ip, ips);
        const double pde = 0.5 * fabs(static_cast<double>(scale));
        err_sqr += 16.0 * pde * pde;
    }
    const float distance = long_d - 2.0f * ips;
    const float err = static_cast<float>(2.0 * static_cast<double>(qn) * sqrt(err_sqr));
    *est = distance;
    *lo_out = distance - err;
    *hi_out = distance + err;
}

// The estimate of residual_interval_thread for two records at once (a, b): the same operations
// in the same order for each, as independent chains sharing the query loads.
template <int D>
__device__ __forceinline__ void residual_estimate_thread2(const uint16_t *__restrict__ sa, const uint8_t *__restrict__ ca,
                                                          float long_a, const uint16_t *__restrict__ sb,
                                                          const uint8_t *__restrict__ cb, float long_b,
                                                          const float *__restrict__ rr, bool fused, float *est_a,
                                                          float *est_b) {
    constexpr int kBlocks = D / 16;
    float ipa = 0.0f, ipb = 0.0f;
    for (int b = 0; b < kBlocks; ++b) {
        const float sca = __half2float(__ushort_as_half(sa[b])), scb = __half2float(__ushort_as_half(sb[b]));
        const uint2 pa = *reinterpret_cast<const uint2 *>(ca + 8 * b);
        const uint2 pb = *reinterpret_cast<const uint2 *>(cb + 8 * b);
        const float4 *q4 = reinterpret_cast<const float4 *>(rr + 16 * b);
        float bia = 0.0f, bib = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float4 q = q4[j >> 1];
            const float qe = (j & 1) ? q.z : q.x;
            const float qo = (j & 1) ? q.w : q.y;
            const uint32_t bya = ((j < 4 ? pa.x : pa.y) >> (8 * (j & 3))) & 0xFFu;
            const uint32_t byb = ((j < 4 ? pb.x : pb.y) >> (8 * (j & 3))) & 0xFFu;
            int la = static_cast<int>(bya & 0x0Fu), ha = static_cast<int>(bya >> 4);
            int lb = static_cast<int>(byb & 0x0Fu), hb = static_cast<int>(byb >> 4);
            la -= (la > 7) ? 16 : 0;
            ha -= (ha > 7) ? 16 : 0;
            lb -= (lb > 7) ? 16 : 0;
            hb -= (hb > 7) ? 16 : 0;
            const float fla = static_cast<float>(la), fha = static_cast<float>(ha);
            const float flb = static_cast<float>(lb), fhb = static_cast<float>(hb);
            const float pra = fused ? __fmaf_rn(fla, qe, __fmul_rn(fha, qo)) : __fmaf_rn(fha, qo, __fmul_rn(fla, qe));
            const float prb = fused ? __fmaf_rn(flb, qe, __fmul_rn(fhb, qo)) : __fmaf_rn(fhb, qo, __fmul_rn(flb, qe));
            bia = bia + pra;
            bib = bib + prb;
        }
        if (sca != 0.0f && f_isfinite(sca)) ipa = __fmaf_rn(sca, bia, ipa);
        if (scb != 0.0f && f_isfinite(scb)) ipb = __fmaf_rn(scb, bib, ipb);
    }
    *est_a = long_a - 2.0f * ipa;
    *est_b = long_b - 2.0f * ipb;
}

// Byte masks of four MSB bits: nibble b3..b0 -> bytes (b0, b1, b2, b3), each 0 or 1. The
// four shifted copies of the nibble occupy disjoint bit ranges, so no carries occur.
__device__ __forceinline__ int nibble_mask(uint32_t word, int shift) {
    return static_cast<int>((((word >> shift) & 0xFu) * 0x00204081u) & 0x01010101u);
}

}  // namespace qg
