// qg_oracle.cpp -- CPU restatement of the Ours-DiskANN query path. TEST INFRASTRUCTURE ONLY:
// used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker;
// never linked into or called by the shipped CUDA library.
//
// Restates the x86-64 `-O3 -march=native` (AVX-512 + FMA) build of the reference
// Ours/core/hnswlib/space_rabitq.h and the Rust hot loop
// experiments/02_diskann_fair/src/ours_diskann.rs:1539-1986. Compile with
// -ffp-contract=off: every product-sum that GCC contracts into an FMA in the reference
// build is written with std::fma here (sites marked "FMA"), every other one is not, and
// the AVX-512 / AVX2 lane orders of the float reductions are spelled out, so the results
// match the reference bit for bit on any host.
//
// Third-party pins: the rotation signs use std::mt19937 + std::uniform_int_distribution and
// the query dither uses std::mt19937_64 + std::uniform_real_distribution<double>, exactly
// the library calls the reference makes (space_rabitq.h:2900-2912, 3582-3591); both sides
// therefore draw from the same libstdc++ implementation.

#include "qg_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <queue>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint32_t kRemainingMax = 7;
constexpr uint32_t kMsbWeight = 8;
constexpr float kUnsignedOffset = 7.5f;
constexpr size_t kBlock = 16;

struct Factors {  // PaperPruneFactors<float> (hnswlib.h:298-305), 20 bytes
    float norm_sqr;
    float data_norm;
    float cross_scale;
    float error_cross_scale;
    uint8_t valid;
};
static_assert(sizeof(Factors) == 20, "PaperPruneFactors layout");

// next_pow2(roundup64(d)) -- space_rabitq.h:217-224
size_t round_up_code_dim(size_t value) {
    const size_t rounded = ((value + 63U) / 64U) * 64U;
    size_t power = 1;
    while (power < rounded) power <<= 1U;
    return power;
}

// floatToHalfScalar / halfToFloatScalar (space_rabitq.h:392-438): the mantissa is rounded
// with +0x1000 and the carry is OR-ed into the exponent field (not round-to-nearest-even).
uint16_t float_to_half_ref(float value) {
    uint32_t bits;
    std::memcpy(&bits, &value, 4);
    const uint32_t sign = (bits >> 16U) & 0x8000U;
    uint32_t mantissa = bits & 0x007FFFFFU;
    const int32_t exponent = static_cast<int32_t>((bits >> 23U) & 0xFFU) - 127 + 15;
    if (exponent <= 0) {
        if (exponent < -10) return static_cast<uint16_t>(sign);
        mantissa = (mantissa | 0x00800000U) >> static_cast<uint32_t>(1 - exponent);
        return static_cast<uint16_t>(sign | ((mantissa + 0x00001000U) >> 13U));
    }
    if (exponent >= 31) return static_cast<uint16_t>(sign | 0x7C00U);
    return static_cast<uint16_t>(sign | (static_cast<uint32_t>(exponent) << 10U) |
                                 ((mantissa + 0x00001000U) >> 13U));
}

float half_to_float_ref(uint16_t value) {
    const uint32_t sign = static_cast<uint32_t>(value & 0x8000U) << 16U;
    uint32_t exponent = (value >> 10U) & 0x1FU;
    uint32_t mantissa = value & 0x03FFU;
    uint32_t bits;
    if (exponent == 0) {
        if (mantissa == 0) {
            bits = sign;
        } else {
            exponent = 1;
            while ((mantissa & 0x0400U) == 0) {
                mantissa <<= 1U;
                --exponent;
            }
            mantissa &= 0x03FFU;
            bits = sign | ((exponent + 127 - 15) << 23U) | (mantissa << 13U);
        }
    } else if (exponent == 31) {
        bits = sign | 0x7F800000U | (mantissa << 13U);
    } else {
        bits = sign | ((exponent + 127 - 15) << 23U) | (mantissa << 13U);
    }
    float out;
    std::memcpy(&out, &bits, 4);
    return out;
}

// _mm512_reduce_add_ps tree of GCC's avx512fintrin.h: (hi8 + lo8) -> (hi4 + lo4) ->
// (x0 + x2, x1 + x3) -> sum.
float reduce16(const float *v) {
    float a[8], b[4];
    for (int j = 0; j < 8; ++j) a[j] = v[8 + j] + v[j];
    for (int j = 0; j < 4; ++j) b[j] = a[4 + j] + a[j];
    const float c0 = b[0] + b[2];
    const float c1 = b[1] + b[3];
    return c0 + c1;
}

}  // namespace

struct qgo_space {
    size_t dim = 0;
    size_t code_dim = 0;
    size_t pair_count = 0;
    size_t code_bytes = 0;      // D/2
    size_t block_count = 0;     // D/16
    size_t scale_bytes = 0;     // D/16 * 2 (fp16 storage)
    size_t full_bytes = 0;
    size_t compact_bytes = 0;
    size_t residual_bytes = 0;
    size_t msb_bytes = 0;
    uint32_t seed = 100;
    int query_bits = 8;  // Int8 (codec 3), Int4 (codec 2), B1 / B1Main (1, sign bits), Full (0, 5, 6: 32)
    int codec = 3;       // the query codec id (rabitq_set_query_coarse_codec)
    std::vector<float> signs;
    std::vector<float> center;
    std::vector<float> rotated_center;
    float center_norm_sqr = 0.0f;

    // full record offsets (space_rabitq.h:261-267, 298-305, 342-350)
    size_t off_short() const { return 8; }
    size_t off_resf() const { return 16; }
    size_t off_scales_full() const { return 24; }
    size_t off_code_full() const { return 24 + scale_bytes; }
    size_t off_cid_full() const { return off_code_full() + code_bytes; }
    size_t off_rescode_full() const { return off_cid_full() + 1; }
    // compact (external residual storage) offsets
    size_t off_code_compact() const { return 16; }
};

struct qgo_prepared {
    const qgo_space *space = nullptr;
    std::vector<float> rotated_residual;  // q' = R q - R c
    std::vector<int8_t> int8_code;
    // gate_tab[16 j + v]: sum of the integer codes of dims 4j..4j+3 whose bit is set in v (built
    // with the codes; the gate's masked sum as one lookup per nibble of the MSB plane)
    std::vector<int16_t> gate_tab;
    float query_norm_sqr = 0.0f;
    float query_norm = 0.0f;
    float half_sum = 0.0f;
    float int8_scale = 1.0f;
    int64_t code_sum = 0;
    // B1 codec (space_rabitq.h:3493-3523): sign bits of q', scales of the 1-bit estimator
    std::vector<uint8_t> b1_code;
    int64_t b1_signed_sum = 0;
    float b1_short_scale = 0.0f;
    float b1_error_scale = 0.0f;
    float b1_alpha = 0.0f;
};

namespace {

// rotate + hadamard (space_rabitq.h:944-1000): pad to D, multiply by signs, butterflies
// with step 1, 2, 4, ...; each output is a single rounded add or subtract.
void rotate_into(const qgo_space &s, const float *raw, float *out) {
    const size_t D = s.code_dim;
    for (size_t i = 0; i < D; ++i) out[i] = 0.0f;
    if (s.seed == 0) {
        std::copy(raw, raw + s.dim, out);
        return;
    }
    for (size_t i = 0; i < s.dim; ++i) out[i] = raw[i] * s.signs[i];
    for (size_t step = 1; step < D; step <<= 1U) {
        for (size_t block = 0; block < D; block += (step << 1U)) {
            for (size_t i = 0; i < step; ++i) {
                const float a = out[block + i];
                const float b = out[block + step + i];
                out[block + i] = a + b;
                out[block + step + i] = a - b;
            }
        }
    }
}

inline uint8_t nib(const uint8_t *code, size_t i) {
    const uint8_t byte = code[i >> 1U];
    return static_cast<uint8_t>((i & 1U) ? (byte >> 4U) : (byte & 0x0FU));
}

// fastQuantizeAbs (space_rabitq.h:867-942).
void fast_quantize_abs(const qgo_space &s, const float *a, uint8_t *code, float &ip_norm) {
    const size_t D = s.code_dim;
    constexpr double eps = 1e-5;
    constexpr int n_enum = 10;
    double max_o = 0.0;
    for (size_t i = 0; i < D; ++i) max_o = std::max(max_o, static_cast<double>(a[i]));
    if (max_o <= eps) {
        std::memset(code, 0, D);
        ip_norm = 1.0f;
        return;
    }
    const double t_start = static_cast<double>(kRemainingMax / 3U) / max_o;
    const double t_end = (static_cast<double>(kRemainingMax) + n_enum) / max_o;
    std::vector<int> cur(D, 0);
    double sqr_den = static_cast<double>(D) * 0.25;
    double num = 0.0;
    for (size_t i = 0; i < D; ++i) {
        cur[i] = static_cast<int>(std::fma(t_start, static_cast<double>(a[i]), eps));  // FMA
        cur[i] = std::min<int>(cur[i], static_cast<int>(kRemainingMax));
        sqr_den += cur[i] * cur[i] + cur[i];
        num += (cur[i] + 0.5) * a[i];  // exact product
    }
    std::priority_queue<std::pair<double, size_t>, std::vector<std::pair<double, size_t>>,
                        std::greater<std::pair<double, size_t>>>
        heap;
    for (size_t i = 0; i < D; ++i)
        if (a[i] > eps) heap.emplace(static_cast<double>(cur[i] + 1) / a[i], i);
    double best_t = 0.0, max_ip = 0.0;
    while (!heap.empty()) {
        const double t = heap.top().first;
        const size_t id = heap.top().second;
        heap.pop();
        const int updated = ++cur[id];
        sqr_den += 2.0 * updated;
        num += a[id];
        const double ip = num / std::sqrt(sqr_den);
        if (ip > max_ip) {
            max_ip = ip;
            best_t = t;
        }
        if (updated < static_cast<int>(kRemainingMax)) {
            const double nt = static_cast<double>(updated + 1) / a[id];
            if (nt < t_end) heap.emplace(nt, id);
        }
    }
    num = 0.0;
    for (size_t i = 0; i < D; ++i) {
        int v = static_cast<int>(std::fma(best_t, static_cast<double>(a[i]), eps));  // FMA
        v = std::min<int>(v, static_cast<int>(kRemainingMax));
        code[i] = static_cast<uint8_t>(v);
        num += (v + 0.5) * a[i];
    }
    ip_norm = num > eps ? static_cast<float>(1.0 / num) : 1.0f;
    if (!std::isfinite(ip_norm)) ip_norm = 1.0f;
}

// residualMseOptimalScale (space_rabitq.h:729-786), 4-bit: qmax 7.
float mse_scale(const float *e, size_t begin, size_t end) {
    float m = 0.0f;
    for (size_t i = begin; i < end; ++i) m = std::max(m, static_cast<float>(std::abs(e[i])));
    if (m <= 0.0f) return 0.0f;
    float scale = m / 7.0f;
    if (scale == 0.0f || !std::isfinite(scale)) return scale;
    for (int iter = 0; iter < 8; ++iter) {
        double n = 0.0, d = 0.0;
        for (size_t i = begin; i < end; ++i) {
            const int32_t q = std::max(
                -7, std::min(7, static_cast<int32_t>(std::round(
                                    static_cast<double>(e[i]) / static_cast<double>(scale)))));
            n += static_cast<double>(e[i]) * static_cast<double>(q);  // exact product
            d += static_cast<double>(q) * static_cast<double>(q);
        }
        if (d <= 0.0) break;
        const float next = static_cast<float>(n / d);
        if (next <= 0.0f || !std::isfinite(next)) break;
        if (std::abs(next - scale) <= 1e-6f * std::max(1.0f, scale)) {
            scale = next;
            break;
        }
        scale = next;
    }
    return scale;
}

void put_f32(uint8_t *dst, float v) { std::memcpy(dst, &v, 4); }
float get_f32(const uint8_t *src) {
    float v;
    std::memcpy(&v, src, 4);
    return v;
}

// ---- restore / traversal / residual arithmetic ----

// queryDistanceLongWithIps (space_rabitq.h:1621-1632) with the FMA contractions of the
// reference build: ((8*short + rem) - 7*half) fused as fma(-7, half, .), and the final
// (norm + qn2) - ls*signed fused as fma(-ls, signed, .).
float finish_long(const qgo_prepared &q, float norm_sqr, float long_scale, float short_ip,
                  float remaining_ip) {
    const float partial = 8.0f * short_ip + remaining_ip;  // 8*x exact
    const float signed_long_ip = std::fma(-7.0f, q.half_sum, partial);  // FMA
    return std::fma(-long_scale, signed_long_ip, norm_sqr + q.query_norm_sqr);  // FMA
}

// query_distance_batch_by_id AVX-512 path / longCodeIpsAvx512 (space_rabitq.h:1551-1597,
// 4080-4202): 16 lanes, lane l takes pairs l, l+16, ...; remaining += lo*qe then += hi*qo
// (both contracted), selected sum by masked adds, then the reduce16 tree.
float restore_distance(const qgo_space &s, const qgo_prepared &q, const uint8_t *record) {
    const float norm_sqr = get_f32(record);
    const float long_scale = get_f32(record + 4);
    if (!(long_scale > 0.0f) || !std::isfinite(long_scale)) return norm_sqr + q.query_norm_sqr;
    const uint8_t *code = record + s.off_code_compact();
    float sel[16] = {}, rem[16] = {};
    const float *r = q.rotated_residual.data();
    for (size_t base = 0; base < s.pair_count; base += 16) {
        for (int l = 0; l < 16; ++l) {
            const size_t pair = base + l;
            const uint8_t packed = code[pair];
            const uint8_t lo = packed & 0x0FU, hi = packed >> 4U;
            const float qe = r[2 * pair], qo = r[2 * pair + 1];
            rem[l] = std::fma(static_cast<float>(lo & 7U), qe, rem[l]);  // FMA
            rem[l] = std::fma(static_cast<float>(hi & 7U), qo, rem[l]);  // FMA
            if (lo > 7U) sel[l] = sel[l] + qe;
            if (hi > 7U) sel[l] = sel[l] + qo;
        }
    }
    const float short_ip = reduce16(sel) - q.half_sum;
    const float remaining = reduce16(rem);
    return finish_long(q, norm_sqr, long_scale, short_ip, remaining);
}

// query_distance_with_paper_msb (space_rabitq.h:3961-3966, 1609-1619): the restore's
// remaining-bit sum (dotRemainingUint8FloatAvx512, :1052-1073: the same 16 lanes and
// contractions) with the gate's FP32 short ip reused.
float full_reuse_distance(const qgo_space &s, const qgo_prepared &q, const uint8_t *record, float short_ip) {
    const float norm_sqr = get_f32(record);
    const float long_scale = get_f32(record + 4);
    if (long_scale <= 0.0f || !std::isfinite(long_scale)) return norm_sqr + q.query_norm_sqr;
    const uint8_t *code = record + s.off_code_compact();
    float rem[16] = {};
    const float *r = q.rotated_residual.data();
    for (size_t base = 0; base < s.pair_count; base += 16) {
        for (int l = 0; l < 16; ++l) {
            const size_t pair = base + l;
            const uint8_t packed = code[pair];
            rem[l] = std::fma(static_cast<float>(packed & 7U), r[2 * pair], rem[l]);           // FMA
            rem[l] = std::fma(static_cast<float>((packed >> 4U) & 7U), r[2 * pair + 1], rem[l]);  // FMA
        }
    }
    return finish_long(q, norm_sqr, long_scale, short_ip, reduce16(rem));
}

// finishQuantizedTraversalDistance (space_rabitq.h:4342-4358); every product is exact.
float finish_traversal(const qgo_prepared &q, float norm_sqr, float long_scale, float short_ip,
                       int64_t remaining_dot) {
    const double centered = static_cast<double>(q.int8_scale) *
                            (static_cast<double>(remaining_dot) -
                             3.5 * static_cast<double>(q.code_sum));
    const double signed_long = 8.0 * static_cast<double>(short_ip) + centered;
    return norm_sqr + q.query_norm_sqr -
           static_cast<float>(static_cast<double>(long_scale) * signed_long);
}

// query_distance_b1 (space_rabitq.h:3741-3753): the 4-bit long code dotted with the query's
// sign code (exact in integers), centred by 7.5 * the sign sum, scaled by long_scale in double.
float distance_b1(const qgo_space &s, const qgo_prepared &q, const uint8_t *record) {
    const float norm_sqr = get_f32(record);
    const float long_scale = get_f32(record + 4);
    if (!(long_scale > 0.0f) || !std::isfinite(long_scale)) return norm_sqr + q.query_norm_sqr;
    const uint8_t *code = record + s.off_code_compact();
    int64_t dot = 0;
    for (size_t i = 0; i < s.code_dim; ++i) {
        const int c = (code[i >> 1U] >> (4U * (i & 1U))) & 0x0F;
        dot += ((q.b1_code[i >> 3U] >> (i & 7U)) & 1U) ? c : -c;
    }
    const double signed_long_ip = static_cast<double>(dot) - 7.5 * static_cast<double>(q.b1_signed_sum);
    const double est_ip = static_cast<double>(long_scale) * signed_long_ip;
    return norm_sqr + q.query_norm_sqr - static_cast<float>(est_ip);
}

// query_distance_with_quantized_paper_msb (space_rabitq.h:4207-4232).
float traversal_distance(const qgo_space &s, const qgo_prepared &q, const uint8_t *record,
                         float short_ip) {
    const float norm_sqr = get_f32(record);
    const float long_scale = get_f32(record + 4);
    if (!(long_scale > 0.0f) || !std::isfinite(long_scale)) return norm_sqr + q.query_norm_sqr;
    const uint8_t *code = record + s.off_code_compact();
    int32_t dot = 0;  // |dot| <= 7 * 128 * D: an int32, exact in any order
    const int8_t *x = q.int8_code.data();
    for (size_t j = 0; j < s.code_dim / 2; ++j)
        dot += static_cast<int32_t>(code[j] & 7U) * x[2 * j] + static_cast<int32_t>((code[j] >> 4U) & 7U) * x[2 * j + 1];
    return finish_traversal(q, norm_sqr, long_scale, short_ip, dot);
}

// finish_paper_prune_estimate_sidecar (space_rabitq.h:4701-4721); the upper bound
// cross + (eps*err)*qn is contracted to fma(eps*err, qn, cross).
qgo_paper_estimate finish_gate(const qgo_prepared &q, float short_ip, const Factors &f,
                               float eps) {
    qgo_paper_estimate r{};
    if (!f.valid) return r;
    const float cross = short_ip * f.cross_scale;
    const float max_cross = 2.0f * f.data_norm * q.query_norm;
    const float upper =
        std::max(-max_cross, std::min(max_cross, cross + eps * f.error_cross_scale * q.query_norm));
    r.lower_bound = f.norm_sqr + q.query_norm_sqr - upper;
    r.short_ip = short_ip;
    r.ip_hat = max_cross > 0.0f ? cross / max_cross : 0.0f;
    r.error_bound = max_cross > 0.0f ? eps * f.error_cross_scale * q.query_norm / max_cross : 0.0f;
    r.valid = std::isfinite(r.lower_bound) ? 1 : 0;
    return r;
}

// compute_paper_prune_estimate (space_rabitq.h:3926-3959), behind rabitq_paper_estimate and
// rabitq_paper_estimate_batch: the gate from the encoded record itself, any codec. The short ip is
// the FP32 restore's selected sum (shortCodeIpFromFullCodeAvx512, :1307-1329: the same 16 lanes
// over pairs and reduce tree) minus the half sum; the bound is formed on the normalised inner
// product and returns alpha; the reference build contracts the final lower bound as
// fma(-two_norms, ip_upper, norm_sqr + qn2).
qgo_paper_estimate gate_encoded_one(const qgo_space &s, const qgo_prepared &q, const uint8_t *record, float eps) {
    qgo_paper_estimate r{};
    const float norm_sqr = get_f32(record);
    const float short_scale = get_f32(record + 8);
    const size_t D = s.code_dim;
    if (D <= 1 || eps < 0.0f || !std::isfinite(eps) || norm_sqr <= 0.0f || q.query_norm <= 0.0f ||
        short_scale <= 0.0f || !std::isfinite(short_scale))
        return r;
    const float data_norm = std::sqrt(norm_sqr);
    const float alpha_raw = 4.0f * data_norm / (short_scale * std::sqrt(static_cast<float>(D)));
    if (!(alpha_raw > 0.0f) || !std::isfinite(alpha_raw)) return r;
    const float alpha = std::min(1.0f, alpha_raw);
    const uint8_t *code = record + s.off_code_compact();
    float sel[16] = {};
    const float *rr = q.rotated_residual.data();
    for (size_t base = 0; base < s.pair_count; base += 16)
        for (int l = 0; l < 16; ++l) {
            const size_t pair = base + l;
            const uint8_t packed = code[pair];
            if ((packed & 0x0FU) > 7U) sel[l] = sel[l] + rr[2 * pair];
            if ((packed >> 4U) > 7U) sel[l] = sel[l] + rr[2 * pair + 1];
        }
    const float short_ip = reduce16(sel) - q.half_sum;
    const float cross = short_ip * short_scale;
    const float two_norms = 2.0f * data_norm * q.query_norm;
    const float ip_hat = cross / two_norms;
    const float alpha2 = alpha * alpha;
    const float error_bound =
        std::sqrt(std::max(0.0f, (1.0f - alpha2) / alpha2)) * eps / std::sqrt(static_cast<float>(D - 1));
    const float ip_upper = std::max(-1.0f, std::min(1.0f, ip_hat + error_bound));
    r.lower_bound = std::fma(-two_norms, ip_upper, norm_sqr + q.query_norm_sqr);  // FMA
    r.short_ip = short_ip;
    r.alpha = alpha;
    r.ip_hat = ip_hat;
    r.error_bound = error_bound;
    r.valid = std::isfinite(r.lower_bound) ? 1 : 0;
    return r;
}

// compute_paper_prune_estimate_int_msb_gate (space_rabitq.h:4873-4899) and the by-id batch
// (space_rabitq.h:4991-5093): integer masked sum, then the float finish.
qgo_paper_estimate gate_one(const qgo_space &s, const qgo_prepared &q, const uint8_t *msb,
                            const Factors &f, float eps) {
    qgo_paper_estimate r{};
    if (!f.valid) return r;
    if (q.query_norm <= 0.0f || f.cross_scale <= 0.0f || !std::isfinite(f.cross_scale))
        return r;
    int64_t selected = 0;  // integer sum: exact in any order
    if (q.gate_tab.size() == s.code_dim / 4 * 16) {
        const int16_t *t = q.gate_tab.data();
        int32_t acc = 0;
        for (size_t j = 0; j < s.code_dim / 8; ++j)
            acc += t[32 * j + (msb[j] & 15U)] + t[32 * j + 16 + (msb[j] >> 4U)];
        selected = acc;
    } else {
        for (size_t i = 0; i < s.code_dim; ++i)
            if ((msb[i >> 3U] >> (i & 7U)) & 1U) selected += q.int8_code[i];
    }
    const float short_ip =
        0.5f * q.int8_scale * static_cast<float>(static_cast<int64_t>(2) * selected - q.code_sum);
    return finish_gate(q, short_ip, f, eps);
}

// compute_b1_paper_prune_estimate_batch_by_id + finish_b1_paper_prune_estimate
// (space_rabitq.h:4607-4695, 4727-4753): popcount of the sign-code mismatches, the symmetric
// 1-bit cross term, and a bound with the database and the query error terms added.
qgo_paper_estimate gate_b1_one(const qgo_space &s, const qgo_prepared &q, const uint8_t *msb,
                               const Factors &f, float eps) {
    qgo_paper_estimate r{};
    const bool query_valid = q.b1_short_scale > 0.0f && std::isfinite(q.b1_short_scale) && q.query_norm > 0.0f;
    if (!query_valid || !f.valid || f.cross_scale <= 0.0f || !std::isfinite(f.cross_scale) || f.data_norm <= 0.0f)
        return r;
    uint64_t mism = 0;
    for (size_t j = 0; j < s.msb_bytes; ++j)
        mism += static_cast<uint64_t>(__builtin_popcount(static_cast<unsigned>(q.b1_code[j] ^ msb[j])));
    const float signed_dot = static_cast<float>(s.code_dim) - 2.0f * static_cast<float>(mism);
    const float short_ip = signed_dot * q.b1_short_scale / 8.0f;
    const float cross = short_ip * f.cross_scale;
    const float max_cross = 2.0f * f.data_norm * q.query_norm;
    const float err_sum = std::fma(f.error_cross_scale, q.query_norm, q.b1_error_scale * f.data_norm);  // FMA
    const float upper = std::max(-max_cross, std::min(max_cross, cross + eps * err_sum));
    r.lower_bound = f.norm_sqr + q.query_norm_sqr - upper;
    r.short_ip = short_ip;
    r.alpha = q.b1_alpha;
    r.ip_hat = max_cross > 0.0f ? cross / max_cross : 0.0f;
    r.error_bound = max_cross > 0.0f ? eps * err_sum / max_cross : 0.0f;
    r.valid = std::isfinite(r.lower_bound) ? 1 : 0;
    return r;
}

// compute_full_paper_prune_estimate_batch_by_id AVX-512 path (space_rabitq.h:4427-4505): lane t
// adds the rotated residual of dims 16k + t whose MSB bit is set (masked adds), the lanes are
// reduced by the _mm512_reduce_add_ps tree, short ip = selected - half sum, then the sidecar finish.
qgo_paper_estimate gate_full_one(const qgo_space &s, const qgo_prepared &q, const uint8_t *msb,
                                 const Factors &f, float eps) {
    float acc[16] = {};
    const float *r = q.rotated_residual.data();
    for (size_t dim = 0; dim < s.code_dim; dim += 16)
        for (int t = 0; t < 16; ++t) {
            const size_t i = dim + t;
            acc[t] = acc[t] + (((msb[i >> 3U] >> (i & 7U)) & 1U) ? r[i] : 0.0f);
        }
    return finish_gate(q, reduce16(acc) - q.half_sum, f, eps);
}

// compute_residual_distance_intervals_batch_by_id AVX2 path (space_rabitq.h:5432-5548):
// per 16-dim block, 8 lanes of lo*qe + hi*qo (the add contracted), summed lane 0..7 in
// order, then ips += scale * block_ip (contracted).
// fused: the residual half of compute_full_residual_distance_intervals_batch_by_id
// (space_rabitq.h:5700-5743, the AVX-512 build), where the compiler contracts the other
// product of the pair: fma(lo, qe, hi*qo) instead of fma(hi, qo, lo*qe). The two orders
// differ by one ulp on rare records.
qgo_interval residual_interval(const qgo_space &s, const qgo_prepared &q, const uint8_t *res,
                               float long_d, bool fused = false) {
    const uint8_t *scales = res + 8;
    const uint8_t *codes = res + 8 + s.scale_bytes;
    const float *r = q.rotated_residual.data();
    float ips = 0.0f;
    double err_sqr = 0.0;
    for (size_t block = 0; block < s.block_count; ++block) {
        uint16_t h;
        std::memcpy(&h, scales + 2 * block, 2);
        const float scale = half_to_float_ref(h);
        if (scale == 0.0f || !std::isfinite(scale)) continue;
        const size_t pair0 = block * 8;
        float block_ip = 0.0f;
        for (int j = 0; j < 8; ++j) {
            const size_t pair = pair0 + j;
            const uint8_t packed = codes[pair];
            int lo = packed & 0x0F, hi = packed >> 4;
            if (lo > 7) lo -= 16;
            if (hi > 7) hi -= 16;
            const float prod =
                fused ? std::fma(static_cast<float>(lo), r[2 * pair], static_cast<float>(hi) * r[2 * pair + 1])
                      : std::fma(static_cast<float>(hi), r[2 * pair + 1], static_cast<float>(lo) * r[2 * pair]);
            block_ip += prod;
        }
        ips = std::fma(scale, block_ip, ips);  // FMA
        const double pde = 0.5 * std::abs(static_cast<double>(scale));
        err_sqr += 16.0 * pde * pde;
    }
    const float distance = long_d - 2.0f * ips;
    const float err =
        static_cast<float>(2.0 * static_cast<double>(q.query_norm) * std::sqrt(err_sqr));
    return qgo_interval{distance, distance - err, distance + err};
}

}  // namespace

extern "C" {

qgo_space *qgo_space_new(size_t dim, uint32_t seed) {
    if (dim == 0) return nullptr;
    auto *s = new qgo_space();
    s->dim = dim;
    s->code_dim = round_up_code_dim(dim);
    s->pair_count = s->code_dim / 2;
    s->code_bytes = (s->code_dim + 1) / 2;
    s->block_count = (s->code_dim + kBlock - 1) / kBlock;
    s->scale_bytes = s->block_count * 2;
    s->full_bytes = 8 + 8 + 8 + s->scale_bytes + s->code_bytes + 1 + s->code_bytes;
    s->compact_bytes = 8 + 8 + s->code_bytes + 1;
    s->residual_bytes = 8 + s->scale_bytes + s->code_bytes;
    s->msb_bytes = (s->code_dim + 7) / 8;
    s->seed = seed;
    const float inv_sqrt = 1.0f / std::sqrt(static_cast<float>(s->code_dim));
    s->signs.assign(s->code_dim, inv_sqrt);
    s->center.assign(dim, 0.0f);
    s->rotated_center.assign(s->code_dim, 0.0f);
    if (seed != 0) {
        // setRandomRotation (space_rabitq.h:2900-2912)
        std::mt19937 rng(seed);
        std::uniform_int_distribution<int> bernoulli(0, 1);
        for (size_t i = 0; i < s->code_dim; ++i)
            s->signs[i] = (bernoulli(rng) ? 1.0f : -1.0f) * inv_sqrt;
    }
    return s;
}

void qgo_space_delete(qgo_space *space) { delete space; }

// setCentroids (space_rabitq.h:2918-2936): ||c||^2 accumulated in double with FMA.
int qgo_space_set_center(qgo_space *s, const float *center) {
    if (!s || !center) return -1;
    std::copy(center, center + s->dim, s->center.begin());
    double norm = 0.0;
    for (size_t i = 0; i < s->dim; ++i)
        norm = std::fma(static_cast<double>(center[i]), static_cast<double>(center[i]), norm);  // FMA
    s->center_norm_sqr = static_cast<float>(norm);
    rotate_into(*s, s->center.data(), s->rotated_center.data());
    return 0;
}

size_t qgo_code_dim(const qgo_space *s) { return s->code_dim; }
size_t qgo_full_bytes(const qgo_space *s) { return s->full_bytes; }
size_t qgo_compact_bytes(const qgo_space *s) { return s->compact_bytes; }
size_t qgo_residual_bytes(const qgo_space *s) { return s->residual_bytes; }
size_t qgo_msb_bytes(const qgo_space *s) { return s->msb_bytes; }
void qgo_space_signs(const qgo_space *s, float *out) {
    std::copy(s->signs.begin(), s->signs.end(), out);
}
void qgo_space_rotated_center(const qgo_space *s, float *out) {
    std::copy(s->rotated_center.begin(), s->rotated_center.end(), out);
}
float qgo_space_center_norm_sqr(const qgo_space *s) { return s->center_norm_sqr; }
void qgo_rotate(const qgo_space *s, const float *raw, float *out) { rotate_into(*s, raw, out); }

// encodeVectorFullWithCentroid (space_rabitq.h:5845-5999), one centroid.
int qgo_encode_full(const qgo_space *sp, const float *raw, uint8_t *out) {
    const qgo_space &s = *sp;
    const size_t D = s.code_dim;
    std::vector<float> residual(s.dim);
    float rns = 0.0f;
    for (size_t i = 0; i < s.dim; ++i) {
        residual[i] = raw[i] - s.center[i];
        rns += residual[i] * residual[i];
    }
    const float rn = std::sqrt(rns);
    if (rn > 0.0f) {
        const float inv = 1.0f / rn;
        for (float &v : residual) v *= inv;
    }
    std::vector<float> ru(D);
    rotate_into(s, residual.data(), ru.data());

    std::memset(out, 0, s.full_bytes);
    uint8_t *code = out + s.off_code_full();
    uint8_t *rescode = out + s.off_rescode_full();
    uint8_t *scales = out + s.off_scales_full();
    out[s.off_cid_full()] = 0;
    const float norm_sqr = rn * rn;

    std::vector<float> abs_unit(D);
    std::vector<uint8_t> abs_code(D);
    for (size_t i = 0; i < D; ++i) abs_unit[i] = std::abs(ru[i]);
    float ip_norm = 1.0f;
    fast_quantize_abs(s, abs_unit.data(), abs_code.data(), ip_norm);
    const float long_scale = 2.0f * rn * ip_norm;

    double o_obar = 0.0, half_l1 = 0.0;
    const double inv_sqrt_d = 1.0 / std::sqrt(static_cast<double>(D));
    for (size_t i = 0; i < D; ++i) {
        const bool positive = ru[i] > 0.0f;
        const uint8_t value = positive ? static_cast<uint8_t>(kMsbWeight + abs_code[i])
                                       : static_cast<uint8_t>(kRemainingMax - abs_code[i]);
        uint8_t &byte = code[i >> 1U];
        byte = (i & 1U) ? static_cast<uint8_t>((byte & 0x0FU) | (value << 4U))
                        : static_cast<uint8_t>((byte & 0xF0U) | value);
        const double sign = positive ? 1.0 : -1.0;
        o_obar = std::fma(static_cast<double>(ru[i]) * sign, inv_sqrt_d, o_obar);  // FMA
        half_l1 += 0.5 * std::abs(static_cast<double>(ru[i]));
    }
    float short_scale = 0.0f, error_scale = 0.0f;
    if (rn > 0.0f && half_l1 > 1e-12) {
        short_scale = static_cast<float>(2.0 * rn / half_l1);
        if (!std::isfinite(o_obar)) o_obar = 0.8;
        o_obar = std::min(0.999999, std::max(1e-6, o_obar));
        const double o2 = o_obar * o_obar;
        const double fac = std::ldexp(5.75, -4) / std::sqrt(static_cast<double>(D));
        error_scale = static_cast<float>(std::sqrt(std::max(0.0, (1.0 - o2) / o2)) * fac * 2.0 * rn);
    }

    std::vector<float> qerr(D);
    for (size_t i = 0; i < D; ++i) {
        const double tv = static_cast<double>(rn) * static_cast<double>(ru[i]);
        const double x4 = 0.5 * static_cast<double>(long_scale) *
                          (static_cast<double>(nib(code, i)) - static_cast<double>(kUnsignedOffset));
        qerr[i] = static_cast<float>(tv - x4);
    }
    double dec_norm = 0.0, x4_ip = 0.0;
    std::vector<int32_t> rcodes(D, 0);
    for (size_t block = 0; block < s.block_count; ++block) {
        const size_t begin = block * kBlock, end = std::min(D, begin + kBlock);
        const float scale = mse_scale(qerr.data(), begin, end);
        const uint16_t h = float_to_half_ref(scale);
        std::memcpy(scales + 2 * block, &h, 2);
        const float stored = half_to_float_ref(h);
        if (stored == 0.0f || !std::isfinite(stored)) continue;
        for (size_t i = begin; i < end; ++i) {
            const int32_t c = std::max(
                -7, std::min(7, static_cast<int32_t>(std::round(static_cast<double>(qerr[i]) /
                                                                static_cast<double>(stored)))));
            rcodes[i] = c;
            const double dec = static_cast<double>(stored) * static_cast<double>(c);
            const double x4 = 0.5 * static_cast<double>(long_scale) *
                              (static_cast<double>(nib(code, i)) - static_cast<double>(kUnsignedOffset));
            dec_norm += dec * dec;
            x4_ip += x4 * dec;
        }
    }
    for (size_t i = 0; i < D; ++i) {
        const uint8_t u = static_cast<uint8_t>(static_cast<uint32_t>(rcodes[i]) & 0x0FU);
        rescode[i >> 1U] |= static_cast<uint8_t>(u << ((i & 1U) * 4U));
    }
    put_f32(out + 0, norm_sqr);
    put_f32(out + 4, long_scale);
    put_f32(out + 8, short_scale);
    put_f32(out + 12, error_scale);
    put_f32(out + 16, static_cast<float>(dec_norm));
    put_f32(out + 20, static_cast<float>(x4_ip));
    return 0;
}

// copyCompactPayloadFromFull / copyResidualRecordFromFull (space_rabitq.h:6005-6029)
void qgo_copy_compact(const qgo_space *s, const uint8_t *full, uint8_t *out) {
    std::memcpy(out, full, 16);
    std::memcpy(out + 16, full + s->off_code_full(), s->code_bytes);
    out[16 + s->code_bytes] = full[s->off_cid_full()];
}

void qgo_copy_residual(const qgo_space *s, const uint8_t *full, uint8_t *out) {
    std::memcpy(out, full + 16, 8);
    std::memcpy(out + 8, full + 24, s->scale_bytes);
    std::memcpy(out + 8 + s->scale_bytes, full + s->off_rescode_full(), s->code_bytes);
}

int qgo_encode_batch(const qgo_space *s, const float *raw, size_t n, uint8_t *compact,
                     uint8_t *residual, int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#endif
    {
        std::vector<uint8_t> full(s->full_bytes);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (long long i = 0; i < static_cast<long long>(n); ++i) {
            qgo_encode_full(s, raw + static_cast<size_t>(i) * s->dim, full.data());
            if (compact) qgo_copy_compact(s, full.data(), compact + static_cast<size_t>(i) * s->compact_bytes);
            if (residual)
                qgo_copy_residual(s, full.data(), residual + static_cast<size_t>(i) * s->residual_bytes);
        }
    }
    (void)threads;
    return 0;
}

// extract_paper_prune_sidecar (space_rabitq.h:4364-4392)
int qgo_export_sidecar(const qgo_space *s, const uint8_t *compact, size_t n, size_t stride,
                       uint8_t *msb_out, void *factors_out) {
    Factors *factors = static_cast<Factors *>(factors_out);
    const size_t D = s->code_dim;
    for (size_t id = 0; id < n; ++id) {
        const uint8_t *rec = compact + id * stride;
        uint8_t *msb = msb_out + id * s->msb_bytes;
        std::memset(msb, 0, s->msb_bytes);
        const uint8_t *code = rec + s->off_code_compact();
        for (size_t i = 0; i < D; ++i)
            if ((nib(code, i) >> 3U) != 0) msb[i >> 3U] |= static_cast<uint8_t>(1U << (i & 7U));
        Factors f{};
        f.norm_sqr = get_f32(rec);
        const float short_scale = get_f32(rec + 8);
        if (!(D <= 1 || f.norm_sqr <= 0.0f || short_scale <= 0.0f)) {
            const float data_norm = std::sqrt(f.norm_sqr);
            f.data_norm = data_norm;
            const float alpha = std::min(
                1.0f, 4.0f * data_norm / (short_scale * std::sqrt(static_cast<float>(D))));
            if (alpha > 0.0f && std::isfinite(alpha)) {
                const float alpha2 = alpha * alpha;
                f.cross_scale = short_scale;
                f.error_cross_scale = 2.0f * data_norm *
                                      std::sqrt(std::max(0.0f, (1.0f - alpha2) / alpha2)) /
                                      std::sqrt(static_cast<float>(D - 1));
                f.valid = std::isfinite(f.error_cross_scale) ? 1 : 0;
            }
        }
        std::memcpy(&factors[id], &f, sizeof(Factors));
    }
    return 0;
}

// distanceBetweenEncoded (space_rabitq.h:2634-2683), one centroid.
float qgo_symmetric_distance(const qgo_space *s, const uint8_t *lhs, const uint8_t *rhs) {
    const float ln2 = get_f32(lhs), rn2 = get_f32(rhs);
    const float lls = get_f32(lhs + 4), rls = get_f32(rhs + 4);
    const double ln = std::sqrt(std::max(0.0, static_cast<double>(ln2)));
    const double rn = std::sqrt(std::max(0.0, static_cast<double>(rn2)));
    if (!(ln > 0.0) || !(rn > 0.0) || !(lls > 0.0f) || !(rls > 0.0f) || !std::isfinite(lls) ||
        !std::isfinite(rls))
        return static_cast<float>(static_cast<double>(ln2) + static_cast<double>(rn2));
    const uint8_t *lc = lhs + s->off_code_compact();
    const uint8_t *rc = rhs + s->off_code_compact();
    int64_t sum = 0;
    for (size_t p = 0; p < s->pair_count; ++p) {
        sum += (2 * static_cast<int32_t>(lc[p] & 0x0F) - 15) * (2 * static_cast<int32_t>(rc[p] & 0x0F) - 15);
        sum += (2 * static_cast<int32_t>(lc[p] >> 4) - 15) * (2 * static_cast<int32_t>(rc[p] >> 4) - 15);
    }
    const double code_ip = 0.25 * static_cast<double>(sum);
    const double lip = static_cast<double>(lls) / (2.0 * ln);
    const double rip = static_cast<double>(rls) / (2.0 * rn);
    double u = code_ip * lip * rip;
    if (!std::isfinite(u)) u = 0.0;
    u = std::max(-1.0, std::min(1.0, u));
    const double rip2 = ln * rn * u;
    return static_cast<float>(static_cast<double>(ln2) + static_cast<double>(rn2) - 2.0 * rip2);
}

qgo_prepared *qgo_prepared_new(const qgo_space *s) {
    auto *p = new qgo_prepared();
    p->space = s;
    p->rotated_residual.assign(s->code_dim, 0.0f);
    p->int8_code.assign(s->code_dim, 0);
    return p;
}

void qgo_prepared_delete(qgo_prepared *p) { delete p; }

// FNV-1a over the raw query bytes mixed with the centroid id (space_rabitq.h:3568-3580)
uint64_t qgo_dither_seed(const float *query, size_t dim, uint32_t centroid_id) {
    uint64_t h = 1469598103934665603ULL;
    const uint8_t *bytes = reinterpret_cast<const uint8_t *>(query);
    for (size_t i = 0; i < dim * sizeof(float); ++i) {
        h ^= bytes[i];
        h *= 1099511628211ULL;
    }
    h ^= static_cast<uint64_t>(centroid_id) + 0x9E3779B97F4A7C15ULL + (h << 6U) + (h >> 2U);
    return h;
}

void qgo_dither_draws(uint64_t seed, size_t count, double *out) {
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    for (size_t i = 0; i < count; ++i) out[i] = u01(rng);
}

// initializePreparedQuery + buildCentroidQuery (space_rabitq.h:3429-3698), INT8 or INT4 codec
// (qgo_space_set_query_codec); the integer codes of either live in int8_code.
int qgo_prepare(const qgo_space *sp, const float *query, qgo_prepared *p) {
    const qgo_space &s = *sp;
    const size_t D = s.code_dim;
    std::vector<float> rq(D);
    rotate_into(s, query, rq.data());
    double rqn = 0.0;
    for (size_t i = 0; i < s.dim; ++i)
        rqn = std::fma(static_cast<double>(query[i]), static_cast<double>(query[i]), rqn);  // FMA
    for (size_t i = 0; i < D; ++i) p->rotated_residual[i] = rq[i] - s.rotated_center[i];
    double dot = 0.0;
    for (size_t i = 0; i < s.dim; ++i)
        dot = std::fma(static_cast<double>(query[i]), static_cast<double>(s.center[i]), dot);  // FMA
    float qn2 = static_cast<float>(rqn + static_cast<double>(s.center_norm_sqr) - 2.0 * dot);
    qn2 = std::max(0.0f, qn2);
    p->query_norm_sqr = qn2;
    float half = 0.0f, max_abs = 0.0f;
    for (size_t pair = 0; pair < s.pair_count; ++pair) {
        const float e = p->rotated_residual[2 * pair], o = p->rotated_residual[2 * pair + 1];
        half += e + o;
        max_abs = std::max(max_abs, std::max(std::fabs(e), std::fabs(o)));
    }
    p->half_sum = half * 0.5f;
    p->query_norm = std::sqrt(qn2);
    p->int8_scale = 1.0f;
    p->code_sum = 0;
    std::fill(p->int8_code.begin(), p->int8_code.end(), 0);
    p->gate_tab.clear();
    if (s.query_bits == 32) return 0;  // Full: the FP32 residual only (space_rabitq.h:3489-3492)
    if (s.query_bits == 1) {  // B1: sign bits and the 1-bit estimator's scales (no integer codes)
        p->b1_code.assign(s.msb_bytes, 0);
        p->b1_signed_sum = 0;
        p->b1_short_scale = p->b1_error_scale = p->b1_alpha = 0.0f;
        float abs_sum = 0.0f;
        for (size_t i = 0; i < D; ++i) {
            const float r = p->rotated_residual[i];
            abs_sum += std::fabs(r);
            if (r > 0.0f) {
                p->b1_code[i >> 3U] = static_cast<uint8_t>(p->b1_code[i >> 3U] | (1U << (i & 7U)));
                p->b1_signed_sum += 1;
            } else {
                p->b1_signed_sum -= 1;
            }
        }
        if (p->query_norm > 0.0f && abs_sum > 0.0f && D > 1) {
            const float a_q = abs_sum / p->query_norm;
            const float alpha_q = std::min(1.0f, a_q / std::sqrt(static_cast<float>(D)));
            const float alpha2 = alpha_q * alpha_q;
            p->b1_alpha = alpha_q;
            p->b1_short_scale = 4.0f * p->query_norm / a_q;
            p->b1_error_scale = 2.0f * p->query_norm * std::sqrt(std::max(0.0f, (1.0f - alpha2) / alpha2)) /
                                std::sqrt(static_cast<float>(D - 1));
        }
        return 0;
    }
    if (max_abs > 0.0f) {
        // Int8: scale max/128, codes in [-128, 127], the first of the two draws per dimension;
        // Int4: scale max/8, codes in [-8, 7], the second (space_rabitq.h:3538-3655)
        const bool int4 = s.query_bits == 4;
        p->int8_scale = max_abs / (int4 ? 8.0f : 128.0f);
        const int32_t lo = int4 ? -8 : -128, hi = int4 ? 7 : 127;
        std::mt19937_64 rng(qgo_dither_seed(query, s.dim, 0));
        std::uniform_real_distribution<double> u01(0.0, 1.0);
        for (size_t i = 0; i < D; ++i) {
            const double u8 = u01(rng);
            const double u4 = u01(rng);
            int32_t x = static_cast<int32_t>(std::floor(
                static_cast<double>(p->rotated_residual[i]) / static_cast<double>(p->int8_scale) +
                (int4 ? u4 : u8)));
            x = std::max(lo, std::min(hi, x));
            p->int8_code[i] = static_cast<int8_t>(x);
            p->code_sum += x;
        }
    }
    p->gate_tab.assign(D / 4 * 16, 0);
    for (size_t j = 0; j < D / 4; ++j)
        for (int v = 0; v < 16; ++v) {
            int sum = 0;
            for (int b = 0; b < 4; ++b)
                if ((v >> b) & 1) sum += p->int8_code[4 * j + b];
            p->gate_tab[16 * j + v] = static_cast<int16_t>(sum);
        }
    return 0;
}

void qgo_prepared_export(const qgo_prepared *p, float *rr, int8_t *codes, float *scalars,
                         int64_t *code_sum) {
    const size_t D = p->space->code_dim;
    if (rr) std::copy(p->rotated_residual.begin(), p->rotated_residual.begin() + D, rr);
    if (codes) std::copy(p->int8_code.begin(), p->int8_code.begin() + D, codes);
    if (scalars) {
        scalars[0] = p->query_norm_sqr;
        scalars[1] = p->query_norm;
        scalars[2] = p->half_sum;
        scalars[3] = p->int8_scale;
    }
    if (code_sum) *code_sum = p->code_sum;
}

void qgo_gate_batch(const qgo_space *s, const qgo_prepared *q, const uint32_t *ids, size_t count,
                    const uint8_t *msb_base, size_t msb_stride, const void *factors_base,
                    size_t factors_stride, float eps, qgo_paper_estimate *out) {
    const uint8_t *fb = static_cast<const uint8_t *>(factors_base);
    for (size_t i = 0; i < count; ++i) {
        Factors f;
        std::memcpy(&f, fb + static_cast<size_t>(ids[i]) * factors_stride, sizeof(Factors));
        const uint8_t *msb = msb_base + static_cast<size_t>(ids[i]) * msb_stride;
        // compute_paper_prune_estimate_sidecar (space_rabitq.h:4510-4531): B1 -> the popcount gate,
        // Int4 / Int8 -> the integer gate, every other codec (Full, B1Main, the Full variants) ->
        // the FP32 Full gate
        out[i] = s->codec == 1                     ? gate_b1_one(*s, *q, msb, f, eps)
                 : (s->codec == 2 || s->codec == 3) ? gate_one(*s, *q, msb, f, eps)
                                                    : gate_full_one(*s, *q, msb, f, eps);
    }
}

// rabitq_query_distance_batch (rabitq_bridge.cpp:885-970): mode 2 = integer traversal reusing
// the gate's short_ip, modes 1 / 3 = the FP32 remaining bits reusing the Full gate's short ip,
// anything else = full FP32 restore (mode 0).
void qgo_distance_batch(const qgo_space *s, const qgo_prepared *q, const uint32_t *ids,
                        const uint8_t *modes, size_t count, const uint8_t *records,
                        size_t stride, const float *short_ips, float *out) {
    for (size_t i = 0; i < count; ++i) {
        const uint8_t *rec = records + static_cast<size_t>(ids[i]) * stride;
        out[i] = modes[i] == 2                     ? traversal_distance(*s, *q, rec, short_ips[i])
                 : (modes[i] == 1 || modes[i] == 3) ? full_reuse_distance(*s, *q, rec, short_ips[i])
                                                    : restore_distance(*s, *q, rec);
    }
}

// rabitq_residual_distance_batch (rabitq_bridge.cpp:972-1042): the AVX2 batch path, or, when the
// space's codec is FullRerankScalar (6), the per-record path (computeResidualDistanceIntervalFromRecord
// -> residualInt4IpAvx2, space_rabitq.h:1723-1734, 2278-2325), whose compiled products take the
// fused kernel's order.
void qgo_residual_batch(const qgo_space *s, const qgo_prepared *q, const uint32_t *ids,
                        size_t count, const uint8_t *records, size_t record_stride,
                        const uint8_t *residual, size_t residual_stride,
                        const float *long_d, qgo_interval *out) {
    (void)records;
    (void)record_stride;
    const bool per_record = s->codec == 6;
    for (size_t i = 0; i < count; ++i)
        out[i] = residual_interval(*s, *q, residual + static_cast<size_t>(ids[i]) * residual_stride,
                                   long_d[i], per_record);
}

// rabitq_paper_estimate / rabitq_paper_estimate_batch (rabitq_bridge.cpp:425-446, 665-700)
void qgo_gate_encoded_batch(const qgo_space *s, const qgo_prepared *q, const uint32_t *ids, size_t count,
                            const uint8_t *records, size_t record_stride, float eps, qgo_paper_estimate *out) {
    for (size_t i = 0; i < count; ++i)
        out[i] = gate_encoded_one(*s, *q, records + static_cast<size_t>(ids[i]) * record_stride, eps);
}

// compute_full_residual_distance_intervals_batch_by_id (space_rabitq.h:5557-5778) behind
// rabitq_full_residual_distance_batch (rabitq_bridge.cpp:1044-1084): the FP32 restore (its
// long distance equals mode 0's, invalid records included) and the residual in the fused
// kernel's product order.
void qgo_full_residual_batch(const qgo_space *s, const qgo_prepared *q, const uint32_t *ids,
                             size_t count, const uint8_t *records, size_t record_stride,
                             const uint8_t *residual, size_t residual_stride, qgo_interval *out) {
    for (size_t i = 0; i < count; ++i) {
        const float long_d = restore_distance(*s, *q, records + static_cast<size_t>(ids[i]) * record_stride);
        out[i] = residual_interval(*s, *q, residual + static_cast<size_t>(ids[i]) * residual_stride,
                                   long_d, true);
    }
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// The search loop: search_ours_paper_active_inner + flush_distance_batch
// (ours_diskann.rs:1539-1986), insert_candidate_sorted / candidate_less (:1096-1126).
// ------------------------------------------------------------------------------------------
namespace {

struct Candidate {
    float distance;
    uint32_t id;
    bool expanded;
    float lower_bound;
};

inline bool candidate_less(const Candidate &a, const Candidate &b) {
    return a.distance < b.distance || (a.distance == b.distance && a.id < b.id);
}

void insert_sorted(std::vector<Candidate> &pool, const Candidate &c, size_t l_value) {
    if (l_value == 0) return;
    if (pool.size() >= l_value && !candidate_less(c, pool.back())) return;
    // binary_search_by + unwrap_or_else: any position of an equal element, else the
    // insertion point; equal (distance, id) pairs cannot occur for distinct ids.
    size_t lo = 0, hi = pool.size();
    while (lo < hi) {
        const size_t mid = (lo + hi) / 2;
        if (candidate_less(pool[mid], c)) lo = mid + 1; else hi = mid;
    }
    pool.insert(pool.begin() + static_cast<long>(lo), c);
    if (pool.size() > l_value) pool.resize(l_value);
}

constexpr size_t kDistBatch = 64;

struct Flush {
    std::vector<uint32_t> ids;
    std::vector<size_t> slots;
    std::vector<uint8_t> modes;
    std::vector<float> short_ips;
    std::vector<float> dists;
};

void flush_batch(const qgo_kernel_table *kt, const void *prep, std::vector<Candidate> &pool,
                 size_t l_value, const std::vector<qgo_paper_estimate> &est, Flush &f,
                 qgo_search_stats &st) {
    if (f.ids.empty()) return;
    f.dists.assign(f.ids.size(), 0.0f);
    kt->distance_batch(kt->ctx, prep, f.ids.data(), f.modes.data(), f.ids.size(),
                       f.short_ips.data(), f.dists.data());
    for (size_t i = 0; i < f.ids.size(); ++i) {
        const qgo_paper_estimate &paper = est[f.slots[i]];
        const bool full = pool.size() >= l_value;
        const float tail = full ? (pool.empty() ? std::numeric_limits<float>::max() : pool.back().distance)
                                : std::numeric_limits<float>::max();
        if (full && paper.valid) {
            st.paper_checked++;
            if (paper.lower_bound > tail) {
                st.paper_would_prune++;
                st.paper_full_saved++;
                continue;
            }
            st.paper_not_pruned++;
        }
        st.paper_remaining_kernel_calls++;
        st.distance_computations++;
        insert_sorted(pool, Candidate{f.dists[i], f.ids[i], false,
                                      paper.valid ? paper.lower_bound : std::numeric_limits<float>::max()},
                      l_value);
    }
    f.ids.clear();
    f.slots.clear();
    f.modes.clear();
    f.short_ips.clear();
}

}  // namespace

extern "C" int qgo_search_one_with(const qgo_kernel_table *kt, const float *query,
                                   const qgo_search_params *prm, const uint32_t *degrees,
                                   const uint32_t *edges, size_t edge_stride, size_t total_points,
                                   size_t base_points, uint32_t *ids_out, float *dists_out,
                                   qgo_search_stats *stats_out) {
    qgo_search_stats st{};
    const size_t k = prm->k;
    for (size_t i = 0; i < k; ++i) {
        ids_out[i] = UINT32_MAX;
        dists_out[i] = std::numeric_limits<float>::infinity();
    }
    if (k == 0 || total_points == 0) {
        if (stats_out) *stats_out = st;
        return 0;
    }
    const size_t l_value = std::max(prm->l_value, k);
    const size_t beam = prm->beam_width == 0 ? 1 : prm->beam_width;
    const void *prep = kt->prepare(kt->ctx, query);
    std::vector<uint8_t> visited(total_points, 0);
    std::vector<Candidate> pool;
    pool.reserve(l_value + 2);
    if (base_points != 0) {
        visited[0] = 1;
        const float d = kt->distance(kt->ctx, prep, 0);
        insert_sorted(pool, Candidate{d, 0, false, std::numeric_limits<float>::max()}, l_value);
        st.visited_nodes++;
        st.distance_computations++;
        st.paper_remaining_kernel_calls++;
    }
    std::vector<uint32_t> frontier, fresh;
    std::vector<qgo_paper_estimate> est;
    Flush f;
    size_t stall = 0;
    for (;;) {
        const float back_before = pool.empty() ? 0.0f : pool.back().distance;
        frontier.clear();
        for (auto &c : pool) {
            if (!c.expanded) {
                c.expanded = true;
                frontier.push_back(c.id);
                if (frontier.size() == beam) break;
            }
        }
        if (frontier.empty()) break;
        for (uint32_t node : frontier) {
            fresh.clear();
            const uint32_t deg = degrees[node];
            const uint32_t *adj = edges + static_cast<size_t>(node) * edge_stride;
            for (uint32_t j = 0; j < deg; ++j) {
                const uint32_t nb = adj[j];
                if (nb >= total_points) return -1;
                if (!visited[nb]) {
                    visited[nb] = 1;
                    fresh.push_back(nb);
                }
            }
            if (fresh.empty()) continue;
            st.visited_nodes += fresh.size();
            if (prm->codec == 4) {  // B1Main: no gate, every fresh neighbour (ours_diskann.rs:1661-1682)
                for (uint32_t id : fresh) {
                    const float d = kt->distance_b1(kt->ctx, prep, id);
                    st.distance_computations++;
                    st.paper_remaining_kernel_calls++;
                    insert_sorted(pool, Candidate{d, id, false, std::numeric_limits<float>::max()}, l_value);
                }
                continue;
            }
            est.assign(fresh.size(), qgo_paper_estimate{});
            kt->gate(kt->ctx, prep, fresh.data(), fresh.size(), prm->epsilon0, est.data());
            st.paper_msb_kernel_calls += fresh.size();
            for (size_t slot = 0; slot < fresh.size(); ++slot) {
                const qgo_paper_estimate &paper = est[slot];
                const bool full = pool.size() >= l_value;
                const float tail = full ? (pool.empty() ? std::numeric_limits<float>::max() : pool.back().distance)
                                        : std::numeric_limits<float>::max();
                if (full && paper.valid && paper.lower_bound > tail) {
                    st.paper_checked++;
                    st.paper_would_prune++;
                    st.paper_full_saved++;
                    continue;
                }
                f.ids.push_back(fresh[slot]);
                f.slots.push_back(slot);
                // survivors: the quantized traversal for the integer codecs, the FP32 restore
                // for B1 and invalid estimates (ours_diskann.rs:1731-1748)
                // DIST_MODE_* of ours_diskann.rs:1734-1749: invalid gate -> recompute (0); Full,
                // FullStaged, FullRerankScalar -> reuse the FP32 short ip (1); FullScalar (7, a
                // Rust-side switch over the Full prepared query) -> its scalar twin (3); Int4 /
                // Int8 -> the quantized remaining bits (2); B1 -> recompute (0)
                const int c = prm->codec;
                f.modes.push_back(!paper.valid                        ? 0
                                  : (c == 0 || c == 5 || c == 6)      ? 1
                                  : c == 7                            ? 3
                                  : (c == 2 || c == 3)                ? 2
                                                                      : 0);
                f.short_ips.push_back(paper.short_ip);
                if (f.ids.size() >= kDistBatch) flush_batch(kt, prep, pool, l_value, est, f, st);
            }
            flush_batch(kt, prep, pool, l_value, est, f, st);
        }
        st.hops += frontier.size();
        if (prm->kth_stop && pool.size() >= k) {
            const float kth = pool[k - 1].distance;
            float min_lb = std::numeric_limits<float>::max();
            for (const auto &c : pool)
                if (!c.expanded && c.lower_bound < min_lb) min_lb = c.lower_bound;
            if (kth <= min_lb) break;
        }
        if (prm->early_stop_hops != 0 && pool.size() >= l_value) {
            const float back_after = pool.empty() ? 0.0f : pool.back().distance;
            stall = back_after >= back_before ? stall + 1 : 0;
            if (stall >= prm->early_stop_hops) break;
        }
    }
    // rerank (ours_diskann.rs:1813-1902): the residual correction of the pool distances, sorted
    // by (estimate, id). After an INT8 / INT4 traversal the rerank set is first recomputed with
    // the FP32 restore (mode 0), or, with the fused rerank switched on, both run as one kernel;
    // the other codecs correct the distances the traversal left in the pool.
    size_t in_base = 0;
    for (const auto &c : pool) in_base += c.id < base_points ? 1 : 0;
    const size_t rerank_count = std::max(std::min(in_base, std::max(prm->rerank_candidates, k)), k);
    std::vector<uint32_t> rids;
    std::vector<float> rlong;
    for (const auto &c : pool) {
        if (c.id >= base_points) continue;
        if (rids.size() >= rerank_count) break;
        rids.push_back(c.id);
        rlong.push_back(c.distance);
    }
    std::vector<qgo_interval> iv(rids.size());
    if (!rids.empty()) {
        const bool int_query = prm->codec == 2 || prm->codec == 3;
        if (int_query && prm->fused_int_rerank) {
            kt->full_residual_batch(kt->ctx, prep, rids.data(), rids.size(), iv.data());
        } else {
            if (int_query) {
                std::vector<uint8_t> modes(rids.size(), 0);
                std::vector<float> zeros(rids.size(), 0.0f);
                kt->distance_batch(kt->ctx, prep, rids.data(), modes.data(), rids.size(), zeros.data(),
                                   rlong.data());
            }
            kt->residual_batch(kt->ctx, prep, rids.data(), rids.size(), rlong.data(), iv.data());
        }
    }
    std::vector<std::pair<float, uint32_t>> rr(rids.size());
    for (size_t i = 0; i < rids.size(); ++i) rr[i] = {iv[i].estimate, rids[i]};
    // sort_unstable_by(partial_cmp.then(id)): ascending estimate, ties by id; NaN compares
    // equal to everything, so NaN estimates are ordered by id among their neighbours.
    std::sort(rr.begin(), rr.end(), [](const std::pair<float, uint32_t> &a,
                                       const std::pair<float, uint32_t> &b) {
        if (a.first < b.first) return true;
        if (b.first < a.first) return false;
        return a.second < b.second;
    });
    for (size_t i = 0; i < k && i < rr.size(); ++i) {
        ids_out[i] = rr[i].second;
        dists_out[i] = rr[i].first;
    }
    if (stats_out) *stats_out = st;
    return 0;
}

namespace {

struct OracleCtx {
    const qgo_space *space;
    qgo_prepared *prep;
    const uint8_t *records;
    size_t record_stride;
    const uint8_t *residual;
    size_t residual_stride;
    const uint8_t *msb;
    size_t msb_stride;
    const void *factors;
    size_t factor_stride;
};

const void *ok_prepare(void *ctx, const float *q) {
    auto *c = static_cast<OracleCtx *>(ctx);
    qgo_prepare(c->space, q, c->prep);
    return c->prep;
}
float ok_distance(void *ctx, const void *p, uint32_t id) {
    auto *c = static_cast<OracleCtx *>(ctx);
    return restore_distance(*c->space, *static_cast<const qgo_prepared *>(p),
                            c->records + static_cast<size_t>(id) * c->record_stride);
}
void ok_gate(void *ctx, const void *p, const uint32_t *ids, size_t n, float eps,
             qgo_paper_estimate *out) {
    auto *c = static_cast<OracleCtx *>(ctx);
    qgo_gate_batch(c->space, static_cast<const qgo_prepared *>(p), ids, n, c->msb, c->msb_stride,
                   c->factors, c->factor_stride, eps, out);
}
void ok_dist(void *ctx, const void *p, const uint32_t *ids, const uint8_t *modes, size_t n,
             const float *sips, float *out) {
    auto *c = static_cast<OracleCtx *>(ctx);
    qgo_distance_batch(c->space, static_cast<const qgo_prepared *>(p), ids, modes, n, c->records,
                       c->record_stride, sips, out);
}
float ok_distance_b1(void *ctx, const void *p, uint32_t id) {
    auto *c = static_cast<OracleCtx *>(ctx);
    return distance_b1(*c->space, *static_cast<const qgo_prepared *>(p), c->records + static_cast<size_t>(id) * c->record_stride);
}
void ok_res(void *ctx, const void *p, const uint32_t *ids, size_t n, const float *ld,
            qgo_interval *out) {
    auto *c = static_cast<OracleCtx *>(ctx);
    qgo_residual_batch(c->space, static_cast<const qgo_prepared *>(p), ids, n, c->records,
                       c->record_stride, c->residual, c->residual_stride, ld, out);
}
void ok_full_res(void *ctx, const void *p, const uint32_t *ids, size_t n, qgo_interval *out) {
    auto *c = static_cast<OracleCtx *>(ctx);
    qgo_full_residual_batch(c->space, static_cast<const qgo_prepared *>(p), ids, n, c->records,
                            c->record_stride, c->residual, c->residual_stride, out);
}

}  // namespace

extern "C" int qgo_search_batch(const qgo_space *space, const float *queries, size_t nq,
                                const qgo_search_params *params, const uint8_t *records,
                                size_t record_stride, const uint8_t *residual,
                                size_t residual_stride, const uint8_t *msb, size_t msb_stride,
                                const void *factors, size_t factor_stride,
                                const uint32_t *degrees, const uint32_t *edges,
                                size_t edge_stride, size_t total_points, size_t base_points,
                                uint32_t *ids_out, float *dists_out,
                                qgo_search_stats *stats_out, int threads) {
    int status = 0;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#endif
    {
        OracleCtx ctx{space, qgo_prepared_new(space), records, record_stride, residual,
                      residual_stride, msb, msb_stride, factors, factor_stride};
        qgo_kernel_table kt{&ctx, ok_prepare, ok_distance, ok_gate, ok_dist, ok_res, ok_distance_b1, ok_full_res};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (long long q = 0; q < static_cast<long long>(nq); ++q) {
            const size_t qi = static_cast<size_t>(q);
            const int rc = qgo_search_one_with(
                &kt, queries + qi * space->dim, params, degrees, edges, edge_stride,
                total_points, base_points, ids_out + qi * params->k, dists_out + qi * params->k,
                stats_out ? stats_out + qi : nullptr);
            if (rc != 0) status = rc;
        }
        qgo_prepared_delete(ctx.prep);
    }
    (void)threads;
    return status;
}

extern "C" void qgo_exact_knn(const float *base, size_t n, const float *queries, size_t nq,
                              size_t dim, size_t k, uint32_t *ids_out, double *dists_out,
                              int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (long long q = 0; q < static_cast<long long>(nq); ++q) {
        const float *qv = queries + static_cast<size_t>(q) * dim;
        std::vector<std::pair<double, uint32_t>> all(n);
        for (size_t i = 0; i < n; ++i) {
            const float *b = base + i * dim;
            double sum = 0.0;
            for (size_t j = 0; j < dim; ++j) {
                const double d = static_cast<double>(qv[j]) - static_cast<double>(b[j]);
                sum += d * d;
            }
            all[i] = {sum, static_cast<uint32_t>(i)};
        }
        const size_t kk = std::min(k, n);
        std::partial_sort(all.begin(), all.begin() + static_cast<long>(kk), all.end());
        for (size_t i = 0; i < k; ++i) {
            ids_out[static_cast<size_t>(q) * k + i] = i < kk ? all[i].second : UINT32_MAX;
            dists_out[static_cast<size_t>(q) * k + i] =
                i < kk ? all[i].first : std::numeric_limits<double>::infinity();
        }
    }
    (void)threads;
}

// ---- Vamana graph build over the symmetric 4-bit estimator --------------------------
// Restates VamanaIndex::buildGraphFromLoadedPayloads (vamana_index.h:452-528),
// refineGraphSymmetric (:328-422), addBackedgesGroupedAndPrune / addBackedgeGroupAndPrune
// (:995-1117), capBuildPrunePool (:201-211), search_vamana (vamana_search.h:98-198) and
// robust_prune_4bit (vamana_prune.h:42-156), as rabitq_build_vamana_graph
// (rabitq_bridge.cpp:224-303) drives them. The build is deterministic: searches of one batch
// read the graph as it was when the batch started, back-edge groups write disjoint sources.
namespace {

struct BuildCand {
    float d;
    uint32_t id;
    bool expanded;
};

inline bool build_less(const BuildCand &a, const BuildCand &b) {
    return a.d != b.d ? a.d < b.d : a.id < b.id;
}

struct BuildState {
    const qgo_space *space;
    const uint8_t *compact;
    size_t stride;
    size_t r, l_build, beam, cap, stop_hops;
    float alpha;
    std::vector<std::vector<uint32_t>> graph;
    uint64_t evals = 0;  // distances evaluated, counted like distance_evaluations_

    float dist(uint32_t lhs, uint32_t rhs) const {
        return qgo_symmetric_distance(space, compact + lhs * stride, compact + rhs * stride);
    }
};

struct BuildScratch {
    std::vector<uint32_t> tags;
    uint32_t epoch = 0;
    std::vector<BuildCand> pool;
    uint64_t evals = 0;
};

// search_vamana: beam search from node 0 over nodes [0, node_count); returns false on an
// out-of-range neighbour (the reference throws there).
bool build_search(const BuildState &st, uint32_t query, size_t node_count, BuildScratch &sc) {
    if (sc.tags.size() < node_count) sc.tags.resize(node_count, 0);
    if (++sc.epoch == 0) {
        std::fill(sc.tags.begin(), sc.tags.end(), 0);
        sc.epoch = 1;
    }
    auto &pool = sc.pool;
    pool.clear();
    pool.push_back({st.dist(query, 0), 0, false});
    sc.evals += 1;
    sc.tags[0] = sc.epoch;
    std::vector<uint32_t> frontier;
    size_t stall = 0;
    for (;;) {
        const float back_before = pool.back().d;
        frontier.clear();
        for (auto &c : pool) {
            if (!c.expanded) {
                c.expanded = true;
                frontier.push_back(c.id);
                if (frontier.size() == st.beam) break;
            }
        }
        if (frontier.empty()) break;
        for (uint32_t node : frontier) {
            for (uint32_t nb : st.graph[node]) {
                if (nb >= node_count) return false;
                if (sc.tags[nb] == sc.epoch) continue;
                sc.tags[nb] = sc.epoch;
                const BuildCand c{st.dist(query, nb), nb, false};
                sc.evals += 1;
                // insert_candidate_sorted (vamana_search.h:79-96)
                if (pool.size() >= st.l_build && !build_less(c, pool.back())) continue;
                pool.insert(std::lower_bound(pool.begin(), pool.end(), c, build_less), c);
                if (pool.size() > st.l_build) pool.resize(st.l_build);
            }
        }
        if (st.stop_hops != 0 && pool.size() >= st.l_build) {
            stall = pool.back().d >= back_before ? stall + 1 : 0;
            if (stall >= st.stop_hops) break;
        }
    }
    return true;
}

void cap_pool(const BuildState &st, std::vector<BuildCand> &pool) {
    if (st.cap == 0 || pool.size() <= st.cap) return;
    std::partial_sort(pool.begin(), pool.begin() + static_cast<long>(st.cap), pool.end(), build_less);
    pool.resize(st.cap);
}

// robust_prune_4bit: alpha ramp 1 -> alpha in steps of x min(alpha, 1.2); pair distances
// (candidate, selected) evaluated lazily and memoised, as the reference does.
std::vector<uint32_t> robust_prune(const BuildState &st, uint32_t source, std::vector<BuildCand> cands,
                                   uint64_t &evals) {
    std::sort(cands.begin(), cands.end(), build_less);
    std::vector<BuildCand> uniq;
    uniq.reserve(cands.size());
    for (const auto &c : cands) {
        if (c.id == source) continue;
        bool dup = false;
        for (const auto &u : uniq) {
            if (u.id == c.id) {
                dup = true;
                break;
            }
        }
        if (!dup) uniq.push_back(c);
    }
    const size_t degree = st.r;
    std::vector<uint32_t> selected;
    std::vector<uint8_t> disabled(uniq.size(), 0);
    std::vector<float> memo(uniq.size() * degree, -1.0f);
    float cur = 1.0f;
    const float step = std::min(st.alpha, 1.2f);
    while (selected.size() < degree) {
        bool promoted = false;
        for (size_t i = 0; i < uniq.size() && selected.size() < degree; ++i) {
            if (disabled[i]) continue;
            bool occluded = false;
            for (size_t k = 0; k < selected.size(); ++k) {
                float &m = memo[i * degree + k];
                if (m < 0.0f) {
                    m = st.dist(uniq[i].id, selected[k]);
                    evals += 1;
                }
                if (cur * m <= uniq[i].d) {
                    occluded = true;
                    break;
                }
            }
            if (occluded) continue;
            selected.push_back(uniq[i].id);
            disabled[i] = 1;
            promoted = true;
        }
        if (cur == st.alpha) break;
        const float next = std::min(st.alpha, cur * step);
        if (next == cur) break;
        cur = next;
        if (!promoted && selected.size() >= degree) break;
    }
    return selected;
}

// addBackedgesGroupedAndPrune: pairs (source, target) grouped by source; each source takes
// its sorted, de-duplicated targets and is re-pruned when it grows past R.
void add_backedges(BuildState &st, std::vector<std::pair<uint32_t, uint32_t>> &pairs, int threads) {
    if (pairs.empty()) return;
    std::sort(pairs.begin(), pairs.end());
    std::vector<size_t> starts{0};
    for (size_t i = 1; i < pairs.size(); ++i)
        if (pairs[i].first != pairs[i - 1].first) starts.push_back(i);
    starts.push_back(pairs.size());
    uint64_t evals = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 32) num_threads(threads) reduction(+ : evals)
#endif
    for (long long g = 0; g < static_cast<long long>(starts.size()) - 1; ++g) {
        const uint32_t source = pairs[starts[g]].first;
        std::vector<uint32_t> targets;
        for (size_t i = starts[g]; i < starts[g + 1]; ++i)
            if (pairs[i].second != source) targets.push_back(pairs[i].second);
        if (targets.empty()) continue;
        std::sort(targets.begin(), targets.end());
        targets.erase(std::unique(targets.begin(), targets.end()), targets.end());
        auto &nb = st.graph[source];
        size_t added = 0;
        for (uint32_t t : targets) {
            if (std::find(nb.begin(), nb.end(), t) == nb.end()) {
                nb.push_back(t);
                ++added;
            }
        }
        if (added == 0 || nb.size() <= st.r) continue;
        std::vector<BuildCand> pool;
        for (uint32_t c : nb) {
            if (c == source) continue;
            pool.push_back({st.dist(source, c), c, false});
            evals += 1;
        }
        nb = robust_prune(st, source, std::move(pool), evals);
    }
    (void)threads;
    st.evals += evals;
}

}  // namespace

extern "C" int qgo_build_vamana(const qgo_space *space, const uint8_t *compact, size_t n, size_t stride,
                                size_t r, size_t l_build, float alpha, size_t beam, size_t batch,
                                size_t refine, size_t cap, size_t stop_hops, uint32_t *degrees,
                                uint32_t *edges, size_t edge_stride, uint64_t *evals_out, int threads) {
    if (space == nullptr || (compact == nullptr && n != 0) || degrees == nullptr || edges == nullptr ||
        edge_stride < r || r == 0 || l_build == 0 || beam == 0 || !(alpha >= 1.0f) || !std::isfinite(alpha))
        return -1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#endif
    if (batch == 0) batch = 1;
    BuildState st{space, compact, stride, r, l_build, beam, cap, stop_hops, alpha, {}, 0};
    st.graph.assign(n, {});
    bool ok = true;
    // bulk insertion in batches (vamana_index.h:452-528)
    for (size_t begin = 1; begin < n && ok; begin += batch) {
        const size_t end = std::min(n, begin + batch);
        std::vector<std::vector<uint32_t>> lists(end - begin);
        uint64_t evals = 0;
        bool bad = false;
#ifdef _OPENMP
#pragma omp parallel num_threads(threads) reduction(+ : evals) reduction(|| : bad)
#endif
        {
            BuildScratch sc;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 32)
#endif
            for (long long off = 0; off < static_cast<long long>(end - begin); ++off) {
                const uint32_t id = static_cast<uint32_t>(begin + static_cast<size_t>(off));
                if (!build_search(st, id, begin, sc)) {
                    bad = true;
                    continue;
                }
                std::vector<BuildCand> pool = sc.pool;
                cap_pool(st, pool);
                lists[static_cast<size_t>(off)] = robust_prune(st, id, std::move(pool), evals);
            }
            evals += sc.evals;
        }
        st.evals += evals;
        if (bad) {
            ok = false;
            break;
        }
        std::vector<std::pair<uint32_t, uint32_t>> pairs;
        for (size_t off = 0; off < lists.size(); ++off) {
            const uint32_t id = static_cast<uint32_t>(begin + off);
            st.graph[id] = std::move(lists[off]);
            for (uint32_t nb : st.graph[id]) pairs.emplace_back(nb, id);
        }
        add_backedges(st, pairs, threads);
    }
    // refinement passes over the whole graph (vamana_index.h:328-422)
    for (size_t pass = 0; pass < refine && ok && n > 1; ++pass) {
        std::vector<std::vector<uint32_t>> refined(n);
        uint64_t evals = 0;
        bool bad = false;
#ifdef _OPENMP
#pragma omp parallel num_threads(threads) reduction(+ : evals) reduction(|| : bad)
#endif
        {
            BuildScratch sc;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 32)
#endif
            for (long long sid = 0; sid < static_cast<long long>(n); ++sid) {
                const uint32_t id = static_cast<uint32_t>(sid);
                if (!build_search(st, id, n, sc)) {
                    bad = true;
                    continue;
                }
                std::vector<BuildCand> pool = sc.pool;
                cap_pool(st, pool);
                for (uint32_t x : st.graph[id]) {
                    pool.push_back({st.dist(id, x), x, false});
                    evals += 1;
                }
                refined[id] = robust_prune(st, id, std::move(pool), evals);
            }
            evals += sc.evals;
        }
        st.evals += evals;
        if (bad) {
            ok = false;
            break;
        }
        st.graph.swap(refined);
        std::vector<std::pair<uint32_t, uint32_t>> pairs;
        for (size_t id = 0; id < n; ++id)
            for (uint32_t nb : st.graph[id]) pairs.emplace_back(nb, static_cast<uint32_t>(id));
        add_backedges(st, pairs, threads);
    }
    if (!ok) return -1;
    for (size_t id = 0; id < n; ++id) {
        if (st.graph[id].size() > edge_stride) return -1;
        degrees[id] = static_cast<uint32_t>(st.graph[id].size());
        std::copy(st.graph[id].begin(), st.graph[id].end(), edges + id * edge_stride);
    }
    if (evals_out != nullptr) *evals_out = st.evals;
    return 0;
}

// rabitq_set_query_coarse_codec for the oracle: 0 Full, 1 B1, 2 Int4, 3 Int8, 4 B1Main, 5 FullStaged,
// 6 FullRerankScalar; others return -1. The space's routines branch only on B1 / B1Main / Int4 /
// Int8 (space_rabitq.h:3464-3469, 4519-4531), so 5 and 6 prepare and gate as Full.
extern "C" int qgo_space_set_query_codec(qgo_space *space, int codec) {
    if (!space || codec < 0 || codec > 6) return -1;
    // B1Main prepares like B1; the Full codecs keep only the FP32 residual
    space->query_bits = (codec == 1 || codec == 4) ? 1 : codec == 2 ? 4 : codec == 3 ? 8 : 32;
    space->codec = codec;
    return 0;
}

extern "C" float qgo_distance_b1(const qgo_space *space, const qgo_prepared *prepared, const uint8_t *record) {
    return distance_b1(*space, *prepared, record);
}

// The B1 prepared fields: sign bits [D/8], {short scale, error scale, alpha}, signed sum.
extern "C" void qgo_prepared_export_b1(const qgo_prepared *p, uint8_t *bits, float *scalars, int64_t *signed_sum) {
    if (bits) std::copy(p->b1_code.begin(), p->b1_code.end(), bits);
    if (scalars) {
        scalars[0] = p->b1_short_scale;
        scalars[1] = p->b1_error_scale;
        scalars[2] = p->b1_alpha;
    }
    if (signed_sum) *signed_sum = p->b1_signed_sum;
}

