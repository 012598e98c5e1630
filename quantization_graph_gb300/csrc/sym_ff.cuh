// sym_ff.cuh -- the symmetric 4-bit estimator (symmetricBuildDistanceFromPrepared,
// space_rabitq.h:2706-2747) without the FP64 pipe on the common path.
//
// The reference evaluates, in double precision,
//   u = clamp((S / 4) * ip_norm_l * ip_norm_r, -1, 1),  r = norm_l * norm_r * u,
//   d = float((double)n2_l + (double)n2_r - 2 r)
// and returns the float nearest to the double result. The fast path below evaluates the same
// expression in float-float arithmetic (pairs of floats, error-free products through fmaf and
// error-free sums, about 44 significant bits), bounds its distance E to the reference's double
// result, and returns float(x) only when no float rounding boundary lies within E of the
// float-float value x: then the double result rounds to the same float. Otherwise (and for
// invalid records, values near the clamp at |u| = 1, and extreme magnitudes) it reports
// failure and the caller evaluates the double expression itself.
//
// Error bound (relative to |T| + 2|r|, T = n2_l + n2_r): splitting each double factor into
// a float pair leaves 2^-48; each float-float product adds at most about 2^-46.5; the double
// expression's own four roundings add 2^-53 each; the final float-float subtraction 2^-47.
// The total stays below 2^-43; the check uses 2^-40.
//
// Compiled for the host too (same code, -ffp-contract=off), so a CPU test can compare it
// with the double expression bit for bit.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define QG_HD __host__ __device__ __forceinline__
#else
#define QG_HD inline
#endif

namespace qg {

// Per-record factors: the double values the reference computes (space_rabitq.h:2691-2704)
// and their float-pair splits.
struct SymFactors {
    double rn;   // sqrt(max(0, (double)norm_sqr))
    double rip;  // long_scale / (2 rn); 0 when invalid
    float rn_hi, rn_lo, rip_hi, rip_lo;
    float n2;
    int32_t nsum;  // sum of the record's 4-bit codes
    int32_t valid;
    int32_t pad;
};
static_assert(sizeof(SymFactors) == 48, "SymFactors is 48 bytes");

QG_HD float qg_bits_to_float(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}
QG_HD uint32_t qg_float_to_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}

QG_HD bool qg_finite(float f) { return (qg_float_to_bits(f) & 0x7f800000u) != 0x7f800000u; }
QG_HD bool qg_finite(double d) {
    uint64_t u;
#ifdef __CUDA_ARCH__
    u = static_cast<uint64_t>(__double_as_longlong(d));
#else
    std::memcpy(&u, &d, 8);
#endif
    return (u & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

QG_HD SymFactors sym_factors(float n2, float long_scale, int32_t nsum) {
    SymFactors f;
    f.rn = sqrt(fmax(0.0, static_cast<double>(n2)));
    f.valid = (f.rn > 0.0 && long_scale > 0.0f && qg_finite(long_scale)) ? 1 : 0;
    f.rip = f.valid ? static_cast<double>(long_scale) / (2.0 * f.rn) : 0.0;
    f.rn_hi = static_cast<float>(f.rn);
    f.rn_lo = static_cast<float>(f.rn - static_cast<double>(f.rn_hi));
    f.rip_hi = static_cast<float>(f.rip);
    f.rip_lo = static_cast<float>(f.rip - static_cast<double>(f.rip_hi));
    f.n2 = n2;
    f.nsum = nsum;
    f.pad = 0;
    return f;
}

// The reference's double expression, lhs the prepared side. s = sum over dims of
// (2a - 15)(2b - 15).
QG_HD float sym_distance_f64(const SymFactors &l, const SymFactors &r, int32_t s) {
    if (!l.valid || !r.valid) return static_cast<float>(static_cast<double>(l.n2) + static_cast<double>(r.n2));
    const double code_ip = 0.25 * static_cast<double>(s);
    double u = (code_ip * l.rip) * r.rip;
    if (!qg_finite(u)) u = 0.0;
    u = fmax(-1.0, fmin(1.0, u));
    const double rip = (l.rn * r.rn) * u;
    return static_cast<float>((static_cast<double>(l.n2) + static_cast<double>(r.n2)) - 2.0 * rip);
}

// (xh + xl) * (yh + yl) as a normalised float pair.
QG_HD void ff_mul(float xh, float xl, float yh, float yl, float &zh, float &zl) {
    const float p = xh * yh;
    float e = fmaf(xh, yh, -p);
    e = fmaf(xh, yl, e);
    e = fmaf(xl, yh, e);
    zh = p + e;
    zl = e - (zh - p);
}

// Fast path; ok = false when the caller must evaluate sym_distance_f64.
QG_HD float sym_distance_ff(const SymFactors &l, const SymFactors &r, int32_t s, bool &ok) {
    ok = false;
    if (!l.valid || !r.valid) return 0.0f;
    // magnitudes where every float-pair low part stays normal
    const float lo_lim = 0x1p-60f, hi_lim = 0x1p60f;
    if (!(l.rn_hi > lo_lim && l.rn_hi < hi_lim && r.rn_hi > lo_lim && r.rn_hi < hi_lim && l.rip_hi > lo_lim &&
          l.rip_hi < hi_lim && r.rip_hi > lo_lim && r.rip_hi < hi_lim && s > -(1 << 24) && s < (1 << 24)))
        return 0.0f;
    const float c = 0.25f * static_cast<float>(s);  // exact: |s| < 2^24
    float th, tl, uh, ul;
    ff_mul(c, 0.0f, l.rip_hi, l.rip_lo, th, tl);
    ff_mul(th, tl, r.rip_hi, r.rip_lo, uh, ul);
    const float au = fabsf(uh);
    if (!(au < 0x1p20f) || (au != 0.0f && au < 0x1p-60f)) return 0.0f;
    if (au > 1.0f - 0x1p-20f && au < 1.0f + 0x1p-20f) return 0.0f;  // too close to the clamp
    if (au >= 1.0f) {
        uh = uh > 0.0f ? 1.0f : -1.0f;
        ul = 0.0f;
    }
    float qh, ql, rh, rl;
    ff_mul(l.rn_hi, l.rn_lo, r.rn_hi, r.rn_lo, qh, ql);
    ff_mul(qh, ql, uh, ul, rh, rl);
    // T = n2_l + n2_r exactly (two-sum), then A = T - 2R
    const float th2 = l.n2 + r.n2;
    const float bv = th2 - l.n2;
    const float tl2 = (l.n2 - (th2 - bv)) + (r.n2 - bv);
    const float m2 = -2.0f * rh;
    const float s0 = th2 + m2;
    const float b0 = s0 - th2;
    float se = (th2 - (s0 - b0)) + (m2 - b0);
    se = se + (tl2 - 2.0f * rl);
    const float ah = s0 + se;  // two-sum: exact even when the pair cancelled
    const float b1 = ah - s0;
    const float al = (s0 - (ah - b1)) + (se - b1);
    const float scale = fabsf(th2) + 2.0f * fabsf(rh);
    if (!(scale > 0x1p-60f && scale < 0x1p60f)) return 0.0f;
    const float f = ah + al;  // the float nearest to ah + al
    const float af = fabsf(f);
    if (!(af >= 0x1p-100f) || !qg_finite(f)) return 0.0f;
    const float g = (ah - f) + al;  // (ah + al) - f, to a relative 2^-24
    const float below = qg_bits_to_float(qg_float_to_bits(af) - 1u);
    const float half = 0.5f * (af - below);  // half the smaller of the two gaps around f
    if (fabsf(g) * (1.0f + 0x1p-22f) + scale * 0x1p-40f < half) {
        ok = true;
        return f;
    }
    return 0.0f;
}

QG_HD float sym_distance_exact(const SymFactors &l, const SymFactors &r, int32_t s) {
    bool ok;
    const float f = sym_distance_ff(l, r, s, ok);
    return ok ? f : sym_distance_f64(l, r, s);
}

}  // namespace qg
