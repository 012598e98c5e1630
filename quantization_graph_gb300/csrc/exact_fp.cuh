// exact_fp.cuh -- exact integer arithmetic for reproducing the reference's double-precision
// results without the FP64 pipe (a narrow pipe on this part): float decomposition, 128-bit
// fixed point, round-to-nearest-even to a given significand width, and the float that a
// double expression rounds to.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace qg {

struct FloatParts {
    long long m;  // signed integer significand, |m| < 2^24
    int e;        // value = m * 2^e
    bool finite;
};

__device__ __forceinline__ FloatParts split_float(float f) {
    const uint32_t b = __float_as_uint(f);
    const int ex = static_cast<int>((b >> 23) & 0xFFu);
    long long m = static_cast<long long>(b & 0x7FFFFFu);
    int e = -149;
    if (ex != 0) {
        m |= 0x800000;
        e = ex - 150;
    }
    if (b >> 31) m = -m;
    return {m, e, ex != 0xFF};
}

// |v| (< 2^49) * 2^sh as a 128-bit fixed-point value; shifts below the grid truncate.
__device__ __forceinline__ unsigned __int128 to_grid(unsigned long long v, int sh) {
    if (sh >= 0) return static_cast<unsigned __int128>(v) << sh;
    if (sh <= -64) return 0;
    return static_cast<unsigned __int128>(v >> (-sh));
}

__device__ __forceinline__ __int128 shfl_xor_i128(__int128 v, int o) {
    const unsigned __int128 u = static_cast<unsigned __int128>(v);
    uint32_t w[4] = {static_cast<uint32_t>(u), static_cast<uint32_t>(u >> 32), static_cast<uint32_t>(u >> 64),
                     static_cast<uint32_t>(u >> 96)};
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = __shfl_xor_sync(0xffffffffu, w[i], o);
    const unsigned __int128 r = static_cast<unsigned __int128>(w[0]) |
                                (static_cast<unsigned __int128>(w[1]) << 32) |
                                (static_cast<unsigned __int128>(w[2]) << 64) |
                                (static_cast<unsigned __int128>(w[3]) << 96);
    return static_cast<__int128>(r);
}

__device__ __forceinline__ int msb_u128(unsigned __int128 v) {
    const unsigned long long hi = static_cast<unsigned long long>(v >> 64);
    if (hi != 0) return 127 - __clzll(static_cast<long long>(hi));
    const unsigned long long lo = static_cast<unsigned long long>(v);
    return lo ? 63 - __clzll(static_cast<long long>(lo)) : -1;
}

// Round mag * 2^e (mag > 0) to `bits` significant bits, ties to even.
__device__ __forceinline__ void round_sig(unsigned __int128 &mag, int &e, int bits) {
    const int m = msb_u128(mag);
    if (m < bits) return;
    int sh = m - bits + 1;
    unsigned __int128 keep = mag >> sh;
    const unsigned __int128 rem = mag - (keep << sh);
    const unsigned __int128 half = static_cast<unsigned __int128>(1) << (sh - 1);
    if (rem > half || (rem == half && (keep & 1))) keep += 1;
    if (keep >> bits) {  // carried into 2^bits: one bit shorter, exponent one up
        keep >>= 1;
        sh += 1;
    }
    mag = keep;
    e += sh;
}

// float(RN53(v)) for v = (neg ? -1 : 1) * mag * 2^e held exactly: the value a double
// expression with exact operands produces after its one double rounding and the conversion.
// ok = false when the double or the float would leave the normal range.
__device__ __forceinline__ float float_via_double(bool neg, unsigned __int128 mag, int e, bool &ok) {
    ok = true;
    if (mag == 0) return 0.0f;
    int m = msb_u128(mag);
    if (e + m < -1000 || e + m > 1000) {
        ok = false;
        return 0.0f;
    }
    round_sig(mag, e, 53);
    round_sig(mag, e, 24);
    m = msb_u128(mag);
    const int ex = e + m;
    if (ex < -126 || ex > 127) {
        ok = false;
        return 0.0f;
    }
    const uint32_t sig = static_cast<uint32_t>(static_cast<unsigned long long>(mag) << (23 - m)) & 0x7FFFFFu;
    return __uint_as_float((neg ? 0x80000000u : 0u) | (static_cast<uint32_t>(ex + 127) << 23) | sig);
}

// std::round(double(x) / double(s)) clamped to [-7, 7] (round half away from zero), decided in
// FP32 with the caller's inv_s = RN(1/s) (one reciprocal serves a block of quotients). With
// q = |x| / s: y = RN(|x| inv_s) is within 2^-20 of q (two roundings, q < 7.25); the FMA remainder
// r = RN(|x| - y s) times inv_s gives c with |y + c - q| < 2^-42; the double quotient is within
// 2^-50 of q. Near a half-integer, g = RN((f - 0.5) + c) (f = y - floor(y), f - 0.5 exact there)
// is within 2^-37.8 of q - floor(y) - 0.5, so the rounding is decided unless that lies within
// 2^-36 of zero, where `undecided` is set and the caller evaluates the double expression.
// Requires finite x and a normal s >= 2^-100.
__device__ __forceinline__ int round_away_quotient(float x, float s, float inv_s, bool &undecided) {
    const float ax = fabsf(x);
    const float y = __fmul_rn(ax, inv_s);
    if (!(y < 7.25f)) return x < 0.0f ? -7 : 7;  // q > 7.24: rounds to 7 or more either way
    const float n = floorf(y);
    const float f = __fsub_rn(y, n);  // exact
    int q = static_cast<int>(n) + (f > 0.5f ? 1 : 0);
    if (fabsf(__fsub_rn(f, 0.5f)) < 0x1p-14f) {
        const float r = __fmaf_rn(-y, s, ax);
        const float c = __fmul_rn(r, inv_s);
        const float g = __fadd_rn(__fsub_rn(f, 0.5f), c);
        if (g > 0x1p-36f) q = static_cast<int>(n) + 1;
        else if (g < -0x1p-36f) q = static_cast<int>(n);
        else undecided = true;
    }
    q = q > 7 ? 7 : q;
    return x < 0.0f ? -q : q;
}

}  // namespace qg
