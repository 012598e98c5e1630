// code_search.cuh -- fastQuantizeAbs (space_rabitq.h:867-942) for one vector held by one warp:
// the search over the rescale factor t that the encoder runs on every rotated residual. Two
// forms give the same t bit for bit: code_search_warp (all lanes; for the vectors whose double
// sums are exact, which exact_sum_unit decides) and code_search_lane0 (one lane, any vector).
// Shared by the encode kernel and the host harness that runs them under a warp emulator
// (tests/native).
//
// Inputs, in shared memory: keys[D] = the dimensions sorted by (|v| descending, index ascending),
// as (~bits(|v|) << 32 | index), which carry every |v| the search reads; c0[D] the initial codes
// floor(t_start |v| + 1e-5) (at most 2, t_start = 2 / max|v|); mx = max|v|. The rotated values
// themselves are read only before the keys are built (lane0_num_start, exact_sum_unit).
#pragma once

#include <cmath>
#include <cstdint>

#include <cuda_runtime.h>

#include "exact_fp.cuh"

namespace qg {

// Bitonic sort of n (a power of two) 64-bit keys in shared memory by one warp, ascending.
__device__ inline void bitonic_sort_warp(unsigned long long *k, int n, int lane) {
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

// The largest float not above the double 1e-5: a > 1e-5 (double) <=> a > kEpsBelowF.
inline constexpr float kEpsBelowF = 9.99999974737875e-06f;

// floor(RN53(t * a + 1e-5)) for t = th + tl (t a double split into two floats, a >= 0) in FP32:
// ph + pl = th * a exactly, the rest is below 2^-16 and positive, so only the boundary above
// can be crossed; decided unless the value lies within 2^-36 of it (`undecided`).
__device__ __forceinline__ int floor_fma_eps(float th, float tl, float a, bool &undecided) {
    const float ph = __fmul_rn(th, a);
    const float pl = __fmaf_rn(th, a, -ph);
    const float tail = __fadd_rn(__fadd_rn(__fadd_rn(pl, __fmul_rn(tl, a)), kEpsBelowF), 2.5262124e-13f);
    const float n = floorf(ph);
    const float d0 = __fsub_rn(ph, n);  // exact
    int v = static_cast<int>(n);
    if (d0 >= 0.5f) {
        const float g = __fadd_rn(__fsub_rn(d0, 1.0f), tail);  // d0 - 1 exact for d0 >= 0.5
        if (g > 0x1p-36f) v += 1;
        else if (!(g < -0x1p-36f)) undecided = true;
    } else if (!(tail > 0.0f)) {
        undecided = true;  // cannot happen for a >= 0; keeps the decision honest
    }
    return v;
}

// sign of c1 / a1 - c2 / a2 for integers 1 <= c <= 17 and positive normal floats a, exactly:
// the sign of c1 a2 - c2 a1, compared on the significands.
__device__ __forceinline__ int ratio_cmp(int c1, float a1, int c2, float a2) {
    const FloatParts p1 = split_float(a1), p2 = split_float(a2);
    long long l = c1 * p2.m, r = c2 * p1.m;  // < 2^29
    const int d = p2.e - p1.e;                 // l * 2^d against r
    if (d > 30) return 1;
    if (d < -30) return -1;
    if (d > 0) l <<= d;
    else r <<= -d;
    return l < r ? -1 : (l > r ? 1 : 0);
}

// Truncation of a positive normal double to float (relative error below 2^-23), by bits.
__device__ __forceinline__ float approx_float(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const int ex = static_cast<int>((b >> 52) & 0x7FF) - 1023 + 127;
    if (ex <= 0) return 0.0f;
    if (ex >= 255) return __int_as_float(0x7f800000);
    return __uint_as_float((static_cast<uint32_t>(ex) << 23) | static_cast<uint32_t>((b >> 29) & 0x7FFFFFu));
}

// Heads of the seven level lists of fastQuantizeAbs's events: the next admissible dim of each
// level in |v| order. Dim i is an event of level c when |v_i| > 1e-5, c > c0_i and
// (c = c0_i + 1 or c / |v_i| < 17 / max|v|).
struct LevelHead {
    int ptr;
    int id;   // -1 when the level is exhausted
    float a;  // |v_id|
    float t;  // RN24(c / a): orders heads unless two are equal
};

__device__ __forceinline__ void advance_level(LevelHead &h, int c, const unsigned long long *keys,
                                              const unsigned char *c0, int D, float mx) {
    while (h.ptr < D) {
        const unsigned long long k = keys[h.ptr];
        const int i = static_cast<int>(k & 0xFFFFFFFFu);
        const float ai = __uint_as_float(0xFFFFFFFFu - static_cast<uint32_t>(k >> 32));
        const int ci = c0[i];
        if (ai > kEpsBelowF && c > ci && (c == ci + 1 || ratio_cmp(c, ai, 17, mx) < 0)) {
            h.id = i;
            h.a = ai;
            h.t = __fdiv_rn(static_cast<float>(c), ai);
            return;
        }
        ++h.ptr;
    }
    h.id = -1;
}

// event (c, h) before event (b, g): t ascending, ties by dim index; the float ratios decide
// unless equal (rounding is monotone), then the exact comparison
__device__ __forceinline__ bool event_before(int c, const LevelHead &h, int b, const LevelHead &g) {
    if (h.t != g.t) return h.t < g.t;
    const int r = ratio_cmp(c, h.a, b, g.a);
    return r < 0 || (r == 0 && h.id < g.id);
}

// fastQuantizeAbs's search over the rescale factor t (space_rabitq.h:867-942), lane 0: the
// (t, i) events of the seven levels in heap order (t = level / |v_i|, ties by i), running
// num and sqr_den, t at the first maximum of ip = num / sqrt(sqr_den). Event order and the t_end
// cut are decided by ratio comparisons (distinct level / |v| ratios differ by far more than a
// double's rounding, so they order as their doubles do); num stays a double sum. The maximum is
// screened in FP32 on squares, (ip_k / ip_best)^2 = num_k^2 sqr_den_best / (num_best^2 sqr_den_k)
// (within 2^-20 of the float products): an event clearly above the running best (by more than
// 2^-17) becomes the best, one clearly below is skipped, and only events inside that band are
// compared exactly, in double, with the best (whose exact ip is computed once).
// The reference's starting num, sum of (c0_i + 0.5) |v_i| in dimension order in double (one lane).
__device__ inline double lane0_num_start(const float *ru, const unsigned char *c0, int D) {
    double num = 0.0;
    for (int i = 0; i < D; ++i) num += (c0[i] + 0.5) * static_cast<double>(fabsf(ru[i]));
    return num;
}

// num_start: lane0_num_start of the vector.
__device__ inline double code_search_lane0(const unsigned long long *keys, const unsigned char *c0, int D, float mx,
                                           double num_start) {
    long long sd4 = D;  // 4 * sqr_den
    double num = num_start;
    for (int i = 0; i < D; ++i) {
        const int c = c0[i];
        sd4 += 4LL * (c * c + c);
    }
    LevelHead hd[8];
#pragma unroll
    for (int c = 1; c <= 7; ++c) {
        hd[c].ptr = 0;
        advance_level(hd[c], c, keys, c0, D, mx);
    }
    // the best so far: its ip is > 0 for every event, the reference starts from max_ip = 0
    bool have = false, best_exact = false;
    float best_n2 = 0.0f, best_sdf = 1.0f;  // num^2 and 4 sqr_den of the best, in float
    double best_num = 0.0, best_ip = 0.0;
    long long best_sd4 = 0;
    int best_c = 0;
    float best_a = 1.0f;
    constexpr float kHi = 1.0f + 0x1p-17f, kLo = 1.0f - 0x1p-17f;
    for (;;) {
        int bc = 0;
        LevelHead cur{0, -1, 0.0f, 0.0f};
#pragma unroll
        for (int c = 1; c <= 7; ++c)
            if (hd[c].id >= 0 && (bc == 0 || event_before(c, hd[c], bc, cur))) {
                bc = c;
                cur = hd[c];
            }
        if (bc == 0) break;
#pragma unroll
        for (int c = 1; c <= 7; ++c)
            if (c == bc) {
                ++hd[c].ptr;
                advance_level(hd[c], c, keys, c0, D, mx);
            }
        sd4 += 8LL * bc;
        num += static_cast<double>(cur.a);
        const float nf = approx_float(num);
        const float n2 = nf * nf, sdf = __ll2float_rn(sd4);  // sd4 < 2^24: exact
        const float lhs = n2 * best_sdf, rhs = best_n2 * sdf;
        bool take;
        double ip = 0.0;
        bool exact = false;
        if (!have || lhs > rhs * kHi) {
            take = true;
        } else if (lhs < rhs * kLo) {
            take = false;
        } else {
            if (!best_exact) {
                best_ip = best_num / sqrt(static_cast<double>(best_sd4) * 0.25);
                best_exact = true;
            }
            ip = num / sqrt(static_cast<double>(sd4) * 0.25);
            exact = true;
            take = ip > best_ip;
        }
        if (take) {
            have = true;
            best_n2 = n2;
            best_sdf = sdf;
            best_num = num;
            best_sd4 = sd4;
            best_c = bc;
            best_a = cur.a;
            best_exact = exact;
            best_ip = ip;
        }
    }
    return have ? static_cast<double>(best_c) / static_cast<double>(best_a) : 0.0;
}

// ---- fastQuantizeAbs across the warp ----------------------------------------------------
//
// The same search as code_search_lane0, with the event order and the running sums formed in
// parallel; it applies when the double sums are exact (checked per vector), else the caller
// runs code_search_lane0.
//
// Structure used: the dimensions sorted by (|v| descending, index ascending) give positions p;
// the initial code c0 is non-increasing in p (one t_start for every dimension), and the events
// of level c are exactly the dimensions with a_p > 1e-5, c0_p < c and (c0_p = c - 1 or
// c / a_p < 17 / max), a contiguous range [lo_c, hi_c) of positions (each condition holds on a
// prefix or a suffix), ordered by t = c / a_p as p grows. The heap's pop order is the merge of
// the seven ranges by (t, index).
//
// Exactness: every term the reference adds to num ((c0 + 0.5) a for the start, a per event) is
// a multiple of 2^E (E: the lowest set bit over all of them) and every partial sum lies below
// 7.5 sum(a); when that bound is below 2^(E + 53) each partial sum is a double, so the running
// double sum equals the exact sum in any order and prefix sums may replace the sequential loop.
// The sums are then kept as int64 multiples of 2^E (exact, and on the integer pipe: this part's
// FP64 pipe is narrow). sqr_den is an integer (times 1/4) throughout.
//
// Each lane takes a contiguous share of the events (levels one after another, positions within
// a level) and walks it with one pointer per other level (the events of that level ordered
// before the current one, found by binary search once per level segment, then advanced), so
// every event's num, sqr_den and rank (events before it in pop order) are known. Each lane keeps
// its best event under an FP32 screen of ip^2 (relative error below 2^-20); events within 2^-17
// of the running best are ordered by the exact integer cross products (ip_sq_order), and only
// near-ties within 2^-33 compute ip = num / sqrt(sqr_den) in double as the reference does. The
// lanes' bests are then compared exactly, and the first (smallest rank) of the largest is the
// reference's t.

// exponent of the lowest set bit of a positive finite float
__device__ __forceinline__ int low_bit_exp(float a) {
    const FloatParts p = split_float(a);
    return p.e + __ffsll(p.m) - 1;
}

// (c1 / a1, i1) < (c2 / a2, i2) exactly: c1 a2 against c2 a1 as exact two-float products
// (small integer times float: the FMA error term is exact), ties by index
__device__ __forceinline__ bool ev_before(int c1, float a1, int i1, int c2, float a2, int i2) {
    const float x = __fmul_rn(static_cast<float>(c1), a2), xl = __fmaf_rn(static_cast<float>(c1), a2, -x);
    const float y = __fmul_rn(static_cast<float>(c2), a1), yl = __fmaf_rn(static_cast<float>(c2), a1, -y);
    if (x != y) return x < y;
    if (xl != yl) return xl < yl;
    return i1 < i2;
}

// the sorted keys hold ~bits(|v|) in the high word and the dimension in the low word
__device__ __forceinline__ float key_a(unsigned long long k) {
    return __uint_as_float(0xFFFFFFFFu - static_cast<uint32_t>(k >> 32));
}
__device__ __forceinline__ int key_id(unsigned long long k) { return static_cast<int>(k & 0xFFFFFFFFu); }

struct SortedView {
    const unsigned long long *keys;
    __device__ __forceinline__ int id(int p) const { return key_id(keys[p]); }
    __device__ __forceinline__ float a(int p) const { return key_a(keys[p]); }
};

// a (>= 0, a multiple of 2^E) as an integer count of 2^E: exact (E is at most a's lowest set bit)
__device__ __forceinline__ long long units(float a, int E) {
    const FloatParts p = split_float(a);
    const int sh = p.e - E;
    return sh >= 0 ? (p.m << sh) : (p.m >> -sh);
}

// 2^e as a float, for -126 <= e <= 127; as a double, for -1022 <= e <= 1023
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }
__device__ __forceinline__ double pow2d(int e) { return __longlong_as_double(static_cast<long long>(e + 1023) << 52); }

// The exactness test above for the vector ru[0, D) (all lanes; the same answer in each): E = the
// lowest set bit over the nonzero |v| minus one, and whether 7.5 sum|v| < 2^(E + 53) (sum in FP32
// with a margin far above its rounding). Every double sum the encoder forms from (c + 0.5) |v|,
// |v| or |v| / 2 is then exact in any order.
__device__ inline bool exact_sum_unit(const float *ru, int D, int lane, int *E_out) {
    int emin = 1 << 30;
    float tot = 0.0f;
    for (int i = lane; i < D; i += 32) {
        const float ai = fabsf(ru[i]);
        if (ai > 0.0f) emin = min(emin, low_bit_exp(ai) - 1);
        tot += ai;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        emin = min(emin, __shfl_xor_sync(0xffffffffu, emin, o));
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    *E_out = emin;
    if (emin < -120 || emin + 53 > 120 || !(tot < 0x1p40f)) return false;
    return 7.5f * tot * 1.001f < pow2f(emin + 53);
}

// Order of num1^2 / sd1 against num2^2 / sd2 (the squared ips of two events; num < 2^53 and
// 0 < sd < 2^24 integers): +1 or -1 when they differ by more than 2^-33 relative, else 0. The nums
// keep their top 40 bits (exact below 2^40; truncation error under 2^-36 relative when the
// smaller keeps at least 2^36, else 0 is returned), and the cross products a1^2 sd2 and a2^2 sd1
// (below 2^104) are compared exactly in 128 bits with a 2^-32 margin.
__device__ __forceinline__ int ip_sq_order(long long num1, long long sd1, long long num2, long long sd2) {
    const unsigned long long n1 = static_cast<unsigned long long>(num1), n2 = static_cast<unsigned long long>(num2);
    const unsigned long long big = n1 > n2 ? n1 : n2;
    const int s = max(0, 64 - __clzll(static_cast<long long>(big)) - 40);
    const unsigned long long a1 = n1 >> s, a2 = n2 >> s;
    if (s > 0 && (a1 < (1ull << 36) || a2 < (1ull << 36))) return 0;
    const unsigned __int128 x = static_cast<unsigned __int128>(a1) * a1 * static_cast<unsigned long long>(sd2);
    const unsigned __int128 y = static_cast<unsigned __int128>(a2) * a2 * static_cast<unsigned long long>(sd1);
    if (x > y + (y >> 32)) return 1;
    if (y > x + (x >> 32)) return -1;
    return 0;
}

// sum of a over sorted positions [0, p), in units of 2^E: the prefix of p's 16-position block
// plus the rest of it
__device__ __forceinline__ long long prefix_a(const SortedView &sv, const long long *blk, int p, int E) {
    long long s = blk[p >> 4];
    for (int q = p & ~15; q < p; ++q) s += units(sv.a(q), E);
    return s;
}

// c / a < T exactly (c a small integer, a > 0, T > 0 finite): c against the exact product
// T a = h + l (FMA error term); c - h is exact wherever the comparison is close (Sterbenz)
__device__ __forceinline__ bool t_below(int c, float a, float T) {
    const float h = __fmul_rn(T, a);
    const float l = __fmaf_rn(T, a, -h);
    return __fsub_rn(static_cast<float>(c), h) < l;
}

// Sign of num1^2 sd2 - num2^2 sd1 (the order of two events' ip^2 = 4 num^2 / sd), exactly:
// num < 2^53 and 0 < sd < 2^20 keep both products below 2^126.
__device__ __forceinline__ unsigned __int128 sq_times(long long num, long long sd) {
    const unsigned long long n = static_cast<unsigned long long>(num);
    return static_cast<unsigned __int128>(n) * n * static_cast<unsigned long long>(sd);
}

// The state of the search after every event with t < T (T = +inf: after all events): num (units
// of 2^E), 4 sqr_den, the number of events (rank of the next) and each level's count.
struct CutState {
    long long num, sd4;
    int rank;
    int cnt[8];  // [1..7]
};

__device__ __forceinline__ void cut_state(const SortedView &sv, const int (&lo_c)[8], const int (&hi_c)[8],
                                          const long long (&base)[8], const long long *blk, int E, float T, bool all,
                                          long long num0, long long sd40, CutState &st) {
    long long acc = 0, w = 0;
    int r = 0;
#pragma unroll
    for (int c = 1; c <= 7; ++c) {
        int lo = lo_c[c], hi = hi_c[c];
        if (all) {
            lo = hi;
        } else {
            while (lo < hi) {
                const int m = (lo + hi) >> 1;
                if (t_below(c, sv.a(m), T)) lo = m + 1;
                else hi = m;
            }
        }
        const int n = lo - lo_c[c];
        st.cnt[c] = n;
        acc += prefix_a(sv, blk, lo, E) - base[c];
        w += static_cast<long long>(c) * n;
        r += n;
    }
    st.num = num0 + acc;
    st.sd4 = sd40 + 8 * w;
    st.rank = r;
}

__device__ __forceinline__ void shfl_state(CutState &d, const CutState &s, int src) {
    d.num = __shfl_sync(0xffffffffu, s.num, src);
    d.sd4 = __shfl_sync(0xffffffffu, s.sd4, src);
    d.rank = __shfl_sync(0xffffffffu, s.rank, src);
#pragma unroll
    for (int c = 1; c <= 7; ++c) d.cnt[c] = __shfl_sync(0xffffffffu, s.cnt[c], src);
}

// index of the n-th (from 0) set bit of mask (n < popc(mask))
__device__ __forceinline__ int nth_set_bit(unsigned int mask, int n) {
    for (int k = 0; k < n; ++k) mask &= mask - 1u;
    return __ffs(static_cast<int>(mask)) - 1;
}

// The warp's best achieved (num, sd4) by exact ip^2 order (any one of equal values).
__device__ __forceinline__ void warp_max_ip(long long &num, long long &sd4) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long on = __shfl_xor_sync(0xffffffffu, num, o);
        const long long os = __shfl_xor_sync(0xffffffffu, sd4, o);
        if (sq_times(on, sd4) > sq_times(num, os)) {
            num = on;
            sd4 = os;
        }
    }
}

// Call only when exact_sum_unit returned true (E its unit); blk holds D / 16 + 1 int64.
//
// Branch and bound over t. An interval [A, B) of t holds the events with A <= t < B; the states at
// its ends come from cut_state, and the last event inside achieves exactly num(B), sd4(B). Every
// event inside has |v| <= level / A, which bounds its ip^2 (see the drop test); an interval whose
// bound is below the best achieved ip^2 by more than 2^-36 (far above the double rounding of the
// reference's ip) cannot hold the maximum and is dropped. Starting from [0, inf), each round splits
// the surviving intervals geometrically among the 32 lanes and drops again; the survivors of the
// last round are walked event by event in (t, index) order, a lane each.
__device__ inline void code_search_warp(const unsigned long long *keys, const unsigned char *c0, int D, float mx,
                                        long long *blk, int E, int lane, double *best_t_out) {
    const SortedView sv{keys};
    // the starting num (in units of 2^E; (c + 0.5) a = (2c + 1) (a / 2), a / 2 a whole number of
    // units) and 4 sqr_den, over the sorted positions (integer sums: any order)
    long long num0 = 0;
    long long sd40 = 0;
    for (int p = lane; p < D; p += 32) {
        const unsigned long long k = keys[p];
        const int c = c0[key_id(k)];
        num0 += static_cast<long long>(2 * c + 1) * (units(key_a(k), E) >> 1);
        sd40 += 4LL * (c * c + c);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        num0 += __shfl_xor_sync(0xffffffffu, num0, o);
        sd40 += __shfl_xor_sync(0xffffffffu, sd40, o);
    }
    sd40 += D;
    const float unit_f = pow2f(E);
    const double unit_d = pow2d(E);

    // level ranges: lanes 0-7 count c0 >= j, lanes 8-14 count c / a < 17 / max (c = lane - 7),
    // lane 15 counts a > 1e-5; each predicate holds on a prefix of the positions
    int cnt = 0;
    if (lane < 16) {
        int lo = 0, hi = D;  // first position where the predicate fails
        while (lo < hi) {
            const int m = (lo + hi) >> 1;
            const float am = sv.a(m);
            bool pr;
            if (lane < 8) pr = c0[sv.id(m)] >= lane;
            else if (lane < 15) pr = am > kEpsBelowF && ratio_cmp(lane - 7, am, 17, mx) < 0;
            else pr = am > kEpsBelowF;
            if (pr) lo = m + 1;
            else hi = m;
        }
        cnt = lo;
    }
    int lo_c[8], hi_c[8];
    const int r = __shfl_sync(0xffffffffu, cnt, 15);
    lo_c[0] = hi_c[0] = 0;
#pragma unroll
    for (int c = 1; c <= 7; ++c) {
        const int ge_c = __shfl_sync(0xffffffffu, cnt, c);
        const int ge_prev = c == 1 ? D : __shfl_sync(0xffffffffu, cnt, c - 1);
        const int q = __shfl_sync(0xffffffffu, cnt, 7 + c);
        lo_c[c] = ge_c;
        int h = min(max(ge_prev, q), r);
        hi_c[c] = h > ge_c ? h : ge_c;
    }
    // prefix sums of a over positions in blocks of 16 (exact, units of 2^E): blk[b] = sum over [0, 16 b)
    const int nblk = D >> 4;
    for (int b = lane; b < nblk; b += 32) {
        long long sb = 0;
        for (int q = b << 4; q < (b << 4) + 16; ++q) sb += units(sv.a(q), E);
        blk[b + 1] = sb;
    }
    __syncwarp();
    if (lane == 0) {
        blk[0] = 0;
        for (int b = 1; b <= nblk; ++b) blk[b] += blk[b - 1];
    }
    __syncwarp();
    long long base[8];  // prefix at each level's first position
    {
        const long long mine = lane >= 1 && lane <= 7 ? prefix_a(sv, blk, lo_c[lane], E) : 0;
        base[0] = 0;
#pragma unroll
        for (int c = 1; c <= 7; ++c) base[c] = __shfl_sync(0xffffffffu, mine, c);
    }
    // spacing of the cuts: events lie in [1 / max, t_top]
    const float t_lo = __frcp_rn(mx);
    float t_top = t_lo;
#pragma unroll
    for (int c = 1; c <= 7; ++c)
        if (hi_c[c] > lo_c[c]) t_top = fmaxf(t_top, __fdiv_rn(static_cast<float>(c), sv.a(hi_c[c] - 1)));

    // the lane's interval [A, B): A = 0 or B = +inf flagged; S, E the states at its ends
    float A = 0.0f, B = 0.0f;
    bool a_zero = true, b_inf = true;
    CutState S, Ee;
    S.num = num0;
    S.sd4 = sd40;
    S.rank = 0;
#pragma unroll
    for (int c = 1; c <= 7; ++c) S.cnt[c] = 0;
    cut_state(sv, lo_c, hi_c, base, blk, E, 0.0f, true, num0, sd40, Ee);
    unsigned int surv = 1u;  // lanes holding a surviving interval: lane 0 holds [0, inf)
    long long lb_num = Ee.num, lb_sd4 = Ee.sd4;  // the best achieved so far: the last event
    for (int round = 0; round < 4; ++round) {
        const int K = __popc(surv), L = 32 / K;
        const int i = lane / L, m = lane - i * L;
        const bool act = i < K;
        const int src = nth_set_bit(surv, act ? i : 0);
        const float sA = __shfl_sync(0xffffffffu, A, src), sB = __shfl_sync(0xffffffffu, B, src);
        const bool sAz = __shfl_sync(0xffffffffu, a_zero ? 1 : 0, src) != 0;
        const bool sBi = __shfl_sync(0xffffffffu, b_inf ? 1 : 0, src) != 0;
        CutState sS, sE;
        shfl_state(sS, S, src);
        shfl_state(sE, Ee, src);
        // this lane's piece m of L: end cut geometric between the survivor's ends
        const float ga = sAz ? t_lo : sA, gb = sBi ? t_top * 1.0001f : sB;
        float T = ga * exp2f(__log2f(gb / ga) * static_cast<float>(m + 1) / static_cast<float>(L));
        if (!sAz) T = fmaxf(T, sA);
        if (!sBi) T = fminf(T, sB);
        const bool last = !act || m == L - 1;
        CutState nE;
        if (!last) cut_state(sv, lo_c, hi_c, base, blk, E, T, false, num0, sd40, nE);
        else nE = sE;
        float nB = last ? sB : T;
        bool nBi = last ? sBi : false;
        // start: the previous piece's end, or the survivor's start
        CutState nS;
        shfl_state(nS, nE, (lane + 31) & 31);
        float nA = __shfl_sync(0xffffffffu, nB, (lane + 31) & 31);
        bool nAz = false;
        if (m == 0) {
            nS = sS;
            nA = sA;
            nAz = sAz;
        }
        const bool nonempty = act && nE.rank > nS.rank;
        // the best achieved: the pieces' last events
        long long cn = nonempty ? nE.num : lb_num, cs = nonempty ? nE.sd4 : lb_sd4;
        if (sq_times(cn, lb_sd4) > sq_times(lb_num, cs)) {
            lb_num = cn;
            lb_sd4 = cs;
        }
        warp_max_ip(lb_num, lb_sd4);
        // drop the pieces whose bound is below the best by the margin
        bool keep = false;
        int n_in = 0;
        if (nonempty) {
            // every event inside has a <= c / A: after events of levels summing to x, num <=
            // min(n0 + k x, nE) (k = 1 / (A 2^E)) and sd4 = s0 + 8 x; (n0 + k x)^2 / (s0 + 8 x) is
            // quasi-convex in x, so the bound is its value at x = 1 or where n0 + k x reaches nE.
            // Double evaluation (relative error below 2^-48) against a 2^-36 margin.
            const double a_eff = nAz ? 1.0 / static_cast<double>(mx) * (1.0 - 0x1p-40) : static_cast<double>(nA);
            const double kk = 1.0 / (a_eff * unit_d);
            const double n0 = __ll2double_rn(nS.num), ne = __ll2double_rn(nE.num), s0 = __ll2double_rn(nS.sd4);
            const double b1 = (n0 + kk) * (n0 + kk) / (s0 + 8.0);
            const double xc = fmax(1.0, (ne - n0) / kk);
            const double b2 = ne * ne / (s0 + 8.0 * xc);
            const double lbn = __ll2double_rn(lb_num);
            const double lbd = lbn * lbn / __ll2double_rn(lb_sd4);
            keep = !(fmax(fmin(b1, ne * ne / (s0 + 8.0)), b2) * (1.0 + 0x1p-36) < lbd);
            n_in = nE.rank - nS.rank;
        }
        surv = __ballot_sync(0xffffffffu, keep);
        A = nA;
        B = nB;
        a_zero = nAz;
        b_inf = nBi;
        S = nS;
        Ee = nE;
        int most = keep ? n_in : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, o));
        if (most <= 24 || L == 1) break;
    }

    // walk the surviving intervals: a 7-way merge of the levels' events in (t, index) order; each
    // lane keeps its best under an FP32 screen of ip^2 (relative error below 2^-20): events within
    // 2^-17 of the best are ordered by the exact cross products, and only near-ties within 2^-33
    // compute ip = num / sqrt(sqr_den) in double as the reference does
    constexpr float kHi = 1.0f + 0x1p-17f, kLo = 1.0f - 0x1p-17f;
    bool have = false, best_exact = false;
    float best_n2 = 0.0f, best_sdf = 1.0f;
    long long best_num = 0, best_sd4 = 1;
    double best_ip = -1.0;
    int best_rank = 0x7FFFFFFF, best_c = 0;
    float best_a = 1.0f;
    const bool walk = (surv >> lane) & 1u;
    int pk[8], ek[8], ik[8];
    float ak[8];
#pragma unroll
    for (int c = 1; c <= 7; ++c) {
        pk[c] = lo_c[c] + S.cnt[c];
        ek[c] = walk ? lo_c[c] + Ee.cnt[c] : pk[c];
        ak[c] = 0.0f;
        ik[c] = 0;
        if (pk[c] < ek[c]) {
            const unsigned long long k0 = keys[pk[c]];
            ak[c] = key_a(k0);
            ik[c] = key_id(k0);
        }
    }
    long long num = S.num, sd4 = S.sd4;
    const int n_walk = walk ? Ee.rank - S.rank : 0;
    for (int k = 0; k < n_walk; ++k) {
        int cm = 0, im = 0;
        float am = 0.0f;
#pragma unroll
        for (int c = 1; c <= 7; ++c)
            if (pk[c] < ek[c] && (cm == 0 || ev_before(c, ak[c], ik[c], cm, am, im))) {
                cm = c;
                am = ak[c];
                im = ik[c];
            }
#pragma unroll
        for (int c = 1; c <= 7; ++c)
            if (c == cm) {
                ++pk[c];
                if (pk[c] < ek[c]) {
                    const unsigned long long kn = keys[pk[c]];
                    ak[c] = key_a(kn);
                    ik[c] = key_id(kn);
                }
            }
        num += units(am, E);
        sd4 += 8LL * cm;
        const int ev_rank = S.rank + k;
        const float nf = __ll2float_rz(num) * unit_f;  // truncated: relative error below 2^-23
        const float n2 = nf * nf, sdf = __ll2float_rn(sd4);  // sd4 < 2^24: exact
        const float lhs = n2 * best_sdf, rhs = best_n2 * sdf;
        bool take;
        double ip = 0.0;
        bool exact = false;
        if (!have || lhs > rhs * kHi) {
            take = true;
        } else if (lhs < rhs * kLo) {
            take = false;
        } else if (const int o = ip_sq_order(num, sd4, best_num, best_sd4); o != 0) {
            take = o > 0;  // the doubles order as the exact values do
        } else {
            if (!best_exact) {
                best_ip = (__ll2double_rn(best_num) * unit_d) / sqrt(static_cast<double>(best_sd4) * 0.25);
                best_exact = true;
            }
            ip = (__ll2double_rn(num) * unit_d) / sqrt(static_cast<double>(sd4) * 0.25);
            exact = true;
            take = ip > best_ip || (ip == best_ip && ev_rank < best_rank);
        }
        if (take) {
            have = true;
            best_n2 = n2;
            best_sdf = sdf;
            best_num = num;
            best_sd4 = sd4;
            best_rank = ev_rank;
            best_c = cm;
            best_a = am;
            best_exact = exact;
            best_ip = ip;
        }
    }
    if (have && !best_exact)
        best_ip = (__ll2double_rn(best_num) * unit_d) / sqrt(static_cast<double>(best_sd4) * 0.25);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double oip = __shfl_xor_sync(0xffffffffu, best_ip, o);
        const int orank = __shfl_xor_sync(0xffffffffu, best_rank, o);
        const int oc = __shfl_xor_sync(0xffffffffu, best_c, o);
        const float oa = __shfl_xor_sync(0xffffffffu, best_a, o);
        if (oip > best_ip || (oip == best_ip && orank < best_rank)) {
            best_ip = oip;
            best_rank = orank;
            best_c = oc;
            best_a = oa;
        }
    }
    *best_t_out = best_c > 0 ? static_cast<double>(best_c) / static_cast<double>(best_a) : 0.0;
}

}  // namespace qg
