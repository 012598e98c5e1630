// warp_emu.h -- runs the device arithmetic of quantization_graph_gb300/csrc/qg_device.cuh on the
// host, for CPU tests: 32 std::threads stand for the 32 lanes of one warp and meet at every
// shuffle (a barrier before the exchange, one after), so a lane function that calls
// __shfl_down_sync runs as it does on the GPU. The round-to-nearest intrinsics and bit casts the
// header uses map to their host equivalents (compile with -ffp-contract=off so that every
// plain multiply and add rounds on its own, as --fmad=false makes them on the device).
//
// Include this before qg_device.cuh; link with -pthread. Only the lane-uniform patterns of that
// header are supported: every lane of the warp calls each shuffle.
#pragma once

#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace warp_emu {

struct Warp {
    std::barrier<> bar{32};
    uint64_t slot[32] = {};
};

inline Warp *g_warp = nullptr;
inline thread_local int t_lane = 0;

template <class T>
T shfl_down(unsigned mask, T v, unsigned delta, int width = 32) {
    static_assert(sizeof(T) <= 8, "shuffled values are at most 8 bytes");
    (void)mask;
    Warp &w = *g_warp;
    uint64_t b = 0;
    std::memcpy(&b, &v, sizeof(T));
    w.slot[t_lane] = b;
    w.bar.arrive_and_wait();
    const int base = t_lane / width * width;
    const int src = t_lane + static_cast<int>(delta);
    T r = v;
    if (src < base + width) std::memcpy(&r, &w.slot[src], sizeof(T));
    w.bar.arrive_and_wait();
    return r;
}

template <class T>
T shfl_xor(unsigned mask, T v, int lane_mask, int width = 32) {
    static_assert(sizeof(T) <= 8, "shuffled values are at most 8 bytes");
    (void)mask;
    (void)width;
    Warp &w = *g_warp;
    uint64_t b = 0;
    std::memcpy(&b, &v, sizeof(T));
    w.slot[t_lane] = b;
    w.bar.arrive_and_wait();
    T r;
    std::memcpy(&r, &w.slot[t_lane ^ lane_mask], sizeof(T));
    w.bar.arrive_and_wait();
    return r;
}

template <class T>
T shfl_idx(unsigned mask, T v, int src, int width = 32) {
    static_assert(sizeof(T) <= 8, "shuffled values are at most 8 bytes");
    (void)mask;
    Warp &w = *g_warp;
    uint64_t b = 0;
    std::memcpy(&b, &v, sizeof(T));
    w.slot[t_lane] = b;
    w.bar.arrive_and_wait();
    T r;
    std::memcpy(&r, &w.slot[t_lane / width * width + src % width], sizeof(T));
    w.bar.arrive_and_wait();
    return r;
}

inline void syncwarp() { g_warp->bar.arrive_and_wait(); }

inline unsigned int ballot(unsigned mask, int pred) {
    (void)mask;
    Warp &w = *g_warp;
    w.slot[t_lane] = pred != 0 ? 1u : 0u;
    w.bar.arrive_and_wait();
    unsigned int r = 0;
    for (int l = 0; l < 32; ++l)
        if (w.slot[l]) r |= 1u << l;
    w.bar.arrive_and_wait();
    return r;
}

// fn(lane) on 32 threads as one warp; returns after every lane has finished.
inline void run_warp(const std::function<void(int)> &fn) {
    Warp w;
    g_warp = &w;
    std::vector<std::thread> lanes;
    lanes.reserve(32);
    for (int l = 0; l < 32; ++l)
        lanes.emplace_back([&fn, l] {
            t_lane = l;
            fn(l);
        });
    for (auto &t : lanes) t.join();
    g_warp = nullptr;
}

}  // namespace warp_emu

#define __shfl_down_sync(...) warp_emu::shfl_down(__VA_ARGS__)
#define __shfl_xor_sync(...) warp_emu::shfl_xor(__VA_ARGS__)
#define __shfl_sync(...) warp_emu::shfl_idx(__VA_ARGS__)
#define __syncwarp(...) warp_emu::syncwarp()
#define __ballot_sync(...) warp_emu::ballot(__VA_ARGS__)

inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
inline double __dmul_rn(double a, double b) { return a * b; }
inline double __dadd_rn(double a, double b) { return a + b; }
inline double __dsub_rn(double a, double b) { return a - b; }
inline float __double2float_rn(double d) { return static_cast<float>(d); }
inline float __int_as_float(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}
inline float __uint_as_float(unsigned int u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline unsigned int __float_as_uint(float f) {
    unsigned int u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline int __float_as_int(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}
inline int __popc(unsigned int x) { return __builtin_popcount(x); }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __ll2float_rn(long long x) { return static_cast<float>(x); }
inline int __ffsll(long long x) { return __builtin_ffsll(x); }
inline int __ffs(int x) { return __builtin_ffs(x); }
inline float __log2f(float x) { return std::log2(x); }
inline int __clzll(long long x) { return x == 0 ? 64 : __builtin_clzll(static_cast<unsigned long long>(x)); }
inline double __longlong_as_double(long long x) {
    double d;
    std::memcpy(&d, &x, 8);
    return d;
}
inline float __ll2float_rz(long long x) {
    // round toward zero: the nearest float, stepped back toward zero when it overshoots
    float f = static_cast<float>(x);
    if (static_cast<long double>(f) > static_cast<long double>(x) && x > 0) f = std::nextafter(f, 0.0f);
    if (static_cast<long double>(f) < static_cast<long double>(x) && x < 0) f = std::nextafter(f, 0.0f);
    return f;
}
inline double __ll2double_rn(long long x) { return static_cast<double>(x); }
inline long long __double_as_longlong(double d) {
    long long x;
    std::memcpy(&x, &d, 8);
    return x;
}
using std::isfinite;
using std::max;
using std::min;
