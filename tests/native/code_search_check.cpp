// code_search_check.cpp -- fastQuantizeAbs's search over t (space_rabitq.h:867-942) three ways on
// the host, for tests/test_code_search.py: the warp-parallel form and the one-lane form of the
// encoder (quantization_graph_gb300/csrc/code_search.cuh, compiled unchanged and run under the
// warp emulator), and the reference's own algorithm with its min-heap, restated here in plain
// C++ (the FMA contraction of its t * a + eps as the reference build makes it).
#include <algorithm>
#include <queue>
#include <vector>

#include "warp_emu.h"
#include "code_search.cuh"

namespace {

double heap_search(const std::vector<float> &a, const std::vector<int> &c0, double max_o) {
    const double t_end = 17.0 / max_o;
    const size_t D = a.size();
    std::vector<int> cur(c0);
    double sqr_den = static_cast<double>(D) * 0.25, num = 0.0;
    for (size_t i = 0; i < D; ++i) {
        sqr_den += cur[i] * cur[i] + cur[i];
        num = std::fma(cur[i] + 0.5, static_cast<double>(a[i]), num);
    }
    std::priority_queue<std::pair<double, size_t>, std::vector<std::pair<double, size_t>>,
                        std::greater<std::pair<double, size_t>>> next;
    for (size_t i = 0; i < D; ++i)
        if (a[i] > 1e-5) next.emplace(static_cast<double>(cur[i] + 1) / a[i], i);
    double best_t = 0.0, max_ip = 0.0;
    while (!next.empty()) {
        const double t = next.top().first;
        const size_t id = next.top().second;
        next.pop();
        const int code = ++cur[id];
        sqr_den += 2.0 * code;
        num += a[id];
        const double ip = num / std::sqrt(sqr_den);
        if (ip > max_ip) {
            max_ip = ip;
            best_t = t;
        }
        if (code < 7) {
            const double ct = static_cast<double>(code + 1) / a[id];
            if (ct < t_end) next.emplace(ct, id);
        }
    }
    return best_t;
}

}  // namespace

// ru: D rotated values. Writes the best t of the reference heap, of the one-lane search and of
// the warp search, and whether the warp search applied (its exactness check passed).
extern "C" int qcs_run(int D, const float *ru, double *t_heap, double *t_lane0, double *t_warp, int *warp_ok) {
    std::vector<float> a(D);
    float mx = 0.0f;
    for (int i = 0; i < D; ++i) {
        a[i] = std::fabs(ru[i]);
        mx = std::max(mx, a[i]);
    }
    const double max_o = mx;
    if (!(max_o > 1e-5)) return -1;
    const double t_start = 2.0 / max_o;
    std::vector<int> c0(D);
    std::vector<unsigned char> c0b(D);
    std::vector<unsigned long long> keys(D);
    for (int i = 0; i < D; ++i) {
        c0[i] = std::min(static_cast<int>(std::fma(t_start, static_cast<double>(a[i]), 1e-5)), 7);
        c0b[i] = static_cast<unsigned char>(c0[i]);
        unsigned int bits;
        std::memcpy(&bits, &a[i], 4);
        keys[i] = (static_cast<unsigned long long>(0xFFFFFFFFu - bits) << 32) | static_cast<unsigned int>(i);
    }
    std::sort(keys.begin(), keys.end());
    *t_heap = heap_search(a, c0, max_o);
    std::vector<long long> blk(D / 16 + 2);
    double t0 = 0.0, tw = 0.0;
    bool ok = false;
    std::vector<float> ruv(ru, ru + D);
    warp_emu::run_warp([&](int lane) {
        if (lane == 0)
            t0 = qg::code_search_lane0(keys.data(), c0b.data(), D, mx, qg::lane0_num_start(ruv.data(), c0b.data(), D));
        int E = 0;
        const bool exact = qg::exact_sum_unit(ruv.data(), D, lane, &E);
        double t = 0.0;
        if (exact) qg::code_search_warp(keys.data(), c0b.data(), D, mx, blk.data(), E, lane, &t);
        if (lane == 0) {
            tw = t;
            ok = exact;
        }
    });
    *t_lane0 = t0;
    *t_warp = tw;
    *warp_ok = ok ? 1 : 0;
    return 0;
}
