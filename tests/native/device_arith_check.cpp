// device_arith_check.cpp -- the device arithmetic of quantization_graph_gb300/csrc/qg_device.cuh,
// compiled for the host from the same source and run under the warp emulator (warp_emu.h), for
// the CPU tests in tests/test_device_arith.py. Each entry applies one device routine to n records
// of one prepared query, laid out as the GPU kernels lay out their work: half a warp per record,
// two records per pass, for the 16-lane FP32 routines; one lane per record for the residual;
// the integer sums the kernels reduce across a warp (exact in any order) are formed directly.
#include "warp_emu.h"
#include "qg_device.cuh"

using namespace qg;

namespace {

#define QG_EMU_DISPATCH(D_, CALL)                                  \
    switch (D_) {                                                  \
        case 64: { constexpr int kD = 64; CALL; return 0; }        \
        case 128: { constexpr int kD = 128; CALL; return 0; }      \
        case 256: { constexpr int kD = 256; CALL; return 0; }      \
        case 512: { constexpr int kD = 512; CALL; return 0; }      \
        case 1024: { constexpr int kD = 1024; CALL; return 0; }    \
        case 2048: { constexpr int kD = 2048; CALL; return 0; }    \
        default: return -1;                                        \
    }

void put_estimate(const GateOut &g, float alpha, float *o) {
    o[0] = g.lower_bound;
    o[1] = g.short_ip;
    o[2] = alpha;
    o[3] = g.ip_hat;
    o[4] = g.error_bound;
    o[5] = g.valid ? 1.0f : 0.0f;
}

// restore_distance_hw (mode 0) or full_distance_hw (mode 1 where reuse[i], else mode 0)
template <int D>
void distances16(const uint8_t *rec, size_t rs, size_t n, const float *rr, float half, float qn2,
                 const uint8_t *reuse, const float *sip, bool restore_fn, float *out) {
    warp_emu::run_warp([&](int lane) {
        for (size_t base = 0; base < n; base += 2) {
            const size_t i = base + static_cast<size_t>(lane >> 4);
            const size_t ii = i < n ? i : base;
            const uint8_t *r = rec + ii * rs;
            const float ns = ld_f32(r), ls = ld_f32(r + 4);
            const float d = restore_fn ? restore_distance_hw<D>(r + 16, rr, ns, ls, half, qn2, lane & 15)
                                       : full_distance_hw<D>(r + 16, rr, ns, ls, half, qn2, reuse[ii] != 0,
                                                             sip[ii], lane & 15);
            if ((lane & 15) == 0 && i < n) out[i] = d;
        }
    });
}

template <int D>
void full_gate(const uint8_t *msb, size_t ms, const uint8_t *fac, size_t fs, size_t n, const float *rr,
               float qn2, float qn, float half, float eps, float *out6) {
    warp_emu::run_warp([&](int lane) {
        for (size_t base = 0; base < n; base += 2) {
            const size_t i = base + static_cast<size_t>(lane >> 4);
            const size_t ii = i < n ? i : base;
            const float sel = full_gate_selected_hw<D>(msb + ii * ms, rr, lane & 15);
            if ((lane & 15) == 0 && i < n)
                put_estimate(finish_gate_full(sel - half, load_factors(fac + i * fs), qn, qn2, eps), 0.0f, out6 + 6 * i);
        }
    });
}

template <int D>
void encoded_gate(const uint8_t *rec, size_t rs, size_t n, const float *rr, float qn2, float qn, float half, float eps,
                  float *out6) {
    warp_emu::run_warp([&](int lane) {
        for (size_t base = 0; base < n; base += 2) {
            const size_t i = base + static_cast<size_t>(lane >> 4);
            const size_t ii = i < n ? i : base;
            const uint8_t *r = rec + ii * rs;
            const float sip = encoded_short_ip_hw<D>(r + 16, rr, half, lane & 15);
            if ((lane & 15) == 0 && i < n) {
                float alpha;
                const GateOut g = finish_gate_encoded(sip, ld_f32(r), ld_f32(r + 8), qn, qn2, eps, D, &alpha);
                put_estimate(g, alpha, out6 + 6 * i);
            }
        }
    });
}

template <int D>
void residual(const uint8_t *res, size_t rs, size_t n, const float *rr, float qn, const float *long_d, bool fused,
              float *out3) {
    for (size_t i = 0; i < n; ++i) {
        const uint8_t *r = res + i * rs;
        residual_interval_thread<D>(reinterpret_cast<const uint16_t *>(r + 8), r + 8 + 2 * (D / 16), rr, long_d[i],
                                    qn, fused, out3 + 3 * i, out3 + 3 * i + 1, out3 + 3 * i + 2);
    }
}

bool msb_bit(const uint8_t *m, int i) { return ((m[i >> 3] >> (i & 7)) & 1) != 0; }
int nibble(const uint8_t *code, int i) { return (i & 1) ? (code[i >> 1] >> 4) : (code[i >> 1] & 15); }

}  // namespace

extern "C" {

// FP32 restore, mode 0
int emu_restore(int D, const uint8_t *rec, size_t rs, size_t n, const float *rr, float half, float qn2, float *out) {
    QG_EMU_DISPATCH(D, distances16<kD>(rec, rs, n, rr, half, qn2, nullptr, nullptr, true, out))
}

// The Full codec's survivor distance: mode 1 (reuse[i] != 0, short ip sip[i]) or mode 0
int emu_full_distance(int D, const uint8_t *rec, size_t rs, size_t n, const float *rr, float half, float qn2,
                      const uint8_t *reuse, const float *sip, float *out) {
    QG_EMU_DISPATCH(D, distances16<kD>(rec, rs, n, rr, half, qn2, reuse, sip, false, out))
}

// The Full codec's gate; out6: [n x 6] lower bound, short ip, alpha, ip hat, error bound, valid
int emu_full_gate(int D, const uint8_t *msb, size_t ms, const uint8_t *fac, size_t fs, size_t n, const float *rr,
                  float qn2, float qn, float half, float eps, float *out6) {
    QG_EMU_DISPATCH(D, full_gate<kD>(msb, ms, fac, fs, n, rr, qn2, qn, half, eps, out6))
}

// The gate from the encoded record (compute_paper_prune_estimate); out6 as emu_full_gate
int emu_encoded_gate(int D, const uint8_t *rec, size_t rs, size_t n, const float *rr, float qn2, float qn, float half,
                     float eps, float *out6) {
    QG_EMU_DISPATCH(D, encoded_gate<kD>(rec, rs, n, rr, qn2, qn, half, eps, out6))
}

// Residual interval (two-kernel order, or the fused kernel's); out3: [n x 3]
int emu_residual(int D, const uint8_t *res, size_t rs, size_t n, const float *rr, float qn, const float *long_d,
                 int fused, float *out3) {
    QG_EMU_DISPATCH(D, residual<kD>(res, rs, n, rr, qn, long_d, fused != 0, out3))
}

// Int8 / Int4 gate: the integer masked sum, then finish_gate
void emu_int_gate(int D, const uint8_t *msb, size_t ms, const uint8_t *fac, size_t fs, size_t n, const int8_t *codes,
                  float qn2, float qn, float scale, long long csum, float eps, float *out6) {
    for (size_t i = 0; i < n; ++i) {
        int sel = 0;
        for (int d = 0; d < D; ++d) sel += msb_bit(msb + i * ms, d) ? codes[d] : 0;
        put_estimate(finish_gate(sel, load_factors(fac + i * fs), scale, csum, qn, qn2, eps), 0.0f, out6 + 6 * i);
    }
}

// Int8 / Int4 traversal (mode 2): the remaining-3-bit integer dot, then finish_traversal
void emu_traversal(int D, const uint8_t *rec, size_t rs, size_t n, const int8_t *codes, const float *sip, float scale,
                   long long csum, float qn2, float *out) {
    for (size_t i = 0; i < n; ++i) {
        const uint8_t *r = rec + i * rs;
        long long dot = 0;
        for (int d = 0; d < D; ++d) dot += static_cast<long long>(nibble(r + 16, d) & 7) * codes[d];
        out[i] = finish_traversal(ld_f32(r), ld_f32(r + 4), sip[i], dot, scale, csum, qn2);
    }
}

// B1 gate: mismatches of the query's sign bits against the MSB plane, then finish_gate_b1
void emu_b1_gate(int D, const uint8_t *msb, size_t ms, const uint8_t *fac, size_t fs, size_t n, const uint8_t *bits,
                 float short_scale, float error_scale, float alpha, float qn2, float qn, float eps, float *out6) {
    for (size_t i = 0; i < n; ++i) {
        int mism = 0;
        for (int j = 0; j < D / 8; ++j) mism += __popc(static_cast<unsigned>(bits[j] ^ msb[i * ms + j]));
        const GateOut g = finish_gate_b1(mism, load_factors(fac + i * fs), short_scale, error_scale, qn, qn2, eps, D);
        put_estimate(g, g.reached ? alpha : 0.0f, out6 + 6 * i);
    }
}

// B1Main: the 4-bit codes against the query's +-1 signs (r > 0 -> +1), then finish_b1main
void emu_b1main(int D, const uint8_t *rec, size_t rs, size_t n, const float *rr, float qn2, float *out) {
    long long sign_sum = 0;
    for (int d = 0; d < D; ++d) sign_sum += rr[d] > 0.0f ? 1 : -1;
    for (size_t i = 0; i < n; ++i) {
        const uint8_t *r = rec + i * rs;
        int dot = 0;
        for (int d = 0; d < D; ++d) dot += nibble(r + 16, d) * (rr[d] > 0.0f ? 1 : -1);
        out[i] = finish_b1main(ld_f32(r), ld_f32(r + 4), dot, sign_sum, qn2);
    }
}

}  // extern "C"
