// Host build of the float-float symmetric estimator (quantization_graph_gb300/csrc/sym_ff.cuh)
// for the CPU tests: compares its fast path with the double-precision expression.
#include <cstddef>
#include <cstdint>

#include "sym_ff.cuh"

extern "C" {

// Pair i: lhs (n2_l[i], ls_l[i]), rhs (n2_r[i], ls_r[i]), centred code product s[i].
// out_ff / out_f64: the fast result (0 when it declined) and the double expression;
// returns the number of pairs where the fast path answered with a different float.
int64_t sym_ff_compare(const float *n2_l, const float *ls_l, const float *n2_r, const float *ls_r,
                       const int32_t *s, size_t n, float *out_ff, float *out_f64, uint8_t *taken) {
    int64_t bad = 0;
    for (size_t i = 0; i < n; ++i) {
        const qg::SymFactors l = qg::sym_factors(n2_l[i], ls_l[i], 0);
        const qg::SymFactors r = qg::sym_factors(n2_r[i], ls_r[i], 0);
        bool ok = false;
        const float f = qg::sym_distance_ff(l, r, s[i], ok);
        const float d = qg::sym_distance_f64(l, r, s[i]);
        out_ff[i] = f;
        out_f64[i] = d;
        taken[i] = ok ? 1 : 0;
        if (ok && qg::qg_float_to_bits(f) != qg::qg_float_to_bits(d)) ++bad;
    }
    return bad;
}
}
