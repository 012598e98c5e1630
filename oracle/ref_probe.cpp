// ref_probe.cpp -- test infrastructure. Compiled only together with the reference's own
// experiments/02_diskann_fair/native/rabitq_bridge.cpp (built from the reference sources in
// place by oracle/Makefile, into oracle/_ref/). It exposes the reference's prepared-query
// internals (space_rabitq.h:98-154) for golden vectors and drives the restated Rust search
// loop (qgo_search_one_with, oracle/qg_oracle.cpp) over the reference's own batched bridge
// kernels, so that golden search results come from the reference's kernels.
#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include <omp.h>

#include "Ours/core/hnswlib/space_rabitq.h"
#include "qg_oracle.h"

extern "C" {

struct RabitqPaperEstimate;
struct RabitqDistanceInterval;

const void *rabitq_prepare_query(const void *space, const float *query);
float rabitq_query_distance(const void *space, const void *prepared, const void *encoded);
float rabitq_query_distance_b1(const void *space, const void *prepared, const void *encoded);
bool rabitq_paper_estimate_batch_sidecar(const void *space, const void *prepared,
                                         const uint32_t *ids, size_t count,
                                         const uint8_t *msb_base, size_t msb_stride,
                                         const void *factors_base, size_t factors_stride,
                                         float epsilon0, RabitqPaperEstimate *out);
bool rabitq_query_distance_batch(const void *space, const void *prepared, const uint32_t *ids,
                                 const uint8_t *modes, size_t count, const void *encoded_base,
                                 size_t encoded_stride, const float *short_ips,
                                 float *out_distances);
bool rabitq_residual_distance_batch(const void *space, const void *prepared,
                                    const uint32_t *ids, size_t count, const void *encoded_base,
                                    size_t encoded_stride, const void *residual_base,
                                    size_t residual_stride, const float *long_distances,
                                    RabitqDistanceInterval *out);
bool rabitq_full_residual_distance_batch(const void *space, const void *prepared,
                                         const uint32_t *ids, size_t count, const void *encoded_base,
                                         size_t encoded_stride, const void *residual_base,
                                         size_t residual_stride, RabitqDistanceInterval *out);

// scalars: [query_norm_sqr, query_norm, half_sum_residual, int8 (or int4) scale]
void qgref_prepared_export(const void *prepared, size_t code_dim, float *rotated_residual,
                           int8_t *codes, float *scalars, int64_t *code_sum) {
    const auto &p = *static_cast<const hnswlib::RaBitQSpace::PreparedQuery *>(prepared);
    const auto &q = p.centroid_queries[0];
    const bool int4 = p.query_coarse_codec == hnswlib::QueryCoarseCodec::Int4;
    const auto &ic = int4 ? q.int4_code : q.int8_code;
    if (rotated_residual) std::memcpy(rotated_residual, q.rotated_residual.data(), code_dim * 4);
    if (codes && ic.size() >= code_dim) std::memcpy(codes, ic.data(), code_dim);
    if (scalars) {
        scalars[0] = q.query_norm_sqr;
        scalars[1] = q.query_norm;
        scalars[2] = q.half_sum_residual;
        scalars[3] = int4 ? q.int4_scale : q.int8_scale;
    }
    if (code_sum) *code_sum = int4 ? q.int4_code_sum : q.int8_code_sum;
}

// The B1 prepared fields (space_rabitq.h:3493-3523): sign bits [D/8], {short scale, error
// scale, alpha}, signed sum.
void qgref_prepared_export_b1(const void *prepared, size_t code_dim, uint8_t *bits, float *scalars,
                              int64_t *signed_sum) {
    const auto &q = static_cast<const hnswlib::RaBitQSpace::PreparedQuery *>(prepared)->centroid_queries[0];
    if (bits && q.b1_code.size() >= (code_dim + 7) / 8) std::memcpy(bits, q.b1_code.data(), (code_dim + 7) / 8);
    if (scalars) {
        scalars[0] = q.b1_short_scale;
        scalars[1] = q.b1_error_scale;
        scalars[2] = q.b1_alpha;
    }
    if (signed_sum) *signed_sum = q.b1_signed_sum;
}

void qgref_rotate(const void *space, const float *raw, float *out) {
    static_cast<const hnswlib::RaBitQSpace *>(space)->rotate(raw, out);
}

// The reference's RaBitQSpace::saveState (space_rabitq.h:3139-3198) into a buffer; returns the
// byte count (0 when it does not fit or fails).
size_t qgref_save_state(const void *space, uint8_t *out, size_t cap) {
    try {
        std::ostringstream os(std::ios::binary);
        static_cast<const hnswlib::RaBitQSpace *>(space)->saveState(os);
        const std::string bytes = os.str();
        if (bytes.size() > cap) return 0;
        std::memcpy(out, bytes.data(), bytes.size());
        return bytes.size();
    } catch (...) {
        return 0;
    }
}

// RaBitQSpace::loadState (space_rabitq.h:3200-3345) from a buffer into an existing space;
// returns 1 on success, 0 when the reference rejects the state.
int qgref_load_state(void *space, const uint8_t *in, size_t n) {
    try {
        std::istringstream is(std::string(reinterpret_cast<const char *>(in), n), std::ios::binary);
        static_cast<hnswlib::RaBitQSpace *>(space)->loadState(is);
        return 1;
    } catch (...) {
        return 0;
    }
}

}  // extern "C"

namespace {

struct RefCtx {
    const void *space;
    const uint8_t *records;
    size_t record_stride;
    const uint8_t *residual;
    size_t residual_stride;
    const uint8_t *msb;
    size_t msb_stride;
    const void *factors;
    size_t factor_stride;
};

const void *rk_prepare(void *ctx, const float *q) {
    return rabitq_prepare_query(static_cast<RefCtx *>(ctx)->space, q);
}
float rk_distance(void *ctx, const void *p, uint32_t id) {
    auto *c = static_cast<RefCtx *>(ctx);
    return rabitq_query_distance(c->space, p, c->records + static_cast<size_t>(id) * c->record_stride);
}
void rk_gate(void *ctx, const void *p, const uint32_t *ids, size_t n, float eps,
             qgo_paper_estimate *out) {
    auto *c = static_cast<RefCtx *>(ctx);
    rabitq_paper_estimate_batch_sidecar(c->space, p, ids, n, c->msb, c->msb_stride, c->factors,
                                        c->factor_stride, eps,
                                        reinterpret_cast<RabitqPaperEstimate *>(out));
}
void rk_dist(void *ctx, const void *p, const uint32_t *ids, const uint8_t *modes, size_t n,
             const float *sips, float *out) {
    auto *c = static_cast<RefCtx *>(ctx);
    rabitq_query_distance_batch(c->space, p, ids, modes, n, c->records, c->record_stride, sips, out);
}
float rk_distance_b1(void *ctx, const void *p, uint32_t id) {
    auto *c = static_cast<RefCtx *>(ctx);
    return rabitq_query_distance_b1(c->space, p, c->records + static_cast<size_t>(id) * c->record_stride);
}
void rk_res(void *ctx, const void *p, const uint32_t *ids, size_t n, const float *ld,
            qgo_interval *out) {
    auto *c = static_cast<RefCtx *>(ctx);
    rabitq_residual_distance_batch(c->space, p, ids, n, c->records, c->record_stride, c->residual,
                                   c->residual_stride, ld,
                                   reinterpret_cast<RabitqDistanceInterval *>(out));
}
void rk_full_res(void *ctx, const void *p, const uint32_t *ids, size_t n, qgo_interval *out) {
    auto *c = static_cast<RefCtx *>(ctx);
    rabitq_full_residual_distance_batch(c->space, p, ids, n, c->records, c->record_stride, c->residual,
                                        c->residual_stride, reinterpret_cast<RabitqDistanceInterval *>(out));
}

}  // namespace

extern "C" int qgref_search_batch(const void *space, size_t dim, const float *queries, size_t nq,
                                  const qgo_search_params *params, const uint8_t *records,
                                  size_t record_stride, const uint8_t *residual,
                                  size_t residual_stride, const uint8_t *msb, size_t msb_stride,
                                  const void *factors, size_t factor_stride,
                                  const uint32_t *degrees, const uint32_t *edges,
                                  size_t edge_stride, size_t total_points, size_t base_points,
                                  uint32_t *ids_out, float *dists_out,
                                  qgo_search_stats *stats_out, int threads) {
    int status = 0;
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
    {
        RefCtx ctx{space, records, record_stride, residual, residual_stride,
                   msb, msb_stride, factors, factor_stride};
        qgo_kernel_table kt{&ctx, rk_prepare, rk_distance, rk_gate, rk_dist, rk_res, rk_distance_b1, rk_full_res};
#pragma omp for schedule(dynamic, 1)
        for (long long q = 0; q < static_cast<long long>(nq); ++q) {
            const size_t qi = static_cast<size_t>(q);
            const int rc = qgo_search_one_with(&kt, queries + qi * dim, params, degrees, edges,
                                               edge_stride, total_points, base_points,
                                               ids_out + qi * params->k, dists_out + qi * params->k,
                                               stats_out ? stats_out + qi : nullptr);
            if (rc != 0) status = rc;
        }
    }
    return status;
}
