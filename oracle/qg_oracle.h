/*
 * qg_oracle.h -- CPU restatement of the Ours-DiskANN query path (test infrastructure).
 *
 * This library is the ORACLE: it exists only so that tests, the smoke check and the
 * CPU-baseline leg of bench.py can check and time the CUDA path. Nothing in the shipped
 * library (libqgraph_gb300.so) links, loads or calls it.
 *
 * It restates, in plain C++, the x86-64 AVX-512 build of the reference
 * (Ours/core/hnswlib/space_rabitq.h built with `-O3 -march=native`, as
 * experiments/02_diskann_fair/build.rs:22-36 does): the lane order of every
 * floating-point reduction and every FMA contraction that GCC applies there is written
 * out explicitly, so the results are bit-identical on x86 and on aarch64 when this file is
 * compiled with -ffp-contract=off. Each function cites the reference lines it follows.
 *
 * Pinning: tests/golden/ holds vectors produced by the reference itself (compiled here
 * from its own sources by oracle/Makefile into oracle/_ref/); tests check this oracle
 * against them bit for bit.
 */
#ifndef QG_ORACLE_H
#define QG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field order as RabitqPaperEstimate (rabitq_bridge.cpp:21-28). */
typedef struct {
    float lower_bound;
    float short_ip;
    float alpha;
    float ip_hat;
    float error_bound;
    uint8_t valid;
} qgo_paper_estimate;

/* Same field order as RabitqDistanceInterval (rabitq_bridge.cpp:15-19). */
typedef struct {
    float estimate;
    float lower_bound;
    float upper_bound;
} qgo_interval;

/* Counters of OursPaperSearchStats (ours_diskann.rs:1056-1075) that the parity
 * check verify_search_parity (ours_diskann.rs:1988-2066) compares. */
typedef struct {
    uint64_t visited_nodes;
    uint64_t distance_computations;
    uint64_t hops;
    uint64_t paper_checked;
    uint64_t paper_would_prune;
    uint64_t paper_not_pruned;
    uint64_t paper_full_saved;
    uint64_t paper_msb_kernel_calls;
    uint64_t paper_remaining_kernel_calls;
} qgo_search_stats;

typedef struct qgo_space qgo_space;
typedef struct qgo_prepared qgo_prepared;

/* ---- space (space_rabitq.h:2836-2936); formal config 4-bit residual, block 16, mse, fp16 ---- */
qgo_space *qgo_space_new(size_t dim, uint32_t seed);
void qgo_space_delete(qgo_space *space);
int qgo_space_set_center(qgo_space *space, const float *center);
size_t qgo_code_dim(const qgo_space *space);
size_t qgo_full_bytes(const qgo_space *space);
size_t qgo_compact_bytes(const qgo_space *space);
size_t qgo_residual_bytes(const qgo_space *space);
size_t qgo_msb_bytes(const qgo_space *space);
void qgo_space_signs(const qgo_space *space, float *out);
void qgo_space_rotated_center(const qgo_space *space, float *out);
float qgo_space_center_norm_sqr(const qgo_space *space);
void qgo_rotate(const qgo_space *space, const float *raw, float *out);

/* ---- encode (space_rabitq.h:5845-6029, 4364-4392) ---- */
int qgo_encode_full(const qgo_space *space, const float *raw, uint8_t *full_out);
void qgo_copy_compact(const qgo_space *space, const uint8_t *full, uint8_t *compact_out);
void qgo_copy_residual(const qgo_space *space, const uint8_t *full, uint8_t *residual_out);
/* Encode n rows into compact + residual stores; threads <= 0 means all cores. */
int qgo_encode_batch(const qgo_space *space, const float *raw, size_t n, uint8_t *compact,
                     uint8_t *residual, int threads);
int qgo_export_sidecar(const qgo_space *space, const uint8_t *compact, size_t n, size_t stride,
                       uint8_t *msb_out, void *factors_out);
float qgo_symmetric_distance(const qgo_space *space, const uint8_t *lhs, const uint8_t *rhs);

/* ---- query preparation (space_rabitq.h:3429-3706), INT8 codec, or INT4 after
 * qgo_space_set_query_codec(space, 2) ---- */
int qgo_space_set_query_codec(qgo_space *space, int codec);
void qgo_prepared_export_b1(const qgo_prepared *prepared, uint8_t *bits, float *scalars, int64_t *signed_sum);
qgo_prepared *qgo_prepared_new(const qgo_space *space);
void qgo_prepared_delete(qgo_prepared *prepared);
int qgo_prepare(const qgo_space *space, const float *query, qgo_prepared *prepared);
/* scalars: [query_norm_sqr, query_norm, half_sum_residual, int8_scale] */
void qgo_prepared_export(const qgo_prepared *prepared, float *rotated_residual, int8_t *codes,
                         float *scalars, int64_t *code_sum);
uint64_t qgo_dither_seed(const float *query, size_t dim, uint32_t centroid_id);
void qgo_dither_draws(uint64_t seed, size_t count, double *out);

/* ---- batched kernels (rabitq_bridge.cpp:747-778, 885-970, 972-1017) ---- */
void qgo_gate_batch(const qgo_space *space, const qgo_prepared *prepared, const uint32_t *ids,
                    size_t count, const uint8_t *msb_base, size_t msb_stride,
                    const void *factors_base, size_t factors_stride, float epsilon0,
                    qgo_paper_estimate *out);
void qgo_distance_batch(const qgo_space *space, const qgo_prepared *prepared,
                        const uint32_t *ids, const uint8_t *modes, size_t count,
                        const uint8_t *records, size_t record_stride, const float *short_ips,
                        float *out);
void qgo_residual_batch(const qgo_space *space, const qgo_prepared *prepared,
                        const uint32_t *ids, size_t count, const uint8_t *records,
                        size_t record_stride, const uint8_t *residual, size_t residual_stride,
                        const float *long_distances, qgo_interval *out);
/* compute_paper_prune_estimate (space_rabitq.h:3926-3959): the gate from the encoded record */
void qgo_gate_encoded_batch(const qgo_space *space, const qgo_prepared *prepared, const uint32_t *ids,
                            size_t count, const uint8_t *records, size_t record_stride, float epsilon0,
                            qgo_paper_estimate *out);
/* compute_full_residual_distance_intervals_batch_by_id (space_rabitq.h:5557-5778) */
void qgo_full_residual_batch(const qgo_space *space, const qgo_prepared *prepared,
                             const uint32_t *ids, size_t count, const uint8_t *records,
                             size_t record_stride, const uint8_t *residual, size_t residual_stride,
                             qgo_interval *out);

/* ---- search loop (ours_diskann.rs:1539-1986), batch of queries, OpenMP over queries ----
 * adjacency: fixed stride `edge_stride`, degrees[i] valid entries per row.
 * Returns 0 on success, -1 on an out-of-range neighbour (the reference errors out). */
typedef struct {
    size_t k;
    size_t l_value;
    size_t beam_width;
    float epsilon0;
    size_t rerank_candidates;
    size_t early_stop_hops;
    int kth_stop;
    int codec; /* 3 Int8, 2 Int4 (quantized traversal), 1 B1 (survivors by the FP32 restore),
                  4 B1Main (no gate: every fresh neighbour by the 4-bit x 1-bit distance),
                  0 Full (FP32 gate; survivors by the remaining bits with the gate's short ip);
                  5 FullStaged and 6 FullRerankScalar run as Full; 7 FullScalar (a Rust-side
                  switch over a Full prepared query) takes distance mode 3, which computes mode 1 */
    int fused_int_rerank; /* Int8 / Int4: rerank by the fused restore + residual kernel
                             (RABITQ_ENABLE_FUSED_INT_RERANK, ours_diskann.rs:1166-1172, 1831-1848) */
} qgo_search_params;

int qgo_search_batch(const qgo_space *space, const float *queries, size_t nq,
                     const qgo_search_params *params, const uint8_t *records,
                     size_t record_stride, const uint8_t *residual, size_t residual_stride,
                     const uint8_t *msb, size_t msb_stride, const void *factors,
                     size_t factor_stride, const uint32_t *degrees, const uint32_t *edges,
                     size_t edge_stride, size_t total_points, size_t base_points,
                     uint32_t *ids_out, float *dists_out, qgo_search_stats *stats_out,
                     int threads);

/* Kernel table so the same loop can run over another implementation of the three
 * batched kernels (the reference bridge, in oracle/ref_probe.cpp). */
typedef struct {
    void *ctx;
    const void *(*prepare)(void *ctx, const float *query);
    float (*distance)(void *ctx, const void *prepared, uint32_t id);
    void (*gate)(void *ctx, const void *prepared, const uint32_t *ids, size_t n, float eps,
                 qgo_paper_estimate *out);
    void (*distance_batch)(void *ctx, const void *prepared, const uint32_t *ids,
                           const uint8_t *modes, size_t n, const float *short_ips, float *out);
    void (*residual_batch)(void *ctx, const void *prepared, const uint32_t *ids, size_t n,
                           const float *long_d, qgo_interval *out);
    /* 4-bit data x 1-bit query distance (B1Main; query_distance_b1, space_rabitq.h:3741-3753) */
    float (*distance_b1)(void *ctx, const void *prepared, uint32_t id);
    /* fused FP32 restore + residual (rabitq_full_residual_distance_batch, rabitq_bridge.cpp:1044-1084) */
    void (*full_residual_batch)(void *ctx, const void *prepared, const uint32_t *ids, size_t n,
                                qgo_interval *out);
} qgo_kernel_table;

int qgo_search_one_with(const qgo_kernel_table *kt, const float *query,
                        const qgo_search_params *params, const uint32_t *degrees,
                        const uint32_t *edges, size_t edge_stride, size_t total_points,
                        size_t base_points, uint32_t *ids_out, float *dists_out,
                        qgo_search_stats *stats_out);

/* ---- Vamana graph build (rabitq_build_vamana_graph, rabitq_bridge.cpp:224-303) ----
 * Bulk insertion in batches from node 0, refinement passes, grouped back-edges, all over the
 * symmetric 4-bit estimator. edges: `edge_stride` slots per node, degrees[i] valid. evals_out
 * (may be NULL) counts the distances evaluated, like VamanaIndex::distance_evaluations().
 * Returns 0 on success, -1 on bad arguments or an out-of-range neighbour. */
int qgo_build_vamana(const qgo_space *space, const uint8_t *compact, size_t n, size_t stride,
                     size_t r, size_t l_build, float alpha, size_t beam, size_t batch,
                     size_t refine, size_t cap, size_t stop_hops, uint32_t *degrees,
                     uint32_t *edges, size_t edge_stride, uint64_t *evals_out, int threads);

/* ---- exact ground truth (FP64 brute force, query_coarse_codec_test.cpp:29-36 style) ---- */
void qgo_exact_knn(const float *base, size_t n, const float *queries, size_t nq, size_t dim,
                   size_t k, uint32_t *ids_out, double *dists_out, int threads);

#ifdef __cplusplus
}
#endif

#endif
