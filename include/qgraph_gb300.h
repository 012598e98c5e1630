/*
 * qgraph_gb300.h -- C ABI of libqgraph_gb300.so, the GB300 (sm_103a) implementation of the
 * Ours-DiskANN query path of Coconutstree/quantization_graph.
 *
 * Two groups of entry points:
 *
 *  1. rabitq_*  -- the 37 symbols of the reference bridge
 *     experiments/02_diskann_fair/native/rabitq_bridge.cpp, with the same signatures, the
 *     same caller-owned host buffers, the same record layouts and the same error sentinels
 *     (false / NULL / +inf / {0,..,valid=0}; batch calls fill failed items with sentinels and
 *     still return true). The Rust caller declares them at
 *     experiments/02_diskann_fair/src/ours_diskann.rs:45-242. Compute runs on the GPU; each
 *     call stages its host operands through device memory.
 *
 *  2. qg_*      -- batched device entry points that the reference has no counterpart for:
 *     a device-resident index, a persistent batched beam search over thousands of queries,
 *     batched GPU encode and query preparation. They take device pointers and a
 *     cudaStream_t (passed as void*), return a qg_status, and never allocate inside a
 *     stream-ordered call except where documented.
 *
 * All structs are plain C; no torch or CUDA types appear in the signatures.
 */
#ifndef QGRAPH_GB300_H
#define QGRAPH_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- shared POD structs (rabitq_bridge.cpp:15-40) ---------------- */

/* rabitq_bridge.cpp:15-19 */
typedef struct RabitqDistanceInterval {
    float estimate;
    float lower_bound;
    float upper_bound;
} RabitqDistanceInterval;

/* rabitq_bridge.cpp:21-28 */
typedef struct RabitqPaperEstimate {
    float lower_bound;
    float short_ip;
    float alpha;
    float ip_hat;
    float error_bound;
    uint8_t valid;
} RabitqPaperEstimate;

/* rabitq_bridge.cpp:30-36 == hnswlib::PaperPruneFactors<float> (hnswlib.h:298-305), 20 bytes */
typedef struct RabitqPaperFactors {
    float norm_sqr;
    float data_norm;
    float cross_scale;
    float error_cross_scale;
    uint8_t valid;
} RabitqPaperFactors;

/* ---------------- 1. reference bridge ABI ---------------- */

/* rabitq_bridge.cpp:42-74. residual_bits must be 4 and block 16 (the formal config). */
void *rabitq_space_new(size_t dim, uint32_t seed, size_t centroid_count, size_t residual_bits,
                       size_t residual_block_size, bool residual_mse, bool residual_fp16);
/* rabitq_bridge.cpp:76-78 */
void rabitq_space_delete(void *space);
/* rabitq_bridge.cpp:80-87 */
bool rabitq_space_set_center(void *space, const float *center);
/* rabitq_bridge.cpp:89-99; only centroid_count == 1 is supported (false otherwise). */
bool rabitq_space_set_centroids(void *space, const float *centroids, size_t centroid_count);
/* rabitq_bridge.cpp:101-172 (k-means on the host; not on the query path) */
bool rabitq_train_centroids(const float *data, size_t count, size_t dim, size_t k,
                            size_t sample_count, uint32_t seed, int iters, float *out);
/* rabitq_bridge.cpp:174-193 */
size_t rabitq_full_record_bytes(const void *space);
size_t rabitq_compact_record_bytes(const void *space);
size_t rabitq_residual_record_bytes(const void *space);
size_t rabitq_residual_block_size(const void *space);
size_t rabitq_residual_bits(const void *space);
/* rabitq_bridge.cpp:195-202 (GPU encode of one row) */
bool rabitq_encode_full(const void *space, const float *raw, void *encoded_out);
/* rabitq_bridge.cpp:204-212 */
bool rabitq_copy_compact(const void *space, const void *full_encoded, void *compact_out);
/* rabitq_bridge.cpp:214-222 */
bool rabitq_copy_residual_record(const void *space, const void *full_encoded, void *residual_out);
/* The rotation's sign vector (code_dim floats, +-1/sqrt(D)): read it, or replace it as
 * RaBitQSpace::loadState does with stored signs (space_rabitq.h:3318-3336; a set centre is
 * re-rotated). Used to save and load the EXRBTQ31 space state. */
bool qg_space_signs(const void *space, float *out);
bool qg_space_set_signs(void *space, const float *signs);
/* rabitq_bridge.cpp:224-303: the reference's Vamana build (bulk insertion in batches,
 * refinement passes, grouped back-edges, robust_prune_4bit over the symmetric 4-bit estimator),
 * run on the GPU; the same graph as the reference for the same arguments. Host buffers; also
 * exports the paper sidecar like the reference. distance_evaluations_out counts the distances
 * this implementation evaluated (its prune evaluates them eagerly, so the count differs from
 * the reference's lazy count). Returns false on bad arguments, R > 64 or beam * R > 1024. */
bool rabitq_build_vamana_graph(void *space, const void *compact_records_in, size_t record_count,
                               size_t compact_stride, size_t r, size_t l_build, float alpha,
                               size_t beam_width, size_t batch_size, size_t refine_passes,
                               size_t prune_candidate_cap, size_t build_early_stop_hops,
                               uint32_t *degrees_out, uint32_t *edges_out, size_t edge_stride,
                               uint8_t *paper_msb_out, void *paper_factors_out,
                               size_t *paper_msb_stride_out, size_t *paper_factor_bytes_out,
                               uint64_t *distance_evaluations_out);
/* rabitq_bridge.cpp:305-315 */
size_t rabitq_paper_msb_code_bytes(const void *space);
size_t rabitq_paper_factor_bytes(void);
/* rabitq_bridge.cpp:317-343 */
bool rabitq_export_paper_sidecar(const void *space, const void *compact_records_in,
                                 size_t record_count, size_t compact_stride, uint8_t *msb_out,
                                 void *factors_out);
/* rabitq_bridge.cpp:345-353 */
float rabitq_symmetric_distance(const void *space, const void *lhs, const void *rhs);
/* rabitq_bridge.cpp:355-362. The prepared query is thread-local to the calling thread and
 * valid until that thread's next prepare call, as in the reference (space_rabitq.h:3700). */
const void *rabitq_prepare_query(const void *space, const float *query);
/* rabitq_bridge.cpp:364-370. Codec ids: Full=0 B1=1 Int4=2 Int8=3 B1Main=4 FullStaged=5
 * FullRerankScalar=6 (space_rabitq.h:36-44). All are implemented; as in the reference, the id is
 * stored as an 8-bit enum and every id other than 1-4 behaves as Full (FullRerankScalar also
 * reranks in the per-record residual order). A new space starts with Full. B1Main prepared codes
 * are +-1 bytes with the sign sum in the code-sum slot; the Full codecs prepare no codes (the
 * rotated residual and the scalars only, scale 1).
 * With B1 the prepared codes hold the sign bits, the scale slot the 1-bit short scale and the
 * code-sum slot the error scale (low word) and alpha (high word). */
void rabitq_set_query_coarse_codec(void *space, int codec);
/* rabitq_bridge.cpp:372-378 (no-op, as in the reference) */
void rabitq_release_query(const void *space, const void *prepared);
/* rabitq_bridge.cpp:380-387 (full FP32 4-bit restore) */
float rabitq_query_distance(const void *space, const void *prepared, const void *encoded);
/* rabitq_bridge.cpp:389-396 / 398-423: the 4-bit x 1-bit distance (query_distance_b1,
 * space_rabitq.h:3741-3753) for a B1Main or B1 prepared query (both prepare the query's signs);
 * +inf otherwise (the batch form fills +inf and returns true). The reference reads a sign vector
 * that the other codecs never prepare, so its value there depends on earlier calls. */
float rabitq_query_distance_b1(const void *space, const void *prepared, const void *encoded);
bool rabitq_query_distance_b1_batch(const void *space, const void *prepared, const uint32_t *ids,
                                    size_t count, const void *encoded_base, size_t encoded_stride,
                                    float *out_distances);
/* rabitq_bridge.cpp:425-446: gate from the compact record (computes its MSB plane) */
RabitqPaperEstimate rabitq_paper_estimate(const void *space, const void *prepared,
                                          const void *encoded, float epsilon0);
/* rabitq_bridge.cpp:448-470 */
RabitqPaperEstimate rabitq_paper_estimate_sidecar(const void *space, const void *prepared,
                                                  const uint8_t *msb_code, const void *factors,
                                                  float epsilon0);
/* rabitq_bridge.cpp:472-498 */
RabitqPaperEstimate rabitq_paper_estimate_codec(const void *space, const void *prepared,
                                                const void *encoded, const uint8_t *msb_code,
                                                const void *factors, float epsilon0);
/* rabitq_bridge.cpp:500-580 */
bool rabitq_paper_estimate_codec_batch(const void *space, const void *prepared,
                                       const uint32_t *ids, size_t count,
                                       const void *encoded_base, size_t encoded_stride,
                                       const uint8_t *msb_base, size_t msb_stride,
                                       const void *factors_base, size_t factors_stride,
                                       float epsilon0, RabitqPaperEstimate *out);
/* rabitq_bridge.cpp:582-593: Full-codec reuse (mode 1): the remaining bits with the given FP32
 * short ip (query_distance_with_paper_msb, space_rabitq.h:3961-3966) */
float rabitq_query_distance_with_paper(const void *space, const void *prepared,
                                       const void *encoded, float short_ip);
/* rabitq_bridge.cpp:595-607 (mode 2: INT8 x remaining 3 bits) */
float rabitq_query_distance_with_quantized_paper(const void *space, const void *prepared,
                                                 const void *encoded, float short_ip);
/* rabitq_bridge.cpp:609-627: needs the full record's inline residual; the formal layout keeps
 * residuals external, so this returns {long,long,long}; use the _from_record form. */
RabitqDistanceInterval rabitq_residual_distance(const void *space, const void *prepared,
                                                const void *encoded, float long_distance);
/* rabitq_bridge.cpp:644-663: the per-record residual (space_rabitq.h:1723-1734), whose products
 * take the fused kernel's order */
RabitqDistanceInterval rabitq_residual_distance_from_record(const void *space,
                                                            const void *prepared,
                                                            const void *encoded,
                                                            const void *residual_record,
                                                            float long_distance);
/* rabitq_bridge.cpp:650-679 */
bool rabitq_paper_estimate_batch(const void *space, const void *prepared, const uint32_t *ids,
                                 size_t count, const void *encoded_base, size_t encoded_stride,
                                 float epsilon0, RabitqPaperEstimate *out);
/* rabitq_bridge.cpp:681-883 (the hot-loop gate, ours_diskann.rs:1692-1703) */
bool rabitq_paper_estimate_batch_sidecar(const void *space, const void *prepared,
                                         const uint32_t *ids, size_t count,
                                         const uint8_t *msb_base, size_t msb_stride,
                                         const void *factors_base, size_t factors_stride,
                                         float epsilon0, RabitqPaperEstimate *out);
/* rabitq_bridge.cpp:885-970 (hot-loop flush and rerank restore; modes 0, 1 / 3 and 2) */
bool rabitq_query_distance_batch(const void *space, const void *prepared, const uint32_t *ids,
                                 const uint8_t *modes, size_t count, const void *encoded_base,
                                 size_t encoded_stride, const float *short_ips,
                                 float *out_distances);
/* rabitq_bridge.cpp:972-1042 (rerank residual correction; the per-record order for
 * FullRerankScalar) */
bool rabitq_residual_distance_batch(const void *space, const void *prepared, const uint32_t *ids,
                                    size_t count, const void *encoded_base,
                                    size_t encoded_stride, const void *residual_base,
                                    size_t residual_stride, const float *long_distances,
                                    RabitqDistanceInterval *out);
/* rabitq_bridge.cpp:1044-1084 (fused restore + residual; its residual contracts the other
 * product of each code pair, space_rabitq.h:5700-5743, so it can differ by one ulp from
 * rabitq_query_distance_batch mode 0 followed by rabitq_residual_distance_batch) */
bool rabitq_full_residual_distance_batch(const void *space, const void *prepared,
                                         const uint32_t *ids, size_t count,
                                         const void *encoded_base, size_t encoded_stride,
                                         const void *residual_base, size_t residual_stride,
                                         RabitqDistanceInterval *out);

/* ---------------- 2. batched GPU entry points (no reference counterpart) ---------------- */

typedef enum qg_status {
    QG_OK = 0,
    QG_ERR_INVALID = 1,       /* bad argument (null pointer, size, unsupported config) */
    QG_ERR_CUDA = 2,          /* a CUDA runtime call failed */
    QG_ERR_OOM = 3,           /* device allocation failed */
    QG_ERR_GRAPH = 4,         /* adjacency holds a neighbour id >= total points */
    QG_ERR_TIMEOUT = 5,       /* a query exceeded its hop cap (device watchdog) */
    QG_ERR_UNSUPPORTED = 6    /* code dim or degree outside what the kernels are built for */
} qg_status;

typedef struct qg_index qg_index;

/* Search knobs of search_ours_paper_active (ours_diskann.rs:1174-1227; defaults in
 * diskann_runner.rs:374-388 and args.rs:56-75). */
typedef struct qg_search_params {
    int k;                  /* results per query (per-query array overrides) */
    int l_value;            /* search list size L (per-query array overrides) */
    int beam_width;         /* frontier size per hop (reference default 1) */
    float epsilon0;         /* paper-prune epsilon (reference 1.9) */
    int rerank_candidates;  /* residual rerank set size (reference 100) */
    int early_stop_hops;    /* stall stop (0 = off) */
    int kth_stop;           /* k-th bound stop (0 = off) */
    int fused_int_rerank;   /* Int8 / Int4: rerank by the fused restore + residual kernel's
                               arithmetic (RABITQ_ENABLE_FUSED_INT_RERANK, ours_diskann.rs:1166-1172,
                               1831-1848; 0 = the two-kernel default) */
} qg_search_params;

/* The counters that verify_search_parity compares (ours_diskann.rs:1988-2066). */
typedef struct qg_search_stats {
    uint64_t visited_nodes;
    uint64_t distance_computations;
    uint64_t hops;
    uint64_t paper_checked;
    uint64_t paper_would_prune;
    uint64_t paper_not_pruned;
    uint64_t paper_full_saved;
    uint64_t paper_msb_kernel_calls;
    uint64_t paper_remaining_kernel_calls;
} qg_search_stats;

/* Last error message of the calling thread (static storage, never NULL). */
const char *qg_last_error(void);
/* Number of SMs of the current device and the library's build arch, for diagnostics. */
int qg_device_sm_count(void);

/* Upload an index given in the reference's host layouts (OursStore, ours_diskann.rs:522-686:
 * compact records, residual records, MSB sidecar, 20-byte factors; adjacency with fixed stride
 * and per-node degrees, diskann .graph.bin order). The device copy is re-laid out as
 * structure-of-arrays rows with 16-byte alignment. `base_points` rows carry payloads;
 * total_points >= base_points counts graph nodes (frozen start points appended last). */
int qg_index_upload_host(const void *space, const void *compact, size_t compact_stride,
                         const void *residual, size_t residual_stride, const uint8_t *msb,
                         size_t msb_stride, const void *factors, size_t factor_stride,
                         const uint32_t *degrees, const uint32_t *edges, size_t edge_stride,
                         size_t base_points, size_t total_points, qg_index **out);
/* Same, with every array already in device memory. */
int qg_index_upload_device(const void *space, const void *d_compact, size_t compact_stride,
                           const void *d_residual, size_t residual_stride, const uint8_t *d_msb,
                           size_t msb_stride, const void *d_factors, size_t factor_stride,
                           const uint32_t *d_degrees, const uint32_t *d_edges,
                           size_t edge_stride, size_t base_points, size_t total_points,
                           void *stream, qg_index **out);
void qg_index_free(qg_index *index);
/* No counterpart in the reference. A second handle on src's resident payload and adjacency (no
 * copy) with its own search scratch, so that searches through different handles may run at the
 * same time on different streams (searches through one handle must not overlap). The payload is
 * freed with the last handle; launch and tile settings are copied, later changes are per handle. */
int qg_index_share(const qg_index *src, qg_index **out);
/* Device bytes held by the index (payload + adjacency + search scratch). */
size_t qg_index_device_bytes(const qg_index *index);

/* Batched beam search with the paper-prune gate, INT8 traversal and residual rerank; all
 * pointers are device pointers. queries [nq x dim] f32; d_k / d_l optional per-query int
 * arrays (NULL = params->k / params->l_value). Outputs: ids [nq x k_max] (UINT32_MAX pad),
 * dists [nq x k_max] (+inf pad), stats [nq] (optional). k_max = params->k when d_k is NULL,
 * else the caller's row stride passed in k_stride. Stream-ordered; returns after launch. */
int qg_search_batch(qg_index *index, const float *d_queries, size_t nq,
                    const qg_search_params *params, const int *d_k, const int *d_l,
                    size_t k_stride, uint32_t *d_ids, float *d_dists, qg_search_stats *d_stats,
                    void *stream);
/* qg_search_batch that also records, per query, the expanded nodes in hop order into
 * d_expanded [nq x expanded_cap] (UINT32_MAX padding); the graph builder uses them as
 * search-based prune candidates (the Vamana pass). */
int qg_search_batch_ex(qg_index *index, const float *d_queries, size_t nq,
                       const qg_search_params *params, const int *d_k, const int *d_l,
                       size_t k_stride, uint32_t *d_ids, float *d_dists, qg_search_stats *d_stats,
                       uint32_t *d_expanded, size_t expanded_cap, void *stream);
/* No counterpart in the reference. qg_search_batch for callers that cannot allocate device
 * memory -- code running while a CUDA graph is captured, or a serving process whose device
 * memory is fixed at start-up and may not call cudaMalloc on the request path. It allocates
 * nothing: its scratch (prepared queries, visited rows, counter, status) is one file-scope
 * device array of QG_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until exit.
 * The index must already exist; queries and outputs are the caller's. Limits: the prepared
 * queries (nq x (5*D + 24) bytes) and at least one visited row (a bit per graph node, n_total / 8
 * bytes) must fit the array, else QG_ERR_INVALID with the reason in qg_last_error(). All calls
 * share the array: calls whose GPU work overlaps race, so serialise them. The first call on a
 * device looks up the array's address (make it before any stream capture). The call itself does
 * not synchronise: failed queries (bad neighbour ids) return UINT32_MAX ids, and
 * qg_search_noalloc_status reads the kernels' status word back. The visited rows limit the warps
 * searching at once to about (64 MiB - prepared queries) / (n_total / 8): ~530 at 1M nodes;
 * an index needs n_total / 8 <= ~64 MiB (about 500M nodes). */
#define QG_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
int qg_search_batch_noalloc(qg_index *index, const float *d_queries, size_t nq,
                            const qg_search_params *params, const int *d_k, const int *d_l,
                            size_t k_stride, uint32_t *d_ids, float *d_dists,
                            qg_search_stats *d_stats, void *stream);
/* No counterpart in the reference. The status of the last qg_search_batch_noalloc call on the
 * current device, read from the no-alloc scratch array on `stream` (synchronises it): QG_OK,
 * QG_ERR_GRAPH (a neighbour id outside the graph; those queries returned no results),
 * QG_ERR_TIMEOUT (the hop cap ended a search) or QG_ERR_INVALID (a per-query L above the
 * call's pool capacity max(params->l_value, k) was clamped), as qg_search_status reports them
 * for qg_search_batch. */
int qg_search_noalloc_status(void *stream);
/* Learned early termination (no counterpart in the reference: its search stops at fixed L or
 * by the kth / stall heuristics, ours_diskann.rs:1784-1809). A network 8 -> 64 -> 64 -> 1 with
 * BF16 weights reads 8 search-state features every `every` hops (never before min_hops). As a
 * stop classifier (kind 0) the query stops expanding when sigmoid(output) > threshold; as a hop
 * budget (kind 1, after Li et al., "Improving Approximate Nearest Neighbor Search through Learned
 * Adaptive Early Termination", SIGMOD 2020) the output predicts log(hops the query needs) and the
 * query stops once its hops reach budget_scale * exp(output). Either way it then reranks its
 * current pool. Weight layout
 * (matrices input-major, W[in][out]): W1[8][64] b1[64] W2[64][64] b2[64] w3[64] b3
 * (QG_MLP_PARAMS values); d_norm = mean[8], inv_std[8] of the features. */
#define QG_MLP_PARAMS 4801
typedef struct qg_stop_model {
    const uint16_t *d_weights;
    const float *d_norm;
    float threshold;     /* kind 0: stop when sigmoid(output) > threshold */
    int every;
    int min_hops;
    int kind;            /* 0: stop classifier; 1: hop budget (output = log of the hops needed) */
    float budget_scale;  /* kind 1: stop once hops >= budget_scale * exp(output) */
    int predict_once;    /* kind 1: predict at the first checkpoint only (else at every one) */
} qg_stop_model;

/* Training traces: at every `every`-th hop, the 8 features and, as the label, how many of the
 * `truth_k` ids of d_truth (for example the final result of the full fixed-L search) the first
 * max(rerank, k) pool entries already contain; at most `cap` rows per query, d_counts[q] rows
 * written. */
typedef struct qg_trace_request {
    const uint32_t *d_truth;
    int truth_k;
    int every;
    int cap;
    float *d_features;
    float *d_labels;
    int *d_counts;
} qg_trace_request;

/* qg_search_batch with an optional stop model and/or trace request (either may be NULL). */
int qg_search_batch_learned(qg_index *index, const float *d_queries, size_t nq,
                            const qg_search_params *params, const int *d_k, const int *d_l,
                            size_t k_stride, uint32_t *d_ids, float *d_dists,
                            qg_search_stats *d_stats, const qg_stop_model *model,
                            const qg_trace_request *trace, void *stream);
/* Network training kernels: outputs of n feature rows; the loss and its gradient w.r.t. the
 * BF16 weights (FP32 accumulation; d_grad and d_loss are overwritten) -- binary cross-entropy
 * with logits for the stop classifier (qg_mlp_backward), half the squared error of the output
 * for the hop budget (qg_mlp_backward_mse), both means over the rows; one Adam step on the FP32
 * master weights that also refreshes the BF16 copy (step counts from 1). */
int qg_mlp_forward(const float *d_x, size_t n, const float *d_norm, const uint16_t *d_weights,
                   float *d_logits, void *stream);
int qg_mlp_backward(const float *d_x, const float *d_y, size_t n, const float *d_norm,
                    const uint16_t *d_weights, float *d_grad, float *d_loss, void *stream);
int qg_mlp_backward_mse(const float *d_x, const float *d_y, size_t n, const float *d_norm,
                        const uint16_t *d_weights, float *d_grad, float *d_loss, void *stream);
int qg_mlp_adam(float *d_master, uint16_t *d_weights, const float *d_grad, float *d_m, float *d_v,
                float lr, float beta1, float beta2, float eps, int step, void *stream);
/* Launch shape of the persistent search kernel: warps per block (2, 4 or 8) and an upper bound
 * on resident blocks per SM; 0 restores the automatic choice. Used by the autotuner. */
int qg_index_set_launch(qg_index *index, int warps_per_block, int blocks_per_sm);
/* The widest search block, in warps, of the kernel this index searches with (its code dim and
 * tile shape): qg_index_set_launch's warps_per_block (at most 8) is capped to it. */
int qg_index_max_block_warps(const qg_index *index);
/* Tile shape of the search's gate and traversal loops for the Int8 / Int4 codecs at code dims
 * 1024 and 2048 (how many neighbours' rows each lane keeps in flight): 0 (the default) 16 MSB
 * chunks per lane and 2 code rows (8 at D = 1024); 1: 8 chunks; 2: 32 chunks; 3: twice the code
 * rows; 4: shape 0 at the other residency (8-warp blocks at 128 registers where shape 0 has
 * 7-warp blocks at 80, as at 2048, and the reverse at 1024); -1 (the default): shape 0, except
 * shape 4 for an index at code dim 2048 of at most four times the L2 size. Results are
 * identical for every shape; only the speed differs. Other codecs and dims ignore it. Used by
 * the autotuner. Returns QG_ERR_INVALID outside -1..4. */
int qg_index_set_tile(qg_index *index, int tile);
/* Allocate the prepared-query workspace for max_nq queries and the visited tags for the launch
 * shape of pools up to max(max_l, max_k), so that qg_search_batch_graph never allocates. */
int qg_index_reserve(qg_index *index, size_t max_nq, int max_l, int max_k);
/* Capturable batched search for streams of uneven batches: the batch size is read on the device
 * from d_nq (<= max_nq), so one captured CUDA graph serves every batch size; per-query k and L
 * via d_k / d_l (params->k / l_value are their maxima). Never allocates: returns QG_ERR_INVALID
 * if qg_index_reserve did not cover max_nq and the pool size. Optional learned-stop model. */
int qg_search_batch_graph(qg_index *index, const float *d_queries, size_t max_nq, const int *d_nq,
                          const qg_search_params *params, const int *d_k, const int *d_l,
                          size_t k_stride, uint32_t *d_ids, float *d_dists, qg_search_stats *d_stats,
                          const qg_stop_model *model, void *stream);
/* Status word of the last qg_search_batch on this index (synchronises the stream). */
int qg_search_status(qg_index *index, void *stream);

/* Global centre (train_global_center_matrix, diskann_runner.rs:1677-1701): f32 mean of the
 * rows `d_rows` (ascending ids; NULL = rows 0..count-1) of a device [n x dim] matrix with row
 * stride `stride` floats, summed in row order. */
int qg_center_mean(const float *d_data, size_t stride, size_t dim, const uint32_t *d_rows,
                   size_t count, float *d_center_out, void *stream);

/* GPU encode (encodeVectorFullWithCentroid, space_rabitq.h:5845-5999) of n rows of device
 * f32 data into compact and residual records (device). */
int qg_encode_batch(const void *space, const float *d_raw, size_t n, uint8_t *d_compact,
                    uint8_t *d_residual, void *stream);
/* The encode rotation as a dense GEMM on the tensor cores (no counterpart in the reference,
 * which runs a fast Hadamard transform, RaBitQSpace::rotate, space_rabitq.h:944-1000): row n of
 * d_rotated [n x code_dim] = H diag(sgn) fl(c * (x_n - centre) / |x_n - centre|), c the stored
 * 1/sqrt(code_dim), computed as one BF16 x BF16 -> FP32 tcgen05 GEMM over the exact three-term
 * BF16 split of the scaled rows; d_norms [n] = |x_n - centre| (the encoder's sequential sum).
 * Every product is exact; only the FP32 summation order differs from the butterflies. Needs a
 * code dim that is a multiple of 256; allocates scratch and synchronises the stream;
 * QG_ERR_TIMEOUT if a tile's wait ran out. */
int qg_rotate_gemm(const void *space, const float *d_raw, size_t n, float *d_rotated, float *d_norms,
                   void *stream);
/* The GEMM of qg_rotate_gemm on operand planes given directly (kernel-level, for tests):
 * d_a3 [n x 3 Kp] BF16 bits (Kp = dim rounded up to 64; three planes side by side along K),
 * d_out [n x code_dim] = d_a3 times the space's +-1 operand (the Hadamard-sign matrix three
 * times along K). */
int qg_rotate_gemm_planes(const void *space, const uint16_t *d_a3, size_t n, float *d_out, void *stream);
/* qg_encode_batch with the rotation from qg_rotate_gemm (same record layout). Codes equal the
 * reference's except where the GEMM's summation order moves a rotated value across a code
 * boundary; allocates scratch and synchronises the stream. */
int qg_encode_batch_gemm(const void *space, const float *d_raw, size_t n, uint8_t *d_compact,
                         uint8_t *d_residual, void *stream);
/* GPU alpha robust prune for graph construction (this library's own builder; the reference
 * prunes on the host, vamana_prune.h:42-156). For each of n nodes, scores its K candidate ids
 * (device [n x K], UINT32_MAX = none; any order, duplicates allowed) with the symmetric 4-bit
 * estimator, keeps at most R out-edges by occlusion with alpha 1.0 then `alpha`, and writes
 * degrees [n] and edges [n x edge_stride] (UINT32_MAX padding). K <= 256, R <= edge_stride. */
int qg_prune_candidates(const void *space, const uint8_t *d_compact, size_t compact_stride, size_t n,
                        const uint32_t *d_candidates, size_t k, size_t r, float alpha,
                        uint32_t *d_degrees, uint32_t *d_edges, size_t edge_stride, void *stream);

/* rabitq_build_vamana_graph over device compact records: degrees [n] and edges
 * [n x edge_stride] (device, zero past each degree); *distance_evaluations (host, may be NULL)
 * as above. Synchronises `stream`. */
int qg_build_vamana_device(const void *space, const uint8_t *d_compact, size_t n, size_t compact_stride,
                           size_t r, size_t l_build, float alpha, size_t beam_width, size_t batch_size,
                           size_t refine_passes, size_t prune_candidate_cap, size_t build_early_stop_hops,
                           uint32_t *d_degrees, uint32_t *d_edges, size_t edge_stride,
                           uint64_t *distance_evaluations, void *stream);

/* GPU sidecar extraction (space_rabitq.h:4364-4392) from device compact records. */
int qg_export_sidecar_device(const void *space, const uint8_t *d_compact, size_t n,
                             size_t compact_stride, uint8_t *d_msb, void *d_factors,
                             void *stream);
/* GPU query preparation (space_rabitq.h:3429-3706, by the space's codec) for nq queries: rotated
 * residual [nq x D] f32, int8 codes [nq x D], scalars [nq x 4] = {query_norm_sqr,
 * query_norm, half_sum_residual, int8_scale}, code sums [nq] int64. */
int qg_prepare_batch(const void *space, const float *d_queries, size_t nq, float *d_rotated,
                     int8_t *d_codes, float *d_scalars, int64_t *d_code_sum, void *stream);
/* Kernel-level check of the INT8 dither decision used by qg_prepare_batch (no reference
 * counterpart; it restates the expression of space_rabitq.h:3625-3643): out[i] =
 * floor(double(x[i]) / double(scale[i]) + u) with u = double(draws[i]) * 2^-64 clamped below 1,
 * before the [-128, 127] clamp; undecided[i] (optional) = 1 where the FP32 decision fell back
 * to double arithmetic. */
int qg_dither_floor_pairs(const float *d_x, const float *d_scale, const uint64_t *d_draws, size_t n,
                          int32_t *d_out, uint8_t *d_undecided, void *stream);
/* Kernel-level check of the residual-code rounding used by the GPU encoder (no reference
 * counterpart; the expression of residualMseOptimalScale and the residual codes,
 * space_rabitq.h:748-786, 5936-5983): out[i] = clamp(round(double(x[i]) / double(s[i])), -7, 7)
 * (half away from zero); undecided[i] (optional) = 1 where the FP32 decision fell back to
 * double arithmetic. */
int qg_round_quotient_pairs(const float *d_x, const float *d_s, size_t n, int32_t *d_out, uint8_t *d_undecided,
                            void *stream);
/* Kernel-level entry points over (query, id) pairs, for parity tests and tools: prepared
 * query arrays as produced by qg_prepare_batch; pair i uses query qidx[i] and record ids[i].
 * Records/sidecars in the reference host layouts, but in device memory. */
int qg_gate_pairs(const void *space, const int8_t *d_codes, const float *d_scalars,
                  const int64_t *d_code_sum, const uint32_t *d_qidx, const uint32_t *d_ids,
                  size_t count, const uint8_t *d_msb, size_t msb_stride, const void *d_factors,
                  size_t factor_stride, float epsilon0, RabitqPaperEstimate *d_out, void *stream);
/* The Full codec's gate over pairs: the FP32 rotated residual (qg_prepare_batch's d_rotated)
 * against the MSB plane (qg_gate_pairs refuses the Full codec). */
int qg_gate_full_pairs(const void *space, const float *d_rotated, const float *d_scalars, const uint32_t *d_qidx,
                       const uint32_t *d_ids, size_t count, const uint8_t *d_msb, size_t msb_stride,
                       const void *d_factors, size_t factor_stride, float epsilon0, RabitqPaperEstimate *d_out,
                       void *stream);
int qg_distance_pairs(const void *space, const float *d_rotated, const int8_t *d_codes,
                      const float *d_scalars, const int64_t *d_code_sum, const uint32_t *d_qidx,
                      const uint32_t *d_ids, const uint8_t *d_modes, size_t count,
                      const uint8_t *d_records, size_t record_stride, const float *d_short_ips,
                      float *d_out, void *stream);
int qg_residual_pairs(const void *space, const float *d_rotated, const float *d_scalars,
                      const uint32_t *d_qidx, const uint32_t *d_ids, size_t count,
                      const uint8_t *d_residual, size_t residual_stride,
                      const float *d_long_distances, RabitqDistanceInterval *d_out,
                      void *stream);

#ifdef __cplusplus
}
#endif

#endif /* QGRAPH_GB300_H */
