// qg_kernels.h -- kernel argument blocks and launchers (host-callable).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "qg_types.h"

namespace qg {

struct PrepArgs {
    const float *queries;
    size_t query_stride;
    int nq;
    int dim;
    int code_dim;
    const float *signs;
    const float *center;
    const float *rotated_center;
    const float *center_norm_sqr;
    float *rr;
    int8_t *codes;
    float4 *scal;
    long long *csum;
    const int *nq_dev;  // optional: the batch size read on the device (CUDA-graph replay)
    int qbits = 8;      // 8: Int8; 4: Int4 (scale max/8, codes in [-8, 7], second draw); 1: B1 (sign
                        // bits); 2: B1Main (+-1 bytes, the sign sum in the code-sum slot); 32: Full
                        // (the FP32 residual and scalars only)
};

struct SearchArgs {
    DevIndex ix;
    const float *rr;
    const int8_t *codes;
    const float4 *scal;
    const long long *csum;
    int nq;
    int k_default;
    int l_default;
    const int *k_per_q;
    const int *l_per_q;
    int k_stride;
    int l_cap;       // pool capacity per warp (>= every L and k)
    int mode;        // 0 Int8 / Int4; 1 B1 (sign bits, popcount gate, survivors by the FP32 restore);
                     // 2 B1Main (+-1 codes, no gate, every fresh neighbour by the 4-bit x 1-bit distance);
                     // 3 Full (FP32 gate, survivors by the remaining bits with the gate's short ip)
    int beam_width;
    int tile;        // tile shape of the Int8 / Int4 search at D >= 1024 (0..4; search.cu, Tile), else 0
    float eps;
    int rerank;
    int early_stop_hops;
    int kth_stop;
    int fused_rerank;    // rerank residual in the fused kernel's product order (the fused Int8 / Int4
                         // rerank, or FullRerankScalar's per-record residual)
    uint32_t *ids_out;
    float *dists_out;
    qg_search_stats *stats_out;
    uint32_t *visited;   // [slots x visited_row_words(n_total)] one bit per node, cleared per query
    unsigned int *counter;
    int *status;
    int hop_cap;
    uint32_t *expanded_out;  // optional [nq x expanded_cap]: expanded nodes in hop order
    int expanded_cap;
    // learned early termination (optional): every stop_every hops (from stop_min_hops on) the
    // warp forms the 8 search-state features and evaluates the network. stop_kind 0: it stops
    // when the logit exceeds stop_logit. stop_kind 1: the output is log(hops the query needs);
    // the query stops once its hops reach stop_scale * exp(output) (re-predicted at every
    // checkpoint, or only at the first one when stop_once)
    const uint16_t *stop_w;
    const float *stop_norm;
    float stop_logit;
    int stop_every;
    int stop_min_hops;
    int stop_kind;
    float stop_scale;
    int stop_once;
    // trace collection (optional): features at every stop_every-th hop with the label "how many
    // ids of trace_truth the first max(rerank, k) pool entries already hold"
    const uint32_t *trace_truth;  // [nq x trace_truth_k]
    int trace_truth_k;
    int trace_cap;
    float *trace_feat;   // [nq x trace_cap x 8]
    float *trace_label;  // [nq x trace_cap]
    int *trace_count;    // [nq]
    const int *nq_dev;   // optional: the batch size read on the device (CUDA-graph replay)
};

struct EncodeArgs {
    const float *raw;
    size_t raw_stride;
    int n;
    int dim;
    int code_dim;
    const float *signs;
    const float *center;
    uint8_t *compact;      // [n x compact_bytes]
    uint8_t *residual;     // [n x residual_bytes]
    size_t compact_bytes;
    size_t residual_bytes;
    const float *rotated = nullptr;  // optional [n x code_dim]: rows already rotated (raw, signs unused)
    const float *norms = nullptr;    // [n] residual norms, with `rotated`
};

// 32-bit words of one warp slot's visited row: a bit per graph node, rounded up to 16 bytes.
__host__ __device__ inline size_t visited_row_words(size_t n_total) { return ((n_total + 31) / 32 + 3) & ~size_t(3); }

// Sets the message qg_last_error() returns on the calling thread.
void record_error(const std::string &msg);

// Checks the arguments of a batched search (qg_search_batch and its variants) and fills every
// field of *out that does not name scratch memory: the prepared-query buffers, the visited
// rows, the work counter and the status word stay null for the caller to place. Returns QG_OK or a
// QG_ERR_* status with the message recorded.
int search_args_fill(const qg_index *index, size_t nq, const qg_search_params *params, const float *d_queries,
                     const int *d_k, const int *d_l, size_t k_stride, uint32_t *d_ids, float *d_dists,
                     qg_search_stats *d_stats, SearchArgs *out);
// Warps per block and resident blocks per SM of the search kernel for a pool of l_cap entries:
// the qg_index_set_launch override clamped to what is resident, else the shape with the most
// resident warps. False (message recorded) when no block can be resident.
bool search_launch_geometry(const qg_index *index, int l_cap, bool stop_model, int *wpb_out, int *per_sm_out);

cudaError_t launch_prepare(const PrepArgs &a, cudaStream_t stream);
cudaError_t launch_round_quotient_pairs(const float *x, const float *s, size_t n, int *out, uint8_t *undecided,
                                        cudaStream_t stream);
cudaError_t launch_dither_pairs(const float *x, const float *scale, const unsigned long long *draws, size_t n,
                                int *out, uint8_t *undecided, cudaStream_t stream);
cudaError_t launch_center_setup(const float *center, const float *signs, int dim, int D,
                                float *rotated, float *norm_out, cudaStream_t stream);
cudaError_t launch_center_mean(const float *data, size_t stride, int dim, const uint32_t *rows,
                               size_t count, float *out, cudaStream_t stream);
cudaError_t launch_search(const SearchArgs &a, int grid, int warps_per_block, cudaStream_t stream);
size_t search_smem_per_warp(int code_dim, int l_cap);
// Resident blocks per SM and dynamic shared memory of one search block; a stop model adds
// the staged network weights to every block.
int search_blocks_per_sm(int code_dim, int l_cap, int warps_per_block, bool stop_model = false, int tile = 0);
// The widest block the search kernel for this code dim and tile shape is compiled for, in warps.
int search_max_block_warps(int code_dim, int tile);
// The block width the automatic launch shape tries first (0: none), ahead of the widest.
int search_first_block_warps(int code_dim, int tile);
size_t search_block_smem(int l_cap, int warps_per_block, bool stop_model);
int search_supported_dim(int code_dim);
cudaError_t launch_encode(const EncodeArgs &a, cudaStream_t stream);
// The encode rotation on the tensor cores (rotate_gemm.cu). Kp = dim rounded up to 64; a3 holds
// n x 3 Kp BF16 (the rows' three exact BF16 terms), r3 code_dim x 3 Kp BF16 (the +-1 Hadamard-
// sign matrix three times). status receives bit 0 when a CTA's wait timed out.
int rotate_gemm_kp(int dim);
bool rotate_gemm_supported(int code_dim);
cudaError_t launch_rotate_split(const float *raw, size_t stride, int n, int dim, const float *center, float c_abs,
                                void *a3, float *norms, cudaStream_t stream);
cudaError_t launch_r_matrix(const float *signs, int dim, int code_dim, void *r3, cudaStream_t stream);
cudaError_t launch_rotate_gemm(const void *a3, const void *r3, int n, int dim, int code_dim, float *out, int *status,
                               cudaStream_t stream);
cudaError_t launch_mlp_forward(const float *X, size_t n, const float *norm, const uint16_t *w, float *logits,
                               cudaStream_t stream);
cudaError_t launch_mlp_backward(const float *X, const float *y, size_t n, const float *norm, const uint16_t *w,
                                float *grad, float *loss, cudaStream_t stream, bool mse = false);
cudaError_t launch_mlp_adam(float *master, uint16_t *w, const float *grad, float *m, float *v, float lr,
                            float beta1, float beta2, float eps, int step, cudaStream_t stream);
cudaError_t launch_prune(int code_dim, const uint8_t *compact, size_t stride, int n, const uint32_t *cand,
                         int K, int R, float alpha, uint32_t *degrees, uint32_t *edges, size_t edge_stride,
                         cudaStream_t stream);
cudaError_t launch_sidecar(const uint8_t *compact, size_t n, size_t stride, int code_dim,
                           uint8_t *msb, RabitqPaperFactors *factors, cudaStream_t stream);
cudaError_t launch_repack(const uint8_t *compact, size_t compact_stride, const uint8_t *residual,
                          size_t residual_stride, const uint8_t *msb, size_t msb_stride,
                          const uint8_t *factors, size_t factor_stride, const uint32_t *degrees,
                          const uint32_t *edges, size_t edge_stride, DevIndex ix,
                          cudaStream_t stream);
cudaError_t launch_gate_pairs(int code_dim, const int8_t *codes, const float4 *scal,
                              const long long *csum, const uint32_t *qidx, const uint32_t *ids,
                              size_t count, const uint8_t *msb, size_t msb_stride,
                              const uint8_t *factors, size_t factor_stride, float eps,
                              RabitqPaperEstimate *out, cudaStream_t stream, bool b1 = false);
// the gate from the encoded record (compute_paper_prune_estimate), any codec
cudaError_t launch_gate_encoded_pairs(int code_dim, const float *rr, const float4 *scal, const uint32_t *qidx,
                                      const uint32_t *ids, size_t count, const uint8_t *records, size_t record_stride,
                                      float eps, RabitqPaperEstimate *out, cudaStream_t stream);
// the Full codec's gate: the FP32 rotated residual (rr) against the MSB plane
cudaError_t launch_gate_full_pairs(int code_dim, const float *rr, const float4 *scal, const uint32_t *qidx,
                                   const uint32_t *ids, size_t count, const uint8_t *msb, size_t msb_stride,
                                   const uint8_t *factors, size_t factor_stride, float eps, RabitqPaperEstimate *out,
                                   cudaStream_t stream);
cudaError_t launch_distance_pairs(int code_dim, const float *rr, const int8_t *codes,
                                  const float4 *scal, const long long *csum,
                                  const uint32_t *qidx, const uint32_t *ids,
                                  const uint8_t *modes, size_t count, const uint8_t *records,
                                  size_t record_stride, const float *short_ips, float *out,
                                  cudaStream_t stream);
// fused: the product order of the fused restore + residual rerank kernel
cudaError_t launch_residual_pairs(int code_dim, const float *rr, const float4 *scal,
                                  const uint32_t *qidx, const uint32_t *ids, size_t count,
                                  const uint8_t *residual, size_t residual_stride,
                                  const float *long_d, bool fused, RabitqDistanceInterval *out,
                                  cudaStream_t stream);
cudaError_t launch_symmetric_pairs(int code_dim, const uint8_t *lhs, const uint8_t *rhs,
                                   size_t count, size_t stride, float *out, cudaStream_t stream);
// query_distance_b1 (space_rabitq.h:3741-3753) over (query, record) pairs; codes = B1Main +-1 bytes,
// or, with sign_bits, a B1 prepared query's sign bits.
cudaError_t launch_distance_b1_pairs(int code_dim, const int8_t *codes, const float4 *scal, const long long *csum,
                                     const uint32_t *qidx, const uint32_t *ids, size_t count, const uint8_t *records,
                                     size_t record_stride, float *out, cudaStream_t stream, bool sign_bits = false);

// rabitq_build_vamana_graph arguments (rabitq_bridge.cpp:224-303)
struct VbBuildParams {
    size_t r;
    size_t l_build;
    float alpha;
    size_t beam;
    size_t batch;
    size_t refine;
    size_t cap;
    size_t stop_hops;
};
// The reference's Vamana build (vamana_index.h:452-528, 328-422, 995-1117) over n device compact
// records; writes degrees [n] and edges [n x edge_stride] (device; zero past each degree).
// evals_out (host, may be null) receives the number of distances this implementation evaluated.
// Synchronises `stream`. r <= 64, beam * r <= 1024.
cudaError_t launch_vamana_build(int code_dim, const uint8_t *d_compact, size_t n, size_t stride,
                                const VbBuildParams &p, uint32_t *d_degrees, uint32_t *d_edges, size_t edge_stride,
                                unsigned long long *evals_out, cudaStream_t stream);

}  // namespace qg
