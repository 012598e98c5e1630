// qg_types.h -- internal structs shared by the host code and the kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include <cuda_runtime.h>

#include "qgraph_gb300.h"

namespace qg {

// Space configuration of RaBitQSpace (space_rabitq.h:2836-2893) in the formal bridge
// config: one centroid, 4-bit residuals in blocks of 16, MSE scale, fp16 scale storage,
// external residual storage.
struct Space {
    size_t dim = 0;
    size_t code_dim = 0;       // D = next_pow2(roundup64(dim))
    size_t code_bytes = 0;     // D/2
    size_t block_count = 0;    // D/16
    size_t scale_bytes = 0;    // 2*D/16
    size_t full_bytes = 0;
    size_t compact_bytes = 0;
    size_t residual_bytes = 0;
    size_t msb_bytes = 0;      // D/8
    uint32_t seed = 100;
    int codec = 0;             // QueryCoarseCodec; Int8 = 3 is the GPU path
    int device = 0;
    std::vector<float> signs;  // +-1/sqrt(D)
    std::vector<float> center;
    bool center_set = false;
    // device copies
    float *d_signs = nullptr;          // [D]
    float *d_center = nullptr;         // [dim]
    float *d_rotated_center = nullptr; // [D]
    float *d_center_norm = nullptr;    // [1] ||c||^2 as float (setCentroids)
    float center_norm_sqr = 0.0f;
    void *d_rot_gemm_b = nullptr;      // the tensor-core rotation's +-1 operand (built on first use)
};

// Query code layout of a codec id: Int8 (3) -> 8, Int4 (2) -> 4 (integer codes), B1 (1) -> 1 (sign
// bits), B1Main (4) -> 2 (+-1 bytes), and 32 (the FP32 residual only) for every other id: Full (0),
// FullStaged (5), FullRerankScalar (6) and any value outside the enum, which the reference's space
// handles as Full (space_rabitq.h:3464-3469, 4519-4531).
inline int codec_query_bits(int c) { return c == 3 ? 8 : (c == 2 ? 4 : (c == 1 ? 1 : (c == 4 ? 2 : 32))); }
// Search mode of a codec id: 0 integer codes (Int8 / Int4), 1 B1 (popcount gate), 2 B1Main (no gate;
// every fresh neighbour by the 4-bit x 1-bit distance), 3 the Full codecs (FP32 gate; survivors by
// the remaining bits with the gate's short ip).
inline int codec_search_mode(int c) { return c == 1 ? 1 : (c == 4 ? 2 : (c == 2 || c == 3 ? 0 : 3)); }
inline int space_query_bits(const Space *s) { return codec_query_bits(s->codec); }
inline int space_search_mode(const Space *s) { return codec_search_mode(s->codec); }

// Device-resident index: structure-of-arrays, every row 16-byte aligned.
struct DevIndex {
    uint32_t n_total = 0;   // graph nodes
    uint32_t n_base = 0;    // nodes with payloads
    uint32_t code_dim = 0;
    uint32_t edge_stride = 0;
    uint32_t max_degree = 0;
    uint8_t *codes = nullptr;       // [n_base x D/2]
    float4 *hdr = nullptr;          // [n_base] {norm_sqr, long_scale, short_scale, error_scale}
    uint8_t *msb = nullptr;         // [n_base x D/8]
    float4 *pf = nullptr;           // [n_base] {norm_sqr, data_norm, cross_scale|NaN, error_cross}
    uint16_t *res_scales = nullptr; // [n_base x D/16]
    uint8_t *res_codes = nullptr;   // [n_base x D/2]
    uint32_t *degrees = nullptr;    // [n_total]
    uint32_t *edges = nullptr;      // [n_total x edge_stride]
};

// Per-query prepared state produced by the query-preparation kernel.
struct DevQueries {
    float *rr = nullptr;        // [nq x D] rotated residual
    int8_t *codes = nullptr;    // [nq x D]
    float4 *scal = nullptr;     // [nq] {qn2, qn, half_sum, int8_scale}
    long long *csum = nullptr;  // [nq]
};

}  // namespace qg

namespace qg {
// Device allocations freed together when the last owner lets go.
struct DeviceBlocks {
    std::vector<void *> ptrs;
    DeviceBlocks() = default;
    DeviceBlocks(const DeviceBlocks &) = delete;
    DeviceBlocks &operator=(const DeviceBlocks &) = delete;
    ~DeviceBlocks() {
        for (void *p : ptrs) cudaFree(p);
    }
};
}  // namespace qg

struct qg_index {
    qg::DevIndex ix;
    const qg::Space *space = nullptr;
    int device = 0;
    // search scratch: a visited bit row per warp slot, queue counter, status word
    uint32_t *visited = nullptr;
    unsigned int *counter = nullptr;
    int *status = nullptr;
    int slots = 0;
    int grid = 0;
    int warps_per_block = 0;
    // prepared-query workspace, grown on demand (not inside graph capture)
    qg::DevQueries q;
    size_t q_capacity = 0;
    size_t device_bytes = 0;
    int launch_wpb = 0;      // qg_index_set_launch override (0 = automatic)
    int launch_per_sm = 0;
    int tile = -1;           // qg_index_set_tile: the search's tile shape (-1: chosen by index size)
    // the payload and adjacency allocations, shared by the handles qg_index_share makes and freed
    // with the last of them; the scratch above belongs to this handle alone
    std::shared_ptr<qg::DeviceBlocks> payload;
};
