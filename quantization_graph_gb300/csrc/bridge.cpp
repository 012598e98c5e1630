// bridge.cpp -- the C ABI of libqgraph_gb300.so (declared in include/qgraph_gb300.h).
//
// rabitq_* entry points keep the reference bridge's contract
// (experiments/02_diskann_fair/native/rabitq_bridge.cpp): caller-owned host buffers, no
// exception crosses the ABI, failures return false / NULL / +inf / {0,..,valid=0}, and batch
// calls fill failed items with sentinels and still return true. Their arithmetic runs in the
// CUDA kernels of this library; host code here only validates, gathers the rows a call names
// into pinned staging buffers and moves bytes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <new>
#include <random>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "qg_kernels.h"
#include "qg_types.h"

namespace qg {
namespace {

thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

bool cuda_ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

size_t round_up_code_dim(size_t value) {  // space_rabitq.h:217-224
    const size_t rounded = ((value + 63U) / 64U) * 64U;
    size_t power = 1;
    while (power < rounded) power <<= 1U;
    return power;
}

template <typename T>
T *dev_alloc(size_t count) {
    void *p = nullptr;
    if (count == 0) count = 1;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return nullptr;
    return static_cast<T *>(p);
}

// Growable device + pinned host staging for the host-pointer rabitq_* calls.
struct Staging {
    void *d = nullptr;
    size_t d_bytes = 0;
    void *h = nullptr;
    size_t h_bytes = 0;
    cudaStream_t stream = nullptr;
    ~Staging() {
        if (d) cudaFree(d);
        if (h) cudaFreeHost(h);
        if (stream) cudaStreamDestroy(stream);
    }
    bool reserve(size_t bytes) {
        if (!stream && cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (bytes > d_bytes) {
            if (d) cudaFree(d);
            d = nullptr;
            d_bytes = 0;
            const size_t want = std::max<size_t>(bytes, 1 << 20);
            if (cudaMalloc(&d, want) != cudaSuccess) return false;
            d_bytes = want;
        }
        if (bytes > h_bytes) {
            if (h) cudaFreeHost(h);
            h = nullptr;
            h_bytes = 0;
            const size_t want = std::max<size_t>(bytes, 1 << 20);
            if (cudaMallocHost(&h, want) != cudaSuccess) return false;
            h_bytes = want;
        }
        return true;
    }
};

thread_local Staging t_stage;

// Bump allocator over the staging buffers (both sides use the same offsets).
struct Carve {
    size_t off = 0;
    size_t take(size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) & ~static_cast<size_t>(255);
        return at;
    }
};

// The thread-local prepared query (space_rabitq.h:3700-3706 keeps one per thread).
struct Prepared {
    const Space *space = nullptr;
    size_t D = 0;
    int device = -1;
    float *d_query = nullptr;
    float *d_rr = nullptr;
    int8_t *d_codes = nullptr;
    float4 *d_scal = nullptr;
    long long *d_csum = nullptr;
    float4 h_scal{};
    long long h_csum = 0;
    int codec = 0;  // the space's codec when the query was prepared (PreparedQuery::query_coarse_codec)
    bool valid = false;
    ~Prepared() { release(); }
    void release() {
        cudaFree(d_query);
        cudaFree(d_rr);
        cudaFree(d_codes);
        cudaFree(d_scal);
        cudaFree(d_csum);
        d_query = nullptr;
        d_rr = nullptr;
        d_codes = nullptr;
        d_scal = nullptr;
        d_csum = nullptr;
        D = 0;
    }
    bool ensure(const Space *s) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (D == s->code_dim && d_query && device == dev) return true;
        release();
        D = s->code_dim;
        device = dev;
        d_query = dev_alloc<float>(s->dim);
        d_rr = dev_alloc<float>(D);
        d_codes = dev_alloc<int8_t>(D);
        d_scal = dev_alloc<float4>(1);
        d_csum = dev_alloc<long long>(1);
        return d_query && d_rr && d_codes && d_scal && d_csum;
    }
};

thread_local Prepared t_prepared;

const Space *as_space(const void *p) { return static_cast<const Space *>(p); }

bool check_prepared(const Space *s, const void *prepared) {
    return s && prepared == &t_prepared && t_prepared.valid && t_prepared.space == s;
}

RabitqPaperEstimate zero_estimate() { return RabitqPaperEstimate{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0}; }

// Gather the rows `ids` of a host table into the staging host buffer at `dst`.
void gather_rows(uint8_t *dst, const uint8_t *base, size_t stride, const uint32_t *ids,
                 size_t count, size_t row_bytes) {
    for (size_t i = 0; i < count; ++i)
        std::memcpy(dst + i * row_bytes, base + static_cast<size_t>(ids[i]) * stride, row_bytes);
}

// Identity (query index 0, local row i) pair lists for a staged batch.
void fill_pairs(uint32_t *qidx, uint32_t *ids, size_t count) {
    for (size_t i = 0; i < count; ++i) {
        qidx[i] = 0;
        ids[i] = static_cast<uint32_t>(i);
    }
}

bool gate_host(const Space *s, const uint32_t *ids, size_t count, const uint8_t *msb_base,
               size_t msb_stride, const uint8_t *factors_base, size_t factor_stride, float eps,
               RabitqPaperEstimate *out) {
    const size_t mb = s->msb_bytes;
    Carve c;
    const size_t o_q = c.take(count * 4), o_i = c.take(count * 4), o_m = c.take(count * mb),
                 o_f = c.take(count * 20), o_o = c.take(count * sizeof(RabitqPaperEstimate));
    if (!t_stage.reserve(c.off)) return false;
    uint8_t *h = static_cast<uint8_t *>(t_stage.h), *d = static_cast<uint8_t *>(t_stage.d);
    fill_pairs(reinterpret_cast<uint32_t *>(h + o_q), reinterpret_cast<uint32_t *>(h + o_i), count);
    gather_rows(h + o_m, msb_base, msb_stride, ids, count, mb);
    gather_rows(h + o_f, factors_base, factor_stride, ids, count, 20);
    cudaStream_t st = t_stage.stream;
    if (!cuda_ok(cudaMemcpyAsync(d, h, o_o, cudaMemcpyHostToDevice, st), "gate upload")) return false;
    // compute_paper_prune_estimate_sidecar (space_rabitq.h:4510-4531): B1 -> the popcount gate,
    // Int4 / Int8 -> the integer gate, every other codec (Full, B1Main, the Full variants) -> the
    // FP32 Full gate
    const int codec = t_prepared.codec;
    const cudaError_t ge =
        (codec != 1 && codec_search_mode(codec) != 0)
            ? launch_gate_full_pairs(static_cast<int>(s->code_dim), t_prepared.d_rr, t_prepared.d_scal,
                                     reinterpret_cast<uint32_t *>(d + o_q), reinterpret_cast<uint32_t *>(d + o_i),
                                     count, d + o_m, mb, d + o_f, 20, eps,
                                     reinterpret_cast<RabitqPaperEstimate *>(d + o_o), st)
            : launch_gate_pairs(static_cast<int>(s->code_dim), t_prepared.d_codes, t_prepared.d_scal,
                                t_prepared.d_csum, reinterpret_cast<uint32_t *>(d + o_q),
                                reinterpret_cast<uint32_t *>(d + o_i), count, d + o_m, mb, d + o_f, 20, eps,
                                reinterpret_cast<RabitqPaperEstimate *>(d + o_o), st, codec == 1);
    if (!cuda_ok(ge, "gate kernel")) return false;
    if (!cuda_ok(cudaMemcpyAsync(h + o_o, d + o_o, count * sizeof(RabitqPaperEstimate),
                                 cudaMemcpyDeviceToHost, st), "gate download"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(st), "gate sync")) return false;
    std::memcpy(out, h + o_o, count * sizeof(RabitqPaperEstimate));
    return true;
}

// compute_paper_prune_estimate for the records ids[i] (compact rows gathered like distance_host).
bool gate_encoded_host(const Space *s, const uint32_t *ids, size_t count, const uint8_t *rec_base,
                       size_t rec_stride, float eps, RabitqPaperEstimate *out) {
    const size_t rb = s->compact_bytes;
    Carve c;
    const size_t o_q = c.take(count * 4), o_i = c.take(count * 4), o_r = c.take(count * rb),
                 o_o = c.take(count * sizeof(RabitqPaperEstimate));
    if (!t_stage.reserve(c.off)) return false;
    uint8_t *h = static_cast<uint8_t *>(t_stage.h), *d = static_cast<uint8_t *>(t_stage.d);
    fill_pairs(reinterpret_cast<uint32_t *>(h + o_q), reinterpret_cast<uint32_t *>(h + o_i), count);
    gather_rows(h + o_r, rec_base, rec_stride, ids, count, rb);
    cudaStream_t st = t_stage.stream;
    if (!cuda_ok(cudaMemcpyAsync(d, h, o_o, cudaMemcpyHostToDevice, st), "gate upload")) return false;
    if (!cuda_ok(launch_gate_encoded_pairs(static_cast<int>(s->code_dim), t_prepared.d_rr, t_prepared.d_scal,
                                           reinterpret_cast<uint32_t *>(d + o_q), reinterpret_cast<uint32_t *>(d + o_i),
                                           count, d + o_r, rb, eps, reinterpret_cast<RabitqPaperEstimate *>(d + o_o), st),
                 "gate kernel"))
        return false;
    if (!cuda_ok(cudaMemcpyAsync(h + o_o, d + o_o, count * sizeof(RabitqPaperEstimate), cudaMemcpyDeviceToHost, st),
                 "gate download"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(st), "gate sync")) return false;
    std::memcpy(out, h + o_o, count * sizeof(RabitqPaperEstimate));
    return true;
}

bool distance_host(const Space *s, const uint32_t *ids, const uint8_t *modes, size_t count,
                   const uint8_t *rec_base, size_t rec_stride, const float *short_ips, float *out) {
    const size_t rb = s->compact_bytes;
    Carve c;
    const size_t o_q = c.take(count * 4), o_i = c.take(count * 4), o_md = c.take(count),
                 o_s = c.take(count * 4), o_r = c.take(count * rb), o_o = c.take(count * 4);
    if (!t_stage.reserve(c.off)) return false;
    uint8_t *h = static_cast<uint8_t *>(t_stage.h), *d = static_cast<uint8_t *>(t_stage.d);
    fill_pairs(reinterpret_cast<uint32_t *>(h + o_q), reinterpret_cast<uint32_t *>(h + o_i), count);
    // modes 2 (quantized remaining bits), 1 and 3 (FP32 remaining bits with the given short ip);
    // every other value recomputes the FP32 restore, as the reference's dispatch does
    for (size_t i = 0; i < count; ++i)
        h[o_md + i] = modes ? (modes[i] == 2 ? 2 : (modes[i] == 1 || modes[i] == 3) ? 1 : 0) : 0;
    for (size_t i = 0; i < count; ++i)
        reinterpret_cast<float *>(h + o_s)[i] = short_ips ? short_ips[i] : 0.0f;
    gather_rows(h + o_r, rec_base, rec_stride, ids, count, rb);
    cudaStream_t st = t_stage.stream;
    if (!cuda_ok(cudaMemcpyAsync(d, h, o_o, cudaMemcpyHostToDevice, st), "distance upload")) return false;
    if (!cuda_ok(launch_distance_pairs(static_cast<int>(s->code_dim), t_prepared.d_rr, t_prepared.d_codes,
                                       t_prepared.d_scal, t_prepared.d_csum,
                                       reinterpret_cast<uint32_t *>(d + o_q),
                                       reinterpret_cast<uint32_t *>(d + o_i), d + o_md, count, d + o_r,
                                       rb, reinterpret_cast<float *>(d + o_s),
                                       reinterpret_cast<float *>(d + o_o), st),
                 "distance kernel"))
        return false;
    if (!cuda_ok(cudaMemcpyAsync(h + o_o, d + o_o, count * 4, cudaMemcpyDeviceToHost, st), "distance download"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(st), "distance sync")) return false;
    std::memcpy(out, h + o_o, count * 4);
    return true;
}

// query_distance_b1 for the records ids[i] (rows gathered like distance_host); the prepared
// query must be a B1Main one (+-1 codes, sign sum in the code-sum slot).
bool distance_b1_host(const Space *s, const uint32_t *ids, size_t count, const uint8_t *rec_base, size_t rec_stride,
                      float *out) {
    const size_t rb = s->compact_bytes;
    Carve c;
    const size_t o_q = c.take(count * 4), o_i = c.take(count * 4), o_r = c.take(count * rb),
                 o_o = c.take(count * 4);
    if (!t_stage.reserve(c.off)) return false;
    uint8_t *h = static_cast<uint8_t *>(t_stage.h), *d = static_cast<uint8_t *>(t_stage.d);
    fill_pairs(reinterpret_cast<uint32_t *>(h + o_q), reinterpret_cast<uint32_t *>(h + o_i), count);
    gather_rows(h + o_r, rec_base, rec_stride, ids, count, rb);
    cudaStream_t st = t_stage.stream;
    if (!cuda_ok(cudaMemcpyAsync(d, h, o_o, cudaMemcpyHostToDevice, st), "b1 distance upload")) return false;
    if (!cuda_ok(launch_distance_b1_pairs(static_cast<int>(s->code_dim), t_prepared.d_codes, t_prepared.d_scal,
                                          t_prepared.d_csum, reinterpret_cast<uint32_t *>(d + o_q),
                                          reinterpret_cast<uint32_t *>(d + o_i), count, d + o_r, rb,
                                          reinterpret_cast<float *>(d + o_o), st, t_prepared.codec == 1),
                 "b1 distance kernel"))
        return false;
    if (!cuda_ok(cudaMemcpyAsync(h + o_o, d + o_o, count * 4, cudaMemcpyDeviceToHost, st), "b1 distance download"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(st), "b1 distance sync")) return false;
    std::memcpy(out, h + o_o, count * 4);
    return true;
}

bool residual_host(const Space *s, const uint32_t *ids, size_t count, const uint8_t *res_base,
                   size_t res_stride, const float *long_d, RabitqDistanceInterval *out,
                   bool fused = false) {
    const size_t rb = s->residual_bytes;
    Carve c;
    const size_t o_q = c.take(count * 4), o_i = c.take(count * 4), o_l = c.take(count * 4),
                 o_r = c.take(count * rb), o_o = c.take(count * sizeof(RabitqDistanceInterval));
    if (!t_stage.reserve(c.off)) return false;
    uint8_t *h = static_cast<uint8_t *>(t_stage.h), *d = static_cast<uint8_t *>(t_stage.d);
    fill_pairs(reinterpret_cast<uint32_t *>(h + o_q), reinterpret_cast<uint32_t *>(h + o_i), count);
    std::memcpy(h + o_l, long_d, count * 4);
    gather_rows(h + o_r, res_base, res_stride, ids, count, rb);
    cudaStream_t st = t_stage.stream;
    if (!cuda_ok(cudaMemcpyAsync(d, h, o_o, cudaMemcpyHostToDevice, st), "residual upload")) return false;
    if (!cuda_ok(launch_residual_pairs(static_cast<int>(s->code_dim), t_prepared.d_rr, t_prepared.d_scal,
                                       reinterpret_cast<uint32_t *>(d + o_q),
                                       reinterpret_cast<uint32_t *>(d + o_i), count, d + o_r, rb,
                                       reinterpret_cast<float *>(d + o_l), fused,
                                       reinterpret_cast<RabitqDistanceInterval *>(d + o_o), st),
                 "residual kernel"))
        return false;
    if (!cuda_ok(cudaMemcpyAsync(h + o_o, d + o_o, count * sizeof(RabitqDistanceInterval),
                                 cudaMemcpyDeviceToHost, st), "residual download"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(st), "residual sync")) return false;
    std::memcpy(out, h + o_o, count * sizeof(RabitqDistanceInterval));
    return true;
}

bool encode_host(const Space *s, const float *raw, size_t n, uint8_t *compact, uint8_t *residual) {
    Carve c;
    const size_t o_x = c.take(n * s->dim * 4), o_c = c.take(n * s->compact_bytes),
                 o_r = c.take(n * s->residual_bytes);
    if (!t_stage.reserve(c.off)) return false;
    uint8_t *h = static_cast<uint8_t *>(t_stage.h), *d = static_cast<uint8_t *>(t_stage.d);
    std::memcpy(h + o_x, raw, n * s->dim * 4);
    cudaStream_t st = t_stage.stream;
    if (!cuda_ok(cudaMemcpyAsync(d + o_x, h + o_x, n * s->dim * 4, cudaMemcpyHostToDevice, st), "encode upload"))
        return false;
    if (qg_encode_batch(s, reinterpret_cast<float *>(d + o_x), n, d + o_c, d + o_r, st) != QG_OK) return false;
    if (!cuda_ok(cudaMemcpyAsync(h + o_c, d + o_c, c.off - o_c, cudaMemcpyDeviceToHost, st), "encode download"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(st), "encode sync")) return false;
    if (compact) std::memcpy(compact, h + o_c, n * s->compact_bytes);
    if (residual) std::memcpy(residual, h + o_r, n * s->residual_bytes);
    return true;
}

// Full record layout (space_rabitq.h:2855-2859): header, short factors, residual factors,
// scales, code, centroid id, residual code.
void assemble_full(const Space *s, const uint8_t *compact, const uint8_t *residual, uint8_t *full) {
    std::memcpy(full, compact, 16);
    std::memcpy(full + 16, residual, 8);
    std::memcpy(full + 24, residual + 8, s->scale_bytes);
    std::memcpy(full + 24 + s->scale_bytes, compact + 16, s->code_bytes);
    full[24 + s->scale_bytes + s->code_bytes] = compact[16 + s->code_bytes];
    std::memcpy(full + 25 + s->scale_bytes + s->code_bytes, residual + 8 + s->scale_bytes, s->code_bytes);
}

}  // namespace

void record_error(const std::string &msg) { set_error(msg); }

// Warps per block and resident blocks per SM for a pool of l_cap entries: the caller's override
// (qg_index_set_launch) clamped to what is resident, else the candidate with the most resident
// warps (large pools need more shared memory per warp, where smaller blocks pack better).
static size_t l2_bytes(int device) {
    static std::mutex mu;
    static std::map<int, size_t> cache;
    std::lock_guard<std::mutex> lock(mu);
    const auto it = cache.find(device);
    if (it != cache.end()) return it->second;
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, device) != cudaSuccess) v = 0;
    cache[device] = static_cast<size_t>(v);
    return static_cast<size_t>(v);
}

// The tile shape the search launches with: the index's for the Int8 / Int4 search at code dims of
// 1024 and more (the instantiations that have shapes), else the default. Unset (-1) at D = 2048:
// shape 0 (80 registers, 24 warps per SM) for an index of more than four times the L2, where the
// extra warps hide the DRAM latency (1M x 1536: +6 % over shape 4); shape 4 (128 registers, 16
// warps) for a smaller one, which the L2 mostly holds (100k x 1536: +30 % over shape 0).
static int search_tile(const qg_index *index) {
    if (space_search_mode(index->space) != 0 || index->space->code_dim < 1024) return 0;
    if (index->tile >= 0) return index->tile;
    if (index->space->code_dim == 2048) return index->device_bytes > 4 * l2_bytes(index->device) ? 0 : 4;
    return 0;
}

bool search_launch_geometry(const qg_index *index, int l_cap, bool stop_model, int *wpb_out, int *per_sm_out) {
    const int D = static_cast<int>(index->space->code_dim);
    const int tile = search_tile(index);
    int wpb = 0, per_sm = 0;
    const int wmax = search_max_block_warps(D, tile);
    if (index->launch_wpb > 0) {
        wpb = std::min(index->launch_wpb, wmax);  // the override, within this instantiation's block
        per_sm = search_blocks_per_sm(D, l_cap, wpb, stop_model, tile);
        if (index->launch_per_sm > 0 && index->launch_per_sm < per_sm) per_sm = index->launch_per_sm;
    } else {
        // the most warps per SM; a tie keeps the earlier candidate
        for (int cand : {search_first_block_warps(D, tile), wmax, wmax / 2, wmax / 4}) {
            if (cand < 1) continue;
            const int b = search_blocks_per_sm(D, l_cap, cand, stop_model, tile);
            if (b * cand > per_sm * wpb) {
                wpb = cand;
                per_sm = b;
            }
        }
    }
    if (per_sm <= 0 || wpb <= 0) {
        set_error("search kernel cannot be resident with this pool size and launch shape");
        return false;
    }
    *wpb_out = wpb;
    *per_sm_out = per_sm;
    return true;
}

int search_args_fill(const qg_index *index, size_t nq, const qg_search_params *params, const float *d_queries,
                     const int *d_k, const int *d_l, size_t k_stride, uint32_t *d_ids, float *d_dists,
                     qg_search_stats *d_stats, SearchArgs *out) {
    if (!index || !params || !out || (nq && (!d_queries || !d_ids || !d_dists))) {
        set_error("search: null argument");
        return QG_ERR_INVALID;
    }
    if (nq > 0x7FFFFFFF) {
        set_error("search: more than 2^31 - 1 queries in one batch");
        return QG_ERR_INVALID;
    }
    const Space *s = index->space;
    const int k_max = d_k ? static_cast<int>(k_stride) : params->k;
    if (k_max <= 0 || (d_k == nullptr && k_stride != 0 && k_stride < static_cast<size_t>(params->k))) {
        set_error("k must be positive and fit the output stride");
        return QG_ERR_INVALID;
    }
    const int l_cap = std::max(params->l_value, k_max);
    if (l_cap > 4096 || params->beam_width < 1 || params->beam_width > 8 || params->rerank_candidates < 0) {
        set_error("L must be <= 4096 and beam width 1..8");
        return QG_ERR_INVALID;
    }
    if (!space_query_bits(s)) {
        set_error("the GPU query path implements the Full (0), B1 (1), Int4 (2), Int8 (3) and B1Main (4) "
                  "query codecs");
        return QG_ERR_INVALID;
    }
    SearchArgs a{};
    a.ix = index->ix;
    a.nq = static_cast<int>(nq);
    a.k_default = params->k;
    a.l_default = params->l_value;
    a.k_per_q = d_k;
    a.l_per_q = d_l;
    a.k_stride = k_max;
    a.l_cap = l_cap;
    a.beam_width = params->beam_width;
    a.tile = search_tile(index);
    a.eps = params->epsilon0;
    a.rerank = params->rerank_candidates;
    a.early_stop_hops = params->early_stop_hops;
    a.kth_stop = params->kth_stop;
    // the rerank residual in the fused kernel's order: the fused Int8 / Int4 rerank, or
    // FullRerankScalar's per-record residual path
    a.fused_rerank = ((space_search_mode(s) == 0 && params->fused_int_rerank != 0) || s->codec == 6) ? 1 : 0;
    a.mode = space_search_mode(s);
    a.ids_out = d_ids;
    a.dists_out = d_dists;
    a.stats_out = d_stats;
    a.hop_cap = static_cast<int>(std::min<size_t>(static_cast<size_t>(index->ix.n_total) + 1, 0x7FFFFFFF));
    a.stop_every = 1;
    *out = a;
    return QG_OK;
}

}  // namespace qg

using namespace qg;

extern "C" {

const char *qg_last_error(void) { return g_last_error.c_str(); }

int qg_device_sm_count(void) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return sms;
}

void *rabitq_space_new(size_t dim, uint32_t seed, size_t centroid_count, size_t residual_bits,
                       size_t residual_block_size, bool residual_mse, bool residual_fp16) {
    try {
        if (dim == 0 || centroid_count != 1 || residual_bits != 4 || residual_block_size != 16 ||
            !residual_mse || !residual_fp16) {
            set_error("only the formal config is supported: K=1, 4-bit residual, block 16, mse, fp16");
            return nullptr;
        }
        auto *s = new Space();
        s->dim = dim;
        s->code_dim = round_up_code_dim(dim);
        if (!search_supported_dim(static_cast<int>(s->code_dim))) {
            set_error("code dim must be 64..2048");
            delete s;
            return nullptr;
        }
        s->code_bytes = s->code_dim / 2;
        s->block_count = s->code_dim / 16;
        s->scale_bytes = s->block_count * 2;
        s->full_bytes = 24 + s->scale_bytes + s->code_bytes + 1 + s->code_bytes;
        s->compact_bytes = 16 + s->code_bytes + 1;
        s->residual_bytes = 8 + s->scale_bytes + s->code_bytes;
        s->msb_bytes = s->code_dim / 8;
        s->seed = seed;
        s->codec = 0;
        cudaGetDevice(&s->device);
        const float inv = 1.0f / std::sqrt(static_cast<float>(s->code_dim));
        s->signs.assign(s->code_dim, inv);
        if (seed != 0) {  // setRandomRotation (space_rabitq.h:2900-2912)
            std::mt19937 rng(seed);
            std::uniform_int_distribution<int> bernoulli(0, 1);
            for (size_t i = 0; i < s->code_dim; ++i) s->signs[i] = (bernoulli(rng) ? 1.0f : -1.0f) * inv;
        }
        // seed 0 selects the identity rotation in the reference (space_rabitq.h:990-995);
        // the GPU kernels always rotate, so it is rejected here.
        if (seed == 0) {
            set_error("seed 0 (identity rotation) is not supported");
            delete s;
            return nullptr;
        }
        s->center.assign(dim, 0.0f);
        s->d_signs = dev_alloc<float>(s->code_dim);
        s->d_center = dev_alloc<float>(dim);
        s->d_rotated_center = dev_alloc<float>(s->code_dim);
        s->d_center_norm = dev_alloc<float>(1);
        if (!s->d_signs || !s->d_center || !s->d_rotated_center || !s->d_center_norm) {
            set_error("device allocation failed");
            rabitq_space_delete(s);
            return nullptr;
        }
        cudaMemcpy(s->d_signs, s->signs.data(), s->code_dim * 4, cudaMemcpyHostToDevice);
        if (!rabitq_space_set_center(s, s->center.data())) {
            rabitq_space_delete(s);
            return nullptr;
        }
        s->center_set = false;
        return s;
    } catch (...) {
        return nullptr;
    }
}

void rabitq_space_delete(void *space) {
    auto *s = static_cast<Space *>(space);
    if (!s) return;
    cudaFree(s->d_signs);
    cudaFree(s->d_center);
    cudaFree(s->d_rotated_center);
    cudaFree(s->d_center_norm);
    cudaFree(s->d_rot_gemm_b);
    delete s;
}

bool rabitq_space_set_center(void *space, const float *center) {
    try {
        auto *s = static_cast<Space *>(space);
        if (!s || !center) return false;
        std::copy(center, center + s->dim, s->center.begin());
        if (!cuda_ok(cudaMemcpy(s->d_center, center, s->dim * 4, cudaMemcpyHostToDevice), "center upload"))
            return false;
        if (!cuda_ok(launch_center_setup(s->d_center, s->d_signs, static_cast<int>(s->dim),
                                         static_cast<int>(s->code_dim), s->d_rotated_center,
                                         s->d_center_norm, nullptr), "center setup"))
            return false;
        if (!cuda_ok(cudaMemcpy(&s->center_norm_sqr, s->d_center_norm, 4, cudaMemcpyDeviceToHost), "center norm"))
            return false;
        s->center_set = true;
        return true;
    } catch (...) {
        return false;
    }
}

// The rotation's sign vector (+-1/sqrt(D), code_dim floats): read, or replaced as
// RaBitQSpace::loadState does with the stored fht_signs_ (space_rabitq.h:3318-3336); a set
// centre is re-rotated with the new signs.
bool qg_space_signs(const void *space, float *out) {
    const Space *s = as_space(space);
    if (!s || !out) return false;
    std::copy(s->signs.begin(), s->signs.end(), out);
    return true;
}

bool qg_space_set_signs(void *space, const float *signs) {
    try {
        auto *s = static_cast<Space *>(space);
        if (!s || !signs) return false;
        std::copy(signs, signs + s->code_dim, s->signs.begin());
        if (!cuda_ok(cudaMemcpy(s->d_signs, signs, s->code_dim * 4, cudaMemcpyHostToDevice), "signs upload"))
            return false;
        cudaFree(s->d_rot_gemm_b);  // built from the signs: rebuilt on next use
        s->d_rot_gemm_b = nullptr;
        if (s->center_set) {
            std::vector<float> c(s->center);
            return rabitq_space_set_center(space, c.data());
        }
        return true;
    } catch (...) {
        return false;
    }
}

bool rabitq_space_set_centroids(void *space, const float *centroids, size_t centroid_count) {
    if (centroid_count != 1) {
        set_error("only one centroid is supported");
        return false;
    }
    return rabitq_space_set_center(space, centroids);
}

// rabitq_bridge.cpp:101-172: host k-means used only to pick K > 1 centroids (not on the
// query path). Same sampling and update rules.
bool rabitq_train_centroids(const float *data, size_t count, size_t dim, size_t k,
                            size_t sample_count, uint32_t seed, int iters, float *out) {
    try {
        if (!data || !out || count == 0 || dim == 0 || k == 0 || k > 256 || sample_count == 0) return false;
        sample_count = std::min(sample_count, count);
        std::mt19937 rng(seed);
        std::vector<size_t> sample(sample_count);
        for (size_t i = 0; i < sample_count; ++i) sample[i] = static_cast<size_t>(rng()) % count;
        std::vector<float> cent(k * dim), next(k * dim);
        std::vector<size_t> cnt(k);
        for (size_t c = 0; c < k; ++c) {
            const float *src = data + sample[c % sample_count] * dim;
            std::copy(src, src + dim, cent.begin() + static_cast<long>(c * dim));
        }
        for (int it = 0; it < iters; ++it) {
            std::fill(next.begin(), next.end(), 0.0f);
            std::fill(cnt.begin(), cnt.end(), 0);
            for (size_t i = 0; i < sample_count; ++i) {
                const float *v = data + sample[i] * dim;
                size_t best = 0;
                float best_d = std::numeric_limits<float>::infinity();
                for (size_t c = 0; c < k; ++c) {
                    float d = 0.0f;
                    for (size_t j = 0; j < dim; ++j) {
                        const float diff = v[j] - cent[c * dim + j];
                        d += diff * diff;
                    }
                    if (d < best_d) {
                        best_d = d;
                        best = c;
                    }
                }
                for (size_t j = 0; j < dim; ++j) next[best * dim + j] += v[j];
                ++cnt[best];
            }
            for (size_t c = 0; c < k; ++c) {
                if (cnt[c] == 0) continue;
                const float inv = 1.0f / static_cast<float>(cnt[c]);
                for (size_t j = 0; j < dim; ++j) cent[c * dim + j] = next[c * dim + j] * inv;
            }
        }
        std::copy(cent.begin(), cent.end(), out);
        return true;
    } catch (...) {
        return false;
    }
}

size_t rabitq_full_record_bytes(const void *space) { return as_space(space)->full_bytes; }
size_t rabitq_compact_record_bytes(const void *space) { return as_space(space)->compact_bytes; }
size_t rabitq_residual_record_bytes(const void *space) { return as_space(space)->residual_bytes; }
size_t rabitq_residual_block_size(const void *space) { return space ? 16 : 0; }
size_t rabitq_residual_bits(const void *space) { return space ? 4 : 0; }
size_t rabitq_paper_msb_code_bytes(const void *space) { return space ? as_space(space)->msb_bytes : 0; }
size_t rabitq_paper_factor_bytes(void) { return sizeof(RabitqPaperFactors); }

bool rabitq_encode_full(const void *space, const float *raw, void *encoded_out) {
    try {
        const Space *s = as_space(space);
        if (!s || !raw || !encoded_out) return false;
        std::vector<uint8_t> compact(s->compact_bytes), residual(s->residual_bytes);
        if (!encode_host(s, raw, 1, compact.data(), residual.data())) return false;
        assemble_full(s, compact.data(), residual.data(), static_cast<uint8_t *>(encoded_out));
        return true;
    } catch (...) {
        return false;
    }
}

bool rabitq_copy_compact(const void *space, const void *full_encoded, void *compact_out) {
    const Space *s = as_space(space);
    if (!s || !full_encoded || !compact_out) return false;
    const uint8_t *f = static_cast<const uint8_t *>(full_encoded);
    uint8_t *c = static_cast<uint8_t *>(compact_out);
    std::memcpy(c, f, 16);
    std::memcpy(c + 16, f + 24 + s->scale_bytes, s->code_bytes);
    c[16 + s->code_bytes] = f[24 + s->scale_bytes + s->code_bytes];
    return true;
}

bool rabitq_copy_residual_record(const void *space, const void *full_encoded, void *residual_out) {
    const Space *s = as_space(space);
    if (!s || !full_encoded || !residual_out) return false;
    const uint8_t *f = static_cast<const uint8_t *>(full_encoded);
    uint8_t *r = static_cast<uint8_t *>(residual_out);
    std::memcpy(r, f + 16, 8);
    std::memcpy(r + 8, f + 24, s->scale_bytes);
    std::memcpy(r + 8 + s->scale_bytes, f + 25 + s->scale_bytes + s->code_bytes, s->code_bytes);
    return true;
}

bool rabitq_build_vamana_graph(void *space, const void *compact_records_in, size_t record_count,
                               size_t compact_stride, size_t r, size_t l_build, float alpha,
                               size_t beam_width, size_t batch_size, size_t refine_passes,
                               size_t prune_candidate_cap, size_t build_early_stop_hops,
                               uint32_t *degrees_out, uint32_t *edges_out, size_t edge_stride,
                               uint8_t *paper_msb_out, void *paper_factors_out,
                               size_t *paper_msb_stride_out, size_t *paper_factor_bytes_out,
                               uint64_t *distance_evaluations_out) {
    try {
        const Space *s = as_space(space);
        if (!s || (!compact_records_in && record_count != 0) || !degrees_out || !edges_out || edge_stride < r ||
            !paper_msb_out || !paper_factors_out || !paper_msb_stride_out || !paper_factor_bytes_out ||
            compact_stride < s->compact_bytes)
            return false;
        Carve c;
        const size_t o_c = c.take(record_count * compact_stride), o_d = c.take(record_count * 4),
                     o_e = c.take(record_count * edge_stride * 4);
        if (!t_stage.reserve(c.off)) return false;
        uint8_t *d = static_cast<uint8_t *>(t_stage.d);
        cudaStream_t st = t_stage.stream;
        if (record_count && !cuda_ok(cudaMemcpyAsync(d + o_c, compact_records_in, record_count * compact_stride,
                                                     cudaMemcpyHostToDevice, st),
                                     "build upload"))
            return false;
        uint64_t evals = 0;
        if (qg_build_vamana_device(s, d + o_c, record_count, compact_stride, r, l_build, alpha, beam_width,
                                   batch_size, refine_passes, prune_candidate_cap, build_early_stop_hops,
                                   reinterpret_cast<uint32_t *>(d + o_d), reinterpret_cast<uint32_t *>(d + o_e),
                                   edge_stride, &evals, st) != QG_OK)
            return false;
        if (record_count &&
            (!cuda_ok(cudaMemcpyAsync(degrees_out, d + o_d, record_count * 4, cudaMemcpyDeviceToHost, st),
                      "build download") ||
             !cuda_ok(cudaMemcpyAsync(edges_out, d + o_e, record_count * edge_stride * 4, cudaMemcpyDeviceToHost,
                                      st),
                      "build download") ||
             !cuda_ok(cudaStreamSynchronize(st), "build sync")))
            return false;
        if (!rabitq_export_paper_sidecar(space, compact_records_in, record_count, compact_stride, paper_msb_out,
                                         paper_factors_out))
            return false;
        *paper_msb_stride_out = s->msb_bytes;
        *paper_factor_bytes_out = 20;
        if (distance_evaluations_out) *distance_evaluations_out = evals;
        return true;
    } catch (...) {
        return false;
    }
}

bool rabitq_export_paper_sidecar(const void *space, const void *compact_records_in,
                                 size_t record_count, size_t compact_stride, uint8_t *msb_out,
                                 void *factors_out) {
    try {
        const Space *s = as_space(space);
        if (!s || (!compact_records_in && record_count != 0) || !msb_out || !factors_out) return false;
        if (record_count == 0) return true;
        Carve c;
        const size_t o_c = c.take(record_count * compact_stride), o_m = c.take(record_count * s->msb_bytes),
                     o_f = c.take(record_count * 20);
        if (!t_stage.reserve(c.off)) return false;
        uint8_t *d = static_cast<uint8_t *>(t_stage.d);
        cudaStream_t st = t_stage.stream;
        if (!cuda_ok(cudaMemcpyAsync(d + o_c, compact_records_in, record_count * compact_stride,
                                     cudaMemcpyHostToDevice, st), "sidecar upload"))
            return false;
        if (qg_export_sidecar_device(s, d + o_c, record_count, compact_stride, d + o_m, d + o_f, st) != QG_OK)
            return false;
        if (!cuda_ok(cudaMemcpyAsync(msb_out, d + o_m, record_count * s->msb_bytes, cudaMemcpyDeviceToHost, st),
                     "sidecar download"))
            return false;
        if (!cuda_ok(cudaMemcpyAsync(factors_out, d + o_f, record_count * 20, cudaMemcpyDeviceToHost, st),
                     "sidecar download"))
            return false;
        return cuda_ok(cudaStreamSynchronize(st), "sidecar sync");
    } catch (...) {
        return false;
    }
}

float rabitq_symmetric_distance(const void *space, const void *lhs, const void *rhs) {
    const float inf = std::numeric_limits<float>::infinity();
    try {
        const Space *s = as_space(space);
        if (!s || !lhs || !rhs) return inf;
        const size_t rb = s->compact_bytes;
        Carve c;
        const size_t o_a = c.take(rb), o_b = c.take(rb), o_o = c.take(4);
        if (!t_stage.reserve(c.off)) return inf;
        uint8_t *h = static_cast<uint8_t *>(t_stage.h), *d = static_cast<uint8_t *>(t_stage.d);
        std::memcpy(h + o_a, lhs, rb);
        std::memcpy(h + o_b, rhs, rb);
        cudaStream_t st = t_stage.stream;
        if (!cuda_ok(cudaMemcpyAsync(d, h, o_o, cudaMemcpyHostToDevice, st), "symmetric upload")) return inf;
        if (!cuda_ok(launch_symmetric_pairs(static_cast<int>(s->code_dim), d + o_a, d + o_b, 1, rb,
                                            reinterpret_cast<float *>(d + o_o), st), "symmetric kernel"))
            return inf;
        float out = inf;
        if (!cuda_ok(cudaMemcpyAsync(h + o_o, d + o_o, 4, cudaMemcpyDeviceToHost, st), "symmetric download")) return inf;
        if (!cuda_ok(cudaStreamSynchronize(st), "symmetric sync")) return inf;
        std::memcpy(&out, h + o_o, 4);
        return out;
    } catch (...) {
        return inf;
    }
}

const void *rabitq_prepare_query(const void *space, const float *query) {
    try {
        const Space *s = as_space(space);
        if (!s || !query) return nullptr;
        if (!space_query_bits(s)) {
            set_error("the GPU query path implements the Full (0), B1 (1), Int4 (2), Int8 (3) and B1Main (4) "
                      "query codecs");
            return nullptr;
        }
        Prepared &p = t_prepared;
        p.valid = false;
        if (!p.ensure(s)) return nullptr;
        if (!cuda_ok(cudaMemcpy(p.d_query, query, s->dim * 4, cudaMemcpyHostToDevice), "query upload")) return nullptr;
        if (qg_prepare_batch(s, p.d_query, 1, p.d_rr, p.d_codes, reinterpret_cast<float *>(p.d_scal),
                             reinterpret_cast<int64_t *>(p.d_csum), nullptr) != QG_OK)
            return nullptr;
        if (!cuda_ok(cudaMemcpy(&p.h_scal, p.d_scal, sizeof(float4), cudaMemcpyDeviceToHost), "prepare download"))
            return nullptr;
        if (!cuda_ok(cudaMemcpy(&p.h_csum, p.d_csum, 8, cudaMemcpyDeviceToHost), "prepare download")) return nullptr;
        p.space = s;
        p.codec = s->codec;
        p.valid = true;
        return &p;
    } catch (...) {
        return nullptr;
    }
}

void rabitq_set_query_coarse_codec(void *space, int codec) {
    // the reference stores static_cast<QueryCoarseCodec>(codec), an 8-bit enum
    if (space) static_cast<Space *>(space)->codec = static_cast<uint8_t>(codec);
}

void rabitq_release_query(const void *space, const void *prepared) {
    (void)space;
    (void)prepared;
}

float rabitq_query_distance(const void *space, const void *prepared, const void *encoded) {
    const float inf = std::numeric_limits<float>::infinity();
    try {
        const Space *s = as_space(space);
        if (!check_prepared(s, prepared) || !encoded) return inf;
        const uint32_t id = 0;
        const uint8_t mode = 0;
        const float sip = 0.0f;
        float out = inf;
        if (!distance_host(s, &id, &mode, 1, static_cast<const uint8_t *>(encoded), s->compact_bytes, &sip, &out))
            return inf;
        return out;
    } catch (...) {
        return inf;
    }
}

float rabitq_query_distance_b1(const void *space, const void *prepared, const void *encoded) {
    const float inf = std::numeric_limits<float>::infinity();
    try {
        const Space *s = as_space(space);
        if (!check_prepared(s, prepared) || !encoded) return inf;
        if (t_prepared.codec != 4 && t_prepared.codec != 1) {
            set_error("rabitq_query_distance_b1: prepare the query with the B1Main (4) or B1 (1) codec");
            return inf;
        }
        const uint32_t id = 0;
        float out = inf;
        if (!distance_b1_host(s, &id, 1, static_cast<const uint8_t *>(encoded), s->compact_bytes, &out)) return inf;
        return out;
    } catch (...) {
        return inf;
    }
}

bool rabitq_query_distance_b1_batch(const void *space, const void *prepared, const uint32_t *ids, size_t count,
                                    const void *encoded_base, size_t encoded_stride, float *out_distances) {
    const float inf = std::numeric_limits<float>::infinity();
    try {
        const Space *s = as_space(space);
        if (!out_distances) return false;
        bool ok = check_prepared(s, prepared) && ids && encoded_base && (t_prepared.codec == 4 || t_prepared.codec == 1);
        for (size_t b = 0; ok && b < count; b += 4096) {
            const size_t n = std::min<size_t>(4096, count - b);
            ok = distance_b1_host(s, ids + b, n, static_cast<const uint8_t *>(encoded_base), encoded_stride,
                                  out_distances + b);
        }
        if (!ok)
            for (size_t i = 0; i < count; ++i) out_distances[i] = inf;  // the reference's failure sentinel
        return true;
    } catch (...) {
        for (size_t i = 0; i < count; ++i) out_distances[i] = inf;
        return true;
    }
}

RabitqPaperEstimate rabitq_paper_estimate_sidecar(const void *space, const void *prepared,
                                                  const uint8_t *msb_code, const void *factors,
                                                  float epsilon0) {
    try {
        const Space *s = as_space(space);
        if (!check_prepared(s, prepared) || !msb_code || !factors) return zero_estimate();
        const uint32_t id = 0;
        RabitqPaperEstimate out = zero_estimate();
        if (!gate_host(s, &id, 1, msb_code, s->msb_bytes, static_cast<const uint8_t *>(factors), 20,
                       epsilon0, &out))
            return zero_estimate();
        return out;
    } catch (...) {
        return zero_estimate();
    }
}

// compute_paper_prune_estimate: the bound from the encoded record itself (not the sidecar gate)
RabitqPaperEstimate rabitq_paper_estimate(const void *space, const void *prepared,
                                          const void *encoded, float epsilon0) {
    try {
        const Space *s = as_space(space);
        if (!check_prepared(s, prepared) || !encoded) return zero_estimate();
        const uint32_t id = 0;
        RabitqPaperEstimate out = zero_estimate();
        if (!gate_encoded_host(s, &id, 1, static_cast<const uint8_t *>(encoded), s->compact_bytes, epsilon0, &out))
            return zero_estimate();
        return out;
    } catch (...) {
        return zero_estimate();
    }
}

RabitqPaperEstimate rabitq_paper_estimate_codec(const void *space, const void *prepared,
                                                const void *encoded, const uint8_t *msb_code,
                                                const void *factors, float epsilon0) {
    (void)encoded;
    return rabitq_paper_estimate_sidecar(space, prepared, msb_code, factors, epsilon0);
}

bool rabitq_paper_estimate_batch_sidecar(const void *space, const void *prepared,
                                         const uint32_t *ids, size_t count,
                                         const uint8_t *msb_base, size_t msb_stride,
                                         const void *factors_base, size_t factors_stride,
                                         float epsilon0, RabitqPaperEstimate *out) {
    try {
        const Space *s = as_space(space);
        bool ok = check_prepared(s, prepared) && ids && msb_base && factors_base;
        if (ok && count)
            ok = gate_host(s, ids, count, msb_base, msb_stride, static_cast<const uint8_t *>(factors_base),
                           factors_stride, epsilon0, out);
        if (!ok)
            for (size_t i = 0; i < count; ++i) out[i] = zero_estimate();
        return true;
    } catch (...) {
        for (size_t i = 0; i < count; ++i) out[i] = zero_estimate();
        return true;
    }
}

bool rabitq_paper_estimate_codec_batch(const void *space, const void *prepared,
                                       const uint32_t *ids, size_t count,
                                       const void *encoded_base, size_t encoded_stride,
                                       const uint8_t *msb_base, size_t msb_stride,
                                       const void *factors_base, size_t factors_stride,
                                       float epsilon0, RabitqPaperEstimate *out) {
    (void)encoded_base;
    (void)encoded_stride;
    return rabitq_paper_estimate_batch_sidecar(space, prepared, ids, count, msb_base, msb_stride,
                                               factors_base, factors_stride, epsilon0, out);
}

bool rabitq_paper_estimate_batch(const void *space, const void *prepared, const uint32_t *ids,
                                 size_t count, const void *encoded_base, size_t encoded_stride,
                                 float epsilon0, RabitqPaperEstimate *out) {
    try {
        const Space *s = as_space(space);
        bool ok = check_prepared(s, prepared) && ids && encoded_base;
        for (size_t b = 0; ok && b < count; b += 4096) {
            const size_t n = std::min<size_t>(4096, count - b);
            ok = gate_encoded_host(s, ids + b, n, static_cast<const uint8_t *>(encoded_base), encoded_stride,
                                   epsilon0, out + b);
        }
        if (!ok)
            for (size_t i = 0; i < count; ++i) out[i] = zero_estimate();
        return true;
    } catch (...) {
        for (size_t i = 0; i < count; ++i) out[i] = zero_estimate();
        return true;
    }
}

float rabitq_query_distance_with_paper(const void *space, const void *prepared, const void *encoded,
                                       float short_ip) {
    const float inf = std::numeric_limits<float>::infinity();
    try {
        const Space *s = as_space(space);
        if (!check_prepared(s, prepared) || !encoded) return inf;
        const uint32_t id = 0;
        const uint8_t mode = 1;
        float out = inf;
        if (!distance_host(s, &id, &mode, 1, static_cast<const uint8_t *>(encoded), s->compact_bytes, &short_ip,
                           &out))
            return inf;
        return out;
    } catch (...) {
        return inf;
    }
}

float rabitq_query_distance_with_quantized_paper(const void *space, const void *prepared,
                                                 const void *encoded, float short_ip) {
    const float inf = std::numeric_limits<float>::infinity();
    try {
        const Space *s = as_space(space);
        if (!check_prepared(s, prepared) || !encoded || codec_search_mode(t_prepared.codec) != 0) return inf;
        const uint32_t id = 0;
        const uint8_t mode = 2;
        float out = inf;
        if (!distance_host(s, &id, &mode, 1, static_cast<const uint8_t *>(encoded), s->compact_bytes,
                           &short_ip, &out))
            return inf;
        return out;
    } catch (...) {
        return inf;
    }
}

bool rabitq_query_distance_batch(const void *space, const void *prepared, const uint32_t *ids,
                                 const uint8_t *modes, size_t count, const void *encoded_base,
                                 size_t encoded_stride, const float *short_ips,
                                 float *out_distances) {
    const float inf = std::numeric_limits<float>::infinity();
    try {
        const Space *s = as_space(space);
        bool ok = check_prepared(s, prepared) && ids && modes && encoded_base;
        if (ok && count)
            ok = distance_host(s, ids, modes, count, static_cast<const uint8_t *>(encoded_base),
                               encoded_stride, short_ips, out_distances);
        if (!ok) std::fill(out_distances, out_distances + count, inf);
        // mode 2 reads the integer query codes, which only Int8 / Int4 prepare
        for (size_t i = 0; ok && i < count; ++i)
            if (modes[i] == 2 && codec_search_mode(t_prepared.codec) != 0) out_distances[i] = inf;
        return true;
    } catch (...) {
        std::fill(out_distances, out_distances + count, inf);
        return true;
    }
}

RabitqDistanceInterval rabitq_residual_distance(const void *, const void *, const void *,
                                                float long_distance) {
    return RabitqDistanceInterval{long_distance, long_distance, long_distance};
}

RabitqDistanceInterval rabitq_residual_distance_from_record(const void *space,
                                                            const void *prepared,
                                                            const void *encoded,
                                                            const void *residual_record,
                                                            float long_distance) {
    const RabitqDistanceInterval fallback{long_distance, long_distance, long_distance};
    try {
        const Space *s = as_space(space);
        (void)encoded;
        if (!check_prepared(s, prepared) || !residual_record) return fallback;
        const uint32_t id = 0;
        RabitqDistanceInterval out = fallback;
        // compute_residual_distance_interval_from_record: the per-record path, whose products take
        // the fused kernel's order (residualInt4IpAvx2, space_rabitq.h:2278-2325)
        if (!residual_host(s, &id, 1, static_cast<const uint8_t *>(residual_record), s->residual_bytes,
                           &long_distance, &out, true))
            return fallback;
        return out;
    } catch (...) {
        return fallback;
    }
}

static bool residual_batch(const void *space, const void *prepared, const uint32_t *ids, size_t count,
                           const void *residual_base, size_t residual_stride, const float *long_distances,
                           RabitqDistanceInterval *out, bool fused) {
    try {
        const Space *s = as_space(space);
        bool ok = check_prepared(s, prepared) && ids && residual_base && long_distances;
        if (ok && count)
            ok = residual_host(s, ids, count, static_cast<const uint8_t *>(residual_base), residual_stride,
                               long_distances, out, fused);
        if (!ok)
            for (size_t i = 0; i < count; ++i)
                out[i] = RabitqDistanceInterval{long_distances[i], long_distances[i], long_distances[i]};
        return true;
    } catch (...) {
        for (size_t i = 0; i < count; ++i)
            out[i] = RabitqDistanceInterval{long_distances[i], long_distances[i], long_distances[i]};
        return true;
    }
}

bool rabitq_residual_distance_batch(const void *space, const void *prepared, const uint32_t *ids,
                                    size_t count, const void *encoded_base,
                                    size_t encoded_stride, const void *residual_base,
                                    size_t residual_stride, const float *long_distances,
                                    RabitqDistanceInterval *out) {
    (void)encoded_base;
    (void)encoded_stride;
    // FullRerankScalar (6) takes the per-record path (rabitq_bridge.cpp:987-1040), in the fused order
    const Space *s = as_space(space);
    return residual_batch(space, prepared, ids, count, residual_base, residual_stride, long_distances, out,
                          s && s->codec == 6);
}

bool rabitq_full_residual_distance_batch(const void *space, const void *prepared,
                                         const uint32_t *ids, size_t count,
                                         const void *encoded_base, size_t encoded_stride,
                                         const void *residual_base, size_t residual_stride,
                                         RabitqDistanceInterval *out) {
    // compute_full_residual_distance_intervals_batch_by_id: per record, the FP32 restore (mode 0)
    // and the residual in the fused kernel's product order (space_rabitq.h:5700-5743); a record
    // whose restore is not finite keeps its own result. The reference runs 64-record chunks and
    // fills only a chunk that throws with +inf (rabitq_bridge.cpp:1044-1084); its chunks throw
    // only on whole-call conditions (no space, no prepared query, null bases), which fail every
    // chunk alike, so filling every item with +inf on a failure gives the same output.
    const float inf = std::numeric_limits<float>::infinity();
    try {
        const Space *s = as_space(space);
        bool ok = check_prepared(s, prepared) && ids && encoded_base && residual_base;
        std::vector<float> longd(count, inf);
        if (ok && count) {
            std::vector<uint8_t> modes(count, 0);
            ok = distance_host(s, ids, modes.data(), count, static_cast<const uint8_t *>(encoded_base), encoded_stride,
                               nullptr, longd.data());
        }
        if (ok && count)
            ok = residual_host(s, ids, count, static_cast<const uint8_t *>(residual_base), residual_stride,
                               longd.data(), out, true);
        if (!ok)
            for (size_t i = 0; i < count; ++i) out[i] = RabitqDistanceInterval{inf, inf, inf};
        return true;
    } catch (...) {
        for (size_t i = 0; i < count; ++i) out[i] = RabitqDistanceInterval{inf, inf, inf};
        return true;
    }
}

// ---------------------------------------------------------------------------------------
// qg_* batched device entry points
// ---------------------------------------------------------------------------------------

int qg_center_mean(const float *d_data, size_t stride, size_t dim, const uint32_t *d_rows,
                   size_t count, float *d_center_out, void *stream) {
    if (!d_data || !d_center_out || count == 0 || dim == 0 || stride < dim) return QG_ERR_INVALID;
    if (!cuda_ok(launch_center_mean(d_data, stride, static_cast<int>(dim), d_rows, count, d_center_out,
                                    static_cast<cudaStream_t>(stream)), "center kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_encode_batch(const void *space, const float *d_raw, size_t n, uint8_t *d_compact,
                    uint8_t *d_residual, void *stream) {
    const Space *s = as_space(space);
    if (!s || (n && (!d_raw || !d_compact || !d_residual))) return QG_ERR_INVALID;
    if (!s->center_set) {
        set_error("set the centre before encoding");
        return QG_ERR_INVALID;
    }
    EncodeArgs a{d_raw, s->dim, 0, static_cast<int>(s->dim), static_cast<int>(s->code_dim), s->d_signs,
                 s->d_center, d_compact, d_residual, s->compact_bytes, s->residual_bytes};
    const size_t chunk = 1u << 30;  // grid.x limit headroom
    for (size_t base = 0; base < n; base += chunk) {
        const size_t m = std::min(chunk, n - base);
        a.raw = d_raw + base * s->dim;
        a.n = static_cast<int>(m);
        a.compact = d_compact + base * s->compact_bytes;
        a.residual = d_residual + base * s->residual_bytes;
        if (!cuda_ok(launch_encode(a, static_cast<cudaStream_t>(stream)), "encode kernel")) return QG_ERR_CUDA;
    }
    return QG_OK;
}

// The tensor-core rotation of rows [0, n) into d_rotated [n x code_dim] and d_norms [n], in chunks
// of at most 2^17 rows through a scratch BF16 operand; builds the space's +-1 operand on first use.
static int rotate_gemm_rows(Space *s, const float *d_raw, size_t n, float *d_rotated, float *d_norms,
                            cudaStream_t st) {
    const int dim = static_cast<int>(s->dim), D = static_cast<int>(s->code_dim);
    if (!rotate_gemm_supported(D)) {
        set_error("the tensor-core rotation needs a code dim that is a multiple of 256");
        return QG_ERR_UNSUPPORTED;
    }
    const size_t kp3 = 3 * static_cast<size_t>(rotate_gemm_kp(dim));
    if (!s->d_rot_gemm_b) {
        s->d_rot_gemm_b = dev_alloc<uint16_t>(static_cast<size_t>(D) * kp3);
        if (!s->d_rot_gemm_b) {
            set_error("device allocation failed for the rotation operand");
            return QG_ERR_OOM;
        }
        if (!cuda_ok(launch_r_matrix(s->d_signs, dim, D, s->d_rot_gemm_b, st), "rotation operand") ||
            !cuda_ok(cudaStreamSynchronize(st), "rotation operand")) {
            cudaFree(s->d_rot_gemm_b);
            s->d_rot_gemm_b = nullptr;
            return QG_ERR_CUDA;
        }
    }
    const size_t chunk = std::min<size_t>(n, 1u << 17);
    uint16_t *a3 = dev_alloc<uint16_t>(chunk * kp3);
    int *status = dev_alloc<int>(1);
    if (!a3 || !status) {
        cudaFree(a3);
        cudaFree(status);
        set_error("device allocation failed for the rotation scratch");
        return QG_ERR_OOM;
    }
    int rc = QG_OK;
    const float c_abs = std::fabs(s->signs[0]);
    if (!cuda_ok(cudaMemsetAsync(status, 0, 4, st), "rotation status")) rc = QG_ERR_CUDA;
    for (size_t base = 0; base < n && rc == QG_OK; base += chunk) {
        const int m = static_cast<int>(std::min(chunk, n - base));
        if (!cuda_ok(launch_rotate_split(d_raw + base * s->dim, s->dim, m, dim, s->d_center, c_abs, a3,
                                         d_norms + base, st), "rotation split") ||
            !cuda_ok(launch_rotate_gemm(a3, s->d_rot_gemm_b, m, dim, D, d_rotated + base * D, status, st),
                     "rotation gemm"))
            rc = QG_ERR_CUDA;
    }
    int h = 0;
    if (rc == QG_OK && (!cuda_ok(cudaMemcpyAsync(&h, status, 4, cudaMemcpyDeviceToHost, st), "rotation status") ||
                        !cuda_ok(cudaStreamSynchronize(st), "rotation sync")))
        rc = QG_ERR_CUDA;
    if (rc == QG_OK && h) {
        set_error("the rotation GEMM timed out waiting for its tiles");
        rc = QG_ERR_TIMEOUT;
    }
    cudaStreamSynchronize(st);
    cudaFree(a3);
    cudaFree(status);
    return rc;
}

int qg_rotate_gemm(const void *space, const float *d_raw, size_t n, float *d_rotated, float *d_norms, void *stream) {
    Space *s = const_cast<Space *>(as_space(space));
    if (!s || (n && (!d_raw || !d_rotated || !d_norms)) || n > 0x7FFFFFFF) return QG_ERR_INVALID;
    if (!s->center_set) {
        set_error("set the centre before encoding");
        return QG_ERR_INVALID;
    }
    if (n == 0) return QG_OK;
    return rotate_gemm_rows(s, d_raw, n, d_rotated, d_norms, static_cast<cudaStream_t>(stream));
}

int qg_rotate_gemm_planes(const void *space, const uint16_t *d_a3, size_t n, float *d_out, void *stream) {
    Space *s = const_cast<Space *>(as_space(space));
    if (!s || (n && (!d_a3 || !d_out)) || n > 0x7FFFFFFF) return QG_ERR_INVALID;
    if (n == 0) return QG_OK;
    // the space's +-1 operand, built on first use (the same one qg_rotate_gemm uses)
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int dim = static_cast<int>(s->dim), D = static_cast<int>(s->code_dim);
    if (!rotate_gemm_supported(D)) {
        set_error("the tensor-core rotation needs a code dim that is a multiple of 256");
        return QG_ERR_UNSUPPORTED;
    }
    if (!s->d_rot_gemm_b) {
        const size_t kp3 = 3 * static_cast<size_t>(rotate_gemm_kp(dim));
        s->d_rot_gemm_b = dev_alloc<uint16_t>(static_cast<size_t>(D) * kp3);
        if (!s->d_rot_gemm_b) return QG_ERR_OOM;
        if (!cuda_ok(launch_r_matrix(s->d_signs, dim, D, s->d_rot_gemm_b, st), "rotation operand")) return QG_ERR_CUDA;
    }
    int *status = dev_alloc<int>(1);
    if (!status) return QG_ERR_OOM;
    int h = 0, rc = QG_OK;
    if (!cuda_ok(cudaMemsetAsync(status, 0, 4, st), "status") ||
        !cuda_ok(launch_rotate_gemm(d_a3, s->d_rot_gemm_b, static_cast<int>(n), dim, D, d_out, status, st), "gemm") ||
        !cuda_ok(cudaMemcpyAsync(&h, status, 4, cudaMemcpyDeviceToHost, st), "status") ||
        !cuda_ok(cudaStreamSynchronize(st), "sync"))
        rc = QG_ERR_CUDA;
    else if (h)
        rc = QG_ERR_TIMEOUT;
    cudaFree(status);
    return rc;
}

int qg_encode_batch_gemm(const void *space, const float *d_raw, size_t n, uint8_t *d_compact, uint8_t *d_residual,
                         void *stream) {
    Space *s = const_cast<Space *>(as_space(space));
    if (!s || (n && (!d_raw || !d_compact || !d_residual)) || n > 0x7FFFFFFF) return QG_ERR_INVALID;
    if (!s->center_set) {
        set_error("set the centre before encoding");
        return QG_ERR_INVALID;
    }
    if (n == 0) return QG_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t chunk = std::min<size_t>(n, 1u << 17);
    float *rot = dev_alloc<float>(chunk * s->code_dim);
    float *norms = dev_alloc<float>(chunk);
    if (!rot || !norms) {
        cudaFree(rot);
        cudaFree(norms);
        set_error("device allocation failed for the rotated rows");
        return QG_ERR_OOM;
    }
    int rc = QG_OK;
    for (size_t base = 0; base < n && rc == QG_OK; base += chunk) {
        const size_t m = std::min(chunk, n - base);
        rc = rotate_gemm_rows(s, d_raw + base * s->dim, m, rot, norms, st);
        if (rc != QG_OK) break;
        EncodeArgs a{nullptr, s->dim, static_cast<int>(m), static_cast<int>(s->dim), static_cast<int>(s->code_dim),
                     s->d_signs, s->d_center, d_compact + base * s->compact_bytes,
                     d_residual + base * s->residual_bytes, s->compact_bytes, s->residual_bytes, rot, norms};
        if (!cuda_ok(launch_encode(a, st), "encode kernel")) rc = QG_ERR_CUDA;
    }
    cudaStreamSynchronize(st);
    cudaFree(rot);
    cudaFree(norms);
    return rc;
}

int qg_prune_candidates(const void *space, const uint8_t *d_compact, size_t compact_stride, size_t n,
                        const uint32_t *d_candidates, size_t k, size_t r, float alpha,
                        uint32_t *d_degrees, uint32_t *d_edges, size_t edge_stride, void *stream) {
    const Space *s = as_space(space);
    if (!s || (n && (!d_compact || !d_candidates || !d_degrees || !d_edges)) || k == 0 || k > 256 || r == 0 ||
        r > edge_stride || n >= 0x7FFFFFFFu || compact_stride < s->compact_bytes)
        return QG_ERR_INVALID;
    if (!cuda_ok(launch_prune(static_cast<int>(s->code_dim), d_compact, compact_stride, static_cast<int>(n),
                              d_candidates, static_cast<int>(k), static_cast<int>(r), alpha, d_degrees, d_edges,
                              edge_stride, static_cast<cudaStream_t>(stream)),
                 "prune kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_build_vamana_device(const void *space, const uint8_t *d_compact, size_t n, size_t compact_stride,
                           size_t r, size_t l_build, float alpha, size_t beam_width, size_t batch_size,
                           size_t refine_passes, size_t prune_candidate_cap, size_t build_early_stop_hops,
                           uint32_t *d_degrees, uint32_t *d_edges, size_t edge_stride,
                           uint64_t *distance_evaluations, void *stream) {
    const Space *s = as_space(space);
    if (!s || (n && (!d_compact || !d_degrees || !d_edges)) || compact_stride < s->compact_bytes || r == 0 ||
        r > 64 || edge_stride < r || l_build == 0 || beam_width == 0 || beam_width * r > 1024 ||
        !(alpha >= 1.0f) || !std::isfinite(alpha) || n >= 0x7FFFFFFFu) {
        set_error("vamana build: invalid arguments (R <= 64, beam * R <= 1024, alpha >= 1)");
        return QG_ERR_INVALID;
    }
    VbBuildParams p{r, l_build, alpha, beam_width, batch_size, refine_passes, prune_candidate_cap,
                    build_early_stop_hops};
    unsigned long long ev = 0;
    const cudaError_t e = launch_vamana_build(static_cast<int>(s->code_dim), d_compact, n, compact_stride, p,
                                              d_degrees, d_edges, edge_stride, &ev,
                                              static_cast<cudaStream_t>(stream));
    if (e == cudaErrorInvalidValue) {
        set_error("vamana build: a neighbour outside the graph or unsupported arguments");
        return QG_ERR_INVALID;
    }
    if (!cuda_ok(e, "vamana build")) return QG_ERR_CUDA;
    if (distance_evaluations) *distance_evaluations = ev;
    return QG_OK;
}

int qg_export_sidecar_device(const void *space, const uint8_t *d_compact, size_t n,
                             size_t compact_stride, uint8_t *d_msb, void *d_factors, void *stream) {
    const Space *s = as_space(space);
    if (!s || (n && (!d_compact || !d_msb || !d_factors))) return QG_ERR_INVALID;
    if (!cuda_ok(launch_sidecar(d_compact, n, compact_stride, static_cast<int>(s->code_dim), d_msb,
                                static_cast<RabitqPaperFactors *>(d_factors), static_cast<cudaStream_t>(stream)),
                 "sidecar kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_prepare_batch(const void *space, const float *d_queries, size_t nq, float *d_rotated,
                     int8_t *d_codes, float *d_scalars, int64_t *d_code_sum, void *stream) {
    const Space *s = as_space(space);
    if (!s || (nq && (!d_queries || !d_rotated || !d_codes || !d_scalars || !d_code_sum))) return QG_ERR_INVALID;
    if (!s->center_set) {
        set_error("set the centre before preparing queries");
        return QG_ERR_INVALID;
    }
    if (!space_query_bits(s)) {
        set_error("the GPU query path implements the Full (0), B1 (1), Int4 (2), Int8 (3) and B1Main (4) query codecs");
        return QG_ERR_INVALID;
    }
    PrepArgs a{d_queries, s->dim, static_cast<int>(nq), static_cast<int>(s->dim),
               static_cast<int>(s->code_dim), s->d_signs, s->d_center, s->d_rotated_center,
               s->d_center_norm, d_rotated, d_codes, reinterpret_cast<float4 *>(d_scalars),
               reinterpret_cast<long long *>(d_code_sum)};
    a.qbits = space_query_bits(s);
    if (!cuda_ok(launch_prepare(a, static_cast<cudaStream_t>(stream)), "prepare kernel")) return QG_ERR_CUDA;
    return QG_OK;
}

int qg_dither_floor_pairs(const float *d_x, const float *d_scale, const uint64_t *d_draws, size_t n,
                          int32_t *d_out, uint8_t *d_undecided, void *stream) {
    if (n && (!d_x || !d_scale || !d_draws || !d_out)) return QG_ERR_INVALID;
    if (!cuda_ok(launch_dither_pairs(d_x, d_scale, reinterpret_cast<const unsigned long long *>(d_draws), n,
                                     reinterpret_cast<int *>(d_out), d_undecided,
                                     static_cast<cudaStream_t>(stream)),
                 "dither kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_round_quotient_pairs(const float *d_x, const float *d_s, size_t n, int32_t *d_out, uint8_t *d_undecided,
                            void *stream) {
    if (n && (!d_x || !d_s || !d_out)) return QG_ERR_INVALID;
    if (!cuda_ok(launch_round_quotient_pairs(d_x, d_s, n, reinterpret_cast<int *>(d_out), d_undecided,
                                             static_cast<cudaStream_t>(stream)),
                 "round quotient kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_gate_pairs(const void *space, const int8_t *d_codes, const float *d_scalars,
                  const int64_t *d_code_sum, const uint32_t *d_qidx, const uint32_t *d_ids,
                  size_t count, const uint8_t *d_msb, size_t msb_stride, const void *d_factors,
                  size_t factor_stride, float epsilon0, RabitqPaperEstimate *d_out, void *stream) {
    const Space *s = as_space(space);
    if (!s) return QG_ERR_INVALID;
    if (s->codec != 1 && space_search_mode(s) != 0) {
        set_error("qg_gate_pairs: this codec's gate (the Full gate) reads the rotated residual; use qg_gate_full_pairs");
        return QG_ERR_INVALID;
    }
    if (!cuda_ok(launch_gate_pairs(static_cast<int>(s->code_dim), d_codes,
                                   reinterpret_cast<const float4 *>(d_scalars),
                                   reinterpret_cast<const long long *>(d_code_sum), d_qidx, d_ids, count,
                                   d_msb, msb_stride, static_cast<const uint8_t *>(d_factors),
                                   factor_stride, epsilon0, d_out, static_cast<cudaStream_t>(stream),
                                   s->codec == 1),
                 "gate kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_gate_full_pairs(const void *space, const float *d_rotated, const float *d_scalars, const uint32_t *d_qidx,
                       const uint32_t *d_ids, size_t count, const uint8_t *d_msb, size_t msb_stride,
                       const void *d_factors, size_t factor_stride, float epsilon0, RabitqPaperEstimate *d_out,
                       void *stream) {
    const Space *s = as_space(space);
    if (!s) return QG_ERR_INVALID;
    if (!cuda_ok(launch_gate_full_pairs(static_cast<int>(s->code_dim), d_rotated,
                                        reinterpret_cast<const float4 *>(d_scalars), d_qidx, d_ids, count, d_msb,
                                        msb_stride, static_cast<const uint8_t *>(d_factors), factor_stride, epsilon0,
                                        d_out, static_cast<cudaStream_t>(stream)),
                 "gate kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_distance_pairs(const void *space, const float *d_rotated, const int8_t *d_codes,
                      const float *d_scalars, const int64_t *d_code_sum, const uint32_t *d_qidx,
                      const uint32_t *d_ids, const uint8_t *d_modes, size_t count,
                      const uint8_t *d_records, size_t record_stride, const float *d_short_ips,
                      float *d_out, void *stream) {
    const Space *s = as_space(space);
    if (!s) return QG_ERR_INVALID;
    if (!cuda_ok(launch_distance_pairs(static_cast<int>(s->code_dim), d_rotated, d_codes,
                                       reinterpret_cast<const float4 *>(d_scalars),
                                       reinterpret_cast<const long long *>(d_code_sum), d_qidx, d_ids,
                                       d_modes, count, d_records, record_stride, d_short_ips, d_out,
                                       static_cast<cudaStream_t>(stream)),
                 "distance kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_residual_pairs(const void *space, const float *d_rotated, const float *d_scalars,
                      const uint32_t *d_qidx, const uint32_t *d_ids, size_t count,
                      const uint8_t *d_residual, size_t residual_stride,
                      const float *d_long_distances, RabitqDistanceInterval *d_out,
                      void *stream) {
    const Space *s = as_space(space);
    if (!s) return QG_ERR_INVALID;
    if (!cuda_ok(launch_residual_pairs(static_cast<int>(s->code_dim), d_rotated,
                                       reinterpret_cast<const float4 *>(d_scalars), d_qidx, d_ids, count,
                                       d_residual, residual_stride, d_long_distances, false, d_out,
                                       static_cast<cudaStream_t>(stream)),
                 "residual kernel"))
        return QG_ERR_CUDA;
    return QG_OK;
}

static void index_free_all(qg_index *ix) {
    ix->payload.reset();
    cudaFree(ix->visited);
    cudaFree(ix->counter);
    cudaFree(ix->status);
    cudaFree(ix->q.rr);
    cudaFree(ix->q.codes);
    cudaFree(ix->q.scal);
    cudaFree(ix->q.csum);
}

int qg_index_upload_device(const void *space, const void *d_compact, size_t compact_stride,
                           const void *d_residual, size_t residual_stride, const uint8_t *d_msb,
                           size_t msb_stride, const void *d_factors, size_t factor_stride,
                           const uint32_t *d_degrees, const uint32_t *d_edges,
                           size_t edge_stride, size_t base_points, size_t total_points,
                           void *stream, qg_index **out) {
    const Space *s = as_space(space);
    if (!s || !out || total_points < base_points || total_points >= 0x7FFFFFFFu) return QG_ERR_INVALID;
    if (base_points == 0 && total_points != 0) return QG_ERR_INVALID;
    if (edge_stride == 0 || edge_stride > 64) {
        set_error("edge stride (max degree) must be 1..64");
        return QG_ERR_UNSUPPORTED;
    }
    if (compact_stride < s->compact_bytes || residual_stride < s->residual_bytes || msb_stride < s->msb_bytes ||
        factor_stride < 20) {
        set_error("record stride smaller than the record");
        return QG_ERR_INVALID;
    }
    auto *ix = new (std::nothrow) qg_index();
    if (!ix) return QG_ERR_OOM;
    ix->payload = std::make_shared<DeviceBlocks>();
    ix->space = s;
    cudaGetDevice(&ix->device);
    const size_t D = s->code_dim, nb = base_points, nt = total_points;
    auto own = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        ix->payload->ptrs.push_back(p);
        ix->device_bytes += bytes;
        return p;
    };
    DevIndex &d = ix->ix;
    d.n_total = static_cast<uint32_t>(nt);
    d.n_base = static_cast<uint32_t>(nb);
    d.code_dim = static_cast<uint32_t>(D);
    d.edge_stride = static_cast<uint32_t>(edge_stride);
    d.max_degree = static_cast<uint32_t>(edge_stride);
    // Payload rows exist for every graph node; rows of frozen points (ids >= base_points) stay
    // zero: degenerate long_scale and invalid factors, so the kernels never read past them.
    d.codes = static_cast<uint8_t *>(own(nt * D / 2));
    d.hdr = static_cast<float4 *>(own(nt * 16));
    d.msb = static_cast<uint8_t *>(own(nt * D / 8));
    d.pf = static_cast<float4 *>(own(nt * 16));
    d.res_scales = static_cast<uint16_t *>(own(nt * D / 16 * 2));
    d.res_codes = static_cast<uint8_t *>(own(nt * D / 2));
    (void)nb;
    d.degrees = static_cast<uint32_t *>(own(nt * 4));
    d.edges = static_cast<uint32_t *>(own(nt * edge_stride * 4));
    ix->counter = dev_alloc<unsigned int>(1);
    ix->status = dev_alloc<int>(1);
    if (!d.codes || !d.hdr || !d.msb || !d.pf || !d.res_scales || !d.res_codes || !d.degrees || !d.edges ||
        !ix->counter || !ix->status) {
        set_error("device allocation failed for the index");
        index_free_all(ix);
        delete ix;
        return QG_ERR_OOM;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaMemsetAsync(ix->status, 0, 4, st);
    if (nt > nb) {
        cudaMemsetAsync(d.codes, 0, nt * D / 2, st);
        cudaMemsetAsync(d.hdr, 0, nt * 16, st);
        cudaMemsetAsync(d.msb, 0, nt * D / 8, st);
        cudaMemsetAsync(d.pf, 0, nt * 16, st);
        cudaMemsetAsync(d.res_scales, 0, nt * D / 16 * 2, st);
        cudaMemsetAsync(d.res_codes, 0, nt * D / 2, st);
    }
    if (!cuda_ok(launch_repack(static_cast<const uint8_t *>(d_compact), compact_stride,
                               static_cast<const uint8_t *>(d_residual), residual_stride, d_msb, msb_stride,
                               static_cast<const uint8_t *>(d_factors), factor_stride, d_degrees, d_edges,
                               edge_stride, d, st), "repack kernel") ||
        !cuda_ok(cudaStreamSynchronize(st), "repack sync")) {
        index_free_all(ix);
        delete ix;
        return QG_ERR_CUDA;
    }
    *out = ix;
    return QG_OK;
}

int qg_index_upload_host(const void *space, const void *compact, size_t compact_stride,
                         const void *residual, size_t residual_stride, const uint8_t *msb,
                         size_t msb_stride, const void *factors, size_t factor_stride,
                         const uint32_t *degrees, const uint32_t *edges, size_t edge_stride,
                         size_t base_points, size_t total_points, qg_index **out) {
    const Space *s = as_space(space);
    if (!s || !out || !degrees || !edges || (base_points && (!compact || !residual || !msb || !factors)))
        return QG_ERR_INVALID;
    for (size_t i = 0; i < total_points; ++i)
        if (degrees[i] > edge_stride) {
            set_error("a node degree exceeds the edge stride");
            return QG_ERR_INVALID;
        }
    const size_t nb = base_points, nt = total_points;
    const size_t sizes[6] = {nb * compact_stride, nb * residual_stride, nb * msb_stride, nb * factor_stride,
                             nt * 4, nt * edge_stride * 4};
    const void *srcs[6] = {compact, residual, msb, factors, degrees, edges};
    void *tmp[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int rc = QG_OK;
    for (int i = 0; i < 6 && rc == QG_OK; ++i) {
        if (cudaMalloc(&tmp[i], sizes[i] ? sizes[i] : 16) != cudaSuccess) {
            rc = QG_ERR_OOM;
            set_error("device allocation failed for the upload");
        } else if (sizes[i] && cudaMemcpy(tmp[i], srcs[i], sizes[i], cudaMemcpyHostToDevice) != cudaSuccess) {
            rc = QG_ERR_CUDA;
            set_error("index upload copy failed");
        }
    }
    if (rc == QG_OK)
        rc = qg_index_upload_device(space, tmp[0], compact_stride, tmp[1], residual_stride,
                                    static_cast<const uint8_t *>(tmp[2]), msb_stride, tmp[3], factor_stride,
                                    static_cast<const uint32_t *>(tmp[4]), static_cast<const uint32_t *>(tmp[5]),
                                    edge_stride, base_points, total_points, nullptr, out);
    for (void *p : tmp) cudaFree(p);
    return rc;
}

int qg_index_share(const qg_index *src, qg_index **out) {
    if (!src || !out || !src->payload) {
        set_error("qg_index_share: null argument");
        return QG_ERR_INVALID;
    }
    auto *ix = new (std::nothrow) qg_index();
    if (!ix) return QG_ERR_OOM;
    ix->ix = src->ix;
    ix->space = src->space;
    ix->device = src->device;
    ix->device_bytes = src->device_bytes;
    ix->launch_wpb = src->launch_wpb;
    ix->launch_per_sm = src->launch_per_sm;
    ix->tile = src->tile;
    ix->payload = src->payload;
    ix->counter = dev_alloc<unsigned int>(1);
    ix->status = dev_alloc<int>(1);
    if (!ix->counter || !ix->status || cudaMemset(ix->status, 0, 4) != cudaSuccess) {
        set_error("qg_index_share: device allocation failed");
        index_free_all(ix);
        delete ix;
        return QG_ERR_OOM;
    }
    *out = ix;
    return QG_OK;
}

void qg_index_free(qg_index *index) {
    if (!index) return;
    index_free_all(index);
    delete index;
}

size_t qg_index_device_bytes(const qg_index *index) { return index ? index->device_bytes : 0; }

int qg_search_status(qg_index *index, void *stream) {
    if (!index) return QG_ERR_INVALID;
    int h = 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!cuda_ok(cudaMemcpyAsync(&h, index->status, 4, cudaMemcpyDeviceToHost, st), "status read") ||
        !cuda_ok(cudaStreamSynchronize(st), "status sync"))
        return QG_ERR_CUDA;
    if (h & 1) return QG_ERR_GRAPH;
    if (h & 2) return QG_ERR_TIMEOUT;
    if (h & 4) return QG_ERR_INVALID;
    return QG_OK;
}

int qg_search_batch(qg_index *index, const float *d_queries, size_t nq,
                    const qg_search_params *params, const int *d_k, const int *d_l,
                    size_t k_stride, uint32_t *d_ids, float *d_dists, qg_search_stats *d_stats,
                    void *stream) {
    return qg_search_batch_ex(index, d_queries, nq, params, d_k, d_l, k_stride, d_ids, d_dists, d_stats,
                              nullptr, 0, stream);
}

static int search_impl(qg_index *index, const float *d_queries, size_t nq, const qg_search_params *params,
                       const int *d_k, const int *d_l, size_t k_stride, uint32_t *d_ids, float *d_dists,
                       qg_search_stats *d_stats, uint32_t *d_expanded, size_t expanded_cap,
                       const qg_stop_model *model, const qg_trace_request *trace, void *stream,
                       const int *d_nq = nullptr, bool allow_alloc = true);

int qg_index_set_launch(qg_index *index, int warps_per_block, int blocks_per_sm) {
    if (!index || warps_per_block < 0 || warps_per_block > 8 || blocks_per_sm < 0) return QG_ERR_INVALID;
    index->launch_wpb = warps_per_block;
    index->launch_per_sm = blocks_per_sm;
    return QG_OK;
}

int qg_index_max_block_warps(const qg_index *index) {
    if (!index) return 0;
    return search_max_block_warps(static_cast<int>(index->space->code_dim), search_tile(index));
}

int qg_index_set_tile(qg_index *index, int tile) {
    if (!index || tile < -1 || tile > 4) {
        set_error("tile shape must be -1 (by index size) or 0..4");
        return QG_ERR_INVALID;
    }
    index->tile = tile;
    return QG_OK;
}

int qg_index_reserve(qg_index *index, size_t max_nq, int max_l, int max_k) {
    if (!index || max_l < 1 || max_k < 1) return QG_ERR_INVALID;
    // an ordinary search of an empty batch sizes the workspace and the visited rows
    qg_search_params p{max_k, max_l, 1, 1.9f, 100, 0, 0};
    const int rc = search_impl(index, nullptr, 0, &p, nullptr, nullptr, static_cast<size_t>(max_k), nullptr,
                               nullptr, nullptr, nullptr, 0, nullptr, nullptr, nullptr);
    if (rc != QG_OK) return rc;
    if (index->q_capacity < max_nq) {
        cudaFree(index->q.rr);
        cudaFree(index->q.codes);
        cudaFree(index->q.scal);
        cudaFree(index->q.csum);
        const Space *s = index->space;
        index->q.rr = dev_alloc<float>(max_nq * s->code_dim);
        index->q.codes = dev_alloc<int8_t>(max_nq * s->code_dim);
        index->q.scal = dev_alloc<float4>(max_nq);
        index->q.csum = dev_alloc<long long>(max_nq);
        if (!index->q.rr || !index->q.codes || !index->q.scal || !index->q.csum) {
            index->q_capacity = 0;
            set_error("device allocation failed for prepared queries");
            return QG_ERR_OOM;
        }
        index->q_capacity = max_nq;
    }
    return QG_OK;
}

// A stop model needs weights, the normalisation block and every >= 1; a classifier (kind 0) a
// threshold in (0, 1), a hop budget (kind 1) a positive finite scale.
static bool stop_model_ok(const qg_stop_model *m) {
    if (!m->d_weights || !m->d_norm || m->every < 1 || m->min_hops < 0) {
        set_error("stop model needs weights, normalisation, every >= 1 and min_hops >= 0");
        return false;
    }
    if (m->kind == 0 && (m->threshold > 0.0f && m->threshold < 1.0f)) return true;
    if (m->kind == 1 && m->budget_scale > 0.0f && std::isfinite(m->budget_scale)) return true;
    set_error("stop model: kind 0 needs 0 < threshold < 1, kind 1 a positive finite budget scale");
    return false;
}

int qg_search_batch_graph(qg_index *index, const float *d_queries, size_t max_nq, const int *d_nq,
                          const qg_search_params *params, const int *d_k, const int *d_l, size_t k_stride,
                          uint32_t *d_ids, float *d_dists, qg_search_stats *d_stats,
                          const qg_stop_model *model, void *stream) {
    if (!d_nq) return QG_ERR_INVALID;
    if (model && !stop_model_ok(model)) return QG_ERR_INVALID;
    return search_impl(index, d_queries, max_nq, params, d_k, d_l, k_stride, d_ids, d_dists, d_stats, nullptr, 0,
                       model, nullptr, stream, d_nq, false);
}

int qg_search_batch_ex(qg_index *index, const float *d_queries, size_t nq,
                       const qg_search_params *params, const int *d_k, const int *d_l,
                       size_t k_stride, uint32_t *d_ids, float *d_dists, qg_search_stats *d_stats,
                       uint32_t *d_expanded, size_t expanded_cap, void *stream) {
    return search_impl(index, d_queries, nq, params, d_k, d_l, k_stride, d_ids, d_dists, d_stats, d_expanded,
                       expanded_cap, nullptr, nullptr, stream);
}

int qg_search_batch_learned(qg_index *index, const float *d_queries, size_t nq,
                            const qg_search_params *params, const int *d_k, const int *d_l,
                            size_t k_stride, uint32_t *d_ids, float *d_dists, qg_search_stats *d_stats,
                            const qg_stop_model *model, const qg_trace_request *trace, void *stream) {
    if (model && !stop_model_ok(model)) return QG_ERR_INVALID;
    if (trace && (!trace->d_truth || trace->truth_k < 1 || trace->every < 1 || trace->cap < 1 ||
                  !trace->d_features || !trace->d_labels || !trace->d_counts)) {
        set_error("trace request needs truth ids, every >= 1, cap >= 1 and output buffers");
        return QG_ERR_INVALID;
    }
    if (model && trace && model->every != trace->every) {
        set_error("stop model and trace must use the same checkpoint interval");
        return QG_ERR_INVALID;
    }
    return search_impl(index, d_queries, nq, params, d_k, d_l, k_stride, d_ids, d_dists, d_stats, nullptr, 0,
                       model, trace, stream);
}

int qg_mlp_forward(const float *d_x, size_t n, const float *d_norm, const uint16_t *d_weights, float *d_logits,
                   void *stream) {
    if (n && (!d_x || !d_norm || !d_weights || !d_logits)) return QG_ERR_INVALID;
    if (!cuda_ok(launch_mlp_forward(d_x, n, d_norm, d_weights, d_logits, static_cast<cudaStream_t>(stream)),
                 "mlp forward"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_mlp_backward(const float *d_x, const float *d_y, size_t n, const float *d_norm, const uint16_t *d_weights,
                    float *d_grad, float *d_loss, void *stream) {
    if (!d_grad || !d_loss || (n && (!d_x || !d_y || !d_norm || !d_weights))) return QG_ERR_INVALID;
    if (!cuda_ok(launch_mlp_backward(d_x, d_y, n, d_norm, d_weights, d_grad, d_loss,
                                     static_cast<cudaStream_t>(stream)),
                 "mlp backward"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_mlp_backward_mse(const float *d_x, const float *d_y, size_t n, const float *d_norm, const uint16_t *d_weights,
                        float *d_grad, float *d_loss, void *stream) {
    if (!d_grad || !d_loss || (n && (!d_x || !d_y || !d_norm || !d_weights))) return QG_ERR_INVALID;
    if (!cuda_ok(launch_mlp_backward(d_x, d_y, n, d_norm, d_weights, d_grad, d_loss,
                                     static_cast<cudaStream_t>(stream), true),
                 "mlp backward (squared error)"))
        return QG_ERR_CUDA;
    return QG_OK;
}

int qg_mlp_adam(float *d_master, uint16_t *d_weights, const float *d_grad, float *d_m, float *d_v, float lr,
                float beta1, float beta2, float eps, int step, void *stream) {
    if (!d_master || !d_weights || !d_grad || !d_m || !d_v || step < 1) return QG_ERR_INVALID;
    if (!cuda_ok(launch_mlp_adam(d_master, d_weights, d_grad, d_m, d_v, lr, beta1, beta2, eps, step,
                                 static_cast<cudaStream_t>(stream)),
                 "mlp adam"))
        return QG_ERR_CUDA;
    return QG_OK;
}

static int search_impl(qg_index *index, const float *d_queries, size_t nq, const qg_search_params *params,
                       const int *d_k, const int *d_l, size_t k_stride, uint32_t *d_ids, float *d_dists,
                       qg_search_stats *d_stats, uint32_t *d_expanded, size_t expanded_cap,
                       const qg_stop_model *model, const qg_trace_request *trace, void *stream,
                       const int *d_nq, bool allow_alloc) {
    SearchArgs a{};
    const int rc = search_args_fill(index, nq, params, d_queries, d_k, d_l, k_stride, d_ids, d_dists, d_stats, &a);
    if (rc != QG_OK) return rc;
    if (d_expanded && (expanded_cap == 0 || expanded_cap > 0x7FFFFFFF)) return QG_ERR_INVALID;
    const Space *s = index->space;
    const int l_cap = a.l_cap;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // prepared-query workspace
    if (index->q_capacity < nq && !allow_alloc) {
        set_error("batch exceeds the reserved query capacity (qg_index_reserve)");
        return QG_ERR_INVALID;
    }
    if (index->q_capacity < nq) {
        cudaFree(index->q.rr);
        cudaFree(index->q.codes);
        cudaFree(index->q.scal);
        cudaFree(index->q.csum);
        const size_t cap = std::max<size_t>(nq, 1024);
        index->q.rr = dev_alloc<float>(cap * s->code_dim);
        index->q.codes = dev_alloc<int8_t>(cap * s->code_dim);
        index->q.scal = dev_alloc<float4>(cap);
        index->q.csum = dev_alloc<long long>(cap);
        if (!index->q.rr || !index->q.codes || !index->q.scal || !index->q.csum) {
            index->q_capacity = 0;
            set_error("device allocation failed for prepared queries");
            return QG_ERR_OOM;
        }
        index->q_capacity = cap;
    }
    // persistent grid: warps per block and resident blocks per SM from the occupancy of
    // this pool size; one visited row per warp slot
    int wpb = 0, per_sm = 0;
    if (!search_launch_geometry(index, l_cap, model != nullptr, &wpb, &per_sm)) return QG_ERR_UNSUPPORTED;
    int sms = qg_device_sm_count();
    if (sms <= 0) sms = 1;
    const int grid = sms * per_sm;
    const int slots = grid * wpb;
    if (index->slots < slots && !allow_alloc) {
        set_error("launch needs more warp slots than reserved (qg_index_reserve)");
        return QG_ERR_INVALID;
    }
    if (index->slots < slots) {
        cudaFree(index->visited);
        index->visited = nullptr;
        const size_t bytes = static_cast<size_t>(slots) * visited_row_words(index->ix.n_total) * 4;
        if (cudaMalloc(&index->visited, bytes) != cudaSuccess) {
            index->slots = 0;
            set_error("device allocation failed for the visited rows");
            return QG_ERR_OOM;
        }
        index->slots = slots;
    }
    if (nq == 0) return QG_OK;
    {
        PrepArgs pa{d_queries, s->dim, static_cast<int>(nq), static_cast<int>(s->dim),
                    static_cast<int>(s->code_dim), s->d_signs, s->d_center, s->d_rotated_center,
                    s->d_center_norm, index->q.rr, index->q.codes, index->q.scal, index->q.csum, d_nq};
        pa.qbits = space_query_bits(s);
        if (!cuda_ok(launch_prepare(pa, st), "prepare kernel")) return QG_ERR_CUDA;
    }
    if (!cuda_ok(cudaMemsetAsync(index->counter, 0, 4, st), "counter reset") ||
        !cuda_ok(cudaMemsetAsync(index->status, 0, 4, st), "status reset"))
        return QG_ERR_CUDA;
    a.rr = index->q.rr;
    a.codes = index->q.codes;
    a.scal = index->q.scal;
    a.csum = index->q.csum;
    a.visited = index->visited;
    a.counter = index->counter;
    a.status = index->status;
    a.nq_dev = d_nq;
    a.expanded_out = d_expanded;
    a.expanded_cap = static_cast<int>(expanded_cap);
    if (model) {
        a.stop_w = model->d_weights;
        a.stop_norm = model->d_norm;
        a.stop_kind = model->kind;
        if (model->kind == 0) a.stop_logit = std::log(model->threshold / (1.0f - model->threshold));
        a.stop_scale = model->budget_scale;
        a.stop_once = model->predict_once;
        a.stop_every = model->every;
        a.stop_min_hops = model->min_hops;
    }
    if (trace) {
        a.trace_truth = trace->d_truth;
        a.trace_truth_k = trace->truth_k;
        a.trace_cap = trace->cap;
        a.trace_feat = trace->d_features;
        a.trace_label = trace->d_labels;
        a.trace_count = trace->d_counts;
        a.stop_every = trace->every;
        if (!cuda_ok(cudaMemsetAsync(trace->d_counts, 0, nq * sizeof(int), st), "trace counts")) return QG_ERR_CUDA;
    }
    index->grid = grid;
    index->warps_per_block = wpb;
    if (!cuda_ok(launch_search(a, grid, wpb, st), "search kernel")) return QG_ERR_CUDA;
    return QG_OK;
}

}  // extern "C"
