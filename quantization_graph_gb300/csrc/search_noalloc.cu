// search_noalloc.cu -- qg_search_batch_noalloc: the batched search for callers that cannot
// allocate device memory (for example code that runs while a CUDA graph is being captured,
// or a serving process whose memory is fixed up front and must not call cudaMalloc on the
// request path).
//
// It runs the same two kernels as qg_search_batch (query preparation and the persistent
// search), but every piece of scratch they need -- prepared queries, the visited-tag rows of
// each warp slot, the per-slot epochs, the work counter and the status word -- lives in one
// file-scope device array of QG_NOALLOC_SCRATCH_BYTES (64 MiB). Every GPU that loads this
// library holds that array until the process exits. The caller passes the index (built
// earlier), the queries and the outputs; nothing here calls cudaMalloc, cudaFree or any
// allocating routine.
//
// The array is shared by all calls and keeps the last call's contents: each call clears the
// parts that must start at zero (counter, status, epochs, the tag rows it uses) on its stream
// before launching. Two calls whose GPU work overlaps (different streams, or different host
// threads on one device) race on the array and give wrong results; serialise them.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress (host code cannot use the symbol itself: on the host it names a
// stand-in, not device memory). Make that first call before any stream capture.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "qg_kernels.h"
#include "qg_types.h"

namespace {

constexpr size_t kScratchBytes = QG_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_scratch_mutex;
void *g_scratch_address[kMaxDevices] = {};

size_t round256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// Device address of the scratch array on the current device (looked up once per device).
cudaError_t scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_address[dev] == nullptr) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_address[dev] = p;
    }
    *out = g_scratch_address[dev];
    return cudaSuccess;
}

int fail(int status, const std::string &msg) {
    qg::record_error(msg);
    return status;
}

}  // namespace

extern "C" int qg_search_batch_noalloc(qg_index *index, const float *d_queries, size_t nq,
                                       const qg_search_params *params, const int *d_k, const int *d_l,
                                       size_t k_stride, uint32_t *d_ids, float *d_dists,
                                       qg_search_stats *d_stats, void *stream) {
    using namespace qg;
    if (!index || !params || (nq && (!d_queries || !d_ids || !d_dists)))
        return fail(QG_ERR_INVALID, "qg_search_batch_noalloc: null argument");
    const Space *s = index->space;
    const int k_max = d_k ? static_cast<int>(k_stride) : params->k;
    if (k_max <= 0 || nq > 0x7FFFFFFF)
        return fail(QG_ERR_INVALID, "qg_search_batch_noalloc: k must be positive");
    const int l_cap = params->l_value > k_max ? params->l_value : k_max;
    if (l_cap > 4096 || params->beam_width < 1 || params->beam_width > 8 || params->rerank_candidates < 0)
        return fail(QG_ERR_INVALID, "qg_search_batch_noalloc: L must be <= 4096 and beam width 1..8");
    void *base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_batch_noalloc: scratch set-up: ") + cudaGetErrorString(e));
    if (nq == 0) return QG_OK;

    const size_t D = s->code_dim;
    const size_t n_total = index->ix.n_total;
    // scratch layout: counter | status | prepared queries (rotated, codes, scalars, sums) | epochs | tags
    size_t off = 0;
    const size_t o_counter = off;
    off += 256;
    const size_t o_status = off;
    off += 256;
    const size_t o_rr = off;
    off += round256(nq * D * sizeof(float));
    const size_t o_codes = off;
    off += round256(nq * D);
    const size_t o_scal = off;
    off += round256(nq * sizeof(float4));
    const size_t o_csum = off;
    off += round256(nq * sizeof(long long));
    if (off > kScratchBytes)
        return fail(QG_ERR_INVALID, "qg_search_batch_noalloc: " + std::to_string(nq) +
                                        " queries do not fit the 64 MiB no-alloc scratch");
    // warp slots: as many resident warps as the tag rows that still fit
    int wpb = 8, per_sm = 0;
    for (int cand : {8, 4, 2}) {
        const int b = search_blocks_per_sm(static_cast<int>(D), l_cap, cand);
        if (b * cand > per_sm * wpb) {
            wpb = cand;
            per_sm = b;
        }
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (per_sm <= 0 || sms <= 0)
        return fail(QG_ERR_UNSUPPORTED, "qg_search_batch_noalloc: search kernel cannot be resident");
    const size_t row_bytes = n_total * sizeof(uint16_t);  // the kernel's tag rows are packed
    const size_t epoch_bytes = round256(static_cast<size_t>(sms) * per_sm * wpb * sizeof(uint32_t));
    if (off + epoch_bytes > kScratchBytes)
        return fail(QG_ERR_INVALID, "qg_search_batch_noalloc: queries leave no room for visited tags");
    const size_t room = kScratchBytes - off - epoch_bytes;
    size_t slots = row_bytes ? room / row_bytes : 0;
    const size_t max_slots = static_cast<size_t>(sms) * per_sm * wpb;
    if (slots > max_slots) slots = max_slots;
    slots -= slots % static_cast<size_t>(wpb);
    if (slots == 0)
        return fail(QG_ERR_INVALID, "qg_search_batch_noalloc: index of " + std::to_string(n_total) +
                                        " nodes is too large for the 64 MiB no-alloc scratch");
    const size_t o_epochs = off;
    off += epoch_bytes;
    const size_t o_tags = off;

    unsigned char *sb = static_cast<unsigned char *>(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // clear what must start at zero; tag rows are laid out for this call's node count
    if ((e = cudaMemsetAsync(sb + o_counter, 0, 512, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(sb + o_epochs, 0, epoch_bytes, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(sb + o_tags, 0, slots * row_bytes, st)) != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_batch_noalloc: clear: ") + cudaGetErrorString(e));

    if (!space_query_bits(s))
        return fail(QG_ERR_INVALID, "qg_search_batch_noalloc: the Full (0), B1 (1), Int4 (2), Int8 (3) and B1Main (4) query codecs only");
    PrepArgs pa{d_queries, s->dim, static_cast<int>(nq), static_cast<int>(s->dim), static_cast<int>(D),
                s->d_signs, s->d_center, s->d_rotated_center, s->d_center_norm,
                reinterpret_cast<float *>(sb + o_rr), reinterpret_cast<int8_t *>(sb + o_codes),
                reinterpret_cast<float4 *>(sb + o_scal), reinterpret_cast<long long *>(sb + o_csum)};
    pa.qbits = space_query_bits(s);
    if ((e = launch_prepare(pa, st)) != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_batch_noalloc: prepare: ") + cudaGetErrorString(e));

    SearchArgs a{};
    a.ix = index->ix;
    a.rr = pa.rr;
    a.codes = pa.codes;
    a.scal = pa.scal;
    a.csum = pa.csum;
    a.nq = static_cast<int>(nq);
    a.k_default = params->k;
    a.l_default = params->l_value;
    a.k_per_q = d_k;
    a.l_per_q = d_l;
    a.k_stride = k_max;
    a.l_cap = l_cap;
    a.beam_width = params->beam_width;
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
    a.tags = reinterpret_cast<uint16_t *>(sb + o_tags);
    a.epochs = reinterpret_cast<uint32_t *>(sb + o_epochs);
    a.counter = reinterpret_cast<unsigned int *>(sb + o_counter);
    a.status = reinterpret_cast<int *>(sb + o_status);
    a.hop_cap = static_cast<int>(n_total + 1 < 0x7FFFFFFF ? n_total + 1 : 0x7FFFFFFF);
    a.expanded_out = nullptr;
    a.expanded_cap = 0;
    if ((e = launch_search(a, static_cast<int>(slots / static_cast<size_t>(wpb)), wpb, st)) != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_batch_noalloc: search: ") + cudaGetErrorString(e));
    return QG_OK;
}
