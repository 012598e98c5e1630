// search_noalloc.cu -- qg_search_batch_noalloc: the batched search for callers that cannot
// allocate device memory (for example code that runs while a CUDA graph is being captured,
// or a serving process whose memory is fixed up front and must not call cudaMalloc on the
// request path).
//
// It runs the same two kernels as qg_search_batch (query preparation and the persistent
// search), but every piece of scratch they need -- prepared queries, the visited rows of the
// warp slots, the work counter and the status word -- lives in one
// file-scope device array of QG_NOALLOC_SCRATCH_BYTES (64 MiB). Every GPU that loads this
// library holds that array until the process exits. The caller passes the index (built
// earlier), the queries and the outputs; nothing here calls cudaMalloc, cudaFree or any
// allocating routine.
//
// The array is shared by all calls and keeps the last call's contents: each call clears the
// parts that must start at zero (counter, status) on its stream before launching; the search
// kernel clears a visited row itself at the start of every query. Two calls whose GPU work overlaps (different streams, or different host
// threads on one device) race on the array and give wrong results; serialise them.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress (host code cannot use the symbol itself: on the host it names a
// stand-in, not device memory). Make that first call before any stream capture.
//
// Failures inside the kernels (a neighbour id outside the graph, the hop cap, a per-query L
// above the pool capacity) are recorded in a status word in the same array;
// qg_search_noalloc_status reads it back after the call, as qg_search_status does for
// qg_search_batch. It is the status of the last call on the device.
//
// The visited set takes one row of n_total / 8 bytes (a bit per node) per resident warp, so the
// number of warps that search at once is about (64 MiB - prepared queries) / (n_total / 8):
// ~530 at 1M nodes, every resident warp (up to 152 SMs x 16) below ~220k nodes.
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
constexpr size_t kCounterOffset = 0;   // the search's work counter
constexpr size_t kStatusOffset = 256;  // the search's status word (qg_search_noalloc_status)

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
    SearchArgs a{};
    const int rc = search_args_fill(index, nq, params, d_queries, d_k, d_l, k_stride, d_ids, d_dists, d_stats, &a);
    if (rc != QG_OK) return rc;
    void *base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_batch_noalloc: scratch set-up: ") + cudaGetErrorString(e));
    if (nq == 0) return QG_OK;

    const Space *s = index->space;
    const size_t D = s->code_dim;
    const size_t n_total = index->ix.n_total;
    // scratch layout: counter | status | prepared queries (rotated, codes, scalars, sums) | visited rows
    size_t off = kStatusOffset + 256;
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
    // the launch shape qg_search_batch would take (with any qg_index_set_launch override) ...
    int wpb = 0, per_sm = 0;
    if (!search_launch_geometry(index, a.l_cap, false, &wpb, &per_sm)) return QG_ERR_UNSUPPORTED;
    int sms = qg_device_sm_count();
    if (sms <= 0) return fail(QG_ERR_CUDA, "qg_search_batch_noalloc: no device");
    size_t max_slots = static_cast<size_t>(sms) * per_sm * wpb;
    // ... cut to the visited rows that fit (one per warp slot); a block narrower than wpb is
    // taken when fewer than wpb rows fit
    const size_t row_bytes = visited_row_words(n_total) * 4;
    const size_t room = kScratchBytes - off;
    size_t fit = room / row_bytes;
    if (fit < static_cast<size_t>(wpb)) {
        int narrow = 0;
        for (int cand : {4, 2, 1})
            if (cand < wpb && static_cast<size_t>(cand) <= fit) {
                narrow = cand;
                break;
            }
        if (narrow == 0)
            return fail(QG_ERR_INVALID, "qg_search_batch_noalloc: index of " + std::to_string(n_total) +
                                            " nodes is too large for the 64 MiB no-alloc scratch");
        wpb = narrow;
        per_sm = search_blocks_per_sm(static_cast<int>(D), a.l_cap, wpb, false, a.tile);
        if (per_sm <= 0) return fail(QG_ERR_UNSUPPORTED, "qg_search_batch_noalloc: search kernel cannot be resident");
        max_slots = static_cast<size_t>(sms) * per_sm * wpb;
    }
    size_t slots = fit < max_slots ? fit : max_slots;
    slots -= slots % static_cast<size_t>(wpb);
    const size_t o_visited = off;

    unsigned char *sb = static_cast<unsigned char *>(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((e = cudaMemsetAsync(sb + kCounterOffset, 0, kStatusOffset + 256, st)) != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_batch_noalloc: clear: ") + cudaGetErrorString(e));

    PrepArgs pa{d_queries, s->dim, static_cast<int>(nq), static_cast<int>(s->dim), static_cast<int>(D),
                s->d_signs, s->d_center, s->d_rotated_center, s->d_center_norm,
                reinterpret_cast<float *>(sb + o_rr), reinterpret_cast<int8_t *>(sb + o_codes),
                reinterpret_cast<float4 *>(sb + o_scal), reinterpret_cast<long long *>(sb + o_csum)};
    pa.qbits = space_query_bits(s);
    if ((e = launch_prepare(pa, st)) != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_batch_noalloc: prepare: ") + cudaGetErrorString(e));

    a.rr = pa.rr;
    a.codes = pa.codes;
    a.scal = pa.scal;
    a.csum = pa.csum;
    a.visited = reinterpret_cast<uint32_t *>(sb + o_visited);
    a.counter = reinterpret_cast<unsigned int *>(sb + kCounterOffset);
    a.status = reinterpret_cast<int *>(sb + kStatusOffset);
    if ((e = launch_search(a, static_cast<int>(slots / static_cast<size_t>(wpb)), wpb, st)) != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_batch_noalloc: search: ") + cudaGetErrorString(e));
    return QG_OK;
}

extern "C" int qg_search_noalloc_status(void *stream) {
    void *base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_noalloc_status: scratch set-up: ") + cudaGetErrorString(e));
    // the status word sits at a fixed offset of the array; the 4-byte copy lands in host stack memory
    int h = 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((e = cudaMemcpyAsync(&h, static_cast<unsigned char *>(base) + kStatusOffset, sizeof(int),
                             cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(QG_ERR_CUDA, std::string("qg_search_noalloc_status: ") + cudaGetErrorString(e));
    if (h & 1) return fail(QG_ERR_GRAPH, "a neighbour id outside the graph: the query returned no results");
    if (h & 2) return fail(QG_ERR_TIMEOUT, "the hop cap ended a search");
    if (h & 4) return fail(QG_ERR_INVALID, "a per-query L above the call's pool capacity was clamped");
    return QG_OK;
}
