// vamana_build.cu -- the reference's Vamana graph build on the GPU, graph for graph.
//
// Follows rabitq_build_vamana_graph (experiments/02_diskann_fair/native/rabitq_bridge.cpp:224-303):
//   bulk insertion in batches from node 0   VamanaIndex::buildGraphFromLoadedPayloads (vamana_index.h:452-528)
//   refinement passes                       refineGraphSymmetric (vamana_index.h:328-422)
//   grouped back-edges                      addBackedgesGroupedAndPrune / addBackedgeGroupAndPrune
//                                           (vamana_index.h:995-1117)
//   build search                            search_vamana (vamana_search.h:98-198)
//   prune                                   robust_prune_4bit (vamana_prune.h:42-156), capBuildPrunePool
//                                           (vamana_index.h:201-211)
//   distance                                symmetricBuildDistanceFromPrepared (space_rabitq.h:2706-2747)
//
// The reference build is deterministic for any thread count (searches of a batch read the graph
// frozen at the start of the batch; back-edge groups write disjoint sources), so a parallel build
// that makes the same decisions yields the same graph. Where the GPU formulation differs:
//   * search: one warp per inserted node. The pool after a hop equals the L smallest (distance,
//     id) of the old pool and every fresh neighbour of the hop, whatever the insertion order, so
//     the fresh neighbours of a hop are scored together, sorted and merged in one step.
//   * prune: the reference checks candidate i against the selected neighbours in order and stops
//     at the first occluder (alpha * d <= dist_i). "Some selected neighbour occludes i" is the
//     same as "alpha * min_k d(i, s_k) <= dist_i" (rounding of alpha * x is monotone in x), so
//     each selection updates a running minimum of every live candidate in parallel instead, and
//     a candidate occluded at every alpha of the ramp is dropped for good. Decisions, and thus
//     the neighbour lists, are the reference's; the number of distances evaluated is not.
//   * back-edges: pairs are bucketed by source with a count / scan / scatter instead of a sort;
//     each group sorts its (distinct) targets itself.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "qg_kernels.h"
#include "sym_ff.cuh"

namespace qg {
namespace {

constexpr uint32_t kNoNode = 0xFFFFFFFFu;
constexpr unsigned long long kKeyMax = ~0ull;
constexpr int kWarpsPerBlock = 4;

// Per-record factors of the symmetric estimator (sym_ff.cuh): norm, ip_norm, their float
// pairs, norm_sqr, code sum, validity.
using VbAux = SymFactors;

// (distance, id) as one ordered 64-bit key: the float mapped to an unsigned order, -0 folded
// onto +0 (candidate_less compares floats, so the two are equal there and the id decides),
// then id << 1; bit 0 is the search pool's "expanded" flag. Keys of different ids never tie,
// so the flag never changes an order.
__device__ __forceinline__ uint32_t ord_bits(float d) {
    const uint32_t u = __float_as_uint(d == 0.0f ? 0.0f : d);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long make_key(float d, uint32_t id) {
    return (static_cast<unsigned long long>(ord_bits(d)) << 32) | (static_cast<unsigned long long>(id) << 1);
}
__device__ __forceinline__ float key_dist(unsigned long long k) {
    uint32_t u = static_cast<uint32_t>(k >> 32);
    u = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    return __uint_as_float(u);
}
__device__ __forceinline__ uint32_t key_id(unsigned long long k) {
    return static_cast<uint32_t>(k >> 1) & 0x7FFFFFFFu;
}

__device__ __forceinline__ uint32_t nib_dot4(uint4 a, uint4 b, uint32_t acc) {
    acc = __dp4a(a.x & 0x0F0F0F0Fu, b.x & 0x0F0F0F0Fu, acc);
    acc = __dp4a((a.x >> 4) & 0x0F0F0F0Fu, (b.x >> 4) & 0x0F0F0F0Fu, acc);
    acc = __dp4a(a.y & 0x0F0F0F0Fu, b.y & 0x0F0F0F0Fu, acc);
    acc = __dp4a((a.y >> 4) & 0x0F0F0F0Fu, (b.y >> 4) & 0x0F0F0F0Fu, acc);
    acc = __dp4a(a.z & 0x0F0F0F0Fu, b.z & 0x0F0F0F0Fu, acc);
    acc = __dp4a((a.z >> 4) & 0x0F0F0F0Fu, (b.z >> 4) & 0x0F0F0F0Fu, acc);
    acc = __dp4a(a.w & 0x0F0F0F0Fu, b.w & 0x0F0F0F0Fu, acc);
    acc = __dp4a((a.w >> 4) & 0x0F0F0F0Fu, (b.w >> 4) & 0x0F0F0F0Fu, acc);
    return acc;
}

// symmetricBuildDistanceFromPrepared with lhs the prepared side: the centred code product
// sum (2a-15)(2b-15) = 4 ab - 30 a - 30 b + 225 from the plain nibble product ab, then the
// estimator; float-float with a proven margin, double precision near rounding boundaries.
template <int D>
__device__ __forceinline__ float sym_distance(const VbAux &l, const VbAux &r, uint32_t ab) {
    const int s = 4 * static_cast<int>(ab) - 30 * (l.nsum + r.nsum) + 225 * D;
    return sym_distance_exact(l, r, s);
}

// Lanes split into groups of G; a group scores one candidate, each lane a fixed set of 16-byte
// chunks (g, g + G, ...), so one side's code can stay in registers.
template <int D>
struct Geo {
    static constexpr int kChunks = D / 32;  // 16-byte chunks of a code (32 dims each)
    static constexpr int kG = kChunks < 8 ? kChunks : 8;
    static constexpr int kPer = kChunks / kG;
    static constexpr int kCands = 32 / kG;  // candidates per warp pass
};

template <int D>
__device__ __forceinline__ void load_code(const uint4 *codes, uint32_t id, int g, uint4 (&c)[Geo<D>::kPer]) {
    const uint4 *row = codes + static_cast<size_t>(id) * Geo<D>::kChunks;
#pragma unroll
    for (int k = 0; k < Geo<D>::kPer; ++k) c[k] = __ldg(row + g + k * Geo<D>::kG);
}

// Scores candidates ids[0..n) against the register-held code `reg` (record `reg_aux`);
// reg_is_lhs selects which side is the prepared one. The group leader gets the distance and
// calls sink(index, distance).
template <int D, typename Sink>
__device__ __forceinline__ void score_batch(const uint4 (&reg)[Geo<D>::kPer], const VbAux &reg_aux, bool reg_is_lhs,
                                            const uint4 *codes, const VbAux *aux, const uint32_t *ids, int n,
                                            Sink sink) {
    const int lane = threadIdx.x & 31, grp = lane / Geo<D>::kG, g = lane % Geo<D>::kG;
    for (int base = 0; base < n; base += Geo<D>::kCands) {
        const int c = base + grp;
        uint32_t acc = 0;
        uint32_t id = 0;
        if (c < n) {
            id = ids[c];
            uint4 x[Geo<D>::kPer];
            load_code<D>(codes, id, g, x);
#pragma unroll
            for (int k = 0; k < Geo<D>::kPer; ++k) acc = nib_dot4(reg[k], x[k], acc);
        }
#pragma unroll
        for (int o = Geo<D>::kG / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (c < n && g == 0) {
            const VbAux a = aux[id];
            sink(c, reg_is_lhs ? sym_distance<D>(reg_aux, a, acc) : sym_distance<D>(a, reg_aux, acc));
        }
    }
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp bitonic sort of keys[0..p2) (p2 a power of two), ascending.
__device__ void warp_bitonic(unsigned long long *keys, int p2) {
    const int lane = threadIdx.x & 31;
    for (int k = 2; k <= p2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < p2; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = keys[i], b = keys[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// ----------------------------------------------------------------------------------------------
// per-record preparation: codes re-laid out 16-byte aligned, factors of the estimator
// ----------------------------------------------------------------------------------------------
__global__ void vb_prepare_kernel(const uint8_t *compact, size_t n, size_t stride, int D, uint8_t *codes,
                                  VbAux *aux) {
    const size_t row = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const uint8_t *rec = compact + row * stride;
    const int bytes = D / 2;
    uint32_t sum = 0;
    for (int b = lane; b < bytes; b += 32) {
        const uint8_t v = rec[16 + b];
        codes[row * bytes + b] = v;
        sum += (v & 15u) + (v >> 4);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) {
        float n2, ls;
        memcpy(&n2, rec, 4);
        memcpy(&ls, rec + 4, 4);
        aux[row] = sym_factors(n2, ls, static_cast<int32_t>(sum));
    }
}

// ----------------------------------------------------------------------------------------------
// build search (search_vamana): one warp per inserted node, persistent, work by atomic counter
// ----------------------------------------------------------------------------------------------
struct VbSearchArgs {
    const uint4 *codes;
    const VbAux *aux;
    const uint32_t *adj;
    const uint32_t *deg;
    uint32_t r;
    uint32_t node_count;
    uint32_t first, count;
    uint32_t l, beam, stop;
    uint32_t fresh_cap;  // power of two >= beam * r
    uint16_t *tags;      // one row of n_total tags per warp slot
    uint16_t *epochs;    // per warp slot
    size_t n_total;
    unsigned long long *pools;  // count x l sorted keys
    uint32_t *pool_n;
    unsigned int *work;
    unsigned long long *evals;
    int *error;
};

// Shared memory of one warp: pool and merge buffer (l keys each), fresh keys, distances and
// ids (fresh_cap each), frontier ids (beam).
__host__ __device__ inline size_t vb_search_words(uint32_t l, uint32_t fresh_cap, uint32_t beam) {
    return 2 * static_cast<size_t>(l) + 2 * static_cast<size_t>(fresh_cap) + (beam + 1) / 2;
}

template <int D>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) vb_search_kernel(VbSearchArgs a) {
    extern __shared__ unsigned long long vb_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long *const base_a = vb_smem + warp * vb_search_words(a.l, a.fresh_cap, a.beam);
    unsigned long long *const base_b = base_a + a.l;
    unsigned long long *const fk = base_b + a.l;
    float *const fd = reinterpret_cast<float *>(fk + a.fresh_cap);
    uint32_t *const fid = reinterpret_cast<uint32_t *>(fd + a.fresh_cap);
    uint32_t *const front = fid + a.fresh_cap;
    const size_t slot = static_cast<size_t>(blockIdx.x) * kWarpsPerBlock + warp;
    uint16_t *const tag = a.tags + slot * a.n_total;
    const int g = lane % Geo<D>::kG;
    unsigned long long my_evals = 0;

    for (;;) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(a.work, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= a.count) break;
        const uint32_t q = a.first + item;
        unsigned long long *pa = base_a, *pb = base_b;

        // epoch of this slot's visited row; a wrap clears the row
        uint16_t e = static_cast<uint16_t>(a.epochs[slot] + 1);
        if (e == 0) {
            for (size_t i = lane; i < a.n_total; i += 32) tag[i] = 0;
            e = 1;
        }
        __syncwarp();
        if (lane == 0) a.epochs[slot] = e;

        uint4 qc[Geo<D>::kPer];
        load_code<D>(a.codes, q, g, qc);
        const VbAux qa = a.aux[q];

        // start node 0
        if (lane == 0) fid[0] = 0;
        __syncwarp();
        score_batch<D>(qc, qa, true, a.codes, a.aux, fid, 1, [&](int, float d) { pa[0] = make_key(d, 0); });
        if (lane == 0) tag[0] = e;
        my_evals += 1;
        __syncwarp();
        uint32_t n = 1, fu = 0, stall = 0;
        bool failed = false;
        for (;;) {
            const float back_before = key_dist(pa[n - 1]);
            // frontier: the first `beam` unexpanded entries, marked expanded
            uint32_t nf = 0, last = 0;
            for (uint32_t base = fu; base < n && nf < a.beam; base += 32) {
                const uint32_t idx = base + lane;
                unsigned m = __ballot_sync(0xffffffffu, idx < n && !(pa[idx] & 1ull));
                while (m && nf < a.beam) {
                    const int b = __ffs(m) - 1;
                    m &= m - 1;
                    if (lane == 0) {
                        pa[base + b] |= 1ull;
                        front[nf] = key_id(pa[base + b]);
                    }
                    last = base + b;
                    ++nf;
                }
            }
            __syncwarp();
            if (nf == 0) break;
            fu = last + 1;
            // fresh neighbours, in adjacency order, frontier node by frontier node
            uint32_t nfresh = 0;
            bool bad = false;
            for (uint32_t f = 0; f < nf; ++f) {
                const uint32_t node = front[f];
                const uint32_t dg = a.deg[node];
                const uint32_t *row = a.adj + static_cast<size_t>(node) * a.r;
                for (uint32_t c = 0; c < dg; c += 32) {
                    const uint32_t j = c + lane;
                    const uint32_t nb = j < dg ? row[j] : kNoNode;
                    const bool in_range = nb < a.node_count;
                    if (j < dg && !in_range) bad = true;
                    const bool fresh = in_range && tag[nb] != e;
                    const unsigned m = __ballot_sync(0xffffffffu, fresh);
                    if (fresh) {
                        tag[nb] = e;
                        fid[nfresh + __popc(m & lanemask_lt())] = nb;
                    }
                    nfresh += __popc(m);
                    __syncwarp();
                }
            }
            if (__any_sync(0xffffffffu, bad)) {
                failed = true;
                break;
            }
            if (nfresh == 0) {
                if (a.stop != 0 && n >= a.l) {
                    stall = key_dist(pa[n - 1]) >= back_before ? stall + 1 : 0;
                    if (stall >= a.stop) break;
                }
                continue;
            }
            my_evals += nfresh;
            score_batch<D>(qc, qa, true, a.codes, a.aux, fid, static_cast<int>(nfresh),
                           [&](int c, float d) { fd[c] = d; });
            __syncwarp();
            uint32_t p2 = 32;
            while (p2 < nfresh) p2 <<= 1;
            for (uint32_t i = lane; i < p2; i += 32) fk[i] = i < nfresh ? make_key(fd[i], fid[i]) : kKeyMax;
            __syncwarp();
            warp_bitonic(fk, static_cast<int>(p2));
            // merge: the l smallest of the pool (n, sorted) and the fresh keys (sorted) into pb
            for (uint32_t i = lane; i < n; i += 32) {
                const unsigned long long k = pa[i];
                uint32_t lo = 0, hi = nfresh;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (fk[mid] < k) lo = mid + 1; else hi = mid;
                }
                if (i + lo < a.l) pb[i + lo] = k;
            }
            for (uint32_t j = lane; j < nfresh; j += 32) {
                const unsigned long long k = fk[j];
                uint32_t lo = 0, hi = n;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (pa[mid] < k) lo = mid + 1; else hi = mid;
                }
                if (j + lo < a.l) pb[j + lo] = k;
            }
            {  // the smallest fresh key's place bounds the first unexpanded entry from below
                const unsigned long long k0 = fk[0];
                uint32_t lo = 0, hi = n;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (pa[mid] < k0) lo = mid + 1; else hi = mid;
                }
                fu = min(fu, lo);
            }
            __syncwarp();
            n = min(a.l, n + nfresh);
            unsigned long long *t = pa;
            pa = pb;
            pb = t;
            if (a.stop != 0 && n >= a.l) {
                stall = key_dist(pa[n - 1]) >= back_before ? stall + 1 : 0;
                if (stall >= a.stop) break;
            }
        }
        if (failed) {
            if (lane == 0) atomicExch(a.error, 1);
            n = 0;
        }
        unsigned long long *out = a.pools + static_cast<size_t>(item) * a.l;
        for (uint32_t i = lane; i < n; i += 32) out[i] = pa[i] & ~1ull;
        if (lane == 0) a.pool_n[item] = n;
        __syncwarp();
    }
    if (lane == 0 && my_evals) atomicAdd(a.evals, my_evals);
}

// ----------------------------------------------------------------------------------------------
// robust_prune_4bit for one source, one warp. ws_* hold m candidates; keys may be unsorted.
// ----------------------------------------------------------------------------------------------
struct PruneWs {
    unsigned long long *in;      // m keys as given
    unsigned long long *sorted;  // m keys, sorted and de-duplicated in place
    float *mind;                 // m
    uint8_t *state;              // m: 0 live, 1 selected, 2 occluded at every alpha
};

struct PruneCfg {
    const float *alphas;  // the ramp 1, x step, ..., alpha (float products, as the reference)
    int npass;
    uint32_t r;
};

// Rank sort of distinct-or-equal keys (equal keys keep input order), then drop the source and
// duplicate keys. Returns the unique count.
__device__ uint32_t prune_sort_unique(const PruneWs &w, uint32_t m, uint32_t source, bool presorted) {
    const int lane = threadIdx.x & 31;
    if (presorted) {
        for (uint32_t i = lane; i < m; i += 32) w.sorted[i] = w.in[i];
    } else {
        for (uint32_t i = lane; i < m; i += 32) {
            const unsigned long long k = w.in[i];
            uint32_t rank = 0;
            for (uint32_t j = 0; j < m; ++j) {
                const unsigned long long o = w.in[j];
                rank += (o < k) || (o == k && j < i);
            }
            w.sorted[rank] = k;
        }
    }
    __syncwarp();
    uint32_t u = 0;
    unsigned long long prev = kKeyMax;  // no key equals it (ids < 2^31)
    for (uint32_t base = 0; base < m; base += 32) {
        const uint32_t i = base + lane;
        const unsigned long long k = i < m ? w.sorted[i] : kKeyMax;
        unsigned long long before = __shfl_up_sync(0xffffffffu, k, 1);
        if (lane == 0) before = prev;
        const bool keep = i < m && key_id(k) != source && k != before;
        prev = __shfl_sync(0xffffffffu, k, 31);
        const unsigned mk = __ballot_sync(0xffffffffu, keep);
        __syncwarp();
        if (keep) {
            const uint32_t pos = u + __popc(mk & lanemask_lt());
            w.sorted[pos] = k;
            w.mind[pos] = __int_as_float(0x7fc00000);  // NaN: no selected neighbour yet
            w.state[pos] = 0;
        }
        u += __popc(mk);
        __syncwarp();
    }
    return u;
}

template <int D>
__device__ uint32_t prune_select(const PruneWs &w, uint32_t u, const PruneCfg &cfg, const uint4 *codes,
                                 const VbAux *aux, uint32_t *out, unsigned long long &evals) {
    const int lane = threadIdx.x & 31, g = lane % Geo<D>::kG, grp = lane / Geo<D>::kG;
    const float a_lo = cfg.alphas[0], a_hi = cfg.alphas[cfg.npass - 1];
    uint32_t nsel = 0;
    for (int p = 0; p < cfg.npass && nsel < cfg.r; ++p) {
        const float alpha = cfg.alphas[p];
        uint32_t i = 0;
        while (nsel < cfg.r) {
            int found = -1;
            for (uint32_t base = i; base < u; base += 32) {
                const uint32_t idx = base + lane;
                bool ok = false;
                if (idx < u && w.state[idx] == 0) ok = !(alpha * w.mind[idx] <= key_dist(w.sorted[idx]));
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (m) {
                    found = static_cast<int>(base) + __ffs(m) - 1;
                    break;
                }
            }
            if (found < 0) break;
            const uint32_t s = key_id(w.sorted[found]);
            if (lane == 0) {
                out[nsel] = s;
                w.state[found] = 1;
            }
            ++nsel;
            __syncwarp();
            if (nsel == cfg.r) break;
            uint4 sc[Geo<D>::kPer];
            load_code<D>(codes, s, g, sc);
            const VbAux sa = aux[s];
            // every live candidate, lhs = candidate, rhs = the new neighbour
            for (uint32_t base = 0; base < u; base += 32) {
                const uint32_t idx = base + lane;
                unsigned m = __ballot_sync(0xffffffffu, idx < u && w.state[idx] == 0);
                while (m) {
                    // group `grp` takes the grp-th remaining live candidate of this chunk
                    unsigned mm = m;
                    for (int k = 0; k < grp && mm; ++k) mm &= mm - 1;
                    const int b = mm ? __ffs(mm) - 1 : -1;
                    uint32_t acc = 0;
                    uint32_t cid = 0;
                    const uint32_t cidx = base + static_cast<uint32_t>(b);
                    if (b >= 0) {
                        cid = key_id(w.sorted[cidx]);
                        uint4 x[Geo<D>::kPer];
                        load_code<D>(codes, cid, g, x);
#pragma unroll
                        for (int k = 0; k < Geo<D>::kPer; ++k) acc = nib_dot4(sc[k], x[k], acc);
                    }
#pragma unroll
                    for (int o = Geo<D>::kG / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                    if (b >= 0 && g == 0) {
                        const float d = sym_distance<D>(aux[cid], sa, acc);
                        const float nm = fminf(w.mind[cidx], d);
                        w.mind[cidx] = nm;
                        const float dist = key_dist(w.sorted[cidx]);
                        if (a_hi * nm <= dist && a_lo * nm <= dist) w.state[cidx] = 2;
                        evals += 1;
                    }
                    for (int k = 0; k < Geo<D>::kCands && m; ++k) m &= m - 1;
                }
            }
            __syncwarp();
            i = static_cast<uint32_t>(found) + 1;
        }
    }
    return nsel;
}

// Prune tasks of the search pools: task t = node first + t; candidates = the first
// min(pool_n, cap) pool entries (+ the node's current neighbours in a refinement pass).
struct VbPoolPruneArgs {
    const uint4 *codes;
    const VbAux *aux;
    const unsigned long long *pools;
    const uint32_t *pool_n;
    uint32_t l, cap;  // cap 0 = no cap
    uint32_t first, count;
    const uint32_t *old_adj;  // refinement: current neighbours appended (else null)
    const uint32_t *old_deg;
    uint32_t *adj_out;
    uint32_t *deg_out;
    uint32_t r;
    PruneCfg cfg;
    unsigned long long *ws_keys;  // 2 x ws_stride per task
    float *ws_mind;
    uint8_t *ws_state;
    uint32_t ws_stride;
    unsigned int *work;
    unsigned long long *evals;
};

template <int D>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) vb_pool_prune_kernel(VbPoolPruneArgs a) {
    const int lane = threadIdx.x & 31, g = lane % Geo<D>::kG;
    unsigned long long evals = 0;
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(a.work, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= a.count) break;
        const uint32_t id = a.first + t;
        PruneWs w;
        w.in = a.ws_keys + static_cast<size_t>(t) * 2 * a.ws_stride;
        w.sorted = w.in + a.ws_stride;
        w.mind = a.ws_mind + static_cast<size_t>(t) * a.ws_stride;
        w.state = a.ws_state + static_cast<size_t>(t) * a.ws_stride;
        uint32_t m = a.pool_n[t];
        if (a.cap != 0 && m > a.cap) m = a.cap;  // the pool is sorted: its first cap entries
        const unsigned long long *pool = a.pools + static_cast<size_t>(t) * a.l;
        for (uint32_t i = lane; i < m; i += 32) w.in[i] = pool[i];
        bool presorted = true;
        if (a.old_adj != nullptr) {
            const uint32_t dg = a.old_deg[id];
            if (dg) {
                presorted = false;
                uint4 qc[Geo<D>::kPer];
                load_code<D>(a.codes, id, g, qc);
                const VbAux qa = a.aux[id];
                const uint32_t *row = a.old_adj + static_cast<size_t>(id) * a.r;
                unsigned long long *dst = w.in + m;
                score_batch<D>(qc, qa, true, a.codes, a.aux, row, static_cast<int>(dg),
                               [&](int c, float d) { dst[c] = make_key(d, row[c]); });
                evals += dg;
                m += dg;
            }
        }
        __syncwarp();
        const uint32_t u = prune_sort_unique(w, m, id, presorted);
        uint32_t *out = a.adj_out + static_cast<size_t>(id) * a.r;
        const uint32_t nsel = prune_select<D>(w, u, a.cfg, a.codes, a.aux, out, evals);
        if (lane == 0) a.deg_out[id] = nsel;
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
    if (lane == 0 && evals) atomicAdd(a.evals, evals);
}

// ----------------------------------------------------------------------------------------------
// back-edges: count by source, exclusive scan, scatter, then one warp per source
// ----------------------------------------------------------------------------------------------
__global__ void vb_count_kernel(const uint32_t *adj, const uint32_t *deg, uint32_t r, uint32_t first, uint32_t count,
                                uint32_t *cnt) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<size_t>(count) * r) return;
    const uint32_t id = first + static_cast<uint32_t>(i / r), j = static_cast<uint32_t>(i % r);
    if (j < deg[id]) atomicAdd(&cnt[adj[static_cast<size_t>(id) * r + j]], 1u);
}

__global__ void vb_scatter_kernel(const uint32_t *adj, const uint32_t *deg, uint32_t r, uint32_t first,
                                  uint32_t count, const uint32_t *offs, uint32_t *fill, uint32_t *tgt) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<size_t>(count) * r) return;
    const uint32_t id = first + static_cast<uint32_t>(i / r), j = static_cast<uint32_t>(i % r);
    if (j < deg[id]) {
        const uint32_t src = adj[static_cast<size_t>(id) * r + j];
        tgt[offs[src] + atomicAdd(&fill[src], 1u)] = id;
    }
}

// Exclusive scan of n counts into offs[0..n] (offs[n] = total), three passes.
constexpr int kScanBlock = 1024;
__global__ void vb_scan_sums_kernel(const uint32_t *in, size_t n, uint32_t *bsum) {
    __shared__ uint32_t s[32];
    const size_t base = static_cast<size_t>(blockIdx.x) * kScanBlock;
    uint32_t v = 0;
    for (int i = threadIdx.x; i < kScanBlock; i += blockDim.x)
        if (base + i < n) v += in[base + i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += s[w];
        bsum[blockIdx.x] = t;
    }
}

__global__ void vb_scan_top_kernel(uint32_t *bsum, int nb) {
    if (threadIdx.x != 0) return;  // at most a few thousand block sums
    uint32_t run = 0;
    for (int i = 0; i < nb; ++i) {
        const uint32_t v = bsum[i];
        bsum[i] = run;
        run += v;
    }
    bsum[nb] = run;
}

__global__ void vb_scan_apply_kernel(const uint32_t *in, size_t n, const uint32_t *bsum, uint32_t *offs) {
    __shared__ uint32_t s[kScanBlock];
    const size_t base = static_cast<size_t>(blockIdx.x) * kScanBlock;
    for (int i = threadIdx.x; i < kScanBlock; i += blockDim.x) s[i] = base + i < n ? in[base + i] : 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = bsum[blockIdx.x];
        for (int i = 0; i < kScanBlock; ++i) {
            const uint32_t v = s[i];
            s[i] = run;
            run += v;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kScanBlock; i += blockDim.x)
        if (base + i < n) offs[base + i] = s[i];
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) offs[n] = bsum[gridDim.x];
}

// Group pass 1: sort the source's targets (rank sort; the targets of one source are distinct
// and never the source), append those not yet neighbours. A list still within R is written
// back; a longer one records its length in need[] for the pruning pass.
__global__ void vb_group_append_kernel(uint32_t *adj, uint32_t *deg, uint32_t r, uint32_t nc, const uint32_t *offs,
                                       const uint32_t *tgt, uint32_t *tgt_sorted, uint32_t *need, uint32_t pmax,
                                       uint32_t pmax_big, uint32_t *glist, uint32_t *gcount, uint32_t *glist_big,
                                       uint32_t *gcount_big) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); s < nc; s += warps) {
        const uint32_t b = offs[s], t = offs[s + 1] - b;
        if (lane == 0) need[s] = 0;
        if (t == 0) continue;
        for (uint32_t i = lane; i < t; i += 32) {
            const uint32_t v = tgt[b + i];
            uint32_t rank = 0;
            for (uint32_t j = 0; j < t; ++j) rank += tgt[b + j] < v;
            tgt_sorted[b + rank] = v;
        }
        __syncwarp();
        uint32_t *row = adj + static_cast<size_t>(s) * r;
        const uint32_t dg = deg[s];
        const uint32_t n0 = lane < dg ? row[lane] : kNoNode, n1 = lane + 32 < dg ? row[lane + 32] : kNoNode;
        uint32_t added = 0;
        for (uint32_t base = 0; base < t; base += 32) {
            const uint32_t i = base + lane;
            const uint32_t v = i < t ? tgt_sorted[b + i] : kNoNode;
            bool present = v == kNoNode;
            for (uint32_t j = 0; j < dg; ++j) {
                const uint32_t nb = j < 32 ? __shfl_sync(0xffffffffu, n0, j) : __shfl_sync(0xffffffffu, n1, j - 32);
                present |= nb == v;
            }
            const unsigned m = __ballot_sync(0xffffffffu, !present);
            if (!present) {
                const uint32_t pos = dg + added + __popc(m & lanemask_lt());
                if (pos < r) row[pos] = v;
            }
            added += __popc(m);
        }
        __syncwarp();
        if (added == 0) continue;
        if (dg + added <= r) {
            if (lane == 0) deg[s] = dg + added;
        } else if (lane == 0) {
            if (dg + added <= pmax) glist[atomicAdd(gcount, 1u)] = s;  // any order: sources are independent
            else if (dg + added <= pmax_big) glist_big[atomicAdd(gcount_big, 1u)] = s;
            else need[s] = dg + added;
        }
    }
}

// Rebuilds a source's candidate list for a re-prune: its current neighbours, then its sorted
// targets that are not among them (the order addBackedgeGroupAndPrune appends them in). One
// warp; returns the count.
__device__ uint32_t vb_merged_list(const uint32_t *row, uint32_t dg, const uint32_t *targets, uint32_t t,
                                   uint32_t *ids) {
    const int lane = threadIdx.x & 31;
    for (uint32_t i = lane; i < dg; i += 32) ids[i] = row[i];
    const uint32_t n0 = lane < dg ? row[lane] : kNoNode, n1 = lane + 32 < dg ? row[lane + 32] : kNoNode;
    uint32_t added = 0;
    for (uint32_t base = 0; base < t; base += 32) {
        const uint32_t i = base + lane;
        const uint32_t v = i < t ? targets[i] : kNoNode;
        bool present = v == kNoNode;
        for (uint32_t j = 0; j < dg; ++j) {
            const uint32_t nb = j < 32 ? __shfl_sync(0xffffffffu, n0, j) : __shfl_sync(0xffffffffu, n1, j - 32);
            present |= nb == v;
        }
        const unsigned mk = __ballot_sync(0xffffffffu, !present);
        if (!present) ids[dg + added + __popc(mk & lanemask_lt())] = v;
        added += __popc(mk);
    }
    __syncwarp();
    return dg + added;
}

// Group pass 2a: re-prune of one source per CTA with every candidate code in shared memory.
// All pairwise centred code products (and those with the source) are computed first, in
// parallel, as an integer Gram matrix; the selection then runs on one warp and finishes each
// distance it needs in double precision from the cached product, lhs = the candidate being
// checked, rhs = the selected neighbour, as robust_prune_4bit does.
// kPmax candidates per CTA: the small configuration fits two or three CTAs per SM, the big one
// (lists grown by many back-edges at once, early in the build) one CTA of eight warps per SM.
template <int D, bool kBig>
struct GramCfg {
    static constexpr int kPmax = kBig ? 150 : (D >= 2048 ? 79 : (D >= 1024 ? 95 : 127));
    static constexpr int kThreads = 256;
    static constexpr int kSlots = kPmax + 1;                // + the source
    static constexpr int kRows = (kSlots + 15) / 16 * 16;   // MMA row blocks of 16
    static constexpr int kCodeBytes = D / 2;
    static constexpr int kStride = kCodeBytes + 16;         // padded: rows start in different banks
    // the codes, then (after the Gram) the distance matrix, share the first region
    static constexpr size_t kCodesBytes = static_cast<size_t>(kRows) * kStride;
    static constexpr size_t kDmatBytes = static_cast<size_t>(kSlots) * kSlots * 4;
    static constexpr size_t kOffLut = ((kCodesBytes > kDmatBytes ? kCodesBytes : kDmatBytes) + 15) & ~static_cast<size_t>(15);
    static constexpr size_t kOffAux = kOffLut + 256 * 4;
    static constexpr size_t kOffGram = kOffAux + static_cast<size_t>(kSlots) * sizeof(VbAux);
    static constexpr size_t kGramWords = static_cast<size_t>(kSlots) * (kSlots - 1) / 2;
    static constexpr size_t kOffKeys = kOffGram + ((kGramWords * 4 + 15) & ~static_cast<size_t>(15));
    static constexpr size_t kOffOrder = kOffKeys + kPmax * 8;
    static constexpr size_t kOffMind = kOffOrder + kPmax * 4;
    static constexpr size_t kOffIds = kOffMind + kPmax * 4;
    static constexpr size_t kOffState = kOffIds + kPmax * 4;
    static constexpr size_t kOffMisc = (kOffState + kPmax + 15) & ~static_cast<size_t>(15);
    static constexpr size_t kBytes = kOffMisc + 16;
};

// D = A B + C, m16n8k16, bf16 inputs, f32 accumulate (row-major A, column-major B).
__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                               uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t tri_index(uint32_t i, uint32_t j) {  // i != j
    const uint32_t lo = min(i, j), hi = max(i, j);
    return hi * (hi - 1) / 2 + lo;
}

struct VbGramArgs {
    const uint4 *codes;
    const VbAux *aux;
    uint32_t *adj;
    uint32_t *deg;
    uint32_t r;
    const uint32_t *offs;
    const uint32_t *tgt_sorted;
    const uint32_t *glist;
    const uint32_t *gcount;
    PruneCfg cfg;
    unsigned int *work;
    unsigned long long *evals;
};

template <int D, bool kBig>
__global__ void __launch_bounds__(GramCfg<D, kBig>::kThreads) vb_group_gram_kernel(VbGramArgs a) {
    using Cfg = GramCfg<D, kBig>;
    extern __shared__ __align__(16) unsigned char gsm[];
    uint32_t *lut = reinterpret_cast<uint32_t *>(gsm + Cfg::kOffLut);
    VbAux *saux = reinterpret_cast<VbAux *>(gsm + Cfg::kOffAux);
    uint32_t *gram = reinterpret_cast<uint32_t *>(gsm + Cfg::kOffGram);
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(gsm + Cfg::kOffKeys);
    uint32_t *order = reinterpret_cast<uint32_t *>(gsm + Cfg::kOffOrder);
    float *mind = reinterpret_cast<float *>(gsm + Cfg::kOffMind);
    uint32_t *ids = reinterpret_cast<uint32_t *>(gsm + Cfg::kOffIds);
    uint8_t *state = gsm + Cfg::kOffState;
    uint32_t *misc = reinterpret_cast<uint32_t *>(gsm + Cfg::kOffMisc);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int kChunks = D / 32;
    constexpr int kG = Geo<D>::kG, kPer = Geo<D>::kPer, kCands = Geo<D>::kCands;
    const int grp = lane / kG, g = lane % kG;
    const uint32_t total = *a.gcount;
    unsigned long long evals = 0;
    for (int b = tid; b < 256; b += blockDim.x) {  // byte -> (bf16(2 lo - 15), bf16(2 hi - 15))
        const __nv_bfloat162 v = __floats2bfloat162_rn(static_cast<float>(2 * (b & 15) - 15),
                                                       static_cast<float>(2 * (b >> 4) - 15));
        lut[b] = *reinterpret_cast<const uint32_t *>(&v);
    }
    for (;;) {
        if (tid == 0) misc[0] = atomicAdd(a.work, 1u);
        __syncthreads();
        const uint32_t item = misc[0];
        if (item >= total) break;
        const uint32_t s = a.glist[item];
        uint32_t *row = a.adj + static_cast<size_t>(s) * a.r;
        if (warp == 0) {
            const uint32_t b = a.offs[s];
            const uint32_t m = vb_merged_list(row, a.deg[s], a.tgt_sorted + b, a.offs[s + 1] - b, ids);
            if (lane == 0) misc[1] = m;
        }
        __syncthreads();
        const uint32_t m = misc[1];  // <= kPmax (the append pass routes larger lists elsewhere)
        // stage codes and factors: slots 0..m-1 the candidates, slot m the source
        // asynchronous copies: every chunk in flight at once, no register round trip
        for (uint32_t x = tid; x < (m + 1) * kChunks; x += blockDim.x) {
            const uint32_t slot = x / kChunks, c = x % kChunks;
            const uint32_t node = slot < m ? ids[slot] : s;
            const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(gsm + slot * Cfg::kStride + c * 16));
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst),
                         "l"(a.codes + static_cast<size_t>(node) * kChunks + c)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        for (uint32_t slot = tid; slot <= m; slot += blockDim.x) saux[slot] = a.aux[slot < m ? ids[slot] : s];
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
        // Gram of slots 0..m on the tensor cores: the centred codes 2a - 15 are integers of at most
        // 15 in magnitude, exact in bf16, and every partial sum of their products (at most
        // 225 D < 2^24) is exact in the f32 accumulator, so the products come out exact. Tiles of
        // 16 x 16 on and above the diagonal; fragments built from the packed nibbles through the
        // byte -> bf16 pair table. Rows past m hold stale codes and are never stored.
        {
            const int Q = static_cast<int>((m + 1 + 15) / 16);
            const int ntiles = Q * (Q + 1) / 2;
            const int gq = lane >> 2, tq = lane & 3;
            for (int ti = warp; ti < ntiles; ti += static_cast<int>(blockDim.x >> 5)) {
                int q = 0, rem = ti;
                while (rem >= Q - q) {
                    rem -= Q - q;
                    ++q;
                }
                const int c = q + rem;
                const uint8_t *ra0 = gsm + (16 * q + gq) * Cfg::kStride + tq;
                const uint8_t *ra1 = ra0 + 8 * Cfg::kStride;
                const uint8_t *rb0 = gsm + (16 * c + gq) * Cfg::kStride + tq;
                const uint8_t *rb1 = rb0 + 8 * Cfg::kStride;
                float acc0[4] = {0.f, 0.f, 0.f, 0.f}, acc1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
                for (int ks = 0; ks < D / 16; ++ks) {
                    const int o = ks * 8;
                    const uint32_t a0 = lut[ra0[o]], a1 = lut[ra1[o]], a2 = lut[ra0[o + 4]], a3 = lut[ra1[o + 4]];
                    const uint32_t b00 = lut[rb0[o]], b01 = lut[rb0[o + 4]];
                    const uint32_t b10 = lut[rb1[o]], b11 = lut[rb1[o + 4]];
                    mma_bf16_16816(acc0, a0, a1, a2, a3, b00, b01);
                    mma_bf16_16816(acc1, a0, a1, a2, a3, b10, b11);
                }
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const float v = k < 4 ? acc0[k] : acc1[k - 4];
                    const uint32_t i = 16 * q + gq + ((k & 2) ? 8 : 0);
                    const uint32_t j = 16 * c + ((k & 4) ? 8 : 0) + 2 * tq + (k & 1);
                    if (i < j && j <= m) gram[j * (j - 1) / 2 + i] = static_cast<uint32_t>(__float2int_rn(v));
                }
            }
        }
        __syncthreads();
        // every distance the selection can need, in parallel: dmat[i][j] = d(lhs i, rhs j) over
        // slots 0..m (row m = the source), written over the codes (no longer needed)
        float *dmat = reinterpret_cast<float *>(gsm);
        const uint32_t w = m + 1;
#pragma unroll 2
        for (uint32_t x = tid; x < w * w; x += blockDim.x) {
            const uint32_t i = x / w, j = x % w;
            if (i == j || j == m) continue;
            dmat[x] = sym_distance_exact(saux[i], saux[j], static_cast<int32_t>(gram[tri_index(i, j)]));
        }
        __syncthreads();
        evals += (m * m) / blockDim.x + (tid < (m * m) % blockDim.x ? 1 : 0);
        for (uint32_t i = tid; i < m; i += blockDim.x) keys[i] = make_key(dmat[m * w + i], ids[i]);
        __syncthreads();
        for (uint32_t i = tid; i < m; i += blockDim.x) {
            const unsigned long long k = keys[i];
            uint32_t rank = 0;
            for (uint32_t j = 0; j < m; ++j) rank += keys[j] < k;  // ids distinct: no ties
            order[rank] = i;
            mind[rank] = __int_as_float(0x7fc00000);
            state[rank] = 0;
        }
        __syncthreads();
        // selection: every warp scans the same shared state and finds the same candidate; the
        // updates of the live candidates are spread over the block
        {
            const float a_lo = a.cfg.alphas[0], a_hi = a.cfg.alphas[a.cfg.npass - 1];
            uint32_t nsel = 0;
            for (int p = 0; p < a.cfg.npass && nsel < a.r; ++p) {
                const float alpha = a.cfg.alphas[p];
                uint32_t i = 0;
                while (nsel < a.r) {
                    int found = -1;
                    for (uint32_t base = i; base < m; base += 32) {
                        const uint32_t x = base + lane;
                        bool ok = false;
                        if (x < m && state[x] == 0) ok = !(alpha * mind[x] <= key_dist(keys[order[x]]));
                        const unsigned mk = __ballot_sync(0xffffffffu, ok);
                        if (mk) {
                            found = static_cast<int>(base) + __ffs(mk) - 1;
                            break;
                        }
                    }
                    __syncthreads();  // every warp has scanned before anything changes
                    if (found < 0) break;
                    const uint32_t fslot = order[found];
                    if (tid == 0) {
                        row[nsel] = ids[fslot];
                        state[found] = 1;
                    }
                    ++nsel;
                    if (nsel == a.r) break;
                    for (uint32_t x = tid; x < m; x += blockDim.x) {
                        if (x == static_cast<uint32_t>(found) || state[x] != 0) continue;
                        const uint32_t cs = order[x];
                        const float nm = fminf(mind[x], dmat[cs * w + fslot]);
                        mind[x] = nm;
                        const float dist = key_dist(keys[cs]);
                        if (a_hi * nm <= dist && a_lo * nm <= dist) state[x] = 2;
                    }
                    __syncthreads();
                    i = static_cast<uint32_t>(found) + 1;
                }
            }
            if (tid == 0) a.deg[s] = nsel;
        }
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
    if (lane == 0 && evals) atomicAdd(a.evals, evals);
}

// Group pass 2: sources whose list grew past R: candidates = old neighbours then the appended
// targets, distances from the source, robust_prune_4bit.
struct VbGroupPruneArgs {
    const uint4 *codes;
    const VbAux *aux;
    uint32_t *adj;
    uint32_t *deg;
    uint32_t r;
    uint32_t nc;
    const uint32_t *offs;
    const uint32_t *tgt_sorted;
    const uint32_t *need;
    const uint32_t *noffs;  // exclusive scan of need
    PruneCfg cfg;
    unsigned long long *ws_keys;  // 2 x noffs[nc]
    float *ws_mind;
    uint8_t *ws_state;
    uint32_t *ws_ids;  // noffs[nc]
    unsigned long long *evals;
};

template <int D>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) vb_group_prune_kernel(VbGroupPruneArgs a) {
    const int lane = threadIdx.x & 31, g = lane % Geo<D>::kG;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    unsigned long long evals = 0;
    const size_t total = a.noffs[a.nc];
    for (uint32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); s < a.nc; s += warps) {
        const uint32_t m = a.need[s];
        if (m == 0) continue;
        const size_t o = a.noffs[s];
        uint32_t *ids = a.ws_ids + o;
        uint32_t *row = a.adj + static_cast<size_t>(s) * a.r;
        const uint32_t dg = a.deg[s];
        for (uint32_t i = lane; i < dg; i += 32) ids[i] = row[i];
        const uint32_t b = a.offs[s], t = a.offs[s + 1] - b;
        const uint32_t n0 = lane < dg ? row[lane] : kNoNode, n1 = lane + 32 < dg ? row[lane + 32] : kNoNode;
        uint32_t added = 0;
        for (uint32_t base = 0; base < t; base += 32) {
            const uint32_t i = base + lane;
            const uint32_t v = i < t ? a.tgt_sorted[b + i] : kNoNode;
            bool present = v == kNoNode;
            for (uint32_t j = 0; j < dg; ++j) {
                const uint32_t nb = j < 32 ? __shfl_sync(0xffffffffu, n0, j) : __shfl_sync(0xffffffffu, n1, j - 32);
                present |= nb == v;
            }
            const unsigned mk = __ballot_sync(0xffffffffu, !present);
            if (!present) ids[dg + added + __popc(mk & lanemask_lt())] = v;
            added += __popc(mk);
        }
        __syncwarp();
        PruneWs w;
        w.in = a.ws_keys + o;
        w.sorted = a.ws_keys + total + o;
        w.mind = a.ws_mind + o;
        w.state = a.ws_state + o;
        uint4 sc[Geo<D>::kPer];
        load_code<D>(a.codes, s, g, sc);
        const VbAux sa = a.aux[s];
        score_batch<D>(sc, sa, true, a.codes, a.aux, ids, static_cast<int>(m),
                       [&](int c, float d) { w.in[c] = make_key(d, ids[c]); });
        evals += m;
        __syncwarp();
        const uint32_t u = prune_sort_unique(w, m, s, false);
        const uint32_t nsel = prune_select<D>(w, u, a.cfg, a.codes, a.aux, row, evals);
        if (lane == 0) a.deg[s] = nsel;
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
    if (lane == 0 && evals) atomicAdd(a.evals, evals);
}

// Final lists into the caller's layout; slots past a node's degree are zero.
__global__ void vb_export_kernel(const uint32_t *adj, const uint32_t *deg, uint32_t r, size_t n, uint32_t *edges,
                                 size_t edge_stride, uint32_t *degrees) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n * edge_stride) return;
    const size_t row = i / edge_stride, j = i % edge_stride;
    const uint32_t dg = deg[row];
    edges[i] = j < dg ? adj[row * r + j] : 0u;
    if (j == 0) degrees[row] = dg;
}

// ----------------------------------------------------------------------------------------------
// host orchestration
// ----------------------------------------------------------------------------------------------
struct DevMem {
    std::vector<void *> ptrs;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T *get(size_t count) {
        void *p = nullptr;
        if (err != cudaSuccess) return nullptr;
        err = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (err != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
    void release(void *p) {
        for (auto &q : ptrs)
            if (q == p) {
                cudaFree(q);
                q = nullptr;
            }
    }
    ~DevMem() {
        for (void *p : ptrs)
            if (p) cudaFree(p);
    }
};

#define VB_TRY(expr)                                  \
    do {                                              \
        const cudaError_t e_ = (expr);                \
        if (e_ != cudaSuccess) return e_;             \
    } while (0)

template <int D>
struct Builder {
    const VbBuildParams &p;
    size_t n;
    cudaStream_t st;
    DevMem mem;
    uint4 *codes = nullptr;
    VbAux *aux = nullptr;
    uint32_t *adj = nullptr, *deg = nullptr, *adj2 = nullptr, *deg2 = nullptr;
    uint16_t *tags = nullptr, *epochs = nullptr;
    unsigned long long *pools = nullptr, *pws_keys = nullptr;
    float *pws_mind = nullptr;
    uint8_t *pws_state = nullptr;
    uint32_t *pool_n = nullptr;
    uint32_t *cnt = nullptr, *fill = nullptr, *offs = nullptr, *tgt = nullptr, *tgt_sorted = nullptr, *need = nullptr,
             *noffs = nullptr, *bsum = nullptr, *glist = nullptr, *gcount = nullptr, *glist_big = nullptr;
    int gram_grid = 0, gram_big_grid = 0;
    unsigned int *work = nullptr;
    unsigned long long *evals = nullptr;
    int *error = nullptr;
    float *alphas = nullptr;
    int npass = 0;
    // group-prune workspace, grown on demand
    unsigned long long *gws_keys = nullptr;
    float *gws_mind = nullptr;
    uint8_t *gws_state = nullptr;
    uint32_t *gws_ids = nullptr;
    size_t gws_cap = 0;
    size_t chunk = 0, ws_stride = 0, pairs_cap = 0;
    int search_grid = 0, prune_grid = 0, group_grid = 0;
    size_t search_smem = 0;
    uint32_t fresh_cap = 0;

    Builder(const VbBuildParams &params, size_t count, cudaStream_t stream) : p(params), n(count), st(stream) {}

    template <bool kBig>
    static cudaError_t gram_grid_for(int sm_count, int &grid) {
        int per_sm = 0;
        VB_TRY(cudaFuncSetAttribute(vb_group_gram_kernel<D, kBig>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(GramCfg<D, kBig>::kBytes)));
        VB_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vb_group_gram_kernel<D, kBig>,
                                                             GramCfg<D, kBig>::kThreads, GramCfg<D, kBig>::kBytes));
        if (per_sm <= 0) return cudaErrorInvalidConfiguration;
        grid = sm_count * per_sm;
        return cudaSuccess;
    }

    template <bool kBig>
    cudaError_t launch_gram(const uint32_t *list, const uint32_t *count, int grid) {
        VB_TRY(cudaMemsetAsync(work, 0, sizeof(unsigned int), st));
        VbGramArgs ga{codes, aux, adj, deg, static_cast<uint32_t>(p.r), offs, tgt_sorted, list, count,
                      PruneCfg{alphas, npass, static_cast<uint32_t>(p.r)}, work, evals};
        vb_group_gram_kernel<D, kBig><<<grid, GramCfg<D, kBig>::kThreads, GramCfg<D, kBig>::kBytes, st>>>(ga);
        return cudaGetLastError();
    }

    cudaError_t scan(const uint32_t *in, size_t len, uint32_t *out) {
        const int nb = static_cast<int>((len + kScanBlock - 1) / kScanBlock);
        if (nb == 0) return cudaMemsetAsync(out, 0, sizeof(uint32_t), st);
        vb_scan_sums_kernel<<<nb, 256, 0, st>>>(in, len, bsum);
        vb_scan_top_kernel<<<1, 32, 0, st>>>(bsum, nb);
        vb_scan_apply_kernel<<<nb, 256, 0, st>>>(in, len, bsum, out);
        return cudaGetLastError();
    }

    cudaError_t setup(const uint8_t *d_compact, size_t stride, int sm_count) {
        codes = mem.get<uint4>(n * (D / 32));
        aux = mem.get<VbAux>(n);
        adj = mem.get<uint32_t>(n * p.r);
        deg = mem.get<uint32_t>(n);
        if (p.refine) {
            adj2 = mem.get<uint32_t>(n * p.r);
            deg2 = mem.get<uint32_t>(n);
        }
        // the ramp of robust_prune_4bit (vamana_prune.h:118-150)
        std::vector<float> ramp{1.0f};
        {
            float cur = 1.0f;
            const float step = std::min(p.alpha, 1.2f);
            for (int guard = 0; guard < 4096; ++guard) {
                if (cur == p.alpha) break;
                const float next = std::min(p.alpha, cur * step);
                if (next == cur) break;
                cur = next;
                ramp.push_back(cur);
            }
        }
        npass = static_cast<int>(ramp.size());
        alphas = mem.get<float>(ramp.size());
        fresh_cap = 32;
        while (fresh_cap < p.beam * p.r) fresh_cap <<= 1;
        search_smem = vb_search_words(static_cast<uint32_t>(p.l_build), fresh_cap, static_cast<uint32_t>(p.beam)) *
                      8 * kWarpsPerBlock;
        int blocks_per_sm = 0;
        VB_TRY(cudaFuncSetAttribute(vb_search_kernel<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(search_smem)));
        VB_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, vb_search_kernel<D>,
                                                             kWarpsPerBlock * 32, search_smem));
        if (blocks_per_sm <= 0) return cudaErrorInvalidConfiguration;
        blocks_per_sm = std::min(blocks_per_sm, 4);
        search_grid = sm_count * blocks_per_sm;
        prune_grid = sm_count * 4;
        group_grid = sm_count * 8;
        const size_t slots = static_cast<size_t>(search_grid) * kWarpsPerBlock;
        tags = mem.get<uint16_t>(slots * n);
        epochs = mem.get<uint16_t>(slots);
        chunk = std::min<size_t>(n, 131072);  // searches per launch
        const size_t capped = p.cap ? std::min<size_t>(p.cap, p.l_build) : p.l_build;
        ws_stride = capped + (p.refine ? p.r : 0);
        pools = mem.get<unsigned long long>(chunk * p.l_build);
        pool_n = mem.get<uint32_t>(chunk);
        pws_keys = mem.get<unsigned long long>(chunk * 2 * ws_stride);
        pws_mind = mem.get<float>(chunk * ws_stride);
        pws_state = mem.get<uint8_t>(chunk * ws_stride);
        cnt = mem.get<uint32_t>(n);
        fill = mem.get<uint32_t>(n);
        offs = mem.get<uint32_t>(n + 1);
        need = mem.get<uint32_t>(n);
        noffs = mem.get<uint32_t>(n + 1);
        bsum = mem.get<uint32_t>((n + kScanBlock - 1) / kScanBlock + 2);
        pairs_cap = std::max(std::min(std::max<size_t>(p.batch, 1), n), p.refine ? n : 0) * p.r;
        tgt = mem.get<uint32_t>(pairs_cap);
        tgt_sorted = mem.get<uint32_t>(pairs_cap);
        glist = mem.get<uint32_t>(n);
        glist_big = mem.get<uint32_t>(n);
        gcount = mem.get<uint32_t>(2);
        VB_TRY(gram_grid_for<false>(sm_count, gram_grid));
        VB_TRY(gram_grid_for<true>(sm_count, gram_big_grid));
        work = mem.get<unsigned int>(1);
        evals = mem.get<unsigned long long>(1);
        error = mem.get<int>(1);
        if (mem.err != cudaSuccess) return mem.err;
        VB_TRY(cudaMemcpyAsync(alphas, ramp.data(), ramp.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        VB_TRY(cudaMemsetAsync(tags, 0, slots * n * sizeof(uint16_t), st));
        VB_TRY(cudaMemsetAsync(epochs, 0, slots * sizeof(uint16_t), st));
        VB_TRY(cudaMemsetAsync(deg, 0, n * sizeof(uint32_t), st));
        VB_TRY(cudaMemsetAsync(evals, 0, sizeof(unsigned long long), st));
        VB_TRY(cudaMemsetAsync(error, 0, sizeof(int), st));
        vb_prepare_kernel<<<static_cast<unsigned>((n * 32 + 255) / 256), 256, 0, st>>>(
            d_compact, n, stride, D, reinterpret_cast<uint8_t *>(codes), aux);
        return cudaGetLastError();
    }

    cudaError_t search(uint32_t first, uint32_t count, uint32_t node_count) {
        VB_TRY(cudaMemsetAsync(work, 0, sizeof(unsigned int), st));
        VbSearchArgs a{codes, aux, adj, deg, static_cast<uint32_t>(p.r), node_count, first, count,
                       static_cast<uint32_t>(p.l_build), static_cast<uint32_t>(p.beam),
                       static_cast<uint32_t>(p.stop_hops), fresh_cap, tags, epochs, n, pools, pool_n, work, evals,
                       error};
        vb_search_kernel<D><<<search_grid, kWarpsPerBlock * 32, search_smem, st>>>(a);
        return cudaGetLastError();
    }

    cudaError_t prune_pools(uint32_t first, uint32_t count, bool refine_pass) {
        VB_TRY(cudaMemsetAsync(work, 0, sizeof(unsigned int), st));
        VbPoolPruneArgs a{codes, aux, pools, pool_n, static_cast<uint32_t>(p.l_build), static_cast<uint32_t>(p.cap),
                          first, count, refine_pass ? adj : nullptr, refine_pass ? deg : nullptr,
                          refine_pass ? adj2 : adj, refine_pass ? deg2 : deg, static_cast<uint32_t>(p.r),
                          PruneCfg{alphas, npass, static_cast<uint32_t>(p.r)}, pws_keys, pws_mind, pws_state,
                          static_cast<uint32_t>(ws_stride), work, evals};
        vb_pool_prune_kernel<D><<<prune_grid, kWarpsPerBlock * 32, 0, st>>>(a);
        return cudaGetLastError();
    }

    // addBackedgesGroupedAndPrune over the lists of nodes [first, first + count); sources < nc
    cudaError_t backedges(uint32_t first, uint32_t count, uint32_t nc) {
        const size_t slots = static_cast<size_t>(count) * p.r;
        if (slots == 0) return cudaSuccess;
        const unsigned eg = static_cast<unsigned>((slots + 255) / 256);
        VB_TRY(sub(0, [&] {
            VB_TRY(cudaMemsetAsync(cnt, 0, nc * sizeof(uint32_t), st));
            VB_TRY(cudaMemsetAsync(fill, 0, nc * sizeof(uint32_t), st));
            vb_count_kernel<<<eg, 256, 0, st>>>(adj, deg, static_cast<uint32_t>(p.r), first, count, cnt);
            return cudaGetLastError();
        }));
        VB_TRY(sub(1, [&] { return scan(cnt, nc, offs); }));
        VB_TRY(sub(2, [&] {
            vb_scatter_kernel<<<eg, 256, 0, st>>>(adj, deg, static_cast<uint32_t>(p.r), first, count, offs, fill,
                                                  tgt);
            VB_TRY(cudaMemsetAsync(gcount, 0, 2 * sizeof(uint32_t), st));
            vb_group_append_kernel<<<group_grid, 256, 0, st>>>(adj, deg, static_cast<uint32_t>(p.r), nc, offs, tgt,
                                                               tgt_sorted, need, GramCfg<D, false>::kPmax,
                                                               GramCfg<D, true>::kPmax, glist, gcount, glist_big,
                                                               gcount + 1);
            return cudaGetLastError();
        }));
        VB_TRY(sub(3, [&] { return launch_gram<false>(glist, gcount, gram_grid); }));
        VB_TRY(sub(4, [&] { return launch_gram<true>(glist_big, gcount + 1, gram_big_grid); }));
        uint32_t total = 0;
        VB_TRY(sub(5, [&] {
            VB_TRY(scan(need, nc, noffs));
            VB_TRY(cudaMemcpyAsync(&total, noffs + nc, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            return cudaStreamSynchronize(st);
        }));
        if (total == 0) return cudaSuccess;
        if (total > gws_cap) {
            mem.release(gws_keys);
            mem.release(gws_mind);
            mem.release(gws_state);
            mem.release(gws_ids);
            gws_cap = std::max<size_t>(total, gws_cap * 2);
            gws_keys = mem.get<unsigned long long>(2 * gws_cap);
            gws_mind = mem.get<float>(gws_cap);
            gws_state = mem.get<uint8_t>(gws_cap);
            gws_ids = mem.get<uint32_t>(gws_cap);
            if (mem.err != cudaSuccess) return mem.err;
        }
        VbGroupPruneArgs a{codes, aux, adj, deg, static_cast<uint32_t>(p.r), nc, offs, tgt_sorted, need, noffs,
                           PruneCfg{alphas, npass, static_cast<uint32_t>(p.r)}, gws_keys, gws_mind, gws_state,
                           gws_ids, evals};
        return sub(6, [&] {
            vb_group_prune_kernel<D><<<group_grid, kWarpsPerBlock * 32, 0, st>>>(a);
            return cudaGetLastError();
        });
    }

    cudaError_t check_error() {
        int h = 0;
        VB_TRY(cudaMemcpyAsync(&h, error, sizeof(int), cudaMemcpyDeviceToHost, st));
        VB_TRY(cudaStreamSynchronize(st));
        return h ? cudaErrorInvalidValue : cudaSuccess;
    }

    // QG_VB_TRACE=1 prints the time of each stage (search, prune, back-edges) of the bulk and
    // refinement phases to stderr; it synchronises around every stage.
    bool trace = false;
    double t_stage[2][3] = {{0, 0, 0}, {0, 0, 0}};
    double t_sub[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // back-edge sub-stages
    template <typename F>
    cudaError_t sub(int k, F f) {
        if (!trace) return f();
        VB_TRY(cudaStreamSynchronize(st));
        const auto t0 = std::chrono::steady_clock::now();
        VB_TRY(f());
        VB_TRY(cudaStreamSynchronize(st));
        t_sub[k] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return cudaSuccess;
    }
    template <typename F>
    cudaError_t timed(int phase, int stage, F f) {
        if (!trace) return f();
        VB_TRY(cudaStreamSynchronize(st));
        const auto t0 = std::chrono::steady_clock::now();
        VB_TRY(f());
        VB_TRY(cudaStreamSynchronize(st));
        t_stage[phase][stage] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return cudaSuccess;
    }

    cudaError_t run() {
        const char *tr = std::getenv("QG_VB_TRACE");
        trace = tr && tr[0] == '1';
        // bulk insertion (vamana_index.h:452-528)
        const size_t batch = std::max<size_t>(p.batch, 1);
        for (size_t begin = 1; begin < n; begin += batch) {
            const size_t end = std::min(n, begin + batch);
            for (size_t c0 = begin; c0 < end; c0 += chunk) {
                const uint32_t cnt_c = static_cast<uint32_t>(std::min(chunk, end - c0));
                VB_TRY(timed(0, 0, [&] {
                    return search(static_cast<uint32_t>(c0), cnt_c, static_cast<uint32_t>(begin));
                }));
                VB_TRY(timed(0, 1, [&] { return prune_pools(static_cast<uint32_t>(c0), cnt_c, false); }));
            }
            VB_TRY(timed(0, 2, [&] {
                return backedges(static_cast<uint32_t>(begin), static_cast<uint32_t>(end - begin),
                                 static_cast<uint32_t>(end));
            }));
            VB_TRY(check_error());
        }
        // refinement passes (vamana_index.h:328-422)
        for (size_t pass = 0; pass < p.refine && n > 1; ++pass) {
            for (size_t c0 = 0; c0 < n; c0 += chunk) {
                const uint32_t cnt_c = static_cast<uint32_t>(std::min(chunk, n - c0));
                VB_TRY(timed(1, 0, [&] {
                    return search(static_cast<uint32_t>(c0), cnt_c, static_cast<uint32_t>(n));
                }));
                VB_TRY(timed(1, 1, [&] { return prune_pools(static_cast<uint32_t>(c0), cnt_c, true); }));
            }
            std::swap(adj, adj2);
            std::swap(deg, deg2);
            VB_TRY(timed(1, 2, [&] {
                return backedges(0, static_cast<uint32_t>(n), static_cast<uint32_t>(n));
            }));
            VB_TRY(check_error());
        }
        if (trace)
            std::fprintf(stderr,
                         "vamana build: bulk search %.3f s prune %.3f s back-edges %.3f s | refine search %.3f s "
                         "prune %.3f s back-edges %.3f s\n",
                         t_stage[0][0], t_stage[0][1], t_stage[0][2], t_stage[1][0], t_stage[1][1], t_stage[1][2]);
        if (trace)
            std::fprintf(stderr,
                         "  back-edges: count %.3f scan %.3f scatter+append %.3f gram %.3f gram-big %.3f need-scan "
                         "%.3f warp-prune %.3f s\n",
                         t_sub[0], t_sub[1], t_sub[2], t_sub[3], t_sub[4], t_sub[5], t_sub[6]);
        return cudaSuccess;
    }
};

template <int D>
cudaError_t build_d(const uint8_t *d_compact, size_t n, size_t stride, const VbBuildParams &p, uint32_t *d_degrees,
                    uint32_t *d_edges, size_t edge_stride, unsigned long long *evals_out, cudaStream_t st) {
    int dev = 0, sms = 0;
    VB_TRY(cudaGetDevice(&dev));
    VB_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    Builder<D> b(p, n, st);
    VB_TRY(b.setup(d_compact, stride, sms));
    VB_TRY(b.run());
    vb_export_kernel<<<static_cast<unsigned>((n * edge_stride + 255) / 256), 256, 0, st>>>(
        b.adj, b.deg, static_cast<uint32_t>(p.r), n, d_edges, edge_stride, d_degrees);
    VB_TRY(cudaGetLastError());
    unsigned long long ev = 0;
    VB_TRY(cudaMemcpyAsync(&ev, b.evals, sizeof(ev), cudaMemcpyDeviceToHost, st));
    VB_TRY(cudaStreamSynchronize(st));
    if (evals_out) *evals_out = ev;
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_vamana_build(int code_dim, const uint8_t *d_compact, size_t n, size_t stride,
                                const VbBuildParams &p, uint32_t *d_degrees, uint32_t *d_edges, size_t edge_stride,
                                unsigned long long *evals_out, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    if (p.r == 0 || p.r > 64 || p.l_build == 0 || p.beam == 0 || p.beam * p.r > 1024 || edge_stride < p.r ||
        !(p.alpha >= 1.0f) || !std::isfinite(p.alpha) || n >= 0x7FFFFFFFull || n * p.r >= 0xFFFFFFFFull)
        return cudaErrorInvalidValue;
    if (n == 1) {
        VB_TRY(cudaMemsetAsync(d_degrees, 0, sizeof(uint32_t), stream));
        return cudaStreamSynchronize(stream);
    }
    switch (code_dim) {
        case 64: return build_d<64>(d_compact, n, stride, p, d_degrees, d_edges, edge_stride, evals_out, stream);
        case 128: return build_d<128>(d_compact, n, stride, p, d_degrees, d_edges, edge_stride, evals_out, stream);
        case 256: return build_d<256>(d_compact, n, stride, p, d_degrees, d_edges, edge_stride, evals_out, stream);
        case 512: return build_d<512>(d_compact, n, stride, p, d_degrees, d_edges, edge_stride, evals_out, stream);
        case 1024: return build_d<1024>(d_compact, n, stride, p, d_degrees, d_edges, edge_stride, evals_out, stream);
        case 2048: return build_d<2048>(d_compact, n, stride, p, d_degrees, d_edges, edge_stride, evals_out, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace qg
