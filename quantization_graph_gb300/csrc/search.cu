// search.cu -- persistent batched beam search of the Ours-DiskANN query path.
//
// Restates search_ours_paper_active_inner + flush_distance_batch
// (experiments/02_diskann_fair/src/ours_diskann.rs:1539-1986) with the Int8 query codec:
// start at node 0, sorted pool of L (distance, id) entries, frontier = first beam_width
// unexpanded entries; per expanded node: fresh = unvisited neighbours in adjacency order,
// the INT8 x 1-bit-MSB paper-prune gate for all fresh neighbours, a first prune check against
// the pool tail, the INT8 x remaining-3-bit traversal distance for the survivors (full FP32
// restore when the gate is invalid), then, in adjacency order, the re-check against the
// current tail and the sorted insert; finally the FP32 restore + residual4 rerank of the
// first max(rerank, k) pool entries sorted by (estimate, id).
//
// GPU mapping: one warp per query, persistent CTAs pulling query indices from a global
// counter. The INT8 query lives in registers: lane l owns the 32-dimension chunks
// l, l+32, ... (or, for D < 1024, a group of D/32 lanes covers one neighbour and the warp
// handles 32/(D/32) neighbours at once). Gate and traversal are exact int32 dot products
// (dp4a over nibble/byte masks), computed for a whole group of neighbours with their row
// loads in flight together, then reduced with a reduce-scatter butterfly that leaves each
// neighbour's sum in one lane. The accept/insert pass is warp-serial over survivors in
// adjacency order (the reference's result depends on that order); each insert is a
// warp-parallel rank + shift of the pool in shared memory. The visited set is one bit per
// graph node in a per-warp-slot row of global memory, cleared at the start of each query.
#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>

#include "mlp.cuh"
#include "qg_device.cuh"
#include "qg_kernels.h"

namespace qg {
namespace {

constexpr uint32_t kExpanded = 0x80000000u;
constexpr uint32_t kIdMask = 0x7FFFFFFFu;
constexpr int kMaxFresh = 64;   // fresh neighbours per expanded node (max degree)
constexpr int kMaxBeam = 8;

template <int D>
struct Lay {
    static constexpr int CH = D / 32;
    static constexpr int LPN = CH < 32 ? CH : 32;   // lanes per neighbour
    static constexpr int CPL = CH / LPN;            // 32-dim chunks per lane
    static constexpr int NBP = 32 / LPN;            // neighbours per pass
    static constexpr int PG = 4;                    // passes per batch (LPN < 32)
};

// Tile shape of the gate and traversal loops when one neighbour spans the warp (D >= 1024): how
// many neighbours' rows a lane keeps in flight, and the block size and residency the kernel is
// compiled for. Shape 0 (the default): 16 MSB chunks per lane in the gate, 2 code rows in the
// traversal (4 in the wide build at D = 2048, 8 at D = 1024); 1: 8 chunks; 2: 32 chunks; 3: twice
// the traversal rows; 4: shape 0 at the other residency. Shapes 1-4 exist for the Int8 / Int4 search at D = 1024 and 2048,
// chosen per index (qg_index_set_tile, the autotuner).
//
// Residency: "wide" = compiled for blocks of up to 7 warps with at least 3 resident per SM, which
// the compiler meets with 80 registers (small spills); the launch geometry then packs 24 warps
// to an SM (2-warp blocks at D = 2048, see search_first_block_warps). Otherwise blocks of up to
// 8 warps, 2 per SM, 128 registers, 16 warps. Measured (10k queries at 1M x 1536, L = 384): wide with 3-warp blocks 259k QPS, wide
// with 7-warp blocks (21 warps) 234k, the other 244k; capping the registers with __maxnreg__
// instead, at 96 / 88 with 21 warps: 240k / 181k. On indexes the L2 mostly holds (100k x 1536,
// and the 120k x 1024 stream) the 128-register build is 20-30 % faster. So shape 0 is wide at
// D = 2048 only, shape 4 takes the other residency, and an unset shape is chosen by index size.
template <int D, int kTile>
struct Tile {
    static constexpr int CPL = Lay<D>::CPL;
    static constexpr int chunks = kTile == 1 ? 8 : (kTile == 2 ? 32 : 16);
    static constexpr int GG = chunks / CPL > 0 ? chunks / CPL : 1;                 // gate group
    static constexpr bool wide = D >= 1024 && ((D == 2048) != (kTile == 4));
    // traversal group: 4 code rows in the wide build at D = 2048 (1 % faster there than 2)
    static constexpr int GT = (CPL == 1 ? 8 : (wide ? 4 : 2)) * (kTile == 3 ? 2 : 1);
    static constexpr int threads = wide ? 224 : 256;
    static constexpr int min_blocks = wide ? 3 : 2;
};

struct WarpSmem {
    float *pd;
    uint32_t *pid;
    float *plb;
    uint32_t *fid;
    float *flb;
    float *fsip;
    uint8_t *fval;
    float4 *fpf;
    uint32_t *sid;
    uint32_t *sslot;
    float *sdist;
    float2 *shdr;
    uint32_t *frontier;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~static_cast<size_t>(15); }

__host__ __device__ inline size_t warp_smem_bytes(int l_cap) {
    size_t s = 0;
    s += align16(static_cast<size_t>(l_cap) * 4) * 3;
    s += align16(kMaxFresh * 4) * 3 + align16(kMaxFresh);
    s += align16(kMaxFresh * 16);
    s += align16(kMaxFresh * 4) * 3 + align16(kMaxFresh * 8);
    s += align16(kMaxBeam * 4);
    return s;
}

__device__ WarpSmem carve(unsigned char *base, int l_cap) {
    WarpSmem w;
    unsigned char *p = base;
    auto take = [&](size_t bytes) {
        unsigned char *r = p;
        p += align16(bytes);
        return r;
    };
    w.pd = reinterpret_cast<float *>(take(static_cast<size_t>(l_cap) * 4));
    w.pid = reinterpret_cast<uint32_t *>(take(static_cast<size_t>(l_cap) * 4));
    w.plb = reinterpret_cast<float *>(take(static_cast<size_t>(l_cap) * 4));
    w.fid = reinterpret_cast<uint32_t *>(take(kMaxFresh * 4));
    w.flb = reinterpret_cast<float *>(take(kMaxFresh * 4));
    w.fsip = reinterpret_cast<float *>(take(kMaxFresh * 4));
    w.fval = take(kMaxFresh);
    w.fpf = reinterpret_cast<float4 *>(take(kMaxFresh * 16));
    w.sid = reinterpret_cast<uint32_t *>(take(kMaxFresh * 4));
    w.sslot = reinterpret_cast<uint32_t *>(take(kMaxFresh * 4));
    w.sdist = reinterpret_cast<float *>(take(kMaxFresh * 4));
    w.shdr = reinterpret_cast<float2 *>(take(kMaxFresh * 8));
    w.frontier = reinterpret_cast<uint32_t *>(take(kMaxBeam * 4));
    return w;
}

__device__ __forceinline__ void prefetch_l1(const void *p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Prefetch `bytes` of `count` rows (row r at base + ids[r] * stride) with the warp's lanes,
// one 128-byte line per lane-step.
__device__ __forceinline__ void prefetch_rows_l1(const uint8_t *base, const uint32_t *ids, int count,
                                                 size_t stride, int bytes, int lane) {
    const int lines = (bytes + 127) >> 7;
    for (int t = lane; t < count * lines; t += 32) {
        const int r = t / lines, l = t - r * lines;
        prefetch_l1(base + static_cast<size_t>(ids[r]) * stride + (l << 7));
    }
}

__device__ __forceinline__ void prefetch_rows_l2(const uint8_t *base, const uint32_t *ids, int count,
                                                 size_t stride, int bytes, int lane) {
    const int lines = (bytes + 127) >> 7;
    for (int t = lane; t < count * lines; t += 32) {
        const int r = t / lines, l = t - r * lines;
        prefetch_l2(base + static_cast<size_t>(ids[r]) * stride + (l << 7));
    }
}

__device__ __forceinline__ bool cand_less(float da, uint32_t ia, float db, uint32_t ib) {
    return da < db || (da == db && ia < ib);
}

// Integer gate partial over one 32-dim chunk: sum of the query bytes whose MSB bit is set.
// xg[k] holds the query bytes of dims k, 8+k, 16+k, 24+k, so (w >> k) & 0x01010101 is the
// byte mask of exactly those four dims: one shift, one AND and one dp4a per four dims.
__device__ __forceinline__ int gate_chunk(uint32_t w, const int (&xg)[8], int acc) {
#pragma unroll
    for (int k = 0; k < 8; ++k) acc = __dp4a(static_cast<int>((w >> k) & 0x01010101u), xg[k], acc);
    return acc;
}

// Unsigned bytes of a times signed bytes of b, summed into c.
__device__ __forceinline__ int dp4a_us(uint32_t a, int b, int c) {
    int d;
    asm("dp4a.u32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// The gate partial over a lane's CPL >= 2 chunks of one row, without the shifts: w & (0x01010101
// << k) has byte values 2^k per set bit, so acc_k = 2^k (the sum of group k) exactly, and the row's
// sum is sum_k acc_k >> k (exact: acc_k is a multiple of 2^k), formed once per row.
template <int CPL>
__device__ __forceinline__ int gate_row(const uint32_t (&w)[CPL], const int (&xg)[CPL][8]) {
    int acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = 0;
#pragma unroll
    for (int j = 0; j < CPL; ++j)
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] = dp4a_us(w[j] & (0x01010101u << k), xg[j][k], acc[k]);
    int sum = acc[0];
#pragma unroll
    for (int k = 1; k < 8; ++k) sum += acc[k] >> k;
    return sum;
}

// Integer traversal partial over one 32-dim chunk: sum of (code & 7) * x, or of the whole 4-bit
// code times x (kFull: the B1Main distance, x = +-1). Both nibbles are masked in place: the low
// ones sum into lo, the high ones (byte values 16 * code) into hi, and the row's sum is
// lo + hi / 16 (exact: hi is a multiple of 16), formed once per row by the caller.
template <bool kFull = false>
__device__ __forceinline__ void trav_chunk(const uint4 c, const int (&xe)[4], const int (&xo)[4], int &lo, int &hi) {
    constexpr uint32_t kMask = kFull ? 0x0F0F0F0Fu : 0x07070707u;
    const uint32_t w[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        lo = dp4a_us(w[k] & kMask, xe[k], lo);
        hi = dp4a_us(w[k] & (kMask << 4), xo[k], hi);
    }
}

// Reduce-scatter of N per-lane partial sums across the warp (N = 32, 16, 8 or 4): on return
// lane l holds the warp total of value (l & (N - 1)).
template <int N>
__device__ __forceinline__ int reduce_scatter(int (&p)[N], int lane) {
    int v[N];
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = p[i];
#pragma unroll
    for (int half = N / 2; half >= 1; half >>= 1) {
        const bool up = (lane & half) != 0;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const int keep = up ? v[i + half] : v[i];
            const int send = up ? v[i] : v[i + half];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, half);
        }
    }
    int t = v[0];
#pragma unroll
    for (int o = N; o < 32; o <<= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// The 8 search-state features of the learned stop (warp-uniform): hops / L; spread of the top
// k relative to ||q - c||^2; hops since the top k last changed / L; hops since the first
// max(rerank, k) entries last changed / L; unexpanded fraction; position of the next expansion;
// its distance above the k-th; log ||q - c||^2.
__device__ void search_features(const WarpSmem &s, int pn, int lval, int k, int hops, float qn2,
                                int last_topk, int last_topr, int lane, float (&f)[kMlpIn]) {
    const float inv_q = 1.0f / (qn2 + 1e-6f);
    const float inv_l = 1.0f / static_cast<float>(lval);
    const int kk = k < pn ? k : pn;
    const float d0 = s.pd[0], dk = s.pd[kk - 1];
    int first = pn, count = 0;
    for (int base = 0; base < pn; base += 32) {
        const int e = base + lane;
        const unsigned int m = __ballot_sync(0xffffffffu, e < pn && !(s.pid[e] & kExpanded));
        if (m != 0u && first == pn) first = base + __ffs(m) - 1;
        count += __popc(m);
    }
    const float dnext = first < pn ? s.pd[first] : dk;
    f[0] = static_cast<float>(hops) * inv_l;
    f[1] = (dk - d0) * inv_q;
    f[2] = static_cast<float>(hops - last_topk) * inv_l;
    f[3] = static_cast<float>(hops - last_topr) * inv_l;
    f[4] = static_cast<float>(count) * inv_l;
    f[5] = static_cast<float>(first) * inv_l;
    f[6] = (dnext - dk) * inv_q;
    f[7] = log1pf(qn2);
}

template <int D>
struct QueryRegs {
    int xg[Lay<D>::CPL][8];
    int xe[Lay<D>::CPL][4];
    int xo[Lay<D>::CPL][4];
};

template <int D>
__device__ __forceinline__ void load_query(QueryRegs<D> &r, const int8_t *codes, int sub) {
    using L = Lay<D>;
#pragma unroll
    for (int j = 0; j < L::CPL; ++j) {
        const int c = sub + L::LPN * j;
        const int4 *src = reinterpret_cast<const int4 *>(codes + 32 * c);
        const int4 a = src[0], b = src[1];
        const int w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            // bytes (x[k], x[8+k], x[16+k], x[24+k]); x[4j+b] is byte b of w[j]
            const uint32_t sel = static_cast<uint32_t>((k & 3) | (((k & 3) + 4) << 4));
            const uint32_t lo = __byte_perm(w[k >> 2], w[2 + (k >> 2)], sel);
            const uint32_t hi = __byte_perm(w[4 + (k >> 2)], w[6 + (k >> 2)], sel);
            r.xg[j][k] = static_cast<int>(__byte_perm(lo, hi, 0x5410));
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r.xe[j][k] = static_cast<int>(__byte_perm(w[2 * k], w[2 * k + 1], 0x6420));
            r.xo[j][k] = static_cast<int>(__byte_perm(w[2 * k], w[2 * k + 1], 0x7531));
        }
    }
}

// ---- the per-query search ------------------------------------------------------------

// kMode 0: Int8 / Int4 query codes. kMode 1, the B1 codec (sign bits; an ablation in the
// reference): the gate counts sign mismatches against the MSB plane (finish_gate_b1) and every
// survivor takes the FP32 restore (mode 0, as the Rust loop assigns, ours_diskann.rs:1731-1748).
// kMode 2, B1Main: no gate; every fresh neighbour is scored by the 4-bit x 1-bit distance
// (query_distance_b1) from +-1 query bytes and inserted (ours_diskann.rs:1661-1682).
// kMode 3, Full: the FP32 rotated residual against the MSB plane (16 lanes over dimensions and
// the reduce tree, half a warp per neighbour) gates; survivors with a valid gate take the
// remaining bits with the gate's short ip (mode 1), the others the FP32 restore (mode 0).
template <int D, int kMode, int kTile>
__device__ void search_one(const SearchArgs &a, const WarpSmem &s, int q, int lane,
                           uint32_t *visited, const uint32_t *stop_smem) {
    using L = Lay<D>;
    using T = Tile<D, kTile>;
    const DevIndex &ix = a.ix;
    const int sub = lane % L::LPN;
    const int grp = lane / L::LPN;
    const float *rr = a.rr + static_cast<size_t>(q) * D;
    const float4 sc = a.scal[q];
    const float qn2 = sc.x, qn = sc.y, half_sum = sc.z, scale = sc.w;
    const long long csum = a.csum[q];

    int k = a.k_per_q ? a.k_per_q[q] : a.k_default;
    int lval = a.l_per_q ? a.l_per_q[q] : a.l_default;
    uint32_t *out_ids = a.ids_out + static_cast<size_t>(q) * a.k_stride;
    float *out_d = a.dists_out + static_cast<size_t>(q) * a.k_stride;
    // OursPaperSearchStats counters, distributed: counter c lives in lane c (two registers
    // per lane instead of eighteen)
    enum { VIS, DC, HOPS, CHK, WPR, NPR, SAVED, MSBC, REMC };
    unsigned long long stc = 0;
    auto bump = [&](unsigned int counters, unsigned long long v) {
        if ((counters >> lane) & 1u) stc += v;
    };
    if (k < 0) k = 0;
    if (k > a.k_stride) k = a.k_stride;
    if (lval < k) lval = k;
    if (lval > a.l_cap) {
        if (lane == 0) atomicOr(a.status, 4);
        lval = a.l_cap;
    }
    for (int i = lane; i < a.k_stride; i += 32) {
        out_ids[i] = 0xFFFFFFFFu;
        out_d[i] = f_inf();
    }
    if (k == 0 || ix.n_total == 0) {
        if (a.stats_out && lane == 0) a.stats_out[q] = qg_search_stats{};
        return;
    }

    QueryRegs<D> qr;
    constexpr bool kB1 = kMode == 1;
    if constexpr (kB1) {
        // the sign-bit word of each 32-dim chunk this lane gates
        const uint32_t *bw = reinterpret_cast<const uint32_t *>(a.codes + static_cast<size_t>(q) * D);
#pragma unroll
        for (int j = 0; j < L::CPL; ++j) qr.xg[j][0] = static_cast<int>(bw[sub + L::LPN * j]);
    } else if constexpr (kMode != 3) {
        load_query<D>(qr, a.codes + static_cast<size_t>(q) * D, sub);
    }
    const float b1_es = kB1 ? b1_error_scale(csum) : 0.0f;

    int pn = 0;  // pool size (warp-uniform)
    if (ix.n_base != 0) {
        if (lane == 0) visited[0] = 1u;
        const float4 h = ix.hdr[0];
        const float d0 = restore_distance_hw<D>(ix.codes, rr, h.x, h.y, half_sum, qn2, lane & 15);
        if (lane == 0) {
            s.pd[0] = d0;
            s.pid[0] = 0;
            s.plb[0] = kFltMax;
        }
        pn = 1;
        bump((1u << VIS) | (1u << DC) | (1u << REMC), 1);
    }
    __syncwarp();

    const int beam = a.beam_width < 1 ? 1 : (a.beam_width > kMaxBeam ? kMaxBeam : a.beam_width);
    int stall = 0;
    int hops_done = 0;
    int n_expanded = 0;
    int last_topk = 0, last_topr = 0;  // last hop that inserted into the top k / top max(rerank, k)
    int fu = 0;                        // every pool entry before fu is expanded
    float budget = 0.0f;               // learned hop budget (stop_kind 1; 0 = none yet)
    const int want_r_all = a.rerank > k ? a.rerank : k;
    bool failed = false;
    for (;;) {
        const float back_before = pn > 0 ? s.pd[pn - 1] : 0.0f;
        // frontier: first `beam` unexpanded pool entries, marked expanded; entries before fu are
        // all expanded (fu moves past each frontier and back to any insert before it)
        int nf = 0;
        for (int base = fu & ~31; base < pn && nf < beam; base += 32) {
            const int i = base + lane;
            const bool un = i < pn && !(s.pid[i] & kExpanded);
            unsigned int m = __ballot_sync(0xffffffffu, un);
            while (m && nf < beam) {
                const int b = __ffs(m) - 1;
                m &= m - 1;
                if (lane == b) {
                    s.frontier[nf] = s.pid[i] & kIdMask;
                    s.pid[i] |= kExpanded;
                }
                ++nf;
                fu = base + b + 1;
            }
        }
        __syncwarp();
        if (nf == 0) break;
        if (++hops_done > a.hop_cap) {
            if (lane == 0) atomicOr(a.status, 2);
            break;
        }
        if (a.expanded_out != nullptr) {
            uint32_t *ex = a.expanded_out + static_cast<size_t>(q) * a.expanded_cap;
            for (int fi = lane; fi < nf; fi += 32)
                if (n_expanded + fi < a.expanded_cap) ex[n_expanded + fi] = s.frontier[fi];
            n_expanded += nf;
        }

        for (int fi = 0; fi < nf; ++fi) {
            const uint32_t node = s.frontier[fi];
            // the degree and the whole adjacency row are loaded together (one round trip)
            const uint32_t *adj = ix.edges + static_cast<size_t>(node) * ix.edge_stride;
            uint32_t row[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t j = static_cast<uint32_t>(lane + 32 * h);
                row[h] = j < ix.edge_stride ? __ldg(adj + j) : 0xFFFFFFFFu;
            }
            const uint32_t deg = min(__ldg(ix.degrees + node), ix.edge_stride);
            // ---- fresh neighbours in adjacency order (VisitedScratch::try_mark) ----
            int F = 0;
            bool oob = false;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int j = lane + 32 * h;
                const bool valid = j < static_cast<int>(deg);
                const uint32_t nb = valid ? row[h] : 0u;
                const bool bad = valid && nb >= ix.n_total;
                const uint32_t key = (valid && !bad) ? nb : (0x80000000u | static_cast<uint32_t>(j));
                const unsigned int same = __match_any_sync(0xffffffffu, key);
                const bool leader = (__ffs(same) - 1) == lane;
                bool fresh = false;
                if (valid && !bad && leader) {
                    // distinct ids of this row may share a word: atomicOr serialises them
                    const uint32_t bit = 1u << (nb & 31u);
                    fresh = (atomicOr(visited + (nb >> 5), bit) & bit) == 0u;
                }
                if (__any_sync(0xffffffffu, bad)) oob = true;
                const unsigned int fm = __ballot_sync(0xffffffffu, fresh);
                if (fresh) s.fid[F + __popc(fm & ((1u << lane) - 1u))] = nb;
                F += __popc(fm);
                __syncwarp();
            }
            if (oob) {
                failed = true;
                break;
            }
            if (F == 0) continue;
            bump((1u << VIS) | (kMode == 2 ? 0u : (1u << MSBC)), static_cast<unsigned>(F));

            if constexpr (kMode == 2) {
                // B1Main: no gate; every fresh neighbour goes on, none can be pruned
                for (int f = lane; f < F; f += 32) s.fval[f] = 0;
                __syncwarp();
            } else if constexpr (kMode == 3) {
                // Full: FP32 gate, two neighbours per pass (one per half-warp)
                for (int f = lane; f < F; f += 32) s.fpf[f] = ix.pf[s.fid[f]];
                __syncwarp();
                for (int base = 0; base < F; base += 2) {
                    const int f = base + (lane >> 4);
                    const int ff = f < F ? f : base;
                    const float sel = full_gate_selected_hw<D>(ix.msb + static_cast<size_t>(s.fid[ff]) * (D / 8), rr,
                                                               lane & 15);
                    if ((lane & 15) == 0 && f < F) {
                        const GateOut go = finish_gate_full(sel - half_sum, s.fpf[f], qn, qn2, a.eps);
                        s.flb[f] = go.lower_bound;
                        s.fsip[f] = go.short_ip;
                        s.fval[f] = go.valid ? 1 : 0;
                    }
                }
                __syncwarp();
            } else {
                // ---- gate (paper-prune lower bound) for every fresh neighbour ----
                // all MSB rows and factor rows are requested at once, then consumed group by group
                prefetch_rows_l1(ix.msb, s.fid, F, D / 8, D / 8, lane);
                prefetch_rows_l1(reinterpret_cast<const uint8_t *>(ix.pf), s.fid, F, 16, 16, lane);
                for (int f = lane; f < F; f += 32) s.fpf[f] = ix.pf[s.fid[f]];
                if constexpr (L::LPN == 32) {
                    constexpr int G = T::GG;
                    for (int gb = 0; gb < F; gb += G) {
                        uint32_t w[G][L::CPL];
    #pragma unroll
                        for (int g = 0; g < G; ++g) {
                            const int f = gb + g < F ? gb + g : gb;
                            const uint32_t *row = reinterpret_cast<const uint32_t *>(
                                ix.msb + static_cast<size_t>(s.fid[f]) * (D / 8));
    #pragma unroll
                            for (int j = 0; j < L::CPL; ++j) w[g][j] = __ldg(row + lane + 32 * j);
                        }
                        int p[G];
    #pragma unroll
                        for (int g = 0; g < G; ++g) {
                            int acc = 0;
                            if constexpr (!kB1 && L::CPL >= 2) {
                                acc = gate_row<L::CPL>(w[g], qr.xg);
                            } else {
    #pragma unroll
                                for (int j = 0; j < L::CPL; ++j) {
                                    if constexpr (kB1)
                                        acc += __popc(w[g][j] ^ static_cast<uint32_t>(qr.xg[j][0]));
                                    else
                                        acc = gate_chunk(w[g][j], qr.xg[j], acc);
                                }
                            }
                            p[g] = acc;
                        }
                        const int tot = reduce_scatter<G>(p, lane);
                        const int f = gb + lane;
                        if (lane < G && f < F) {
                            const GateOut go = kB1 ? finish_gate_b1(tot, s.fpf[f], scale, b1_es, qn, qn2, a.eps, D)
                                                   : finish_gate(tot, s.fpf[f], scale, csum, qn, qn2, a.eps);
                            s.flb[f] = go.lower_bound;
                            s.fsip[f] = go.short_ip;
                            s.fval[f] = go.valid ? 1 : 0;
                        }
                    }
                } else {
                    constexpr int P = L::PG;
                    for (int fb = 0; fb < F; fb += P * L::NBP) {
                        uint32_t w[P];
    #pragma unroll
                        for (int pp = 0; pp < P; ++pp) {
                            int f = fb + pp * L::NBP + grp;
                            f = f < F ? f : fb;
                            const uint32_t *row = reinterpret_cast<const uint32_t *>(
                                ix.msb + static_cast<size_t>(s.fid[f]) * (D / 8));
                            w[pp] = __ldg(row + sub);
                        }
    #pragma unroll
                        for (int pp = 0; pp < P; ++pp) {
                            int acc = kB1 ? __popc(w[pp] ^ static_cast<uint32_t>(qr.xg[0][0])) : gate_chunk(w[pp], qr.xg[0], 0);
    #pragma unroll
                            for (int o = 1; o < L::LPN; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                            const int f = fb + pp * L::NBP + grp;
                            if (sub == 0 && f < F) {
                                const GateOut go = kB1 ? finish_gate_b1(acc, s.fpf[f], scale, b1_es, qn, qn2, a.eps, D)
                                                       : finish_gate(acc, s.fpf[f], scale, csum, qn, qn2, a.eps);
                                s.flb[f] = go.lower_bound;
                                s.fsip[f] = go.short_ip;
                                s.fval[f] = go.valid ? 1 : 0;
                            }
                        }
                    }
                }
                __syncwarp();
            }

            // ---- first check against the pool tail (ours_diskann.rs:1708-1725) ----
            int S = 0;
            {
                const bool full = pn >= lval;
                const float tail = full ? s.pd[lval - 1] : kFltMax;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int f = lane + 32 * h;
                    const bool in = f < F;
                    const bool prune = in && full && s.fval[f] && s.flb[f] > tail;
                    const bool keep = in && !prune;
                    const unsigned int pm = __ballot_sync(0xffffffffu, prune);
                    const unsigned int km = __ballot_sync(0xffffffffu, keep);
                    if (keep) {
                        const int at = S + __popc(km & ((1u << lane) - 1u));
                        s.sid[at] = s.fid[f];
                        s.sslot[at] = static_cast<uint32_t>(f);
                    }
                    bump((1u << CHK) | (1u << WPR) | (1u << SAVED), static_cast<unsigned>(__popc(pm)));
                    S += __popc(km);
                }
            }
            __syncwarp();
            if (S == 0) continue;

            // ---- traversal distances of the survivors ----
            prefetch_rows_l1(ix.codes, s.sid, S, D / 2, D / 2, lane);
            prefetch_rows_l1(reinterpret_cast<const uint8_t *>(ix.hdr), s.sid, S, 16, 16, lane);
            for (int i = lane; i < S; i += 32) {
                const float4 h = ix.hdr[s.sid[i]];
                s.shdr[i] = make_float2(h.x, h.y);
            }
            __syncwarp();  // the survivor passes below read headers other lanes loaded
            if constexpr (kMode == 3) {
                // Full: mode 1 (the gate's short ip reused) for valid gates, mode 0 otherwise; two
                // survivors per pass (one per half-warp)
                for (int base = 0; base < S; base += 2) {
                    const int i = base + (lane >> 4);
                    const int ii = i < S ? i : base;
                    const float2 h = s.shdr[ii];
                    const uint32_t slot = s.sslot[ii];
                    const float d = full_distance_hw<D>(ix.codes + static_cast<size_t>(s.sid[ii]) * (D / 2), rr, h.x,
                                                        h.y, half_sum, qn2, s.fval[slot] != 0, s.fsip[slot], lane & 15);
                    if ((lane & 15) == 0 && i < S) s.sdist[i] = d;
                }
                __syncwarp();
            } else if constexpr (kB1) {
                // B1: every survivor by the FP32 restore, two per pass (one per half-warp)
                for (int base = 0; base < S; base += 2) {
                    const int i = base + (lane >> 4);
                    const int ii = i < S ? i : base;
                    const float2 h = s.shdr[ii];
                    const float d = restore_distance_hw<D>(ix.codes + static_cast<size_t>(s.sid[ii]) * (D / 2), rr,
                                                           h.x, h.y, half_sum, qn2, lane & 15);
                    if ((lane & 15) == 0 && i < S) s.sdist[i] = d;
                }
                __syncwarp();
            } else {
                bool any_full = false;
                if constexpr (L::LPN == 32) {
                    constexpr int G = T::GT;
                    for (int gb = 0; gb < S; gb += G) {
                        uint4 c[G][L::CPL];
    #pragma unroll
                        for (int g = 0; g < G; ++g) {
                            const int i = gb + g < S ? gb + g : gb;
                            const uint4 *row = reinterpret_cast<const uint4 *>(
                                ix.codes + static_cast<size_t>(s.sid[i]) * (D / 2));
    #pragma unroll
                            for (int j = 0; j < L::CPL; ++j) c[g][j] = __ldg(row + lane + 32 * j);
                        }
                        int p[G];
    #pragma unroll
                        for (int g = 0; g < G; ++g) {
                            int lo = 0, hi = 0;
    #pragma unroll
                            for (int j = 0; j < L::CPL; ++j) trav_chunk<kMode == 2>(c[g][j], qr.xe[j], qr.xo[j], lo, hi);
                            p[g] = lo + (hi >> 4);
                        }
                        const int tot = reduce_scatter<G>(p, lane);
                        const int i = gb + lane;
                        if (lane < G && i < S) s.sdist[i] = __int_as_float(tot);  // finished below
                    }
                } else {
                    constexpr int P = L::PG;
                    for (int ib = 0; ib < S; ib += P * L::NBP) {
                        uint4 c[P];
    #pragma unroll
                        for (int pp = 0; pp < P; ++pp) {
                            int i = ib + pp * L::NBP + grp;
                            i = i < S ? i : ib;
                            const uint4 *row = reinterpret_cast<const uint4 *>(
                                ix.codes + static_cast<size_t>(s.sid[i]) * (D / 2));
                            c[pp] = __ldg(row + sub);
                        }
    #pragma unroll
                        for (int pp = 0; pp < P; ++pp) {
                            int lo = 0, hi = 0;
                            trav_chunk<kMode == 2>(c[pp], qr.xe[0], qr.xo[0], lo, hi);
                            int acc = lo + (hi >> 4);
    #pragma unroll
                            for (int o = 1; o < L::LPN; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                            const int i = ib + pp * L::NBP + grp;
                            if (sub == 0 && i < S) s.sdist[i] = __int_as_float(acc);  // finished below
                        }
                    }
                }
                __syncwarp();
                // finish every survivor at once, one lane each (finishQuantizedTraversalDistance)
                for (int i = lane; i < S; i += 32) {
                    const float2 h = s.shdr[i];
                    if constexpr (kMode == 2)
                        s.sdist[i] = finish_b1main(h.x, h.y, __float_as_int(s.sdist[i]), csum, qn2);
                    else
                        s.sdist[i] = finish_traversal(h.x, h.y, s.fsip[s.sslot[i]], __float_as_int(s.sdist[i]),
                                                      scale, csum, qn2);
                }
                __syncwarp();
                // survivors whose gate was invalid use the full FP32 restore (mode 0)
                if constexpr (kMode != 2) {
                    for (int i = lane; i < S; i += 32) any_full |= s.fval[s.sslot[i]] == 0;
                    any_full = __any_sync(0xffffffffu, any_full);
                }
                if (any_full) {
                    for (int i = 0; i < S; ++i) {
                        if (s.fval[s.sslot[i]]) continue;
                        const uint32_t id = s.sid[i];
                        const float2 h = s.shdr[i];
                        const float d = restore_distance_hw<D>(ix.codes + static_cast<size_t>(id) * (D / 2),
                                                               rr, h.x, h.y, half_sum, qn2, lane & 15);
                        if (lane == 0) s.sdist[i] = d;
                        __syncwarp();
                    }
                }
                __syncwarp();
            }
            // ---- re-check and sorted insert in adjacency order (ours_diskann.rs:1944-1979) ----
            for (int i = 0; i < S; ++i) {
                const uint32_t slot = s.sslot[i];
                const bool valid = s.fval[slot] != 0;
                const float lb = s.flb[slot];
                const float d = s.sdist[i];
                const uint32_t id = s.sid[i];
                const bool full = pn >= lval;
                if (full && valid) {
                    if (lb > s.pd[lval - 1]) {
                        bump((1u << CHK) | (1u << WPR) | (1u << SAVED), 1);
                        continue;
                    }
                    bump((1u << CHK) | (1u << NPR), 1);
                }
                bump((1u << REMC) | (1u << DC), 1);
                // insert_candidate_sorted (ours_diskann.rs:1100-1126)
                if (full && !cand_less(d, id, s.pd[lval - 1], s.pid[lval - 1] & kIdMask)) continue;
                // rank in the sorted pool: small pools by a scan that stops at the first
                // 32-entry chunk not entirely below the candidate; large pools by two ballots per
                // 1024 entries (the chunk, from the chunks' last entries; then the entry)
                int pos = 0;
                if (pn <= 256) {
                    for (int base = 0; base < pn; base += 32) {
                        const int e = base + lane;
                        const bool lt = e < pn && cand_less(s.pd[e], s.pid[e] & kIdMask, d, id);
                        const unsigned int m = __ballot_sync(0xffffffffu, lt);
                        pos += __popc(m);
                        if (m != 0xffffffffu) break;
                    }
                } else for (int sb = 0; sb < pn; sb += 1024) {
                    const int last = sb + 32 * lane + 31;
                    const int probe = last < pn ? last : pn - 1;
                    const bool clt = sb + 32 * lane < pn && cand_less(s.pd[probe], s.pid[probe] & kIdMask, d, id);
                    const unsigned int cm = __ballot_sync(0xffffffffu, clt);
                    const int chunk = __popc(cm);  // chunks entirely before the candidate
                    const int base = sb + 32 * chunk;
                    if (base >= pn) {  // after every entry of the pool
                        pos = pn;
                        break;
                    }
                    if (chunk < 32) {
                        const int e = base + lane;
                        const bool lt = e < pn && cand_less(s.pd[e], s.pid[e] & kIdMask, d, id);
                        pos = base + __popc(__ballot_sync(0xffffffffu, lt));
                        break;
                    }
                    pos = sb + 1024;
                }
                const int newn = pn + 1 < lval ? pn + 1 : lval;
                // shift (pos, newn) up by one, 32 entries per pass from the top: a pass reads
                // (top - 32, top - 1] and writes (top - 31, top]; the next pass writes entry top - 32
                // only after its own __syncwarp, which every lane reaches after this pass's reads
                for (int top = newn - 1; top > pos; top -= 32) {
                    const int e = top - lane;
                    float vd = 0.0f, vl = 0.0f;
                    uint32_t vi = 0;
                    const bool mv = e > pos;
                    if (mv) {
                        vd = s.pd[e - 1];
                        vi = s.pid[e - 1];
                        vl = s.plb[e - 1];
                    }
                    __syncwarp();
                    if (mv) {
                        s.pd[e] = vd;
                        s.pid[e] = vi;
                        s.plb[e] = vl;
                    }
                }
                __syncwarp();
                if (lane == 0) {
                    s.pd[pos] = d;
                    s.pid[pos] = id;
                    s.plb[pos] = valid ? lb : kFltMax;
                }
                if (pos < k) last_topk = hops_done;
                if (pos < want_r_all) last_topr = hops_done;
                if (pos < fu) fu = pos;
                pn = newn;
                __syncwarp();
            }
        }
        if (failed) break;
        bump(1u << HOPS, static_cast<unsigned>(nf));
        if (a.kth_stop && pn >= k) {
            const float kth = s.pd[k - 1];
            float mlb = kFltMax;
            for (int e = lane; e < pn; e += 32)
                if (!(s.pid[e] & kExpanded)) mlb = fminf(mlb, s.plb[e]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mlb = fminf(mlb, __shfl_xor_sync(0xffffffffu, mlb, o));
            if (kth <= mlb) break;
        }
        if (a.early_stop_hops != 0 && pn >= lval) {
            const float back_after = pn > 0 ? s.pd[pn - 1] : 0.0f;
            stall = back_after >= back_before ? stall + 1 : 0;
            if (stall >= a.early_stop_hops) break;
        }
        // ---- learned early termination / trace rows (off unless requested) ----
        if (a.stop_w != nullptr || a.trace_feat != nullptr) {
            if (hops_done % a.stop_every == 0) {
                float feat[kMlpIn];
                search_features(s, pn, lval, k, hops_done, qn2, last_topk, last_topr, lane, feat);
                if (a.trace_feat != nullptr) {
                    int row = a.trace_count[q];
                    if (row < a.trace_cap) {
                        // label: how many truth ids already sit in the first max(rerank, k) entries
                        const int want_r = a.rerank > k ? a.rerank : k;
                        const int lim = want_r < pn ? want_r : pn;
                        int found = 0;
                        for (int t = 0; t < a.trace_truth_k; ++t) {
                            const uint32_t tid = a.trace_truth[static_cast<size_t>(q) * a.trace_truth_k + t];
                            bool hit = false;
                            for (int base = 0; base < lim && !hit; base += 32) {
                                const int e = base + lane;
                                hit = __any_sync(0xffffffffu, e < lim && (s.pid[e] & kIdMask) == tid);
                            }
                            found += hit ? 1 : 0;
                        }
                        float mine = 0.0f;
#pragma unroll
                        for (int i = 0; i < kMlpIn; ++i) mine = lane == i ? feat[i] : mine;
                        if (lane < kMlpIn)
                            a.trace_feat[(static_cast<size_t>(q) * a.trace_cap + row) * kMlpIn + lane] = mine;
                        if (lane == 0) {
                            a.trace_label[static_cast<size_t>(q) * a.trace_cap + row] = static_cast<float>(found);
                            a.trace_count[q] = row + 1;
                        }
                        __syncwarp();
                    }
                }
                if (a.stop_w != nullptr && hops_done >= a.stop_min_hops && !(a.stop_once && budget > 0.0f)) {
                    float f[kMlpIn];
#pragma unroll
                    for (int i = 0; i < kMlpIn; ++i) f[i] = (feat[i] - a.stop_norm[i]) * a.stop_norm[kMlpIn + i];
                    const float z = mlp_forward_warp_smem(f, stop_smem, lane);
                    if (a.stop_kind == 0) {
                        if (z > a.stop_logit) break;
                    } else {
                        // the network's output is log(hops this query needs): the budget
                        budget = expf(fminf(z, 30.0f)) * a.stop_scale;
                    }
                }
            }
            if (budget > 0.0f && static_cast<float>(hops_done) >= budget) break;
        }
    }

    if (a.expanded_out != nullptr) {
        uint32_t *ex = a.expanded_out + static_cast<size_t>(q) * a.expanded_cap;
        for (int i = n_expanded + lane; i < a.expanded_cap; i += 32) ex[i] = 0xFFFFFFFFu;
    }
    if (failed) {
        if (lane == 0) atomicOr(a.status, 1);
        if (a.stats_out && lane == 0) a.stats_out[q] = qg_search_stats{};
        return;
    }

    // ---- rerank (ours_diskann.rs:1813-1902) ----
    // candidates: the first min(#base entries, max(rerank, k)) pool entries with id < n_base,
    // compacted in place (write index <= read index).
    const int want = a.rerank > k ? a.rerank : k;
    int m = 0;
    for (int base = 0; base < pn && m < want; base += 32) {
        const int e = base + lane;
        uint32_t id = 0;
        float d = 0.0f;
        bool in = false;
        if (e < pn) {
            id = s.pid[e] & kIdMask;
            d = s.pd[e];
            in = id < ix.n_base;
        }
        const unsigned int bm = __ballot_sync(0xffffffffu, in);
        const int at = m + __popc(bm & ((1u << lane) - 1u));
        __syncwarp();
        if (in && at < want) {
            s.pid[at] = id;
            s.pd[at] = d;
        }
        m += __popc(bm);
        __syncwarp();
    }
    if (m > want) m = want;
    if constexpr (kMode <= 1) prefetch_rows_l2(ix.codes, s.pid, m, D / 2, D / 2, lane);
    prefetch_rows_l2(reinterpret_cast<const uint8_t *>(ix.res_scales), s.pid, m, D / 8, D / 8, lane);
    prefetch_rows_l2(ix.res_codes, s.pid, m, D / 2, D / 2, lane);
    // Int8 / Int4: the rerank set is recomputed by the FP32 4-bit restore (mode 0), two records
    // per pass (one per half-warp). B1's pool already holds that distance (recomputing it changes
    // nothing); B1Main's and Full's residuals correct the distances in the pool (4-bit x 1-bit,
    // mode 1) (ours_diskann.rs:1849-1883).
    if constexpr (kMode <= 1) {
        // four records per pass: e and e + 2 on each half-warp
        for (int base = 0; base < m; base += 4) {
            const int e0 = base + (lane >> 4), e1 = e0 + 2;
            const uint32_t id0 = s.pid[e0 < m ? e0 : base], id1 = s.pid[e1 < m ? e1 : base];
            float d0, d1;
            restore_distance_hw2<D>(ix.codes + static_cast<size_t>(id0) * (D / 2),
                                    ix.codes + static_cast<size_t>(id1) * (D / 2), rr, ix.hdr[id0], ix.hdr[id1],
                                    half_sum, qn2, lane & 15, &d0, &d1);
            if ((lane & 15) == 0) {
                if (e0 < m) s.pd[e0] = d0;
                if (e1 < m) s.pd[e1] = d1;
            }
        }
        __syncwarp();
    }
    // residual correction: records e and e + 32 on each lane
    (void)qn;
    for (int e0 = lane; e0 < m; e0 += 64) {
        const int e1 = e0 + 32 < m ? e0 + 32 : e0;
        const uint32_t id0 = s.pid[e0], id1 = s.pid[e1];
        float est0, est1;
        residual_estimate_thread2<D>(ix.res_scales + static_cast<size_t>(id0) * (D / 16),
                                     ix.res_codes + static_cast<size_t>(id0) * (D / 2), s.pd[e0],
                                     ix.res_scales + static_cast<size_t>(id1) * (D / 16),
                                     ix.res_codes + static_cast<size_t>(id1) * (D / 2), s.pd[e1], rr,
                                     a.fused_rerank != 0, &est0, &est1);
        s.plb[e0] = est0;
        if (e1 != e0) s.plb[e1] = est1;
    }
    __syncwarp();
    // top-k by (estimate, id): rank of each candidate among all candidates
    for (int e = lane; e < m; e += 32) {
        const float me = s.plb[e];
        const uint32_t mi = s.pid[e];
        int rank = 0;
        for (int o = 0; o < m; ++o) {
            const float oe = s.plb[o];
            const uint32_t oi = s.pid[o];
            rank += (oe < me || (!(me < oe) && oi < mi)) ? 1 : 0;
        }
        if (rank < k) {
            out_ids[rank] = mi;
            out_d[rank] = me;
        }
    }
    if (a.stats_out && lane < 9) {
        static_assert(sizeof(qg_search_stats) == 9 * sizeof(unsigned long long), "stats layout");
        reinterpret_cast<unsigned long long *>(a.stats_out + q)[lane] = stc;
    }
}

template <int D, int kMode, int kTile>
__global__ void __launch_bounds__((Tile<D, kTile>::threads), (Tile<D, kTile>::min_blocks)) search_kernel(SearchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    // the stop network's weights (when a model is given) precede the per-warp regions
    const size_t wsm = a.stop_w != nullptr ? kMlpSmemBytes : 0;
    const uint32_t *stop_smem = reinterpret_cast<const uint32_t *>(smem);
    if (a.stop_w != nullptr) {
        mlp_stage_smem(a.stop_w, reinterpret_cast<uint32_t *>(smem), threadIdx.x, blockDim.x);
        __syncthreads();
    }
    const WarpSmem s = carve(smem + wsm + warp * warp_smem_bytes(a.l_cap), a.l_cap);
    const int slot = blockIdx.x * wpb + warp;
    const size_t words = visited_row_words(a.ix.n_total);
    uint32_t *visited = a.visited + static_cast<size_t>(slot) * words;
    const int nq = a.nq_dev != nullptr ? min(a.nq, *a.nq_dev) : a.nq;
    for (;;) {
        int q = 0;
        if (lane == 0) q = static_cast<int>(atomicAdd(a.counter, 1u));
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= nq) break;
        // a clear visited row for every query (n_total / 8 bytes, 16-byte stores)
        uint4 *row = reinterpret_cast<uint4 *>(visited);
        for (size_t i = lane; i < words / 4; i += 32) row[i] = make_uint4(0u, 0u, 0u, 0u);
        __syncwarp();
        search_one<D, kMode, kTile>(a, s, q, lane, visited, stop_smem);
        __syncwarp();
    }
}

}  // namespace

size_t search_smem_per_warp(int code_dim, int l_cap) {
    (void)code_dim;
    return warp_smem_bytes(l_cap);
}

int search_supported_dim(int code_dim) {
    return code_dim == 64 || code_dim == 128 || code_dim == 256 || code_dim == 512 ||
           code_dim == 1024 || code_dim == 2048;
}

template <int D, int kMode, int kTile = 0>
static cudaError_t launch_dc(const SearchArgs &a, int grid, int wpb, cudaStream_t stream) {
    const size_t smem = search_block_smem(a.l_cap, wpb, a.stop_w != nullptr);
    cudaError_t e = cudaFuncSetAttribute(search_kernel<D, kMode, kTile>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    search_kernel<D, kMode, kTile><<<grid, wpb * 32, smem, stream>>>(a);
    return cudaGetLastError();
}

template <int D>
static cudaError_t launch_d(const SearchArgs &a, int grid, int wpb, cudaStream_t stream) {
    switch (a.mode) {
        case 1: return launch_dc<D, 1>(a, grid, wpb, stream);
        case 2: return launch_dc<D, 2>(a, grid, wpb, stream);
        case 3: return launch_dc<D, 3>(a, grid, wpb, stream);
        default: break;
    }
    if constexpr (D >= 1024) {
        switch (a.tile) {
            case 1: return launch_dc<D, 0, 1>(a, grid, wpb, stream);
            case 2: return launch_dc<D, 0, 2>(a, grid, wpb, stream);
            case 3: return launch_dc<D, 0, 3>(a, grid, wpb, stream);
            case 4: return launch_dc<D, 0, 4>(a, grid, wpb, stream);
            default: break;
        }
    }
    return launch_dc<D, 0>(a, grid, wpb, stream);
}

int search_max_block_warps(int code_dim, int tile) {
    if (code_dim == 2048) return (tile == 4 ? Tile<2048, 4>::threads : Tile<2048, 0>::threads) / 32;
    if (code_dim == 1024) return (tile == 4 ? Tile<1024, 4>::threads : Tile<1024, 0>::threads) / 32;
    return Tile<512, 0>::threads / 32;
}

// Block width the automatic launch shape tries first: 2 warps for the 24-warp build at D = 2048.
// It ties with 3-warp blocks on warps per SM, and with a second launch queued behind this one a
// smaller block frees its slots sooner (1M x 1536, two 10k-query launches in flight: 273k QPS
// against 268k; one launch at a time the same; 1-warp blocks 251k). 0 (none) otherwise.
int search_first_block_warps(int code_dim, int tile) { return code_dim == 2048 && tile != 4 ? 2 : 0; }

size_t search_block_smem(int l_cap, int wpb, bool stop_model) {
    return warp_smem_bytes(l_cap) * static_cast<size_t>(wpb) + (stop_model ? kMlpSmemBytes : 0);
}

template <typename K>
static int blocks_per_sm_k(K kernel, int l_cap, int wpb, bool stop_model) {
    const size_t smem = search_block_smem(l_cap, wpb, stop_model);
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
        cudaSuccess)
        return 0;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, wpb * 32, smem) != cudaSuccess) return 0;
    return blocks;
}

// Every codec mode and tile shapes 0-3 share the launch bounds and shared memory of
// search_kernel<D, 0, 0>; shape 4 has its own launch bounds.
template <int D>
static int blocks_per_sm_d(int l_cap, int wpb, bool stop_model, int tile) {
    if constexpr (D >= 1024)
        if (tile == 4) return blocks_per_sm_k(search_kernel<D, 0, 4>, l_cap, wpb, stop_model);
    return blocks_per_sm_k(search_kernel<D, 0, 0>, l_cap, wpb, stop_model);
}

static int blocks_per_sm_uncached(int code_dim, int l_cap, int wpb, bool stop_model, int tile) {
    switch (code_dim) {
        case 64: return blocks_per_sm_d<64>(l_cap, wpb, stop_model, tile);
        case 128: return blocks_per_sm_d<128>(l_cap, wpb, stop_model, tile);
        case 256: return blocks_per_sm_d<256>(l_cap, wpb, stop_model, tile);
        case 512: return blocks_per_sm_d<512>(l_cap, wpb, stop_model, tile);
        case 1024: return blocks_per_sm_d<1024>(l_cap, wpb, stop_model, tile);
        case 2048: return blocks_per_sm_d<2048>(l_cap, wpb, stop_model, tile);
        default: return 0;
    }
}

// Occupancy queries cost host time on every call; their answers depend only on the device and
// the launch parameters, so they are kept.
int search_blocks_per_sm(int code_dim, int l_cap, int wpb, bool stop_model, int tile) {
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, int, bool, int>, int> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    const auto key = std::make_tuple(dev, code_dim, l_cap, wpb, stop_model, tile);
    {
        std::lock_guard<std::mutex> lock(mu);
        const auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    const int b = blocks_per_sm_uncached(code_dim, l_cap, wpb, stop_model, tile);
    std::lock_guard<std::mutex> lock(mu);
    cache[key] = b;
    return b;
}

cudaError_t launch_search(const SearchArgs &a, int grid, int wpb, cudaStream_t stream) {
    switch (a.ix.code_dim) {
        case 64: return launch_d<64>(a, grid, wpb, stream);
        case 128: return launch_d<128>(a, grid, wpb, stream);
        case 256: return launch_d<256>(a, grid, wpb, stream);
        case 512: return launch_d<512>(a, grid, wpb, stream);
        case 1024: return launch_d<1024>(a, grid, wpb, stream);
        case 2048: return launch_d<2048>(a, grid, wpb, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace qg
