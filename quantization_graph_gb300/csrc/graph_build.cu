// graph_build.cu -- GPU graph construction helpers (the reference builds its graph on the host,
// vamana_index.h / vamana_prune.h; this library's builder is its own and does not reproduce
// the reference graph bit for bit).
//
// prune_kernel: one warp per node. Candidate ids (any order, duplicates and padding allowed)
// are scored with the symmetric 4-bit estimator (distanceBetweenEncoded,
// space_rabitq.h:2634-2683, the distance the reference builder uses; here in FP32), sorted by
// (distance, id), de-duplicated, and reduced to at most R out-edges by alpha robust pruning
// with the occlusion-factor schedule alpha = 1.0 then alpha (the "alpha ramp" of
// robust_prune_4bit, vamana_prune.h:42-156): candidate j is occluded once a kept neighbour i
// has d(p, j) / d(i, j) > current alpha.
//
// The centred nibble dot sum_i (2a_i - 15)(2b_i - 15) is computed from unsigned nibble dots:
// 4 sum(ab) - 30 (sum a + sum b) + 225 D, exact in int32.
#include <cstdint>

#include "qg_device.cuh"
#include "qg_kernels.h"

namespace qg {
namespace {

constexpr int kMaxCand = 256;

__device__ __forceinline__ float ld_f32u(const uint8_t *p) {
    const uint32_t v = static_cast<uint32_t>(p[0]) | (static_cast<uint32_t>(p[1]) << 8) |
                       (static_cast<uint32_t>(p[2]) << 16) | (static_cast<uint32_t>(p[3]) << 24);
    return __uint_as_float(v);
}

// Per-record factors of the symmetric estimator: norm_sqr, ||r|| = sqrt(norm_sqr) and
// ip_norm = long_scale / (2 ||r||), computed once per record (FP32: this builder's graph is its
// own, and the FP64 pipe is narrow on this part).
struct CodeRef {
    float norm_sqr;
    float rn;
    float ipn;  // NaN when the record is degenerate (zero norm or bad long_scale)
};

__device__ __forceinline__ CodeRef code_ref(const uint8_t *rec) {
    const float ns = ld_f32u(rec), ls = ld_f32u(rec + 4);
    const float rn = sqrtf(fmaxf(0.0f, ns));
    const bool ok = rn > 0.0f && ls > 0.0f && isfinite(ls);
    return CodeRef{ns, rn, ok ? ls / (2.0f * rn) : __int_as_float(0x7fc00000)};
}

// symmetric estimator (distanceBetweenEncoded, space_rabitq.h:2634-2683) from the unsigned
// nibble dot: u = clamp(code_ip * ipn_a * ipn_b, +-1), d = n_a + n_b - 2 ||r_a|| ||r_b|| u
__device__ __forceinline__ float symmetric_from_dot(const CodeRef &a, const CodeRef &b, int dot_ab, int sum_a,
                                                    int sum_b, int D) {
    if (!(a.ipn == a.ipn) || !(b.ipn == b.ipn)) return a.norm_sqr + b.norm_sqr;
    const int centred = 4 * dot_ab - 30 * (sum_a + sum_b) + 225 * D;  // |centred| <= 225 D
    float u = (0.25f * static_cast<float>(centred)) * a.ipn * b.ipn;
    if (!isfinite(u)) u = 0.0f;
    u = fmaxf(-1.0f, fminf(1.0f, u));
    return a.norm_sqr + b.norm_sqr - 2.0f * (a.rn * b.rn * u);
}

template <int D>
__device__ __forceinline__ void load_code_words(const uint8_t *rec, uint32_t (&w)[D / 256 > 0 ? D / 256 : 1],
                                                int lane) {
    // D/2 code bytes = D/8 words; lane takes words lane, lane+32, ...
    constexpr int W = D / 8;
    constexpr int PER = (W + 31) / 32;
    const uint8_t *code = rec + 16;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int wi = lane + 32 * j;
        uint32_t v = 0;
        if (wi < W) {
            const uint8_t *b = code + 4 * wi;
            v = static_cast<uint32_t>(b[0]) | (static_cast<uint32_t>(b[1]) << 8) |
                (static_cast<uint32_t>(b[2]) << 16) | (static_cast<uint32_t>(b[3]) << 24);
        }
        w[j] = v;
    }
}

template <int D>
__device__ __forceinline__ int nibble_dot_words(const uint32_t (&a)[D / 256 > 0 ? D / 256 : 1],
                                                const uint32_t (&b)[D / 256 > 0 ? D / 256 : 1]) {
    constexpr int PER = ((D / 8) + 31) / 32;
    int acc = 0;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        acc = static_cast<int>(__dp4a(a[j] & 0x0F0F0F0Fu, b[j] & 0x0F0F0F0Fu, static_cast<unsigned>(acc)));
        acc = static_cast<int>(__dp4a((a[j] >> 4) & 0x0F0F0F0Fu, (b[j] >> 4) & 0x0F0F0F0Fu,
                                      static_cast<unsigned>(acc)));
    }
    return acc;
}

template <int D>
__device__ __forceinline__ int nibble_sum_words(const uint32_t (&a)[D / 256 > 0 ? D / 256 : 1]) {
    constexpr int PER = ((D / 8) + 31) / 32;
    int acc = 0;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        acc = static_cast<int>(__dp4a(a[j] & 0x0F0F0F0Fu, 0x01010101u, static_cast<unsigned>(acc)));
        acc = static_cast<int>(__dp4a((a[j] >> 4) & 0x0F0F0F0Fu, 0x01010101u, static_cast<unsigned>(acc)));
    }
    return acc;
}

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int D>
__global__ void __launch_bounds__(128) prune_kernel(const uint8_t *compact, size_t stride, int n,
                                                    const uint32_t *cand, int K, int R, float alpha,
                                                    uint32_t *degrees, uint32_t *edges, size_t edge_stride) {
    constexpr int PER = D / 256 > 0 ? D / 256 : 1;
    __shared__ float s_d[4][kMaxCand];
    __shared__ uint32_t s_id[4][kMaxCand];
    __shared__ float s_occ[4][kMaxCand];
    __shared__ unsigned char s_state[4][kMaxCand];  // 0 live, 1 kept, 2 dead
    __shared__ int s_nsum[4][kMaxCand];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p = blockIdx.x * 4 + warp;
    if (p >= n) return;
    float *dd = s_d[warp];
    uint32_t *ids = s_id[warp];
    float *occ = s_occ[warp];
    unsigned char *state = s_state[warp];
    int *nsum = s_nsum[warp];

    const uint8_t *prec = compact + static_cast<size_t>(p) * stride;
    uint32_t pw[PER];
    load_code_words<D>(prec, pw, lane);
    const CodeRef pref = code_ref(prec);
    const int psum = warp_sum(nibble_sum_words<D>(pw));

    int KP = 1;
    while (KP < K) KP <<= 1;
    for (int i = lane; i < KP; i += 32) {
        const uint32_t c = i < K ? cand[static_cast<size_t>(p) * K + i] : 0xFFFFFFFFu;
        ids[i] = (c < static_cast<uint32_t>(n) && c != static_cast<uint32_t>(p)) ? c : 0xFFFFFFFFu;
        dd[i] = kFltMax;
    }
    __syncwarp();
    for (int i = 0; i < K; ++i) {
        const uint32_t c = ids[i];
        if (c == 0xFFFFFFFFu) continue;
        const uint8_t *crec = compact + static_cast<size_t>(c) * stride;
        uint32_t cw[PER];
        load_code_words<D>(crec, cw, lane);
        const int dot = warp_sum(nibble_dot_words<D>(pw, cw));
        const int s = warp_sum(nibble_sum_words<D>(cw));
        if (lane == 0) {
            dd[i] = symmetric_from_dot(pref, code_ref(crec), dot, psum, s, D);
            nsum[i] = s;
        }
    }
    __syncwarp();
    // bitonic sort of (distance, id) pairs; padding sorts last
    for (int size = 2; size <= KP; size <<= 1) {
        for (int str = size >> 1; str > 0; str >>= 1) {
            for (int t = lane; t < KP / 2; t += 32) {
                const int lo = 2 * t - (t & (str - 1)), hi = lo + str;
                const bool asc = (lo & size) == 0;
                const bool gt = dd[lo] > dd[hi] || (dd[lo] == dd[hi] && ids[lo] > ids[hi]);
                if (gt == asc) {
                    const float tdv = dd[lo];
                    dd[lo] = dd[hi];
                    dd[hi] = tdv;
                    const uint32_t ti = ids[lo];
                    ids[lo] = ids[hi];
                    ids[hi] = ti;
                    const int ts = nsum[lo];
                    nsum[lo] = nsum[hi];
                    nsum[hi] = ts;
                }
            }
            __syncwarp();
        }
    }
    for (int i = lane; i < KP; i += 32) {
        occ[i] = 0.0f;
        const bool dup = i > 0 && ids[i] == ids[i - 1];
        state[i] = (ids[i] == 0xFFFFFFFFu || dup) ? 2 : 0;
    }
    __syncwarp();
    int kept = 0;
    uint32_t *out = edges + static_cast<size_t>(p) * edge_stride;
    const float alphas[2] = {1.0f, alpha};
    for (int pass = 0; pass < 2 && kept < R; ++pass) {
        const float cur = alphas[pass];
        for (int i = 0; i < KP && kept < R; ++i) {
            if (state[i] != 0 || occ[i] > cur) continue;
            if (lane == 0) {
                state[i] = 1;
                out[kept] = ids[i];
            }
            ++kept;
            __syncwarp();
            if (kept >= R) break;
            const uint8_t *irec = compact + static_cast<size_t>(ids[i]) * stride;
            uint32_t iw[PER];
            load_code_words<D>(irec, iw, lane);
            const CodeRef iref = code_ref(irec);
            for (int j = i + 1; j < KP; ++j) {
                if (state[j] != 0 || occ[j] > alpha) continue;
                const uint8_t *jrec = compact + static_cast<size_t>(ids[j]) * stride;
                uint32_t jw[PER];
                load_code_words<D>(jrec, jw, lane);
                const int dot = warp_sum(nibble_dot_words<D>(iw, jw));
                if (lane == 0) {
                    const float dij = symmetric_from_dot(iref, code_ref(jrec), dot, nsum[i], nsum[j], D);
                    const float ratio = dij > 0.0f ? dd[j] / dij : kFltMax;
                    occ[j] = fmaxf(occ[j], ratio);
                }
                __syncwarp();
            }
        }
    }
    if (lane == 0) degrees[p] = static_cast<uint32_t>(kept);
    for (int j = kept + lane; j < static_cast<int>(edge_stride); j += 32) out[j] = 0xFFFFFFFFu;
}

}  // namespace

cudaError_t launch_prune(int code_dim, const uint8_t *compact, size_t stride, int n, const uint32_t *cand,
                         int K, int R, float alpha, uint32_t *degrees, uint32_t *edges, size_t edge_stride,
                         cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    if (K <= 0 || K > kMaxCand || R <= 0 || static_cast<size_t>(R) > edge_stride) return cudaErrorInvalidValue;
    const unsigned grid = static_cast<unsigned>((n + 3) / 4);
    switch (code_dim) {
        case 64: prune_kernel<64><<<grid, 128, 0, stream>>>(compact, stride, n, cand, K, R, alpha, degrees, edges, edge_stride); break;
        case 128: prune_kernel<128><<<grid, 128, 0, stream>>>(compact, stride, n, cand, K, R, alpha, degrees, edges, edge_stride); break;
        case 256: prune_kernel<256><<<grid, 128, 0, stream>>>(compact, stride, n, cand, K, R, alpha, degrees, edges, edge_stride); break;
        case 512: prune_kernel<512><<<grid, 128, 0, stream>>>(compact, stride, n, cand, K, R, alpha, degrees, edges, edge_stride); break;
        case 1024: prune_kernel<1024><<<grid, 128, 0, stream>>>(compact, stride, n, cand, K, R, alpha, degrees, edges, edge_stride); break;
        case 2048: prune_kernel<2048><<<grid, 128, 0, stream>>>(compact, stride, n, cand, K, R, alpha, degrees, edges, edge_stride); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace qg
