// batch_kernels.cu -- kernels over (query, record) pairs in the reference's record layouts,
// behind the rabitq_* batch entry points and the qg_*_pairs parity entry points, plus the
// device re-layout of an uploaded index and the MSB sidecar extraction.
//
//   gate      rabitq_paper_estimate_batch_sidecar, Int8 branch (rabitq_bridge.cpp:747-778 ->
//             space_rabitq.h:4991-5093, 4701-4721), B1 (:4607-4695) and Full (:4427-4505); and
//             rabitq_paper_estimate(_batch), the gate from the encoded record (:3926-3959)
//   distance  rabitq_query_distance_batch modes 2, 1 / 3 and 0 (rabitq_bridge.cpp:885-970 ->
//             space_rabitq.h:4234-4358, 3961-3966, 4080-4202)
//   residual  rabitq_residual_distance_batch (rabitq_bridge.cpp:972-1017 ->
//             space_rabitq.h:5432-5548)
//   sidecar   extract_paper_prune_sidecar (space_rabitq.h:4364-4392)
//   symmetric distanceBetweenEncoded (space_rabitq.h:2634-2683)
#include <cstdint>

#include "qg_device.cuh"
#include "qg_kernels.h"

namespace qg {
namespace {

template <int D>
__global__ void gate_pairs_kernel(const int8_t *codes, const float4 *scal, const long long *csum,
                                  const uint32_t *qidx, const uint32_t *ids, size_t count,
                                  const uint8_t *msb, size_t msb_stride, const uint8_t *factors,
                                  size_t factor_stride, float eps, RabitqPaperEstimate *out) {
    const size_t pair = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pair >= count) return;
    const uint32_t q = qidx[pair], id = ids[pair];
    const int8_t *x = codes + static_cast<size_t>(q) * D;
    const uint8_t *m = msb + static_cast<size_t>(id) * msb_stride;
    int sel = 0;
    for (int i = lane; i < D; i += 32) sel += ((m[i >> 3] >> (i & 7)) & 1) ? x[i] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sel += __shfl_xor_sync(0xffffffffu, sel, o);
    if (lane == 0) {
        const float4 pf = load_factors(factors + static_cast<size_t>(id) * factor_stride);
        const float4 s = scal[q];
        const GateOut g = finish_gate(sel, pf, s.w, csum[q], s.y, s.x, eps);
        RabitqPaperEstimate r;
        r.lower_bound = g.lower_bound;
        r.short_ip = g.short_ip;
        r.alpha = 0.0f;
        r.ip_hat = g.ip_hat;
        r.error_bound = g.error_bound;
        r.valid = g.valid ? 1 : 0;
        out[pair] = r;
    }
}

// compute_b1_paper_prune_estimate_batch_by_id (space_rabitq.h:4607-4695): popcount of the
// query's sign bits against the MSB plane, then finish_b1_paper_prune_estimate.
template <int D>
__global__ void gate_b1_pairs_kernel(const int8_t *codes, const float4 *scal, const long long *csum,
                                     const uint32_t *qidx, const uint32_t *ids, size_t count,
                                     const uint8_t *msb, size_t msb_stride, const uint8_t *factors,
                                     size_t factor_stride, float eps, RabitqPaperEstimate *out) {
    const size_t pair = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pair >= count) return;
    const uint32_t q = qidx[pair], id = ids[pair];
    const uint8_t *qb = reinterpret_cast<const uint8_t *>(codes + static_cast<size_t>(q) * D);
    const uint8_t *m = msb + static_cast<size_t>(id) * msb_stride;
    int mism = 0;
    for (int j = lane; j < D / 8; j += 32) mism += __popc(static_cast<uint32_t>(qb[j] ^ m[j]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mism += __shfl_xor_sync(0xffffffffu, mism, o);
    if (lane == 0) {
        const float4 pf = load_factors(factors + static_cast<size_t>(id) * factor_stride);
        const float4 s = scal[q];
        const GateOut g = finish_gate_b1(mism, pf, s.w, b1_error_scale(csum[q]), s.y, s.x, eps, D);
        RabitqPaperEstimate r;
        r.lower_bound = g.lower_bound;
        r.short_ip = g.short_ip;
        r.alpha = g.reached ? b1_alpha(csum[q]) : 0.0f;
        r.ip_hat = g.ip_hat;
        r.error_bound = g.error_bound;
        r.valid = g.valid ? 1 : 0;
        out[pair] = r;
    }
}

// compute_full_paper_prune_estimate_batch_by_id (space_rabitq.h:4427-4505): the FP32 rotated
// residual against the MSB plane, 16 lanes over dimensions and the reduce tree (each half-warp
// computes the same sum), then the sidecar finish. One warp per pair.
template <int D>
__global__ void gate_full_pairs_kernel(const float *rr, const float4 *scal, const uint32_t *qidx,
                                       const uint32_t *ids, size_t count, const uint8_t *msb, size_t msb_stride,
                                       const uint8_t *factors, size_t factor_stride, float eps,
                                       RabitqPaperEstimate *out) {
    const size_t pair = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pair >= count) return;
    const uint32_t q = qidx[pair], id = ids[pair];
    const float sel = full_gate_selected_hw<D>(msb + static_cast<size_t>(id) * msb_stride,
                                               rr + static_cast<size_t>(q) * D, lane & 15);
    if (lane == 0) {
        const float4 pf = load_factors(factors + static_cast<size_t>(id) * factor_stride);
        const float4 s = scal[q];
        const GateOut g = finish_gate_full(sel - s.z, pf, s.y, s.x, eps);
        RabitqPaperEstimate r;
        r.lower_bound = g.lower_bound;
        r.short_ip = g.short_ip;
        r.alpha = 0.0f;
        r.ip_hat = g.ip_hat;
        r.error_bound = g.error_bound;
        r.valid = g.valid ? 1 : 0;
        out[pair] = r;
    }
}

// compute_paper_prune_estimate over (query, record) pairs (the gate from the encoded record),
// one warp per pair.
template <int D>
__global__ void gate_encoded_pairs_kernel(const float *rr, const float4 *scal, const uint32_t *qidx,
                                          const uint32_t *ids, size_t count, const uint8_t *records,
                                          size_t record_stride, float eps, RabitqPaperEstimate *out) {
    const size_t pair = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pair >= count) return;
    const uint32_t q = qidx[pair], id = ids[pair];
    const uint8_t *rec = records + static_cast<size_t>(id) * record_stride;
    const float4 s = scal[q];
    const float sip = encoded_short_ip_hw<D>(rec + 16, rr + static_cast<size_t>(q) * D, s.z, lane & 15);
    if (lane == 0) {
        float alpha;
        const GateOut g = finish_gate_encoded(sip, ld_f32(rec), ld_f32(rec + 8), s.y, s.x, eps, D, &alpha);
        RabitqPaperEstimate r;
        r.lower_bound = g.lower_bound;
        r.short_ip = g.short_ip;
        r.alpha = alpha;
        r.ip_hat = g.ip_hat;
        r.error_bound = g.error_bound;
        r.valid = g.valid ? 1 : 0;
        out[pair] = r;
    }
}

// query_distance_b1 over (query, record) pairs, one warp per pair; codes are the B1Main +-1
// bytes with the sign sum in csum, or (sign_bits) a B1 prepared query's sign bits.
template <int D>
__global__ void distance_b1_pairs_kernel(const int8_t *codes, const float4 *scal, const long long *csum,
                                         const uint32_t *qidx, const uint32_t *ids, size_t count,
                                         const uint8_t *records, size_t record_stride, bool sign_bits, float *out) {
    const size_t pair = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pair >= count) return;
    const uint32_t q = qidx[pair], id = ids[pair];
    const int8_t *x = codes + static_cast<size_t>(q) * D;
    const uint8_t *qb = reinterpret_cast<const uint8_t *>(x);
    const uint8_t *rec = records + static_cast<size_t>(id) * record_stride;
    int dot = 0;
    for (int p = lane; p < D / 2; p += 32) {
        const int b = rec[16 + p];
        int x0, x1;
        if (sign_bits) {  // B1: bit i of byte i / 8 set where q'_i > 0
            const int i0 = 2 * p, i1 = 2 * p + 1;
            x0 = ((qb[i0 >> 3] >> (i0 & 7)) & 1) ? 1 : -1;
            x1 = ((qb[i1 >> 3] >> (i1 & 7)) & 1) ? 1 : -1;
        } else {
            x0 = x[2 * p];
            x1 = x[2 * p + 1];
        }
        dot += (b & 15) * x0 + (b >> 4) * x1;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
    long long sign_sum = csum[q];
    if (sign_bits) {  // B1 keeps other scalars in the code-sum slot: count the positive signs
        int pos = 0;
        for (int j = lane; j < D / 8; j += 32) pos += __popc(static_cast<uint32_t>(qb[j]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) pos += __shfl_xor_sync(0xffffffffu, pos, o);
        sign_sum = 2LL * pos - D;
    }
    if (lane == 0) out[pair] = finish_b1main(ld_f32(rec), ld_f32(rec + 4), dot, sign_sum, scal[q].x);
}

template <int D>
__global__ void distance_pairs_kernel(const float *rr, const int8_t *codes, const float4 *scal,
                                      const long long *csum, const uint32_t *qidx,
                                      const uint32_t *ids, const uint8_t *modes, size_t count,
                                      const uint8_t *records, size_t record_stride,
                                      const float *short_ips, float *out) {
    const size_t pair = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pair >= count) return;
    const uint32_t q = qidx[pair], id = ids[pair];
    const uint8_t *rec = records + static_cast<size_t>(id) * record_stride;
    const uint8_t *code = rec + 16;
    const float norm_sqr = ld_f32(rec), long_scale = ld_f32(rec + 4);
    const float4 s = scal[q];
    if (modes[pair] == 2) {
        const int8_t *x = codes + static_cast<size_t>(q) * D;
        int dot = 0;
        for (int i = lane; i < D; i += 32) {
            const uint32_t byte = code[i >> 1];
            const int c = static_cast<int>(((i & 1) ? (byte >> 4) : byte) & 7u);
            dot += c * x[i];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        if (lane == 0)
            out[pair] = finish_traversal(norm_sqr, long_scale, short_ips[pair], dot, s.w, csum[q], s.x);
    } else if (modes[pair] == 1 || modes[pair] == 3) {
        // query_distance_with_paper_msb: the remaining bits with the given FP32 short ip
        const float d = full_distance_hw<D>(code, rr + static_cast<size_t>(q) * D, norm_sqr, long_scale, s.z,
                                            s.x, true, short_ips[pair], lane & 15);
        if (lane == 0) out[pair] = d;
    } else {
        const float d = restore_distance_hw<D>(code, rr + static_cast<size_t>(q) * D, norm_sqr,
                                                long_scale, s.z, s.x, lane & 15);
        if (lane == 0) out[pair] = d;
    }
}

template <int D>
__global__ void residual_pairs_kernel(const float *rr, const float4 *scal, const uint32_t *qidx,
                                      const uint32_t *ids, size_t count, const uint8_t *residual,
                                      size_t residual_stride, const float *long_d, bool fused,
                                      RabitqDistanceInterval *out) {
    const size_t pair = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (pair >= count) return;
    const uint32_t q = qidx[pair], id = ids[pair];
    const uint8_t *rec = residual + static_cast<size_t>(id) * residual_stride;
    const uint16_t *scales = reinterpret_cast<const uint16_t *>(rec + 8);
    const uint8_t *rc = rec + 8 + 2 * (D / 16);
    float est, lo, hi;
    residual_interval_thread<D>(scales, rc, rr + static_cast<size_t>(q) * D, long_d[pair],
                                scal[q].y, fused, &est, &lo, &hi);
    out[pair] = RabitqDistanceInterval{est, lo, hi};
}

// distanceBetweenEncoded, one centroid (space_rabitq.h:2634-2683): centred nibble dot
// times four, then the double-precision symmetric estimator. One warp per pair.
template <int D>
__global__ void symmetric_pairs_kernel(const uint8_t *lhs, const uint8_t *rhs, size_t count,
                                       size_t stride, float *out) {
    const size_t pair = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pair >= count) return;
    const uint8_t *a = lhs + pair * stride, *b = rhs + pair * stride;
    long long sum = 0;
    for (int p = lane; p < D / 2; p += 32) {
        const int ab = a[16 + p], bb = b[16 + p];
        sum += (2 * (ab & 15) - 15) * (2 * (bb & 15) - 15) + (2 * (ab >> 4) - 15) * (2 * (bb >> 4) - 15);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane != 0) return;
    const float ln2 = ld_f32(a), rn2 = ld_f32(b), lls = ld_f32(a + 4), rls = ld_f32(b + 4);
    const double ln = sqrt(fmax(0.0, static_cast<double>(ln2)));
    const double rn = sqrt(fmax(0.0, static_cast<double>(rn2)));
    if (!(ln > 0.0) || !(rn > 0.0) || !(lls > 0.0f) || !(rls > 0.0f) || !isfinite(lls) ||
        !isfinite(rls)) {
        out[pair] = static_cast<float>(static_cast<double>(ln2) + static_cast<double>(rn2));
        return;
    }
    const double code_ip = 0.25 * static_cast<double>(sum);
    const double lip = static_cast<double>(lls) / (2.0 * ln);
    const double rip = static_cast<double>(rls) / (2.0 * rn);
    double u = code_ip * lip * rip;
    if (!isfinite(u)) u = 0.0;
    u = fmax(-1.0, fmin(1.0, u));
    const double rip2 = ln * rn * u;
    out[pair] = static_cast<float>(static_cast<double>(ln2) + static_cast<double>(rn2) - 2.0 * rip2);
}

// extract_paper_prune_sidecar (space_rabitq.h:4364-4392), one warp per record.
__global__ void sidecar_kernel(const uint8_t *compact, size_t n, size_t stride, int D,
                               uint8_t *msb, RabitqPaperFactors *factors) {
    const size_t row = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const uint8_t *rec = compact + row * stride;
    const uint8_t *code = rec + 16;
    const int msb_bytes = D / 8;
    for (int j = lane; j < msb_bytes; j += 32) {
        uint32_t bits = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const uint32_t byte = code[4 * j + b];
            bits |= ((byte >> 3) & 1u) << (2 * b);
            bits |= ((byte >> 7) & 1u) << (2 * b + 1);
        }
        msb[row * msb_bytes + j] = static_cast<uint8_t>(bits);
    }
    if (lane == 0) {
        RabitqPaperFactors f{};
        f.norm_sqr = ld_f32(rec);
        const float short_scale = ld_f32(rec + 8);
        if (!(D <= 1 || f.norm_sqr <= 0.0f || short_scale <= 0.0f)) {
            const float data_norm = sqrtf(f.norm_sqr);
            f.data_norm = data_norm;
            const float alpha = fminf(1.0f, 4.0f * data_norm / (short_scale * sqrtf(static_cast<float>(D))));
            if (alpha > 0.0f && isfinite(alpha)) {
                const float alpha2 = alpha * alpha;
                f.cross_scale = short_scale;
                f.error_cross_scale = 2.0f * data_norm * sqrtf(fmaxf(0.0f, (1.0f - alpha2) / alpha2)) /
                                      sqrtf(static_cast<float>(D - 1));
                f.valid = isfinite(f.error_cross_scale) ? 1 : 0;
            }
        }
        factors[row] = f;
    }
}

// Reference host layouts -> device structure-of-arrays rows (16-byte aligned). One warp
// per node.
__global__ void repack_kernel(const uint8_t *compact, size_t compact_stride,
                              const uint8_t *residual, size_t residual_stride, const uint8_t *msb,
                              size_t msb_stride, const uint8_t *factors, size_t factor_stride,
                              const uint32_t *degrees, const uint32_t *edges, size_t edge_stride,
                              DevIndex ix) {
    const size_t row = (static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= ix.n_total) return;
    const int D = static_cast<int>(ix.code_dim);
    if (row < ix.n_base) {
        const uint8_t *c = compact + row * compact_stride;
        for (int j = lane; j < D / 2; j += 32) ix.codes[row * (D / 2) + j] = c[16 + j];
        const uint8_t *r = residual + row * residual_stride;
        for (int j = lane; j < D / 16; j += 32)
            ix.res_scales[row * (D / 16) + j] =
                static_cast<uint16_t>(r[8 + 2 * j] | (static_cast<uint16_t>(r[9 + 2 * j]) << 8));
        for (int j = lane; j < D / 2; j += 32) ix.res_codes[row * (D / 2) + j] = r[8 + D / 8 + j];
        const uint8_t *m = msb + row * msb_stride;
        for (int j = lane; j < D / 8; j += 32) ix.msb[row * (D / 8) + j] = m[j];
        if (lane == 0) {
            ix.hdr[row] = make_float4(ld_f32(c), ld_f32(c + 4), ld_f32(c + 8), ld_f32(c + 12));
            ix.pf[row] = load_factors(factors + row * factor_stride);
        }
    }
    const uint32_t deg = degrees[row];
    if (lane == 0) ix.degrees[row] = deg;
    for (uint32_t j = lane; j < ix.edge_stride; j += 32)
        ix.edges[row * ix.edge_stride + j] = j < deg ? edges[row * edge_stride + j] : 0xFFFFFFFFu;
}

template <template <int> class K>
struct Dispatch;

}  // namespace

#define QG_DISPATCH_D(D_, ...)                                   \
    switch (D_) {                                                \
        case 64: { constexpr int kD = 64; __VA_ARGS__; break; }   \
        case 128: { constexpr int kD = 128; __VA_ARGS__; break; } \
        case 256: { constexpr int kD = 256; __VA_ARGS__; break; } \
        case 512: { constexpr int kD = 512; __VA_ARGS__; break; } \
        case 1024: { constexpr int kD = 1024; __VA_ARGS__; break; } \
        case 2048: { constexpr int kD = 2048; __VA_ARGS__; break; } \
        default: return cudaErrorInvalidValue;                   \
    }

static unsigned int warp_grid(size_t count) {
    return static_cast<unsigned int>((count * 32 + 255) / 256);
}

cudaError_t launch_gate_pairs(int code_dim, const int8_t *codes, const float4 *scal,
                              const long long *csum, const uint32_t *qidx, const uint32_t *ids,
                              size_t count, const uint8_t *msb, size_t msb_stride,
                              const uint8_t *factors, size_t factor_stride, float eps,
                              RabitqPaperEstimate *out, cudaStream_t stream, bool b1) {
    if (count == 0) return cudaSuccess;
    if (b1) {
        QG_DISPATCH_D(code_dim, gate_b1_pairs_kernel<kD><<<warp_grid(count), 256, 0, stream>>>(
                                    codes, scal, csum, qidx, ids, count, msb, msb_stride, factors,
                                    factor_stride, eps, out));
    } else {
        QG_DISPATCH_D(code_dim, gate_pairs_kernel<kD><<<warp_grid(count), 256, 0, stream>>>(
                                    codes, scal, csum, qidx, ids, count, msb, msb_stride, factors,
                                    factor_stride, eps, out));
    }
    return cudaGetLastError();
}

cudaError_t launch_gate_full_pairs(int code_dim, const float *rr, const float4 *scal, const uint32_t *qidx,
                                   const uint32_t *ids, size_t count, const uint8_t *msb, size_t msb_stride,
                                   const uint8_t *factors, size_t factor_stride, float eps, RabitqPaperEstimate *out,
                                   cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    QG_DISPATCH_D(code_dim, gate_full_pairs_kernel<kD><<<warp_grid(count), 256, 0, stream>>>(
                                rr, scal, qidx, ids, count, msb, msb_stride, factors, factor_stride, eps, out));
    return cudaGetLastError();
}

cudaError_t launch_gate_encoded_pairs(int code_dim, const float *rr, const float4 *scal, const uint32_t *qidx,
                                      const uint32_t *ids, size_t count, const uint8_t *records, size_t record_stride,
                                      float eps, RabitqPaperEstimate *out, cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    QG_DISPATCH_D(code_dim, gate_encoded_pairs_kernel<kD><<<warp_grid(count), 256, 0, stream>>>(
                                rr, scal, qidx, ids, count, records, record_stride, eps, out));
    return cudaGetLastError();
}

cudaError_t launch_distance_b1_pairs(int code_dim, const int8_t *codes, const float4 *scal, const long long *csum,
                                     const uint32_t *qidx, const uint32_t *ids, size_t count, const uint8_t *records,
                                     size_t record_stride, float *out, cudaStream_t stream, bool sign_bits) {
    if (count == 0) return cudaSuccess;
    QG_DISPATCH_D(code_dim, distance_b1_pairs_kernel<kD><<<warp_grid(count), 256, 0, stream>>>(
                                codes, scal, csum, qidx, ids, count, records, record_stride, sign_bits, out));
    return cudaGetLastError();
}

cudaError_t launch_distance_pairs(int code_dim, const float *rr, const int8_t *codes,
                                  const float4 *scal, const long long *csum,
                                  const uint32_t *qidx, const uint32_t *ids,
                                  const uint8_t *modes, size_t count, const uint8_t *records,
                                  size_t record_stride, const float *short_ips, float *out,
                                  cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    QG_DISPATCH_D(code_dim, distance_pairs_kernel<kD><<<warp_grid(count), 256, 0, stream>>>(
                                rr, codes, scal, csum, qidx, ids, modes, count, records,
                                record_stride, short_ips, out));
    return cudaGetLastError();
}

cudaError_t launch_residual_pairs(int code_dim, const float *rr, const float4 *scal,
                                  const uint32_t *qidx, const uint32_t *ids, size_t count,
                                  const uint8_t *residual, size_t residual_stride,
                                  const float *long_d, bool fused, RabitqDistanceInterval *out,
                                  cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    const unsigned int grid = static_cast<unsigned int>((count + 127) / 128);
    QG_DISPATCH_D(code_dim, residual_pairs_kernel<kD><<<grid, 128, 0, stream>>>(
                                rr, scal, qidx, ids, count, residual, residual_stride, long_d, fused, out));
    return cudaGetLastError();
}

cudaError_t launch_symmetric_pairs(int code_dim, const uint8_t *lhs, const uint8_t *rhs,
                                   size_t count, size_t stride, float *out, cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    QG_DISPATCH_D(code_dim, symmetric_pairs_kernel<kD><<<warp_grid(count), 256, 0, stream>>>(
                                lhs, rhs, count, stride, out));
    return cudaGetLastError();
}

cudaError_t launch_sidecar(const uint8_t *compact, size_t n, size_t stride, int code_dim,
                           uint8_t *msb, RabitqPaperFactors *factors, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    sidecar_kernel<<<warp_grid(n), 256, 0, stream>>>(compact, n, stride, code_dim, msb, factors);
    return cudaGetLastError();
}

cudaError_t launch_repack(const uint8_t *compact, size_t compact_stride, const uint8_t *residual,
                          size_t residual_stride, const uint8_t *msb, size_t msb_stride,
                          const uint8_t *factors, size_t factor_stride, const uint32_t *degrees,
                          const uint32_t *edges, size_t edge_stride, DevIndex ix,
                          cudaStream_t stream) {
    if (ix.n_total == 0) return cudaSuccess;
    repack_kernel<<<warp_grid(ix.n_total), 256, 0, stream>>>(
        compact, compact_stride, residual, residual_stride, msb, msb_stride, factors,
        factor_stride, degrees, edges, edge_stride, ix);
    return cudaGetLastError();
}

}  // namespace qg
