// rotate_gemm.cu -- the encode rotation as a dense GEMM on the tcgen05 tensor cores.
//
// The reference rotates the normalised residual u = (x - c) / |x - c| by random signs and an
// unnormalised fast Hadamard transform (RaBitQSpace::rotate / hadamard, space_rabitq.h:944-1000,
// signs +-1/sqrt(D) from std::mt19937, :2900-2912): v = H diag(s) pad(u). With the scale
// factored out of the signs, s_i = sgn_i * c (c = the float 1/sqrt(D) the reference stores),
// the rotation is the GEMM
//
//     V[n][j] = sum_i a[n][i] * R[j][i],   a[n][i] = fl(u_i * c),   R[j][i] = H[j][i] * sgn_i,
//
// whose second operand is exactly +-1 in BF16. The first is split exactly into three BF16
// terms (a = hi + mid + lo: 8 + 8 + 8 significand bits cover a float's 24), laid side by side
// along K, and R is repeated three times, so one BF16 x BF16 -> FP32 GEMM with K = 3 * Kp
// forms every product exactly and accumulates in FP32. Only the summation order differs from
// the butterflies; the code-mismatch rate against the reference encoder measures that.
//
// Kernels:
//   rotate_split_kernel  one warp per row: residual, norm (sequential, the reference order),
//                        a = fl(fl(r * (1/|r|)) * c), the three BF16 planes, |r| per row.
//   rotate_gemm_kernel   one 128 x 256 output tile per CTA: TMA (cp.async.bulk.tensor, 128-byte
//                        swizzle) stages 128 x 64 A and 256 x 64 B tiles into a 4-deep shared-
//                        memory ring (mbarrier transaction counts); one elected thread issues
//                        tcgen05.mma (kind::f16, M = 128, N = 256, K = 16 per instruction) into
//                        a 128 x 256 FP32 accumulator in tensor memory; four epilogue warps read
//                        it back with tcgen05.ld and write the FP32 rows. Every wait is bounded:
//                        on a timeout the CTA sets bit 0 of *status, drains what it issued,
//                        frees its tensor memory and returns.
//   r_matrix_kernel      R repeated three times along K (BF16, K-major), built once per space.
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda.h>  // CUtensorMap and its enums; the encoder itself is fetched through the runtime
#include <cuda_bf16.h>

#include "qg_kernels.h"

namespace qg {
namespace {

constexpr int kBM = 128, kBN = 256, kBK = 64, kStages = 4;
constexpr int kATile = kBM * kBK * 2;  // 16 KB
constexpr int kBTile = kBN * kBK * 2;  // 32 KB
constexpr int kStageBytes = kATile + kBTile;
constexpr int kSmemBytes = kStages * kStageBytes + 1024 + 256;
constexpr uint32_t kTmemCols = 256;
constexpr int kThreads = 192;  // warp 0: TMA producer; warp 1: TMEM owner + MMA issuer; 2-5: epilogue
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz: far beyond any legitimate wait

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Waits for the phase of `parity` to complete; false after kWaitCycles, or when this CTA's
// `abort` flag or the grid's status word (any CTA timed out) is set.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort,
                                          volatile int *grid_status) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done = 0;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort || *grid_status) return false;
        if (clock64() - t0 > kWaitCycles) return false;
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// Shared-memory matrix descriptor of a K-major tile in the 128-byte swizzle layout TMA writes:
// rows of 128 bytes, 8-row (1024-byte) swizzle atoms one after another (stride 1024 bytes).
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);  // start address
    d |= static_cast<uint64_t>(1) << 16;                  // leading byte offset (unused by swizzled K-major)
    d |= static_cast<uint64_t>(1024 >> 4) << 32;          // stride byte offset: next 8-row group
    d |= static_cast<uint64_t>(1) << 46;                  // descriptor version
    d |= static_cast<uint64_t>(2) << 61;                  // 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major, N = 256, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kBN >> 3) << 17) |
                            (static_cast<uint32_t>(kBM >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

// Arrives on `bar` once every tcgen05.mma this thread issued before has completed.
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_load_32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    rotate_gemm_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                       float *out, int n_rows, int n_cols, int ksteps, int *status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    unsigned char *sa = smem;
    unsigned char *sb = smem + kStages * kATile;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * kStageBytes);
    uint64_t *empty = full + kStages;
    uint64_t *accum = empty + kStages;
    uint64_t *drain = accum + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    volatile int *gstat = status;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(accum, 1);
        mbar_init(drain, 1);
        *abort_flag = *gstat ? 1 : 0;  // an earlier CTA timed out: the result is void, skip the work
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const bool skip = *abort_flag != 0;  // read after the barrier: the same in every thread

    if (skip) {
    } else if (warp == 0) {
        if (lane == 0) {
            int issued = 0;
            for (int k = 0; k < ksteps; ++k) {
                const int s = k % kStages;
                const uint32_t ph = static_cast<uint32_t>(k / kStages) & 1u;
                if (!mbar_wait(empty + s, ph ^ 1u, abort_flag, gstat)) {
                    *abort_flag = 1;
                    atomicOr(status, 1);
                    break;
                }
                mbar_expect_tx(full + s, kStageBytes);
                tma_load_2d(sa + s * kATile, &map_a, k * kBK, m0, full + s);
                tma_load_2d(sb + s * kBTile, &map_b, k * kBK, n0, full + s);
                ++issued;
            }
            if (*abort_flag || *gstat) {
                // on a timeout: the copies already issued land before the shared memory goes away
                // (stage s has seen issued_s loads; its last phase has parity (issued_s - 1) & 1)
                volatile int never = 0;
                for (int s = 0; s < kStages && s < issued; ++s) {
                    const int issued_s = (issued - s + kStages - 1) / kStages;
                    mbar_wait(full + s, static_cast<uint32_t>(issued_s - 1) & 1u, &never, &never);
                }
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            int issued = 0;
            for (int k = 0; k < ksteps; ++k) {
                const int s = k % kStages;
                const uint32_t ph = static_cast<uint32_t>(k / kStages) & 1u;
                if (!mbar_wait(full + s, ph, abort_flag, gstat)) {
                    *abort_flag = 1;
                    atomicOr(status, 1);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = smem_addr(sa + s * kATile), b0 = smem_addr(sb + s * kBTile);
#pragma unroll
                for (int kk = 0; kk < kBK / 16; ++kk)  // 16 BF16 = 32 bytes along K per instruction
                    umma_bf16(tmem, umma_desc(a0 + 32 * kk), umma_desc(b0 + 32 * kk), (k | kk) != 0 ? 1u : 0u);
                umma_commit(empty + s);
                ++issued;
            }
            umma_commit(accum);
            if (issued < ksteps) {
                // on a timeout: let the multiplies already issued finish before the memory goes away
                umma_commit(drain);
                volatile int never = 0;
                mbar_wait(drain, 0, &never, &never);
            }
        }
        __syncwarp();
    } else {
        // epilogue: warp w reads tensor-memory lanes 32 * (w % 4) .. + 31 (rows of the tile)
        const int lane_base = 32 * (warp & 3);
        volatile int never = 0;
        const bool ok = mbar_wait(accum, 0, &never, &never);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // tcgen05.ld is warp-collective: the warp decides as one
        if (__all_sync(0xffffffffu, ok && !*abort_flag)) {
            const int row = m0 + lane_base + lane;
            float *dst = out + static_cast<size_t>(row) * n_cols + n0;
            for (int c = 0; c < kBN; c += 32) {
                uint32_t r[32];
                tmem_load_32(tmem + (static_cast<uint32_t>(lane_base) << 16) + static_cast<uint32_t>(c), r);
                if (row < n_rows) {
                    float4 *d4 = reinterpret_cast<float4 *>(dst + c);
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        d4[q] = make_float4(__uint_as_float(r[4 * q]), __uint_as_float(r[4 * q + 1]),
                                            __uint_as_float(r[4 * q + 2]), __uint_as_float(r[4 * q + 3]));
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// One warp per row (the encoder's own steps, space_rabitq.h:5851-5865 and rotate's sign
// multiply): r = x - c, |r| by a sequential float sum of r * r (no contraction), u = r * (1 / |r|)
// (u = r when |r| = 0), a = fl(u * c); writes a's three BF16 terms at K offsets 0, kp, 2 kp
// (zero past dim) and |r|.
__global__ void __launch_bounds__(32) rotate_split_kernel(const float *raw, size_t stride, int n, int dim, int kp,
                                                          const float *center, float c_abs,
                                                          __nv_bfloat16 *a3, float *norms) {
    extern __shared__ float ru[];
    const int v = blockIdx.x, lane = threadIdx.x;
    if (v >= n) return;
    const float *x = raw + static_cast<size_t>(v) * stride;
    for (int i = lane; i < dim; i += 32) ru[i] = x[i] - center[i];
    __syncwarp();
    __shared__ float s_rn;
    if (lane == 0) {
        float rns = 0.0f;
        for (int i = 0; i < dim; ++i) rns = rns + ru[i] * ru[i];
        s_rn = sqrtf(rns);
    }
    __syncwarp();
    const float rn = s_rn;
    const float inv = rn > 0.0f ? 1.0f / rn : 1.0f;
    __nv_bfloat16 *row = a3 + static_cast<size_t>(v) * 3 * kp;
    for (int i = lane; i < kp; i += 32) {
        float a = 0.0f;
        if (i < dim) a = (rn > 0.0f ? ru[i] * inv : ru[i]) * c_abs;
        const __nv_bfloat16 hi = __float2bfloat16_rn(a);
        const float r1 = a - __bfloat162float(hi);
        const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
        const float r2 = r1 - __bfloat162float(mid);
        row[i] = hi;
        row[kp + i] = mid;
        row[2 * kp + i] = __float2bfloat16_rn(r2);
    }
    if (lane == 0) norms[v] = rn;
}

// R'[j][t * kp + i] = (-1)^popcount(i & j) * sgn_i for i < dim (0 past dim), t = 0, 1, 2.
__global__ void r_matrix_kernel(const float *signs, int dim, int kp, int D, __nv_bfloat16 *r3) {
    const size_t total = static_cast<size_t>(D) * 3 * kp;
    for (size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int j = static_cast<int>(t / (3 * kp));
        const int i = static_cast<int>(t % kp);
        float v = 0.0f;
        if (i < dim) v = ((__popc(static_cast<unsigned>(i & j)) & 1) ? -1.0f : 1.0f) * (signs[i] > 0.0f ? 1.0f : -1.0f);
        r3[t] = __float2bfloat16_rn(v);
    }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// A [rows x k] BF16 matrix, K contiguous, read in boxes of box_rows x 64 with the 128-byte swizzle.
bool make_map(CUtensorMap *map, const void *base, size_t rows, size_t k, uint32_t box_rows) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(k), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(k * 2)};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(kBK), box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int rotate_gemm_kp(int dim) { return (dim + kBK - 1) / kBK * kBK; }

bool rotate_gemm_supported(int code_dim) { return code_dim >= kBN && code_dim % kBN == 0; }

cudaError_t launch_rotate_split(const float *raw, size_t stride, int n, int dim, const float *center, float c_abs,
                                void *a3, float *norms, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    rotate_split_kernel<<<n, 32, static_cast<size_t>(dim) * 4, stream>>>(
        raw, stride, n, dim, rotate_gemm_kp(dim), center, c_abs, static_cast<__nv_bfloat16 *>(a3), norms);
    return cudaGetLastError();
}

cudaError_t launch_r_matrix(const float *signs, int dim, int code_dim, void *r3, cudaStream_t stream) {
    r_matrix_kernel<<<1024, 256, 0, stream>>>(signs, dim, rotate_gemm_kp(dim), code_dim,
                                              static_cast<__nv_bfloat16 *>(r3));
    return cudaGetLastError();
}

cudaError_t launch_rotate_gemm(const void *a3, const void *r3, int n, int dim, int code_dim, float *out, int *status,
                               cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    if (!rotate_gemm_supported(code_dim)) return cudaErrorInvalidValue;
    const size_t k = 3 * static_cast<size_t>(rotate_gemm_kp(dim));
    CUtensorMap ma, mb;
    if (!make_map(&ma, a3, static_cast<size_t>(n), k, kBM) || !make_map(&mb, r3, static_cast<size_t>(code_dim), k, kBN))
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(rotate_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    const dim3 grid(code_dim / kBN, (n + kBM - 1) / kBM);
    rotate_gemm_kernel<<<grid, kThreads, kSmemBytes, stream>>>(ma, mb, out, n, code_dim, static_cast<int>(k / kBK),
                                                              status);
    return cudaGetLastError();
}

}  // namespace qg
