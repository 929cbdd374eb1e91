// Split-precision GEMM on the 5th-generation tensor cores (tcgen05) for the
// Chebyshev GEMM regime:
//
//   Y (rows x n2, FP32, row-major) = sum_t A_t (rows x K) * B_t^T,   B_t: n2 x K
//
// A is the scaled Hamiltonian Hs split in three BF16 terms (Hs = A0 + A1 + A2,
// each the BF16 rounding of what the previous terms left), B the current
// Chebyshev block split the same way.  The six products A_i B_j with i + j <= 2
// reproduce FP32 products to about 2^-24 relative (the dropped terms are below
// 2^-27).  They accumulate in FP32 in tensor memory (TMEM).  A0 B0 rotates over
// 512/n2 - 1 accumulators MMA by MMA; the five smaller products (2^-8 and below)
// share the last one.  The FP32 accumulation chains stay short: the tensor
// cores' accumulation error over a long chain dominated an earlier single-
// accumulator version by 10x.  K is also split over `splits` CTAs per row tile,
// which keeps every SM busy; each CTA writes its partial tile, and the caller
// sums the partials in FP64.
//
// One CTA computes a 128-row tile of Y over all n2 columns for its K range:
//   warp 0  one elected thread issues the TMA loads (cp.async.bulk.tensor, 128B
//           swizzle) of the six K-chunks (64 BF16 = 128 B per row) of a stage,
//   warp 1  allocates TMEM and one elected thread issues tcgen05.mma
//           (kind::f16, BF16 x BF16 -> FP32, M = 128, N = n2, K = 16) and
//           tcgen05.commit to release a stage or signal the end,
//   warps 2-5 read the accumulator back with tcgen05.ld (32 lanes x 32 columns
//           per instruction) and store Y.
// Two stages of 6 tiles are double-buffered through mbarriers.  Every wait is
// bounded (globaltimer, 2 s): on a timeout the CTA records ELHL_ERR_TIMEOUT,
// stops issuing work, waits for what it issued and frees its TMEM.
#include <cuda.h>

#include <algorithm>

#include "elhl_internal.cuh"
#include "tc_ptx.cuh"

namespace elhl {
namespace {

constexpr int kBM = 128;        // rows per CTA (MMA M)
constexpr int kBK = 64;         // K per chunk: 64 BF16 = one 128-byte swizzle row
constexpr int kStages = 2;
constexpr int kThreads = 192;   // 6 warps
constexpr int kNumPairs = 6;    // (i, j) with i + j <= 2
constexpr unsigned long long kWaitNs = 2000000000ull;

using namespace tc;

// bounded wait (kWaitNs) for the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, unsigned long long t0) {
    return tc::mbar_wait(bar, parity, t0, kWaitNs);
}

struct UmmaParams {
    int rows, K, n2;       // Y is rows x n2; K multiple of 64 after zero fill by TMA
    int splits;            // CTAs along K per row tile (blockIdx.y)
    float *Y;              // [splits][rows][n2] partial tiles
    int *error;
};

// dynamic shared memory: [stage][3 A tiles (128 x 64)][3 B tiles (n2 x 64)], then barriers
__global__ void __launch_bounds__(kThreads, 1)
    umma_bf16x3_kernel(const __grid_constant__ CUtensorMap mA0, const __grid_constant__ CUtensorMap mA1,
                       const __grid_constant__ CUtensorMap mA2, const __grid_constant__ CUtensorMap mB0,
                       const __grid_constant__ CUtensorMap mB1, const __grid_constant__ CUtensorMap mB2,
                       UmmaParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte alignment for the 128B-swizzled tiles
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    const int n2 = p.n2;
    const size_t a_tile = (size_t)kBM * kBK * 2, b_tile = (size_t)n2 * kBK * 2;
    const size_t stage_bytes = 3 * a_tile + 3 * b_tile;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * stage_bytes);
    uint64_t *empty = full + kStages;
    uint64_t *done = empty + kStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * kBM;
    const int nk_all = (p.K + kBK - 1) / kBK;
    const int kc0 = (int)((long long)nk_all * blockIdx.y / p.splits);
    const int nk = (int)((long long)nk_all * (blockIdx.y + 1) / p.splits) - kc0;  // K chunks of this CTA
    float *Yp = p.Y + (size_t)blockIdx.y * p.rows * n2;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // TMEM: all 512 columns = 512 / n2 accumulators of n2 FP32 columns x 128 lanes;
    // A0 B0 rotates over the first nbig, the smaller products use the last
    const int nbig = 512 / n2 - 1;
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    const unsigned long long t0 = now_ns();

    if (warp == 0 && lane == 0) {
        // ---- TMA producer
        const CUtensorMap *ma[3] = {&mA0, &mA1, &mA2};
        const CUtensorMap *mb[3] = {&mB0, &mB1, &mB2};
        int issued = 0;
        for (int kc = 0; kc < nk; ++kc) {
            const int s = kc % kStages;
            if (kc >= kStages && !mbar_wait(&empty[s], ((kc / kStages) - 1) & 1, t0)) {
                atomicExch(abort_flag, 1);
                break;
            }
            if (*(volatile int *)abort_flag) break;
            unsigned char *st = smem + s * stage_bytes;
            mbar_expect_tx(&full[s], (unsigned)stage_bytes);
            for (int t = 0; t < 3; ++t) tma_load_2d(st + t * a_tile, ma[t], &full[s], (kc0 + kc) * kBK, row0);
            for (int t = 0; t < 3; ++t)
                tma_load_2d(st + 3 * a_tile + t * b_tile, mb[t], &full[s], (kc0 + kc) * kBK, 0);
            ++issued;
        }
        // loads still in flight land before the CTA ends: wait for every issued stage
        for (int kc = (issued > kStages ? issued - kStages : 0); kc < issued; ++kc)
            mbar_wait(&full[kc % kStages], (kc / kStages) & 1, now_ns());
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer
        const uint32_t idesc = idesc_bf16(kBM, n2);
        const int pa[kNumPairs] = {0, 0, 1, 0, 1, 2};
        const int pb[kNumPairs] = {0, 1, 0, 2, 1, 0};
        for (int kc = 0; kc < nk; ++kc) {
            const int s = kc % kStages;
            if (!mbar_wait(&full[s], (kc / kStages) & 1, t0)) {
                atomicExch(abort_flag, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            unsigned char *st = smem + s * stage_bytes;
            for (int q = 0; q < kNumPairs; ++q) {
                const uint64_t da = smem_desc_sw128(st + pa[q] * a_tile);
                const uint64_t db = smem_desc_sw128(st + 3 * a_tile + pb[q] * b_tile);
                for (int k = 0; k < kBK / 16; ++k) {  // K = 16 per MMA: +32 bytes along the swizzled row
                    uint32_t acc;
                    int accumulate;
                    if (q == 0) {  // A0 B0 rotates over the nbig leading accumulators
                        const int i = kc * (kBK / 16) + k;
                        acc = tmem + (uint32_t)((i % nbig) * n2);
                        accumulate = i >= nbig;
                    } else {       // the five smaller products share the last accumulator
                        acc = tmem + (uint32_t)(nbig * n2);
                        accumulate = !(kc == 0 && q == 1 && k == 0);
                    }
                    umma_bf16(acc, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), idesc, accumulate);
                }
            }
            umma_commit(&empty[s]);  // the stage is free once these MMAs have read it
        }
        umma_commit(done);
    } else if (warp >= 2) {
        // ---- epilogue: TMEM -> registers -> Y
        const bool ok = mbar_wait(done, 0, t0);
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (ok && !*(volatile int *)abort_flag) {
            const int quad = warp & 3;  // this warp may read TMEM lanes [32 quad, 32 quad + 32)
            const int row = row0 + quad * 32 + lane;
            const int nused = min(nbig, nk * (kBK / 16));  // leading accumulators written
            for (int c0 = 0; c0 < n2; c0 += 32) {
                uint32_t r[32];
                float sum[32];
                const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0;
                tmem_ld32(taddr + (uint32_t)(nbig * n2), r);  // the small products first
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int q = 0; q < 32; ++q) sum[q] = __uint_as_float(r[q]);
                for (int a = 0; a < nused; ++a) {
                    tmem_ld32(taddr + (uint32_t)(a * n2), r);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                    for (int q = 0; q < 32; ++q) sum[q] += __uint_as_float(r[q]);
                }
                if (row < p.rows && nk > 0) {
                    float4 *dst = reinterpret_cast<float4 *>(Yp + (size_t)row * n2 + c0);
#pragma unroll
                    for (int q = 0; q < 8; ++q) dst[q] = make_float4(sum[4 * q], sum[4 * q + 1], sum[4 * q + 2], sum[4 * q + 3]);
                } else if (row < p.rows) {
                    float4 *dst = reinterpret_cast<float4 *>(Yp + (size_t)row * n2 + c0);
#pragma unroll
                    for (int q = 0; q < 8; ++q) dst[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
        } else if (lane == 0) {
            atomicExch(abort_flag, 1);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (threadIdx.x == 0 && *(volatile int *)abort_flag) atomicExch(p.error, (int)ELHL_ERR_TIMEOUT);
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// 2D BF16 map: inner dimension K (contiguous), outer `rows` with stride ld
// elements; box kBK x box_rows, 128B swizzle, zero fill outside.
int make_map(CUtensorMap *m, const __nv_bfloat16 *base, int K, int rows, int ld, int box_rows) {
    EncodeTiled fn = encode_fn();
    if (!fn) return ELHL_ERR_UNSUPPORTED;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(base), dims, strides, box,
                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? ELHL_OK : ELHL_ERR_BAD_ARG;
}

// x = x0 + x1 + x2 in BF16 terms (each the rounding of the remainder)
__global__ void split3_kernel(const float *__restrict__ src, int rows, int cols, int lds, __nv_bfloat16 *d0,
                              __nv_bfloat16 *d1, __nv_bfloat16 *d2, int ldd, bool transpose) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (c >= cols || r >= rows) return;
    const float x = src[(size_t)r * lds + c];
    const __nv_bfloat16 a = __float2bfloat16_rn(x);
    const float ra = x - __bfloat162float(a);
    const __nv_bfloat16 b = __float2bfloat16_rn(ra);
    const __nv_bfloat16 e = __float2bfloat16_rn(ra - __bfloat162float(b));
    const size_t o = transpose ? (size_t)c * ldd + r : (size_t)r * ldd + c;
    d0[o] = a;
    d1[o] = b;
    d2[o] = e;
}

// transposing split: src rows x cols (lds) -> dst[c][r] (ldd), through a 32 x 32
// shared-memory tile so that both the reads (along c) and the writes (along r)
// are coalesced
__global__ void split3_t_kernel(const float *__restrict__ src, int rows, int cols, int lds, __nv_bfloat16 *d0,
                                __nv_bfloat16 *d1, __nv_bfloat16 *d2, int ldd) {
    __shared__ float tile[32][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        tile[i][threadIdx.x] = (r < rows && c < cols) ? src[(size_t)r * lds + c] : 0.f;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (c >= cols || r >= rows) continue;
        const float x = tile[threadIdx.x][i];
        const __nv_bfloat16 a = __float2bfloat16_rn(x);
        const float ra = x - __bfloat162float(a);
        const __nv_bfloat16 b = __float2bfloat16_rn(ra);
        const __nv_bfloat16 e = __float2bfloat16_rn(ra - __bfloat162float(b));
        const size_t o = (size_t)c * ldd + r;
        d0[o] = a;
        d1[o] = b;
        d2[o] = e;
    }
}

}  // namespace

size_t umma_smem_bytes(int n2) {
    return 1024 + kStages * (3 * (size_t)kBM * kBK * 2 + 3 * (size_t)n2 * kBK * 2) + 64;
}

int umma_supported_n2(int n2) { return n2 >= 32 && n2 <= 128 && (n2 & (n2 - 1)) == 0; }

int split3_bf16(const float *src, int rows, int cols, int lds, __nv_bfloat16 *const dst[3], int ldd, bool transpose,
                cudaStream_t st) {
    if (transpose) {
        dim3 grid((cols + 31) / 32, (rows + 31) / 32);
        split3_t_kernel<<<grid, dim3(32, 8), 0, st>>>(src, rows, cols, lds, dst[0], dst[1], dst[2], ldd);
        count_launch();
        return cudaGetLastError() == cudaSuccess ? ELHL_OK : ELHL_ERR_CUDA;
    }
    dim3 grid((cols + 255) / 256, rows);
    split3_kernel<<<grid, 256, 0, st>>>(src, rows, cols, lds, dst[0], dst[1], dst[2], ldd, false);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? ELHL_OK : ELHL_ERR_CUDA;
}

int umma_splits(int rows, int K) {
    // enough CTAs for two per SM, and at most 16 K-chunks (64 MMAs on the leading accumulator) per CTA
    const int tiles = (rows + kBM - 1) / kBM, nk = (K + kBK - 1) / kBK;
    int s = std::max((2 * 152 + tiles - 1) / tiles, (nk + 15) / 16);
    s = std::min(s, std::min(16, nk));
    return std::max(s, 1);
}

int umma_bf16x3_gemm(const __nv_bfloat16 *const A[3], int lda, const __nv_bfloat16 *const B[3], int ldb, int rows,
                     int K, int n2, int splits, float *Y, int *d_error, cudaStream_t st) {
    if (!umma_supported_n2(n2) || rows <= 0 || K <= 0 || (lda % 8) || (ldb % 8)) return ELHL_ERR_UNSUPPORTED;
    for (int t = 0; t < 3; ++t)
        if ((reinterpret_cast<uintptr_t>(A[t]) | reinterpret_cast<uintptr_t>(B[t])) & 15) return ELHL_ERR_BAD_ARG;
    CUtensorMap m[6];
    for (int t = 0; t < 3; ++t) {
        if (int rc = make_map(&m[t], A[t], K, rows, lda, kBM)) return rc;
        if (int rc = make_map(&m[3 + t], B[t], K, n2, ldb, n2)) return rc;
    }
    const size_t smem = umma_smem_bytes(n2);
    if (cudaFuncSetAttribute(umma_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return ELHL_ERR_CUDA;
    if (splits < 1) return ELHL_ERR_BAD_ARG;
    UmmaParams p{rows, K, n2, splits, Y, d_error};
    dim3 grid((rows + kBM - 1) / kBM, splits);
    umma_bf16x3_kernel<<<grid, kThreads, smem, st>>>(m[0], m[1], m[2], m[3], m[4], m[5], p);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? ELHL_OK : ELHL_ERR_CUDA;
}

}  // namespace elhl
