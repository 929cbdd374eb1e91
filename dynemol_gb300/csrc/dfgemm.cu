// FP64 matrix product evaluated in double-float arithmetic on the FP32 pipes:
//   C = alpha A op(B) + beta C   (column-major, FP64 in and out, op(B) = B or B^T).
// Each FP64 operand is split on load into a pair hi + lo of FP32 numbers (48-bit
// significand); products use the exact FMA product error and sums use TwoSum,
// 12 FP32 instructions per FMA, so the product is accurate to about 4e-15
// relative while the FP64 pipe (1/58 of the FP32 rate on this part) stays
// idle.  Used by the DF64 rebuild (the recursive Cholesky factor and its inverse).
//
// Triangular operands (flags in `tri`, local block coordinates): elements on the
// zero side of a triangular operand are treated as zero whatever is stored
// there, and k tiles that are zero for the whole output tile are skipped, so a
// triangular product costs half a square one.  With kTriLowerC only output
// tiles that reach the diagonal or below it are written (a symmetric update).
//
// Tiling: 64 x 64 output tile per CTA of 256 threads, 4 x 4 outputs per thread,
// K in steps of 16 staged in shared memory as (hi, lo) pairs.
#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16, kThreads = 256;

__device__ __forceinline__ float2 split_d(double x) {
    const float h = __double2float_rn(x);
    return make_float2(h, __double2float_rn(x - (double)h));
}

// (sh, sl) += (ah + al)(bh + bl), dropping al bl
__device__ __forceinline__ void fma_df(float &sh, float &sl, float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float t = __fadd_rn(sh, p);
    const float z = __fsub_rn(t, sh);
    const float y = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z));
    sl = __fadd_rn(sl, __fadd_rn(y, e));
    sh = t;
}

template <bool TB>
__global__ void __launch_bounds__(kThreads) dfgemm_kernel(int m, int n, int k, double alpha, const double *__restrict__ A,
                                                          int lda, const double *__restrict__ B, int ldb, double beta,
                                                          double *__restrict__ C, int ldc, int tri) {
    __shared__ float2 As[kBK][kBM + 1];
    __shared__ float2 Bs[kBK][kBN + 1];
    const int tid = threadIdx.x;
    const int i0 = blockIdx.x * kBM, j0 = blockIdx.y * kBN;
    if ((tri & kTriLowerC) && i0 + kBM <= j0) return;  // tile strictly above the diagonal
    // k range holding non-zero products for this tile
    int klo = 0, khi = k;
    if (tri & kTriA) khi = min(khi, i0 + kBM);   // A(i, l) = 0 for l > i
    if (tri & kTriB) klo = j0;                   // B(l, j) = 0 for l < j
    if (tri & kTriBt) khi = min(khi, j0 + kBN);  // B^T(l, j) = B(j, l) = 0 for l > j
    const int tr = tid % 16, tc = tid / 16;  // 4 x 4 outputs: rows i0 + tr + 16 q, columns j0 + tc + 16 p
    float sh[4][4], sl[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) sh[q][p] = sl[q][p] = 0.f;
    for (int k0 = klo; k0 < khi; k0 += kBK) {
        // A tile kBM x kBK: consecutive threads on consecutive rows (coalesced)
        for (int t = tid; t < kBM * kBK; t += kThreads) {
            const int ii = t % kBM, kk = t / kBM;
            const int gi = i0 + ii, gk = k0 + kk;
            const bool nz = gi < m && gk < k && !((tri & kTriA) && gk > gi);
            As[kk][ii] = nz ? split_d(A[(size_t)gk * lda + gi]) : make_float2(0.f, 0.f);
        }
        // op(B) tile kBK x kBN, consecutive threads along the contiguous index
        for (int t = tid; t < kBK * kBN; t += kThreads) {
            const int kk = TB ? t / kBN : t % kBK, jj = TB ? t % kBN : t / kBK;
            const int gk = k0 + kk, gj = j0 + jj;
            const bool nz = gk < k && gj < n && !((tri & kTriB) && gk < gj) && !((tri & kTriBt) && gk > gj);
            const double b = nz ? (TB ? B[(size_t)gk * ldb + gj] : B[(size_t)gj * ldb + gk]) : 0.0;
            Bs[kk][jj] = split_d(b);
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kBK; ++kk) {
            float2 a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) a[q] = As[kk][tr + 16 * q];
#pragma unroll
            for (int p = 0; p < 4; ++p) b[p] = Bs[kk][tc + 16 * p];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int p = 0; p < 4; ++p) fma_df(sh[q][p], sl[q][p], a[q], b[p]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int gi = i0 + tr + 16 * q, gj = j0 + tc + 16 * p;
            if (gi < m && gj < n) {
                double *c = C + (size_t)gj * ldc + gi;
                const double v = alpha * ((double)sh[q][p] + (double)sl[q][p]);
                *c = beta == 0.0 ? v : v + beta * *c;
            }
        }
}

}  // namespace

cudaError_t dfgemm(int m, int n, int k, double alpha, const double *A, int lda, const double *B, int ldb, double beta,
                   double *C, int ldc, cudaStream_t st, bool transB, int tri) {
    if (m <= 0 || n <= 0) return cudaSuccess;
    dim3 grid((m + kBM - 1) / kBM, (n + kBN - 1) / kBN);
    if (transB)
        dfgemm_kernel<true><<<grid, kThreads, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
    else
        dfgemm_kernel<false><<<grid, kThreads, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
    return cudaGetLastError();
}

}  // namespace elhl
