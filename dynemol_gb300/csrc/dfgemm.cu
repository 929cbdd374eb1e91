// FP64 matrix product evaluated in double-float arithmetic on the FP32 pipes:
//   C = alpha A B + beta C   (column-major, FP64 in and out, no transposes).
// Each FP64 operand is split on load into a pair hi + lo of FP32 numbers (48-bit
// significand); products use the exact FMA product error and sums use TwoSum,
// 12 FP32 instructions per FMA, so the product is accurate to about 4e-15
// relative while the FP64 pipe (1/58 of the FP32 rate on this part) stays
// idle.  Used by the DF64 rebuild (the inverse of the Cholesky factor).
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

__global__ void __launch_bounds__(kThreads) dfgemm_kernel(int m, int n, int k, double alpha, const double *__restrict__ A,
                                                          int lda, const double *__restrict__ B, int ldb, double beta,
                                                          double *__restrict__ C, int ldc) {
    __shared__ float2 As[kBK][kBM + 1];
    __shared__ float2 Bs[kBK][kBN + 1];
    const int tid = threadIdx.x;
    const int i0 = blockIdx.x * kBM, j0 = blockIdx.y * kBN;
    const int tr = tid % 16, tc = tid / 16;  // 4 x 4 outputs: rows i0 + tr + 16 q, columns j0 + tc + 16 p
    float sh[4][4], sl[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) sh[q][p] = sl[q][p] = 0.f;
    for (int k0 = 0; k0 < k; k0 += kBK) {
        // A tile kBM x kBK: consecutive threads on consecutive rows (coalesced)
        for (int t = tid; t < kBM * kBK; t += kThreads) {
            const int ii = t % kBM, kk = t / kBM;
            const int gi = i0 + ii, gk = k0 + kk;
            As[kk][ii] = (gi < m && gk < k) ? split_d(A[(size_t)gk * lda + gi]) : make_float2(0.f, 0.f);
        }
        // B tile kBK x kBN: consecutive threads on consecutive k (coalesced)
        for (int t = tid; t < kBK * kBN; t += kThreads) {
            const int kk = t % kBK, jj = t / kBK;
            const int gk = k0 + kk, gj = j0 + jj;
            Bs[kk][jj] = (gk < k && gj < n) ? split_d(B[(size_t)gj * ldb + gk]) : make_float2(0.f, 0.f);
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
                   double *C, int ldc, cudaStream_t st) {
    if (m <= 0 || n <= 0) return cudaSuccess;
    dim3 grid((m + kBM - 1) / kBM, (n + kBN - 1) / kBN);
    dfgemm_kernel<<<grid, kThreads, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    return cudaGetLastError();
}

}  // namespace elhl
