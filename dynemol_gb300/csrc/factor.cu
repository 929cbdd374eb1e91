// Dense factorisations of the diagonal blocks of a lower-triangular matrix, in
// FP64, one CTA of 256 threads per block of at most kLeaf = 64 rows, entirely
// in shared memory.  They are the leaves of the rebuild's recursive inverse of
// the Cholesky factor and of the recursive Cholesky-with-inverse:
//   leaf_inverse_kernel:   G_cc = L_cc^-1 for every diagonal block c at once;
//   leaf_chol_inv_kernel:  L = chol(A) and G = L^-1 for one diagonal block.
// Library triangular kernels at these sizes (cuSOLVER trtri on 256 rows,
// cuBLAS DTRMM/DTRSM panels) run on a handful of CTAs for 65-106 us per call;
// one leaf here is a few microseconds of FP64 work and one barrier per column.
//
// Both are column sweeps.  Cholesky, step k (right-looking):
//   r = 1/sqrt(a_kk);  a_ij -= (a_ik r)(a_jk r)   for i >= j > k,
// leaving column k unscaled (L(i, k) = a_ik r), so that a step only writes
// columns right of the ones it reads and needs one barrier.  Inverse, step k:
// row k of X holds L(k, k) G(k, :) and, for rows i > k,
//   x_ij -= L(i, k) / L(k, k) * x_kj   for j <= k;
// at the end G(i, j) = x_ij / L(i, i).
#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kLeaf = 64, kPitch = kLeaf + 1, kThreads = 256;
constexpr int kRowsPerThread = kLeaf * kLeaf / kThreads;  // 16
constexpr size_t kLeafSmem = (size_t)(2 * kLeaf * kPitch + 2 * kLeaf) * sizeof(double);

// Thread t owns column j = t % 64 and rows r0 + 4 q (r0 = t / 64, q < 16).
__device__ __forceinline__ int own_col() { return threadIdx.x % kLeaf; }
__device__ __forceinline__ int own_row0() { return threadIdx.x / kLeaf; }

// X <- L(k, k) L^-1 row by row (see above).  As holds L's columns unscaled by
// sc: L(i, k) / L(k, k) = As[i][k] * sc[k].  On return X holds G up to the row
// scale rd (G(i, j) = X[i][j] * rd[i]).
__device__ void sweep_inverse(const double *As, const double *sc, double *X, int nb) {
    const int j = own_col(), r0 = own_row0();
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
        const int i = r0 + 4 * q;
        X[i * kPitch + j] = (i == j && i < nb) ? 1.0 : 0.0;
    }
    for (int k = 0; k < nb - 1; ++k) {
        __syncthreads();
        if (j <= k) {
            const double xk = X[k * kPitch + j] * sc[k];
#pragma unroll
            for (int q = 0; q < kRowsPerThread; ++q) {
                const int i = r0 + 4 * q;
                if (i > k && i < nb) X[i * kPitch + j] = fma(-As[i * kPitch + k], xk, X[i * kPitch + j]);
            }
        }
    }
    __syncthreads();
}

// Load the lower triangle of the nb x nb block at src (leading dimension ld)
// into As (row-major, pitch kPitch); the rest of As is zero.
__device__ void load_lower(const double *__restrict__ src, int ld, int nb, double *As) {
    const int j = own_col(), r0 = own_row0();
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
        const int i = r0 + 4 * q;
        As[i * kPitch + j] = (i < nb && j < nb && i >= j) ? src[(size_t)j * ld + i] : 0.0;
    }
}

// dst(i, j) = X[i][j] * rd[i] * scale on and below the diagonal, 0 above
__device__ void store_lower(const double *X, const double *rd, double scale, int nb, double *__restrict__ dst, int ld) {
    const int j = own_col(), r0 = own_row0();
    if (j >= nb) return;
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
        const int i = r0 + 4 * q;
        if (i < nb) dst[(size_t)j * ld + i] = (i >= j) ? X[i * kPitch + j] * rd[i] * scale : 0.0;
    }
}

// G_cc = L_cc^-1 for the diagonal blocks c of the n x n lower-triangular L, in
// place (blockIdx.x = c; the last block may be short).
__global__ void __launch_bounds__(kThreads) leaf_inverse_kernel(double *A, int n, int ld) {
    extern __shared__ double smem[];
    double *As = smem, *X = smem + kLeaf * kPitch, *rd = X + kLeaf * kPitch, *sc = rd + kLeaf;
    const int r = blockIdx.x * kLeaf, nb = min(kLeaf, n - r);
    double *blk = A + (size_t)r * ld + r;
    load_lower(blk, ld, nb, As);
    __syncthreads();
    if (threadIdx.x < nb) {
        const double d = As[threadIdx.x * kPitch + threadIdx.x];
        rd[threadIdx.x] = 1.0 / d;
        sc[threadIdx.x] = 1.0 / d;
    }
    __syncthreads();
    sweep_inverse(As, sc, X, nb);
    store_lower(X, rd, 1.0, nb, blk, ld);
}

// L = chol(A) in place and G = L^-1 for the nb x nb diagonal block at offset r
// (global row of its first column, for the status word).  A non-positive
// pivot sets *info to its 1-based global column (the first one found) and the
// factorisation carries on with a zero scale, so the launch always ends.
__global__ void __launch_bounds__(kThreads) leaf_chol_inv_kernel(double *A, double *G, int nb, int ld, int r,
                                                                 int *info) {
    extern __shared__ double smem[];
    double *As = smem, *X = smem + kLeaf * kPitch, *rd = X + kLeaf * kPitch, *sc = rd + kLeaf;
    const int j = own_col(), r0 = own_row0();
    load_lower(A, ld, nb, As);
    for (int k = 0; k < nb; ++k) {
        __syncthreads();
        const double d = As[k * kPitch + k];
        const double rk = d > 0.0 ? rsqrt(d) : 0.0;
        if (threadIdx.x == 0) {
            rd[k] = rk;
            sc[k] = rk * rk;
            if (!(d > 0.0)) atomicCAS(info, 0, r + k + 1);
        }
        if (j > k && j < nb) {
            const double ajk = As[j * kPitch + k] * (rk * rk);
#pragma unroll
            for (int q = 0; q < kRowsPerThread; ++q) {
                const int i = r0 + 4 * q;
                if (i >= j && i < nb) As[i * kPitch + j] = fma(-As[i * kPitch + k], ajk, As[i * kPitch + j]);
            }
        }
    }
    __syncthreads();
    sweep_inverse(As, sc, X, nb);
    store_lower(X, rd, 1.0, nb, G, ld);
    // L(i, k) = As[i][k] * rd[k]: column scale
    if (j < nb) {
#pragma unroll
        for (int q = 0; q < kRowsPerThread; ++q) {
            const int i = r0 + 4 * q;
            if (i < nb) A[(size_t)j * ld + i] = (i >= j) ? As[i * kPitch + j] * rd[j] : 0.0;
        }
    }
}

}  // namespace

int leaf_rows() { return kLeaf; }

cudaError_t leaf_inverse(double *A, int n, int ld, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(leaf_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kLeafSmem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (n <= 0) return cudaSuccess;
    leaf_inverse_kernel<<<(n + kLeaf - 1) / kLeaf, kThreads, kLeafSmem, st>>>(A, n, ld);
    return cudaGetLastError();
}

cudaError_t leaf_chol_inv(double *A, double *G, int nb, int ld, int row0, int *info, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(leaf_chol_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kLeafSmem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (nb <= 0 || nb > kLeaf) return cudaErrorInvalidValue;
    leaf_chol_inv_kernel<<<1, kThreads, kLeafSmem, st>>>(A, G, nb, ld, row0, info);
    return cudaGetLastError();
}

}  // namespace elhl
