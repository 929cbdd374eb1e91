// Dense factorisations of the diagonal blocks of a lower-triangular matrix,
// one CTA of 256 threads per block of at most kLeaf = 64 rows, entirely in
// shared memory.  They are the leaves of the rebuild's recursive inverse of
// the Cholesky factor and of the recursive Cholesky-with-inverse:
//   leaf_inverse_kernel:      G_cc = L_cc^-1 for every diagonal block c at
//                             once (FP64);
//   leaf_chol_inv_df_kernel:  L = chol(A) and G = L^-1 for one diagonal block,
//                             in DF64 pairs on the FP32 pipes (the DF64
//                             rebuild), pivots' 1/sqrt included.
// Library triangular kernels at these sizes (cuSOLVER trtri on 256 rows,
// cuBLAS DTRMM/DTRSM panels) run on a handful of CTAs for 65-106 us per call;
// one leaf here is one barrier per column and little more FP64 work than
// the flops themselves: the FP64 pipe of one SM retires about two FMAs per
// clock, so a warp instruction with idle lanes costs as much as a full one.
// Work is therefore laid out by rows: warp w takes rows i = w (mod 8) of the
// active part and its lanes the active columns of the row, and the pivot's
// reciprocal square root is taken once, by the thread that finished the pivot.
//
// Both are column sweeps.  Cholesky, step k (right-looking):
//   r = 1/sqrt(a_kk);  a_ij -= (a_ik r)(a_jk r)   for i >= j > k,
// leaving column k unscaled (L(i, k) = a_ik r), so that a step only writes
// columns right of the ones it reads and needs one barrier.  Inverse, step k:
// row k of X holds L(k, k) G(k, :) and, for rows i > k,
//   x_ij -= L(i, k) / L(k, k) * x_kj   for j <= k;
// at the end G(i, j) = x_ij / L(i, i).
#include "df64.cuh"
#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kLeaf = 64, kPitch = kLeaf + 1, kThreads = 256;
constexpr int kRowsPerThread = kLeaf * kLeaf / kThreads;  // 16
constexpr size_t kLeafSmem = (size_t)(2 * kLeaf * kPitch + 2 * kLeaf) * sizeof(double);

constexpr int kWarps = kThreads / 32;

// For whole-block loads and stores: thread t owns column j = t % 64 and rows
// r0 + 4 q (r0 = t / 64, q < 16).
__device__ __forceinline__ int own_col() { return threadIdx.x % kLeaf; }
__device__ __forceinline__ int own_row0() { return threadIdx.x / kLeaf; }
// first row >= lo owned by this warp in the row layout (rows = warp mod 8)
__device__ __forceinline__ int first_row(int lo) {
    const int w = threadIdx.x / 32;
    return lo + ((w - lo) % kWarps + kWarps) % kWarps;
}

// X <- L(k, k) L^-1 row by row (see above).  As holds L's columns unscaled by
// sc: L(i, k) / L(k, k) = As[i][k] * sc[k].  On return X holds G up to the row
// scale rd (G(i, j) = X[i][j] * rd[i]).
__device__ void sweep_inverse(const double *As, const double *sc, double *X, int nb) {
    const int j0 = own_col(), r0 = own_row0(), lane = threadIdx.x % 32;
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
        const int i = r0 + 4 * q;
        X[i * kPitch + j0] = (i == j0 && i < nb) ? 1.0 : 0.0;
    }
    for (int k = 0; k < nb - 1; ++k) {
        __syncthreads();
        const double s = sc[k];
        for (int i = first_row(k + 1); i < nb; i += kWarps) {
            const double mik = As[i * kPitch + k] * s;
            for (int j = lane; j <= k; j += 32) X[i * kPitch + j] = fma(-mik, X[k * kPitch + j], X[i * kPitch + j]);
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
// (global row of its first column, for the status word), A and G as DF64
// pairs.  A non-positive pivot sets *info to its 1-based global column (the
// first one found) and the factorisation carries on with a zero scale, so the
// launch always ends.
__global__ void __launch_bounds__(kThreads) leaf_chol_inv_df_kernel(float2 *A, float2 *G, int nb, int ld, int r,
                                                                    int *info) {
    extern __shared__ double smem[];
    float2 *As = reinterpret_cast<float2 *>(smem), *X = As + kLeaf * kPitch;
    float2 *rd = X + kLeaf * kPitch, *sc = rd + kLeaf;
    const int j = own_col(), r0 = own_row0(), lane = threadIdx.x % 32;
    const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
        const int i = r0 + 4 * q;
        As[i * kPitch + j] = (i < nb && j < nb && i >= j) ? A[(size_t)j * ld + i] : zero;
        X[i * kPitch + j] = (i == j && i < nb) ? make_float2(1.f, 0.f) : zero;
    }
    __syncthreads();
    // the pivot of column k is final once step k - 1 has updated it; its owner
    // (row k, lane 0) records r = 1 / sqrt(pivot) and r^2
    auto pivot = [&](int k) {
        const float2 d = As[k * kPitch + k];
        const bool ok = d.x > 0.f;
        const float2 rk = ok ? df_rsqrt(d) : zero;
        rd[k] = rk;
        sc[k] = df_mul(rk, rk);
        if (!ok) atomicCAS(info, 0, r + k + 1);
    };
    if (threadIdx.x == 0) pivot(0);
    for (int k = 0; k < nb - 1; ++k) {  // Cholesky: a_ij -= (a_ik r^2) a_jk
        __syncthreads();
        const float2 s = sc[k];
        for (int i = first_row(k + 1); i < nb; i += kWarps) {
            const float2 lik = df_mul(As[i * kPitch + k], s);
            for (int c = k + 1 + lane; c <= i; c += 32) {
                float2 a = As[i * kPitch + c];
                const float2 b = As[c * kPitch + k];
                df_fma(a.x, a.y, -lik.x, -lik.y, b.x, b.y);
                As[i * kPitch + c] = df_renorm(a.x, a.y);
            }
            if (i == k + 1 && lane == 0) pivot(i);
        }
    }
    for (int k = 0; k < nb - 1; ++k) {  // inverse: x_ij -= (a_ik r^2) x_kj, j <= k
        __syncthreads();
        const float2 s = sc[k];
        for (int i = first_row(k + 1); i < nb; i += kWarps) {
            const float2 mik = df_mul(As[i * kPitch + k], s);
            for (int c = lane; c <= k; c += 32) {
                float2 x = X[i * kPitch + c];
                const float2 b = X[k * kPitch + c];
                df_fma(x.x, x.y, -mik.x, -mik.y, b.x, b.y);
                X[i * kPitch + c] = df_renorm(x.x, x.y);
            }
        }
    }
    __syncthreads();
    // G(i, j) = x_ij / L(i, i) and L(i, j) = a_ij r_j on and below the diagonal
    if (j < nb) {
#pragma unroll
        for (int q = 0; q < kRowsPerThread; ++q) {
            const int i = r0 + 4 * q;
            if (i >= nb) continue;
            const bool low = i >= j;
            G[(size_t)j * ld + i] = low ? df_mul(X[i * kPitch + j], rd[i]) : zero;
            A[(size_t)j * ld + i] = low ? df_mul(As[i * kPitch + j], rd[j]) : zero;
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

cudaError_t leaf_chol_inv_df(float2 *A, float2 *G, int nb, int ld, int row0, int *info, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(leaf_chol_inv_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kLeafSmem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (nb <= 0 || nb > kLeaf) return cudaErrorInvalidValue;
    leaf_chol_inv_df_kernel<<<1, kThreads, kLeafSmem, st>>>(A, G, nb, ld, row0, info);
    return cudaGetLastError();
}

}  // namespace elhl
