// Dense factorisations of the diagonal blocks of a lower-triangular matrix,
// one CTA of 256 threads per block of at most kLeaf = 64 rows, entirely in
// shared memory.  They are the leaves of the rebuild's recursive inverse of
// the Cholesky factor and of the recursive Cholesky-with-inverse:
//   leaf_inverse_kernel:      G_cc = L_cc^-1 for every diagonal block c at
//                             once (FP64);
//   leaf_chol_inv_df_kernel:  L = chol(A) and G = L^-1 for one diagonal block,
//                             in DF64 pairs on the FP32 pipes (the DF64
//                             rebuild), pivots' 1/sqrt included, blocked by 8.
// Library triangular kernels at these sizes (cuSOLVER trtri on 256 rows,
// cuBLAS DTRMM/DTRSM panels) run on a handful of CTAs for 65-106 us per call.
//
// The FP64 leaf is a column sweep, one barrier per column.  Row k of X holds
// L(k, k) G(k, :) after step k and, for rows i > k,
//   x_ij -= L(i, k) / L(k, k) * x_kj   for j <= k;
// at the end G(i, j) = x_ij / L(i, i).  The FP64 pipe of one SM retires about
// two FMAs per clock, so a warp instruction with idle lanes costs as much as a
// full one: warp w takes rows i = w (mod 8) and its lanes the active columns.
// The DF64 leaf is blocked to need few barriers (see its comment).
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
// pairs, blocked so that few steps wait at a block-wide barrier:
//   Cholesky, for each 8-column block b (rows past nb padded with identity):
//     (1) warp 0 factors and inverts the 8 x 8 diagonal block (column sweeps
//         under __syncwarp only);
//     (2) panel L_rb = A_rb G_bb^T for the rows below;
//     (3) trailing update A_rr -= L_rb L_rb^T;
//   inverse by doubling, s = 8, 16, 32: G21 = -G22 (L21 G11) for all pairs.
// About 30 barriers instead of one per column.  A non-positive pivot sets
// *info to its 1-based global column (the first one found) and the
// factorisation carries on with a zero scale, so the launch always ends.
constexpr int kDiag = 8, kPPitch = kDiag + 1;
constexpr size_t kLeafDfSmem =
    (size_t)(2 * kLeaf * kPitch + kLeaf * kPPitch + 32 * kLeaf + 2 * kDiag) * sizeof(float2);

__global__ void __launch_bounds__(kThreads) leaf_chol_inv_df_kernel(float2 *A, float2 *G, int nb, int ld, int r,
                                                                    int *info) {
    extern __shared__ double smem[];
    float2 *As = reinterpret_cast<float2 *>(smem);  // [64][kPitch]: A, then L
    float2 *Gs = As + kLeaf * kPitch;               // [64][kPitch]: G
    float2 *P = Gs + kLeaf * kPitch;                // [64][kPPitch]: panel of the current block
    float2 *Wm = P + kLeaf * kPPitch;               // [32 * 64]: products of a doubling level
    float2 *rb = Wm + 32 * kLeaf, *sb = rb + kDiag;  // 1/L(k, k) and its square, current block
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    const float2 zero = make_float2(0.f, 0.f), one = make_float2(1.f, 0.f);
    for (int e = tid; e < kLeaf * kLeaf; e += kThreads) {
        const int i = e % kLeaf, j = e / kLeaf;
        float2 v = zero;
        if (i < nb && j < nb) {
            if (i >= j) v = A[(size_t)j * ld + i];
        } else if (i == j) {
            v = one;
        }
        As[i * kPitch + j] = v;
        Gs[i * kPitch + j] = zero;
    }
    __syncthreads();
    for (int b0 = 0; b0 < kLeaf; b0 += kDiag) {
        float2 *Ab = As + b0 * kPitch + b0, *Gb = Gs + b0 * kPitch + b0;
        if (warp == 0) {  // (1)
            for (int kk = 0; kk < kDiag; ++kk) {
                __syncwarp();
                const float2 d = Ab[kk * kPitch + kk];
                const bool ok = d.x > 0.f;
                const float2 rr = ok ? df_rsqrt(d) : zero, sq = df_mul(rr, rr);
                if (lane == 0) {
                    rb[kk] = rr;
                    sb[kk] = sq;
                    if (!ok && b0 + kk < nb) atomicCAS(info, 0, r + b0 + kk + 1);
                }
                for (int e = lane; e < kDiag * kDiag; e += 32) {
                    const int i = e / kDiag, j = e % kDiag;
                    if (j > kk && i >= j) {
                        float2 a = Ab[i * kPitch + j];
                        const float2 l = df_mul(Ab[i * kPitch + kk], sq), c = Ab[j * kPitch + kk];
                        df_fma(a.x, a.y, -l.x, -l.y, c.x, c.y);
                        Ab[i * kPitch + j] = df_renorm(a.x, a.y);
                    }
                }
            }
            for (int e = lane; e < kDiag * kDiag; e += 32) {
                const int i = e / kDiag, j = e % kDiag;
                Gb[i * kPitch + j] = i == j ? one : zero;
            }
            for (int kk = 0; kk < kDiag - 1; ++kk) {
                __syncwarp();
                for (int e = lane; e < kDiag * kDiag; e += 32) {
                    const int i = e / kDiag, j = e % kDiag;
                    if (i > kk && j <= kk) {
                        const float2 m = df_mul(Ab[i * kPitch + kk], sb[kk]), xk = Gb[kk * kPitch + j];
                        float2 x = Gb[i * kPitch + j];
                        df_fma(x.x, x.y, -m.x, -m.y, xk.x, xk.y);
                        Gb[i * kPitch + j] = df_renorm(x.x, x.y);
                    }
                }
            }
            __syncwarp();
            for (int e = lane; e < kDiag * kDiag; e += 32) {  // G = x_ij / L(i, i), L = a_ij / L(j, j)
                const int i = e / kDiag, j = e % kDiag;
                if (i >= j) {
                    Gb[i * kPitch + j] = df_mul(Gb[i * kPitch + j], rb[i]);
                    Ab[i * kPitch + j] = df_mul(Ab[i * kPitch + j], rb[j]);
                }
            }
        }
        __syncthreads();
        const int r0 = b0 + kDiag, nr = kLeaf - r0;
        for (int e = tid; e < nr * kDiag; e += kThreads) {  // (2) L(i, b0 + j) = sum_t A(i, b0 + t) G_bb(j, t)
            const int i = r0 + e / kDiag, j = e % kDiag;
            float h = 0.f, l = 0.f;
            for (int t = 0; t <= j; ++t) {
                const float2 a = As[i * kPitch + b0 + t], g = Gb[j * kPitch + t];
                df_fma(h, l, a.x, a.y, g.x, g.y);
            }
            P[i * kPPitch + j] = df_renorm(h, l);
        }
        __syncthreads();
        for (int e = tid; e < nr * kDiag; e += kThreads) {
            const int i = r0 + e / kDiag, j = e % kDiag;
            As[i * kPitch + b0 + j] = P[i * kPPitch + j];
        }
        for (int e = tid; e < kLeaf * kLeaf; e += kThreads) {  // (3), a warp on one row
            const int i = e / kLeaf, j = e % kLeaf;
            if (j < r0 || j > i) continue;
            float2 a = As[i * kPitch + j];
#pragma unroll
            for (int t = 0; t < kDiag; ++t) {
                const float2 p = P[i * kPPitch + t], q = P[j * kPPitch + t];
                df_fma(a.x, a.y, -p.x, -p.y, q.x, q.y);
            }
            As[i * kPitch + j] = df_renorm(a.x, a.y);
        }
        __syncthreads();
    }
    for (int s = kDiag; s < kLeaf; s *= 2) {  // inverse by doubling
        const int per = s * s, count = (kLeaf / (2 * s)) * per;
        for (int e = tid; e < count; e += kThreads) {  // W = L21 G11 (G11 lower: t >= j)
            const int o = 2 * s * (e / per), i = (e % per) / s, j = e % s;
            float h = 0.f, l = 0.f;
            for (int t = j; t < s; ++t) {
                const float2 a = As[(o + s + i) * kPitch + o + t], g = Gs[(o + t) * kPitch + o + j];
                df_fma(h, l, a.x, a.y, g.x, g.y);
            }
            Wm[e] = df_renorm(h, l);
        }
        __syncthreads();
        for (int e = tid; e < count; e += kThreads) {  // G21 = -G22 W (G22 lower: t <= i)
            const int o = 2 * s * (e / per), i = (e % per) / s, j = e % s;
            const float2 *W = Wm + (e / per) * per;
            float h = 0.f, l = 0.f;
            for (int t = 0; t <= i; ++t) {
                const float2 g = Gs[(o + s + i) * kPitch + o + s + t], w = W[t * s + j];
                df_fma(h, l, g.x, g.y, w.x, w.y);
            }
            const float2 v = df_renorm(h, l);
            Gs[(o + s + i) * kPitch + o + j] = make_float2(-v.x, -v.y);
        }
        __syncthreads();
    }
    for (int e = tid; e < kLeaf * kLeaf; e += kThreads) {
        const int i = e % kLeaf, j = e / kLeaf;
        if (i < nb && j < nb) {
            const bool low = i >= j;
            G[(size_t)j * ld + i] = low ? Gs[i * kPitch + j] : zero;
            A[(size_t)j * ld + i] = low ? As[i * kPitch + j] : zero;
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
    count_launch();
    return cudaGetLastError();
}

cudaError_t leaf_chol_inv_df(float2 *A, float2 *G, int nb, int ld, int row0, int *info, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(leaf_chol_inv_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kLeafDfSmem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (nb <= 0 || nb > kLeaf) return cudaErrorInvalidValue;
    leaf_chol_inv_df_kernel<<<1, kThreads, kLeafDfSmem, st>>>(A, G, nb, ld, row0, info);
    count_launch();
    return cudaGetLastError();
}

}  // namespace elhl
