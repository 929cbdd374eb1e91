// Dense Cholesky-with-inverse of one diagonal block of at most kLeaf = 64
// rows in FP64, one CTA of 256 threads, entirely in shared memory: the leaves
// of the rebuild's recursive factorisation (S = L L^T with G = L^-1) for every
// precision, and of the drop-in's H' = S^-1 h.  Blocked by 8 columns so that
// few steps wait at a block-wide barrier; library triangular kernels at these
// sizes (cuSOLVER trtri on 256 rows, cuBLAS DTRMM/DTRSM panels) ran on a
// handful of CTAs for 65-106 us per call.
#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kLeaf = 64, kPitch = kLeaf + 1, kThreads = 256;
constexpr int kDiag = 8, kPPitch = kDiag + 1;

// L = chol(A) in place and G = L^-1 for the nb x nb diagonal block at offset r
// (global row of its first column, for the status word), pivots' 1/sqrt by
// rsqrt, blocked so that few steps wait at a block-wide barrier:
//   Cholesky, for each 8-column block b (rows past nb padded with identity):
//     (1) warp 0 factors and inverts the 8 x 8 diagonal block (column sweeps
//         under __syncwarp only);
//     (2) panel L_rb = A_rb G_bb^T for the rows below;
//     (3) trailing update A_rr -= L_rb L_rb^T;
//   inverse by doubling, s = 8, 16, 32: G21 = -G22 (L21 G11) for all pairs.
// About 30 barriers instead of one per column.  A non-positive pivot sets
// *info to its 1-based global column (the first one found) and the
// factorisation carries on with a zero scale, so the launch always ends.
constexpr size_t kLeaf64Smem = (size_t)(2 * kLeaf * kPitch + kLeaf * kPPitch + 32 * kLeaf + 2 * kDiag) * sizeof(double);

__global__ void __launch_bounds__(kThreads) leaf_chol_inv64_kernel(double *A, double *G, int nb, int ld, int r,
                                                                   int *info) {
    extern __shared__ double smem[];
    double *As = smem;                 // [64][kPitch]: A, then L
    double *Gs = As + kLeaf * kPitch;  // [64][kPitch]: G
    double *P = Gs + kLeaf * kPitch;   // [64][kPPitch]: panel of the current block
    double *Wm = P + kLeaf * kPPitch;  // [32 * 64]: products of a doubling level
    double *rb = Wm + 32 * kLeaf, *sb = rb + kDiag;  // 1/L(k, k) and its square, current block
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    for (int e = tid; e < kLeaf * kLeaf; e += kThreads) {
        const int i = e % kLeaf, j = e / kLeaf;
        double v = 0.0;
        if (i < nb && j < nb) {
            if (i >= j) v = A[(size_t)j * ld + i];
        } else if (i == j) {
            v = 1.0;
        }
        As[i * kPitch + j] = v;
        Gs[i * kPitch + j] = 0.0;
    }
    __syncthreads();
    for (int b0 = 0; b0 < kLeaf; b0 += kDiag) {
        double *Ab = As + b0 * kPitch + b0, *Gb = Gs + b0 * kPitch + b0;
        if (warp == 0) {  // (1) factor and invert the 8 x 8 diagonal block
            for (int kk = 0; kk < kDiag; ++kk) {
                __syncwarp();
                const double d = Ab[kk * kPitch + kk];
                const bool ok = d > 0.0;
                const double rr = ok ? rsqrt(d) : 0.0, sq = rr * rr;
                if (lane == 0) {
                    rb[kk] = rr;
                    sb[kk] = sq;
                    if (!ok && b0 + kk < nb) atomicCAS(info, 0, r + b0 + kk + 1);
                }
                for (int e = lane; e < kDiag * kDiag; e += 32) {
                    const int i = e / kDiag, j = e % kDiag;
                    if (j > kk && i >= j)
                        Ab[i * kPitch + j] = fma(-Ab[i * kPitch + kk] * sq, Ab[j * kPitch + kk], Ab[i * kPitch + j]);
                }
            }
            for (int e = lane; e < kDiag * kDiag; e += 32) {
                const int i = e / kDiag, j = e % kDiag;
                Gb[i * kPitch + j] = i == j ? 1.0 : 0.0;
            }
            for (int kk = 0; kk < kDiag - 1; ++kk) {
                __syncwarp();
                for (int e = lane; e < kDiag * kDiag; e += 32) {
                    const int i = e / kDiag, j = e % kDiag;
                    if (i > kk && j <= kk)
                        Gb[i * kPitch + j] = fma(-Ab[i * kPitch + kk] * sb[kk], Gb[kk * kPitch + j], Gb[i * kPitch + j]);
                }
            }
            __syncwarp();
            for (int e = lane; e < kDiag * kDiag; e += 32) {  // G = x_ij / L(i, i), L = a_ij / L(j, j)
                const int i = e / kDiag, j = e % kDiag;
                if (i >= j) {
                    Gb[i * kPitch + j] *= rb[i];
                    Ab[i * kPitch + j] *= rb[j];
                }
            }
        }
        __syncthreads();
        const int r0 = b0 + kDiag, nr = kLeaf - r0;
        for (int e = tid; e < nr * kDiag; e += kThreads) {  // (2) L(i, b0 + j) = sum_t A(i, b0 + t) G_bb(j, t)
            const int i = r0 + e / kDiag, j = e % kDiag;
            double a = 0.0;
            for (int t = 0; t <= j; ++t) a = fma(As[i * kPitch + b0 + t], Gb[j * kPitch + t], a);
            P[i * kPPitch + j] = a;
        }
        __syncthreads();
        for (int e = tid; e < nr * kDiag; e += kThreads) {
            const int i = r0 + e / kDiag, j = e % kDiag;
            As[i * kPitch + b0 + j] = P[i * kPPitch + j];
        }
        for (int e = tid; e < kLeaf * kLeaf; e += kThreads) {  // (3) trailing update, a warp on one row
            const int i = e / kLeaf, j = e % kLeaf;
            if (j < r0 || j > i) continue;
            double a = As[i * kPitch + j];
#pragma unroll
            for (int t = 0; t < kDiag; ++t) a = fma(-P[i * kPPitch + t], P[j * kPPitch + t], a);
            As[i * kPitch + j] = a;
        }
        __syncthreads();
    }
    for (int s = kDiag; s < kLeaf; s *= 2) {  // inverse by doubling
        const int per = s * s, count = (kLeaf / (2 * s)) * per;
        for (int e = tid; e < count; e += kThreads) {  // W = L21 G11 (G11 lower: t >= j)
            const int o = 2 * s * (e / per), i = (e % per) / s, j = e % s;
            double a = 0.0;
            for (int t = j; t < s; ++t) a = fma(As[(o + s + i) * kPitch + o + t], Gs[(o + t) * kPitch + o + j], a);
            Wm[e] = a;
        }
        __syncthreads();
        for (int e = tid; e < count; e += kThreads) {  // G21 = -G22 W (G22 lower: t <= i)
            const int o = 2 * s * (e / per), i = (e % per) / s, j = e % s;
            const double *W = Wm + (e / per) * per;
            double a = 0.0;
            for (int t = 0; t <= i; ++t) a = fma(Gs[(o + s + i) * kPitch + o + s + t], W[t * s + j], a);
            Gs[(o + s + i) * kPitch + o + j] = -a;
        }
        __syncthreads();
    }
    for (int e = tid; e < kLeaf * kLeaf; e += kThreads) {
        const int i = e % kLeaf, j = e / kLeaf;
        if (i < nb && j < nb) {
            const bool low = i >= j;
            G[(size_t)j * ld + i] = low ? Gs[i * kPitch + j] : 0.0;
            A[(size_t)j * ld + i] = low ? As[i * kPitch + j] : 0.0;
        }
    }
}

}  // namespace

int leaf_rows() { return kLeaf; }

cudaError_t leaf_chol_inv64(double *A, double *G, int nb, int ld, int row0, int *info, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(leaf_chol_inv64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kLeaf64Smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (nb <= 0 || nb > kLeaf) return cudaErrorInvalidValue;
    leaf_chol_inv64_kernel<<<1, kThreads, kLeaf64Smem, st>>>(A, G, nb, ld, row0, info);
    count_launch();
    return cudaGetLastError();
}

}  // namespace elhl
