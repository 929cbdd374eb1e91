// Matrix product in double-float (DF64) arithmetic on the FP32 pipes:
//   C = alpha A op(B) + beta C   (column-major, op(B) = B or B^T),
// with A, B and C stored as DF64 pairs (float2 = hi + lo, 48-bit significand).
// Products use the exact FMA product error and sums TwoSum (df64.cuh), 12 FP32
// instructions per FMA, accurate to about 4e-15 relative, while the FP64 pipe
// (1/58 of the FP32 rate on this part) stays idle.  Operands are split into
// pairs once, outside: splitting on every load took 3 conversions and an add
// on the FP64-rate units per element, as much time as the products.  The
// epilogue (alpha, beta, split-K sums) is double-float too: in FP64 it was
// most of the time of the small products.  Used by the DF64 rebuild (the
// recursive Cholesky factor and its inverse).
//
// Triangular operands (flags in `tri`, local block coordinates): elements on the
// zero side of a triangular operand are treated as zero whatever is stored
// there, and k tiles that are zero for the whole output tile are skipped, so a
// triangular product costs half a square one.  With kTriLowerC only output
// tiles that reach the diagonal or below it are written (a symmetric update).
//
// Tiling: 64 x 64 output tile per CTA of 256 threads, kTM x kTN = 4 x 4 outputs per thread,
// K in steps of 16 staged in shared memory, two stages: cp.async fetches the
// next k tile (zero-filling masked elements) while the current one is used.  Products with fewer tiles than SMs
// (the lower levels of the recursive factorisations) split K over gridDim.z
// CTAs per tile: each writes its partial tile (pairs) to a workspace, and the
// CTA that arrives last at the tile's counter sums the partials in split order
// (deterministic) and writes C; no CTA waits.
#include <algorithm>

#include "df64.cuh"
#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16;
// outputs per thread (rows x columns); measured on the N = 3720 DF64 factorisation:
// 4 x 4 (64 registers) 23.2 ms, 8 x 4 24.9 ms, 4 x 8 25.4 ms (124-128 registers)
constexpr int kTM = 4, kTN = 4;
constexpr int kRT = kBM / kTM, kCT = kBN / kTN;      // threads along rows and columns
constexpr int kThreads = kRT * kCT;
constexpr int kMaxPartials = 1024;     // tiles x splits held by the split-K workspace
constexpr int kSplitBelowTiles = 152;  // one tile per SM
float2 *g_part = nullptr;              // [tile][split][kBM * kBN]
int *g_count = nullptr;                // [tile] arrivals, back to 0 after each fix-up

// 8-byte global -> shared copy, asynchronous; src_bytes = 0 writes zeros
__device__ __forceinline__ void cp_async8(float2 *dst, const float2 *src, int src_bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// c <- alpha v + beta c (beta = 0: c not read)
__device__ __forceinline__ void store_df(float2 *c, float2 v, float2 alpha, float2 beta) {
    v = df_mul(v, alpha);
    if (beta.x != 0.f) v = df_sum(v, df_mul(*c, beta));
    *c = v;
}

template <bool TB>
__global__ void __launch_bounds__(kThreads) dfgemm_kernel(int m, int n, int k, float2 alpha, const float2 *__restrict__ A,
                                                          int lda, const float2 *__restrict__ B, int ldb, float2 beta,
                                                          float2 *__restrict__ C, int ldc, int tri,
                                                          float2 *__restrict__ part, int *__restrict__ count) {
    __shared__ float2 As[2][kBK][kBM + 1];
    __shared__ float2 Bs[2][kBK][kBN + 1];
    const int tid = threadIdx.x;
    const int i0 = blockIdx.x * kBM, j0 = blockIdx.y * kBN;
    if ((tri & kTriLowerC) && i0 + kBM <= j0) return;  // tile strictly above the diagonal
    // k range holding non-zero products for this tile
    int klo = 0, khi = k;
    if (tri & kTriA) khi = min(khi, i0 + kBM);   // A(i, l) = 0 for l > i
    if (tri & kTriB) klo = j0;                   // B(l, j) = 0 for l < j
    if (tri & kTriBt) khi = min(khi, j0 + kBN);  // B^T(l, j) = B(j, l) = 0 for l > j
    {  // this split's share of the tile's k tiles
        const int S = gridDim.z, z = blockIdx.z;
        const int nkt = khi > klo ? (khi - klo + kBK - 1) / kBK : 0;
        const int kt0 = z * nkt / S, kt1 = (z + 1) * nkt / S;
        khi = min(khi, klo + kt1 * kBK);
        klo += kt0 * kBK;
    }
    const int tr = tid % kRT, tc = tid / kRT;  // outputs: rows i0 + tr + kRT q, columns j0 + tc + kCT p
    float sh[kTM][kTN], sl[kTM][kTN];
#pragma unroll
    for (int q = 0; q < kTM; ++q)
#pragma unroll
        for (int p = 0; p < kTN; ++p) sh[q][p] = sl[q][p] = 0.f;
    // stage s <- the k tile at k0: A tile kBM x kBK with consecutive threads on
    // consecutive rows, op(B) tile kBK x kBN along its contiguous index (both
    // coalesced); masked elements are zero-filled from an in-bounds address
    auto fetch = [&](int s, int k0) {
        for (int t = tid; t < kBM * kBK; t += kThreads) {
            const int ii = t % kBM, kk = t / kBM;
            const int gi = i0 + ii, gk = k0 + kk;
            const bool nz = gi < m && gk < k && !((tri & kTriA) && gk > gi);
            cp_async8(&As[s][kk][ii], nz ? A + (size_t)gk * lda + gi : A, nz ? 8 : 0);
        }
        for (int t = tid; t < kBK * kBN; t += kThreads) {
            const int kk = TB ? t / kBN : t % kBK, jj = TB ? t % kBN : t / kBK;
            const int gk = k0 + kk, gj = j0 + jj;
            const bool nz = gk < k && gj < n && !((tri & kTriB) && gk < gj) && !((tri & kTriBt) && gk > gj);
            const float2 *src = TB ? B + (size_t)gk * ldb + gj : B + (size_t)gj * ldb + gk;
            cp_async8(&Bs[s][kk][jj], nz ? src : B, nz ? 8 : 0);
        }
        cp_async_commit();
    };
    if (klo < khi) fetch(0, klo);
    int s = 0;
    for (int k0 = klo; k0 < khi; k0 += kBK, s ^= 1) {
        if (k0 + kBK < khi) {
            fetch(s ^ 1, k0 + kBK);
            cp_async_wait<1>();  // this tile's group is complete, the next one may be in flight
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kBK; ++kk) {
            float2 a[kTM], b[kTN];
#pragma unroll
            for (int q = 0; q < kTM; ++q) a[q] = As[s][kk][tr + kRT * q];
#pragma unroll
            for (int p = 0; p < kTN; ++p) b[p] = Bs[s][kk][tc + kCT * p];
#pragma unroll
            for (int q = 0; q < kTM; ++q)
#pragma unroll
                for (int p = 0; p < kTN; ++p) df_fma(sh[q][p], sl[q][p], a[q].x, a[q].y, b[p].x, b[p].y);
        }
        __syncthreads();  // stage s is refilled by the next iteration's fetch
    }
    if (gridDim.z == 1) {
#pragma unroll
        for (int q = 0; q < kTM; ++q)
#pragma unroll
            for (int p = 0; p < kTN; ++p) {
                const int gi = i0 + tr + kRT * q, gj = j0 + tc + kCT * p;
                if (gi < m && gj < n) store_df(C + (size_t)gj * ldc + gi, df_renorm(sh[q][p], sl[q][p]), alpha, beta);
            }
        return;
    }
    // split K: partial tile out, then the last CTA of the tile sums the splits in order
    const int S = gridDim.z, tile = blockIdx.y * gridDim.x + blockIdx.x;
    float2 *mine = part + ((size_t)tile * S + blockIdx.z) * (kBM * kBN);
#pragma unroll
    for (int q = 0; q < kTM; ++q)
#pragma unroll
        for (int p = 0; p < kTN; ++p) mine[(tc + kCT * p) * kBM + tr + kRT * q] = df_renorm(sh[q][p], sl[q][p]);
    __threadfence();
    __syncthreads();
    __shared__ int last;
    if (tid == 0) last = atomicAdd(count + tile, 1) == S - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const float2 *all = part + (size_t)tile * S * (kBM * kBN);
#pragma unroll
    for (int q = 0; q < kTM; ++q)
#pragma unroll
        for (int p = 0; p < kTN; ++p) {
            const int gi = i0 + tr + kRT * q, gj = j0 + tc + kCT * p, e = (tc + kCT * p) * kBM + tr + kRT * q;
            float2 sum = __ldcg(all + e);
            for (int z = 1; z < S; ++z) sum = df_sum(sum, __ldcg(all + (size_t)z * (kBM * kBN) + e));
            if (gi < m && gj < n) store_df(C + (size_t)gj * ldc + gi, sum, alpha, beta);
        }
    if (tid == 0) count[tile] = 0;
}

// x <- its DF64 pair in place (to_pairs) or back to FP64, for an ld x n matrix
__global__ void df_convert_kernel(double *x, int rows, int n, int ld, bool to_pairs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= rows || j >= n) return;
    double *p = x + (size_t)j * ld + i;
    if (to_pairs) *reinterpret_cast<float2 *>(p) = df_split(*p);
    else *p = df_value(*reinterpret_cast<const float2 *>(p));
}

}  // namespace

cudaError_t df_convert(double *x, int rows, int n, int ld, bool to_pairs, cudaStream_t st) {
    if (rows <= 0 || n <= 0) return cudaSuccess;
    df_convert_kernel<<<dim3((rows + 127) / 128, n), 128, 0, st>>>(x, rows, n, ld, to_pairs);
    count_launch();
    return cudaGetLastError();
}

cudaError_t dfgemm(int m, int n, int k, double alpha, const float2 *A, int lda, const float2 *B, int ldb, double beta,
                   float2 *C, int ldc, cudaStream_t st, bool transB, int tri) {
    if (m <= 0 || n <= 0) return cudaSuccess;
    if (!g_part) {
        cudaError_t e = cudaMalloc(&g_part, (size_t)kMaxPartials * kBM * kBN * sizeof(float2));
        if (e == cudaSuccess) e = cudaMalloc(&g_count, kMaxPartials * sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(g_count, 0, kMaxPartials * sizeof(int));
        if (e != cudaSuccess) return e;
    }
    dim3 grid((m + kBM - 1) / kBM, (n + kBN - 1) / kBN);
    // split K until about two CTAs per SM, at least one k tile per split
    const int tiles = grid.x * grid.y, ktiles = (k + kBK - 1) / kBK;
    int splits = 1;
    if (tiles < kSplitBelowTiles)
        splits = std::max(1, std::min({(2 * kSplitBelowTiles + tiles - 1) / tiles, ktiles, 16, kMaxPartials / tiles}));
    grid.z = splits;
    const float ah = (float)alpha, bh = (float)beta;  // alpha and beta as pairs
    const float2 a2 = make_float2(ah, (float)(alpha - ah)), b2 = make_float2(bh, (float)(beta - bh));
    if (transB) {
        dfgemm_kernel<true><<<grid, kThreads, 0, st>>>(m, n, k, a2, A, lda, B, ldb, b2, C, ldc, tri, g_part, g_count);
        count_launch();
    } else {
        dfgemm_kernel<false><<<grid, kThreads, 0, st>>>(m, n, k, a2, A, lda, B, ldb, b2, C, ldc, tri, g_part, g_count);
        count_launch();
    }
    return cudaGetLastError();
}

}  // namespace elhl
