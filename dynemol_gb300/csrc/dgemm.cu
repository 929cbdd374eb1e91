// FP64 matrix products on the FP64 pipe:
//   C = alpha op(A) op(B) + beta C   (column-major, op = identity or transpose).
// They carry the FP64 rebuild (the recursive Cholesky factor with its inverse),
// H' = S^-1 h = G^T (G h) of the drop-in, H~ = G h G^T of fixed nuclei and the
// Ehrenfest contraction, replacing the reference's MAGMA / cuBLAS calls
// (GPU_Interface.cpp:910-928, Taylor_gpu.cpp:686-695, :776-790).
//
// GB300's FP64 pipe retires about two FMAs per clock per SM (1.2 TFLOP/s), so
// the tile only has to keep that pipe fed: 64 x 64 outputs per CTA of 256
// threads, 4 x 4 per thread (16 independent FMA chains), K in steps of 16 staged
// in shared memory by cp.async, double buffered.  Eight shared-memory reads per
// 16 FMAs are far inside the shared-memory bandwidth.
//
// Triangular operands (flags in `tri`, local block coordinates): elements on the
// zero side of a triangular operand are treated as zero whatever is stored
// there, and k tiles that are zero for the whole output tile are skipped, so a
// triangular product costs half a square one.  With kTriLowerC only output
// tiles that reach the diagonal or below it are written (a symmetric update).
// Products with fewer tiles than SMs split K over gridDim.z CTAs per tile: each
// writes its partial tile to a workspace, and the CTA that arrives last at the
// tile's counter sums the partials in split order (deterministic) and writes C;
// no CTA waits.
#include <algorithm>

#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16;
constexpr int kTM = 4, kTN = 4;
constexpr int kRT = kBM / kTM, kCT = kBN / kTN;  // threads along rows and columns
constexpr int kThreads = kRT * kCT;
constexpr int kMaxPartials = 1024;     // tiles x splits held by the split-K workspace
constexpr int kSplitBelowTiles = 152;  // one tile per SM
double *g_part = nullptr;              // [tile][split][kBM * kBN]
int *g_count = nullptr;                // [tile] arrivals, back to 0 after each fix-up

__device__ __forceinline__ void cp_async8(double *dst, const double *src, int src_bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <bool TA, bool TB>
__global__ void __launch_bounds__(kThreads) dgemm_kernel(int m, int n, int k, double alpha,
                                                         const double *__restrict__ A, int lda,
                                                         const double *__restrict__ B, int ldb, double beta,
                                                         double *__restrict__ C, int ldc, int tri,
                                                         double *__restrict__ part, int *__restrict__ count) {
    __shared__ double As[2][kBK][kBM + 1];
    __shared__ double Bs[2][kBK][kBN + 1];
    const int tid = threadIdx.x;
    // blocks start roughly in index order: the tiles with the longest k range
    // (kTriA: the last row tiles; kTriBt: the last column tiles) go first, so
    // that the last wave holds the short ones
    const int bx = (tri & kTriA) ? gridDim.x - 1 - blockIdx.x : blockIdx.x;
    const int by = (tri & kTriBt) ? gridDim.y - 1 - blockIdx.y : blockIdx.y;
    const int i0 = bx * kBM, j0 = by * kBN;
    if ((tri & kTriLowerC) && i0 + kBM <= j0) return;  // tile strictly above the diagonal
    // k range holding non-zero products for this tile
    int klo = 0, khi = k;
    if (tri & kTriA) khi = min(khi, i0 + kBM);   // op(A)(i, l) = A(i, l) = 0 for l > i
    if (tri & kTriAt) klo = max(klo, i0);        // op(A)(i, l) = A(l, i) = 0 for l < i
    if (tri & kTriB) klo = max(klo, j0);         // op(B)(l, j) = B(l, j) = 0 for l < j
    if (tri & kTriBt) khi = min(khi, j0 + kBN);  // op(B)(l, j) = B(j, l) = 0 for l > j
    {  // this split's share of the tile's k tiles
        const int S = gridDim.z, z = blockIdx.z;
        const int nkt = khi > klo ? (khi - klo + kBK - 1) / kBK : 0;
        const int kt0 = z * nkt / S, kt1 = (z + 1) * nkt / S;
        khi = min(khi, klo + kt1 * kBK);
        klo += kt0 * kBK;
    }
    const int tr = tid % kRT, tc = tid / kRT;  // outputs: rows i0 + tr + kRT q, columns j0 + tc + kCT p
    double acc[kTM][kTN];
#pragma unroll
    for (int q = 0; q < kTM; ++q)
#pragma unroll
        for (int p = 0; p < kTN; ++p) acc[q][p] = 0.0;
    // stage s <- the k tile at k0, threads along each operand's contiguous index;
    // masked elements are zero-filled from an in-bounds address
    auto fetch = [&](int s, int k0) {
        for (int t = tid; t < kBM * kBK; t += kThreads) {
            const int ii = TA ? t / kBK : t % kBM, kk = TA ? t % kBK : t / kBM;
            const int gi = i0 + ii, gk = k0 + kk;
            const bool nz = gi < m && gk < k && !((tri & kTriA) && gk > gi) && !((tri & kTriAt) && gk < gi);
            const double *src = TA ? A + (size_t)gi * lda + gk : A + (size_t)gk * lda + gi;
            cp_async8(&As[s][kk][ii], nz ? src : A, nz ? 8 : 0);
        }
        for (int t = tid; t < kBK * kBN; t += kThreads) {
            const int kk = TB ? t / kBN : t % kBK, jj = TB ? t % kBN : t / kBK;
            const int gk = k0 + kk, gj = j0 + jj;
            const bool nz = gk < k && gj < n && !((tri & kTriB) && gk < gj) && !((tri & kTriBt) && gk > gj);
            const double *src = TB ? B + (size_t)gk * ldb + gj : B + (size_t)gj * ldb + gk;
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
            double a[kTM], b[kTN];
#pragma unroll
            for (int q = 0; q < kTM; ++q) a[q] = As[s][kk][tr + kRT * q];
#pragma unroll
            for (int p = 0; p < kTN; ++p) b[p] = Bs[s][kk][tc + kCT * p];
#pragma unroll
            for (int q = 0; q < kTM; ++q)
#pragma unroll
                for (int p = 0; p < kTN; ++p) acc[q][p] = fma(a[q], b[p], acc[q][p]);
        }
        __syncthreads();  // stage s is refilled by the next iteration's fetch
    }
    if (gridDim.z == 1) {
#pragma unroll
        for (int q = 0; q < kTM; ++q)
#pragma unroll
            for (int p = 0; p < kTN; ++p) {
                const int gi = i0 + tr + kRT * q, gj = j0 + tc + kCT * p;
                if (gi < m && gj < n) {
                    double *c = C + (size_t)gj * ldc + gi;
                    *c = beta == 0.0 ? alpha * acc[q][p] : fma(alpha, acc[q][p], beta * *c);
                }
            }
        return;
    }
    // split K: partial tile out, then the last CTA of the tile sums the splits in order
    const int S = gridDim.z, tile = by * gridDim.x + bx;
    double *mine = part + ((size_t)tile * S + blockIdx.z) * (kBM * kBN);
#pragma unroll
    for (int q = 0; q < kTM; ++q)
#pragma unroll
        for (int p = 0; p < kTN; ++p) mine[(tc + kCT * p) * kBM + tr + kRT * q] = acc[q][p];
    __threadfence();
    __syncthreads();
    __shared__ int last;
    if (tid == 0) last = atomicAdd(count + tile, 1) == S - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const double *all = part + (size_t)tile * S * (kBM * kBN);
#pragma unroll
    for (int q = 0; q < kTM; ++q)
#pragma unroll
        for (int p = 0; p < kTN; ++p) {
            const int gi = i0 + tr + kRT * q, gj = j0 + tc + kCT * p, e = (tc + kCT * p) * kBM + tr + kRT * q;
            double sum = __ldcg(all + e);
            for (int z = 1; z < S; ++z) sum += __ldcg(all + (size_t)z * (kBM * kBN) + e);
            if (gi < m && gj < n) {
                double *c = C + (size_t)gj * ldc + gi;
                *c = beta == 0.0 ? alpha * sum : fma(alpha, sum, beta * *c);
            }
        }
    if (tid == 0) count[tile] = 0;
}

}  // namespace

cudaError_t dgemm64(int m, int n, int k, double alpha, const double *A, int lda, bool transA, const double *B, int ldb,
                    bool transB, double beta, double *C, int ldc, cudaStream_t st, int tri) {
    if (m <= 0 || n <= 0) return cudaSuccess;
    if (!g_part) {
        cudaError_t e = cudaMalloc(&g_part, (size_t)kMaxPartials * kBM * kBN * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&g_count, kMaxPartials * sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(g_count, 0, kMaxPartials * sizeof(int));
        if (e != cudaSuccess) return e;
    }
    dim3 grid((m + kBM - 1) / kBM, (n + kBN - 1) / kBN);
    // split K until about two CTAs per SM, at least one k tile per split
    const int tiles = grid.x * grid.y, ktiles = (k + kBK - 1) / kBK;
    int splits = 1;
    if (tiles < kSplitBelowTiles && k > 0)
        splits = std::max(1, std::min({(2 * kSplitBelowTiles + tiles - 1) / tiles, ktiles, 16, kMaxPartials / tiles}));
    grid.z = splits;
#define ELHL_DGEMM(TA_, TB_)                                                                                     \
    dgemm_kernel<TA_, TB_><<<grid, kThreads, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, g_part, \
                                                      g_count)
    if (transA && transB) ELHL_DGEMM(true, true);
    else if (transA) ELHL_DGEMM(true, false);
    else if (transB) ELHL_DGEMM(false, true);
    else ELHL_DGEMM(false, false);
#undef ELHL_DGEMM
    count_launch();
    return cudaGetLastError();
}

}  // namespace elhl
