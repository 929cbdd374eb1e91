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
// 16 FMAs are far inside the shared-memory bandwidth.  Products too small to
// give every SM work in 64 x 64 tiles (the 64- to 256-row blocks of the
// factorisations: one 64^3 product is 4 units of 64 x 64 x 16) take 32 x 32 or
// 16 x 16 tiles (2 x 2 or 1 x 1 outputs per thread), so that up to 64 times as
// many SMs share them.
//
// Triangular operands (flags in `tri`, local block coordinates): elements on the
// zero side of a triangular operand are treated as zero whatever is stored
// there, and k tiles that are zero for the whole output tile are skipped, so a
// triangular product costs half a square one.  With kTriLowerC only output
// tiles that reach the diagonal or below it are written (a symmetric update).
// Work is scheduled dynamically: the FP64 pipe is saturated while a CTA runs
// (ncu: 99.6 % of its active cycles on the top-level product of an N = 2790
// factorisation), so what costs time is SMs left idle when the tiles of a
// triangular product (k ranges from one k tile to all of them) are dealt out
// statically.  Persistent CTAs pull (tile, k-chunk) units from a counter; a
// tile split into chunks is summed by its last arriving unit in chunk order
// (deterministic); no CTA waits.
#include <algorithm>

#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kBK = 16;
constexpr int kRT = 16, kCT = 16;      // threads along rows and columns
constexpr int kThreads = kRT * kCT;
constexpr int kMaxTile = 64;           // output tiles of BM x BM, BM = 64, 32 or 16
constexpr int kMaxPartials = 4096;     // partial 64 x 64 tiles held by the workspace (128 MB)
constexpr int kUnitsPerSlot = 6;       // work units per resident CTA the chunk length aims at
constexpr int kLanes = 2;              // products that may run concurrently (streams), each with its own state
struct Lane {
    double *part = nullptr;            // [tile * chunks + chunk][BM * BM]
    int *count = nullptr;              // [tile] arrivals, back to 0 after each fix-up
    int *sched = nullptr;              // next unit (64-bit), CTAs finished; back to 0 after each launch
};
Lane g_lane[kLanes];
int g_sms = 0;
int g_slots[3] = {0, 0, 0};            // resident CTAs of the whole GPU for BM = 64, 32, 16

__device__ __forceinline__ void cp_async8(double *dst, const double *src, int src_bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

struct DgemmArgs {
    int m, n, k;
    double alpha, beta;
    const double *A, *B;
    double *C;
    int lda, ldb, ldc, tri;
    int gx, gy;        // output tiles along rows and columns
    int chunk;         // k tiles per work unit
    int nchunk;        // chunks of the longest k range (units per tile)
    long long units;   // gx * gy * nchunk
    double *part;
    int *count, *sched;
};

// Persistent CTAs pull work units u = (tile, k-chunk) from an atomic counter:
// the FP64 pipe of every SM stays busy until the last units, whatever the
// mix of long and short (triangular) k ranges.  A tile with one chunk writes C
// directly; otherwise each chunk writes its partial tile and the unit arriving
// last at the tile's counter sums the partials in chunk order (deterministic)
// and writes C.  The last CTA to finish resets the counter for the next launch.
template <bool TA, bool TB, int BM>
__global__ void __launch_bounds__(kThreads) dgemm_kernel(const DgemmArgs g) {
    constexpr int kBM = BM, kBN = BM, kTM = BM / kRT, kTN = BM / kCT;
    __shared__ double As[2][kBK][kBM + 1];
    __shared__ double Bs[2][kBK][kBN + 1];
    __shared__ long long s_unit;
    __shared__ int s_last;
    const int tid = threadIdx.x, tri = g.tri, m = g.m, n = g.n, k = g.k;
    const double *__restrict__ A = g.A;
    const double *__restrict__ B = g.B;
    const int tr = tid % kRT, tc = tid / kRT;  // outputs: rows i0 + tr + kRT q, columns j0 + tc + kCT p
    for (;;) {
        if (tid == 0) s_unit = atomicAdd(reinterpret_cast<unsigned long long *>(g.sched), 1ull);
        __syncthreads();
        const long long u = s_unit;
        __syncthreads();  // s_unit is rewritten by the next fetch
        if (u >= g.units) break;
        const int t = (int)(u / g.nchunk), ch = (int)(u % g.nchunk);
        // tiles with the longest k range (kTriA: the last row tiles; kTriBt: the last
        // column tiles) come first
        const int bx0 = t % g.gx, by0 = t / g.gx;
        const int bx = (tri & kTriA) ? g.gx - 1 - bx0 : bx0;
        const int by = (tri & kTriBt) ? g.gy - 1 - by0 : by0;
        const int i0 = bx * kBM, j0 = by * kBN;
        if ((tri & kTriLowerC) && i0 + kBM <= j0) continue;  // tile strictly above the diagonal
        // k range holding non-zero products for this tile
        int klo = 0, khi = k;
        if (tri & kTriA) khi = min(khi, i0 + kBM);   // op(A)(i, l) = A(i, l) = 0 for l > i
        if (tri & kTriAt) klo = max(klo, i0);        // op(A)(i, l) = A(l, i) = 0 for l < i
        if (tri & kTriB) klo = max(klo, j0);         // op(B)(l, j) = B(l, j) = 0 for l < j
        if (tri & kTriBt) khi = min(khi, j0 + kBN);  // op(B)(l, j) = B(j, l) = 0 for l > j
        const int nkt = khi > klo ? (khi - klo + kBK - 1) / kBK : 0;
        const int nch = max(1, (nkt + g.chunk - 1) / g.chunk);  // chunks of this tile
        if (ch >= nch) continue;
        {  // this chunk's k tiles
            const int kt0 = ch * g.chunk, kt1 = min(nkt, kt0 + g.chunk);
            khi = min(khi, klo + kt1 * kBK);
            klo += kt0 * kBK;
        }
        double acc[kTM][kTN];
#pragma unroll
        for (int q = 0; q < kTM; ++q)
#pragma unroll
            for (int p = 0; p < kTN; ++p) acc[q][p] = 0.0;
        // stage s <- the k tile at k0, threads along each operand's contiguous index;
        // masked elements are zero-filled from an in-bounds address
        auto fetch = [&](int s, int k0) {
            for (int e = tid; e < kBM * kBK; e += kThreads) {
                const int ii = TA ? e / kBK : e % kBM, kk = TA ? e % kBK : e / kBM;
                const int gi = i0 + ii, gk = k0 + kk;
                const bool nz = gi < m && gk < k && !((tri & kTriA) && gk > gi) && !((tri & kTriAt) && gk < gi);
                const double *src = TA ? A + (size_t)gi * g.lda + gk : A + (size_t)gk * g.lda + gi;
                cp_async8(&As[s][kk][ii], nz ? src : A, nz ? 8 : 0);
            }
            for (int e = tid; e < kBK * kBN; e += kThreads) {
                const int kk = TB ? e / kBN : e % kBK, jj = TB ? e % kBN : e / kBK;
                const int gk = k0 + kk, gj = j0 + jj;
                const bool nz = gk < k && gj < n && !((tri & kTriB) && gk < gj) && !((tri & kTriBt) && gk > gj);
                const double *src = TB ? B + (size_t)gk * g.ldb + gj : B + (size_t)gj * g.ldb + gk;
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
        if (nch == 1) {
#pragma unroll
            for (int q = 0; q < kTM; ++q)
#pragma unroll
                for (int p = 0; p < kTN; ++p) {
                    const int gi = i0 + tr + kRT * q, gj = j0 + tc + kCT * p;
                    if (gi < m && gj < n) {
                        double *c = g.C + (size_t)gj * g.ldc + gi;
                        *c = g.beta == 0.0 ? g.alpha * acc[q][p] : fma(g.alpha, acc[q][p], g.beta * *c);
                    }
                }
            continue;
        }
        // partial tile out, then the last unit of the tile sums the chunks in order
        const int tile = by * g.gx + bx;
        double *mine = g.part + ((size_t)tile * g.nchunk + ch) * (kBM * kBN);
#pragma unroll
        for (int q = 0; q < kTM; ++q)
#pragma unroll
            for (int p = 0; p < kTN; ++p) mine[(tc + kCT * p) * kBM + tr + kRT * q] = acc[q][p];
        __threadfence();
        __syncthreads();
        if (tid == 0) s_last = atomicAdd(g.count + tile, 1) == nch - 1;
        __syncthreads();
        if (!s_last) continue;
        __threadfence();
        const double *all = g.part + (size_t)tile * g.nchunk * (kBM * kBN);
#pragma unroll
        for (int q = 0; q < kTM; ++q)
#pragma unroll
            for (int p = 0; p < kTN; ++p) {
                const int gi = i0 + tr + kRT * q, gj = j0 + tc + kCT * p, e = (tc + kCT * p) * kBM + tr + kRT * q;
                double sum = __ldcg(all + e);
                for (int z = 1; z < nch; ++z) sum += __ldcg(all + (size_t)z * (kBM * kBN) + e);
                if (gi < m && gj < n) {
                    double *c = g.C + (size_t)gj * g.ldc + gi;
                    *c = g.beta == 0.0 ? g.alpha * sum : fma(g.alpha, sum, g.beta * *c);
                }
            }
        if (tid == 0) g.count[tile] = 0;
    }
    // the last CTA out resets the scheduler for the next launch (stream order)
    if (tid == 0 && atomicAdd(g.sched + 2, 1) == (int)gridDim.x - 1) {
        *reinterpret_cast<unsigned long long *>(g.sched) = 0ull;
        g.sched[2] = 0;
    }
}

template <int BM>
cudaError_t launch_dgemm(const DgemmArgs &g, bool transA, bool transB, int grid, cudaStream_t st) {
#define ELHL_DGEMM(TA_, TB_) dgemm_kernel<TA_, TB_, BM><<<grid, kThreads, 0, st>>>(g)
    if (transA && transB) ELHL_DGEMM(true, true);
    else if (transA) ELHL_DGEMM(true, false);
    else if (transB) ELHL_DGEMM(false, true);
    else ELHL_DGEMM(false, false);
#undef ELHL_DGEMM
    return cudaGetLastError();
}

template <int BM>
cudaError_t resident(int &slots) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dgemm_kernel<false, false, BM>, kThreads, 0);
    slots = std::max(1, per_sm) * g_sms;
    return e;
}

}  // namespace

cudaError_t dgemm64(int m, int n, int k, double alpha, const double *A, int lda, bool transA, const double *B, int ldb,
                    bool transB, double beta, double *C, int ldc, cudaStream_t st, int tri, int lane) {
    if (m <= 0 || n <= 0) return cudaSuccess;
    if (lane < 0 || lane >= kLanes) return cudaErrorInvalidValue;
    if (!g_sms) {
        int dev = 0, sms = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        g_sms = sms;
        if ((e = resident<64>(g_slots[0])) != cudaSuccess) return e;
        if ((e = resident<32>(g_slots[1])) != cudaSuccess) return e;
        if ((e = resident<16>(g_slots[2])) != cudaSuccess) return e;
    }
    Lane &ln = g_lane[lane];
    if (!ln.part) {
        cudaError_t e = cudaMalloc(&ln.part, (size_t)kMaxPartials * kMaxTile * kMaxTile * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&ln.count, (size_t)kMaxPartials * 16 * sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(ln.count, 0, (size_t)kMaxPartials * 16 * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc(&ln.sched, 4 * sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(ln.sched, 0, 4 * sizeof(int));
        if (e != cudaSuccess) return e;
    }
    const int kt = std::max(1, (k + kBK - 1) / kBK);
    // the largest tile at most twice the product's narrow side whose (tile, k tile)
    // units number at least half of kUnitsPerSlot per resident CTA slot; else the
    // smallest
    int v = 0;
    while (v < 2) {
        const int bm = kMaxTile >> v;
        const long long units = (long long)((m + bm - 1) / bm) * ((n + bm - 1) / bm) * kt;
        if (bm <= 2 * std::min(m, n) && 2 * units >= (long long)kUnitsPerSlot * g_slots[v]) break;
        ++v;
    }
    const int bm = kMaxTile >> v, scale = 1 << (2 * v);  // partial tiles per 64 x 64 of workspace
    // lane 1 runs beside lane 0's work (single-CTA leaves, small products): it leaves
    // a quarter of the resident CTA slots free
    const int slots = lane == 0 ? g_slots[v] : std::max(1, g_slots[v] * 3 / 4);
    DgemmArgs g{m, n, k, alpha, beta, A, B, C, lda, ldb, ldc, tri, (m + bm - 1) / bm, (n + bm - 1) / bm,
                1, 1, 0, ln.part, ln.count, ln.sched};
    const long long tiles = (long long)g.gx * g.gy, max_part = (long long)kMaxPartials * scale;
    // chunk length: about kUnitsPerSlot units per resident CTA, whole k ranges when
    // the tiles alone are enough, and no more partial tiles than the workspace holds
    long long chunk = (tiles * kt + (long long)kUnitsPerSlot * slots - 1) / ((long long)kUnitsPerSlot * slots);
    chunk = std::max(1ll, std::min<long long>(chunk, kt));
    while (chunk < kt && tiles * ((kt + chunk - 1) / chunk) > max_part) chunk *= 2;
    if (chunk >= kt) chunk = kt;
    g.chunk = (int)chunk;
    g.nchunk = (kt + g.chunk - 1) / g.chunk;
    if (g.nchunk > 1 && tiles > max_part) return cudaErrorInvalidValue;  // never: chunk = kt above
    g.units = tiles * g.nchunk;
    const int grid = (int)std::min<long long>(g.units, slots);
    cudaError_t e = v == 0   ? launch_dgemm<64>(g, transA, transB, grid, st)
                    : v == 1 ? launch_dgemm<32>(g, transA, transB, grid, st)
                             : launch_dgemm<16>(g, transA, transB, grid, st);
    count_launch();
    return e;
}

}  // namespace elhl
