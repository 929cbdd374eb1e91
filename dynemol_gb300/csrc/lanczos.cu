// Spectral bounds of the Chebyshev operator by Lanczos, in FP64 on the FP64
// pipe, all k steps in one cooperative launch (no host round trip, no library
// GEMV).  The operator is
//   explicit: H~ (symmetric, both triangles stored), w = H~ q;
//   implicit: H~ = G h G^T with G = L^-1 lower triangular and its transpose
//             Gt stored, w = G (h (G^T q)) in three column-dot phases.
// Every product is a set of column dot products M(:, i) . x (columns are
// contiguous in the column-major storage, so the reads coalesce): CTA c takes
// the columns i = c, c + grid, ..., one warp per column, so that every SM
// reads the same share of the matrix; x sits in shared memory when it fits.
// A product with q_j = r_{j-1} / beta_{j-1} is formed from the unnormalised
// r_{j-1} and scaled afterwards, so q_j is never written out.  The dot
// products alpha_j = w.q_j and |w|^2 are summed per CTA in a fixed order and
// then over the CTAs in CTA order: the same grid gives the same bits.
// The reference's adaptive-tau Taylor steps (ElHl_Chebyshev.f:148-268) need
// no spectral interval; the Chebyshev expansion does, and this is its source.
#include <algorithm>

#include "elhl_internal.cuh"
#include "grid_sync.cuh"

namespace elhl {
namespace {

constexpr int kLzThreads = 512, kLzWarps = kLzThreads / 32;
constexpr int kXsCap = 25600;  // x in shared memory up to 200 KB

struct LzArgs {
    int n, ld, k;
    const double *H;   // explicit H~, or h of the implicit operator
    const double *G;   // implicit: G (lower), nullptr for the explicit operator
    const double *Gt;  // implicit: G^T (upper)
    double *r;         // [4][ld] rotating unnormalised Lanczos vectors r_{j-1}
    double *t;         // [2][ld] implicit intermediates G^T q, h G^T q
    double *part;      // [2][grid] per-CTA partial sums
    double *rec;       // alpha [k], beta [k], steps used [1]
    unsigned *bar_count;  // grid barrier: two words, one 64-bit count (zero at the launch)
    int *err;
};

// Scalar work is done by one warp and broadcast through shared memory: GB300's
// FP64 pipe retires under two FMAs per clock per SM, so 512 threads repeating a
// 152-term sum or a square root would cost tens of microseconds per step.
// red: kLzWarps warp partials, then the broadcast slots.
constexpr int kRedSlots = kLzWarps + 3;

// block sum of one value per thread in a fixed order (every thread returns it)
__device__ double block_sum(double v, double *red) {
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double s = lane < kLzWarps ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) red[kLzWarps] = s;
    }
    __syncthreads();
    const double s = red[kLzWarps];
    __syncthreads();
    return s;
}

// the sum of part[0 .. g) in a fixed order (lane-strided partial sums, then a
// shuffle tree), or its square root when root is set (then *inv = 1 / root);
// every thread returns it
__device__ double grid_sum(const double *part, int g, bool root, double *red, double *inv = nullptr) {
    const int lane = threadIdx.x % 32;
    if (threadIdx.x < 32) {
        double s = 0.0;
        for (int c = lane; c < g; c += 32) s += __ldcg(part + c);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) {
            if (root) s = sqrt(s);
            red[kLzWarps + 1] = s;
            red[kLzWarps + 2] = root ? 1.0 / s : 0.0;
        }
    }
    __syncthreads();
    const double s = red[kLzWarps + 1];
    if (inv) *inv = red[kLzWarps + 2];
    __syncthreads();
    return s;
}

// x[l]: shared memory, or global memory written earlier in this launch by other
// CTAs (read through L2, never a possibly stale L1 line)
template <bool kGlobal>
__device__ __forceinline__ double xload(const double *x, int l) {
    if constexpr (kGlobal) return __ldcg(x + l);
    else return x[l];
}

// out[i] = scale * sum_l M(l, i) x[l] over the rows l of column i that may be
// non-zero (tri 0: all; 1: l >= i, M lower; 2: l <= i, M upper), for the columns
// of this CTA; returns this CTA's sum of out[i] * y[i] * ys (y may be null).
template <bool kGlobal>
__device__ double column_dots(const double *__restrict__ M, int ld, int n, int tri, const double *x, double *out,
                              double scale, const double *y, double ys, double *red) {
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    double mine = 0.0;
    for (int i = blockIdx.x + (int)gridDim.x * warp; i < n; i += (int)gridDim.x * kLzWarps) {
        const int lo = tri == 1 ? i : 0, hi = tri == 2 ? i + 1 : n;
        const double *col = M + (size_t)i * ld;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        int l = lo + lane;
        for (; l + 96 < hi; l += 128) {
            a0 = fma(__ldcs(col + l), xload<kGlobal>(x, l), a0);
            a1 = fma(__ldcs(col + l + 32), xload<kGlobal>(x, l + 32), a1);
            a2 = fma(__ldcs(col + l + 64), xload<kGlobal>(x, l + 64), a2);
            a3 = fma(__ldcs(col + l + 96), xload<kGlobal>(x, l + 96), a3);
        }
        for (; l < hi; l += 32) a0 = fma(__ldcs(col + l), xload<kGlobal>(x, l), a0);
        double s = (a0 + a1) + (a2 + a3);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            s *= scale;
            out[i] = s;
            if (y) mine = fma(s, __ldcg(y + i) * ys, mine);
        }
    }
    return block_sum(lane == 0 ? mine : 0.0, red);
}

// out <- scale * M^T x (column dots as above) with x = src staged in shared
// memory when it fits, read through L2 otherwise
__device__ double product(const double *__restrict__ M, int ld, int n, int tri, const double *src, double *out,
                          double scale, const double *y, double ys, double *xs, double *red) {
    if (n > kXsCap) return column_dots<true>(M, ld, n, tri, src, out, scale, y, ys, red);
    for (int i = threadIdx.x; i < n; i += kLzThreads) xs[i] = __ldcg(src + i);
    __syncthreads();
    const double r = column_dots<false>(M, ld, n, tri, xs, out, scale, y, ys, red);
    return r;  // block_sum's barriers keep xs until every warp is done
}

__global__ void __launch_bounds__(kLzThreads) lanczos64_kernel(const LzArgs a) {
    extern __shared__ double xs[];  // [min(n, kXsCap)], then kRedSlots reduction slots
    double *red = xs + (a.n > kXsCap ? 0 : a.n);
    const int n = a.n, ld = a.ld, k = a.k, g = gridDim.x;
    const int stride = g * kLzThreads;
    double *pa = a.part, *pb = a.part + g;
    // r_{-1}: a deterministic start with every component present; q_0 = r_{-1} / |r_{-1}|
    double acc = 0.0;
    for (int i = blockIdx.x * kLzThreads + threadIdx.x; i < n; i += stride) {
        const double v = 1.0 + 0.5 * sin(1.37 * i + 0.2);
        a.r[i] = v;
        acc = fma(v, v, acc);
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) pb[blockIdx.x] = acc;
    if (!grid_barrier(a.bar_count, g, a.err)) return;
    double sq = 0.0;  // q_j = r[j & 3] * sq
    grid_sum(pb, g, true, red, &sq);
    double sp = 0.0, bprev = 0.0;              // q_{j-1} = r[(j + 3) & 3] * sp
    for (int j = 0; j < k; ++j) {
        const double *rq = a.r + (size_t)(j & 3) * ld, *rp = a.r + (size_t)((j + 3) & 3) * ld;
        double *rw = a.r + (size_t)((j + 1) & 3) * ld;
        double part;
        if (!a.G) {
            part = product(a.H, ld, n, 0, rq, rw, sq, rq, sq, xs, red);
        } else {
            double *t1 = a.t, *t2 = a.t + ld;
            product(a.G, ld, n, 1, rq, t1, 1.0, nullptr, 0.0, xs, red);  // G^T r
            if (!grid_barrier(a.bar_count, g, a.err)) return;
            product(a.H, ld, n, 0, t1, t2, 1.0, nullptr, 0.0, xs, red);  // h (.)
            if (!grid_barrier(a.bar_count, g, a.err)) return;
            part = product(a.Gt, ld, n, 2, t2, rw, sq, rq, sq, xs, red);  // G (.) sq
        }
        if (threadIdx.x == 0) pa[blockIdx.x] = part;
        if (!grid_barrier(a.bar_count, g, a.err)) return;
        const double alpha = grid_sum(pa, g, false, red);
        // r_j = w - alpha q_j - beta_{j-1} q_{j-1}
        acc = 0.0;
        for (int i = blockIdx.x * kLzThreads + threadIdx.x; i < n; i += stride) {
            double x = __ldcg(rw + i) - alpha * (__ldcg(rq + i) * sq);
            if (j > 0) x -= bprev * (__ldcg(rp + i) * sp);
            rw[i] = x;
            acc = fma(x, x, acc);
        }
        acc = block_sum(acc, red);
        if (threadIdx.x == 0) pb[blockIdx.x] = acc;
        if (!grid_barrier(a.bar_count, g, a.err)) return;
        double ibeta = 0.0;
        const double beta = grid_sum(pb, g, true, red, &ibeta);
        const bool stop = !(beta > 1e-10 * (fabs(alpha) + 1.0));  // invariant subspace found
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.rec[j] = alpha;
            a.rec[k + j] = beta;
            if (stop) a.rec[2 * k] = j + 1;
        }
        if (stop) return;
        sp = sq;
        sq = ibeta;
        bprev = beta;
    }
}

}  // namespace

cudaError_t launch_lanczos64(int n, int ld, int k, const double *H, const double *G, const double *Gt, double *r,
                             double *t, double *part, int part_cap, double *rec, unsigned *bar, int *err,
                             cudaStream_t st) {
    static int grid = 0;
    if (!grid) {  // one CTA per SM, co-resident at the largest shared-memory size
        const int smem_max = (int)((kXsCap + kRedSlots) * sizeof(double));
        int dev = 0, sms = 0, per = 0;
        cudaError_t e = cudaFuncSetAttribute(lanczos64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lanczos64_kernel, kLzThreads, smem_max);
        if (e != cudaSuccess) return e;
        if (per < 1) return cudaErrorInvalidConfiguration;
        grid = sms;
    }
    const size_t smem = (size_t)(std::min(n, kXsCap) + kRedSlots) * sizeof(double);
    if (grid > part_cap || k < 1 || n < 1 || (G && !Gt)) return cudaErrorInvalidValue;
    LzArgs a{n, ld, k, H, G, Gt, r, t, part, rec, bar, err};
    void *args[] = {&a};
    cudaError_t e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st);
    if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel((const void *)lanczos64_kernel, dim3(grid), dim3(kLzThreads), args, smem, st);
    count_launch();
    return e;
}

}  // namespace elhl
