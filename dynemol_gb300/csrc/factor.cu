// Dense Cholesky-with-inverse of one diagonal block of at most L = 64 rows in
// FP64, one CTA of 256 threads, entirely in shared memory: the leaves of the
// rebuild's recursive factorisation (S = L L^T with G = L^-1) for every
// precision, and of the drop-in's H' = S^-1 h.  Library triangular kernels at
// these sizes (cuSOLVER trtri on 256 rows, cuBLAS DTRMM/DTRSM panels) ran on a
// handful of CTAs for 65-106 us per call.
//
// The cost model is GB300's FP64 pipe: one FP64 warp instruction occupies its
// SM sub-partition (SMSP) for 76 cycles whether 1 or 32 lanes are active, and
// a dependent FP64 operation waits 64 cycles (rsqrt: about 370).  So the
// kernel counts warp instructions, not flops:
//   - every element loop runs over a dense list of the elements that change
//     (triangles enumerated column by column from the last column, so that
//     "columns >= c" is a prefix of the list), never over a square with
//     predicated-off lanes;
//   - the products of the inverse give the lanes of a warp equal trip counts;
//   - the serial chain (pivots of the 8 x 8 diagonal blocks) runs in warp 0
//     alone while the warps of the other three SMSPs do the trailing update
//     of the previous block (one block of lookahead), so that the chain and
//     the bulk work overlap instead of adding up.
#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kLeafRows = 64, kThreads = 256;
constexpr int kDiag = 8, kPPitch = kDiag + 1;
constexpr int kOthers = 192;  // threads of warps 1-3 and 5-7 (not on warp 0's SMSP)

// element e of the lower triangle of an n x n block, columns from the last:
// column n - 1 - q holds e in [q (q + 1) / 2, (q + 1) (q + 2) / 2), rows from
// the diagonal down; "columns >= c" are the first (n - c)(n - c + 1) / 2
__device__ __forceinline__ void tri_elem(int e, int n, int &i, int &j) {
    int q = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
    while ((q + 1) * (q + 2) / 2 <= e) ++q;
    while (q * (q + 1) / 2 > e) --q;
    j = n - 1 - q;
    i = j + (e - q * (q + 1) / 2);
}

template <int L>
__host__ __device__ constexpr int tri_count() { return L * (L + 1) / 2; }

// products of the doubling inverse: [L * L / 4] for one level at a time, or for
// L = 64 the 8-, 16- and 32-row levels side by side (4 x 64 + 2 x 256 + 1024)
template <int L>
__host__ __device__ constexpr int leaf_wm() { return 7 * L * L / 16; }

template <int L>
constexpr size_t leaf_smem() {
    return (size_t)(2 * L * (L + 1) + L * kPPitch + leaf_wm<L>() + 2 * kDiag) * sizeof(double) +
           (size_t)tri_count<L>() * sizeof(int);
}

// The doubling inverse of one s x s pair of diagonal blocks at o = 2 s blk
// (pitch p): W = L21 G11 (G11 lower: t >= j) and G21 = -G22 W (G22 lower: t <= i).
// W's rows of L21 come from `l21` (row i at l21 + i * lp: As, or the panel while
// its copy into As is in flight).  Columns j0 .. j1 of W only; lanes along i for
// W (equal trips s - j), along j for G21 (equal trips i + 1).
__device__ void inv_w(const double *l21, int lp, const double *Gs, int p, double *W, int s, int o, int j0, int j1,
                      int tid, int nthr) {
    const int count = (j1 - j0) * s;
    for (int e = tid; e < count; e += nthr) {
        const int j = j0 + e / s, i = e % s;
        double a = 0.0;
        for (int t = j; t < s; ++t) a = fma(l21[i * lp + t], Gs[(o + t) * p + o + j], a);
        W[i * s + j] = a;
    }
}
__device__ void inv_g(double *Gs, int p, const double *W, int s, int o, int tid, int nthr) {
    for (int e = tid; e < s * s; e += nthr) {
        const int i = e / s, j = e % s;
        double a = 0.0;
        for (int t = 0; t <= i; ++t) a = fma(Gs[(o + s + i) * p + o + s + t], W[t * s + j], a);
        Gs[(o + s + i) * p + o + j] = -a;
    }
}

// Warp 0: factor and invert the 8 x 8 diagonal block at Ab / Gb (pitch p):
// a_ij -= a_ik a_jk / a_kk for the pivots k (the elements of columns > k: a
// prefix of at most 28 of the block's list, one lane each), then the unit
// lower inverse x and the scalings G = x_ij / L(i, i), L = a_ij / L(j, j).
// A non-positive pivot of a real row (< nb) sets *info (first one found) and
// is carried on with a zero scale, so the launch always ends.
__device__ void diag_block(double *Ab, double *Gb, int p, double *rb, double *sb, int b0, int nb, int r, int *info) {
    const int lane = threadIdx.x % 32;
    int di, dj;
    tri_elem(lane, kDiag, di, dj);  // this lane's element of the 8 x 8 list (36 elements: 32 here)
    for (int kk = 0; kk < kDiag; ++kk) {
        __syncwarp();
        const double d = Ab[kk * p + kk];
        const bool ok = d > 0.0;
        const double rr = ok ? rsqrt(d) : 0.0, sq = rr * rr;
        if (lane == 0) {
            rb[kk] = rr;
            sb[kk] = sq;
            if (!ok && b0 + kk < nb) atomicCAS(info, 0, r + b0 + kk + 1);
        }
        const int m = kDiag - 1 - kk;  // columns kk + 1 .. 7
        if (lane < m * (m + 1) / 2)
            Ab[di * p + dj] = fma(-Ab[di * p + kk] * sq, Ab[dj * p + kk], Ab[di * p + dj]);
    }
    __syncwarp();
    for (int e = lane; e < kDiag * kDiag; e += 32) Gb[(e / kDiag) * p + e % kDiag] = (e / kDiag == e % kDiag) ? 1.0 : 0.0;
    for (int kk = 0; kk < kDiag - 1; ++kk) {  // x(i, j) -= (a_ik / a_kk) x(k, j), i > k >= j
        __syncwarp();
        if (lane < (kDiag - 1 - kk) * (kk + 1)) {
            const int i = kk + 1 + lane / (kk + 1), j = lane % (kk + 1);
            Gb[i * p + j] = fma(-Ab[i * p + kk] * sb[kk], Gb[kk * p + j], Gb[i * p + j]);
        }
    }
    __syncwarp();
    for (int e = lane; e < kDiag * (kDiag + 1) / 2; e += 32) {
        int i, j;
        tri_elem(e, kDiag, i, j);
        Gb[i * p + j] *= rb[i];
        Ab[i * p + j] *= rb[j];
    }
    __syncwarp();
}

// L = chol(A) in place and G = L^-1 for the nb x nb diagonal block at offset r
// (rows past nb padded with the identity), by 8-column blocks b:
//   panel   L_rb = A_rb G_bb^T for the rows r >= b0 + 8 below block b;
//   then, concurrently: warp 0 updates the next diagonal block with the panel
//   and factors it (diag_block); warps 1-3 and 5-7 update the rest of the
//   trailing matrix, A_rr -= L_rb L_rb^T (the columns past the next block, and
//   the next block's own rows below its diagonal block);
// and the inverse by doubling, s = 8, 16, 32: G21 = -G22 (L21 G11) for all
// pairs of s x s blocks.
template <int L>
__global__ void __launch_bounds__(kThreads) leaf_chol_inv64_kernel(double *A, double *G, int nb, int ld, int r,
                                                                   int *info) {
    constexpr int kP = L + 1;
    extern __shared__ double smem[];
    double *As = smem;                 // [L][kP], row-major: A, then L
    double *Gs = As + L * kP;          // [L][kP]: G
    double *Pn = Gs + L * kP;          // [L][kPPitch]: panel of the current block
    double *Wm = Pn + L * kPPitch;     // [leaf_wm<L>()]: L21 G11 of the doubling levels
    double *rb = Wm + leaf_wm<L>(), *sb = rb + kDiag;  // 1/L(k, k) and its square, warp 0's block
    int *tab = reinterpret_cast<int *>(sb + kDiag);  // [tri_count<L>()]: (i << 8) | j, columns from the last
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const bool other = (warp & 3) != 0;
    const int ot = other ? (warp - 1 - (warp > 4)) * 32 + lane : -1;  // 0 .. kOthers - 1
    for (int e = tid; e < L * L; e += kThreads) {
        const int i = e % L, j = e / L;
        double v = 0.0;
        if (i < nb && j < nb) {
            if (i >= j) v = A[(size_t)j * ld + i];
        } else if (i == j) {
            v = 1.0;
        }
        As[i * kP + j] = v;
        Gs[i * kP + j] = 0.0;
    }
    for (int e = tid; e < tri_count<L>(); e += kThreads) {
        int i, j;
        tri_elem(e, L, i, j);
        tab[e] = (i << 8) | j;
    }
    __syncthreads();
    if (warp == 0) diag_block(As, Gs, kP, rb, sb, 0, nb, r, info);
    __syncthreads();
    for (int b0 = 0; b0 + kDiag < L; b0 += kDiag) {
        const int r0 = b0 + kDiag, nr = L - r0;
        const double *Gb = Gs + b0 * kP + b0;
        // panel: L(i, b0 + t) = sum_{s <= t} A(i, b0 + s) G_bb(t, s), lanes along i
        for (int e = tid; e < kDiag * nr; e += kThreads) {
            const int t = e / nr, i = r0 + e % nr;
            double a = 0.0;
            for (int s = 0; s <= t; ++s) a = fma(As[i * kP + b0 + s], Gb[t * kP + s], a);
            Pn[i * kPPitch + t] = a;
        }
        __syncthreads();
        for (int e = tid; e < kDiag * nr; e += kThreads) {
            const int t = e / nr, i = r0 + e % nr;
            As[i * kP + b0 + t] = Pn[i * kPPitch + t];
        }
        if (warp == 0) {
            // the next diagonal block (rows and columns r0 .. r0 + 7), then its factor
            for (int e = lane; e < kDiag * (kDiag + 1) / 2; e += 32) {
                int i, j;
                tri_elem(e, kDiag, i, j);
                i += r0;
                j += r0;
                double a = As[i * kP + j];
#pragma unroll
                for (int t = 0; t < kDiag; ++t) a = fma(-Pn[i * kPPitch + t], Pn[j * kPPitch + t], a);
                As[i * kP + j] = a;
            }
            diag_block(As + r0 * kP + r0, Gs + r0 * kP + r0, kP, rb, sb, r0, nb, r, info);
        } else if (other) {
            // the trailing triangle of the columns past the next block
            const int m = L - r0 - kDiag, cnt = m * (m + 1) / 2;
            for (int e = ot; e < cnt; e += kOthers) {
                const int i = tab[e] >> 8, j = tab[e] & 255;
                double a = As[i * kP + j];
#pragma unroll
                for (int t = 0; t < kDiag; ++t) a = fma(-Pn[i * kPPitch + t], Pn[j * kPPitch + t], a);
                As[i * kP + j] = a;
            }
            // the next block's rows below its diagonal block (the next panel's input), lanes along i
            for (int e = ot; e < kDiag * m; e += kOthers) {
                const int j = r0 + e / m, i = r0 + kDiag + e % m;
                double a = As[i * kP + j];
#pragma unroll
                for (int t = 0; t < kDiag; ++t) a = fma(-Pn[i * kPPitch + t], Pn[j * kPPitch + t], a);
                As[i * kP + j] = a;
            }
            if constexpr (L == 64) {
                // the doubling inverse's products whose blocks are final, in the time warp 0's
                // pivot chain leaves these warps idle (b: this block; the pair (2q, 2q + 1) of
                // 8 rows, the quad of 16, the halves of 32)
                const int b = b0 / kDiag;
                double *W8 = Wm, *W16 = Wm + 4 * 64, *W32 = Wm + 4 * 64 + 2 * 256;
                if ((b & 1) == 0)  // W of pair b / 2: L21 rows are the panel's (its copy into As is in flight)
                    inv_w(Pn + (size_t)r0 * kPPitch, kPPitch, Gs, kP, W8 + (b / 2) * 64, 8, 16 * (b / 2), 0, 8, ot,
                          kOthers);
                else  // G21 of pair (b - 1) / 2: its second diagonal block was factored in the last block
                    inv_g(Gs, kP, W8 + (b / 2) * 64, 8, 16 * (b / 2), ot, kOthers);
                if (b == 2 || b == 6)  // W of quad b / 4: pairs inverted, panels final
                    inv_w(As + (size_t)(32 * (b / 4) + 16) * kP + 32 * (b / 4), kP, Gs, kP, W16 + (b / 4) * 256, 16,
                          32 * (b / 4), 0, 16, ot, kOthers);
                if (b == 4)  // G21 of quad 0
                    inv_g(Gs, kP, W16, 16, 0, ot, kOthers);
                if (b >= 5)  // W of the halves, columns 0-15 then 16-31: the first half is inverted
                    inv_w(As + (size_t)32 * kP, kP, Gs, kP, W32, 32, 0, 16 * (b - 5), 16 * (b - 4), ot, kOthers);
            }
        }
        __syncthreads();
    }
    if constexpr (L == 64) {  // the doubling inverse's last products (their other halves ran in the loop)
        inv_g(Gs, kP, Wm + 3 * 64, 8, 48, tid, kThreads);  // pair 3
        __syncthreads();
        inv_g(Gs, kP, Wm + 4 * 64 + 256, 16, 32, tid, kThreads);  // quad 1
        __syncthreads();
        inv_g(Gs, kP, Wm + 4 * 64 + 2 * 256, 32, 0, tid, kThreads);  // the halves
        __syncthreads();
    } else
    for (int s = kDiag; s < L; s *= 2) {  // inverse by doubling
        const int per = s * s, count = (L / (2 * s)) * per;
        // W = L21 G11 (G11 lower: t >= j), lanes along i: equal trips s - j
        for (int e = tid; e < count; e += kThreads) {
            const int blk = e / per, o = 2 * s * blk, j = (e % per) / s, i = e % s;
            double a = 0.0;
            for (int t = j; t < s; ++t) a = fma(As[(o + s + i) * kP + o + t], Gs[(o + t) * kP + o + j], a);
            Wm[blk * per + i * s + j] = a;
        }
        __syncthreads();
        // G21 = -G22 W (G22 lower: t <= i), lanes along j: equal trips i + 1
        for (int e = tid; e < count; e += kThreads) {
            const int blk = e / per, o = 2 * s * blk, i = (e % per) / s, j = e % s;
            const double *W = Wm + blk * per;
            double a = 0.0;
            for (int t = 0; t <= i; ++t) a = fma(Gs[(o + s + i) * kP + o + s + t], W[t * s + j], a);
            Gs[(o + s + i) * kP + o + j] = -a;
        }
        __syncthreads();
    }
    for (int e = tid; e < L * L; e += kThreads) {
        const int i = e % L, j = e / L;
        if (i < nb && j < nb) {
            const bool low = i >= j;
            G[(size_t)j * ld + i] = low ? Gs[i * kP + j] : 0.0;
            A[(size_t)j * ld + i] = low ? As[i * kP + j] : 0.0;
        }
    }
}

}  // namespace

int leaf_rows() { return kLeafRows; }

cudaError_t leaf_chol_inv64(double *A, double *G, int nb, int ld, int row0, int *info, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(leaf_chol_inv64_kernel<kLeafRows>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)leaf_smem<kLeafRows>());
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (nb <= 0 || nb > kLeafRows) return cudaErrorInvalidValue;
    leaf_chol_inv64_kernel<kLeafRows><<<1, kThreads, leaf_smem<kLeafRows>(), st>>>(A, G, nb, ld, row0, info);
    count_launch();
    return cudaGetLastError();
}

}  // namespace elhl
