// FP64 matrix products on the tensor cores by exact BF16 slices (Ozaki scheme
// I: Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59, 2012):
//
//   C = alpha op(A) op(B) + beta C   (column-major, the conventions and
//                                     triangular flags of dgemm64)
//
// Every row of op(A) and every column of op(B) is cut into kS = 7 slices of 8
// bits on a power-of-two scale of its largest element (slice7: |n_0| <= 256,
// |n_s| <= 128 after it), each exact in BF16.  The slice products with s_a + s_b = d are
// accumulated together in FP32 in tensor memory over one 64-K block: a k adds
// at most 2^17.2 in magnitude to any weight d, so 64 of them stay below 2^24
// and the FP32 sums are exact integers.  After each block the seven weights
// (d <= 6; the rest lie below 2^-64 of the scales) are folded into two 64-bit
// integers per output, H = sum_{d<=2} acc_d 2^(8 (2 - d)) and L = sum_{d>=3}
// acc_d 2^(8 (6 - d)), exactly; the output is 2^-64 (2^32 H + L) times the two
// scales, rounded once to FP64.  The FP64 pipe (1.2 TFLOP/s on GB300) is left
// for the small products; this kernel runs the large ones on the BF16 tensor
// pipe with 28 slice products per FP64 product.
//
// One CTA computes a 128 x 32 tile of C over the tile's non-zero K blocks:
//   warp 0     TMA producer: per 64-K block the 7 op(B) slices (32 x 64 each) into
//              a B stage, then the 7 op(A) slices (128 x 64) into a ring of A stages;
//   warp 1     allocates TMEM; one thread issues tcgen05.mma (M = 128, K = 16)
//              of A slice a against the B slices b <= 6 - a at once (N = 32 (7 - a),
//              D from column 32 a, so that B slice b lands on the weight
//              accumulator a + b) in one of two 224-column buffers;
//   warps 2-5  fold each block's accumulators into H and L (one thread per row)
//              and write C.
// Operands are sliced by oz_partmax_kernel and oz_slice_kernel beforehand
// (K-major, zero outside the triangle a flag names).  Every wait is bounded (ELHL_ERR_TIMEOUT).
#include <cuda.h>

#include <algorithm>

#include "elhl_internal.cuh"
#include "tc_ptx.cuh"

namespace elhl {
namespace {

using namespace tc;

constexpr int kS = 7;
constexpr int kTM = 128, kTN = 32, kKB = 64;
constexpr int kAStages = 8;
constexpr int kBStages = 2;
constexpr int kThreads = 192;
constexpr int kATile = kTM * kKB * 2;       // 16 KB
constexpr int kBSlice = kTN * kKB * 2;      // 4 KB
constexpr int kBStage = kS * kBSlice;       // 28 KB
constexpr int kAccCols = kS * kTN;          // 224 TMEM columns: one 32-column accumulator per weight
constexpr unsigned long long kWaitNs = 2000000000ull;

struct Smem {
    static constexpr size_t a_off = 0;
    static constexpr size_t b_off = (size_t)kAStages * kATile;
    static constexpr size_t bar_off = b_off + (size_t)kBStages * kBStage;
    static constexpr size_t n_bars = 2 * kAStages + 2 * kBStages + 2 + 2 + 1;
    static constexpr size_t misc_off = bar_off + n_bars * 8;
    static constexpr size_t bytes = misc_off + 64;
};

__device__ __forceinline__ double pow2(int e) { return __longlong_as_double((long long)(1023 + e) << 52); }
__device__ __forceinline__ int scale_exp(double x) {  // |x| < 2^e for the finite x > 0 (0 for x = 0)
    if (!(x > 0.0)) return 0;
    return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1022;
}

// element (r, j) of an operand row: row r of op(A) (or column r of op(B)), j the K index
struct OperandView {
    const double *X;
    int ld;
    bool kcontig;  // the K index runs along X's columns (X[j + r ld]) instead of its rows (X[r + j ld])
    int rows, k;
    int mask;      // 0: all; 1: zero for j > r; 2: zero for j < r
    int tile;      // rows of the operand per output tile of the product (kTM for op(A), kTN for op(B)^T)
};

// The K range [lo, hi) the product reads for the rows of the output tile that
// holds row r: the triangular mask of the tile's rows cut out to whole 64-K
// blocks, as ozgemm_kernel's k range does.  Slices outside it are never read,
// so the slicing kernels skip them (they are zero there in any case).
__device__ __forceinline__ void read_range(const OperandView &v, int r, int &lo, int &hi) {
    const int t0 = r / v.tile * v.tile;
    lo = v.mask == 2 ? t0 / kKB * kKB : 0;
    hi = v.mask == 1 ? (min(v.k, t0 + v.tile) + kKB - 1) / kKB * kKB : 1 << 30;
}

// 32 x 32 tile of the operand rows [r0, r0+32) x K [j0, j0+32) in shared memory
// (t[rr][jj]), loaded along X's contiguous index; masked and out-of-range entries 0
__device__ __forceinline__ void load_tile(const OperandView &v, int r0, int j0, double (&t)[32][33]) {
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        int r, j;
        if (v.kcontig) {
            r = r0 + q;
            j = j0 + threadIdx.x;
        } else {
            r = r0 + threadIdx.x;
            j = j0 + q;
        }
        double x = 0.0;
        const bool keep = r < v.rows && j < v.k && !(v.mask == 1 && j > r) && !(v.mask == 2 && j < r);
        if (keep) x = v.kcontig ? v.X[(size_t)r * v.ld + j] : v.X[(size_t)j * v.ld + r];
        if (v.kcontig) t[q][threadIdx.x] = x;
        else t[threadIdx.x][q] = x;
    }
}

// Slicing of both operands in two passes over pieces of 32 operand rows x
// chunk K (blockIdx.z: 0 = op(A), 1 = op(B)^T), tiles of 32 x 32 loaded along
// X's contiguous index: oz_partmax_kernel writes each row's largest |element|
// of the piece to pm[r][piece]; oz_slice_kernel reduces a row's pieces to its
// scale 2^e_r (scale[r], written by the pieces at K = 0) and cuts every element
// of its piece with slice7 into out[s][r][j] (row stride kp, zero for k <= j < kp).
// The piece is 256 K, or 128 / 64 for K up to 1024 / 512: a piece's tiles run one
// after another, so short operands take more, shorter pieces (more CTAs, each
// with fewer dependent tile loads).
__host__ __device__ constexpr int slice_chunk(int kp) { return kp <= 512 ? 64 : kp <= 1024 ? 128 : 256; }

__global__ void __launch_bounds__(256) oz_partmax_kernel(OperandView va, OperandView vb, double *pmA, double *pmB,
                                                         int npiece, int chunk) {
    __shared__ double t[32][33];
    const bool isB = blockIdx.z == 1;
    const OperandView &v = isB ? vb : va;
    const int r0 = blockIdx.y * 32, j00 = blockIdx.x * chunk;
    if (r0 >= v.rows) return;
    int lo, hi;  // the same for the 32 rows: they lie in one output tile
    read_range(v, r0, lo, hi);
    double mx = 0.0;  // thread (x, y): row r0 + x over K columns y, y + 8, ... of each tile
    for (int j0 = j00; j0 < min(v.k, j00 + chunk); j0 += 32) {
        if (j0 >= hi || j0 + 32 <= lo) continue;  // masked out: zero (uniform over the block)
        __syncthreads();
        load_tile(v, r0, j0, t);
        __syncthreads();
        for (int q = threadIdx.y; q < 32; q += 8) mx = fmax(mx, fabs(t[threadIdx.x][q]));
    }
    __shared__ double s_max[8][32];
    s_max[threadIdx.y][threadIdx.x] = mx;
    __syncthreads();
    if (threadIdx.y == 0 && r0 + threadIdx.x < v.rows) {
        double m = s_max[0][threadIdx.x];
        for (int q = 1; q < 8; ++q) m = fmax(m, s_max[q][threadIdx.x]);
        (isB ? pmB : pmA)[(size_t)(r0 + threadIdx.x) * npiece + blockIdx.x] = m;
    }
}

__global__ void __launch_bounds__(256) oz_slice_kernel(OperandView va, OperandView vb, const double *pmA,
                                                       const double *pmB, int npiece, __nv_bfloat16 *outA,
                                                       __nv_bfloat16 *outB, int kp, double *scA, double *scB,
                                                       int chunk) {
    __shared__ double t[32][33];
    __shared__ int s_e[32];
    const bool isB = blockIdx.z == 1;
    const OperandView &v = isB ? vb : va;
    const double *pm = isB ? pmB : pmA;
    __nv_bfloat16 *out = isB ? outB : outA;
    const int r0 = blockIdx.y * 32, j00 = blockIdx.x * chunk;
    if (r0 >= v.rows) return;
    if (threadIdx.y == 0) {
        const int r = r0 + threadIdx.x;
        double m = 0.0;
        if (r < v.rows)
            for (int q = 0; q < npiece; ++q) m = fmax(m, pm[(size_t)r * npiece + q]);
        const int e = scale_exp(m);
        s_e[threadIdx.x] = e;
        if (blockIdx.x == 0 && r < v.rows) (isB ? scB : scA)[r] = pow2(e);
    }
    const size_t sstride = (size_t)v.rows * kp;
    int lo, hi;  // the same for the 32 rows: they lie in one output tile
    read_range(v, r0, lo, hi);
    for (int j0 = j00; j0 < min(kp, j00 + chunk); j0 += 32) {
        if (j0 >= hi || j0 + 32 <= lo) continue;  // never read by the product (uniform over the block)
        __syncthreads();
        load_tile(v, r0, j0, t);
        __syncthreads();
        for (int rr = threadIdx.y; rr < 32; rr += 8) {
            const int r = r0 + rr, j = j0 + threadIdx.x;
            if (r >= v.rows || j >= kp) continue;
            int dig[kS];
            slice7(t[rr][threadIdx.x], s_e[rr], dig);
#pragma unroll
            for (int sl = 0; sl < kS; ++sl) out[sl * sstride + (size_t)r * kp + j] = __float2bfloat16_rn((float)dig[sl]);
        }
    }
}

struct OzGemmArgs {
    int m, n, k;
    double alpha, beta;
    double *C;
    int ldc, tri;
    int gx, gy;               // tiles along rows and columns
    const double *rs, *cs;    // row scales of op(A), column scales of op(B)
    int *error;
};

__global__ void __launch_bounds__(kThreads, 1)
    ozgemm_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, OzGemmArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // tile, longest k ranges first (kTriA: the last row tiles; kTriBt: the last column tiles)
    const int bx0 = blockIdx.x % g.gx, by0 = blockIdx.x / g.gx;
    const int bx = (g.tri & kTriA) ? g.gx - 1 - bx0 : bx0;
    const int by = (g.tri & kTriBt) ? g.gy - 1 - by0 : by0;
    const int i0 = bx * kTM, j0 = by * kTN;
    if ((g.tri & kTriLowerC) && i0 + kTM <= j0) return;  // tile strictly above the diagonal
    int klo = 0, khi = g.k;
    if (g.tri & kTriA) khi = min(khi, i0 + kTM);    // op(A)(i, l) = A(i, l) = 0 for l > i
    if (g.tri & kTriAt) klo = max(klo, i0);         // op(A)(i, l) = A(l, i) = 0 for l < i
    if (g.tri & kTriB) klo = max(klo, j0);          // op(B)(l, j) = B(l, j) = 0 for l < j
    if (g.tri & kTriBt) khi = min(khi, j0 + kTN);   // op(B)(l, j) = B(j, l) = 0 for l > j
    const int kb0 = klo / kKB, kb1 = khi > klo ? (khi + kKB - 1) / kKB : kb0;

    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                            ~static_cast<uintptr_t>(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + Smem::bar_off);
    uint64_t *full = bars, *empty = full + kAStages, *bfull = empty + kAStages, *bempty = bfull + kBStages;
    uint64_t *accfull = bempty + kBStages, *accempty = accfull + 2, *done = accempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + Smem::misc_off);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
    unsigned *flag = reinterpret_cast<unsigned *>(tmem_slot + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kAStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int s = 0; s < kBStages; ++s) {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(&accfull[s], 1);
            mbar_init(&accempty[s], 128);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    unsigned issued = 0;  // A stages loaded (producer)

    if (warp == 0 && lane == 0) {
        // ---- TMA producer
        unsigned acnt = 0;
        for (int kb = kb0, bi = 0; kb < kb1; ++kb, ++bi) {
            const int sb = bi % kBStages;
            if (bi >= kBStages && !mbar_wait(&bempty[sb], ((bi / kBStages) - 1) & 1, now_ns(), kWaitNs)) {
                atomicExch(abort_flag, 1);
                break;
            }
            if (*(volatile int *)abort_flag) break;
            mbar_expect_tx(&bfull[sb], (unsigned)kBStage);
            for (int b = 0; b < kS; ++b)
                tma_load_3d(smem + Smem::b_off + (size_t)sb * kBStage + (size_t)b * kBSlice, &mB, &bfull[sb],
                            kb * kKB, j0, b);
            bool stop = false;
            for (int a = 0; a < kS; ++a) {
                const unsigned s = acnt % kAStages;
                if (acnt >= kAStages && !mbar_wait(&empty[s], ((acnt / kAStages) - 1) & 1, now_ns(), kWaitNs)) {
                    atomicExch(abort_flag, 1);
                    stop = true;
                    break;
                }
                mbar_expect_tx(&full[s], (unsigned)kATile);
                tma_load_3d(smem + Smem::a_off + (size_t)s * kATile, &mA, &full[s], kb * kKB, i0, a);
                ++acnt;
            }
            if (stop) break;
        }
        issued = acnt;
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer
        unsigned acnt = 0;
        for (int kb = kb0, bi = 0; kb < kb1; ++kb, ++bi) {
            const unsigned tb = bi & 1, sb = bi % kBStages;
            if (bi >= 2 && !mbar_wait(&accempty[tb], ((bi >> 1) - 1) & 1, now_ns(), kWaitNs)) {
                atomicExch(abort_flag, 1);
                break;
            }
            if (!mbar_wait(&bfull[sb], (bi / kBStages) & 1, now_ns(), kWaitNs)) {
                atomicExch(abort_flag, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            bool stop = false;
            for (int a = 0; a < kS; ++a) {
                const unsigned s = acnt % kAStages;
                if (!mbar_wait(&full[s], (acnt / kAStages) & 1, now_ns(), kWaitNs)) {
                    atomicExch(abort_flag, 1);
                    stop = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                // one MMA of A slice a against the B slices 0 .. 6 - a, which lie one after
                // another in the stage (32 rows each): column block b of its D lands on
                // weight a + b at TMEM column 32 (a + b); N = 32 (7 - a)
                const uint64_t da = smem_desc_sw128(smem + Smem::a_off + (size_t)s * kATile);
                const uint64_t db = smem_desc_sw128(smem + Smem::b_off + (size_t)sb * kBStage);
                const uint32_t acc = tmem + tb * kAccCols + (uint32_t)(a * kTN);
                const uint32_t idesc = idesc_bf16(kTM, kTN * (kS - a));
#pragma unroll
                for (int k = 0; k < kKB / 16; ++k)  // the first MMA (a = 0: all weights) starts the block
                    umma_bf16(acc, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), idesc, !(a == 0 && k == 0));
                umma_commit(&empty[s]);
                ++acnt;
            }
            if (stop) break;
            umma_commit(&bempty[sb]);
            umma_commit(&accfull[tb]);
        }
    } else if (warp >= 2) {
        // ---- fold the weights of each block into H and L, then write C
        const int t = threadIdx.x - 64;          // 0 .. 127
        const int quad = warp & 3;               // TMEM lanes [32 quad, 32 quad + 32)
        const int row = i0 + quad * 32 + lane;
        long long H[kTN], L[kTN];
#pragma unroll
        for (int c = 0; c < kTN; ++c) {
            H[c] = 0;
            L[c] = 0;
        }
        bool ok = true;
        for (int bi = 0; bi < kb1 - kb0; ++bi) {
            const unsigned tb = bi & 1;
            if (t == 0) *flag = mbar_wait(&accfull[tb], (bi >> 1) & 1, now_ns(), kWaitNs) ? 1u : 0u;
            asm volatile("bar.sync 1, 128;" ::: "memory");
            ok = *(volatile unsigned *)flag != 0;
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (!ok) {
                if (t == 0) atomicExch(abort_flag, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + tb * kAccCols;
#pragma unroll
            for (int d = 0; d < kS; ++d) {
                uint32_t v[32];
                tmem_ld32(taddr + (uint32_t)(d * kTN), v);
                tmem_wait_ld();
#pragma unroll
                for (int c = 0; c < kTN; ++c) {
                    const long long x = (long long)__float2int_rn(__uint_as_float(v[c]));
                    if (d <= 2) H[c] += x * (1ll << (8 * (2 - d)));
                    else L[c] += x * (1ll << (8 * (kS - 1 - d)));
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            mbar_arrive(&accempty[tb]);
        }
        if (ok && row < g.m) {
            const double rs = g.rs[row] * pow2(-64);
#pragma unroll
            for (int c = 0; c < kTN; ++c) {
                const int col = j0 + c;
                if (col >= g.n) continue;
                const double val = ((double)H[c] * 0x1p32 + (double)L[c]) * rs * g.cs[col];
                double *cp = g.C + (size_t)col * g.ldc + row;
                *cp = g.beta == 0.0 ? g.alpha * val : fma(g.alpha, val, g.beta * *cp);
            }
        }
    }
    // drain: loads and MMAs complete before the CTA frees its TMEM and leaves
    if (warp == 0 && lane == 0) {
        const unsigned n = min(issued, (unsigned)kAStages);
        for (unsigned q = issued - n; q < issued; ++q) mbar_wait(&full[q % kAStages], (q / kAStages) & 1, now_ns(), kWaitNs);
    }
    if (warp == 1 && lane == 0) {
        umma_commit(done);
        mbar_wait(done, 0, now_ns(), kWaitNs);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (threadIdx.x == 0 && *(volatile int *)abort_flag) atomicExch(g.error, (int)ELHL_ERR_TIMEOUT);
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// slices [kS][rows][kp] BF16: x = K, y = row, z = slice; box 64 x box_rows x 1, 128B swizzle
bool make_map(CUtensorMap *m, const __nv_bfloat16 *base, int rows, int kp, int box_rows) {
    EncodeTiled fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)kp, (cuuint64_t)rows, (cuuint64_t)kS};
    const cuuint64_t strides[2] = {(cuuint64_t)kp * 2, (cuuint64_t)kp * rows * 2};
    const cuuint32_t box[3] = {(cuuint32_t)kKB, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// per-lane workspace: slices of op(A) and op(B)^T, their maxima and scales, the error word
struct Lane {
    __nv_bfloat16 *sl = nullptr;
    size_t sl_elems = 0;
    double *sc = nullptr;
    size_t rows_cap = 0;
    double *pm = nullptr;    // row maxima per K piece of both operands
    size_t pm_cap = 0;
    int *err = nullptr;
};
Lane g_lane[2];

cudaError_t ensure(Lane &ln, size_t sl_elems, size_t rows) {
    if (!ln.err) {
        cudaError_t e = cudaMalloc(&ln.err, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(ln.err, 0, sizeof(int));
        if (e != cudaSuccess) return e;
    }
    if (sl_elems > ln.sl_elems) {
        if (ln.sl) cudaFree(ln.sl);
        ln.sl = nullptr;
        ln.sl_elems = 0;
        cudaError_t e = cudaMalloc(&ln.sl, sl_elems * sizeof(__nv_bfloat16));
        if (e != cudaSuccess) return e;
        ln.sl_elems = sl_elems;
    }
    if (rows > ln.rows_cap) {
        if (ln.sc) cudaFree(ln.sc);
        ln.sc = nullptr;
        ln.rows_cap = 0;
        cudaError_t e = cudaMalloc(&ln.sc, rows * sizeof(double));
        if (e != cudaSuccess) return e;
        ln.rows_cap = rows;
    }
    return cudaSuccess;
}

cudaError_t ensure_pm(Lane &ln, size_t n) {
    if (n <= ln.pm_cap) return cudaSuccess;
    if (ln.pm) cudaFree(ln.pm);
    ln.pm = nullptr;
    ln.pm_cap = 0;
    cudaError_t e = cudaMalloc(&ln.pm, n * sizeof(double));
    if (e == cudaSuccess) ln.pm_cap = n;
    return e;
}

}  // namespace

size_t ozgemm_smem_bytes() { return 1024 + Smem::bytes; }

cudaError_t ozgemm(int m, int n, int k, double alpha, const double *A, int lda, bool transA, const double *B, int ldb,
                   bool transB, double beta, double *C, int ldc, cudaStream_t st, int tri, int lane) {
    if (m <= 0 || n <= 0) return cudaSuccess;
    if (lane < 0 || lane > 1 || k <= 0) return cudaErrorInvalidValue;
    Lane &ln = g_lane[lane];
    const int kp = round_up(k, 8);  // 16-byte row stride of the slices
    // op(A) rows: A(i, l) (K along A's rows) or A^T: A(l, i) (K along A's columns)
    const OperandView va{A, lda, transA, m, k, (tri & kTriA) ? 1 : (tri & kTriAt) ? 2 : 0, kTM};
    // op(B) columns: B(l, j) (K along B's columns) or B^T: B(j, l) (K along B's rows)
    const OperandView vb{B, ldb, !transB, n, k, (tri & kTriB) ? 2 : (tri & kTriBt) ? 1 : 0, kTN};
    // op(B) = op(A)^T (the Schur update L21 L21^T): op(B)^T has op(A)'s rows, so
    // one set of slices and scales serves both operands
    const bool same = A == B && lda == ldb && va.kcontig == vb.kcontig && m == n && va.mask == vb.mask;
    const size_t sa = (size_t)kS * m * kp, sb = same ? 0 : (size_t)kS * n * kp;
    if (cudaError_t e = ensure(ln, sa + sb, (size_t)m + n)) return e;
    __nv_bfloat16 *slA = ln.sl, *slB = same ? ln.sl : ln.sl + sa;  // sa is a multiple of 8 elements: 16-byte aligned
    double *scB = same ? ln.sc : ln.sc + m;
    const int chunk = slice_chunk(kp), npiece = (kp + chunk - 1) / chunk;
    if (cudaError_t e = ensure_pm(ln, (size_t)(m + n) * npiece)) return e;
    const dim3 grid(npiece, (std::max(m, n) + 31) / 32, same ? 1 : 2), blk(32, 8);
    oz_partmax_kernel<<<grid, blk, 0, st>>>(va, vb, ln.pm, ln.pm + (size_t)m * npiece, npiece, chunk);
    count_launch();
    oz_slice_kernel<<<grid, blk, 0, st>>>(va, vb, ln.pm, ln.pm + (size_t)m * npiece, npiece, slA, slB, kp, ln.sc,
                                          ln.sc + m, chunk);
    count_launch();
    CUtensorMap ma, mb;
    if (!make_map(&ma, slA, m, kp, kTM) || !make_map(&mb, slB, n, kp, kTN)) return cudaErrorInvalidValue;
    const size_t smem = ozgemm_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(ozgemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    OzGemmArgs g{m, n, k, alpha, beta, C, ldc, tri, (m + kTM - 1) / kTM, (n + kTN - 1) / kTN, ln.sc, scB, ln.err};
    ozgemm_kernel<<<g.gx * g.gy, kThreads, smem, st>>>(ma, mb, g);
    count_launch();
    return cudaGetLastError();
}

int *ozgemm_error(int lane) { return lane >= 0 && lane < 2 ? g_lane[lane].err : nullptr; }

}  // namespace elhl
