// FP64 Chebyshev propagation on the tensor cores by exact BF16 slices
// (Ozaki scheme I: Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59, 2012).
//
// GB300 runs FP64 FMAs at 1/58 of its FP32 rate, so the FP64 propagation on
// the FP64 pipe is bound by that pipe (1.2 TFLOP/s), not by HBM.  Here every
// FP64 operand is cut into kS = 7 slices of 8 bits each on a power-of-two
// scale shared by a matrix row or a vector column (slice7):
//
//   a = 2^e_row  sum_{s<7} n_s 2^(-8(s+1)),   n_s integers, |n_0| <= 256, |n_s| <= 128,
//
// which represents a to 2^-57 relative to its row's largest element.  Each
// n_s is exact in BF16, each product of two slices is an integer below 2^16,
// and a sum of 256 of them is an integer below 2^24: a BF16 tcgen05.mma with
// FP32 accumulation therefore computes every slice product exactly, as long
// as no accumulation runs over more than K = 256.  The products with
// s_a + s_b <= 6 (28 of the 49; the rest lie below 2^-64) are taken from TMEM
// after every 256-K group, converted to integers and added, shifted by their
// weight 2^-8(s_a+s_b+2), into one 128-bit integer per row and column: a CTA's
// partial product is exact until its single rounding to FP64.  The operator is
// read as 14 bytes per element (7 BF16 slices) instead of 8, but the work
// moves from the FP64 pipe to the tensor pipe, which leaves HBM as the bound.
//
// One cooperative launch runs every order of one nuclear step.  An order is 1
// (explicit Hs) or 3 (implicit G (h/b) G^T) grid phases y = A x, A a row-scaled
// sliced matrix and x the FP64 output of the previous phase.  A phase's work
// is a list of 64-K blocks of 128-row tiles (the non-zero ones of a triangular
// A), split evenly over the CTAs; a CTA's blocks form segments (runs within a
// row tile).  Per CTA:
//   warp 0     TMA producer: the 7 slices of each block (128 x 64 BF16, 16 KB,
//              128B swizzle) into a ring of kAStages stages;
//   warp 1     allocates TMEM; one thread issues tcgen05.mma (M = 128, K = 16,
//              N = 64 ... 16: slice s_a against the vector slices s_b <= 6 - s_a)
//              into one of two 256-column accumulator buffers;
//   warps 2-3  build the vector operand of each block: 64 rows x 8 real columns
//              of x cut into 7 slices, written in the swizzled K-major layout;
//   warps 4-7  flush each 256-K group from TMEM (one thread per row), and at
//              the end of a segment store the 128 x 8 FP64 partial; the last
//              segment of a row tile to finish sums the partials in segment
//              order (deterministic) and applies the phase epilogue: store w or
//              y, or the Chebyshev recurrence and c_k v_k accumulation.
// The column scales of x come from an integer max over the bits of |x| taken
// by the producing epilogue.  Every wait is bounded: on a timeout the CTA sets
// ELHL_ERR_TIMEOUT, stops, waits for its own copies and MMAs, and frees TMEM.
#include <cuda.h>

#include <algorithm>

#include "elhl_internal.cuh"
#include "grid_sync.cuh"
#include "tc_ptx.cuh"

namespace elhl {
namespace {

using namespace tc;

constexpr int kS = 7;                 // slices per operand
constexpr int kTileM = 128;           // rows per tile (MMA M)
constexpr int kKB = 64;               // K per block: 64 BF16 = one 128-byte swizzled row
constexpr int kGroupBlocks = 4;       // blocks per exact accumulation (K = 256)
constexpr int kAStages = 10;
constexpr int kBStages = 4;
constexpr int kThreads = 256;
constexpr int kATile = kTileM * kKB * 2;  // 16 KB
constexpr int kBTile = 64 * kKB * 2;      // 8 KB: 8 slots of 8 real columns (slot 7 stays zero)
constexpr int kAccCols = 256;             // TMEM columns per accumulator buffer
constexpr unsigned long long kWaitNs = 2000000000ull;

// TMEM column offset and MMA N of matrix slice a: its valid columns are the
// 8 (7 - a) real columns of the vector slices b <= 6 - a, rounded up to 16
__host__ __device__ constexpr int acc_n(int a) { return ((8 * (kS - a) + 15) / 16) * 16; }
__host__ __device__ constexpr int acc_off(int a) {  // sum of acc_n(t) for t < a, written out so it folds
    return a <= 0 ? 0 : a == 1 ? 64 : a == 2 ? 112 : a == 3 ? 160 : a == 4 ? 192 : a == 5 ? 224 : a == 6 ? 240 : 256;
}
constexpr bool acc_layout_ok() {
    for (int a = 0, off = 0; a <= kS; off += a < kS ? acc_n(a) : 0, ++a)
        if (acc_off(a) != off) return false;
    return true;
}
static_assert(kS == 7 && acc_layout_ok() && acc_off(kS) == kAccCols, "accumulator layout");
// matrix slice whose accumulator holds TMEM column col of a buffer
__host__ __device__ constexpr int acc_slice(int col) {
    return col >= 240 ? 6 : col >= 224 ? 5 : col >= 192 ? 4 : col >= 160 ? 3 : col >= 112 ? 2 : col >= 64 ? 1 : 0;
}

__device__ __forceinline__ double pow2(int e) {  // 2^e for |e| < 1000
    return __longlong_as_double((long long)(1023 + e) << 52);
}
// column maximum written by atomics of other CTAs (read past L1)
__device__ __forceinline__ double col_max(const unsigned long long *cmax, int c) {
    return __longlong_as_double(__ldcg(reinterpret_cast<const long long *>(cmax) + c));
}
// exponent e with |x| < 2^e for the non-zero finite x = max |column| (0 for x = 0)
__device__ __forceinline__ int scale_exp(double x) {
    if (!(x > 0.0)) return 0;
    return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1022;
}

struct SmemLayout {
    static constexpr size_t a_off = 0;
    static constexpr size_t b_off = a_off + (size_t)kAStages * kATile;
    static constexpr size_t bar_off = b_off + (size_t)kBStages * kBTile;
    static constexpr size_t n_bars = 2 * kAStages + 2 * kBStages + 2 + 2 + 1;
    static constexpr size_t misc_off = bar_off + n_bars * 8;
    static constexpr size_t bytes = misc_off + 64;
};

struct Roles {  // counters every role advances in the same order
    unsigned acnt = 0;   // A stages
    unsigned bcnt = 0;   // B stages
    unsigned gcnt = 0;   // 256-K groups
};

struct Ctx {
    unsigned char *smem;
    uint64_t *full, *empty, *bfull, *bempty, *accfull, *accempty, *done;
    uint32_t tmem;
    int *abort_flag;
    unsigned *last_flag;
};

__device__ __forceinline__ bool aborted(const Ctx &c) { return *(volatile int *)c.abort_flag != 0; }
__device__ __forceinline__ void set_abort(const Ctx &c, int *err) {
    atomicExch(c.abort_flag, 1);
    atomicExch(err, (int)ELHL_ERR_TIMEOUT);
}

// The bounded grid barrier of grid_sync.cuh among the 192 threads of warps 2-7
// (named barrier 2) instead of the whole CTA: thread 64 arrives for the CTA.
__device__ __forceinline__ bool grid_barrier_sub(unsigned *count, unsigned *gen, unsigned nblocks, int *err,
                                                 unsigned long long limit_ns) {
    asm volatile("bar.sync 2, 192;" ::: "memory");
    if (threadIdx.x == 64) {
        volatile unsigned *vgen = gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned prev = atomicAdd(count, 1u);
        if (prev == nblocks - 1) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            const unsigned long long t0 = globaltimer_ns();
            while (*vgen == g) {
                if (globaltimer_ns() - t0 > limit_ns) {
                    atomicExch(err, ELHL_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(40);
            }
        }
        __threadfence();
    }
    asm volatile("bar.sync 2, 192;" ::: "memory");
    return *(volatile int *)err == 0;
}

// ---- phase roles ----------------------------------------------------------------

__device__ void produce(const Ctx &c, const OzLaunch &L, const CUtensorMap *map, int sched, Roles &r) {
    const int s0 = L.seg_begin[sched][blockIdx.x], s1 = L.seg_begin[sched][blockIdx.x + 1];
    for (int q = s0; q < s1; ++q) {
        const OzSeg sg = L.segs[sched][q];
        for (int kb = sg.kb0; kb < sg.kb1; ++kb) {
            for (int a = 0; a < kS; ++a) {
                const unsigned s = r.acnt % kAStages;
                if (r.acnt >= kAStages && !mbar_wait(&c.empty[s], ((r.acnt / kAStages) - 1) & 1, now_ns(), kWaitNs)) {
                    set_abort(c, L.error);
                    return;
                }
                if (aborted(c)) return;
                mbar_expect_tx(&c.full[s], (unsigned)kATile);
                tma_load_3d(c.smem + SmemLayout::a_off + (size_t)s * kATile, map, &c.full[s], kb * kKB,
                            sg.rt * kTileM, a);
                ++r.acnt;
            }
        }
    }
}

__device__ void issue_mma(const Ctx &c, const OzLaunch &L, int sched, Roles &r) {
    const int s0 = L.seg_begin[sched][blockIdx.x], s1 = L.seg_begin[sched][blockIdx.x + 1];
    for (int q = s0; q < s1; ++q) {
        const OzSeg sg = L.segs[sched][q];
        for (int kb = sg.kb0; kb < sg.kb1; ++kb) {
            const int kin = (kb - sg.kb0) % kGroupBlocks;
            const bool first = kin == 0, last = kin == kGroupBlocks - 1 || kb == sg.kb1 - 1;
            const unsigned tb = r.gcnt & 1;
            if (first && r.gcnt >= 2 && !mbar_wait(&c.accempty[tb], ((r.gcnt >> 1) - 1) & 1, now_ns(), kWaitNs)) {
                set_abort(c, L.error);
                return;
            }
            const unsigned sb = r.bcnt % kBStages;
            if (!mbar_wait(&c.bfull[sb], (r.bcnt / kBStages) & 1, now_ns(), kWaitNs)) {
                set_abort(c, L.error);
                return;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint64_t db = smem_desc_sw128(c.smem + SmemLayout::b_off + (size_t)sb * kBTile);
#pragma unroll
            for (int a = 0; a < kS; ++a) {
                const unsigned s = r.acnt % kAStages;
                if (!mbar_wait(&c.full[s], (r.acnt / kAStages) & 1, now_ns(), kWaitNs)) {
                    set_abort(c, L.error);
                    return;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint64_t da = smem_desc_sw128(c.smem + SmemLayout::a_off + (size_t)s * kATile);
                const uint32_t acc = c.tmem + tb * kAccCols + (uint32_t)acc_off(a);
                const uint32_t idesc = idesc_bf16(kTileM, acc_n(a));
#pragma unroll
                for (int k = 0; k < kKB / 16; ++k)  // K = 16 per MMA: +32 bytes along the swizzled row
                    umma_bf16(acc, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), idesc, !(first && k == 0));
                umma_commit(&c.empty[s]);  // the A stage is free once these MMAs have read it
                ++r.acnt;
            }
            umma_commit(&c.bempty[sb]);
            ++r.bcnt;
            if (last) {
                umma_commit(&c.accfull[tb]);
                ++r.gcnt;
            }
        }
    }
}

// vector operand of one block: rows kb*64 .. +64 of x ([ld][8] FP64), column c
// cut into slices b on the scale 2^e_c; slice b, column c is row 8 b + c of the
// K-major tile (128 B per row, 16-byte chunk j stored at j ^ (row & 7))
__device__ void build(const Ctx &c, const OzLaunch &L, int sched, const double *x, const unsigned long long *cmax,
                      Roles &r) {
    const int t = threadIdx.x - 64;  // 0 .. 63
    const int col = t & 7, chunk = t >> 3;
    const double inv = pow2(-scale_exp(col_max(cmax, col)));
    const int s0 = L.seg_begin[sched][blockIdx.x], s1 = L.seg_begin[sched][blockIdx.x + 1];
    for (int q = s0; q < s1; ++q) {
        const OzSeg sg = L.segs[sched][q];
        for (int kb = sg.kb0; kb < sg.kb1; ++kb) {
            const unsigned sb = r.bcnt % kBStages;
            if (r.bcnt >= kBStages &&
                !mbar_wait(&c.bempty[sb], ((r.bcnt / kBStages) - 1) & 1, now_ns(), kWaitNs)) {
                set_abort(c, L.error);
                return;
            }
            if (aborted(c)) return;
            int dig[8][kS];
            const int k0 = kb * kKB + chunk * 8;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int k = k0 + u;
                slice7(k < L.ld ? __ldcg(x + (size_t)k * 8 + col) * inv : 0.0, dig[u]);
            }
            unsigned char *tile = c.smem + SmemLayout::b_off + (size_t)sb * kBTile;
#pragma unroll
            for (int b = 0; b < kS; ++b) {
                uint32_t w[4];
#pragma unroll
                for (int u = 0; u < 8; u += 2) {
                    const __nv_bfloat162 p = __floats2bfloat162_rn((float)dig[u][b], (float)dig[u + 1][b]);
                    w[u / 2] = *reinterpret_cast<const uint32_t *>(&p);
                }
                const int row = 8 * b + col;
                *reinterpret_cast<uint4 *>(tile + row * 128 + ((chunk ^ col) * 16)) = make_uint4(w[0], w[1], w[2], w[3]);
            }
            fence_proxy_async_smem();
            mbar_arrive(&c.bfull[sb]);
            ++r.bcnt;
        }
    }
}

// One row of a group's accumulators, added exactly into the 128-bit integer
// T = (Th, Tl) = sum over the segment of acc(a, b) 2^(8 (6 - a - b)), so that
// the row's product is 2^-64 T: every accumulator is an integer below 2^24 and
// the shift is at most 48 bits, so T stays far inside 128 bits.  Columns of
// pairs with a + b > 6 (pad columns and products below 2^-64) are skipped.
__device__ __forceinline__ void flush_group(uint32_t taddr, long long (&Th)[8], unsigned long long (&Tl)[8]) {
#pragma unroll 1
    for (int ch = 0; ch < kAccCols / 16; ch += 2) {  // two 16-column loads per wait
        uint32_t v[32];
        tmem_ld16(taddr + (uint32_t)(16 * ch), *reinterpret_cast<uint32_t(*)[16]>(&v[0]));
        tmem_ld16(taddr + (uint32_t)(16 * ch + 16), *reinterpret_cast<uint32_t(*)[16]>(&v[16]));
        tmem_wait_ld();
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int col = 16 * ch + 8 * h;
            const int a = acc_slice(col);
            const int d = a + (col - acc_off(a)) / 8;
            if (d >= kS) continue;
            const int sh = 8 * (kS - 1 - d);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const long long x = (long long)__float2int_rn(__uint_as_float(v[8 * h + q]));
                const unsigned long long lo = (unsigned long long)x << sh;
                const long long hi = sh ? (x >> (64 - sh)) : (x >> 63);
                const unsigned long long t = Tl[q] + lo;
                Th[q] += hi + (t < lo ? 1ll : 0ll);
                Tl[q] = t;
            }
        }
    }
}

struct PhaseIO {
    const double *x;     // input vector [ld][8]
    double *y;           // output vector [ld][8]
    int kind;            // 0: store y; 1: Chebyshev order epilogue
    int k;               // order
    double cre, cim;     // c_k
    const double *vm1;   // v_{k-1} (shift term of the implicit operator; nullptr: none)
    const double *vm2;   // v_{k-2} (k >= 2)
};

__device__ void flush_and_epilogue(const Ctx &c, const OzLaunch &L, int sched, int mat, const PhaseIO &io,
                                   const unsigned long long *cmax, unsigned long long *colmax_out, Roles &r) {
    const int t = threadIdx.x - 128;  // 0 .. 127: TMEM lane / row in the tile
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double cs[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) cs[q] = pow2(scale_exp(col_max(cmax, q)));
    const int s0 = L.seg_begin[sched][blockIdx.x], s1 = L.seg_begin[sched][blockIdx.x + 1];
    for (int q = s0; q < s1; ++q) {
        const OzSeg sg = L.segs[sched][q];
        long long Th[8];
        unsigned long long Tl[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            Th[u] = 0;
            Tl[u] = 0ull;
        }
        for (int g0 = sg.kb0; g0 < sg.kb1; g0 += kGroupBlocks) {
            const unsigned tb = r.gcnt & 1;
            // one thread waits and all 128 follow its outcome, so that none is left
            // alone at the named barriers below
            if (t == 0) *c.last_flag = mbar_wait(&c.accfull[tb], (r.gcnt >> 1) & 1, now_ns(), kWaitNs) ? 1u : 0u;
            asm volatile("bar.sync 1, 128;" ::: "memory");
            const bool ready = *(volatile unsigned *)c.last_flag != 0;
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (!ready) {
                if (t == 0) set_abort(c, L.error);
                return;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            flush_group(c.tmem + ((uint32_t)((warp & 3) * 32) << 16) + tb * kAccCols, Th, Tl);
            asm volatile("tcgen05.fence::before_thread_sync;");
            mbar_arrive(&c.accempty[tb]);
            ++r.gcnt;
        }
        const int row = sg.rt * kTileM + t;
        const double rs = L.rscale[mat][row] * pow2(-64);
        double R[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) R[u] = ((double)Th[u] * 0x1p64 + (double)Tl[u]) * rs * cs[u];
        double *part = L.part + ((size_t)(L.part_base[sched][sg.rt] + sg.slot) * kTileM + t) * 8;
#pragma unroll
        for (int u = 0; u < 8; u += 2) *reinterpret_cast<double2 *>(part + u) = make_double2(R[u], R[u + 1]);
        __threadfence();
        asm volatile("bar.sync 1, 128;" ::: "memory");
        const int np = L.part_count[sched][sg.rt];
        if (t == 0) *c.last_flag = atomicAdd(&L.tile_cnt[sg.rt], 1u) == (unsigned)(np - 1);
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (!*(volatile unsigned *)c.last_flag) continue;
        // last segment of this row tile: partials in segment order, then the epilogue
        __threadfence();
        double y[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) y[u] = 0.0;
        const double *p0 = L.part + ((size_t)L.part_base[sched][sg.rt] * kTileM + t) * 8;
        for (int s = 0; s < np; ++s) {
            const double2 *pp = reinterpret_cast<const double2 *>(p0 + (size_t)s * kTileM * 8);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const double2 v = __ldcg(pp + u);
                y[2 * u] += v.x;
                y[2 * u + 1] += v.y;
            }
        }
        if (t == 0) L.tile_cnt[sg.rt] = 0u;  // next used after a grid barrier
        double amax[8];
        if (row < L.N) {
            if (io.kind == 0) {
#pragma unroll
                for (int u = 0; u < 8; ++u) io.y[(size_t)row * 8 + u] = y[u];
            } else {
                double v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    double yv = y[u];
                    if (io.vm1) yv -= L.shift * __ldcg(io.vm1 + (size_t)row * 8 + u);
                    v[u] = io.k == 1 ? yv : 2.0 * yv - __ldcg(io.vm2 + (size_t)row * 8 + u);
                    io.y[(size_t)row * 8 + u] = v[u];
                }
                for (int col = 0; col < L.m; ++col) {  // acc += c_k v_k, complex column col
                    double2 *ap = L.acc + (size_t)row * L.m + col;
                    double2 a = __ldcg(ap);  // the row's last writer may have been another CTA
                    const double vr = v[2 * col], vi = v[2 * col + 1];
                    a.x += io.cre * vr - io.cim * vi;
                    a.y += io.cre * vi + io.cim * vr;
                    *ap = a;
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) y[u] = v[u];
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) amax[u] = fabs(y[u]);
        } else {
#pragma unroll
            for (int u = 0; u < 8; ++u) amax[u] = 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            double mx = amax[u];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0 && mx > 0.0) atomicMax(colmax_out + u, (unsigned long long)__double_as_longlong(mx));
        }
    }
}

// order 0: v_0 = s phi (s: pending renormalisation factor), acc = c_0 v_0, column maxima
__device__ void order_zero(const OzLaunch &L, double *v0, unsigned long long *colmax_out) {
    const int lane = threadIdx.x & 31;
    double amax[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) amax[u] = 0.0;
    const double2 c0 = L.coef[0];
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.N; i += stride) {
        for (int col = 0; col < L.m; ++col) {
            double2 p = L.phi[(size_t)i * L.m + col];
            if (L.scale) {
                const double sc = L.scale[col % L.P];
                p.x *= sc;
                p.y *= sc;
            }
            v0[(size_t)i * 8 + 2 * col] = p.x;
            v0[(size_t)i * 8 + 2 * col + 1] = p.y;
            L.acc[(size_t)i * L.m + col] = make_double2(c0.x * p.x - c0.y * p.y, c0.x * p.y + c0.y * p.x);
            amax[2 * col] = fmax(amax[2 * col], fabs(p.x));
            amax[2 * col + 1] = fmax(amax[2 * col + 1], fabs(p.y));
        }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        double mx = amax[u];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0 && mx > 0.0) atomicMax(colmax_out + u, (unsigned long long)__double_as_longlong(mx));
    }
}

__global__ void __launch_bounds__(kThreads, 1)
    oz_cheb_kernel(const __grid_constant__ CUtensorMap m0, const __grid_constant__ CUtensorMap m1,
                   const __grid_constant__ CUtensorMap m2, OzLaunch L) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    if ((int)blockIdx.x + 1 == L.exit_cta1) return;  // test hook: the other CTAs' barrier waits run out
    Ctx c;
    c.smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~static_cast<uintptr_t>(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(c.smem + SmemLayout::bar_off);
    c.full = bars;
    c.empty = c.full + kAStages;
    c.bfull = c.empty + kAStages;
    c.bempty = c.bfull + kBStages;
    c.accfull = c.bempty + kBStages;
    c.accempty = c.accfull + 2;
    c.done = c.accempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(c.smem + SmemLayout::misc_off);
    c.abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
    c.last_flag = reinterpret_cast<unsigned *>(tmem_slot + 2);
    const int warp = threadIdx.x >> 5;
    const CUtensorMap *maps[3] = {&m0, &m1, &m2};
    if (threadIdx.x == 0) {
        for (int s = 0; s < kAStages; ++s) {
            mbar_init(&c.full[s], 1);
            mbar_init(&c.empty[s], 1);
        }
        for (int s = 0; s < kBStages; ++s) {
            mbar_init(&c.bfull[s], 64);
            mbar_init(&c.bempty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(&c.accfull[s], 1);
            mbar_init(&c.accempty[s], 128);
        }
        mbar_init(c.done, 1);
        *c.abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // slot 7 (rows 56-63) of every B stage stays zero: the MMA of slice 0 reads 64 rows
    for (int q = threadIdx.x; q < kBStages * 8 * 128 / 16; q += kThreads) {
        const int s = q / (8 * 8), o = q % (8 * 8);
        *reinterpret_cast<uint4 *>(c.smem + SmemLayout::b_off + (size_t)s * kBTile + 56 * 128 + o * 16) =
            make_uint4(0u, 0u, 0u, 0u);
    }
    fence_proxy_async_smem();
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * kAccCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    c.tmem = *tmem_slot;
    const unsigned long long bar_ns = L.barrier_ns ? L.barrier_ns : kBarrierNs;
    const int G = gridDim.x;
    Roles r;

    // order 0 (phase sequence 0 writes column-max slot 0)
    order_zero(L, L.v, L.colmax);
    const bool ok0 = grid_barrier(L.bar_count, L.bar_gen, G, L.error, bar_ns);
    // The producer and the MMA issuer run through every phase without grid
    // barriers: the operator tiles do not depend on the previous phase, and the
    // MMAs wait for the vector operand, which the builders form only after the
    // phase's grid barrier.  So the next phase's loads and MMAs overlap the
    // barrier.  The builders and the flush warps (192 threads) meet every phase's
    // grid barrier on named barrier 2.
    int seq = 0;
    bool ok = ok0;
    for (int k = 1; ok && k <= L.K; ++k) {
        const double2 ck = L.coef[k];
        double *vk = L.v + (size_t)(k % 3) * L.ld * 8;
        const double *vm1 = L.v + (size_t)((k + 2) % 3) * L.ld * 8, *vm2 = L.v + (size_t)((k + 1) % 3) * L.ld * 8;
        for (int ph = 0; ph < L.nphase && ok; ++ph) {
            ++seq;
            // implicit: 0: w = G^T v (sched upper, matrix 0), 1: y = (h/b) w (full, 1),
            // 2: G y (lower, 2) + recurrence;  explicit: Hs v (full, 1) + recurrence
            const int sched = L.nphase == 3 ? ph : 1, mat = sched;
            if (warp == 0) {
                if ((threadIdx.x & 31) == 0) produce(c, L, maps[mat], sched, r);
                ok = !aborted(c) && *(volatile int *)L.error == 0;
                continue;
            }
            if (warp == 1) {
                if ((threadIdx.x & 31) == 0) issue_mma(c, L, sched, r);
                ok = !aborted(c) && *(volatile int *)L.error == 0;
                continue;
            }
            const unsigned long long *cm_in = L.colmax + (size_t)((seq + 2) % 3) * 8;
            unsigned long long *cm_out = L.colmax + (size_t)(seq % 3) * 8;
            if (blockIdx.x == 0 && threadIdx.x >= 64 && threadIdx.x < 72)
                L.colmax[(size_t)((seq + 1) % 3) * 8 + threadIdx.x - 64] = 0ull;
            PhaseIO io{};
            io.k = k;
            io.cre = ck.x;
            io.cim = ck.y;
            io.vm2 = vm2;
            if (L.nphase == 3) {
                io.x = ph == 0 ? vm1 : L.w + (size_t)(ph - 1) * L.ld * 8;
                io.y = ph == 2 ? vk : L.w + (size_t)ph * L.ld * 8;
                io.kind = ph == 2 ? 1 : 0;
                io.vm1 = ph == 2 ? vm1 : nullptr;
            } else {
                io.x = vm1;
                io.y = vk;
                io.kind = 1;
                io.vm1 = nullptr;
            }
            if (warp < 4) build(c, L, sched, io.x, cm_in, r);
            else flush_and_epilogue(c, L, sched, mat, io, cm_in, cm_out, r);
            ok = grid_barrier_sub(L.bar_count, L.bar_gen, G, L.error, bar_ns) && !aborted(c);
            if (!ok && threadIdx.x == 64) atomicExch(c.abort_flag, 1);  // stops this CTA's producer and MMA issuer
        }
    }
    // drain: copies issued into the A ring and every MMA complete before the CTA
    // leaves and frees its TMEM (all consumed already unless a wait gave up)
    if (threadIdx.x == 0) {
        const unsigned n = min(r.acnt, (unsigned)kAStages);
        for (unsigned q = r.acnt - n; q < r.acnt; ++q)
            mbar_wait(&c.full[q % kAStages], (q / kAStages) & 1, now_ns(), kWaitNs);
    }
    if (threadIdx.x == 32) {
        umma_commit(c.done);
        mbar_wait(c.done, 0, now_ns(), kWaitNs);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "r"(2 * kAccCols));
    }
}

// matrix slices: storage column j of M (ld rows, the row j of the operand A)
// on the scale 2^e_j of its largest element; out[s][j][i], rscale[j] = 2^e_j
__global__ void oz_slice_kernel(const double *__restrict__ M, int n, int ld, __nv_bfloat16 *__restrict__ out,
                                double *__restrict__ rscale) {
    __shared__ double s_max[32];
    const int j = blockIdx.x;
    const double *col = M + (size_t)j * ld;
    double mx = 0.0;
    for (int i = threadIdx.x; i < ld; i += blockDim.x) mx = fmax(mx, fabs(col[i]));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        mx = threadIdx.x < (blockDim.x >> 5) ? s_max[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (threadIdx.x == 0) s_max[0] = mx;
    }
    __syncthreads();
    const int e = scale_exp(s_max[0]);
    const double inv = pow2(-e);
    if (threadIdx.x == 0) rscale[j] = pow2(e);
    const size_t sstride = (size_t)n * ld;
    for (int i = threadIdx.x; i < ld; i += blockDim.x) {
        int dig[kS];
        slice7(col[i] * inv, dig);
#pragma unroll
        for (int s = 0; s < kS; ++s) out[s * sstride + (size_t)j * ld + i] = __float2bfloat16_rn((float)dig[s]);
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

// 3D BF16 map over the slices [kS][n][ld]: x = K (contiguous, ld), y = row, z =
// slice; box 64 x 128 x 1, 128B swizzle, zero fill outside
int make_slice_map(CUtensorMap *m, const __nv_bfloat16 *base, int n, int ld) {
    EncodeTiled fn = encode_fn();
    if (!fn) return ELHL_ERR_UNSUPPORTED;
    const cuuint64_t dims[3] = {(cuuint64_t)ld, (cuuint64_t)n, (cuuint64_t)kS};
    const cuuint64_t strides[2] = {(cuuint64_t)ld * 2, (cuuint64_t)ld * n * 2};
    const cuuint32_t box[3] = {(cuuint32_t)kKB, (cuuint32_t)kTileM, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(base), dims, strides,
                          box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? ELHL_OK : ELHL_ERR_BAD_ARG;
}

}  // namespace

int oz_slices() { return kS; }
int oz_tile_rows() { return kTileM; }
int oz_block_k() { return kKB; }
size_t oz_smem_bytes() { return 1024 + SmemLayout::bytes; }

cudaError_t oz_slice_matrix(const double *M, int n, int ld, __nv_bfloat16 *out, double *rscale, cudaStream_t st) {
    oz_slice_kernel<<<n, 256, 0, st>>>(M, n, ld, out, rscale);
    count_launch();
    return cudaGetLastError();
}

void oz_schedule(int n, int grid, int type, std::vector<OzSeg> &segs, std::vector<int> &seg_begin,
                 std::vector<int> &part_base, std::vector<int> &part_count) {
    const int nkb = (n + kKB - 1) / kKB, ntiles = (n + kTileM - 1) / kTileM;
    // blocks of row tile rt: full [0, nkb); upper (A = G^T, k >= row) [2 rt, nkb);
    // lower (A = G, k <= row) [0, 2 rt + 2)
    std::vector<int> lo(ntiles), hi(ntiles);
    long long total = 0;
    for (int rt = 0; rt < ntiles; ++rt) {
        lo[rt] = type == 0 ? 2 * rt : 0;
        hi[rt] = type == 2 ? std::min(nkb, 2 * rt + 2) : nkb;
        lo[rt] = std::min(lo[rt], hi[rt]);
        total += hi[rt] - lo[rt];
    }
    segs.clear();
    seg_begin.assign(grid + 1, 0);
    part_base.assign(ntiles, 0);
    part_count.assign(ntiles, 0);
    // CTA b takes the blocks [total b / grid, total (b + 1) / grid) in (row tile, block) order
    int rt = 0;
    long long pos = 0;  // blocks before row tile rt
    for (int b = 0; b < grid; ++b) {
        long long u0 = total * b / grid;
        const long long u1 = total * (b + 1) / grid;
        while (u0 < u1) {
            while (rt < ntiles && u0 >= pos + (hi[rt] - lo[rt])) {
                pos += hi[rt] - lo[rt];
                ++rt;
            }
            const long long end = std::min(u1, pos + (hi[rt] - lo[rt]));
            OzSeg s;
            s.rt = rt;
            s.kb0 = lo[rt] + (int)(u0 - pos);
            s.kb1 = lo[rt] + (int)(end - pos);
            s.slot = part_count[rt]++;
            segs.push_back(s);
            u0 = end;
        }
        seg_begin[b + 1] = (int)segs.size();
    }
    for (int t = 1; t < ntiles; ++t) part_base[t] = part_base[t - 1] + part_count[t - 1];
}

cudaError_t launch_oz_cheb(const OzLaunch &L, const __nv_bfloat16 *const slices[3], int grid, cudaStream_t st) {
    CUtensorMap m[3];
    for (int t = 0; t < 3; ++t) {
        const __nv_bfloat16 *base = slices[t] ? slices[t] : slices[1];
        if (make_slice_map(&m[t], base, L.N, L.ld)) return cudaErrorInvalidValue;
    }
    const size_t smem = oz_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(oz_cheb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    OzLaunch copy = L;
    void *args[] = {&m[0], &m[1], &m[2], &copy};
    e = cudaLaunchCooperativeKernel((const void *)oz_cheb_kernel, dim3(grid), dim3(kThreads), args, smem, st);
    count_launch();
    return e;
}

}  // namespace elhl
