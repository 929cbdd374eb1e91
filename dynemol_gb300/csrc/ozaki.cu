// FP64 Chebyshev propagation on the tensor cores by exact BF16 slices
// (Ozaki scheme I: Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59, 2012).
//
// GB300 runs FP64 FMAs at 1/58 of its FP32 rate, so the FP64 propagation on
// the FP64 pipe is bound by that pipe (1.2 TFLOP/s), not by HBM.  Here every
// FP64 operand is cut into kS = 7 slices of 8 bits each on a power-of-two
// scale (slice7):
//
//   a = 2^e  sum_{s<7} n_s 2^(-8(s+1)),   n_s integers, |n_0| <= 256, |n_s| <= 128,
//
// which represents a to 2^-57 relative to the scale.  An operator row has one
// scale; a vector column has one per 64-row chunk.  Each n_s is exact in BF16,
// each product of two slices is an integer below 2^16, and a sum of 256 of them
// an integer below 2^24: a BF16 tcgen05.mma with FP32 accumulation computes
// slice products exactly as long as the sums stay below 2^24.  The products with s_a + s_b <= 6
// (28 of the 49; the rest lie below 2^-64 of the scales) are summed per weight
// s_a + s_b in TMEM over one 64-K block (each sum below 2^23.2: exact), folded
// exactly into two 64-bit integers per row and column, and added as integers in the
// frame of the column's largest chunk scale (exact to 2^-64 of it): a row
// tile's product is one exact 128-bit integer per column until its single
// rounding to FP64, whatever the order its partial sums arrive in.  The
// operator is read as 14 bytes per element (7 BF16 slices) instead of 8, but
// the work moves from the FP64 pipe to the tensor pipe, which leaves HBM as
// the bound.
//
// One cooperative launch runs every order of one nuclear step: an order is one
// grid phase y = Hs x with the row-scaled sliced Hs = (H~ - a)/b.  Its work is
// the 64-K blocks of the 128-row tiles of Hs, split evenly over the CTAs; a
// CTA's blocks form segments (runs within a row tile).  Per CTA:
//   warp 0     TMA producer: the 7 slices of each block (128 x 64 BF16, 16 KB,
//              128B swizzle) into a ring of kAStages stages, through every order
//              without waiting for grid barriers (the operator does not change);
//   warp 1     allocates TMEM; one thread issues tcgen05.mma (M = 128, K = 16,
//              N = 64 ... 16: slice s_a against the vector slices s_b <= 6 - s_a)
//              into one of two 64-column accumulator buffers, one 8-column sum
//              per weight s_a + s_b, also through every order (it waits for
//              each block's vector operand);
//   warp 2     one thread loads each block's vector operand (9 KB, already sliced
//              and swizzled by the previous order) with one bulk copy, after the
//              order's grid barrier;
//   warps 4-7  fold each block from TMEM (one thread per row); at the end of a
//              segment they store its partial (exact 128-bit integers); a CTA
//              designated per half of a 64-row chunk (4 of the 8 columns) sums
//              the tile's partials once all are counted (exact, in any order),
//              applies the Chebyshev recurrence and the c_k v_k accumulation
//              in FP64, and slices its rows of v_k for the next order.
// Warps 2-7 meet the grid barrier of every order.  Every wait is bounded: on a
// timeout the CTA sets ELHL_ERR_TIMEOUT, stops, waits for its own copies and
// MMAs, and frees TMEM.
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
constexpr int kAStages = 10;
constexpr int kBStages = 4;
constexpr int kXeCap = 2048;  // chunk exponents held in shared memory (N <= 16384; larger N reads them from L2)
constexpr int kThreads = 256;
constexpr int kATile = kTileM * kKB * 2;  // 16 KB
// vector operand tile: 9 slots of 8 rows (one per real column) x 128 bytes:
// a zero slot, the slices 0-6, a zero slot
constexpr int kBSlots = kS + 2;
constexpr int kBTile = kBSlots * 8 * 128;     // 9 KB
constexpr int kAccCols = 64;                  // TMEM columns per accumulator buffer: weights d = 0..7 x 8
constexpr unsigned long long kWaitNs = 2000000000ull;

// Every slice product of weight d = a + b accumulates into the 8 TMEM columns
// [8 d, 8 d + 8) of the buffer.  Slice a's MMA writes column block j of its D
// region from B block j: for even a the region starts at column 8 a and B at
// slice 0 (block j = slice j, weight a + j); for odd a both start one block
// earlier, at column 8 (a - 1) and at the leading zero slot (block j = slice
// j - 1, weight a + j - 1), so that every D region starts on a multiple of 16
// columns.  N covers the slices b <= 6 - a, rounded up to 16 (the extra block
// reads a zero slot or lands in columns [56, 64), weight 7, never read).
__host__ __device__ constexpr int mma_col(int a) { return 8 * (a & ~1); }
__host__ __device__ constexpr int mma_n(int a) { return ((8 * (kS - a) + 8 * (a & 1) + 15) / 16) * 16; }
__host__ __device__ constexpr int mma_brow(int a) { return (a & 1) ? 0 : 8; }  // first B row (slot) read
constexpr bool acc_layout_ok() {
    for (int a = 0; a < kS; ++a)
        if (mma_col(a) % 16 || mma_col(a) + mma_n(a) > kAccCols || mma_brow(a) + mma_n(a) > 8 * kBSlots ||
            mma_col(a) - 8 * (mma_brow(a) / 8 - 1) != 8 * a)  // column block j holds weight a + b, b = block - brow/8
            return false;
    return true;
}
static_assert(kS == 7 && acc_layout_ok(), "accumulator layout");

__device__ __forceinline__ double pow2(int e) {  // 2^e for |e| < 1000
    return __longlong_as_double((long long)(1023 + e) << 52);
}
// exponent e with |x| < 2^e for the non-zero finite x (0 for x = 0)
__device__ __forceinline__ int scale_exp(double x) {
    if (!(x > 0.0)) return 0;
    return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1022;
}
// byte offset of (row R, K index kk) in a 128B-swizzled K-major tile of 128-byte rows
__device__ __forceinline__ int swz_off(int R, int kk) { return R * 128 + (((kk >> 3) ^ (R & 7)) << 4) + ((kk & 7) << 1); }

__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// generic-proxy global writes made visible to (and ordered with) the async proxy
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

struct SmemLayout {
    static constexpr size_t a_off = 0;
    static constexpr size_t b_off = a_off + (size_t)kAStages * kATile;
    static constexpr size_t bar_off = b_off + (size_t)kBStages * kBTile;
    static constexpr size_t n_bars = 2 * kAStages + 2 * kBStages + 2 + 2 + 1;
    static constexpr size_t red_off = bar_off + n_bars * 8;        // [4][8] ints: column maxima of the warps
    static constexpr size_t out_off = (red_off + 4 * 8 * 4 + 1023) / 1024 * 1024;
    static constexpr size_t misc_off = out_off + (size_t)kBTile;  // one output tile
    static constexpr size_t xe_off = misc_off + 64;                // [kXeCap] the order's chunk exponents
    static constexpr size_t bytes = xe_off + (size_t)kXeCap * 4;
};
static_assert(SmemLayout::bytes + 1024 <= 227 * 1024, "shared memory of one CTA");

struct Roles {  // counters every role advances in the same order
    unsigned acnt = 0;   // A stages
    unsigned bcnt = 0;   // B stages
    unsigned gcnt = 0;   // groups
};

struct Ctx {
    unsigned char *smem;
    uint64_t *full, *empty, *bfull, *bempty, *accfull, *accempty, *done;
    int *red;
    int *xe;
    unsigned char *out;
    uint32_t tmem;
    int *abort_flag;
    unsigned *last_flag;
};

__device__ __forceinline__ bool aborted(const Ctx &c) { return *(volatile int *)c.abort_flag != 0; }
__device__ __forceinline__ void set_abort(const Ctx &c, int *err) {
    atomicExch(c.abort_flag, 1);
    atomicExch(err, (int)ELHL_ERR_TIMEOUT);
}

// Grid barrier among the 192 threads of warps 2-7 (named barrier 2): thread
// 64 arrives for the CTA by a release add to a count that only grows (zero at
// the launch) and waits, with acquire loads, until all nblocks CTAs have
// arrived at this barrier (the count reaches `target` = nblocks x barriers so
// far).  No reset and no generation word: the last arrival itself releases
// the others.  Bounded: false (with ELHL_ERR_TIMEOUT) after limit_ns.
__device__ __forceinline__ bool grid_barrier_sub(unsigned *count, unsigned target, int *err,
                                                 unsigned long long limit_ns) {
    asm volatile("bar.sync 2, 192;" ::: "memory");
    if (threadIdx.x == 64) {
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
        const unsigned long long t0 = globaltimer_ns();
        while (true) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(count) : "memory");
            if (v >= target) break;
            if (globaltimer_ns() - t0 > limit_ns) {
                atomicExch(err, ELHL_ERR_TIMEOUT);
                break;
            }
            __nanosleep(20);
        }
    }
    asm volatile("bar.sync 2, 192;" ::: "memory");
    return *(volatile int *)err == 0;
}

// ---- phase roles ----------------------------------------------------------------

// The CTA's blocks of one order: its segments and their blocks in order, or (rev)
// both backwards.  Odd orders run backwards: the operator's slices (14 N^2 bytes,
// 194 MB at N = 3720) exceed the 129 MB L2, so a forward walk every order finds
// none of them there, while turning back starts each order on the part the last
// one read most recently.  The sums are exact, so the direction changes no bit.
__device__ __forceinline__ int walk_seg(int s0, int s1, int i, bool rev) { return rev ? s1 - 1 - i : s0 + i; }
__device__ __forceinline__ int walk_kb(const OzSeg &sg, int i, bool rev) { return rev ? sg.kb1 - 1 - i : sg.kb0 + i; }

__device__ void produce(const Ctx &c, const OzLaunch &L, const CUtensorMap *map, Roles &r, bool rev) {
    const int s0 = L.seg_begin[blockIdx.x], s1 = L.seg_begin[blockIdx.x + 1];
    for (int qi = 0; qi < s1 - s0; ++qi) {
        const OzSeg sg = L.segs[walk_seg(s0, s1, qi, rev)];
        for (int ki = 0; ki < sg.kb1 - sg.kb0; ++ki) {
            const int kb = walk_kb(sg, ki, rev);
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

// One block per accumulator buffer: over 64 K every weight's sum of slice
// products stays below 2^23.2, exact in FP32.
__device__ void issue_mma(const Ctx &c, const OzLaunch &L, Roles &r, bool rev) {
    const int s0 = L.seg_begin[blockIdx.x], s1 = L.seg_begin[blockIdx.x + 1];
    for (int qi = 0; qi < s1 - s0; ++qi) {
        const OzSeg sg = L.segs[walk_seg(s0, s1, qi, rev)];
        for (int ki = 0; ki < sg.kb1 - sg.kb0; ++ki) {
            const unsigned tb = r.gcnt & 1;
            if (r.gcnt >= 2 && !mbar_wait(&c.accempty[tb], ((r.gcnt >> 1) - 1) & 1, now_ns(), kWaitNs)) {
                set_abort(c, L.error);
                return;
            }
            const unsigned sb = r.bcnt % kBStages;
            if (!mbar_wait(&c.bfull[sb], (r.bcnt / kBStages) & 1, now_ns(), kWaitNs)) {
                set_abort(c, L.error);
                return;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const unsigned char *btile = c.smem + SmemLayout::b_off + (size_t)sb * kBTile;
#pragma unroll
            for (int a = 0; a < kS; ++a) {
                const unsigned s = r.acnt % kAStages;
                if (!mbar_wait(&c.full[s], (r.acnt / kAStages) & 1, now_ns(), kWaitNs)) {
                    set_abort(c, L.error);
                    return;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint64_t da = smem_desc_sw128(c.smem + SmemLayout::a_off + (size_t)s * kATile);
                const uint64_t db = smem_desc_sw128(btile + mma_brow(a) * 128);
                const uint32_t acc = c.tmem + tb * kAccCols + (uint32_t)mma_col(a);
                const uint32_t idesc = idesc_bf16(kTileM, mma_n(a));
#pragma unroll
                for (int k = 0; k < kKB / 16; ++k)  // K = 16 per MMA: +32 bytes along the swizzled row
                    umma_bf16(acc, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), idesc, !(a == 0 && k == 0));
                umma_commit(&c.empty[s]);  // the A stage is free once these MMAs have read it
                ++r.acnt;
            }
            umma_commit(&c.bempty[sb]);
            ++r.bcnt;
            umma_commit(&c.accfull[tb]);
            ++r.gcnt;
        }
    }
}

// vector operand of each block: the 9 KB tile the previous order wrote
__device__ void load_vectors(const Ctx &c, const OzLaunch &L, const unsigned char *xs, Roles &r, bool rev) {
    fence_proxy_async_global();  // the tiles were written by generic stores before the grid barrier
    const int s0 = L.seg_begin[blockIdx.x], s1 = L.seg_begin[blockIdx.x + 1];
    for (int qi = 0; qi < s1 - s0; ++qi) {
        const OzSeg sg = L.segs[walk_seg(s0, s1, qi, rev)];
        for (int ki = 0; ki < sg.kb1 - sg.kb0; ++ki) {
            const int kb = walk_kb(sg, ki, rev);
            const unsigned sb = r.bcnt % kBStages;
            if (r.bcnt >= kBStages &&
                !mbar_wait(&c.bempty[sb], ((r.bcnt / kBStages) - 1) & 1, now_ns(), kWaitNs)) {
                set_abort(c, L.error);
                return;
            }
            if (aborted(c)) return;
            mbar_expect_tx(&c.bfull[sb], (unsigned)kBTile);
            bulk_load(c.smem + SmemLayout::b_off + (size_t)sb * kBTile, xs + (size_t)kb * kBTile, (unsigned)kBTile,
                      &c.bfull[sb]);
            ++r.bcnt;
        }
    }
}

// One row of a block's weight sums acc_d (TMEM columns 8 d + q, d <= 6) added
// exactly into H += sum_{d<=2} acc_d 2^(8 (2 - d)) and L += sum_{d>=3} acc_d
// 2^(8 (6 - d)) per column q: every acc_d is an integer below 2^23.2, so over
// the two blocks of a chunk H < 2^40.2 and L < 2^48.2.
__device__ __forceinline__ void flush_block(uint32_t taddr, long long (&H)[8], long long (&Lo)[8]) {
    uint32_t v[64];
    tmem_ld32(taddr, *reinterpret_cast<uint32_t(*)[32]>(&v[0]));
    tmem_ld32(taddr + 32u, *reinterpret_cast<uint32_t(*)[32]>(&v[32]));
    tmem_wait_ld();
#pragma unroll
    for (int d = 0; d < kS; ++d)
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const long long x = (long long)__float2int_rn(__uint_as_float(v[8 * d + q]));
            if (d <= 2) H[q] += x * (1ll << (8 * (2 - d)));
            else Lo[q] += x * (1ll << (8 * (kS - 1 - d)));
        }
}

struct OrderIO {
    int k;                    // order
    double cre, cim;          // c_k
    const double *vm2;        // v_{k-2} FP64 (k >= 2)
    double *vk;               // v_k FP64 out (kind 1)
    const int *xe_in;         // [chunks][8] exponents e of the input vector's chunk scales 2^e
    const int *emax_in;       // [8] the largest of them per column
    unsigned char *xs_out;    // sliced output tiles
    int *xe_out;              // [chunks][8] their exponents
    int *emax_out;            // [8] their maxima (integer max)
};

// 128-bit two's complement integers (hi, lo) for the exact sums of slice products
struct I128 {
    long long hi;
    unsigned long long lo;
};
__device__ __forceinline__ void add128(I128 &a, const I128 &b) {
    const unsigned long long t = a.lo + b.lo;
    a.hi += b.hi + (t < b.lo ? 1ll : 0ll);
    a.lo = t;
}
// (H 2^32 + L) 2^-sft, rounded toward minus infinity (sft >= 0): |H 2^32 + L| < 2^76
__device__ __forceinline__ I128 group_term(long long H, long long L, int sft) {
    long long th = H >> 32;
    unsigned long long tl = (unsigned long long)H << 32;
    const unsigned long long t2 = tl + (unsigned long long)L;
    th += (L >> 63) + (t2 < tl ? 1ll : 0ll);
    tl = t2;
    I128 r;
    if (sft >= 127) {
        r.hi = th >> 63;
        r.lo = (unsigned long long)(th >> 63);
    } else if (sft >= 64) {
        r.lo = (unsigned long long)(th >> (sft - 64));
        r.hi = th >> 63;
    } else if (sft > 0) {
        r.lo = (tl >> sft) | ((unsigned long long)th << (64 - sft));
        r.hi = th >> sft;
    } else {
        r.lo = tl;
        r.hi = th;
    }
    return r;
}
// exact integer -> double for 0 <= x < 2^52 (the bits of 2^52 + x, less 2^52)
__device__ __forceinline__ double u52_to_double(unsigned long long x) {
    return __longlong_as_double((long long)(0x4330000000000000ull | x)) - 0x1p52;
}
// A 128-bit integer (|s| < 2^116) rounded to FP64 from its magnitude, by exact
// conversions of three positive parts: no FP64 conversion instructions, no
// cancellation.
__device__ __forceinline__ double i128_to_double(I128 s) {
    const bool neg = s.hi < 0;
    if (neg) {  // two's complement negation
        s.lo = ~s.lo + 1ull;
        s.hi = ~s.hi + (s.lo == 0ull ? 1ll : 0ll);
    }
    const double d = fma(u52_to_double((unsigned long long)s.hi), 0x1p64,
                         fma(u52_to_double(s.lo >> 32), 0x1p32, u52_to_double(s.lo & 0xffffffffull)));
    return neg ? -d : d;
}
constexpr int kNoExp = (int)0x80808080;  // the column maximum before any chunk (bytes 0x80: a memset)

// The epilogue of one 64-row chunk h of v_k (rows 64 h ...) runs in two
// halves of 4 columns, half c on the 128 threads of warps 4-7 of the CTA
// designated for (h, c): thread t handles row 64 h + (t & 63) and the columns
// 4 c + 2 (t >> 6) and the next (one complex column).  The halves share
// nothing: every column has its own scale.
struct EpiThread {
    int t, r, p, row, col;  // thread, row in the chunk, column pair, global row, first column
};
__device__ __forceinline__ EpiThread epi_thread(int h, int c, int t) {
    return EpiThread{t, t & 63, t >> 6, 64 * h + (t & 63), 4 * c + 2 * (t >> 6)};
}

// The half's 64 new rows (2 columns per thread, 0 past N) cut into slices on
// one scale 2^e per column: tile h of xs (this half's rows of it), the
// exponents at xe[h], their maximum over the chunks in emax (non-zero
// columns); slice b goes to slot b + 1, slots 0 and 8 stay zero.  Digits formed
// in shared memory, copied out in 16-byte stores.  Named barrier 1 (the 128
// threads).
__device__ void slice_chunk_out(const Ctx &c, int h, int half, const EpiThread &et, const double (&y)[2],
                                unsigned char *xs, int *xe, int *emax) {
    const int w = et.t >> 5;  // warps 0, 1: the half's columns 0-1; warps 2, 3: columns 2-3
#pragma unroll
    for (int u = 0; u < 2; ++u) {  // largest exponent field of the column over the warp's rows
        const int m = __reduce_max_sync(0xffffffffu, exp_field(y[u]));
        if ((et.t & 31) == 0) c.red[w * 2 + u] = m;
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
    int e[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const int be = max(c.red[(2 * et.p) * 2 + u], c.red[(2 * et.p + 1) * 2 + u]);
        e[u] = be ? be - 1022 : 0;  // |column| < 2^e (0 for a zero column)
        if (et.r == 0) {
            xe[h * 8 + et.col + u] = e[u];
            if (be) atomicMax(emax + et.col + u, e[u]);
        }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        int dig[kS];
        slice7(y[u], e[u], dig);
#pragma unroll
        for (int b = 0; b < kS; ++b)
            *reinterpret_cast<__nv_bfloat16 *>(c.out + swz_off(8 * (b + 1) + et.col + u, et.r)) =
                __float2bfloat16_rn((float)dig[b]);
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");  // the rows are complete; c.red is free again
    constexpr int kPieces = kS * 4 * 8;  // slots 1-7 x the half's 4 rows x 8 pieces of 16 bytes
    for (int q = et.t; q < kPieces; q += 128) {
        const int o = (8 * (1 + q / 32) + 4 * half + (q / 8) % 4) * 128 + (q % 8) * 16;
        *reinterpret_cast<uint4 *>(xs + (size_t)h * kBTile + o) = *reinterpret_cast<const uint4 *>(c.out + o);
    }
    fence_proxy_async_global();  // read by bulk copies after the next grid barrier
}

// bounded wait until *cnt reaches target (segments of a row tile written)
__device__ __forceinline__ bool wait_count(const unsigned *cnt, unsigned target) {
    const unsigned long long t0 = now_ns();
    while (*(volatile const unsigned *)cnt < target) {
        if (now_ns() - t0 > kWaitNs) return false;
        __nanosleep(32);
    }
    return true;
}

// What a half-chunk epilogue reads besides the partials, loaded before it
// waits for them: v_{k-2} and the accumulated sum of its rows.
struct EpiPre {
    double vm2[2];
    double2 acc;
};
__device__ __forceinline__ EpiPre epi_prefetch(const OzLaunch &L, const OrderIO &io, const EpiThread &et) {
    EpiPre q{{0.0, 0.0}, make_double2(0.0, 0.0)};
    if (et.row < L.N) {
        if (io.k > 1)
#pragma unroll
            for (int u = 0; u < 2; ++u) q.vm2[u] = io.vm2[(size_t)et.row * 8 + et.col + u];
        if (et.col / 2 < L.m) q.acc = L.acc[(size_t)et.row * L.m + et.col / 2];
    }
    return q;
}

// Epilogue of half c of chunk h once its row tile's np segments are written:
// the exact sum of their partials, the row's product in FP64, the recurrence
// and accumulation of order k, and the slices of the half's rows of v_k for the
// next order.  The rows and columns of a half are only ever touched by this
// CTA (order 0 included), so v and acc use plain (L1) loads.
__device__ void chunk_epilogue(const Ctx &c, const OzLaunch &L, const OrderIO &io, int h, int half, int np,
                               const int (&E)[8], const EpiThread &et, const EpiPre &pre) {
    const int rt = h >> 1, trow = (h & 1) * 64 + et.r;  // row tile, row in it
    I128 S[2] = {I128{0, 0ull}, I128{0, 0ull}};
    const longlong2 *p0 = reinterpret_cast<const longlong2 *>(L.part) +
                          ((size_t)L.part_base[rt] * kTileM + trow) * 8 + et.col;
    for (int s0 = 0; s0 < np; s0 += 8) {  // up to 16 loads in flight
        longlong2 v[8][2];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (s0 + j < np)
#pragma unroll
                for (int u = 0; u < 2; ++u) v[j][u] = __ldcg(p0 + (size_t)(s0 + j) * kTileM * 8 + u);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (s0 + j < np)
#pragma unroll
                for (int u = 0; u < 2; ++u) add128(S[u], I128{v[j][u].x, (unsigned long long)v[j][u].y});
    }
    const double rs = L.rscale[et.row];
    double y[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const int col = et.col + u;
        const double yv = i128_to_double(S[u]) * (pow2(max(E[col], -900) - 64) * rs);
        double v = 0.0;  // v_k = Hs v_{k-1} (k = 1), 2 Hs v_{k-1} - v_{k-2} after; rows past N stay zero
        if (et.row < L.N) {
            v = io.k == 1 ? yv : 2.0 * yv - pre.vm2[u];
            io.vk[(size_t)et.row * 8 + col] = v;
        }
        y[u] = v;
    }
    if (et.row < L.N && et.col / 2 < L.m) {  // acc += c_k v_k, the thread's complex column
        double2 a = pre.acc;
        a.x += io.cre * y[0] - io.cim * y[1];
        a.y += io.cre * y[1] + io.cim * y[0];
        L.acc[(size_t)et.row * L.m + et.col / 2] = a;
    }
    slice_chunk_out(c, h, half, et, y, io.xs_out, io.xe_out, io.emax_out);
}

// A row tile's partial (exact 128-bit integers, 8 columns per row) into its
// slot.  It is counted at its row tile later (release_partials), once the next
// segment's work has given the stores time to complete.
__device__ __forceinline__ void store_partial(const OzLaunch &L, int slot, int t, const I128 (&A)[8]) {
    longlong2 *part = reinterpret_cast<longlong2 *>(L.part) + ((size_t)slot * kTileM + t) * 8;
#pragma unroll
    for (int u = 0; u < 8; ++u) part[u] = make_longlong2(A[u].hi, (long long)A[u].lo);
}
// the stored partial of row tile `tile` (if >= 0) made visible, then counted
__device__ __forceinline__ void release_partial(const OzLaunch &L, int &tile, int t) {
    if (tile < 0) return;
    __threadfence();
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (t == 0) atomicAdd(&L.tile_cnt[tile], 1u);
    tile = -1;
}

// The CTA's segments: each 64-K block's weight sums folded, with that chunk's
// vector scale, into one exact 128-bit integer per row and column, stored as
// the segment's partial and counted at its row tile.  The chunk exponents of
// the order's vector are read once into shared memory.  Then the epilogues of
// the half-chunks this CTA is designated for (half-chunk q = 2 h + c by CTA
// floor(q grid / halves): spread over the grid, at most one per CTA while
// halves <= grid), each once its row tile's segments are all counted.
__device__ void flush_and_epilogue(const Ctx &c, const OzLaunch &L, const OrderIO &io, Roles &r, bool rev) {
    const int t = threadIdx.x - 128;  // 0 .. 127: TMEM lane / row in the tile
    const int warp = threadIdx.x >> 5;
    const int s0 = L.seg_begin[blockIdx.x], s1 = L.seg_begin[blockIdx.x + 1];
    const int nkb = (L.N + kKB - 1) / kKB, ntiles = (L.N + kTileM - 1) / kTileM;
    // every block of this order is added exactly in the frame 2^(E - 64) of its
    // column's largest chunk scale 2^E
    int E[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) E[u] = __ldcg(io.emax_in + u);
    const bool xe_smem = nkb * 8 <= kXeCap;
    if (xe_smem) {
        for (int i = t; i < nkb * 8; i += 128) c.xe[i] = __ldcg(io.xe_in + i);
        asm volatile("bar.sync 1, 128;" ::: "memory");
    }
    int pend = -1;  // row tile of the stored, not yet counted partial
    for (int qi = 0; qi < s1 - s0; ++qi) {
        const OzSeg sg = L.segs[walk_seg(s0, s1, qi, rev)];
        I128 A[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) A[u] = I128{0, 0ull};
        for (int ki = 0; ki < sg.kb1 - sg.kb0; ++ki) {
            const int kb = walk_kb(sg, ki, rev);
            const unsigned tb = r.gcnt & 1;
            // one thread waits and all 128 follow its outcome, so that none is left
            // alone at the named barriers
            if (t == 0) *c.last_flag = mbar_wait(&c.accfull[tb], (r.gcnt >> 1) & 1, now_ns(), kWaitNs) ? 1u : 0u;
            asm volatile("bar.sync 1, 128;" ::: "memory");
            const bool ready = *(volatile unsigned *)c.last_flag != 0;
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (!ready) {
                if (t == 0) set_abort(c, L.error);
                return;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            long long H[8], Lo[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                H[u] = 0;
                Lo[u] = 0;
            }
            flush_block(c.tmem + ((uint32_t)((warp & 3) * 32) << 16) + tb * kAccCols, H, Lo);
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if ((t & 31) == 0) mbar_arrive(&c.accempty[tb]);  // one arrival per warp: its loads are done
            ++r.gcnt;
#pragma unroll
            for (int u = 0; u < 8; ++u) {  // the block's vector chunk exponents
                const int ec = xe_smem ? c.xe[kb * 8 + u] : __ldcg(io.xe_in + (size_t)kb * 8 + u);
                add128(A[u], group_term(H[u], Lo[u], max(0, E[u] - ec)));
            }
        }
        release_partial(L, pend, t);
        store_partial(L, L.part_base[sg.rt] + sg.slot, t, A);
        pend = sg.rt;
    }
    release_partial(L, pend, t);
    const int nhc = 4 * ntiles, G = gridDim.x;
    const int q1 = (int)(((long long)(blockIdx.x + 1) * nhc + G - 1) / G);
    for (int q = (int)(((long long)blockIdx.x * nhc + G - 1) / G); q < q1; ++q) {
        const int h = q >> 1, half = q & 1;
        const EpiThread et = epi_thread(h, half, t);
        const EpiPre pre = epi_prefetch(L, io, et);
        const int np = L.part_count[h >> 1];
        // the count only grows (np per order, zero at the launch): order k waits for k np
        if (t == 0) *c.last_flag = wait_count(&L.tile_cnt[h >> 1], (unsigned)(np * io.k)) ? 1u : 0u;
        asm volatile("bar.sync 1, 128;" ::: "memory");
        const bool ready = *(volatile unsigned *)c.last_flag != 0;
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (!ready) {
            if (t == 0) set_abort(c, L.error);
            return;
        }
        __threadfence();
        chunk_epilogue(c, L, io, h, half, np, E, et, pre);
    }
}

// order 0: v_0 = s phi (s: pending renormalisation factor), acc = c_0 v_0, and
// the slices of v_0, by warps 4-7 of the CTA designated for each half-chunk
__device__ void order_zero(const Ctx &c, const OzLaunch &L) {
    const int t = threadIdx.x - 128;
    const int nhc = 4 * ((L.N + kTileM - 1) / kTileM), G = gridDim.x;
    const double2 c0 = L.coef[0];
    const int q1 = (int)(((long long)(blockIdx.x + 1) * nhc + G - 1) / G);
    for (int q = (int)(((long long)blockIdx.x * nhc + G - 1) / G); q < q1; ++q) {
        const int h = q >> 1, half = q & 1;
        const EpiThread et = epi_thread(h, half, t);
        double y[2] = {0.0, 0.0};
        const int cc = et.col / 2;  // the thread's complex column
        if (et.row < L.N && cc < L.m) {
            double2 p = L.phi[(size_t)et.row * L.m + cc];
            if (L.scale) {
                const double sc = L.scale[cc % L.P];
                p.x *= sc;
                p.y *= sc;
            }
            L.v[(size_t)et.row * 8 + 2 * cc] = p.x;
            L.v[(size_t)et.row * 8 + 2 * cc + 1] = p.y;
            L.acc[(size_t)et.row * L.m + cc] = make_double2(c0.x * p.x - c0.y * p.y, c0.x * p.y + c0.y * p.x);
            y[0] = p.x;
            y[1] = p.y;
        }
        slice_chunk_out(c, h, half, et, y, L.xs[0], L.xe[0], L.emax[0]);
    }
}

__global__ void __launch_bounds__(kThreads, 1)
    oz_cheb_kernel(const __grid_constant__ CUtensorMap mH, OzLaunch L) {
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
    c.red = reinterpret_cast<int *>(c.smem + SmemLayout::red_off);
    c.out = c.smem + SmemLayout::out_off;
    c.xe = reinterpret_cast<int *>(c.smem + SmemLayout::xe_off);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(c.smem + SmemLayout::misc_off);
    c.abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
    c.last_flag = reinterpret_cast<unsigned *>(tmem_slot + 2);
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kAStages; ++s) {
            mbar_init(&c.full[s], 1);
            mbar_init(&c.empty[s], 1);
        }
        for (int s = 0; s < kBStages; ++s) {
            mbar_init(&c.bfull[s], 1);
            mbar_init(&c.bempty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(&c.accfull[s], 1);
            mbar_init(&c.accempty[s], 4);  // one arrival per flush warp
        }
        mbar_init(c.done, 1);
        *c.abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
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

    if (warp >= 4) order_zero(c, L);  // slices of v_0 into vector buffer 0
    // The producer and the MMA issuer run through every order without grid
    // barriers: the operator tiles do not change, and the MMAs wait for each
    // block's vector operand, which thread 64 loads only after the order's grid
    // barrier.  So the next order's loads and MMAs overlap the barrier.  Warps
    // 2-7 meet every grid barrier on named barrier 2.
    bool ok = true;
    if (warp >= 2) ok = grid_barrier_sub(L.bar_count, (unsigned)G, L.error, bar_ns);
    // the sliced vector v_k is in buffer k % 3
    for (int k = 1; ok && k <= L.K; ++k) {
        const int bin = (k + 2) % 3, bout = k % 3;
        if (warp == 0) {
            if ((threadIdx.x & 31) == 0) produce(c, L, &mH, r, k & 1);
            ok = !aborted(c) && *(volatile int *)L.error == 0;
            continue;
        }
        if (warp == 1) {
            if ((threadIdx.x & 31) == 0) issue_mma(c, L, r, k & 1);
            ok = !aborted(c) && *(volatile int *)L.error == 0;
            continue;
        }
        if (warp < 4) {
            // buffer (k + 1) % 3 was written two orders ago and read in the last one
            if (blockIdx.x == 0 && threadIdx.x >= 96 && threadIdx.x < 104)
                L.emax[(k + 1) % 3][threadIdx.x - 96] = kNoExp;
            if (threadIdx.x == 64) load_vectors(c, L, L.xs[bin], r, k & 1);
        } else {
            OrderIO io{};
            const double2 ck = L.coef[k];
            io.k = k;
            io.cre = ck.x;
            io.cim = ck.y;
            io.vm2 = L.v + (size_t)((k + 1) % 3) * L.ld * 8;
            io.vk = L.v + (size_t)(k % 3) * L.ld * 8;
            io.xe_in = L.xe[bin];
            io.emax_in = L.emax[bin];
            io.xs_out = L.xs[bout];
            io.xe_out = L.xe[bout];
            io.emax_out = L.emax[bout];
            flush_and_epilogue(c, L, io, r, k & 1);
        }
        ok = grid_barrier_sub(L.bar_count, (unsigned)G * (unsigned)(k + 1), L.error, bar_ns) && !aborted(c);
        if (!ok && threadIdx.x == 64) atomicExch(c.abort_flag, 1);  // stops this CTA's producer and MMA issuer
    }
    // drain: copies issued into the A ring and every MMA complete before the CTA
    // leaves and frees its TMEM (all consumed already unless a wait gave up)
    if (threadIdx.x == 0) {
        const unsigned n = min(r.acnt, (unsigned)kAStages);
        for (unsigned q = r.acnt - n; q < r.acnt; ++q)
            mbar_wait(&c.full[q % kAStages], (q / kAStages) & 1, now_ns(), kWaitNs);
    }
    if (threadIdx.x == 64) {  // the vector loads of stages not consumed
        const unsigned n = min(r.bcnt, (unsigned)kBStages);
        for (unsigned q = r.bcnt - n; q < r.bcnt; ++q)
            mbar_wait(&c.bfull[q % kBStages], (q / kBStages) & 1, now_ns(), kWaitNs);
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

// operator slices: storage column j of the symmetric Hs (ld rows, its row j)
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
    if (threadIdx.x == 0) rscale[j] = pow2(e);
    const size_t sstride = (size_t)n * ld;
    for (int i = threadIdx.x; i < ld; i += blockDim.x) {
        int dig[kS];
        slice7(col[i], e, dig);
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
size_t oz_vector_tile_bytes() { return kBTile; }
size_t oz_smem_bytes() { return 1024 + SmemLayout::bytes; }

cudaError_t oz_slice_matrix(const double *M, int n, int ld, __nv_bfloat16 *out, double *rscale, cudaStream_t st) {
    oz_slice_kernel<<<n, 256, 0, st>>>(M, n, ld, out, rscale);
    count_launch();
    return cudaGetLastError();
}

void oz_schedule(int n, int grid, std::vector<OzSeg> &segs, std::vector<int> &seg_begin, std::vector<int> &part_base,
                 std::vector<int> &part_count) {
    const int nkb = (n + kKB - 1) / kKB, ntiles = (n + kTileM - 1) / kTileM;
    const long long total = (long long)nkb * ntiles;
    segs.clear();
    seg_begin.assign(grid + 1, 0);
    part_base.assign(ntiles, 0);
    part_count.assign(ntiles, 0);
    // CTA b takes the blocks [total b / grid, total (b + 1) / grid) in (row tile, block) order
    for (int b = 0; b < grid; ++b) {
        long long u0 = total * b / grid;
        const long long u1 = total * (b + 1) / grid;
        while (u0 < u1) {
            const int rt = (int)(u0 / nkb);
            const long long end = std::min(u1, (long long)(rt + 1) * nkb);
            OzSeg s;
            s.rt = rt;
            s.kb0 = (int)(u0 - (long long)rt * nkb);
            s.kb1 = (int)(end - (long long)rt * nkb);
            s.slot = part_count[rt]++;
            segs.push_back(s);
            u0 = end;
        }
        seg_begin[b + 1] = (int)segs.size();
    }
    for (int t = 1; t < ntiles; ++t) part_base[t] = part_base[t - 1] + part_count[t - 1];
}

cudaError_t launch_oz_cheb(const OzLaunch &L, const __nv_bfloat16 *hs_slices, int grid, cudaStream_t st) {
    CUtensorMap m;
    if (make_slice_map(&m, hs_slices, L.N, L.ld)) return cudaErrorInvalidValue;
    const size_t smem = oz_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(oz_cheb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    OzLaunch copy = L;
    void *args[] = {&m, &copy};
    e = cudaLaunchCooperativeKernel((const void *)oz_cheb_kernel, dim3(grid), dim3(kThreads), args, smem, st);
    count_launch();
    return e;
}

}  // namespace elhl
