// Inline-PTX helpers of the tcgen05 / TMA kernels (umma_gemm.cu, ozaki.cu):
// mbarriers with bounded waits, TMA tile loads, shared-memory matrix
// descriptors of 128B-swizzled K-major tiles, BF16 MMAs into tensor memory
// (TMEM) and TMEM loads.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace elhl {
namespace tc {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// bounded wait for the phase with the given parity to complete; false once
// limit_ns have passed since t0
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, unsigned long long t0,
                                          unsigned long long limit_ns) {
    const unsigned a = smem_u32(bar);
    while (true) {
        unsigned done = 0;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (now_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
        "[%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

// generic-proxy shared-memory writes made visible to the async proxy (tcgen05.mma operands)
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Shared-memory matrix descriptor of a K-major tile with 128B swizzle: rows of
// 128 B, 8-row atoms of 1024 B (stride byte offset), leading byte offset
// unused, descriptor version 1, layout type 2 (128B swizzle).
__device__ __forceinline__ uint64_t smem_desc_sw128(const void *tile) {
    const uint64_t addr = smem_u32(tile);
    uint64_t d = 0;
    d |= (addr & 0x3FFFFull) >> 4;          // start address, bits 0-13
    d |= (uint64_t)1 << 16;                 // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset, bits 32-45
    d |= (uint64_t)1 << 46;                 // version
    d |= (uint64_t)2 << 61;                 // 128B swizzle
    return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, int accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

// the mbarrier completes a phase once every tcgen05 operation issued so far by this thread has
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 lanes x 32 consecutive FP32 columns of TMEM into registers (no wait)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}

// 32 lanes x 16 consecutive FP32 columns of TMEM into registers (no wait)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Exact slices of the Ozaki scheme: x on the scale 2^e (|x| < 2^e) as 7
// balanced base-256 digits, x 2^-e ~ sum_s n_s 2^(-8 (s+1)) to the nearest
// 2^-56: T = rint(x 2^(56-e)) (round half to even) taken from the bits of x,
// then the digits from the bottom (n_s in [-128, 127] for s >= 1, |n_0| <= 256).
// Integer arithmetic only: GB300's FP64 pipe and its conversions are slow.
__device__ __forceinline__ void slice7(double x, int e, int (&n)[7]) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int be = (int)((b >> 52) & 0x7ff);
    const unsigned long long m = (b & 0xfffffffffffffull) | (be ? (1ull << 52) : 0ull);
    const int sh = (be ? be : 1) - 1075 + 56 - e;  // x = m 2^((be ? be : 1) - 1075), |x 2^(56-e)| < 2^56
    long long T;
    if (sh >= 0) {
        T = (long long)(m << sh);
    } else if (sh > -64) {
        const int k = -sh;
        const unsigned long long q = m >> k, rem = m & ((1ull << k) - 1), half = 1ull << (k - 1);
        T = (long long)(q + ((rem > half || (rem == half && (q & 1))) ? 1ull : 0ull));
    } else {
        T = 0;
    }
    if (b >> 63) T = -T;
#pragma unroll
    for (int s = 6; s >= 1; --s) {
        const int d = (int)(((T + 128) & 255) - 128);
        n[s] = d;
        T = (T - d) >> 8;
    }
    n[0] = (int)T;
}

// exponent e with |x| < 2^e for the finite x != 0 (0 for x = 0), from its bits:
// the biased exponent field minus 1022 (subnormals: -1021)
__device__ __forceinline__ int exp_field(double x) {
    return (int)((__double_as_longlong(x) >> 52) & 0x7ff);
}

}  // namespace tc
}  // namespace elhl
