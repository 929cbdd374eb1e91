// Double-float (DF64) arithmetic on the FP32 pipes.  A value is the unevaluated
// sum hi + lo of two FP32 numbers (48-bit significand, about 4e-15 relative).
// Products use Dekker's exact product error by FMA, sums Knuth's TwoSum; every
// step is a round-to-nearest intrinsic so that the compiler contracts nothing.
// GB300's FP64 pipe runs at 1/58 of its FP32 rate, so about a dozen FP32
// instructions per FP64-equivalent operation still leaves DF64 5x ahead.
#pragma once

#include <cuda_runtime.h>

namespace elhl {

__device__ __forceinline__ float2 df_split(double x) {
    const float h = __double2float_rn(x);
    return make_float2(h, __double2float_rn(x - (double)h));
}

__device__ __forceinline__ double df_value(float2 a) { return (double)a.x + (double)a.y; }

// (sh, sl) += (ah + al)(bh + bl), dropping al bl (2^-48 relative)
__device__ __forceinline__ void df_fma(float &sh, float &sl, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float t = __fadd_rn(sh, p);
    const float z = __fsub_rn(t, sh);
    const float y = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z));
    sl = __fadd_rn(sl, __fadd_rn(y, e));
    sh = t;
}

// (ah, al) + (bh, bl) in FP32 pairs (TwoSum of the high parts, low parts added)
__device__ __forceinline__ void df_add(float &ah, float &al, float bh, float bl) {
    const float t = __fadd_rn(ah, bh);
    const float z = __fsub_rn(t, ah);
    const float y = __fadd_rn(__fsub_rn(ah, __fsub_rn(t, z)), __fsub_rn(bh, z));
    al = __fadd_rn(al, __fadd_rn(y, bl));
    ah = t;
}

// the same value with |lo| <= ulp(hi) / 2 (TwoSum, exact for any h and l)
__device__ __forceinline__ float2 df_renorm(float h, float l) {
    const float s = __fadd_rn(h, l);
    const float z = __fsub_rn(s, h);
    return make_float2(s, __fadd_rn(__fsub_rn(h, __fsub_rn(s, z)), __fsub_rn(l, z)));
}

// a b, normalised
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return df_renorm(p, e);
}

// a + b, normalised
__device__ __forceinline__ float2 df_sum(float2 a, float2 b) {
    df_add(a.x, a.y, b.x, b.y);
    return df_renorm(a.x, a.y);
}

// 1 / sqrt(d) for d > 0: the FP32 estimate y0 = rsqrtf(d_hi) (about 2^-22
// relative), then with the residual r = 1 - d y0^2 formed in double-float,
// y0 (1 - r)^-1/2 = y0 (1 + r/2 + 3 r^2/8 + ...) to second order: the dropped
// term is about 2^-62, the result accurate to the pair's rounding
__device__ __forceinline__ float2 df_rsqrt(float2 d) {
    const float y0 = rsqrtf(d.x);
    const float p = __fmul_rn(y0, y0);
    const float2 y2 = make_float2(p, __fmaf_rn(y0, y0, -p));  // y0^2 exactly
    const float2 dy2 = df_mul(d, y2);
    const float2 res = df_sum(make_float2(1.f, 0.f), make_float2(-dy2.x, -dy2.y));  // r
    const float r = __fadd_rn(res.x, res.y);
    const float corr = __fmul_rn(__fmul_rn(0.5f, y0), __fmul_rn(r, __fmaf_rn(0.75f, r, 1.f)));
    return df_renorm(y0, corr);
}

}  // namespace elhl
