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

}  // namespace elhl
