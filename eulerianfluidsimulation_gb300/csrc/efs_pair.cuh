// efs_pair.cuh — values held as a pair of floats (hi + lo, |lo| at most half an ulp of hi: about 48 significant
// bits) and computed on the FP32 pipe with error-free transformations.  GB300 runs FP64 at a small fraction of
// its FP32 rate; the solvers' extended-precision accumulators (CG's residual replacement, FCG's x) use these.
// Every operation is written with explicitly rounded intrinsics, so no FMA contraction can change the
// transformations.
#pragma once

#include <cuda_runtime.h>

namespace efs {

// s + e = a + b exactly, s = fl(a + b)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ float2 df_renorm(float s, float e) {
    const float hi = __fadd_rn(s, e);
    return make_float2(hi, __fsub_rn(e, __fsub_rn(hi, s)));
}
__device__ __forceinline__ float2 df_add(float2 x, float2 y) {
    float s, e;
    two_sum(x.x, y.x, s, e);
    return df_renorm(s, __fadd_rn(e, __fadd_rn(x.y, y.y)));
}
__device__ __forceinline__ float2 df_add_f(float2 x, float y) {
    float s, e;
    two_sum(x.x, y, s, e);
    return df_renorm(s, __fadd_rn(e, x.y));
}
__device__ __forceinline__ float2 df_neg(float2 x) { return make_float2(-x.x, -x.y); }
// x times a small integer k (a diagonal count): the product's rounding error by FMA
__device__ __forceinline__ float2 df_mul_k(float2 x, float k) {
    const float ph = __fmul_rn(k, x.x);
    return df_renorm(ph, fmaf(k, x.y, fmaf(k, x.x, -ph)));
}
// x + (ah + al) d
__device__ __forceinline__ float2 df_axpy(float2 x, float ah, float al, float d) {
    const float p = __fmul_rn(ah, d);
    const float pe = fmaf(al, d, fmaf(ah, d, -p));
    float s, t;
    two_sum(x.x, p, s, t);
    return df_renorm(s, __fadd_rn(__fadd_rn(t, x.y), pe));
}
__device__ __forceinline__ double df_val(float2 x) { return (double)x.x + (double)x.y; }

}  // namespace efs
