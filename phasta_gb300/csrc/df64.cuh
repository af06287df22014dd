// df64.cuh -- double-float arithmetic: a value is an unevaluated sum hi + lo of
// two floats (|lo| <= ulp(hi)/2), carrying about 48 significant bits.
//
// GB300 runs FP32 at 64x its FP64 rate, so the few sums that need more than
// FP32 accuracy are done on the FP32 pipe with error-free transformations:
//   two_sum       Knuth, TAOCP vol. 2, 4.2.2 (exact a + b = s + e)
//   quick_two_sum Dekker 1971 (|a| >= |b|)
//   two_prod      exact a * b = p + e with one fused multiply-add
// and Dekker's add2/mul2 built on them.  The additions below have an absolute
// error of ~2^-48 times the larger operand, which is what a sum whose terms
// cancel needs.  The __fadd_rn/__fmul_rn intrinsics are never contracted
// into an FMA, so each rounding step happens as written.
#pragma once

namespace phgpu {

struct df64 {
    float hi, lo;
};

__device__ __forceinline__ df64 df_make(float hi, float lo) { return {hi, lo}; }

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

__device__ __forceinline__ df64 quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df64 df_add(df64 a, df64 b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return quick_two_sum(s, e);
}

__device__ __forceinline__ df64 df_add(df64 a, float b) {
    float s, e;
    two_sum(a.hi, b, s, e);
    e = __fadd_rn(e, a.lo);
    return quick_two_sum(s, e);
}

__device__ __forceinline__ df64 df_neg(df64 a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return quick_two_sum(p, e);
}

__device__ __forceinline__ df64 df_mul(df64 a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return quick_two_sum(p, e);
}

// 1 / b: a float reciprocal refined by one Newton step evaluated in double-float
__device__ __forceinline__ df64 df_rcp(df64 b) {
    const float r = 1.0f / b.hi;
    const float p = __fmul_rn(b.hi, r);
    const float e = __fmaf_rn(b.hi, r, -p);             // b.hi * r = p + e exactly
    // residual 1 - b r = (1 - p) - e - b.lo r
    const float rem = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), e), __fmul_rn(b.lo, r));
    return quick_two_sum(r, __fmul_rn(rem, r));
}

__device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

// (ah + al) - (bh + bl) of two hi/lo pairs, as a double-float
__device__ __forceinline__ df64 df_diff(float ah, float al, float bh, float bl) {
    float s, e;
    two_sum(ah, -bh, s, e);
    e = __fadd_rn(e, __fsub_rn(al, bl));
    return quick_two_sum(s, e);
}

}  // namespace phgpu
