// Double-float ("df64") arithmetic: a value is the unevaluated sum hi + lo of
// two FP32 numbers (|lo| <= ulp(hi)/2), giving ~44-48 significant bits on the
// FP32 pipe.  GB300 issues FP64 at 1/64 of the FP32 rate, so the FP64-class
// stages (bulge chase, bisection) run their inner loops in this format.
//
// Error-free transformations: TwoSum (Knuth, TAOCP vol. 2), FastTwoSum
// (Dekker 1971), TwoProduct with a fused multiply-add; the composite
// operations follow Hida, Li & Bailey, "Library for double-double and
// quad-double arithmetic" (2007), "sloppy" variants.  The exponent range is
// FP32's: callers keep their data normalised.
#pragma once

#include <cuda_runtime.h>

namespace avs {

struct df64 {
    float hi, lo;
};

__device__ __forceinline__ df64 df_make(float h, float l) { return df64{h, l}; }

__device__ __forceinline__ df64 df_from_double(double x) {
    const float h = (float)x;
    return df64{h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

// |a| >= |b| (or a == 0): s + e == a + b exactly
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return df64{s, e};
}
__device__ __forceinline__ df64 two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df64{s, e};
}
__device__ __forceinline__ df64 two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return df64{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df64 df_add(df64 a, df64 b) {
    df64 s = two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 df_neg(df64 a) { return df64{-a.hi, -a.lo}; }
__device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
    df64 p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df64 df_mul_f(df64 a, float b) {
    df64 p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
// a * b + c
__device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c) { return df_add(df_mul(a, b), c); }

// 1 / a: FP32 reciprocal estimate refined by one Newton-Raphson step in df64,
// r' = r + r (1 - a r).
__device__ __forceinline__ df64 df_rcp(df64 a) {
    const float r = __frcp_rn(a.hi);
    // e = 1 - a * r, computed in df64
    df64 ar = df_mul_f(a, r);
    df64 e = df_sub(df64{1.0f, 0.0f}, ar);
    return df_add(df64{r, 0.0f}, df_mul_f(e, r));
}
__device__ __forceinline__ df64 df_div(df64 a, df64 b) { return df_mul(a, df_rcp(b)); }

// sqrt(a), a >= 0: FP32 estimate s, one Newton step s' = s + (a - s^2) / (2 s).
__device__ __forceinline__ df64 df_sqrt(df64 a) {
    if (a.hi <= 0.0f) return df64{0.0f, 0.0f};
    const float s = __fsqrt_rn(a.hi);
    const df64 s2 = two_prod(s, s);
    const df64 r = df_sub(a, s2);
    return fast_two_sum(s, __fdiv_rn(r.hi, 2.0f * s));
}

__device__ __forceinline__ bool df_lt0(df64 a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f); }
__device__ __forceinline__ float df_abs_hi(df64 a) { return fabsf(a.hi); }

// A double-float value with arithmetic operators: the compute type of kernels
// templated on their element type when the data is stored in FP64 (converted
// on load, ~48 of the 53 significant bits kept, FP32's exponent range; rounded
// back to FP64 on store).
struct dfx {
    df64 v;
    __device__ __forceinline__ dfx() {}
    __device__ __forceinline__ dfx(int x) : v(df64{(float)x, 0.0f}) {}
    __device__ __forceinline__ explicit dfx(double x) : v(df_from_double(x)) {}
    __device__ __forceinline__ explicit dfx(df64 x) : v(x) {}
    __device__ __forceinline__ explicit operator double() const { return df_to_double(v); }
};
__device__ __forceinline__ dfx operator+(dfx a, dfx b) { return dfx(df_add(a.v, b.v)); }
__device__ __forceinline__ dfx operator-(dfx a, dfx b) { return dfx(df_sub(a.v, b.v)); }
__device__ __forceinline__ dfx operator*(dfx a, dfx b) { return dfx(df_mul(a.v, b.v)); }
__device__ __forceinline__ dfx operator-(dfx a) { return dfx(df_neg(a.v)); }
__device__ __forceinline__ dfx &operator+=(dfx &a, dfx b) { return a = a + b; }
__device__ __forceinline__ dfx &operator-=(dfx &a, dfx b) { return a = a - b; }
__device__ __forceinline__ bool operator==(dfx a, dfx b) { return a.v.hi == b.v.hi && a.v.lo == b.v.lo; }
__device__ __forceinline__ bool operator!=(dfx a, dfx b) { return !(a == b); }

}  // namespace avs
