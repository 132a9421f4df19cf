// Scalar arithmetic of the bulge chases (stage2_chase.cu, stage2_window.cu):
// FP64, or double-float pairs stored as float2 (df64.cuh).
#pragma once

#include <cuda_runtime.h>

#include "df64.cuh"

namespace avs {

// Scalar arithmetic of the chase: FP64, or double-float pairs stored as float2.
template <typename S>
struct ChaseAr;

template <>
struct ChaseAr<double> {
    using V = double;   // register value
    using St = double;  // storage element
    static __device__ __forceinline__ V zero() { return 0.0; }
    static __device__ __forceinline__ V one() { return 1.0; }
    static __device__ __forceinline__ V ld(const St *p) { return __ldcg(p); }
    static __device__ __forceinline__ V lds(const St *p) { return *p; }  // plain (shared memory) load
    static __device__ __forceinline__ void st(St *p, V v) { *p = v; }
    static __device__ __forceinline__ V add(V a, V b) { return a + b; }
    static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
    static __device__ __forceinline__ V mul(V a, V b) { return a * b; }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return ::fma(a, b, c); }
    static __device__ __forceinline__ V neg(V a) { return -a; }
    static __device__ __forceinline__ V div(V a, V b) { return a / b; }
    static __device__ __forceinline__ V sqrt(V a) { return ::sqrt(a); }
    static __device__ __forceinline__ bool ge0(V a) { return a >= 0.0; }
    static __device__ __forceinline__ bool gt0(V a) { return a > 0.0; }
    static __device__ __forceinline__ bool iszero(V a) { return a == 0.0; }
    static __device__ __forceinline__ V shfl_xor(V a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
    static __device__ __forceinline__ V shfl(V a, int src) { return __shfl_sync(0xffffffffu, a, src); }
    static __device__ __forceinline__ V rcp(V a) { return 1.0 / a; }
    static __device__ __forceinline__ double to_double(V a) { return a; }
    static __device__ __forceinline__ St from_double(double a) { return a; }
    static __device__ __forceinline__ V v_from_double(double a) { return a; }
    // dot-product accumulator: plain FMA chain
    using Acc = double;
    static __device__ __forceinline__ Acc acc_zero() { return 0.0; }
    static __device__ __forceinline__ void acc_add(Acc &a, V x, V y) { a = ::fma(x, y, a); }
    static __device__ __forceinline__ V acc_value(Acc a) { return a; }
};

template <>
struct ChaseAr<df64> {
    using V = df64;
    using St = float2;
    static __device__ __forceinline__ V zero() { return df64{0.0f, 0.0f}; }
    static __device__ __forceinline__ V one() { return df64{1.0f, 0.0f}; }
    static __device__ __forceinline__ V ld(const St *p) {
        const float2 v = __ldcg(p);
        return df64{v.x, v.y};
    }
    static __device__ __forceinline__ V lds(const St *p) {
        const float2 v = *p;
        return df64{v.x, v.y};
    }
    static __device__ __forceinline__ void st(St *p, V v) { *p = make_float2(v.hi, v.lo); }
    static __device__ __forceinline__ V add(V a, V b) { return df_add(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return df_sub(a, b); }
    static __device__ __forceinline__ V mul(V a, V b) { return df_mul(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return df_add(df_mul(a, b), c); }
    static __device__ __forceinline__ V neg(V a) { return df_neg(a); }
    static __device__ __forceinline__ V div(V a, V b) { return df_div(a, b); }
    static __device__ __forceinline__ V sqrt(V a) { return df_sqrt(a); }
    static __device__ __forceinline__ bool ge0(V a) { return !df_lt0(a); }
    static __device__ __forceinline__ bool gt0(V a) { return a.hi > 0.0f || (a.hi == 0.0f && a.lo > 0.0f); }
    static __device__ __forceinline__ bool iszero(V a) { return a.hi == 0.0f && a.lo == 0.0f; }
    static __device__ __forceinline__ V shfl_xor(V a, int o) {
        return df64{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
    }
    static __device__ __forceinline__ V shfl(V a, int src) {
        return df64{__shfl_sync(0xffffffffu, a.hi, src), __shfl_sync(0xffffffffu, a.lo, src)};
    }
    static __device__ __forceinline__ V rcp(V a) { return df_rcp(a); }
    static __device__ __forceinline__ double to_double(V a) { return df_to_double(a); }
    // Dot-product accumulator in compensated FP32 (Ogita, Rump & Oishi,
    // "Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005), Dot2):
    // s carries the running FP32 sum, c the exact rounding errors of the sums
    // and of the double-float products; the loop-carried chain is one add.
    struct Acc {
        float s, c;
    };
    static __device__ __forceinline__ Acc acc_zero() { return Acc{0.0f, 0.0f}; }
    static __device__ __forceinline__ void acc_add(Acc &a, V x, V y) {
        const float p = __fmul_rn(x.hi, y.hi);
        float ep = __fmaf_rn(x.hi, y.hi, -p);
        ep = __fmaf_rn(x.hi, y.lo, ep);
        ep = __fmaf_rn(x.lo, y.hi, ep);
        const float t = __fadd_rn(a.s, p);
        const float z = __fsub_rn(t, a.s);
        const float es = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, z)), __fsub_rn(p, z));
        a.s = t;
        a.c = __fadd_rn(a.c, __fadd_rn(es, ep));
    }
    static __device__ __forceinline__ V acc_value(Acc a) { return two_sum(a.s, a.c); }
    static __device__ __forceinline__ St from_double(double a) {
        const df64 v = df_from_double(a);
        return make_float2(v.hi, v.lo);
    }
    static __device__ __forceinline__ V v_from_double(double a) { return df_from_double(a); }
};

__device__ __forceinline__ double st_to_double(double v) { return v; }
__device__ __forceinline__ double st_to_double(float2 v) { return (double)v.x + (double)v.y; }

}  // namespace avs
