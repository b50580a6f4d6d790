// tpal_common.cuh -- shared device helpers for the Transform-PAL kernels.
//
// Double-float ("df") arithmetic: a value is hi + lo with |lo| <= ulp(hi)/2,
// about 44 significant bits, built from FP32 error-free transformations
// (Knuth two-sum, FMA two-product). The kernels use it only on the rare
// threshold decisions whose FP32 margin is inside the error bound, so those
// decisions match an FP64 evaluation of the same spectrum.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tpal {

// Paired FP32 (sm_100+): each lane of the pair rounds exactly like the scalar op.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_make(float a) { return {a, 0.0f}; }

__device__ __forceinline__ df quick_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ df df_add(df x, df y)
{
    const df s = two_sum(x.hi, y.hi);
    const df t = two_sum(x.lo, y.lo);
    float e = __fadd_rn(s.lo, t.hi);
    df r = quick_two_sum(s.hi, e);
    e = __fadd_rn(t.lo, r.lo);
    return quick_two_sum(r.hi, e);
}

__device__ __forceinline__ df df_neg(df x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ df df_mul(df x, df y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return quick_two_sum(p, e);
}

// x * f where f is exactly representable (e.g. an integer sample value)
__device__ __forceinline__ df df_mul_f(df x, float f)
{
    const float p = __fmul_rn(x.hi, f);
    float e = __fmaf_rn(x.hi, f, -p);
    e = __fmaf_rn(x.lo, f, e);
    return quick_two_sum(p, e);
}

struct dfc {
    df re, im;
};

__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b)
{
    return {df_sub(df_mul(a.re, b.re), df_mul(a.im, b.im)), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}

__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }

__device__ __forceinline__ df df_shfl_xor(df v, int mask)
{
    return {__shfl_xor_sync(0xffffffffu, v.hi, mask), __shfl_xor_sync(0xffffffffu, v.lo, mask)};
}

__device__ __forceinline__ dfc dfc_shfl_xor(dfc v, int mask) { return {df_shfl_xor(v.re, mask), df_shfl_xor(v.im, mask)}; }

// sign of a double-float value: -1, 0, +1
__device__ __forceinline__ int df_sign(df x)
{
    if (x.hi > 0.0f) return 1;
    if (x.hi < 0.0f) return -1;
    if (x.lo > 0.0f) return 1;
    if (x.lo < 0.0f) return -1;
    return 0;
}

__device__ __forceinline__ int rev4(int i)
{
    return ((i & 1) << 3) | ((i & 2) << 1) | ((i & 4) >> 1) | ((i & 8) >> 3);
}

}  // namespace tpal
