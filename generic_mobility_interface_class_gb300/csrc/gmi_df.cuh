// gmi_df.cuh -- double-float arithmetic: a value is an unevaluated sum
// h + l of two FP32 numbers with |l| <= ulp(h)/2, about 48 significant
// bits, computed entirely on the FP32 pipe (64x the FP64 throughput per SM
// on this GPU).  The error-free transformations are the published ones:
// Knuth's two-sum, Dekker's fast two-sum (|a| >= |b|) and the FMA-based
// exact product; the compound operations follow the "sloppy" double-double
// add and multiply of Hida, Li and Bailey's QD library, which keep a
// relative error of a few units of 2^-44 when the operands do not cancel.
// Every step uses the _rn intrinsics so that the compiler neither contracts
// nor reorders them.
#pragma once

#include <cuda_runtime.h>

namespace gmi {

struct df2 {
    float h, l;
};

__device__ __forceinline__ df2 df_make(float h) { return df2{h, 0.0f}; }

// a + b exactly as s + e (Knuth)
__device__ __forceinline__ df2 df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df2{s, e};
}

// a + b exactly as s + e, given |a| >= |b| or a == 0 (Dekker)
__device__ __forceinline__ df2 df_fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return df2{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// a * b exactly as p + e (one FMA)
__device__ __forceinline__ df2 df_two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return df2{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df2 df_add(df2 a, df2 b)
{
    const df2 s = df_two_sum(a.h, b.h);
    return df_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

__device__ __forceinline__ df2 df_neg(df2 a) { return df2{-a.h, -a.l}; }

__device__ __forceinline__ df2 df_sub(df2 a, df2 b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df2 df_mul(df2 a, df2 b)
{
    const df2 p = df_two_prod(a.h, b.h);
    float e = __fmaf_rn(a.h, b.l, p.l);
    e = __fmaf_rn(a.l, b.h, e);
    return df_fast_two_sum(p.h, e);
}

__device__ __forceinline__ df2 df_mul_f(df2 a, float b)
{
    const df2 p = df_two_prod(a.h, b);
    return df_fast_two_sum(p.h, __fmaf_rn(a.l, b, p.l));
}

__device__ __forceinline__ df2 df_sqr(df2 a)
{
    const df2 p = df_two_prod(a.h, a.h);
    return df_fast_two_sum(p.h, __fmaf_rn(__fmul_rn(2.0f, a.h), a.l, p.l));
}

// 1/sqrt(x), x > 0: the hardware FP32 estimate y (relative error below
// 2^-22) and one Newton step y (1 + (1 - x y^2)/2), whose residual
// 1 - x y^2 is formed in double-float; the step squares the estimate's
// error, leaving ~2^-44.
__device__ __forceinline__ df2 df_rsqrt(df2 x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x.h));
    const df2 xy2 = df_mul(x, df_two_prod(y, y));
    const float r = __fsub_rn(__fsub_rn(1.0f, xy2.h), xy2.l);  // 1 - xy2.h is exact (xy2.h ~ 1)
    return df_fast_two_sum(y, __fmul_rn(__fmul_rn(0.5f, y), r));
}

// (double)(h + l) -> double-float, and back
__host__ __device__ __forceinline__ df2 df_from_double(double v)
{
    const float h = (float)v;
    return df2{h, (float)(v - (double)h)};
}

__device__ __forceinline__ double df_to_double(df2 a) { return (double)a.h + (double)a.l; }

}  // namespace gmi
