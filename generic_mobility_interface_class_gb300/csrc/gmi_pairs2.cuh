// gmi_pairs2.cuh -- FP32 pair arithmetic on two sources at once.
//
// Every float2 holds one quantity of two sources (lane .x: source j, lane .y:
// source j+1) against the same target, so the whole far-field formula runs
// on the packed FP32 instructions of sm_100+ (fma/add/mul .f32x2: one issue
// slot for two lanes).  The formulas are those of gmi_pairs.cuh (which cites
// the reference kernels); lanes whose pair is in the near field get their
// coefficients from the scalar near-field code there.
//
// Loads: the caller passes every load component already multiplied by
// 1/(8 pi mu) (the far-field prefactor of all four kinds), so the far-field
// coefficients below are pure powers of 1/r; the near-field coefficients,
// which carry their own prefactors, are divided by it again.
//
// Signs: the cross-product terms are accumulated into a separate "minus"
// accumulator (out = plus - minus), which keeps every update a plain
// packed fused multiply-add.
#pragma once

#include <cuda_runtime.h>

#include "gmi_pairs.cuh"

namespace gmi {

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }

// 1/sqrt per lane.  The argument already carries kTinyR2, which keeps it
// normal for the self pair (r^2 = 0): the role of the clamp in rsq<float>.
__device__ __forceinline__ float rsq_raw(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float2 rsq2(float2 x) { return make_float2(rsq_raw(x.x), rsq_raw(x.y)); }

constexpr float kTinyR2 = 1e-30f;

// r^2 + kTinyR2 (the offset rides on the first fused multiply-add).
__device__ __forceinline__ float2 dist2(float2 dx, float2 dy, float2 dz)
{
    return fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, bc2(kTinyR2))));
}

// Near-field fix-ups: out of line (taken by the self pair and overlapping
// particles only), arguments and results by value so that no packed
// coefficient has its address taken (which would move it to local memory on
// the fast path).
struct SSCoeffs {
    float At, Bt, Ar, Br, c3;
};
static __device__ __noinline__ SSCoeffs ss_near2(float r2, float ir, float dF, float dT, EqualK<float> k)
{
    SSCoeffs c;
    ss_near_coeffs<float>(r2, ir, dF, dT, k, c.At, c.Bt, c.Ar, c.Br, c.c3);
    const float u = 1.0f / k.f8pm;
    c.At *= u; c.Bt *= u; c.Ar *= u; c.Br *= u; c.c3 *= u;
    return c;
}

struct UnequalCoeffs {
    float A, Bd, Cd;
};
// The middle and overlapping branches of unequal_coeffs.
static __device__ __noinline__ UnequalCoeffs unequal_near2(float r2, float ir, float dF, UnequalK<float> k)
{
    UnequalCoeffs c;
    unequal_coeffs<float>(r2, ir, dF, k, c.A, c.Bd, c.Cd);
    const float u = 1.0f / k.f8pm;
    c.A *= u; c.Bd *= u; c.Cd *= u;
    return c;
}

// segment <- segment, 6 -> 6 (pair_ss).  F[0..2] force, F[3..5] torque.
// p[0..2] / m[0..2]: velocity plus / minus parts, p[3..5] / m[3..5]: angular.
__device__ __forceinline__ void pair2_ss(float2 dx, float2 dy, float2 dz, const float2 *F, const EqualK<float> &k,
                                         float2 *p, float2 *m)
{
    const float2 r2 = dist2(dx, dy, dz);
    const float2 ir = rsq2(r2);
    const float2 dF = fma2(dz, F[2], fma2(dy, F[1], mul2(dx, F[0])));
    const float2 dT = fma2(dz, F[5], fma2(dy, F[4], mul2(dx, F[3])));
    const float2 ir2 = mul2(ir, ir);
    const float2 ns = mul2(bc2(-k.two_a2), ir2);               // -s = -2a^2/r^2
    float2 At = fma2(mul2(ir, ns), bc2(-1.0f / 3.0f), ir);     // (1 + s/3) / r
    float2 c3 = mul2(ir, ir2);                                 // 1/r^3
    const float2 c3dF = mul2(c3, dF);
    float2 Bt = fma2(ns, c3dF, c3dF);                          // (1 - s) dF / r^3
    float2 Ar = mul2(bc2(-0.5f), c3);                          // -1/(2 r^3)
    float2 Br = mul2(mul2(c3, ir2), mul2(bc2(1.5f), dT));      // 3 dT / (2 r^5)
    if (!(fminf(r2.x, r2.y) > k.four_a2)) {  // one test per step; near pairs are rare
        if (!(r2.x > k.four_a2)) {
            const SSCoeffs c = ss_near2(r2.x, ir.x, dF.x, dT.x, k);
            At.x = c.At; Bt.x = c.Bt; Ar.x = c.Ar; Br.x = c.Br; c3.x = c.c3;
        }
        if (!(r2.y > k.four_a2)) {
            const SSCoeffs c = ss_near2(r2.y, ir.y, dF.y, dT.y, k);
            At.y = c.At; Bt.y = c.Bt; Ar.y = c.Ar; Br.y = c.Br; c3.y = c.c3;
        }
    }
    const float2 cx = mul2(c3, dx), cy = mul2(c3, dy), cz = mul2(c3, dz);
    p[0] = fma2(At, F[0], p[0]); p[0] = fma2(Bt, dx, p[0]); p[0] = fma2(F[4], cz, p[0]); m[0] = fma2(F[5], cy, m[0]);
    p[1] = fma2(At, F[1], p[1]); p[1] = fma2(Bt, dy, p[1]); p[1] = fma2(F[5], cx, p[1]); m[1] = fma2(F[3], cz, m[1]);
    p[2] = fma2(At, F[2], p[2]); p[2] = fma2(Bt, dz, p[2]); p[2] = fma2(F[3], cy, p[2]); m[2] = fma2(F[4], cx, m[2]);
    p[3] = fma2(Ar, F[3], p[3]); p[3] = fma2(Br, dx, p[3]); p[3] = fma2(F[1], cz, p[3]); m[3] = fma2(F[2], cy, m[3]);
    p[4] = fma2(Ar, F[4], p[4]); p[4] = fma2(Br, dy, p[4]); p[4] = fma2(F[2], cx, p[4]); m[4] = fma2(F[0], cz, m[4]);
    p[5] = fma2(Ar, F[5], p[5]); p[5] = fma2(Br, dz, p[5]); p[5] = fma2(F[0], cy, p[5]); m[5] = fma2(F[1], cx, m[5]);
}

// blob <- blob, 3 -> 3 (pair_bb).  No minus part.
__device__ __forceinline__ void pair2_bb(float2 dx, float2 dy, float2 dz, const float2 *F, const EqualK<float> &k,
                                         float2 *p)
{
    const float2 r2 = dist2(dx, dy, dz);
    const float2 ir = rsq2(r2);
    const float2 dF = fma2(dz, F[2], fma2(dy, F[1], mul2(dx, F[0])));
    const float2 ir2 = mul2(ir, ir);
    const float2 ns = mul2(bc2(-k.two_a2), ir2);
    float2 At = fma2(mul2(ir, ns), bc2(-1.0f / 3.0f), ir);
    const float2 c3dF = mul2(mul2(ir, ir2), dF);
    float2 Bt = fma2(ns, c3dF, c3dF);
    if (!(fminf(r2.x, r2.y) > k.four_a2)) {
        if (!(r2.x > k.four_a2)) {
            const float q = r2.x * ir.x * k.q32, u = k.f6pma / k.f8pm;
            At.x = (1.0f - 3.0f * q) * u;
            Bt.x = q * u * (ir.x * ir.x) * dF.x;
        }
        if (!(r2.y > k.four_a2)) {
            const float q = r2.y * ir.y * k.q32, u = k.f6pma / k.f8pm;
            At.y = (1.0f - 3.0f * q) * u;
            Bt.y = q * u * (ir.y * ir.y) * dF.y;
        }
    }
    p[0] = fma2(At, F[0], p[0]); p[0] = fma2(Bt, dx, p[0]);
    p[1] = fma2(At, F[1], p[1]); p[1] = fma2(Bt, dy, p[1]);
    p[2] = fma2(At, F[2], p[2]); p[2] = fma2(Bt, dz, p[2]);
}

// Far-field unequal-radius coefficients (first branch of unequal_coeffs) on
// both lanes, then the other branches for the lanes that need them.
__device__ __forceinline__ void unequal_coeffs2(float2 r2, float2 ir, float2 dF, const UnequalK<float> &k, float2 &A,
                                                float2 &Bd, float2 &Cd)
{
    const float2 ir2 = mul2(ir, ir);
    const float2 t = mul2(ir2, bc2(k.far_c));                 // (as^2 + ab^2) / (3 r^2)
    A = fma2(t, ir, ir);                                      // (1 + t) / r
    Cd = mul2(ir, ir2);                                       // 1/r^3
    Bd = mul2(mul2(fma2(t, bc2(-3.0f), bc2(1.0f)), Cd), dF);  // (1 - 3t) dF / r^3
    if (!(fminf(r2.x, r2.y) > k.sum2)) {
        if (!(r2.x > k.sum2)) {
            const UnequalCoeffs c = unequal_near2(r2.x, ir.x, dF.x, k);
            A.x = c.A; Bd.x = c.Bd; Cd.x = c.Cd;
        }
        if (!(r2.y > k.sum2)) {
            const UnequalCoeffs c = unequal_near2(r2.y, ir.y, dF.y, k);
            A.y = c.A; Bd.y = c.Bd; Cd.y = c.Cd;
        }
    }
}

// segment <- blob force, 3 -> 6 (pair_sb).
__device__ __forceinline__ void pair2_sb(float2 dx, float2 dy, float2 dz, const float2 *F, const UnequalK<float> &k,
                                         float2 *p, float2 *m)
{
    const float2 r2 = dist2(dx, dy, dz);
    const float2 ir = rsq2(r2);
    const float2 dF = fma2(dz, F[2], fma2(dy, F[1], mul2(dx, F[0])));
    float2 A, Bd, Cd;
    unequal_coeffs2(r2, ir, dF, k, A, Bd, Cd);
    const float2 cx = mul2(Cd, dx), cy = mul2(Cd, dy), cz = mul2(Cd, dz);
    p[0] = fma2(A, F[0], p[0]); p[0] = fma2(Bd, dx, p[0]);
    p[1] = fma2(A, F[1], p[1]); p[1] = fma2(Bd, dy, p[1]);
    p[2] = fma2(A, F[2], p[2]); p[2] = fma2(Bd, dz, p[2]);
    p[3] = fma2(F[1], cz, p[3]); m[3] = fma2(F[2], cy, m[3]);
    p[4] = fma2(F[2], cx, p[4]); m[4] = fma2(F[0], cz, m[4]);
    p[5] = fma2(F[0], cy, p[5]); m[5] = fma2(F[1], cx, m[5]);
}

// blob <- segment force and torque, 6 -> 3 (pair_bs).
__device__ __forceinline__ void pair2_bs(float2 dx, float2 dy, float2 dz, const float2 *F, const UnequalK<float> &k,
                                         float2 *p, float2 *m)
{
    const float2 r2 = dist2(dx, dy, dz);
    const float2 ir = rsq2(r2);
    const float2 dF = fma2(dz, F[2], fma2(dy, F[1], mul2(dx, F[0])));
    float2 A, Bd, Cd;
    unequal_coeffs2(r2, ir, dF, k, A, Bd, Cd);
    const float2 cx = mul2(Cd, dx), cy = mul2(Cd, dy), cz = mul2(Cd, dz);
    p[0] = fma2(A, F[0], p[0]); p[0] = fma2(Bd, dx, p[0]); p[0] = fma2(F[4], cz, p[0]); m[0] = fma2(F[5], cy, m[0]);
    p[1] = fma2(A, F[1], p[1]); p[1] = fma2(Bd, dy, p[1]); p[1] = fma2(F[5], cx, p[1]); m[1] = fma2(F[3], cz, m[1]);
    p[2] = fma2(A, F[2], p[2]); p[2] = fma2(Bd, dz, p[2]); p[2] = fma2(F[3], cy, p[2]); m[2] = fma2(F[4], cx, m[2]);
}

}  // namespace gmi
