// gmi_pairs.cuh -- per-pair RPY arithmetic, templated on the scalar type.
//
// Each function adds the contribution of one source j to one target i,
// given d = x_i - x_j.  The formulas and their near/far branches restate the
// reference kernels (cuda_functions.cu, line ranges on each function); the
// self pair (d = 0) takes the near-field branch with r = 0, which is what
// the reference's r + 1e-20 guard produces (cuda_functions.cu:307).
#pragma once

#include <cuda_runtime.h>

namespace gmi {

template <class R> __device__ __forceinline__ R rsq(R x);
// FP32: the hardware approximate reciprocal square root (PTX rsqrt.approx,
// relative error below 2^-22.9), flushing denormals; the clamp keeps the
// argument normal (the self pair has r^2 = 0).
template <> __device__ __forceinline__ float rsq<float>(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(fmaxf(x, 1e-30f)));
    return y;
}
template <> __device__ __forceinline__ double rsq<double>(double x) { return rsqrt(fmax(x, 1e-300)); }

// Equal-radius constants (segment<-segment with a = a_seg, blob<-blob with a = a_blob).
template <class R> struct EqualK {
    R four_a2, two_a2, f8pm, f6pma, q32, inv_a, f8pma3, f16pma3, q8;
};

// Unequal-radius constants for segment<->blob pairs (radii as, ab).
template <class R> struct UnequalK {
    R sum2, dmin2, far_c, half_sum, f8pm, f6pmab, fmax, c_mid_den, ab, as, ab2, inner_c, dmin;
};

// The pair formulas below are the reference's, rewritten in terms of the
// separation d = x_i - x_j instead of the unit vector e = d/r: every power
// of 1/r is folded into the scalar coefficients, so a pair costs one
// reciprocal square root and its accumulation is a chain of fused
// multiply-adds.  Near/far is decided on r^2.

// translation<-force, rotation<-torque and the two cross couplings, equal
// radii: cuda_functions.cu:315-398.
//   v += At F + Bt d + c3 (T x d),   w += Ar T + Br d + c3 (F x d)
// Near-field (overlapping, r <= 2a) coefficients of pair_ss, out of line:
// the branch is taken only by the self pair and overlapping particles, and a
// real branch keeps its arithmetic off the issue slots of every other pair.
template <class R>
__device__ __noinline__ void ss_near_coeffs(R r2, R ir, R dF, R dT, const EqualK<R> &k, R &At, R &Bt, R &Ar, R &Br,
                                            R &c3)
{
    const R r = r2 * ir;
    const R ir2 = ir * ir;
    const R q = r * k.q32;                      // 3r/(32a)
    At = (R(1) - R(3) * q) * k.f6pma;
    Bt = q * k.f6pma * ir2 * dF;
    const R ra = r * k.inv_a;
    const R ra3 = ra * ra * ra;
    const R b = R(9.0 / 32.0) * ra;
    Ar = (R(-3) * b + (R(1) + R(5.0 / 64.0) * ra3)) * k.f8pma3;
    Br = (b - R(3.0 / 64.0) * ra3) * k.f8pma3 * ir2 * dT;
    c3 = r * (R(1) - r * k.q8) * k.f16pma3 * ir;
}

template <class R>
__device__ __forceinline__ void pair_ss(R dx, R dy, R dz, const R *F, const EqualK<R> &k, R *v, R *w)
{
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R ir = rsq<R>(r2);
    const R dF = dx * F[0] + dy * F[1] + dz * F[2];
    const R dT = dx * F[3] + dy * F[4] + dz * F[5];
    R At, Bt, Ar, Br, c3;
    if (r2 > k.four_a2) {
        const R ir2 = ir * ir;
        const R ir3 = ir2 * ir;
        const R s = k.two_a2 * ir2;                 // 2a^2/r^2
        const R ik = ir * k.f8pm;                   // 1/(8 pi mu r)
        At = ik * (R(1) + s * R(1.0 / 3.0));
        c3 = ir3 * k.f8pm;
        const R c3dF = c3 * dF;
        Bt = c3dF - s * c3dF;                       // (1 - s) dF / (8 pi mu r^3)
        Ar = R(-0.5) * c3;                          // -1/(16 pi mu r^3)
        Br = (R(1.5) * c3 * ir2) * dT;              // 3 dT / (16 pi mu r^5)
    } else {
        ss_near_coeffs<R>(r2, ir, dF, dT, k, At, Bt, Ar, Br, c3);
    }
    const R cx = c3 * dx, cy = c3 * dy, cz = c3 * dz;
    v[0] += At * F[0] + Bt * dx + F[4] * cz - F[5] * cy;
    v[1] += At * F[1] + Bt * dy + F[5] * cx - F[3] * cz;
    v[2] += At * F[2] + Bt * dz + F[3] * cy - F[4] * cx;
    w[0] += Ar * F[3] + Br * dx + F[1] * cz - F[2] * cy;
    w[1] += Ar * F[4] + Br * dy + F[2] * cx - F[0] * cz;
    w[2] += Ar * F[5] + Br * dz + F[0] * cy - F[1] * cx;
}

// translation<-force, equal radii: cuda_functions.cu:465-520.
template <class R>
__device__ __forceinline__ void pair_bb(R dx, R dy, R dz, const R *F, const EqualK<R> &k, R *v)
{
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R ir = rsq<R>(r2);
    const R dF = dx * F[0] + dy * F[1] + dz * F[2];
    R At, Bt;
    if (r2 > k.four_a2) {
        const R ir2 = ir * ir;
        const R s = k.two_a2 * ir2;
        const R ik = ir * k.f8pm;
        At = ik * (R(1) + s * R(1.0 / 3.0));
        const R c3dF = ik * ir2 * dF;
        Bt = c3dF - s * c3dF;
    } else {
        const R r = r2 * ir;
        const R q = r * k.q32;
        At = (R(1) - R(3) * q) * k.f6pma;
        Bt = q * k.f6pma * (ir * ir) * dF;
    }
    v[0] += At * F[0] + Bt * dx;
    v[1] += At * F[1] + Bt * dy;
    v[2] += At * F[2] + Bt * dz;
}

// Unequal-radius coefficients, cuda_functions.cu:608-667 (segment<-blob) and
// :770-829 (blob<-segment), which share the same expressions in (RSEG, RBLOB):
//   A (of F), Bd (of d, already times d.F), Cd (of the cross product with d).
template <class R>
__device__ __forceinline__ void unequal_coeffs(R r2, R ir, R dF, const UnequalK<R> &k, R &A, R &Bd, R &Cd)
{
    const R ir2 = ir * ir;
    if (r2 > k.sum2) {
        const R t = ir2 * k.far_c;  // (as^2 + ab^2) / (3 r^2)
        const R ik = ir * k.f8pm;
        A = (t + R(1)) * ik;
        Cd = ik * ir2;
        Bd = (R(1) - R(3) * t) * Cd * dF;
    } else if (r2 > k.dmin2) {
        const R r = r2 * ir;
        const R id3 = R(1.0 / 32.0) * ir2 * ir;  // 1/(32 r^3)
        const R t = k.dmin2 + R(3) * r2;
        A = (k.half_sum - t * t * id3) * k.f6pmab;
        const R b = k.dmin2 - r2;
        Bd = R(3) * b * b * id3 * k.f6pmab * ir2 * dF;
        const R u = k.as - k.ab + r;
        const R p = k.ab2 + R(2) * k.ab * (r + k.as) - R(3) * (k.as - r) * (k.as - r);
        Cd = ir2 * u * u * p * k.c_mid_den * ir;
    } else {
        A = k.fmax;
        Bd = R(0);
        Cd = k.inner_c * (r2 * ir) * ir;
    }
}

// segment <- blob force (3 -> 6): cuda_functions.cu:582-667.
template <class R>
__device__ __forceinline__ void pair_sb(R dx, R dy, R dz, const R *F, const UnequalK<R> &k, R *v, R *w)
{
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R ir = rsq<R>(r2);
    const R dF = dx * F[0] + dy * F[1] + dz * F[2];
    R A, Bd, Cd;
    unequal_coeffs<R>(r2, ir, dF, k, A, Bd, Cd);
    const R cx = Cd * dx, cy = Cd * dy, cz = Cd * dz;
    v[0] += A * F[0] + Bd * dx;
    v[1] += A * F[1] + Bd * dy;
    v[2] += A * F[2] + Bd * dz;
    w[0] += F[1] * cz - F[2] * cy;
    w[1] += F[2] * cx - F[0] * cz;
    w[2] += F[0] * cy - F[1] * cx;
}

// blob <- segment force and torque (6 -> 3): cuda_functions.cu:744-829.
template <class R>
__device__ __forceinline__ void pair_bs(R dx, R dy, R dz, const R *F, const UnequalK<R> &k, R *v)
{
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R ir = rsq<R>(r2);
    const R dF = dx * F[0] + dy * F[1] + dz * F[2];
    R A, Bd, Cd;
    unequal_coeffs<R>(r2, ir, dF, k, A, Bd, Cd);
    const R cx = Cd * dx, cy = Cd * dy, cz = Cd * dz;
    v[0] += A * F[0] + Bd * dx + F[4] * cz - F[5] * cy;
    v[1] += A * F[1] + Bd * dy + F[5] * cx - F[3] * cz;
    v[2] += A * F[2] + Bd * dz + F[3] * cy - F[4] * cx;
}

// Segment <- segment above a no-slip wall at z = 0, a = mu = 1 (Swan & Brady):
// cuda_functions.cu:78-229.  dx, dy are x_i - x_j; zi, zj the heights; self
// marks i == j.  The wall-image rotation/translation coupling uses the
// reference's sign convention (cuda_functions.cu:13-20).
template <class R>
__device__ __forceinline__ void pair_ss_wall(R dx, R dy, R dz, R zs, R zi, R zj, bool self, const R *F,
                                             R *v, R *w)
{
    const R K6 = R(1.0 / (6.0 * 3.14159265358979323846));
    const R K8 = R(1.0 / (8.0 * 3.14159265358979323846));
    const R K16 = R(1.0 / (16.0 * 3.14159265358979323846));
    const R fx = F[0], fy = F[1], fz = F[2], tx = F[3], ty = F[4], tz = F[5];
    if (self) {
        const R h1 = R(1) / zi, h3 = h1 * h1 * h1, h4 = h3 * h1, h5 = h4 * h1;
        R p = K6 - (R(9) * h1 - R(2) * h3 + h5) * (K6 * R(1.0 / 16.0));
        R q = K6 - (R(9) * h1 - R(4) * h3 + h5) * (K6 * R(1.0 / 8.0));
        const R c = (K6 * R(3.0 / 32.0)) * h4;
        v[0] += p * fx + c * ty;
        v[1] += p * fy - c * tx;
        v[2] += q * fz;
        p = K8 - (K6 * R(15.0 / 64.0)) * h3;
        q = K8 - (K6 * R(3.0 / 32.0)) * h3;
        w[0] += p * tx - c * fy;
        w[1] += p * ty + c * fx;
        w[2] += q * tz;
        return;
    }
    // unbounded part
    R ir = rsq<R>(dx * dx + dy * dy + dz * dz);
    const R ex = dx * ir, ey = dy * ir, ez = dz * ir;
    const R ef = ex * fx + ey * fy + ez * fz;
    const R et = ex * tx + ey * ty + ez * tz;
    R c0 = K8 * ir;
    R ir2 = ir * ir;
    const R c1 = R(1) + R(2.0 / 3.0) * ir2;
    const R c2 = R(1) - R(2) * ir2;
    v[0] += c0 * (c1 * fx + c2 * ef * ex);
    v[1] += c0 * (c1 * fy + c2 * ef * ey);
    v[2] += c0 * (c1 * fz + c2 * ef * ez);
    c0 = K16 * ir2 * ir;
    w[0] += c0 * (R(3) * et * ex - tx);
    w[1] += c0 * (R(3) * et * ey - ty);
    w[2] += c0 * (R(3) * et * ez - tz);
    c0 = K8 * ir2;
    v[0] += c0 * (ty * ez - tz * ey);
    v[1] += c0 * (tz * ex - tx * ez);
    v[2] += c0 * (tx * ey - ty * ex);
    w[0] += c0 * (fy * ez - fz * ey);
    w[1] += c0 * (fz * ex - fx * ez);
    w[2] += c0 * (fx * ey - fy * ex);
    // image system: zs = z_i + z_j
    ir = rsq<R>(dx * dx + dy * dy + zs * zs);
    const R r2 = ir * ir, r3 = r2 * ir, r4 = r3 * ir, r5 = r4 * ir;
    R gx = dx * ir, gy = dy * ir;
    const R gz = zs * ir;
    R h = zj / zs;
    const R gf = gx * fx + gy * fy + gz * fz;
    const R gt = gx * tx + gy * ty + gz * tz;
    const R gz2 = gz * gz;
    R a0 = -(R(0.75) * ir * (R(1) + R(2) * h * (R(1) - h) * gz2) +
             R(0.5) * (r3 * (R(1) - R(3) * gz2) - r5 * (R(1) - R(5) * gz2)));
    R a1 = -(R(0.75) * ir * (R(1) - R(6) * h * (R(1) - h) * gz2) - R(1.5) * r3 * (R(1) - R(5) * gz2) +
             R(2.5) * r5 * (R(1) - R(7) * gz2)) * gf;
    R a2 = gz * fz * (R(1.5) * h * ir * (R(1) - R(6) * (R(1) - h) * gz2) - R(3) * r3 * (R(1) - R(5) * gz2) +
                      R(5) * r5 * (R(2) - R(7) * gz2));
    R a3 = (R(1.5) * h * ir - R(5) * r5) * gf;
    const R a4 = -((R(3) * h * h * ir + R(3) * r3) * gz2 + (R(2) - R(15) * gz2) * r5) * fz;
    v[0] += K6 * (a0 * fx + (a1 + a2) * gx);
    v[1] += K6 * (a0 * fy + (a1 + a2) * gy);
    v[2] += K6 * (a0 * fz + (a1 + a2 + a3) * gz + a4);
    a0 = r3 * (R(0.375) - R(2.25) * gz2);
    a1 = R(-1.125) * r3 * gt;
    a2 = R(2.25) * gz * r3 * gt;
    a3 = R(2.25) * r3 * (gx * ty - gy * tx);
    w[0] += K6 * (a0 * tx + a1 * gx - a3 * gy);
    w[1] += K6 * (a0 * ty + a1 * gy + a3 * gx);
    w[2] += K6 * (a0 * tz + a1 * gz + a2);
    a0 = R(0.75) * r2;
    a1 = fz * (R(9) * h * gz2 * r2 + (R(1.5) - R(15) * gz2) * r4);
    a2 = -gz * gf * (R(4.5) * h * r2 - R(7.5) * r4);
    a3 = R(-1.5) * gz * (h * r2 - r4);
    w[0] -= K6 * (a0 * (fy * gz - fz * gy) - (a1 + a2) * gy + a3 * fy);
    w[1] -= K6 * (a0 * (fz * gx - fx * gz) + (a1 + a2) * gx - a3 * fx);
    w[2] -= K6 * a0 * (fx * gy - fy * gx);
    h = R(1) - h;
    gx = -gx;
    gy = -gy;
    const R gct = gx * ty - gy * tx;
    a1 = (R(9) * h * gz2 * r2 + (R(1.5) - R(15) * gz2) * r4) * gct;
    a2 = -gz * (R(4.5) * h * r2 - R(7.5) * r4) * gct;
    a3 = R(-1.5) * gz * (h * r2 - r4);
    v[0] -= K6 * (a0 * (tz * gy - ty * gz) + a2 * gx - a3 * ty);
    v[1] -= K6 * (a0 * (tx * gz - tz * gx) + a2 * gy + a3 * tx);
    v[2] -= K6 * (a0 * (ty * gx - tx * gy) + a2 * gz + a1);
}

}  // namespace gmi
