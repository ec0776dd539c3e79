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
template <> __device__ __forceinline__ float rsq<float>(float x) { return rsqrtf(fmaxf(x, 1e-30f)); }
template <> __device__ __forceinline__ double rsq<double>(double x) { return rsqrt(fmax(x, 1e-300)); }

// Equal-radius constants (segment<-segment with a = a_seg, blob<-blob with a = a_blob).
template <class R> struct EqualK {
    R two_a, two_a2, f8pm, f16pm, f6pma, q32, inv_a, f8pma3, f16pma3, q8;
};

// Unequal-radius constants for segment<->blob pairs (radii as, ab).
template <class R> struct UnequalK {
    R sum, dmin, dmin2, far_c, half_sum, f8pm, f6pmab, fmax, c_mid_den, ab, as, ab2, f8pmas3, seg_bigger;
};

// translation<-force, rotation<-torque and the two cross couplings, equal radii:
// cuda_functions.cu:315-398.
template <class R>
__device__ __forceinline__ void pair_ss(R dx, R dy, R dz, const R *F, const EqualK<R> &k, R *v, R *w)
{
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R ir = rsq<R>(r2);
    const R r = r2 * ir;
    const R ex = dx * ir, ey = dy * ir, ez = dz * ir;
    const R ef = ex * F[0] + ey * F[1] + ez * F[2];
    const R et = ex * F[3] + ey * F[4] + ez * F[5];
    R t_id, t_ee, r_id, r_ee, cx;
    if (r > k.two_a) {
        const R ir2 = ir * ir;
        const R s = k.two_a2 * ir2;
        const R ik = ir * k.f8pm;
        t_id = (R(1) + s * R(1.0 / 3.0)) * ik;
        t_ee = (R(1) - s) * ik * ef;
        const R ir3k = ir2 * ir * k.f16pm;
        r_id = -ir3k;
        r_ee = R(3) * ir3k * et;
        cx = ir2 * k.f8pm;
    } else {
        const R q = r * k.q32;
        t_id = (R(1) - R(3) * q) * k.f6pma;
        t_ee = q * k.f6pma * ef;
        const R ra = r * k.inv_a;
        const R ra3 = ra * ra * ra;
        const R b = R(9.0 / 32.0) * ra;
        r_id = (R(-3) * b + (R(1) + R(5.0 / 64.0) * ra3)) * k.f8pma3;
        r_ee = (b - R(3.0 / 64.0) * ra3) * k.f8pma3 * et;
        cx = r * (R(1) - r * k.q8) * k.f16pma3;
    }
    v[0] += t_id * F[0] + t_ee * ex + cx * (F[4] * ez - F[5] * ey);
    v[1] += t_id * F[1] + t_ee * ey + cx * (F[5] * ex - F[3] * ez);
    v[2] += t_id * F[2] + t_ee * ez + cx * (F[3] * ey - F[4] * ex);
    w[0] += r_id * F[3] + r_ee * ex + cx * (F[1] * ez - F[2] * ey);
    w[1] += r_id * F[4] + r_ee * ey + cx * (F[2] * ex - F[0] * ez);
    w[2] += r_id * F[5] + r_ee * ez + cx * (F[0] * ey - F[1] * ex);
}

// translation<-force, equal radii: cuda_functions.cu:465-520.
template <class R>
__device__ __forceinline__ void pair_bb(R dx, R dy, R dz, const R *F, const EqualK<R> &k, R *v)
{
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R ir = rsq<R>(r2);
    const R r = r2 * ir;
    const R ex = dx * ir, ey = dy * ir, ez = dz * ir;
    const R ef = ex * F[0] + ey * F[1] + ez * F[2];
    R t_id, t_ee;
    if (r > k.two_a) {
        const R s = k.two_a2 * ir * ir;
        const R ik = ir * k.f8pm;
        t_id = (R(1) + s * R(1.0 / 3.0)) * ik;
        t_ee = (R(1) - s) * ik * ef;
    } else {
        const R q = r * k.q32;
        t_id = (R(1) - R(3) * q) * k.f6pma;
        t_ee = q * k.f6pma * ef;
    }
    v[0] += t_id * F[0] + t_ee * ex;
    v[1] += t_id * F[1] + t_ee * ey;
    v[2] += t_id * F[2] + t_ee * ez;
}

// Unequal-radius coefficients: cuda_functions.cu:608-667 (segment<-blob) and
// :770-829 (blob<-segment), which share the same expressions in (RSEG, RBLOB).
template <class R>
__device__ __forceinline__ void unequal_coeffs(R r, R ir, const UnequalK<R> &k, R &A, R &B, R &C)
{
    if (r > k.sum) {
        const R ir2 = ir * ir;
        const R t = ir2 * k.far_c;  // (as^2 + ab^2) / (3 r^2)
        const R ik = ir * k.f8pm;
        A = (t + R(1)) * ik;
        B = (R(1) - R(3) * t) * ik;
        C = ir2 * k.f8pm;
    } else if (r > k.dmin) {
        const R r_2 = r * r;
        const R d3 = R(32) * r_2 * r;
        const R id3 = R(1) / d3;
        R t = k.dmin2 + R(3) * r_2;
        A = (k.half_sum - t * t * id3) * k.f6pmab;
        const R b = k.dmin2 - r_2;
        B = R(3) * b * b * id3 * k.f6pmab;
        const R u = k.as - k.ab + r;
        const R p = k.ab2 + R(2) * k.ab * (r + k.as) - R(3) * (k.as - r) * (k.as - r);
        C = ir * ir * u * u * p * k.c_mid_den;
    } else {
        A = k.fmax;
        B = R(0);
        C = k.seg_bigger * r * k.f8pmas3;
    }
}

// segment <- blob force (3 -> 6): cuda_functions.cu:582-667.
template <class R>
__device__ __forceinline__ void pair_sb(R dx, R dy, R dz, const R *F, const UnequalK<R> &k, R *v, R *w)
{
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R ir = rsq<R>(r2);
    const R r = r2 * ir;
    const R ex = dx * ir, ey = dy * ir, ez = dz * ir;
    R A, B, C;
    unequal_coeffs<R>(r, ir, k, A, B, C);
    const R ef = (ex * F[0] + ey * F[1] + ez * F[2]) * B;
    v[0] += A * F[0] + ef * ex;
    v[1] += A * F[1] + ef * ey;
    v[2] += A * F[2] + ef * ez;
    w[0] += C * (F[1] * ez - F[2] * ey);
    w[1] += C * (F[2] * ex - F[0] * ez);
    w[2] += C * (F[0] * ey - F[1] * ex);
}

// blob <- segment force and torque (6 -> 3): cuda_functions.cu:744-829.
template <class R>
__device__ __forceinline__ void pair_bs(R dx, R dy, R dz, const R *F, const UnequalK<R> &k, R *v)
{
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R ir = rsq<R>(r2);
    const R r = r2 * ir;
    const R ex = dx * ir, ey = dy * ir, ez = dz * ir;
    R A, B, C;
    unequal_coeffs<R>(r, ir, k, A, B, C);
    const R ef = (ex * F[0] + ey * F[1] + ez * F[2]) * B;
    v[0] += A * F[0] + ef * ex + C * (F[4] * ez - F[5] * ey);
    v[1] += A * F[1] + ef * ey + C * (F[5] * ex - F[3] * ez);
    v[2] += A * F[2] + ef * ez + C * (F[3] * ey - F[4] * ex);
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
