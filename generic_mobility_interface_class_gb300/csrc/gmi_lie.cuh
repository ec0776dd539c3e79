// gmi_lie.cuh -- FP64 quaternion, Lie-algebra and 3x3 helpers for the
// filament and body state updates, restating the reference's quaternion.cpp
// (lie_exp :455-478, midpoint_quaternion :488-497, dexp :507-541, dexpinv
// :543-566, dexpinv_transpose :568-591, rot_mat :260-298, tangent/normal/
// binormal :218-258, sqrt_in_place :180-210, psi_mat/left_mult_mat
// :302-343) and the matrix helpers it relies on (rcross, matrix.cpp:665-679).
// Orders of operations follow the reference so results agree to rounding.
#pragma once

#include <cuda_runtime.h>

namespace gmi {

#define GMI_HD __host__ __device__ __forceinline__

constexpr double kSmallAngle = 1e-5;  // quaternion.cpp:7

struct Q4 {
    double s, x, y, z;  // scalar part, vector part
};

// 3x3, row-major: a[3*i + j] = M(i, j)
struct M3 {
    double a[9];
    GMI_HD double &operator()(int i, int j) { return a[3 * i + j]; }
    GMI_HD double operator()(int i, int j) const { return a[3 * i + j]; }
};

GMI_HD Q4 qmul(const Q4 &p, const Q4 &q)  // quaternion::operator*= (quaternion.cpp:86-100)
{
    Q4 r;
    r.s = p.s * q.s - (p.x * q.x + p.y * q.y + p.z * q.z);
    r.x = p.s * q.x + q.s * p.x + p.y * q.z - p.z * q.y;
    r.y = p.s * q.y + q.s * p.y + p.z * q.x - p.x * q.z;
    r.z = p.s * q.z + q.s * p.z + p.x * q.y - p.y * q.x;
    return r;
}
GMI_HD Q4 qconj(Q4 q) { q.x = -q.x; q.y = -q.y; q.z = -q.z; return q; }
GMI_HD Q4 qsub(const Q4 &a, const Q4 &b) { return Q4{a.s - b.s, a.x - b.x, a.y - b.y, a.z - b.z}; }
GMI_HD Q4 qscale(Q4 q, double f) { q.s *= f; q.x *= f; q.y *= f; q.z *= f; return q; }
GMI_HD Q4 qdiv(Q4 q, double f) { q.s /= f; q.x /= f; q.y /= f; q.z /= f; return q; }

GMI_HD void qsqrt_in_place(Q4 &q)
{
    if (q.s < -0.999999999) {
        q.s = 0.0; q.x = 0.0; q.y = 0.0; q.z = 1.0;
    } else {
        q.s = sqrt(0.5 * (1.0 + q.s));
        const double t = 2.0 * q.s;
        q.x /= t; q.y /= t; q.z /= t;
    }
}

GMI_HD Q4 lie_exp(const double *u)
{
    const double th = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (th < 1e-10) return Q4{1.0, 0.0, 0.0, 0.0};
    const double cs = cos(0.5 * th), sn = sin(0.5 * th) / th;
    return Q4{cs, sn * u[0], sn * u[1], sn * u[2]};
}

GMI_HD Q4 midpoint_quaternion(const Q4 &q1, const Q4 &q2)  // (q2 conj(q1))^(1/2) q1
{
    Q4 m = qmul(q2, qconj(q1));
    qsqrt_in_place(m);
    return qmul(m, q1);
}

GMI_HD void q_tangent(const Q4 &q, double *t)
{
    t[0] = 1.0 - 2.0 * (q.y * q.y + q.z * q.z);
    t[1] = 2.0 * (q.x * q.y + q.s * q.z);
    t[2] = 2.0 * (q.x * q.z - q.s * q.y);
}
GMI_HD void q_normal(const Q4 &q, double *n)
{
    n[0] = 2.0 * (q.x * q.y - q.s * q.z);
    n[1] = 1.0 - 2.0 * (q.x * q.x + q.z * q.z);
    n[2] = 2.0 * (q.y * q.z + q.s * q.x);
}
GMI_HD void q_binormal(const Q4 &q, double *b)
{
    b[0] = 2.0 * (q.x * q.z + q.s * q.y);
    b[1] = 2.0 * (q.y * q.z - q.s * q.x);
    b[2] = 1.0 - 2.0 * (q.x * q.x + q.y * q.y);
}

GMI_HD M3 q_rot_mat(const Q4 &q)
{
    M3 R;
    double R00 = 1.0, R11 = 1.0, R22 = 1.0;
    double t = 2.0 * q.x * q.x;
    R11 -= t; R22 -= t;
    t = 2.0 * q.y * q.y;
    R00 -= t; R22 -= t;
    t = 2.0 * q.z * q.z;
    R00 -= t; R11 -= t;
    t = 2.0 * q.x * q.y;
    double R10 = t, R01 = t;
    t = 2.0 * q.x * q.z;
    double R20 = t, R02 = t;
    t = 2.0 * q.y * q.z;
    double R12 = t, R21 = t;
    t = 2.0 * q.s * q.z;
    R10 += t; R01 -= t;
    t = 2.0 * q.s * q.y;
    R20 -= t; R02 += t;
    t = 2.0 * q.s * q.x;
    R21 += t; R12 -= t;
    R(0, 0) = R00; R(0, 1) = R01; R(0, 2) = R02;
    R(1, 0) = R10; R(1, 1) = R11; R(1, 2) = R12;
    R(2, 0) = R20; R(2, 1) = R21; R(2, 2) = R22;
    return R;
}

GMI_HD void dexp(double *out, const double *u, const double *v)
{
    const double th2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const double th = sqrt(th2);
    double alpha, beta;
    if (th < kSmallAngle) {
        const double th4 = th2 * th2;
        beta = (1.0 / 3.0 + th2 / 72.0) / (2.0 + th2 / 6.0 + th4 / 72.0);
        alpha = 1.0 / 6.0 + 2.0 * beta * (1.0 - th2 / 12.0);
    } else {
        const double th3 = th * th2;
        alpha = sin(0.5 * th);
        alpha *= 2.0 * alpha / th2;
        beta = (th - sin(th)) / th3;
    }
    const double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
    out[0] = v[0] + alpha * c[0] + beta * (u[1] * c[2] - u[2] * c[1]);
    out[1] = v[1] + alpha * c[1] + beta * (u[2] * c[0] - u[0] * c[2]);
    out[2] = v[2] + alpha * c[2] + beta * (u[0] * c[1] - u[1] * c[0]);
}

GMI_HD double dexpinv_fac(const double *u)
{
    const double th2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const double th = sqrt(th2);
    if (th < kSmallAngle) return -1.0 / 12.0;
    return (0.5 * th * cos(0.5 * th) / sin(0.5 * th) - 1.0) / th2;
}

GMI_HD void dexpinv(double *out, const double *u, const double *v)
{
    const double fac = dexpinv_fac(u);
    const double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
    out[0] = v[0] - 0.5 * c[0] - fac * (u[1] * c[2] - u[2] * c[1]);
    out[1] = v[1] - 0.5 * c[1] - fac * (u[2] * c[0] - u[0] * c[2]);
    out[2] = v[2] - 0.5 * c[2] - fac * (u[0] * c[1] - u[1] * c[0]);
}

GMI_HD void dexpinv_transpose(double *out, const double *u, const double *v)
{
    const double fac = dexpinv_fac(u);
    const double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
    out[0] = v[0] + 0.5 * c[0] - fac * (u[1] * c[2] - u[2] * c[1]);
    out[1] = v[1] + 0.5 * c[1] - fac * (u[2] * c[0] - u[0] * c[2]);
    out[2] = v[2] + 0.5 * c[2] - fac * (u[0] * c[1] - u[1] * c[0]);
}

// ---- 3x3 helpers ----------------------------------------------------------
GMI_HD M3 m3_zero() { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = 0.0; return m; }
GMI_HD M3 m3_eye() { M3 m = m3_zero(); m.a[0] = m.a[4] = m.a[8] = 1.0; return m; }
// the reference's rcross(v): rcross(v) b = b x v (matrix.cpp:665-679)
GMI_HD M3 rcross(const double *v)
{
    M3 m;
    m(0, 0) = 0.0; m(1, 0) = -v[2]; m(2, 0) = v[1];
    m(0, 1) = v[2]; m(1, 1) = 0.0; m(2, 1) = -v[0];
    m(0, 2) = -v[1]; m(1, 2) = v[0]; m(2, 2) = 0.0;
    return m;
}
GMI_HD M3 m3_mul(const M3 &A, const M3 &B)
{
    M3 C;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C(i, j) = A(i, 0) * B(0, j) + A(i, 1) * B(1, j) + A(i, 2) * B(2, j);
    return C;
}
GMI_HD M3 m3_add(const M3 &A, const M3 &B) { M3 C; for (int k = 0; k < 9; ++k) C.a[k] = A.a[k] + B.a[k]; return C; }
GMI_HD M3 m3_sub(const M3 &A, const M3 &B) { M3 C; for (int k = 0; k < 9; ++k) C.a[k] = A.a[k] - B.a[k]; return C; }
GMI_HD M3 m3_scale(const M3 &A, double s) { M3 C; for (int k = 0; k < 9; ++k) C.a[k] = s * A.a[k]; return C; }
GMI_HD M3 m3_T(const M3 &A) { M3 C; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) C(i, j) = A(j, i); return C; }
GMI_HD void m3_vec(const M3 &A, const double *v, double *o)
{
    o[0] = A(0, 0) * v[0] + A(0, 1) * v[1] + A(0, 2) * v[2];
    o[1] = A(1, 0) * v[0] + A(1, 1) * v[1] + A(1, 2) * v[2];
    o[2] = A(2, 0) * v[0] + A(2, 1) * v[1] + A(2, 2) * v[2];
}

// Column-major dense matrix block access (the reference's matrix storage).
GMI_HD void put_block(double *Mat, int ld, int r0, int c0, const M3 &B)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Mat[(r0 + i) + (size_t)ld * (c0 + j)] = B(i, j);
}
GMI_HD void add_block(double *Mat, int ld, int r0, int c0, const M3 &B)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Mat[(r0 + i) + (size_t)ld * (c0 + j)] += B(i, j);
}
GMI_HD M3 get_block(const double *Mat, int ld, int r0, int c0)
{
    M3 B;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B(i, j) = Mat[(r0 + i) + (size_t)ld * (c0 + j)];
    return B;
}

// psi_mat (4x3) and left_mult_mat (4x4) of a quaternion, row-major.
GMI_HD void q_psi_mat(const Q4 &q, double *P)
{
    const double v[3] = {q.x, q.y, q.z};
    const M3 rc = rcross(v);
    P[0] = -q.x; P[1] = -q.y; P[2] = -q.z;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) P[3 * (i + 1) + j] = rc(i, j);
    P[3 * 1 + 0] += q.s; P[3 * 2 + 1] += q.s; P[3 * 3 + 2] += q.s;
    for (int k = 0; k < 12; ++k) P[k] *= 0.5;
}
GMI_HD void q_left_mult_mat(const Q4 &q, double *L)
{
    const double v[3] = {q.x, q.y, q.z};
    const M3 rc = rcross(v);
    L[0] = q.s; L[1] = -q.x; L[2] = -q.y; L[3] = -q.z;
    L[4] = q.x; L[8] = q.y; L[12] = q.z;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) L[4 * (i + 1) + (j + 1)] = -rc(i, j);
    L[5] += q.s; L[10] += q.s; L[15] += q.s;
}

}  // namespace gmi
