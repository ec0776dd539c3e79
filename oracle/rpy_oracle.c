/*
 * rpy_oracle.c -- CPU FP64 restatement of the reference's RPY pair sums.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product
 * path: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load it.  Nothing in the product library links or calls it.
 *
 * Each function restates one kernel of the reference (file:line into the
 * reference project), branch for branch, with the same per-target summation
 * order (sources j = 0 .. n-1) and the same self-pair treatment (the
 * r + 1e-20 guard, which sends the self pair down the near-field branch with
 * r = 0).  Sizes and radii are run-time arguments instead of the
 * reference's compile-time macros.  OpenMP parallelises over target rows;
 * each target is summed by one thread in source order, so the result does
 * not depend on the thread count.
 *
 * Layouts (all FP64, array-of-structures as in the reference's host arrays):
 *   segment positions  xs[3*S]   segment forces/torques fs[6*S] (f, tau)
 *   blob positions     xb[3*B]   blob forces           fb[3*B]
 *   segment velocities vs[6*S] (v, omega)   blob velocities vb[3*B]
 *
 * Parity of this file is pinned against the reference's own kernels compiled
 * for the CPU (oracle/Makefile, target "ref") in tests/test_oracle_pin.py and
 * by the committed fixtures in tests/golden/.
 */
#include <math.h>
#include <stddef.h>

#define ORC_PI 3.14159265358979323846264338327950288

/* ------------------------------------------------------------------------ */
/* Segment <- segment, free space: cuda_functions.cu:246-425 (Mss_mult).     */
/* Targets t0 .. t0+nt-1 of the S segments; writes vs[6*(i-t0)..] (=).      */
/* ------------------------------------------------------------------------ */
void orc_mss(int S, const double *xs, const double *fs, double a, double mu,
             int t0, int nt, double *vs)
{
    const double f8pm = 1.0 / (8.0 * ORC_PI * mu);
    const double f16pm = 1.0 / (16.0 * ORC_PI * mu);
    const double f6pma = 1.0 / (6.0 * ORC_PI * mu * a);
    const double f8pma3 = 1.0 / (8.0 * ORC_PI * mu * a * a * a);
    const double f16pma3 = 1.0 / (16.0 * ORC_PI * mu * a * a * a);
#pragma omp parallel for schedule(dynamic, 16)
    for (int ii = 0; ii < nt; ++ii) {
        const int i = t0 + ii;
        const double xi = xs[3 * i], yi = xs[3 * i + 1], zi = xs[3 * i + 2];
        double v0 = 0, v1 = 0, v2 = 0, w0 = 0, w1 = 0, w2 = 0;
        for (int j = 0; j < S; ++j) {
            const double *F = fs + 6 * j;
            double ex = xi - xs[3 * j], ey = yi - xs[3 * j + 1], ez = zi - xs[3 * j + 2];
            const double r = sqrt(ex * ex + ey * ey + ez * ez);
            const double ir = 1.0 / (r + 1e-20);
            ex *= ir; ey *= ir; ez *= ir;
            const int far = r > 2.0 * a;
            /* translation <- force */
            double ef = ex * F[0] + ey * F[1] + ez * F[2];
            double c_id, c_ee;
            if (far) {
                const double s = 2.0 * a * a * ir * ir;
                c_id = (1.0 + s / 3.0) * (ir * f8pm);
                c_ee = (1.0 - s) * (ir * f8pm * ef);
            } else {
                const double q = 3.0 * r / (32.0 * a);
                c_id = (1.0 - 3.0 * q) * f6pma;
                c_ee = q * (f6pma * ef);
            }
            v0 += c_id * F[0] + c_ee * ex;
            v1 += c_id * F[1] + c_ee * ey;
            v2 += c_id * F[2] + c_ee * ez;
            /* rotation <- torque */
            const double et = ex * F[3] + ey * F[4] + ez * F[5];
            if (far) {
                c_id = -ir * ir * ir * f16pm;
                c_ee = -3.0 * et * c_id;
            } else {
                const double ra = r / a;
                const double ra3 = ra * ra * ra;
                c_ee = 9.0 * ra / 32.0;
                c_id = -3.0 * c_ee + (1.0 + 5.0 * ra3 / 64.0);
                c_ee -= 3.0 * ra3 / 64.0;
                c_id *= f8pma3;
                c_ee *= f8pma3 * et;
            }
            w0 += c_id * F[3] + c_ee * ex;
            w1 += c_id * F[4] + c_ee * ey;
            w2 += c_id * F[5] + c_ee * ez;
            /* rotation <- force and translation <- torque (cross terms) */
            const double c_x = far ? ir * ir * f8pm : r * (1.0 - 3.0 * r / (8.0 * a)) * f16pma3;
            w0 += c_x * (F[1] * ez - F[2] * ey);
            w1 += c_x * (F[2] * ex - F[0] * ez);
            w2 += c_x * (F[0] * ey - F[1] * ex);
            v0 += c_x * (F[4] * ez - F[5] * ey);
            v1 += c_x * (F[5] * ex - F[3] * ez);
            v2 += c_x * (F[3] * ey - F[4] * ex);
        }
        double *V = vs + 6 * ii;
        V[0] = v0; V[1] = v1; V[2] = v2; V[3] = w0; V[4] = w1; V[5] = w2;
    }
}

/* ------------------------------------------------------------------------ */
/* Segment <- segment above a no-slip wall at z = 0 (Swan & Brady 2007):      */
/* cuda_functions.cu:10-242.  The reference hard-wires a = mu = 1 (:22); so   */
/* does this restatement.  The rotation/translation coupling of the wall     */
/* image is applied with the reference's sign convention (:13-20).           */
/* ------------------------------------------------------------------------ */
void orc_mss_wall(int S, const double *xs, const double *fs, int t0, int nt, double *vs)
{
    const double K6 = 1.0 / (6.0 * ORC_PI);   /* force factor  */
    const double K8 = 1.0 / (8.0 * ORC_PI);   /* torque factor */
    const double K16 = 1.0 / (16.0 * ORC_PI);
#pragma omp parallel for schedule(dynamic, 16)
    for (int ii = 0; ii < nt; ++ii) {
        const int i = t0 + ii;
        const double xi = xs[3 * i], yi = xs[3 * i + 1], zi = xs[3 * i + 2];
        double v0 = 0, v1 = 0, v2 = 0, w0 = 0, w1 = 0, w2 = 0;
        for (int j = 0; j < S; ++j) {
            const double *F = fs + 6 * j;
            const double fx = F[0], fy = F[1], fz = F[2], tx = F[3], ty = F[4], tz = F[5];
            if (i == j) {
                /* self mobility with the wall correction at height h = z_i */
                const double h1 = 1.0 / zi, h3 = h1 * h1 * h1, h4 = h3 * h1, h5 = h4 * h1;
                double p = K6 - (9.0 * h1 - 2.0 * h3 + h5) * (K6 / 16.0);
                double q = K6 - (9.0 * h1 - 4.0 * h3 + h5) * (K6 / 8.0);
                const double c = (3.0 * K6 / 32.0) * h4;
                v0 += p * fx + c * ty;
                v1 += p * fy - c * tx;
                v2 += q * fz;
                p = K8 - (15.0 * K6 / 64.0) * h3;
                q = K8 - (3.0 * K6 / 32.0) * h3;
                w0 += p * tx - c * fy;
                w1 += p * ty + c * fx;
                w2 += q * tz;
                continue;
            }
            const double dx = xi - xs[3 * j], dy = yi - xs[3 * j + 1], zj = xs[3 * j + 2];
            /* unbounded RPY part (far-field form, as in the reference) */
            double ir = 1.0 / sqrt(dx * dx + dy * dy + (zi - zj) * (zi - zj));
            const double ex = dx * ir, ey = dy * ir, ez = (zi - zj) * ir;
            const double ef = ex * fx + ey * fy + ez * fz;
            const double et = ex * tx + ey * ty + ez * tz;
            double c0 = K8 * ir;
            double c1 = 1.0 + (2.0 / 3.0) * ir * ir;
            double c2 = 1.0 - 2.0 * ir * ir;
            v0 += c0 * (c1 * fx + c2 * ef * ex);
            v1 += c0 * (c1 * fy + c2 * ef * ey);
            v2 += c0 * (c1 * fz + c2 * ef * ez);
            c0 = K16 * ir * ir * ir;
            w0 += c0 * (3.0 * et * ex - tx);
            w1 += c0 * (3.0 * et * ey - ty);
            w2 += c0 * (3.0 * et * ez - tz);
            c0 = K8 * ir * ir;
            v0 += c0 * (ty * ez - tz * ey);
            v1 += c0 * (tz * ex - tx * ez);
            v2 += c0 * (tx * ey - ty * ex);
            w0 += c0 * (fy * ez - fz * ey);
            w1 += c0 * (fz * ex - fx * ez);
            w2 += c0 * (fx * ey - fy * ex);
            /* image-system corrections: separation to the mirror image of j */
            ir = 1.0 / sqrt(dx * dx + dy * dy + (zi + zj) * (zi + zj));
            const double r2 = ir * ir, r3 = r2 * ir, r4 = r3 * ir, r5 = r4 * ir;
            double gx = dx * ir, gy = dy * ir;
            const double gz = (zi + zj) * ir;
            double h = zj / (zi + zj);
            const double gf = gx * fx + gy * fy + gz * fz;
            const double gt = gx * tx + gy * ty + gz * tz;
            const double gz2 = gz * gz;
            double a0 = -(0.75 * ir * (1.0 + 2.0 * h * (1.0 - h) * gz2)
                          + 0.5 * (r3 * (1.0 - 3.0 * gz2) - r5 * (1.0 - 5.0 * gz2)));
            double a1 = -(0.75 * ir * (1.0 - 6.0 * h * (1.0 - h) * gz2)
                          - 1.5 * r3 * (1.0 - 5.0 * gz2) + 2.5 * r5 * (1.0 - 7.0 * gz2)) * gf;
            double a2 = gz * fz * (1.5 * h * ir * (1.0 - 6.0 * (1.0 - h) * gz2)
                                   - 3.0 * r3 * (1.0 - 5.0 * gz2) + 5.0 * r5 * (2.0 - 7.0 * gz2));
            double a3 = (1.5 * h * ir - 5.0 * r5) * gf;
            const double a4 = -((3.0 * h * h * ir + 3.0 * r3) * gz2 + (2.0 - 15.0 * gz2) * r5) * fz;
            v0 += K6 * (a0 * fx + (a1 + a2) * gx);
            v1 += K6 * (a0 * fy + (a1 + a2) * gy);
            v2 += K6 * (a0 * fz + (a1 + a2 + a3) * gz + a4);
            a0 = r3 * (0.375 - 2.25 * gz2);
            a1 = -1.125 * r3 * gt;
            a2 = 2.25 * gz * r3 * gt;
            a3 = 2.25 * r3 * (gx * ty - gy * tx);
            w0 += K6 * (a0 * tx + a1 * gx - a3 * gy);
            w1 += K6 * (a0 * ty + a1 * gy + a3 * gx);
            w2 += K6 * (a0 * tz + a1 * gz + a2);
            a0 = 0.75 * r2;
            a1 = fz * (9.0 * h * gz2 * r2 + (1.5 - 15.0 * gz2) * r4);
            a2 = -gz * gf * (4.5 * h * r2 - 7.5 * r4);
            a3 = -1.5 * gz * (h * r2 - r4);
            w0 -= K6 * (a0 * (fy * gz - fz * gy) - (a1 + a2) * gy + a3 * fy);
            w1 -= K6 * (a0 * (fz * gx - fx * gz) + (a1 + a2) * gx - a3 * fx);
            w2 -= K6 * a0 * (fx * gy - fy * gx);
            /* translation <- torque through the transpose of the (omega_j <- F_i) block */
            h = 1.0 - h;
            gx = -gx;
            gy = -gy;
            const double gct = gx * ty - gy * tx;
            a1 = (9.0 * h * gz2 * r2 + (1.5 - 15.0 * gz2) * r4) * gct;
            a2 = -gz * (4.5 * h * r2 - 7.5 * r4) * gct;
            a3 = -1.5 * gz * (h * r2 - r4);
            v0 -= K6 * (a0 * (tz * gy - ty * gz) + a2 * gx - a3 * ty);
            v1 -= K6 * (a0 * (tx * gz - tz * gx) + a2 * gy + a3 * tx);
            v2 -= K6 * (a0 * (ty * gx - tx * gy) + a2 * gz + a1);
        }
        double *V = vs + 6 * ii;
        V[0] = v0; V[1] = v1; V[2] = v2; V[3] = w0; V[4] = w1; V[5] = w2;
    }
}

/* ------------------------------------------------------------------------ */
/* Blob <- blob, translation only: cuda_functions.cu:429-539 (Mbb_mult).     */
/* ------------------------------------------------------------------------ */
void orc_mbb(int B, const double *xb, const double *fb, double a, double mu,
             int t0, int nt, double *vb)
{
    const double f8pm = 1.0 / (8.0 * ORC_PI * mu);
    const double f6pma = 1.0 / (6.0 * ORC_PI * mu * a);
#pragma omp parallel for schedule(dynamic, 16)
    for (int ii = 0; ii < nt; ++ii) {
        const int i = t0 + ii;
        const double xi = xb[3 * i], yi = xb[3 * i + 1], zi = xb[3 * i + 2];
        double v0 = 0, v1 = 0, v2 = 0;
        for (int j = 0; j < B; ++j) {
            const double *F = fb + 3 * j;
            double ex = xi - xb[3 * j], ey = yi - xb[3 * j + 1], ez = zi - xb[3 * j + 2];
            const double r = sqrt(ex * ex + ey * ey + ez * ez);
            const double ir = 1.0 / (r + 1e-20);
            ex *= ir; ey *= ir; ez *= ir;
            const double ef = ex * F[0] + ey * F[1] + ez * F[2];
            double c_id, c_ee;
            if (r > 2.0 * a) {
                const double s = 2.0 * a * a * ir * ir;
                c_id = (1.0 + s / 3.0) * (ir * f8pm);
                c_ee = (1.0 - s) * (ir * f8pm * ef);
            } else {
                const double q = 3.0 * r / (32.0 * a);
                c_id = (1.0 - 3.0 * q) * f6pma;
                c_ee = q * (f6pma * ef);
            }
            v0 += c_id * F[0] + c_ee * ex;
            v1 += c_id * F[1] + c_ee * ey;
            v2 += c_id * F[2] + c_ee * ez;
        }
        double *V = vb + 3 * ii;
        V[0] = v0; V[1] = v1; V[2] = v2;
    }
}

/* Unequal-radius RPY coefficients shared by Msb and Mbs                       */
/* (cuda_functions.cu:608-667 and :770-829): translation-translation A, B and   */
/* the rotation-translation coupling C for radii as (segment) and ab (blob).    */
static inline void orc_unequal_coeffs(double r, double ir, double as, double ab, double mu,
                                      double *A, double *Bc, double *C)
{
    const double dmin = fabs(as - ab);
    if (r > as + ab) {
        double t = ir * ir * (as * as + ab * ab) / 3.0;
        const double b = 1.0 - 3.0 * t;
        t += 1.0;
        const double k = ir / (8.0 * ORC_PI * mu);
        *A = t * k;
        *Bc = b * k;
    } else if (r > dmin) {
        const double d3 = 32.0 * r * r * r;
        double t = dmin * dmin + 3.0 * r * r;
        t = -t * t / d3 + 0.5 * (as + ab);
        double b = dmin * dmin - r * r;
        b = 3.0 * b * b / d3;
        const double k = 1.0 / (6.0 * ORC_PI * mu * as * ab);
        *A = t * k;
        *Bc = b * k;
    } else {
        *A = 1.0 / (6.0 * ORC_PI * mu * (as > ab ? as : ab));
        *Bc = 0.0;
    }
    if (r > as + ab) {
        *C = ir * ir / (8.0 * ORC_PI * mu);
    } else if (r > dmin) {
        double t = as - ab + r;
        t = ir * ir * t * t * (ab * ab + 2.0 * ab * (r + as) - 3.0 * (as - r) * (as - r))
            / (128.0 * ORC_PI * mu * ab * as * as * as);
        *C = t;
    } else {
        *C = (double)(as > ab) * r / (8.0 * ORC_PI * mu * as * as * as);
    }
}

/* ------------------------------------------------------------------------ */
/* Segment <- blob: cuda_functions.cu:541-694 (Msb_mult).  ACCUMULATES into  */
/* vs (+=), as the reference does.                                           */
/* ------------------------------------------------------------------------ */
void orc_msb(int S, int B, const double *xs, const double *xb, const double *fb,
             double as, double ab, double mu, int t0, int nt, double *vs)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int ii = 0; ii < nt; ++ii) {
        const int i = t0 + ii;
        const double xi = xs[3 * i], yi = xs[3 * i + 1], zi = xs[3 * i + 2];
        double v0 = 0, v1 = 0, v2 = 0, w0 = 0, w1 = 0, w2 = 0;
        for (int j = 0; j < B; ++j) {
            const double *F = fb + 3 * j;
            double ex = xi - xb[3 * j], ey = yi - xb[3 * j + 1], ez = zi - xb[3 * j + 2];
            const double r = sqrt(ex * ex + ey * ey + ez * ez);
            const double ir = 1.0 / (r + 1e-20);
            ex *= ir; ey *= ir; ez *= ir;
            double A, Bc, C;
            orc_unequal_coeffs(r, ir, as, ab, mu, &A, &Bc, &C);
            const double ef = ex * F[0] + ey * F[1] + ez * F[2];
            Bc *= ef;
            v0 += A * F[0] + Bc * ex;
            v1 += A * F[1] + Bc * ey;
            v2 += A * F[2] + Bc * ez;
            w0 += C * (F[1] * ez - F[2] * ey);
            w1 += C * (F[2] * ex - F[0] * ez);
            w2 += C * (F[0] * ey - F[1] * ex);
        }
        double *V = vs + 6 * ii;
        V[0] += v0; V[1] += v1; V[2] += v2; V[3] += w0; V[4] += w1; V[5] += w2;
    }
}

/* ------------------------------------------------------------------------ */
/* Blob <- segment: cuda_functions.cu:697-863 (Mbs_mult).  OVERWRITES vb.    */
/* ------------------------------------------------------------------------ */
void orc_mbs(int B, int S, const double *xb, const double *xs, const double *fs,
             double as, double ab, double mu, int t0, int nt, double *vb)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int ii = 0; ii < nt; ++ii) {
        const int i = t0 + ii;
        const double xi = xb[3 * i], yi = xb[3 * i + 1], zi = xb[3 * i + 2];
        double v0 = 0, v1 = 0, v2 = 0;
        for (int j = 0; j < S; ++j) {
            const double *F = fs + 6 * j;
            double ex = xi - xs[3 * j], ey = yi - xs[3 * j + 1], ez = zi - xs[3 * j + 2];
            const double r = sqrt(ex * ex + ey * ey + ez * ez);
            const double ir = 1.0 / (r + 1e-20);
            ex *= ir; ey *= ir; ez *= ir;
            double A, Bc, C;
            orc_unequal_coeffs(r, ir, as, ab, mu, &A, &Bc, &C);
            const double ef = ex * F[0] + ey * F[1] + ez * F[2];
            Bc *= ef;
            v0 += A * F[0] + Bc * ex;
            v1 += A * F[1] + Bc * ey;
            v2 += A * F[2] + Bc * ez;
            v0 += C * (F[4] * ez - F[5] * ey);
            v1 += C * (F[5] * ex - F[3] * ez);
            v2 += C * (F[3] * ey - F[4] * ex);
        }
        double *V = vb + 3 * ii;
        V[0] = v0; V[1] = v1; V[2] = v2;
    }
}

/* ------------------------------------------------------------------------ */
/* Short-range barrier forces: cuda_functions.cu:961-1157 (barrier_forces).  */
/* Sources are all S segments followed by all B blobs.  Segment targets add  */
/* into fs[6*i+0..2] (+=); blob targets overwrite fbrep[3*i..] (=).          */
/* nseg = segments per filament (adjacent segments of one filament exclude   */
/* each other, :1040).  scale = REPULSIVE_FORCE_FACTOR*END_FORCE_MAGNITUDE.  */
/* wall != 0 adds the reference's z = 0 wall repulsion (:988-996) for        */
/* segment targets and skips blob targets (prescribed bodies there).         */
/* ------------------------------------------------------------------------ */
void orc_barrier(int S, int B, int nseg, const double *xs, const double *xb,
                 double as, double ab, double scale, int wall,
                 double *fs, double *fbrep)
{
    const double DL = 2.2 * as;
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < S; ++i) {
        const double xi = xs[3 * i], yi = xs[3 * i + 1], zi = xs[3 * i + 2];
        const int fi = i / nseg;
        double g0 = 0, g1 = 0, g2 = 0;
        if (wall && zi < 0.5 * DL) {
            double fz = fmin(1.0, 1.0 - (zi - as) / (0.5 * DL - as));
            g2 = scale * fz * fz * fz * fz;
        }
        for (int j = 0; j < S + B; ++j) {
            const int is_seg = j < S;
            const double asum = is_seg ? 2.0 * as : as + ab;
            const double *xj = is_seg ? xs + 3 * j : xb + 3 * (j - S);
            const double dx = xi - xj[0], dy = yi - xj[1], dz = zi - xj[2];
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            const int fj = j / nseg;
            const int di = i - j;
            if (!(fi == fj && (di <= 1 && di >= -1)) && d < 1.1 * asum) {
                double c = fmin(1.0, 1.0 - (10.0 / asum) * (d - asum));
                c = scale * c * c * c * c;
                const double id = 1.0 / d;
                g0 += c * dx * id;
                g1 += c * dy * id;
                g2 += c * dz * id;
            }
        }
        fs[6 * i] += g0;
        fs[6 * i + 1] += g1;
        fs[6 * i + 2] += g2;
    }
    if (wall) return;
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < B; ++i) {
        const double xi = xb[3 * i], yi = xb[3 * i + 1], zi = xb[3 * i + 2];
        double g0 = 0, g1 = 0, g2 = 0;
        for (int j = 0; j < S + B; ++j) {
            const int is_seg = j < S;
            const double asum = is_seg ? ab + as : 2.0 * ab;
            const double *xj = is_seg ? xs + 3 * j : xb + 3 * (j - S);
            const double dx = xi - xj[0], dy = yi - xj[1], dz = zi - xj[2];
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            if (j != i + S && d < 1.1 * asum) {
                double c = fmin(1.0, 1.0 - (10.0 / asum) * (d - asum));
                c = scale * c * c * c * c;
                const double id = 1.0 / d;
                g0 += c * dx * id;
                g1 += c * dy * id;
                g2 += c * dz * id;
            }
        }
        fbrep[3 * i] = g0;
        fbrep[3 * i + 1] = g1;
        fbrep[3 * i + 2] = g2;
    }
}
