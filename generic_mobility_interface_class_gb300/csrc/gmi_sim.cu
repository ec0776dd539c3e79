// gmi_sim.cu -- the implicit time step of the ciliated-swimmer simulator on
// the GPU: Broyden's method over the filament Lagrange multipliers, segment
// Lie-algebra rotations and body state, each iteration evaluating the
// velocities through the device-resident mobility solver (gmi_solver.cu).
//
// Restates, for free-swimming spherical bodies with instability-driven
// (end-force) filaments and the GMRES linear solve:
//   cilia_sim_main.cpp:205-343         the step / Broyden loop (host, below)
//   rigid_body.cpp:247-381              body initial guess, update
//   segment.cpp:38-90                   segment initial guess, update
//   filament.cpp:416-463, 825-1018      robot arm, state from body, initial guess
//   filament.cpp:1096-1220              elastic moments, internal forces
//   filament.cpp:1222-1539              approximate Jacobian and its inverse
//   swimmer.cpp:276-325, 329-688 (GMRES branch 466-682)  forces, Schur complement
//   swimmer.cpp:690-845 (branch 793-837)                  inverse-Jacobian apply
//   swimmer.cpp:847-871                 state update
//   mobility_solver.cpp:1404-1689       Broyden residual (compute_errors)
//   broyden_solver.cpp:26-130           rank-one inverse-Jacobian updates
// All state is FP64 in HBM; one thread (or one CTA) per filament, one
// thread per segment where the work is per segment.
//
// Layout (F = nswim*nfil filaments, S = F*nseg segments, W swimmers):
//   segments: x (solver), q[4S] qm1[4S] u[3S] um1[3S] xm1[3S] xm2[3S]
//   filaments: lambda[3(nseg-1)F] (+m1, m2), tether[3F], clamp[3F] (+m1, m2),
//              inverse Jacobian [F][6nseg x 6nseg] column-major, jacB [F][6 x 6nseg]
//   bodies: x, q, f (solver), xm1 xm2 u um1 [3W], qm1 [4W], Q_init [9W] row-major,
//           schur_inv [36W] column-major
//   Broyden: C, D [nbroy x max_iter] column-major, error/new_error/update [nbroy]
//   with nbroy = W * (6*nfil*nseg + 6), the reference's unknown ordering
//   (per swimmer: per filament [tether, lambdas, clamp, segment u's], then body).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "gmi_context.hpp"
#include "gmi_gauss_jordan.hpp"
#include "gmi_lie.cuh"
#include "gmi_mlp.hpp"
#include "gmi_solver_device.cuh"
#include "gmi_solver_internal.hpp"

namespace gmi {

struct SimP {
    int W, NF, NS, NB, F, S, nbroy, per_body, n6, neuler;
    int wall;  // filaments on an infinite no-slip wall: no body unknowns (INFINITE_PLANE_WALL)
    double DL, DT, KB, KT, MU, RSEG, EFM, TOL, Rbody, conf;
    // segment state
    double *x, *f, *v;  // solver arrays: x_segs, f_segs, v_segs
    double *q, *qm1, *u, *um1, *xm1, *xm2;
    // filament state
    double *lam, *lam1, *lam2, *tl, *tl1, *tl2, *cl, *cl1, *cl2, *p1, *p2, *st, *fref;
    double *invJ, *ecb1, *ecb2, *jacB;
    // body state
    double *bx, *bq, *bf, *vb;  // solver arrays: body_x, body_q, body_f, v_bodies
    double *bxm1, *bxm2, *bu, *bum1, *bqm1, *bQ, *schur;
    double *mob_ref;
    double *lk;    // per link (F x (NS-1)): hdl t_i x lam, hdl t_{i+1} x lam, R(q_mid) M_body
    double *tang;  // per segment: tangent of q (filament update)
    int *flags;  // [0] error too large, [1] non-finite error, [2] singular Jacobian
};

__device__ __forceinline__ Q4 ldq(const double *p) { return Q4{p[0], p[1], p[2], p[3]}; }
__device__ __forceinline__ void stq(double *p, const Q4 &q) { p[0] = q.s; p[1] = q.x; p[2] = q.y; p[3] = q.z; }
__device__ __forceinline__ M3 ldm3(const double *p) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = p[k]; return m; }

// robot_arm (filament.cpp:416-436): positions by midpoint-tangent chaining.
__device__ void robot_arm(const SimP &P, int fil)
{
    const int s0 = fil * P.NS;
    double t1[3], t2[3];
    q_tangent(ldq(P.q + 4 * s0), t1);
    for (int i = 1; i < P.NS; ++i) {
        const int s = s0 + i;
        q_tangent(ldq(P.q + 4 * s), t2);
        for (int c = 0; c < 3; ++c) P.x[3 * s + c] = P.x[3 * (s - 1) + c] + 0.5 * P.DL * (t1[c] + t2[c]);
        t1[0] = t2[0]; t1[1] = t2[1]; t1[2] = t2[2];
    }
}

// segment::update (segment.cpp:68-74): u += du; q = lie_exp(u) qm1
__device__ void segment_update(const SimP &P, int s, const double *du)
{
    for (int c = 0; c < 3; ++c) P.u[3 * s + c] += du[c];
    stq(P.q + 4 * s, qmul(lie_exp(P.u + 3 * s), ldq(P.qm1 + 4 * s)));
}

// filament base position: body x + R(body q) ref (swimmer.cpp:252-254, 858-860)
__device__ void base_position(const SimP &P, int fil, double *base)
{
    const int n = fil / P.NF;
    const M3 R = q_rot_mat(ldq(P.bq + 4 * n));
    double d[3];
    m3_vec(R, P.fref + 3 * fil, d);
    for (int c = 0; c < 3; ++c) base[c] = P.bx[3 * n + c] + d[c];
}

// accept_state_from_rigid_body (filament.cpp:438-463)
__device__ void accept_state_from_body(const SimP &P, int fil)
{
    const int n = fil / P.NF, s0 = fil * P.NS;
    double base[3];
    base_position(P, fil, base);
    for (int c = 0; c < 3; ++c) P.x[3 * s0 + c] = base[c];
    const double du[3] = {P.bu[3 * n] - P.u[3 * s0], P.bu[3 * n + 1] - P.u[3 * s0 + 1], P.bu[3 * n + 2] - P.u[3 * s0 + 2]};
    segment_update(P, s0, du);
    robot_arm(P, fil);
}

// rigid_body::initial_guess (rigid_body.cpp:247-290)
__global__ void body_initial_guess_kernel(SimP P, int nt)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= P.W) return;
    double *x = P.bx + 3 * n, *xm1 = P.bxm1 + 3 * n, *xm2 = P.bxm2 + 3 * n, *u = P.bu + 3 * n, *um1 = P.bum1 + 3 * n;
    double gx[3], gu[3];
    for (int c = 0; c < 3; ++c) {
        if (nt <= P.neuler) {
            gx[c] = 2.0 * x[c] - xm1[c];
            gu[c] = u[c];
        } else {
            gx[c] = 3.0 * (x[c] - xm1[c]) + xm2[c];
            gu[c] = 2.0 * u[c] - um1[c];
        }
    }
    for (int c = 0; c < 3; ++c) {
        xm2[c] = xm1[c];
        xm1[c] = x[c];
        x[c] = gx[c];
        um1[c] = u[c];
        u[c] = gu[c];
    }
    const Q4 q = ldq(P.bq + 4 * n);
    stq(P.bqm1 + 4 * n, q);
    const Q4 qn = qmul(lie_exp(u), q);
    stq(P.bq + 4 * n, qn);
    const M3 R = q_rot_mat(qn);
    for (int k = 0; k < 9; ++k) P.bQ[9 * n + k] = R.a[k];
}

__device__ void extrapolate3(double *a, double *a1, double *a2, int count, int nt)
{
    for (int k = 0; k < count; ++k) {
        if (nt == 1) {
            a1[k] = a[k];
        } else if (nt == 2) {
            a2[k] = a1[k];
            a1[k] = a[k];
            a[k] = 2.0 * a1[k] - a2[k];
        } else if (nt > 2) {
            const double t = 3.0 * (a[k] - a1[k]) + a2[k];
            a2[k] = a1[k];
            a1[k] = a[k];
            a[k] = t;
        }
    }
}

// filament::initial_guess (filament.cpp:825-1018) with segment::initial_guess
// (segment.cpp:38-66) and the state taken from the body.
// In two passes: one thread per segment for the segments' own guesses (each
// its own u and q, with an FP64 sin/cos in lie_exp), then one thread per
// filament for the chain that depends on all of them.  The arithmetic of
// every segment is the reference's, in its order.
__global__ void segment_initial_guess_kernel(SimP P, int nt)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.S) return;
    for (int c = 0; c < 3; ++c) {
        P.xm2[3 * s + c] = P.xm1[3 * s + c];
        P.xm1[3 * s + c] = P.x[3 * s + c];
    }
    if (nt <= P.neuler) {
        for (int c = 0; c < 3; ++c) P.um1[3 * s + c] = P.u[3 * s + c];
    } else {
        for (int c = 0; c < 3; ++c) {
            const double t = 2.0 * P.u[3 * s + c] - P.um1[3 * s + c];
            P.um1[3 * s + c] = P.u[3 * s + c];
            P.u[3 * s + c] = t;
        }
    }
    const Q4 q = ldq(P.q + 4 * s);
    stq(P.qm1 + 4 * s, q);
    stq(P.q + 4 * s, qmul(lie_exp(P.u + 3 * s), q));
}

__global__ void filament_initial_guess_kernel(SimP P, int nt)
{
    const int fil = blockIdx.x * blockDim.x + threadIdx.x;
    if (fil >= P.F) return;
    accept_state_from_body(P, fil);
    const int nl = 3 * (P.NS - 1);
    extrapolate3(P.lam + nl * fil, P.lam1 + nl * fil, P.lam2 + nl * fil, nl, nt);
    extrapolate3(P.tl + 3 * fil, P.tl1 + 3 * fil, P.tl2 + 3 * fil, 3, nt);
    extrapolate3(P.cl + 3 * fil, P.cl1 + 3 * fil, P.cl2 + 3 * fil, 3, nt);
}

// body_frame_moment (filament.cpp:1096-1110)
__device__ void body_frame_moment(const SimP &P, int fil, int link, double *M)
{
    const int s = fil * P.NS + link;
    const Q4 qa = ldq(P.q + 4 * s), qb = ldq(P.q + 4 * (s + 1));
    Q4 mq = qconj(midpoint_quaternion(qa, qb));
    mq = qscale(qdiv(qmul(mq, qsub(qb, qa)), P.DL), 2.0);
    const double *st = P.st + 3 * fil;
    M[0] = P.KT * (mq.x - st[0]);
    M[1] = P.KB * (mq.y - st[1]);
    M[2] = P.KB * (mq.z - st[2]);
}

// filament::internal_forces_and_torques (filament.cpp:1112-1220), instability
// cilia, in two passes so that the FP64 work spreads over one thread per link
// and then one thread per segment (GB300's FP64 pipe makes a per-filament
// loop in one thread the slowest part of the Broyden iteration).
// Pass 1, thread per link i of a filament: the terms the reference's link
// loop adds to segments i and i+1.
__global__ void filament_link_terms_kernel(SimP P)
{
    const int nl = P.NS - 1;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (nl <= 0 || g >= P.F * nl) return;
    const int fil = g / nl, i = g % nl, s0 = fil * P.NS;
    const double hdl = 0.5 * P.DL;
    const double *lam = P.lam + 3 * (size_t)g;
    double *o = P.lk + 9 * (size_t)g;
    double t[3];
    q_tangent(ldq(P.q + 4 * (s0 + i)), t);
    o[0] = hdl * (t[1] * lam[2] - t[2] * lam[1]);
    o[1] = hdl * (t[2] * lam[0] - t[0] * lam[2]);
    o[2] = hdl * (t[0] * lam[1] - t[1] * lam[0]);
    q_tangent(ldq(P.q + 4 * (s0 + i + 1)), t);
    o[3] = hdl * (t[1] * lam[2] - t[2] * lam[1]);
    o[4] = hdl * (t[2] * lam[0] - t[0] * lam[2]);
    o[5] = hdl * (t[0] * lam[1] - t[1] * lam[0]);
    const Q4 qmid = midpoint_quaternion(ldq(P.q + 4 * (s0 + i)), ldq(P.q + 4 * (s0 + i + 1)));
    const M3 R = q_rot_mat(qmid);
    double Mb[3];
    body_frame_moment(P, fil, i, Mb);
    m3_vec(R, Mb, o + 6);
}

// Pass 2, thread per segment: the link terms in the order the reference's
// loop adds them (link i-1, then link i), then tether, end force, the
// one-off perturbation and the clamp torque.
__global__ void filament_forces_kernel(SimP P, int nt)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.S) return;
    const int NS = P.NS, fil = s / NS, i = s % NS, nl = NS - 1;
    double f[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (i > 0) {
        const size_t l = (size_t)fil * nl + (i - 1);
        const double *lam = P.lam + 3 * l, *o = P.lk + 9 * l;
        for (int c = 0; c < 3; ++c) f[c] += lam[c];
        for (int c = 0; c < 3; ++c) f[3 + c] -= o[3 + c];
        for (int c = 0; c < 3; ++c) f[3 + c] -= o[6 + c];
    }
    if (i < nl) {
        const size_t l = (size_t)fil * nl + i;
        const double *lam = P.lam + 3 * l, *o = P.lk + 9 * l;
        for (int c = 0; c < 3; ++c) f[c] -= lam[c];
        for (int c = 0; c < 3; ++c) f[3 + c] -= o[c];
        for (int c = 0; c < 3; ++c) f[3 + c] += o[6 + c];
    }
    if (i == 0)
        for (int c = 0; c < 3; ++c) f[c] += P.tl[3 * fil + c];
    if (i == NS - 1) {
        double t[3];
        q_tangent(ldq(P.q + 4 * s), t);
        for (int c = 0; c < 3; ++c) f[c] -= P.EFM * t[c];
    }
    if (nt == 0) {  // one-off perturbation of segments 4 and 12 (filament.cpp:1181-1196)
        if (i == 4)
            for (int c = 0; c < 3; ++c) f[c] += P.p1[3 * fil + c];
        if (i == 12)
            for (int c = 0; c < 3; ++c) f[c] += P.p2[3 * fil + c];
    }
    if (i == 0) {
        double ct[3];
        dexpinv_transpose(ct, P.u + 3 * s, P.cl + 3 * fil);
        for (int c = 0; c < 3; ++c) f[3 + c] += ct[c];
    }
    double *fs = P.f + 6 * (size_t)s;
    for (int c = 0; c < 6; ++c) fs[c] = f[c];
}

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Free-swimming force/torque balance (swimmer.cpp:276-325): body f = -sum of
// segment forces and torques about the body centre, in one launch: kFsSegs
// segments per CTA into part[(n gx + x) 6 + c]; the last CTA to arrive adds
// the CTA partials in order, one thread per (swimmer, component).
constexpr int kFsSegs = 128;

__global__ void __launch_bounds__(kFsSegs) swimmer_force_kernel(SimP P, double *part, int *ticket)
{
    __shared__ double red[6][kFsSegs / 32];
    const int n = blockIdx.y, k = blockIdx.x * kFsSegs + threadIdx.x, gx = gridDim.x;
    const int per = P.NF * P.NS;
    const double *X = P.bx + 3 * n;
    double a[6] = {0, 0, 0, 0, 0, 0};
    if (k < per) {
        const int s = n * per + k;
        const double *fs = P.f + 6 * (size_t)s;
        const double dx = P.x[3 * s] - X[0], dy = P.x[3 * s + 1] - X[1], dz = P.x[3 * s + 2] - X[2];
        a[0] = fs[0];
        a[1] = fs[1];
        a[2] = fs[2];
        a[3] = fs[3] + dy * fs[2] - dz * fs[1];
        a[4] = fs[4] + dz * fs[0] - dx * fs[2];
        a[5] = fs[5] + dx * fs[1] - dy * fs[0];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int c = 0; c < 6; ++c) {
        const double v = warp_sum_d(a[c]);
        if (lane == 0) red[c][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double t = 0.0;
        for (int w = 0; w < kFsSegs / 32; ++w) t += red[threadIdx.x][w];
        part[((size_t)n * gx + blockIdx.x) * 6 + threadIdx.x] = t;
    }
    if (!last_cta(ticket, gx * gridDim.y)) return;
    for (int e = threadIdx.x; e < 6 * P.W; e += kFsSegs) {
        const int sw = e / 6, c = e % 6;
        double t = 0.0;
        for (int x = 0; x < gx; ++x) t += __ldcg(part + ((size_t)sw * gx + x) * 6 + c);
        P.bf[e] = -t;
    }
}

// compute_errors (mobility_solver.cpp:1404-1689), GMRES branch.
__global__ void compute_errors_kernel(SimP P, int nt, double *err)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const double c1 = -4.0 / 3.0, c2 = 1.0 / 3.0, c3 = -2.0 / 3.0;
    const bool euler = nt < P.neuler;
    bool big = false, bad = false;
    if (g < P.S) {
        const int per = P.NF * P.NS;
        const int n = g / per, i = (g / P.NS) % P.NF, j = g % P.NS;
        const double *v = P.v + 6 * (size_t)g, *om = v + 3;
        int id = n * P.per_body + 6 * i * P.NS + 3 * j;
        for (int c = 0; c < 3; ++c) {
            const double x = P.x[3 * g + c], xm1 = P.xm1[3 * g + c], xm2 = P.xm2[3 * g + c];
            const double e = euler ? x - xm1 - P.DT * v[c] : x + c1 * xm1 + c2 * xm2 + c3 * P.DT * v[c];
            err[id + c] = e;
            big |= fabs(e) > P.DL * P.TOL;
            bad |= !isfinite(e);
        }
        id += 3 * P.NS;
        double Wv[3];
        dexpinv(Wv, P.u + 3 * g, om);
        for (int c = 0; c < 3; ++c) {
            const double u = P.u[3 * g + c], um1 = P.um1[3 * g + c];
            const double e = euler ? u - P.DT * Wv[c] : u - c2 * um1 + c3 * P.DT * Wv[c];
            err[id + c] = e;
            big |= fabs(e) > P.TOL;
            bad |= !isfinite(e);
        }
    } else if (g < P.S + P.W) {
        const int n = g - P.S;
        const int id = n * P.per_body + 6 * P.NF * P.NS;
        const double *V = P.vb + 6 * n;
        double w[3];
        dexpinv(w, P.bu + 3 * n, V + 3);
        for (int c = 0; c < 3; ++c) {
            const double x = P.bx[3 * n + c], xm1 = P.bxm1[3 * n + c], xm2 = P.bxm2[3 * n + c];
            const double e = euler ? x - xm1 - P.DT * V[c] : x + c1 * xm1 + c2 * xm2 + c3 * P.DT * V[c];
            err[id + c] = e;
            big |= fabs(e) > P.TOL * P.DL;
            bad |= !isfinite(e);
        }
        for (int c = 0; c < 3; ++c) {
            const double u = P.bu[3 * n + c], um1 = P.bum1[3 * n + c];
            const double e = euler ? u - P.DT * w[c] : u - c2 * um1 + c3 * P.DT * w[c];
            err[id + 3 + c] = e;
            big |= fabs(e) > P.TOL;
            bad |= !isfinite(e);
        }
    }
    if (big) atomicOr(P.flags, 1);
    if (bad) atomicOr(P.flags + 1, 1);
}

// body_frame_moment_lie_derivative (filament.cpp:8-55): 3x3
__device__ M3 bfm_lie_derivative(const SimP &P, const Q4 &q1, const Q4 &q2, bool upper)
{
    double A[12], L[16];
    if (upper) {
        q_psi_mat(q2, A);
        for (int k = 0; k < 12; ++k) A[k] /= P.DL;
    } else {
        q_psi_mat(q1, A);
        for (int k = 0; k < 12; ++k) A[k] /= -P.DL;
    }
    Q4 mq = qconj(midpoint_quaternion(q1, q2));
    q_left_mult_mat(mq, L);
    double dM[12];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += L[4 * i + k] * A[3 * k + j];
            dM[3 * i + j] = s;
        }
    mq = qdiv(qsub(q2, q1), P.DL);
    q_left_mult_mat(mq, L);
    const double sc = upper ? 0.5 * P.DL : -0.5 * P.DL;
    for (int k = 0; k < 12; ++k) A[k] *= sc;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += L[4 * i + k] * A[3 * k + j];
            dM[3 * i + j] += s;
        }
    M3 out;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out(i, j) = 2.0 * dM[3 * (i + 1) + j];
    for (int j = 0; j < 3; ++j) {
        out(0, j) *= P.KT;
        out(1, j) *= P.KB;
        out(2, j) *= P.KB;
    }
    return out;
}

__device__ M3 frame_cross(const double K0, const double K1, const double K2, const Q4 &q)
{
    double t[3], nn[3], b[3];
    q_tangent(q, t);
    q_normal(q, nn);
    q_binormal(q, b);
    return m3_add(m3_add(m3_scale(rcross(t), K0), m3_scale(rcross(nn), K1)), m3_scale(rcross(b), K2));
}

// -tsf (dOmega - 0.5 (OmegaMat + LieMat dOmega) + (rcross(OmegaMat u) + LieMat OmegaMat + LieMat^2 dOmega)/12)
__device__ M3 diag_block(double tsf, const M3 &dOm, const M3 &Lie, const M3 &Om, const double *u)
{
    double Ou[3];
    m3_vec(Om, u, Ou);
    const M3 LdO = m3_mul(Lie, dOm);
    M3 t = m3_sub(dOm, m3_scale(m3_add(Om, LdO), 0.5));
    const M3 q = m3_add(m3_add(rcross(Ou), m3_mul(Lie, Om)), m3_mul(m3_mul(Lie, Lie), dOm));
    t = m3_add(t, m3_scale(q, 1.0 / 12.0));
    return m3_scale(t, -tsf);
}

// -tsf (dOmega - 0.5 LieMat dOmega + LieMat^2 dOmega / 12)
__device__ M3 off_block(double tsf, const M3 &dOm, const M3 &Lie)
{
    M3 t = m3_sub(dOm, m3_scale(m3_mul(Lie, dOm), 0.5));
    t = m3_add(t, m3_scale(m3_mul(m3_mul(Lie, Lie), dOm), 1.0 / 12.0));
    return m3_scale(t, -tsf);
}

// filament::jacobian_lie_algebra_block (filament.cpp:1222-1404) for segment
// k: the 3x3 blocks of rows [3NS + 3k, 3NS + 3k + 3) (diagonal, and the
// neighbours' columns), written into J; the unit diagonal is added later.
// Segments 0 and NS-1 are the reference's first and last cases (NS >= 2).
__device__ void lie_segment_blocks(const SimP &P, int fil, int nt, int k, double *J, int ld)
{
    const int NS = P.NS, s0 = fil * NS, o = 3 * NS;
    const double tsf = (nt < P.neuler) ? P.DT : 2.0 * P.DT / 3.0;
    const double Tfac = 1.0 / (8.0 * kPi * P.MU * P.RSEG * P.RSEG * P.RSEG);
    const double *lam = P.lam + 3 * (NS - 1) * fil;
    const double *f = P.f + 6 * (size_t)s0;
    auto Q = [&](int m) { return ldq(P.q + 4 * (s0 + m)); };
    double Kph[3], Kmh[3], t[3], om[3];
    q_tangent(Q(k), t);
    const M3 Lie = m3_scale(rcross(P.u + 3 * (s0 + k)), -1.0);
    for (int c = 0; c < 3; ++c) om[c] = Tfac * f[6 * k + 3 + c];
    const M3 Om = rcross(om);
    if (k == 0) {
        const M3 Cp = m3_mul(m3_scale(rcross(lam), -0.5 * P.DL), rcross(t));
        const Q4 qph = midpoint_quaternion(Q(0), Q(1));
        body_frame_moment(P, fil, 0, Kph);
        M3 LD = bfm_lie_derivative(P, Q(0), Q(1), false);
        M3 El = m3_scale(frame_cross(Kph[0], Kph[1], Kph[2], Q(0)), 0.5);
        const M3 R = q_rot_mat(qph);
        El = m3_add(El, m3_mul(R, LD));
        M3 dOm = m3_scale(m3_add(El, Cp), Tfac);
        put_block(J, ld, o, o, diag_block(tsf, dOm, Lie, Om, P.u + 3 * s0));
        LD = bfm_lie_derivative(P, Q(0), Q(1), true);
        El = m3_scale(frame_cross(Kph[0], Kph[1], Kph[2], Q(1)), 0.5);
        El = m3_add(El, m3_mul(R, LD));
        dOm = m3_scale(El, Tfac);
        put_block(J, ld, o, o + 3, off_block(tsf, dOm, Lie));
    } else if (k == NS - 1) {
        const int e = NS - 1;
        const M3 Cp = m3_mul(m3_scale(rcross(lam + 3 * (NS - 2)), -0.5 * P.DL), rcross(t));
        const Q4 qmh = midpoint_quaternion(Q(e - 1), Q(e));
        body_frame_moment(P, fil, NS - 2, Kmh);
        M3 LD = bfm_lie_derivative(P, Q(e - 1), Q(e), true);
        M3 El = m3_scale(frame_cross(Kmh[0], Kmh[1], Kmh[2], Q(e)), -0.5);
        const M3 R = q_rot_mat(qmh);
        El = m3_sub(El, m3_mul(R, LD));
        M3 dOm = m3_scale(m3_add(El, Cp), Tfac);
        put_block(J, ld, o + 3 * e, o + 3 * e, diag_block(tsf, dOm, Lie, Om, P.u + 3 * (s0 + e)));
        LD = bfm_lie_derivative(P, Q(e - 1), Q(e), false);
        El = m3_scale(frame_cross(Kmh[0], Kmh[1], Kmh[2], Q(e - 1)), -0.5);
        El = m3_sub(El, m3_mul(R, LD));
        dOm = m3_scale(El, Tfac);
        put_block(J, ld, o + 3 * e, o + 3 * e - 3, off_block(tsf, dOm, Lie));
    } else {
        body_frame_moment(P, fil, k, Kph);
        body_frame_moment(P, fil, k - 1, Kmh);
        const Q4 qph = midpoint_quaternion(Q(k), Q(k + 1));
        const Q4 qmh = midpoint_quaternion(Q(k - 1), Q(k));
        const double lv[3] = {lam[3 * (k - 1)] + lam[3 * k], lam[3 * (k - 1) + 1] + lam[3 * k + 1],
                              lam[3 * (k - 1) + 2] + lam[3 * k + 2]};
        const M3 Cp = m3_mul(m3_scale(rcross(lv), -0.5 * P.DL), rcross(t));
        M3 LD = bfm_lie_derivative(P, Q(k), Q(k + 1), false);
        M3 El = m3_scale(frame_cross(Kph[0], Kph[1], Kph[2], Q(k)), 0.5);
        const M3 Rph = q_rot_mat(qph);
        El = m3_add(El, m3_mul(Rph, LD));
        M3 LDm = bfm_lie_derivative(P, Q(k - 1), Q(k), true);
        El = m3_sub(El, m3_scale(frame_cross(Kmh[0], Kmh[1], Kmh[2], Q(k)), 0.5));
        const M3 Rmh = q_rot_mat(qmh);
        El = m3_sub(El, m3_mul(Rmh, LDm));
        M3 dOm = m3_scale(m3_add(Cp, El), Tfac);
        put_block(J, ld, o + 3 * k, o + 3 * k, diag_block(tsf, dOm, Lie, Om, P.u + 3 * (s0 + k)));
        LDm = bfm_lie_derivative(P, Q(k - 1), Q(k), false);
        El = m3_scale(frame_cross(Kmh[0], Kmh[1], Kmh[2], Q(k - 1)), -0.5);
        El = m3_sub(El, m3_mul(Rmh, LDm));
        dOm = m3_scale(El, Tfac);
        put_block(J, ld, o + 3 * k, o + 3 * k - 3, off_block(tsf, dOm, Lie));
        LD = bfm_lie_derivative(P, Q(k), Q(k + 1), true);
        El = m3_scale(frame_cross(Kph[0], Kph[1], Kph[2], Q(k + 1)), 0.5);
        El = m3_add(El, m3_mul(Rph, LD));
        dOm = m3_scale(El, Tfac);
        put_block(J, ld, o + 3 * k, o + 3 * k + 3, off_block(tsf, dOm, Lie));
    }
}

// filament::invert_approx_jacobian (filament.cpp:1406-1539) up to the
// inversion: the approximate Jacobian in invJ, the two clamping blocks saved.
// The reference's block writes fall into disjoint regions (constraint
// diagonal; position couplings, rows < 3NS; Lie-algebra rows >= 3NS, columns
// < 3NS; the Lie-algebra block, one row band per segment), built in parallel
// as 3NS - 1 tasks per filament: grid (filament blocks, task), one thread per
// (filament, task), so the 32 lanes of a warp run the same task for 32
// filaments.  Each task is a serial FP64 chain, and a warp FP64 instruction
// costs the same on one lane as on 32: lanes of one task for many filaments
// keep every lane busy and the warp on one code path (the reference's
// boundary cases, segments 0 and NS-1, are whole tasks).  The matrix is
// zeroed before the launch; the writes that depend on earlier ones
// (end-force term, unit diagonal, clamping blocks) follow in
// jacobian_finish_kernel.
constexpr int kJacTpb = 128;

__global__ void __launch_bounds__(kJacTpb) build_jacobian_kernel(SimP P, int nt)
{
    const int fil = blockIdx.x * kJacTpb + threadIdx.x, task = blockIdx.y;
    if (fil >= P.F) return;
    const int NS = P.NS, ld = P.n6, s0 = fil * NS;
    double *J = P.invJ + (size_t)fil * ld * ld;
    const bool euler = nt < P.neuler;
    const double fac0 = euler ? -P.DT / (6.0 * kPi * P.MU * P.RSEG) : -P.DT / (9.0 * kPi * P.MU * P.RSEG);
    const double fac1 = euler ? P.DL * P.DT / (16.0 * kPi * P.MU * P.RSEG * P.RSEG * P.RSEG)
                              : P.DL * P.DT / (24.0 * kPi * P.MU * P.RSEG * P.RSEG * P.RSEG);
    // tasks: [0, NS-1) position columns j+1; [NS-1, 2NS-2) Lie-to-position
    // rows for j+1; [2NS-2, 3NS-2) Lie-algebra segment k; 3NS-2 the
    // constraint diagonal
    double t[3];
    if (task < NS - 1) {
        const int j = task + 1, jpos = 3 * (NS + j);
        q_tangent(ldq(P.q + 4 * (s0 + j)), t);
        const M3 temp = m3_scale(rcross(t), P.DL);
        put_block(J, ld, 3 * j, jpos, m3_scale(temp, 0.5));
        for (int i = j + 1; i < NS; ++i) put_block(J, ld, 3 * i, jpos, temp);
    } else if (task < 2 * NS - 2) {
        const int j = task - (NS - 1) + 1, jpos = 3 * j;
        int ipos = 3 * (NS + j - 1);
        q_tangent(ldq(P.q + 4 * (s0 + j - 1)), t);
        M3 um = rcross(P.u + 3 * (s0 + j - 1));
        M3 tm = m3_scale(rcross(t), -1.0);
        M3 blk =
            m3_add(m3_add(tm, m3_scale(m3_mul(um, tm), 0.5)), m3_scale(m3_mul(m3_mul(um, um), tm), 1.0 / 12.0));
        put_block(J, ld, ipos, jpos, m3_scale(blk, fac1));
        ipos += 3;
        q_tangent(ldq(P.q + 4 * (s0 + j)), t);
        um = rcross(P.u + 3 * (s0 + j));
        tm = m3_scale(rcross(t), -1.0);
        blk = m3_add(m3_add(tm, m3_scale(m3_mul(um, tm), 0.5)), m3_scale(m3_mul(m3_mul(um, um), tm), 1.0 / 12.0));
        put_block(J, ld, ipos, jpos, m3_scale(blk, fac1));
    } else if (task < 3 * NS - 2) {
        lie_segment_blocks(P, fil, nt, task - (2 * NS - 2), J, ld);
    } else {
        for (int i = 0; i < 3 * NS; ++i) {
            J[i + (size_t)ld * i] = fac0;
            if (i < 3 * NS - 3) J[i + (size_t)ld * (i + 3)] = -fac0;
        }
    }
}

// The writes of invert_approx_jacobian that depend on the task blocks: the
// end-force term, the unit diagonal of the Lie-algebra block, and the two
// clamping blocks (saved, then replaced).  One CTA per filament.
__global__ void __launch_bounds__(kJacTpb) jacobian_finish_kernel(SimP P, int nt)
{
    const int fil = blockIdx.x, tid = threadIdx.x;
    const int NS = P.NS, ld = P.n6, s0 = fil * NS;
    double *J = P.invJ + (size_t)fil * ld * ld;
    const bool euler = nt < P.neuler;
    const double fac0 = euler ? -P.DT / (6.0 * kPi * P.MU * P.RSEG) : -P.DT / (9.0 * kPi * P.MU * P.RSEG);
    for (int k = tid; k < 3 * NS; k += kJacTpb) J[(3 * NS + k) + (size_t)ld * (3 * NS + k)] += 1.0;
    if (tid == 0) {
        double t[3];
        q_tangent(ldq(P.q + 4 * (s0 + NS - 1)), t);
        const M3 sub = m3_scale(rcross(t), fac0 * P.EFM);
        add_block(J, ld, 3 * (NS - 1), 3 * (2 * NS - 1), m3_scale(sub, -1.0));
    }
    __syncthreads();
    if (tid == 0) {
        const double fac = euler ? -P.DT / (8.0 * kPi * P.MU * P.RSEG * P.RSEG * P.RSEG)
                                 : -P.DT / (12.0 * kPi * P.MU * P.RSEG * P.RSEG * P.RSEG);
        const M3 um = rcross(P.u + 3 * s0);
        M3 blk = m3_add(m3_scale(um, 0.5), m3_scale(m3_mul(um, um), 1.0 / 12.0));
        M3 blkT = m3_add(m3_scale(um, -0.5), m3_scale(m3_mul(um, um), 1.0 / 12.0));
        for (int d = 0; d < 3; ++d) {
            blk(d, d) += 1.0;
            blkT(d, d) += 1.0;
        }
        const M3 e1 = get_block(J, ld, 3 * NS, 3 * NS), e2 = get_block(J, ld, 3 * NS + 3, 3 * NS);
        for (int k = 0; k < 9; ++k) {
            P.ecb1[9 * fil + k] = e1.a[k];
            P.ecb2[9 * fil + k] = e2.a[k];
        }
        put_block(J, ld, 3 * NS, 3 * NS, m3_scale(m3_mul(blk, blkT), fac));
        put_block(J, ld, 3 * NS + 3, 3 * NS, m3_zero());
    }
}

// rotated body mobility: Q B Q^T blockwise (swimmer.cpp:522-527)
__device__ void rotated_mobility(const SimP &P, const M3 &Q, double *bm /*36, column-major*/)
{
    const M3 QT = m3_T(Q);
    for (int bi = 0; bi < 2; ++bi)
        for (int bj = 0; bj < 2; ++bj) {
            const M3 b = get_block(P.mob_ref, 6, 3 * bi, 3 * bj);
            put_block(bm, 6, 3 * bi, 3 * bj, m3_mul(m3_mul(Q, b), QT));
        }
}

__device__ M3 mat6_block_mul(const double *bm6, int r0, int c0, const M3 &B)  // bm[r0.., c0..] (3x3) * B
{
    return m3_mul(get_block(bm6, 6, r0, c0), B);
}

// The B block of one filament (swimmer.cpp:553-670), then jacB = B * invJ
// (swimmer.cpp:671).  One CTA per filament, in phases that each spread the
// FP64 work over threads (a warp FP64 instruction costs the same on one
// lane as on 32): the fixed blocks; B = (rotated body mobility) B, one
// column per thread; the sphere-correction matrices, one segment per thread;
// their addition, one (column block, row half) per thread in the reference's
// segment order; the D^-1 products, one column block per thread; the scale.
// Needs NS >= 2 (as the Jacobian build does).
__global__ void __launch_bounds__(128) filament_B_kernel(SimP P, int nt)
{
    extern __shared__ double Bs[];  // 6 x n6, column-major; then scratch
    const int fil = blockIdx.x, tid = threadIdx.x, nthr = blockDim.x;
    const int n = fil / P.NF, NS = P.NS, n6 = P.n6, s0 = fil * NS;
    double *seg = Bs + 6 * n6;    // per segment: add (rows 0-2, 3-5), sub (rows 0-2, 3-5), 3x3 each
    double *spec = seg + 36 * NS;  // segment 0's columns 3NS.. terms, the last segment's end-force terms
    double *Dm = spec + 36;        // Dinv, DinvT, Bend
    double *bm = Dm + 27;          // rotated body mobility, 6 x 6 column-major
    auto ld3 = [](const double *p) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = p[k]; return m; };
    auto st3 = [](double *p, const M3 &m) { for (int k = 0; k < 9; ++k) p[k] = m.a[k]; };
    const double dt_fac = (nt < P.neuler) ? -P.DT : -2.0 * P.DT / 3.0;
    const double *u = P.bu + 3 * n, *x = P.bx + 3 * n;
    const M3 Qi = ldm3(P.bQ + 9 * n);
    for (int k = tid; k < 6 * n6; k += nthr) Bs[k] = 0.0;
    if (tid == 0) {
        const M3 blc = m3_scale(rcross(u), -1.0);
        const M3 blc2 = m3_scale(m3_mul(blc, blc), 1.0 / 12.0);
        st3(Dm, m3_sub(m3_add(m3_eye(), blc2), m3_scale(blc, 0.5)));
        st3(Dm + 9, m3_add(m3_add(m3_eye(), blc2), m3_scale(blc, 0.5)));
        double t[3], te[3];
        q_tangent(ldq(P.q + 4 * (s0 + NS - 1)), t);
        for (int c = 0; c < 3; ++c) te[c] = P.EFM * t[c];
        st3(Dm + 18, rcross(te));
    }
    if (tid >= 32 && tid < 36) {  // rotated_mobility: Q B Q^T, one 3x3 block per thread
        const int bi = (tid - 32) / 2, bj = (tid - 32) % 2;
        const M3 b = get_block(P.mob_ref, 6, 3 * bi, 3 * bj);
        put_block(bm, 6, 3 * bi, 3 * bj, m3_mul(m3_mul(Qi, b), m3_T(Qi)));
    }
    __syncthreads();
    const M3 Dinv = ld3(Dm), DinvT = ld3(Dm + 9), Bend = ld3(Dm + 18);
    if (tid == 0) {
        double fbd[3];
        m3_vec(Qi, P.fref + 3 * fil, fbd);
        Bs[0 + 6 * 0] = -1.0;
        Bs[1 + 6 * 1] = -1.0;
        Bs[2 + 6 * 2] = -1.0;
        put_block(Bs, 6, 3, 0, rcross(fbd));
        put_block(Bs, 6, 3, 3 * NS, m3_scale(DinvT, -1.0));
        put_block(Bs, 6, 0, 6 * NS - 3, Bend);
        double t[3], diff[3], w[3];
        q_tangent(ldq(P.q + 4 * (s0 + NS - 1)), t);
        for (int c = 0; c < 3; ++c) diff[c] = P.x[3 * (s0 + NS - 1) + c] - x[c];
        for (int c = 0; c < 3; ++c) w[c] = 0.5 * P.DL * t[c] - diff[c];
        put_block(Bs, 6, 3, 6 * NS - 3, m3_mul(rcross(w), Bend));
    }
    for (int m = 1 + tid; m < NS - 1; m += nthr) {
        double tm[3], dtm[3];
        q_tangent(ldq(P.q + 4 * (s0 + m)), tm);
        for (int c = 0; c < 3; ++c) dtm[c] = P.DL * tm[c];
        put_block(Bs, 6, 3, 3 * (NS + m), m3_mul(Bend, rcross(dtm)));
    }
    __syncthreads();
    // B = body_mobility * B, one column per thread
    for (int c = tid; c < n6; c += nthr) {
        double colv[6];
        for (int r = 0; r < 6; ++r) {
            double acc = 0.0;
            for (int k = 0; k < 6; ++k) acc += bm[r + 6 * k] * Bs[k + 6 * c];
            colv[r] = acc;
        }
        for (int r = 0; r < 6; ++r) Bs[r + 6 * c] = colv[r];
    }
    // sphere corrections (swimmer.cpp:604-658), one segment per thread
    const double R = P.Rbody;
    const double R2 = R * R + P.RSEG * P.RSEG;
    for (int k = tid; k < NS; k += nthr) {
        double rh[3];
        for (int c = 0; c < 3; ++c) rh[c] = P.x[3 * (s0 + k) + c] - x[c];
        const double r = sqrt(rh[0] * rh[0] + rh[1] * rh[1] + rh[2] * rh[2]);
        for (int c = 0; c < 3; ++c) rh[c] /= r;
        M3 rr, I = m3_eye();
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) rr(i, j) = rh[i] * rh[j];
        const M3 Mtt = m3_scale(m3_add(m3_scale(I, 1.0 + R2 / (3.0 * r * r)), m3_scale(rr, 1.0 - R2 / (r * r))),
                                1.0 / (8.0 * kPi * P.MU * r));
        const M3 Mtr = m3_scale(rcross(rh), 1.0 / (8.0 * kPi * P.MU * r * r));
        const M3 Mrr = m3_scale(m3_sub(m3_scale(rr, 3.0), I), 1.0 / (16.0 * kPi * P.MU * r * r * r));
        double tk[3];
        q_tangent(ldq(P.q + 4 * (s0 + k)), tk);
        const M3 temp = rcross(tk);
        const M3 Mtr_t = m3_mul(m3_scale(Mtr, 0.5 * P.DL), temp);
        const M3 Mrr_t = m3_mul(m3_scale(Mrr, 0.5 * P.DL), temp);
        double *o = seg + 36 * k;
        if (k == 0) {
            st3(o, Mtt);
            st3(o + 9, Mtr);
            st3(spec, m3_mul(Mtr, DinvT));
            st3(spec + 9, m3_mul(Mrr, DinvT));
            st3(o + 18, m3_sub(Mtr_t, Mtt));
            st3(o + 27, m3_sub(Mrr_t, Mtr));
        } else if (k == NS - 1) {
            st3(spec + 18, m3_mul(m3_scale(Mtt, -P.EFM), temp));
            st3(spec + 27, m3_mul(m3_scale(Mtr, -P.EFM), temp));
            st3(o, m3_add(Mtr_t, Mtt));
            st3(o + 9, m3_add(Mrr_t, Mtr));
        } else {
            st3(o, m3_add(Mtr_t, Mtt));
            st3(o + 9, m3_add(Mrr_t, Mtr));
            st3(o + 18, m3_sub(Mtr_t, Mtt));
            st3(o + 27, m3_sub(Mrr_t, Mtr));
        }
    }
    __syncthreads();
    // column block cb gets segment cb-1's second pair of terms, then segment
    // cb's first (the order of the reference's segment loop)
    for (int t = tid; t < 4 * NS; t += nthr) {
        const int cb = t / 2, half = t % 2, r0 = 3 * half;
        if (cb == 0) {
            add_block(Bs, 6, r0, 0, ld3(seg + 9 * half));
        } else if (cb < NS) {
            add_block(Bs, 6, r0, 3 * cb, ld3(seg + 36 * (cb - 1) + 18 + 9 * half));
            add_block(Bs, 6, r0, 3 * cb, ld3(seg + 36 * cb + 9 * half));
        } else if (cb == NS) {
            add_block(Bs, 6, r0, 3 * NS, ld3(spec + 9 * half));
        } else if (cb == 2 * NS - 1) {
            add_block(Bs, 6, r0, 6 * NS - 3, ld3(spec + 18 + 9 * half));
        }
    }
    __syncthreads();
    for (int cb = tid; cb < 2 * NS; cb += nthr) put_block(Bs, 6, 3, 3 * cb, m3_mul(Dinv, get_block(Bs, 6, 3, 3 * cb)));
    __syncthreads();
    for (int k = tid; k < 6 * n6; k += nthr) Bs[k] *= dt_fac;
    __syncthreads();
    const double *Jinv = P.invJ + (size_t)fil * n6 * n6;
    double *jB = P.jacB + (size_t)fil * 6 * n6;
    for (int c = threadIdx.x; c < n6; c += blockDim.x) {
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < n6; ++k) {
            const double jv = Jinv[k + (size_t)n6 * c];
            for (int r = 0; r < 6; ++r) acc[r] += Bs[r + 6 * k] * jv;
        }
        for (int r = 0; r < 6; ++r) jB[r + 6 * c] = acc[r];
    }
}

// 6x6 inverse (Gauss-Jordan, partial pivoting), column-major in place.
__device__ bool invert6_dev(double *A)
{
    double M[6][12];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            M[i][j] = A[i + 6 * j];
            M[i][6 + j] = i == j ? 1.0 : 0.0;
        }
    for (int c = 0; c < 6; ++c) {
        int p = c;
        for (int r = c + 1; r < 6; ++r)
            if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
        if (M[p][c] == 0.0) return false;
        if (p != c)
            for (int j = 0; j < 12; ++j) {
                const double t = M[c][j];
                M[c][j] = M[p][j];
                M[p][j] = t;
            }
        const double d = M[c][c];
        for (int j = 0; j < 12; ++j) M[c][j] /= d;
        for (int r = 0; r < 6; ++r)
            if (r != c) {
                const double f = M[r][c];
                if (f != 0.0)
                    for (int j = 0; j < 12; ++j) M[r][j] -= f * M[c][j];
            }
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) A[i + 6 * j] = M[i][6 + j];
    return true;
}

// A_f * (U, Omega) for the swimmer.cpp:800-812 block A of filament fil.
__device__ void A_apply(const SimP &P, int fil, const double *ub, int row, double *out3)
{
    const int NS = P.NS, n = fil / P.NF;
    const M3 Qi = ldm3(P.bQ + 9 * n);
    if (row < 3 * NS) {
        double fbd[3], dd[3];
        m3_vec(Qi, P.fref + 3 * fil, fbd);
        const double dn = sqrt(fbd[0] * fbd[0] + fbd[1] * fbd[1] + fbd[2] * fbd[2]);
        for (int c = 0; c < 3; ++c) dd[c] = (0.5 * P.DL + dn) * fbd[c] / dn;
        const M3 D = rcross(dd);
        double t[3];
        m3_vec(D, ub + 3, t);
        for (int c = 0; c < 3; ++c) out3[c] = ub[c] + t[c];
    } else if (row == 3 * NS) {
        m3_vec(ldm3(P.ecb1 + 9 * fil), ub + 3, out3);
    } else if (row == 3 * NS + 3) {
        m3_vec(ldm3(P.ecb2 + 9 * fil), ub + 3, out3);
    } else {
        out3[0] = out3[1] = out3[2] = 0.0;
    }
}

// Per-filament parts of the swimmer's 6x6 Schur complement
// (swimmer.cpp:466-682, GMRES branch), one CTA per filament: thread c < 6
// forms column c of jacB_f * A_f (A_f applied to the unit body velocity e_c,
// row block by row block, in row order); thread 6 forms the filament's 3x3
// term of the body rotation block.  part[45 fil + 6c + r] and part[45 fil + 36 + 3i + j].
__global__ void __launch_bounds__(32) schur_filament_kernel(SimP P, double *part)
{
    const int fil = blockIdx.x, n = fil / P.NF, NS = P.NS, n6 = P.n6, c = threadIdx.x;
    double *out = part + 45 * (size_t)fil;
    const M3 Qi = ldm3(P.bQ + 9 * n);
    double fbd[3], dd[3];
    m3_vec(Qi, P.fref + 3 * fil, fbd);
    const double dn = sqrt(fbd[0] * fbd[0] + fbd[1] * fbd[1] + fbd[2] * fbd[2]);
    for (int k = 0; k < 3; ++k) dd[k] = (0.5 * P.DL + dn) * fbd[k] / dn;
    if (c < 6) {
        // the rows of A_f e_c (A_apply): [I | rcross(dd)] on the position rows,
        // the end-clamp blocks on rows 3NS and 3NS+3, zero elsewhere
        double ub[6] = {0, 0, 0, 0, 0, 0};
        ub[c] = 1.0;
        double at[3], a1[3], a2[3], t[3];
        m3_vec(rcross(dd), ub + 3, t);
        for (int k = 0; k < 3; ++k) at[k] = ub[k] + t[k];
        m3_vec(ldm3(P.ecb1 + 9 * fil), ub + 3, a1);
        m3_vec(ldm3(P.ecb2 + 9 * fil), ub + 3, a2);
        const double *jB = P.jacB + (size_t)fil * 6 * n6;
        double colv[6] = {0, 0, 0, 0, 0, 0};
        for (int row = 0; row < n6; row += 3) {
            const double *a3 = row < 3 * NS ? at : row == 3 * NS ? a1 : row == 3 * NS + 3 ? a2 : nullptr;
            if (a3 == nullptr) continue;
            for (int r = 0; r < 6; ++r)
                colv[r] += jB[r + 6 * row] * a3[0] + jB[r + 6 * (row + 1)] * a3[1] + jB[r + 6 * (row + 2)] * a3[2];
        }
        for (int r = 0; r < 6; ++r) out[6 * c + r] = colv[r];
    } else if (c == 6) {
        const double *u = P.bu + 3 * n;
        const M3 blc = m3_scale(rcross(u), -1.0);
        M3 o = m3_sub(m3_zero(), m3_mul(rcross(P.tl + 3 * fil), rcross(fbd)));
        const double *cl = P.cl + 3 * fil;
        const double ucl[3] = {u[1] * cl[2] - u[2] * cl[1], u[2] * cl[0] - u[0] * cl[2], u[0] * cl[1] - u[1] * cl[0]};
        o = m3_add(o, m3_sub(m3_scale(rcross(cl), 0.5),
                             m3_scale(m3_add(rcross(ucl), m3_mul(blc, rcross(cl))), 1.0 / 12.0)));
        double tg[3], te[3];
        q_tangent(ldq(P.q + 4 * (fil * NS + NS - 1)), tg);
        for (int k = 0; k < 3; ++k) te[k] = P.EFM * tg[k];
        o = m3_add(o, m3_mul(rcross(te), rcross(dd)));
        for (int k = 0; k < 9; ++k) out[36 + k] = o.a[k];
    }
}

// The swimmer's Schur complement from the per-filament parts (summed in
// filament order), inverted in place.  One CTA per swimmer.
__global__ void __launch_bounds__(64) swimmer_schur_kernel(SimP P, int nt, const double *part)
{
    __shared__ double sums[45];
    const int n = blockIdx.x;
    if (threadIdx.x < 45) {
        double t = 0.0;
        for (int i = 0; i < P.NF; ++i) t += part[45 * (size_t)(n * P.NF + i) + threadIdx.x];
        sums[threadIdx.x] = t;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double dt_fac = (nt < P.neuler) ? -P.DT : -2.0 * P.DT / 3.0;
    const double *u = P.bu + 3 * n;
    const M3 Qi = ldm3(P.bQ + 9 * n);
    const M3 blc = m3_scale(rcross(u), -1.0);
    const M3 cbo = m3_scale(blc, -1.0 / dt_fac);
    double S6[36];
    for (int k = 0; k < 36; ++k) S6[k] = 0.0;
    for (int d = 0; d < 6; ++d) S6[d + 6 * d] = 1.0;
    add_block(S6, 6, 3, 3, m3_scale(m3_sub(m3_scale(m3_mul(blc, cbo), 1.0 / 12.0), m3_scale(cbo, 0.5)), dt_fac));
    M3 old;
    for (int k = 0; k < 9; ++k) old.a[k] = sums[36 + k];
    double bm[36];
    rotated_mobility(P, Qi, bm);
    old = m3_mul(get_block(bm, 6, 3, 3), old);
    const M3 add = m3_add(m3_sub(old, m3_scale(m3_mul(blc, old), 0.5)), m3_scale(m3_mul(m3_mul(blc, blc), old), 1.0 / 12.0));
    add_block(S6, 6, 3, 3, m3_scale(add, dt_fac));
    for (int k = 0; k < 36; ++k) S6[k] -= sums[k];
    if (!invert6_dev(S6)) atomicOr(P.flags + 2, 1);
    for (int k = 0; k < 36; ++k) P.schur[36 * n + k] = S6[k];
}

// jacobian_inv_mult (swimmer.cpp:793-837), in two launches.
// (1)+(2) per filament: part[6 fil..] = jacB_f * in_f; then, in the last CTA
// to arrive, per swimmer (one warp each): out_body = schur_inv *
// (in_body - sum_f part_f), the filaments' parts added by lanes strided over
// the filaments and a warp sum.
__global__ void __launch_bounds__(128) jim_partial_body_kernel(SimP P, const double *in, double *part, double *out,
                                                               int *ticket)
{
    __shared__ double red[6][4];
    __shared__ double b2[4][6];
    const int fil = blockIdx.x, n = fil / P.NF, i = fil % P.NF;
    const double *x = in + (size_t)n * P.per_body + (size_t)6 * P.NS * i;
    const double *jB = P.jacB + (size_t)fil * 6 * P.n6;
    double a[6] = {0, 0, 0, 0, 0, 0};
    for (int c = threadIdx.x; c < P.n6; c += 128)
        for (int r = 0; r < 6; ++r) a[r] += jB[r + 6 * c] * x[c];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int r = 0; r < 6; ++r) {
        const double v = warp_sum_d(a[r]);
        if (lane == 0) red[r][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) part[6 * fil + threadIdx.x] = red[threadIdx.x][0] + red[threadIdx.x][1] +
                                                       red[threadIdx.x][2] + red[threadIdx.x][3];
    if (!last_cta(ticket, gridDim.x)) return;
    for (int sw = wid; sw < P.W; sw += 4) {
        const size_t b = (size_t)sw * P.per_body + 6 * P.NF * P.NS;
        for (int r = 0; r < 6; ++r) {
            double v = 0.0;
            for (int f = lane; f < P.NF; f += 32) v += __ldcg(part + 6 * (sw * P.NF + f) + r);
            v = warp_sum_d(v);
            if (lane == 0) b2[wid][r] = in[b + r] - v;
        }
        __syncwarp();
        if (lane < 6) {
            const double *Si = P.schur + 36 * sw;
            double s = 0.0;
            for (int k = 0; k < 6; ++k) s += Si[lane + 6 * k] * b2[wid][k];
            out[b + lane] = s;
        }
        __syncwarp();
    }
}

// (3) per filament: out_f = invJ_f * (in_f - A_f out_body)
__global__ void __launch_bounds__(128) jim_fil_kernel(SimP P, const double *in, double *out)
{
    extern __shared__ double rhs[];
    const int fil = blockIdx.x, n = fil / P.NF, i = fil % P.NF, n6 = P.n6;
    const size_t base = (size_t)n * P.per_body + (size_t)6 * P.NS * i;
    const double *ub = out + (size_t)n * P.per_body + 6 * P.NF * P.NS;
    for (int row = threadIdx.x * 3; row < n6; row += 3 * 128) {
        double a3[3] = {0.0, 0.0, 0.0};
        if (!P.wall) A_apply(P, fil, ub, row, a3);  // the wall branch is invJ_f in_f (swimmer.cpp:696-702)
        for (int c = 0; c < 3; ++c) rhs[row + c] = in[base + row + c] - a3[c];
    }
    __syncthreads();
    const double *Ji = P.invJ + (size_t)fil * n6 * n6;
    for (int r = threadIdx.x; r < n6; r += 128) {
        double s = 0.0;
        for (int k = 0; k < n6; ++k) s += Ji[r + (size_t)n6 * k] * rhs[k];
        out[base + r] = s;
    }
}

// rigid_body::update (rigid_body.cpp:354-381) for the body part of the update.
__global__ void body_update_kernel(SimP P, const double *upd)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= P.W) return;
    const double *b = upd + (size_t)n * P.per_body + 6 * P.NF * P.NS;
    for (int c = 0; c < 3; ++c) {
        P.bx[3 * n + c] += b[c];
        P.bu[3 * n + c] += b[3 + c];
    }
    stq(P.bq + 4 * n, qmul(lie_exp(P.bu + 3 * n), ldq(P.bqm1 + 4 * n)));
}

// swimmer::update's per-filament part (swimmer.cpp:858-868) with
// filament::update (filament.cpp:1541-1575), in two passes.  Pass 1, thread
// per segment: segment 0 takes the body's state (accept_state_from_rigid_body,
// filament.cpp:438-463: base position, u = body u); the others add their
// update to u and the multiplier of the link before them; each segment's new
// tangent goes to scratch.  (accept_state_from_rigid_body's own robot_arm is
// left out: every position it writes is rewritten by the final robot_arm from
// the same base.)
__global__ void filament_update_segments_kernel(SimP P, const double *upd)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.S) return;
    const int NS = P.NS, fil = s / NS, k = s % NS, n = fil / P.NF, i = fil % P.NF;
    const double *du = upd + (size_t)n * P.per_body + (size_t)6 * NS * i;
    if (k == 0) {
        double base[3];
        base_position(P, fil, base);
        for (int c = 0; c < 3; ++c) P.x[3 * s + c] = base[c];
        const double d0[3] = {P.bu[3 * n] - P.u[3 * s], P.bu[3 * n + 1] - P.u[3 * s + 1],
                              P.bu[3 * n + 2] - P.u[3 * s + 2]};
        segment_update(P, s, d0);
        for (int c = 0; c < 3; ++c) P.tl[3 * fil + c] += du[c];
        for (int c = 0; c < 3; ++c) P.cl[3 * fil + c] += du[3 * NS + c];
    } else {
        double *lam = P.lam + 3 * (NS - 1) * (size_t)fil;
        for (int c = 0; c < 3; ++c) lam[3 * (k - 1) + c] += du[3 * k + c];
        segment_update(P, s, du + 3 * (NS + k));
    }
    q_tangent(ldq(P.q + 4 * s), P.tang + 3 * (size_t)s);
}

// Pass 2, thread per (filament, coordinate): robot_arm (filament.cpp:416-436),
// positions by midpoint-tangent chaining from the base.
__global__ void filament_robot_arm_kernel(SimP P)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= 3 * P.F) return;
    const int fil = g / 3, c = g % 3, s0 = fil * P.NS;
    for (int i = 1; i < P.NS; ++i) {
        const int s = s0 + i;
        P.x[3 * s + c] = P.x[3 * (s - 1) + c] + 0.5 * P.DL * (P.tang[3 * (s - 1) + c] + P.tang[3 * s + c]);
    }
}

// ---- Broyden vector kernels ----------------------------------------------
constexpr int kVecTpb = 256;
constexpr int kVecChunk = 2048;

// dots[i] = M[:, i] . v (i < k) in one launch: part[i * nch + c] = the sum
// over chunk c; the last CTA to arrive adds each column's chunks in order.
__global__ void __launch_bounds__(kVecTpb) coldot_kernel(const double *M, size_t ld, int k, const double *v, int n,
                                                          int nch, double *part, double *dots, int *ticket)
{
    __shared__ double red[8];
    const int c = blockIdx.x, i = blockIdx.y;
    double a = 0.0;
    const int r1 = min(n, (c + 1) * kVecChunk);
    for (int r = c * kVecChunk + threadIdx.x; r < r1; r += kVecTpb) a += M[ld * i + r] * v[r];
    a = warp_sum_d(a);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kVecTpb / 32; ++w) s += red[w];
        part[(size_t)i * nch + c] = s;
    }
    if (!last_cta(ticket, gridDim.x * gridDim.y)) return;
    for (int j = threadIdx.x; j < k; j += kVecTpb) {
        double s = 0.0;
        for (int cc = 0; cc < nch; ++cc) s += __ldcg(part + (size_t)j * nch + cc);
        dots[j] = s;
    }
}

// out[r] = a * x[r] - sum_{i<k} dots[i] C[r, i]   (in order of i)
__global__ void broyden_combine_kernel(int n, double a, const double *x, const double *C, size_t ld, const double *dots,
                                       int k, double *out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double v = a * x[r];
    for (int i = 0; i < k; ++i) v -= dots[i] * C[ld * i + r];
    out[r] = v;
}

__global__ void vec_sub_kernel(int n, const double *a, const double *b, double *out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) out[r] = a[r] - b[r];
}

__global__ void vec_div2_kernel(int n, double *a, double *b, const double *nrm2)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const double d = sqrt(nrm2[0]);
    if (r < n) {
        a[r] /= d;
        b[r] /= d;
    }
}

// ---- prescribed preferred-curvature beat ----------------------------------
// filament::body_frame_moment's strain_twist (filament.cpp:1104-1106) as a
// time-dependent preferred bending curvature: for time step nt (solving for
// t = (nt + 1) dt), strain_twist = (0, A sin(2 pi t / T + phase_f), 0).
__global__ void beat_strain_kernel(SimP P, const double *phase, double amplitude, double omega, double t)
{
    const int fil = blockIdx.x * blockDim.x + threadIdx.x;
    if (fil >= P.F) return;
    P.st[3 * fil] = 0.0;
    P.st[3 * fil + 1] = amplitude * sin(omega * t + phase[fil]);
    P.st[3 * fil + 2] = 0.0;
}

// ---- learned initial inverse Jacobian ------------------------------------
// Each filament's local frame: e3 along its base direction (R_body fref; +z
// on the wall), e1 the body's x axis (its y axis near the poles) made
// orthogonal to e3, e2 = e3 x e1.  frames[9 fil + 3 c + j] = (e_c)_j.
__device__ void filament_frame(const SimP &P, int fil, double E[9])
{
    double e1[3], e3[3];
    if (P.wall) {
        e3[0] = 0.0; e3[1] = 0.0; e3[2] = 1.0;
        e1[0] = 1.0; e1[1] = 0.0; e1[2] = 0.0;
    } else {
        const int n = fil / P.NF;
        const M3 R = q_rot_mat(ldq(P.bq + 4 * n));
        double a[3];
        m3_vec(R, P.fref + 3 * fil, a);
        const double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        for (int c = 0; c < 3; ++c) e3[c] = a[c] / na;
        double x[3] = {R(0, 0), R(1, 0), R(2, 0)};
        if (fabs(x[0] * e3[0] + x[1] * e3[1] + x[2] * e3[2]) > 0.9) {
            x[0] = R(0, 1); x[1] = R(1, 1); x[2] = R(2, 1);
        }
        const double d = x[0] * e3[0] + x[1] * e3[1] + x[2] * e3[2];
        for (int c = 0; c < 3; ++c) e1[c] = x[c] - d * e3[c];
        const double n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        for (int c = 0; c < 3; ++c) e1[c] /= n1;
    }
    const double e2[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
    for (int c = 0; c < 3; ++c) {
        E[c] = e1[c];
        E[3 + c] = e2[c];
        E[6 + c] = e3[c];
    }
}

// Thread per filament: its frame and its features phi (per segment, the
// position relative to the base over the filament length, then the
// tangent, both in the local frame), FP32 and bf16.
__global__ void filament_features_kernel(SimP P, double *frames, float *phi, __nv_bfloat16 *phi16)
{
    const int fil = blockIdx.x * blockDim.x + threadIdx.x;
    if (fil >= P.F) return;
    double E[9];
    filament_frame(P, fil, E);
    for (int k = 0; k < 9; ++k) frames[9 * (size_t)fil + k] = E[k];
    const int s0 = fil * P.NS, n6 = P.n6;
    const double inv_len = 1.0 / (P.NS * P.DL);
    for (int i = 0; i < P.NS; ++i) {
        const int sg = s0 + i;
        double d[3], t[3];
        for (int c = 0; c < 3; ++c) d[c] = P.x[3 * sg + c] - P.x[3 * s0 + c];
        q_tangent(ldq(P.q + 4 * sg), t);
        for (int c = 0; c < 3; ++c) {
            const double pv = (E[3 * c] * d[0] + E[3 * c + 1] * d[1] + E[3 * c + 2] * d[2]) * inv_len;
            const double tv = E[3 * c] * t[0] + E[3 * c + 1] * t[1] + E[3 * c + 2] * t[2];
            const size_t o = (size_t)fil * n6 + 6 * i;
            phi[o + c] = (float)pv;
            phi[o + 3 + c] = (float)tv;
            phi16[o + c] = __float2bfloat16_rn((float)pv);
            phi16[o + 3 + c] = __float2bfloat16_rn((float)tv);
        }
    }
}

// tmp_f <- sigma (.) tmp_f + (1/conf) E^T U V^T E in_f for every filament f
// (tmp holds Jinv in from jacobian_inv_mult; the caller's combine step
// multiplies by -conf), one CTA per filament; the body rows are left as
// they are.  O: the network's output rows [F x n_out] (see gmi_mlp.cu).
template <int R>
__global__ void __launch_bounds__(128) learned_apply_kernel(SimP P, const float *__restrict__ O, int n_out,
                                                            const double *__restrict__ frames,
                                                            const double *__restrict__ in, double *__restrict__ tmp,
                                                            double inv_conf)
{
    extern __shared__ double dl[];  // n6: in_f in the local frame
    __shared__ double red[4][R], y[R];
    const int fil = blockIdx.x, n = fil / P.NF, i = fil % P.NF, NS = P.NS, n6 = P.n6, nblk = 2 * NS;
    const size_t base = (size_t)n * P.per_body + (size_t)6 * NS * i;
    const double *E = frames + 9 * (size_t)fil;
    const float *o = O + (size_t)fil * n_out, *U = o + nblk, *V = U + (size_t)n6 * R;
    for (int k = threadIdx.x; k < nblk; k += 128) {
        const double *v = in + base + 3 * k;
        for (int c = 0; c < 3; ++c) dl[3 * k + c] = E[3 * c] * v[0] + E[3 * c + 1] * v[1] + E[3 * c + 2] * v[2];
    }
    __syncthreads();
    double yp[R];
#pragma unroll
    for (int j = 0; j < R; ++j) yp[j] = 0.0;
    for (int r = threadIdx.x; r < n6; r += 128)
#pragma unroll
        for (int j = 0; j < R; ++j) yp[j] += (double)V[r * R + j] * dl[r];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const double v = warp_sum_d(yp[j]);
        if (lane == 0) red[w][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < R) y[threadIdx.x] = red[0][threadIdx.x] + red[1][threadIdx.x] + red[2][threadIdx.x] +
                                          red[3][threadIdx.x];
    __syncthreads();
    for (int k = threadIdx.x; k < nblk; k += 128) {
        double cl[3];
        for (int c = 0; c < 3; ++c) {
            double a = 0.0;
#pragma unroll
            for (int j = 0; j < R; ++j) a += (double)U[(3 * k + c) * R + j] * y[j];
            cl[c] = a;
        }
        const double sg = exp((double)fminf(fmaxf(o[k], -3.f), 3.f));
        double *t = tmp + base + 3 * k;
        for (int c = 0; c < 3; ++c) {
            const double lab = E[c] * cl[0] + E[3 + c] * cl[1] + E[6 + c] * cl[2];
            t[c] = sg * t[c] + inv_conf * lab;
        }
    }
}

// One secant-pair record per filament (layout in gmi_mlp.cu): phi, then
// d = dv_f, b = conf jv_f, t = upd_f rotated into the local frame; record
// index first + fil, skipped past capacity.
__global__ void secant_record_kernel(SimP P, const double *__restrict__ frames, const float *__restrict__ phi,
                                     const double *__restrict__ dv, const double *__restrict__ jv,
                                     const double *__restrict__ upd, double conf, float *__restrict__ rec,
                                     long long first, long long cap)
{
    const int fil = blockIdx.x, n = fil / P.NF, i = fil % P.NF, n6 = P.n6, nblk = 2 * P.NS;
    const long long r = first + fil;
    if (r >= cap) return;
    float *out = rec + r * (long long)(4 * n6);
    const size_t base = (size_t)n * P.per_body + (size_t)6 * P.NS * i;
    const double *E = frames + 9 * (size_t)fil;
    for (int c = threadIdx.x; c < n6; c += blockDim.x) out[c] = phi[(size_t)fil * n6 + c];
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
        const double *src[3] = {dv + base + 3 * k, jv + base + 3 * k, upd + base + 3 * k};
        const double sc[3] = {1.0, conf, 1.0};
        for (int q = 0; q < 3; ++q)
            for (int c = 0; c < 3; ++c)
                out[(q + 1) * n6 + 3 * k + c] =
                    (float)(sc[q] * (E[3 * c] * src[q][0] + E[3 * c + 1] * src[q][1] + E[3 * c + 2] * src[q][2]));
    }
}

// Random probe directions for the Jacobian, one CTA per filament: on the
// filament's 6 NS rows r_i = g_i (|e_i| + e_f / 4), g_i standard normal
// (splitmix64 counter hash, Box-Muller), e = the Broyden error of the step's
// initial guess and e_f its RMS over the filament's rows, so that a probe
// carries every component of the error in its own units; body rows are
// zero.  The probe update is then -conf Jinv r: a first Broyden step from a
// random error of the current one's size.
__device__ __forceinline__ unsigned long long probe_hash(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void __launch_bounds__(128) probe_direction_kernel(SimP P, const double *__restrict__ err,
                                                              unsigned long long seed, double *__restrict__ r)
{
    const int fil = blockIdx.x, n = fil / P.NF, i = fil % P.NF, n6 = P.n6;
    const size_t base = (size_t)n * P.per_body + (size_t)6 * P.NS * i;
    __shared__ double red[4];
    double s = 0.0;
    for (int k = threadIdx.x; k < n6; k += 128) s += err[base + k] * err[base + k];
    s = warp_sum_d(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    const double ef = sqrt((red[0] + red[1] + red[2] + red[3]) / n6);
    for (int k = threadIdx.x; k < n6; k += 128) {
        const unsigned long long h = probe_hash(seed ^ probe_hash(base + k));
        const double u1 = ((double)(h >> 11) + 1.0) * 0x1.0p-53;  // (0, 1]
        const double u2 = (double)(probe_hash(h) >> 11) * 0x1.0p-53;
        const double g = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
        r[base + k] = g * (fabs(err[base + k]) + 0.25 * ef);
    }
    if (i == 0 && !P.wall)  // the swimmer's body rows (6, after its filaments)
        for (int k = threadIdx.x; k < 6; k += 128) r[(size_t)n * P.per_body + (size_t)6 * P.NS * P.NF + k] = 0.0;
}

__global__ void vec_scale_kernel(int n, double a, const double *__restrict__ x, double *__restrict__ y)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) y[r] = a * x[r];
}
}  // namespace gmi

// ---------------------------------------------------------------------------
// simulation object and host control flow
// ---------------------------------------------------------------------------
struct gmi_sim {
    gmi_sim_config cfg{};
    gmi_solver *solver = nullptr;
    gmi::SimP P{};
    int maxb = 100;
    double *C = nullptr, *D = nullptr, *err = nullptr, *nerr = nullptr, *upd = nullptr, *tmp = nullptr;
    double *dots = nullptr, *part = nullptr, *jpart = nullptr, *scal = nullptr;
    double *spart = nullptr;  // per-filament parts of the Schur complement (45 each)
    double *f_internal = nullptr;  // segment forces before the barrier (the reference's f_segs_host)
    double *fs_part = nullptr;     // per-CTA partials of the swimmer force/torque sums
    int *tickets = nullptr;        // swimmer_force_kernel [0], jim_partial_body_kernel [1], coldot_kernel [2]
    int *h_flags = nullptr;
    std::vector<void *> allocs;
    bool prepared = false;
    int broyden_iter = 0;
    bool use_gj_cluster = true;   // GMI_GJ_CLUSTER=0: one CTA per Jacobian inversion always
    bool use_gj_registers = true;  // GMI_GJ_REGISTERS=0: the columns stepped through shared memory
    bool gj_fp32 = false;          // FP32C steps: the approximate Jacobians inverted in FP32 (GMI_GJ_FP32=0: FP64)
    float *invJ32 = nullptr;       // their FP32 copy
    // learned initial inverse Jacobian (gmi_sim_set_learned_jacobian)
    const gmi_mlp *mlp = nullptr;
    int rank = 0;
    gmi_learned_policy policy{};
    bool learned_now = false;       // this Broyden solve applies the network's H0
    double *frames = nullptr;       // [F x 9] local frames
    float *phi = nullptr;           // [F x n6] features
    __nv_bfloat16 *phi16 = nullptr, *H1 = nullptr, *H2 = nullptr;
    float *O = nullptr;             // [F x n_out] network outputs of this step
    bool features_ready = false;
    // secant-pair collection (gmi_sim_set_secant_buffer)
    float *sec = nullptr;
    long long sec_cap = 0, sec_count = 0;
    double *dv = nullptr, *jv = nullptr;  // d = change of the error, Jinv d
    // Jacobian probes recorded with the secant pairs (gmi_sim_set_jacobian_probes)
    int probes = 0;
    bool secant_pairs = true;
    unsigned long long probe_seed = 0, probe_serial = 0;
    double *probe_r = nullptr;
    // prescribed preferred-curvature beat (gmi_sim_set_beat)
    double *beat_phase = nullptr;
    double beat_amplitude = 0.0, beat_period = 1.0;
    bool beat = false;
    // the state after the initial guess, for a learned step that is restarted plain
    struct Field {
        double *p;
        size_t n;
    };
    std::vector<Field> snap_fields;
    double *snap = nullptr;
};

namespace gmi {

static inline int gridN(int n, int tpb = 128) { return (n + tpb - 1) / tpb; }


static gmi_status sim_alloc(gmi_sim *m, double **p, size_t count)
{
    if (count == 0) count = 1;
    GMI_CUDA_TRY(dev_malloc(p, count * sizeof(double)));
    m->allocs.push_back(*p);
    GMI_CUDA_TRY(cudaMemsetAsync(*p, 0, count * sizeof(double), m->solver->ctx->stream));
    return GMI_OK;
}

static gmi_status sim_alloc_bytes(gmi_sim *m, void **p, size_t bytes)
{
    if (bytes < 16) bytes = 16;
    GMI_CUDA_TRY(dev_malloc(p, bytes));
    m->allocs.push_back(*p);
    GMI_CUDA_TRY(cudaMemsetAsync(*p, 0, bytes, m->solver->ctx->stream));
    return GMI_OK;
}

static gmi_status sim_launched(gmi_sim *m, int k = 1)
{
    m->solver->ctx->launches += k;
    GMI_CUDA_TRY(cudaGetLastError());
    return GMI_OK;
}

static cudaStream_t sst(gmi_sim *m) { return m->solver->ctx->stream; }

static gmi_status read_flags(gmi_sim *m)
{
    GMI_CUDA_TRY(cudaMemcpyAsync(m->h_flags, m->P.flags, 3 * sizeof(int), cudaMemcpyDeviceToHost, sst(m)));
    GMI_CUDA_TRY(cudaStreamSynchronize(sst(m)));
    return GMI_OK;
}

static gmi_status forces_and_torques(gmi_sim *m, int nt)
{
    if (m->P.NS > 1) filament_link_terms_kernel<<<gridN(m->P.F * (m->P.NS - 1), 64), 64, 0, sst(m)>>>(m->P);
    filament_forces_kernel<<<gridN(m->P.S, 64), 64, 0, sst(m)>>>(m->P, nt);
    GMI_TRY(sim_launched(m, m->P.NS > 1 ? 2 : 1));
    // the host copy of the segment forces never receives the barrier forces
    // (mobility_solver.cpp:132-192); keep it for the writers
    GMI_CUDA_TRY(cudaMemcpyAsync(m->f_internal, m->P.f, 6 * (size_t)m->P.S * sizeof(double),
                                 cudaMemcpyDeviceToDevice, sst(m)));
    if (m->P.wall) return GMI_OK;
    const int gx = gridN(m->P.NF * m->P.NS, kFsSegs);
    swimmer_force_kernel<<<dim3(gx, m->P.W), kFsSegs, 0, sst(m)>>>(m->P, m->fs_part, m->tickets);
    return sim_launched(m);
}

// compute_velocities + compute_errors; sets *too_large, *nonfinite
static gmi_status velocities_and_errors(gmi_sim *m, int nt, double *err_out, bool *too_large, bool *nonfinite,
                                        int *gmres_iters)
{
    GMI_TRY(solver_compute_velocities_device(m->solver, gmres_iters));
    GMI_CUDA_TRY(cudaMemsetAsync(m->P.flags, 0, 3 * sizeof(int), sst(m)));
    const int rows = m->P.S + (m->P.wall ? 0 : m->P.W);  // the wall has no body equations
    compute_errors_kernel<<<gridN(rows), 128, 0, sst(m)>>>(m->P, nt, err_out);
    GMI_TRY(sim_launched(m));
    GMI_TRY(read_flags(m));
    *too_large = m->h_flags[0] != 0;
    *nonfinite = m->h_flags[1] != 0;
    return GMI_OK;
}

// FP64 <-> FP32 copies of the Jacobians (grid-stride)
__global__ void narrow_kernel(size_t n, const double *__restrict__ in, float *__restrict__ out)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}
__global__ void widen_kernel(size_t n, const float *__restrict__ in, double *__restrict__ out)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

static gmi_status prepare_jacobian_inv(gmi_sim *m, int nt)
{
    const SimP &P = m->P;
    GMI_CUDA_TRY(cudaMemsetAsync(P.invJ, 0, (size_t)P.F * P.n6 * P.n6 * sizeof(double), sst(m)));
    build_jacobian_kernel<<<dim3((P.F + kJacTpb - 1) / kJacTpb, 3 * P.NS - 1), kJacTpb, 0, sst(m)>>>(P, nt);
    jacobian_finish_kernel<<<P.F, kJacTpb, 0, sst(m)>>>(P, nt);
    // few filaments: each inversion spread over a cluster of CTAs
    const int csize = m->use_gj_cluster ? gj_cluster_size(P.F, P.n6, m->solver->ctx->sm_count) : 1;
    const size_t jn = (size_t)P.F * P.n6 * P.n6;
    if (m->gj_fp32) {
        // the mixed-precision step: the approximate inverse in FP32, widened
        if (!m->invJ32) {
            GMI_CUDA_TRY(dev_malloc(reinterpret_cast<void **>(&m->invJ32), jn * sizeof(float)));
            m->allocs.push_back(m->invJ32);
        }
        const unsigned g = (unsigned)std::min<size_t>((jn + 255) / 256, 65535u * 8u);
        narrow_kernel<<<g, 256, 0, sst(m)>>>(jn, P.invJ, m->invJ32);
        GMI_TRY(gj_invert(sst(m), m->invJ32, P.F, P.n6, csize, m->use_gj_registers, m->solver->ctx->device,
                          P.flags));
        widen_kernel<<<g, 256, 0, sst(m)>>>(jn, m->invJ32, P.invJ);
        GMI_TRY(sim_launched(m, 2));
    } else {
        GMI_TRY(gj_invert(sst(m), P.invJ, P.F, P.n6, csize, m->use_gj_registers, m->solver->ctx->device, P.flags));
    }
    if (!P.wall) {  // the body coupling (swimmer.cpp:466-682); none on the wall
        filament_B_kernel<<<P.F, 128, (6 * (size_t)P.n6 + 36 * (size_t)P.NS + 36 + 27 + 36) * sizeof(double),
                            sst(m)>>>(P, nt);
        schur_filament_kernel<<<P.F, 32, 0, sst(m)>>>(P, m->spart);
        swimmer_schur_kernel<<<P.W, 64, 0, sst(m)>>>(P, nt, m->spart);
    }
    GMI_TRY(sim_launched(m, P.wall ? 3 : 6));
    GMI_TRY(read_flags(m));
    if (m->h_flags[2]) {
        set_last_error_msg("the approximate Jacobian is singular (matrix.cpp:549-554 stops the reference here)");
        return GMI_ERR_NONFINITE;
    }
    return GMI_OK;
}

static gmi_status jacobian_inv_mult(gmi_sim *m, const double *in, double *out)
{
    const SimP &P = m->P;
    if (P.wall) {
        jim_fil_kernel<<<P.F, 128, P.n6 * sizeof(double), sst(m)>>>(P, in, out);
        return sim_launched(m);
    }
    jim_partial_body_kernel<<<P.F, 128, 0, sst(m)>>>(P, in, m->jpart, out, m->tickets + 1);
    jim_fil_kernel<<<P.F, 128, P.n6 * sizeof(double), sst(m)>>>(P, in, out);
    return sim_launched(m, 2);
}

// dots[i] = v . D[:, i], i < k
static gmi_status dots_with_D(gmi_sim *m, const double *v, int k)
{
    if (k == 0) return GMI_OK;
    const int n = m->P.nbroy, nch = (n + kVecChunk - 1) / kVecChunk;
    coldot_kernel<<<dim3(nch, k), kVecTpb, 0, sst(m)>>>(m->D, (size_t)n, k, v, n, nch, m->part, m->dots,
                                                         m->tickets + 2);
    return sim_launched(m);
}

// The network's H0 on top of jacobian_inv_mult's result (learned steps only).
static gmi_status learned_apply(gmi_sim *m, const double *in, double *tmp)
{
    const SimP &P = m->P;
    const size_t smem = (size_t)P.n6 * sizeof(double);
    const int no = m->mlp->n_out;
    const double ic = 1.0 / P.conf;
    switch (m->rank) {
    case 2: learned_apply_kernel<2><<<P.F, 128, smem, sst(m)>>>(P, m->O, no, m->frames, in, tmp, ic); break;
    case 4: learned_apply_kernel<4><<<P.F, 128, smem, sst(m)>>>(P, m->O, no, m->frames, in, tmp, ic); break;
    default: learned_apply_kernel<8><<<P.F, 128, smem, sst(m)>>>(P, m->O, no, m->frames, in, tmp, ic); break;
    }
    return sim_launched(m);
}

// features and frames of this step's state (after the initial guess), and
// the network's output when the step is a learned one
static gmi_status learned_prepare(gmi_sim *m)
{
    const SimP &P = m->P;
    m->features_ready = false;
    if (!(m->learned_now || m->sec)) return GMI_OK;
    filament_features_kernel<<<gridN(P.F, 64), 64, 0, sst(m)>>>(P, m->frames, m->phi, m->phi16);
    GMI_TRY(sim_launched(m));
    if (m->learned_now) {
        GMI_TRY(mlp_forward_ws(m->mlp, sst(m), m->phi16, P.F, m->H1, m->H2, m->O));
        GMI_TRY(sim_launched(m, 3));
    }
    m->features_ready = true;
    return GMI_OK;
}

// one secant-pair record per filament for this iteration (plain steps only)
static gmi_status record_secant_pairs(gmi_sim *m)
{
    const SimP &P = m->P;
    if (!m->sec || !m->secant_pairs || m->learned_now || !m->features_ready || m->sec_count >= m->sec_cap)
        return GMI_OK;
    const int n = P.nbroy;
    vec_sub_kernel<<<gridN(n, 256), 256, 0, sst(m)>>>(n, m->nerr, m->err, m->dv);
    GMI_TRY(sim_launched(m));
    GMI_TRY(jacobian_inv_mult(m, m->dv, m->jv));
    secant_record_kernel<<<P.F, 64, 0, sst(m)>>>(P, m->frames, m->phi, m->dv, m->jv, m->upd, P.conf, m->sec,
                                                  m->sec_count, m->sec_cap);
    GMI_TRY(sim_launched(m));
    m->sec_count = std::min(m->sec_cap, m->sec_count + P.F);
    return GMI_OK;
}

// broyden_solver::find_update (broyden_solver.cpp:26-68)
static gmi_status find_update(gmi_sim *m)
{
    const int n = m->P.nbroy, it = m->broyden_iter;
    GMI_TRY(jacobian_inv_mult(m, m->err, m->tmp));
    if (m->learned_now) GMI_TRY(learned_apply(m, m->err, m->tmp));
    GMI_TRY(dots_with_D(m, m->err, it));
    broyden_combine_kernel<<<gridN(n, 256), 256, 0, sst(m)>>>(n, -m->P.conf, m->tmp, m->C, (size_t)n, m->dots, it,
                                                              m->upd);
    return sim_launched(m);
}

// broyden_solver::end_of_iter (broyden_solver.cpp:70-130)
static gmi_status end_of_iter(gmi_sim *m, bool too_large)
{
    const int n = m->P.nbroy, it = m->broyden_iter;
    GMI_TRY(record_secant_pairs(m));
    if (too_large && it < m->maxb - 1) {
        double *Ccol = m->C + (size_t)n * it, *Dcol = m->D + (size_t)n * it;
        GMI_TRY(jacobian_inv_mult(m, m->nerr, m->tmp));
        if (m->learned_now) GMI_TRY(learned_apply(m, m->nerr, m->tmp));
        GMI_TRY(dots_with_D(m, m->nerr, it));
        broyden_combine_kernel<<<gridN(n, 256), 256, 0, sst(m)>>>(n, -m->P.conf, m->tmp, m->C, (size_t)n, m->dots,
                                                                  it, Ccol);
        vec_sub_kernel<<<gridN(n, 256), 256, 0, sst(m)>>>(n, m->nerr, m->err, Dcol);
        GMI_TRY(sim_launched(m, 2));
        const int nch = (n + kVecChunk - 1) / kVecChunk;
        coldot_kernel<<<dim3(nch, 1), kVecTpb, 0, sst(m)>>>(Dcol, (size_t)n, 1, Dcol, n, nch, m->part, m->scal,
                                                            m->tickets + 2);
        vec_div2_kernel<<<gridN(n, 256), 256, 0, sst(m)>>>(n, Ccol, Dcol, m->scal);
        GMI_TRY(sim_launched(m, 2));
        std::swap(m->err, m->nerr);
    }
    m->broyden_iter++;
    return GMI_OK;
}

// swimmer::update (swimmer.cpp:847-871)
static gmi_status swimmer_update(gmi_sim *m)
{
    if (!m->P.wall) body_update_kernel<<<gridN(m->P.W, 32), 32, 0, sst(m)>>>(m->P, m->upd);
    filament_update_segments_kernel<<<gridN(m->P.S, 64), 64, 0, sst(m)>>>(m->P, m->upd);
    filament_robot_arm_kernel<<<gridN(3 * m->P.F, 64), 64, 0, sst(m)>>>(m->P);
    GMI_TRY(sim_launched(m));
    return sim_launched(m, m->P.wall ? 1 : 2);
}

}  // namespace gmi

using namespace gmi;

#define SIM_ARG_CHECK(cond, msg)     \
    do {                             \
        if (!(cond)) {               \
            set_last_error_msg(msg); \
            return GMI_ERR_ARG;      \
        }                            \
    } while (0)

namespace {

struct BackupHost {
    std::vector<double> q, x, xm1, xm2, u, um1, tl, tl1, tl2, cl, cl1, cl2, lam, lam1, lam2;
    std::vector<double> bq, bx, bxm1, bxm2, bu, bum1;
};

size_t per_fil_count(const SimP &P) { return 9 + 28 * (size_t)P.NS; }
size_t per_swimmer_count(const SimP &P) { return 19 + (size_t)P.NF * per_fil_count(P); }

// pairs (device array, host vector) of everything the backup holds
template <class F> gmi_status for_each_field(const SimP &P, BackupHost &h, F &&fn)
{
    const size_t S = P.S, F_ = P.F, W = P.W, nl = 3 * (size_t)(P.NS - 1) * F_;
    struct Field {
        double *d;
        std::vector<double> *h;
        size_t n;
    } f[] = {{P.q, &h.q, 4 * S},       {P.x, &h.x, 3 * S},       {P.xm1, &h.xm1, 3 * S},  {P.xm2, &h.xm2, 3 * S},
             {P.u, &h.u, 3 * S},       {P.um1, &h.um1, 3 * S},   {P.tl, &h.tl, 3 * F_},   {P.tl1, &h.tl1, 3 * F_},
             {P.tl2, &h.tl2, 3 * F_},  {P.cl, &h.cl, 3 * F_},    {P.cl1, &h.cl1, 3 * F_}, {P.cl2, &h.cl2, 3 * F_},
             {P.lam, &h.lam, nl},      {P.lam1, &h.lam1, nl},    {P.lam2, &h.lam2, nl},   {P.bq, &h.bq, 4 * W},
             {P.bx, &h.bx, 3 * W},     {P.bxm1, &h.bxm1, 3 * W}, {P.bxm2, &h.bxm2, 3 * W}, {P.bu, &h.bu, 3 * W},
             {P.bum1, &h.bum1, 3 * W}};
    for (auto &e : f) {
        gmi_status st = fn(e.d, *e.h, e.n);
        if (st != GMI_OK) return st;
    }
    return GMI_OK;
}

// Walk the backup order; op(value_in_backup, host_slot) for every entry.
template <class Op> void walk_backup(const SimP &P, BackupHost &h, Op &&op)
{
    const int NS = P.NS;
    for (int n = 0; n < P.W; ++n) {
        for (int i = 0; i < P.NF; ++i) {
            const int fil = n * P.NF + i;
            for (int k = 0; k < NS; ++k) {
                const size_t sg = (size_t)fil * NS + k;
                for (int c = 0; c < 4; ++c) op(h.q[4 * sg + c]);
                for (int c = 0; c < 3; ++c) op(h.x[3 * sg + c]);
                for (int c = 0; c < 3; ++c) op(h.xm1[3 * sg + c]);
                for (int c = 0; c < 3; ++c) op(h.xm2[3 * sg + c]);
                for (int c = 0; c < 3; ++c) op(h.u[3 * sg + c]);
                for (int c = 0; c < 3; ++c) op(h.um1[3 * sg + c]);
            }
            for (auto *v : {&h.tl, &h.tl1, &h.tl2, &h.cl, &h.cl1, &h.cl2})
                for (int c = 0; c < 3; ++c) op((*v)[3 * (size_t)fil + c]);
            const size_t l0 = 3 * (size_t)(NS - 1) * fil;
            for (int k = 0; k < NS - 1; ++k)
                for (auto *v : {&h.lam, &h.lam1, &h.lam2})
                    for (int c = 0; c < 3; ++c) op((*v)[l0 + 3 * k + c]);
        }
        for (int c = 0; c < 4; ++c) op(h.bq[4 * (size_t)n + c]);
        for (auto *v : {&h.bx, &h.bxm1, &h.bxm2, &h.bu, &h.bum1})
            for (int c = 0; c < 3; ++c) op((*v)[3 * (size_t)n + c]);
    }
}

}  // namespace

extern "C" {

gmi_status gmi_sim_destroy(gmi_sim *m)
{
    if (m == nullptr) return GMI_OK;
    if (m->solver) {
        cudaSetDevice(m->solver->ctx->device);
        cudaStreamSynchronize(m->solver->ctx->stream);
    }
    for (void *p : m->allocs) dev_free(p);
    if (m->h_flags) host_free(m->h_flags);
    if (m->solver) gmi_solver_destroy(m->solver);
    delete m;
    return GMI_OK;
}

gmi_status gmi_sim_create(const gmi_sim_config *cfg, const double *blob_refs, const double *fil_refs,
                          const double *body_x0, const double *perturb1, const double *perturb2, gmi_sim **out)
{
    SIM_ARG_CHECK(cfg && out && fil_refs, "gmi_sim_create: null argument");
    *out = nullptr;
    const gmi_solver_config &mc = cfg->mobility;
    const bool wall = mc.wall != 0;
    if (wall) {
        // filaments standing on the wall z = 0 (config.hpp:276-287): one
        // "swimmer", no blobs, the body fixed at the origin
        SIM_ARG_CHECK(mc.nswim == 1 && mc.nblob == 0 && mc.nfil >= 1 && mc.nseg >= 2,
                      "gmi_sim_create: the wall configuration has nswim = 1, nblob = 0");
    } else {
        SIM_ARG_CHECK(body_x0 != nullptr, "gmi_sim_create: null body positions");
        SIM_ARG_CHECK(mc.nfil >= 1 && mc.nseg >= 2 && mc.nblob >= 1 && mc.nswim >= 1, "gmi_sim_create: bad sizes");
        SIM_ARG_CHECK(blob_refs != nullptr, "gmi_sim_create: null blob references");
        SIM_ARG_CHECK(cfg->body_radius > 0, "gmi_sim_create: body_radius must be positive");
    }
    SIM_ARG_CHECK(cfg->dt > 0 && cfg->kb > 0 && cfg->kt > 0, "gmi_sim_create: dt, kb and kt must be positive");
    gmi_sim *m = new (std::nothrow) gmi_sim();
    if (m != nullptr) {
        const char *gj = std::getenv("GMI_GJ_CLUSTER");
        m->use_gj_cluster = !(gj && gj[0] == '0');
        const char *gr = std::getenv("GMI_GJ_REGISTERS");
        m->use_gj_registers = !(gr && gr[0] == '0');
        const char *gf = std::getenv("GMI_GJ_FP32");
        m->gj_fp32 = cfg->mobility.precision == GMI_FP32C && !(gf && gf[0] == '0');
    }
    SIM_ARG_CHECK(m != nullptr, "gmi_sim_create: out of host memory");
    m->cfg = *cfg;
    gmi_status st = gmi_solver_create(&mc, &m->solver);
    if (st != GMI_OK) {
        gmi_sim_destroy(m);
        return st;
    }
    gmi_solver *s = m->solver;
    m->maxb = cfg->max_broyden_iter > 0 ? cfg->max_broyden_iter : 100;
    SimP &P = m->P;
    P.W = mc.nswim;
    P.NF = mc.nfil;
    P.NS = mc.nseg;
    P.NB = mc.nblob;
    P.F = P.W * P.NF;
    P.S = P.F * P.NS;
    P.wall = wall ? 1 : 0;
    P.per_body = 6 * P.NF * P.NS + (wall ? 0 : 6);
    P.nbroy = P.W * P.per_body;
    P.n6 = 6 * P.NS;
    P.neuler = cfg->num_euler_steps > 0 ? cfg->num_euler_steps : 1;
    P.DL = 2.2 * mc.rseg;
    P.DT = cfg->dt;
    P.KB = cfg->kb;
    P.KT = cfg->kt;
    P.MU = mc.mu;
    P.RSEG = mc.rseg;
    P.EFM = mc.end_force_magnitude;
    P.TOL = cfg->tol > 0 ? cfg->tol : 1e-4;
    P.Rbody = cfg->body_radius;
    P.conf = cfg->jacobian_confidence > 0 ? cfg->jacobian_confidence : 0.1;
    P.x = s->x_segs;
    P.f = s->f_segs;
    P.v = s->v_segs;
    P.bx = s->body_x;
    P.bq = s->body_q;
    P.bf = s->body_f;
    P.vb = s->v_bodies;
    const size_t S = P.S, F = P.F, W = P.W, n6 = P.n6, nb = P.nbroy;
#define SIM_ALLOC(ptr, count)                  \
    do {                                       \
        st = sim_alloc(m, &(ptr), (count));    \
        if (st != GMI_OK) {                    \
            gmi_sim_destroy(m);                \
            return st;                         \
        }                                      \
    } while (0)
    SIM_ALLOC(P.q, 4 * S);
    SIM_ALLOC(P.qm1, 4 * S);
    SIM_ALLOC(P.u, 3 * S);
    SIM_ALLOC(P.um1, 3 * S);
    SIM_ALLOC(P.xm1, 3 * S);
    SIM_ALLOC(P.xm2, 3 * S);
    SIM_ALLOC(P.lam, 3 * (P.NS - 1) * F);
    SIM_ALLOC(P.lam1, 3 * (P.NS - 1) * F);
    SIM_ALLOC(P.lam2, 3 * (P.NS - 1) * F);
    SIM_ALLOC(P.tl, 3 * F);
    SIM_ALLOC(P.tl1, 3 * F);
    SIM_ALLOC(P.tl2, 3 * F);
    SIM_ALLOC(P.cl, 3 * F);
    SIM_ALLOC(P.cl1, 3 * F);
    SIM_ALLOC(P.cl2, 3 * F);
    SIM_ALLOC(P.p1, 3 * F);
    SIM_ALLOC(P.p2, 3 * F);
    SIM_ALLOC(P.st, 3 * F);
    SIM_ALLOC(P.fref, 3 * F);
    SIM_ALLOC(P.invJ, F * n6 * n6);
    SIM_ALLOC(P.ecb1, 9 * F);
    SIM_ALLOC(P.ecb2, 9 * F);
    SIM_ALLOC(P.jacB, F * 6 * n6);
    SIM_ALLOC(P.bxm1, 3 * W);
    SIM_ALLOC(P.bxm2, 3 * W);
    SIM_ALLOC(P.bu, 3 * W);
    SIM_ALLOC(P.bum1, 3 * W);
    SIM_ALLOC(P.bqm1, 4 * W);
    SIM_ALLOC(P.bQ, 9 * W);
    SIM_ALLOC(P.schur, 36 * W);
    SIM_ALLOC(P.mob_ref, 36);
    SIM_ALLOC(m->C, nb * m->maxb);
    SIM_ALLOC(m->D, nb * m->maxb);
    SIM_ALLOC(m->err, nb);
    SIM_ALLOC(m->nerr, nb);
    SIM_ALLOC(m->upd, nb);
    SIM_ALLOC(m->tmp, nb);
    SIM_ALLOC(m->dots, m->maxb + 1);
    SIM_ALLOC(m->part, (size_t)((nb + kVecChunk - 1) / kVecChunk) * (m->maxb + 1));
    SIM_ALLOC(m->jpart, 6 * F);
    SIM_ALLOC(m->spart, 45 * F);
    SIM_ALLOC(m->f_internal, 6 * S);
    SIM_ALLOC(P.lk, 9 * F * (size_t)(P.NS > 1 ? P.NS - 1 : 1));
    SIM_ALLOC(P.tang, 3 * (size_t)S);
    SIM_ALLOC(m->fs_part, 6 * W * (size_t)gridN(P.NF * P.NS, kFsSegs));
    SIM_ALLOC(m->scal, 4);
    {
        double *fl = nullptr;
        SIM_ALLOC(fl, 4);
        P.flags = reinterpret_cast<int *>(fl);
        double *tk = nullptr;
        SIM_ALLOC(tk, 4);  // zeroed arrival tickets of the one-launch reductions
        m->tickets = reinterpret_cast<int *>(tk);
    }
#undef SIM_ALLOC
    if (host_alloc(&m->h_flags, 4 * sizeof(int)) != cudaSuccess) {
        set_last_error_msg("gmi_sim_create: pinned allocation failed");
        gmi_sim_destroy(m);
        return GMI_ERR_CUDA;
    }
    // initial state: swimmer::initial_setup for spheres (swimmer.cpp:169-230),
    // rigid_body::initial_setup (rigid_body.cpp:184-213), filament::initial_setup
    // (filament.cpp:60-81, 265-323), built on the host then copied.
    const int NS = P.NS;
    std::vector<double> hx(3 * S), hq(4 * S), hbx(3 * W), hbq(4 * W, 0.0), hfref(3 * F), hp1(3 * F, 0.0),
        hp2(3 * F, 0.0);
    for (size_t n = 0; n < W; ++n) {
        for (int c = 0; c < 3; ++c) hbx[3 * n + c] = wall || !body_x0 ? 0.0 : body_x0[3 * n + c];
        hbq[4 * n] = 1.0;
    }
    for (size_t fil = 0; fil < F; ++fil) {
        const size_t n = fil / P.NF, i = fil % P.NF;
        const double *dref = fil_refs + 3 * i;
        for (int c = 0; c < 3; ++c) hfref[3 * fil + c] = dref[c];
        if (perturb1)
            for (int c = 0; c < 3; ++c) hp1[3 * fil + c] = perturb1[3 * fil + c];
        if (perturb2)
            for (int c = 0; c < 3; ++c) hp2[3 * fil + c] = perturb2[3 * fil + c];
        // radial on a sphere; along +z on the wall (swimmer.cpp:82)
        const double nrm = std::sqrt(dref[0] * dref[0] + dref[1] * dref[1] + dref[2] * dref[2]);
        const double dir[3] = {wall ? 0.0 : dref[0] / nrm, wall ? 0.0 : dref[1] / nrm, wall ? 1.0 : dref[2] / nrm};
        Q4 qt{dir[0], 0.0, -dir[2], dir[1]};
        qsqrt_in_place(qt);
        double pos[3] = {hbx[3 * n] + dref[0], hbx[3 * n + 1] + dref[1], hbx[3 * n + 2] + dref[2]};
        for (int k = 0; k < NS; ++k) {
            const size_t sidx = fil * NS + k;
            for (int c = 0; c < 3; ++c) hx[3 * sidx + c] = pos[c];
            hq[4 * sidx] = qt.s;
            hq[4 * sidx + 1] = qt.x;
            hq[4 * sidx + 2] = qt.y;
            hq[4 * sidx + 3] = qt.z;
            for (int c = 0; c < 3; ++c) pos[c] += P.DL * dir[c];
        }
    }
    auto up = [&](double *d, const std::vector<double> &h) -> gmi_status {
        GMI_CUDA_TRY(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, sst(m)));
        return GMI_OK;
    };
    if ((st = up(P.x, hx)) != GMI_OK || (st = up(P.xm1, hx)) != GMI_OK || (st = up(P.xm2, hx)) != GMI_OK ||
        (st = up(P.q, hq)) != GMI_OK || (st = up(P.qm1, hq)) != GMI_OK || (st = up(P.bx, hbx)) != GMI_OK ||
        (st = up(P.bxm1, hbx)) != GMI_OK || (st = up(P.bxm2, hbx)) != GMI_OK || (st = up(P.bq, hbq)) != GMI_OK ||
        (st = up(P.bqm1, hbq)) != GMI_OK || (st = up(P.fref, hfref)) != GMI_OK || (st = up(P.p1, hp1)) != GMI_OK ||
        (st = up(P.p2, hp2)) != GMI_OK) {
        gmi_sim_destroy(m);
        return st;
    }
    if (!wall) {
        st = gmi_solver_set_blob_references(s, blob_refs);
        if (st != GMI_OK) {
            gmi_sim_destroy(m);
            return st;
        }
    }
    if (cudaStreamSynchronize(sst(m)) != cudaSuccess) {
        set_last_error_msg("gmi_sim_create: the initial state did not reach the device");
        gmi_sim_destroy(m);
        return GMI_ERR_CUDA;
    }
    *out = m;
    return GMI_OK;
}

gmi_solver *gmi_sim_solver(gmi_sim *m) { return m ? m->solver : nullptr; }

// mobility_solver::make_body_reference_matrices on the initial state
// (cilia_sim_main.cpp:159-165)
gmi_status gmi_sim_prepare(gmi_sim *m, double *body_mobility_out)
{
    SIM_ARG_CHECK(m != nullptr, "gmi_sim_prepare: null simulation");
    GMI_CUDA_TRY(cudaSetDevice(m->solver->ctx->device));
    double mob[36] = {0};
    if (m->P.wall) {  // prescribed (zero) body velocity: no reference matrices
        if (body_mobility_out) std::memcpy(body_mobility_out, mob, sizeof mob);
        m->prepared = true;
        return GMI_OK;
    }
    GMI_TRY(solver_make_body_reference_matrices_device(m->solver, nullptr, mob));
    GMI_CUDA_TRY(cudaMemcpyAsync(m->P.mob_ref, mob, sizeof mob, cudaMemcpyHostToDevice, sst(m)));
    GMI_CUDA_TRY(cudaStreamSynchronize(sst(m)));
    if (body_mobility_out) std::memcpy(body_mobility_out, mob, sizeof mob);
    m->prepared = true;
    return GMI_OK;
}

}  // extern "C"

namespace gmi {

// The snapshot of the state a Broyden solve changes (snapshot_state),
// allocated on first use.
static gmi_status ensure_snapshot(gmi_sim *m)
{
    if (m->snap) return GMI_OK;
    const SimP &P = m->P;
    const size_t S = P.S, W = P.W, F = P.F;
    gmi_solver *s = m->solver;
    m->snap_fields = {{P.x, 3 * S},  {P.q, 4 * S},  {P.u, 3 * S},  {P.lam, 3 * (P.NS - 1) * F},
                      {P.tl, 3 * F}, {P.cl, 3 * F}, {P.bx, 3 * W}, {P.bu, 3 * W},
                      {P.bq, 4 * W}, {P.vb, 6 * W}};
    if (s->B > 0) m->snap_fields.push_back({s->f_blobs, 3 * (size_t)s->B});
    size_t total = 0;
    for (const auto &f : m->snap_fields) total += f.n;
    return sim_alloc(m, &m->snap, total);
}

// Copy the state a Broyden solve changes to the snapshot (restore = false)
// or back (restore = true): segment x, q, u, the filament multipliers, the
// body x, u, q and the linear solver's warm start.
static gmi_status snapshot_state(gmi_sim *m, bool restore)
{
    size_t off = 0;
    for (const auto &f : m->snap_fields) {
        double *a = m->snap + off;
        GMI_CUDA_TRY(cudaMemcpyAsync(restore ? f.p : a, restore ? a : f.p, f.n * sizeof(double),
                                     cudaMemcpyDeviceToDevice, sst(m)));
        off += f.n;
    }
    return GMI_OK;
}

// Jacobian probes (collection runs only): from the step's initial guess,
// m->probes times a random update v = -conf Jinv r (probe_direction_kernel)
// is applied, the error is evaluated there and one record per filament,
// [phi | d = e(x + v) - e(x) | conf Jinv d | v], is appended beside the
// secant pairs; the state is restored after each probe.  Unlike the secant
// pairs of plain Broyden runs, whose updates stay in the directions the
// damped plain start explores, the probes sample every direction of the
// plain start's range, the stiff ones included.
static gmi_status record_jacobian_probes(gmi_sim *m, int nt, int *gtot)
{
    const SimP &P = m->P;
    if (!m->sec || m->probes <= 0 || m->learned_now || !m->features_ready) return GMI_OK;
    const int n = P.nbroy;
    if (!m->probe_r) GMI_TRY(sim_alloc(m, &m->probe_r, n));
    GMI_TRY(ensure_snapshot(m));
    for (int p = 0; p < m->probes && m->sec_count < m->sec_cap; ++p) {
        const unsigned long long seed = m->probe_seed ^ (0x5851F42D4C957F2Dull * (++m->probe_serial));
        probe_direction_kernel<<<P.F, 128, 0, sst(m)>>>(P, m->err, seed, m->probe_r);
        GMI_TRY(sim_launched(m));
        GMI_TRY(jacobian_inv_mult(m, m->probe_r, m->tmp));
        vec_scale_kernel<<<gridN(n, 256), 256, 0, sst(m)>>>(n, -P.conf, m->tmp, m->upd);
        GMI_TRY(sim_launched(m));
        GMI_TRY(snapshot_state(m, false));
        GMI_TRY(swimmer_update(m));
        GMI_TRY(forces_and_torques(m, nt));
        bool too_large = false, nonfinite = false;
        int gi = 0;
        GMI_TRY(velocities_and_errors(m, nt, m->nerr, &too_large, &nonfinite, &gi));
        *gtot += gi;
        if (!nonfinite) {
            vec_sub_kernel<<<gridN(n, 256), 256, 0, sst(m)>>>(n, m->nerr, m->err, m->dv);
            GMI_TRY(sim_launched(m));
            GMI_TRY(jacobian_inv_mult(m, m->dv, m->jv));
            secant_record_kernel<<<P.F, 64, 0, sst(m)>>>(P, m->frames, m->phi, m->dv, m->jv, m->upd, P.conf, m->sec,
                                                          m->sec_count, m->sec_cap);
            GMI_TRY(sim_launched(m));
            m->sec_count = std::min(m->sec_cap, m->sec_count + P.F);
        }
        GMI_TRY(snapshot_state(m, true));
    }
    return GMI_OK;
}

// Broyden's method from the initial guess (cilia_sim_main.cpp:266-314), at
// most cap iterations.  *too_large: the error still above tolerance at the
// end; *diverged: a non-finite error.
static gmi_status broyden_solve(gmi_sim *m, int nt, int cap, int *iters, int *gtot, bool *too_large,
                                bool *diverged)
{
    int gi = 0;
    bool nonfinite = false;
    *too_large = false;
    *diverged = false;
    GMI_TRY(forces_and_torques(m, nt));
    GMI_TRY(velocities_and_errors(m, nt, m->err, too_large, &nonfinite, &gi));
    *gtot += gi;
    if (*too_large) {
        GMI_TRY(prepare_jacobian_inv(m, nt));
        GMI_TRY(learned_prepare(m));
        GMI_TRY(record_jacobian_probes(m, nt, gtot));
    }
    m->broyden_iter = 0;
    while (*too_large && m->broyden_iter < cap) {
        GMI_TRY(find_update(m));
        GMI_TRY(swimmer_update(m));
        GMI_TRY(forces_and_torques(m, nt));
        GMI_TRY(velocities_and_errors(m, nt, m->nerr, too_large, &nonfinite, &gi));
        *gtot += gi;
        if (nonfinite) {
            *diverged = true;
            break;
        }
        GMI_TRY(end_of_iter(m, *too_large));
    }
    *iters = m->broyden_iter;
    return GMI_OK;
}

}  // namespace gmi

extern "C" {

// One time step, cilia_sim_main.cpp:207-343 (GMRES branch).  With a learned
// initial inverse Jacobian the policy decides whether this step tries it; a
// learned attempt that misses the policy's iteration cap or diverges is
// restarted from the step's initial guess with the plain H0, so the step's
// outcome never depends on the network.  broyden_iters counts every
// iteration done, the abandoned attempt's included.
gmi_status gmi_sim_step(gmi_sim *m, int nt, int *broyden_iters, int *gmres_iters_total)
{
    SIM_ARG_CHECK(m != nullptr && nt >= 0, "gmi_sim_step: bad argument");
    SIM_ARG_CHECK(m->prepared, "gmi_sim_step: call gmi_sim_prepare first");
    GMI_CUDA_TRY(cudaSetDevice(m->solver->ctx->device));
    const SimP &P = m->P;
    if (!P.wall) body_initial_guess_kernel<<<gridN(P.W, 32), 32, 0, sst(m)>>>(P, nt);
    segment_initial_guess_kernel<<<gridN(P.S, 64), 64, 0, sst(m)>>>(P, nt);
    filament_initial_guess_kernel<<<gridN(P.F, 64), 64, 0, sst(m)>>>(P, nt);
    GMI_TRY(sim_launched(m, P.wall ? 2 : 3));
    if (m->beat) {
        beat_strain_kernel<<<gridN(P.F, 64), 64, 0, sst(m)>>>(P, m->beat_phase, m->beat_amplitude,
                                                              2.0 * kPi / m->beat_period, (nt + 1) * P.DT);
        GMI_TRY(sim_launched(m));
    }
    const bool policy_on = m->mlp != nullptr;
    m->learned_now = policy_on && gmi_learned_policy_use_learned(&m->policy);
    if (m->learned_now) GMI_TRY(snapshot_state(m, false));
    const int cap = m->learned_now ? gmi_learned_policy_iteration_cap(&m->policy, m->maxb) : m->maxb;
    int iters = 0, gtot = 0;
    bool too_large = false, diverged = false;
    gmi_status st = broyden_solve(m, nt, cap, &iters, &gtot, &too_large, &diverged);
    if (st == GMI_ERR_NONFINITE && m->learned_now) {
        // the learned H0 drove the state non-finite (a linear solve met a
        // non-finite right-hand side): a divergence like any other, the
        // step is restarted plain below
        diverged = true;
        iters = m->broyden_iter;
        st = GMI_OK;
    }
    int total = iters;
    if (st == GMI_OK && m->learned_now) {
        const bool ok = !too_large && !diverged;
        gmi_learned_policy_record(&m->policy, 1, ok ? 1 : 0, iters);
        if (!ok) {  // restart from the initial guess with the plain H0
            m->learned_now = false;
            st = snapshot_state(m, true);
            int it2 = 0;
            if (st == GMI_OK) st = broyden_solve(m, nt, m->maxb, &it2, &gtot, &too_large, &diverged);
            if (st == GMI_OK) gmi_learned_policy_record(&m->policy, 0, (!too_large && !diverged) ? 1 : 0, it2);
            total += it2;
        }
    } else if (st == GMI_OK && policy_on) {
        gmi_learned_policy_record(&m->policy, 0, (!too_large && !diverged) ? 1 : 0, iters);
    }
    m->learned_now = false;
    GMI_TRY(st);
    if (broyden_iters) *broyden_iters = total;
    if (gmres_iters_total) *gmres_iters_total = gtot;
    GMI_TRY(context_check_device_errors(m->solver->ctx));
    if (diverged) {
        set_last_error_msg("Broyden's method diverged (non-finite residual)");
        return GMI_ERR_NONFINITE;
    }
    if (too_large) {
        set_last_error_msg("Broyden's method did not converge within max_broyden_iter iterations");
        return GMI_ERR_NOT_CONVERGED;
    }
    return GMI_OK;
}

gmi_status gmi_sim_set_beat(gmi_sim *m, double amplitude, double period, const double *phases_h,
                            double end_force_scale)
{
    SIM_ARG_CHECK(m != nullptr && phases_h != nullptr && period > 0 && std::isfinite(amplitude) &&
                      end_force_scale >= 0,
                  "gmi_sim_set_beat: bad argument");
    GMI_CUDA_TRY(cudaSetDevice(m->solver->ctx->device));
    if (!m->beat_phase) GMI_TRY(sim_alloc(m, &m->beat_phase, m->P.F));
    GMI_CUDA_TRY(cudaMemcpyAsync(m->beat_phase, phases_h, (size_t)m->P.F * sizeof(double), cudaMemcpyHostToDevice,
                                 sst(m)));
    GMI_CUDA_TRY(cudaStreamSynchronize(sst(m)));
    m->beat_amplitude = amplitude;
    m->beat_period = period;
    m->beat = true;
    m->P.EFM = m->cfg.mobility.end_force_magnitude * end_force_scale;
    return GMI_OK;
}

gmi_status gmi_sim_set_secant_buffer(gmi_sim *m, float *records_d, long long capacity)
{
    SIM_ARG_CHECK(m != nullptr && capacity >= 0, "gmi_sim_set_secant_buffer: bad argument");
    GMI_CUDA_TRY(cudaSetDevice(m->solver->ctx->device));
    GMI_CUDA_TRY(cudaStreamSynchronize(sst(m)));
    m->sec_count = 0;
    if (records_d == nullptr || capacity == 0) {
        m->sec = nullptr;
        m->sec_cap = 0;
        return GMI_OK;
    }
    const SimP &P = m->P;
    const size_t F = P.F, n6 = P.n6;
    if (!m->dv) {
        GMI_TRY(sim_alloc(m, &m->dv, P.nbroy));
        GMI_TRY(sim_alloc(m, &m->jv, P.nbroy));
    }
    if (!m->frames) {
        GMI_TRY(sim_alloc(m, &m->frames, 9 * F));
        GMI_TRY(sim_alloc_bytes(m, (void **)&m->phi, F * n6 * sizeof(float)));
        GMI_TRY(sim_alloc_bytes(m, (void **)&m->phi16, F * n6 * sizeof(__nv_bfloat16)));
    }
    m->sec = records_d;
    m->sec_cap = capacity;
    return GMI_OK;
}

gmi_status gmi_sim_set_jacobian_probes(gmi_sim *m, int probes_per_step, unsigned long long seed, int secant_pairs)
{
    SIM_ARG_CHECK(m != nullptr && probes_per_step >= 0 && probes_per_step <= 64,
                  "gmi_sim_set_jacobian_probes: probes_per_step must be 0..64");
    m->probes = probes_per_step;
    m->probe_seed = seed;
    m->probe_serial = 0;
    m->secant_pairs = secant_pairs != 0;
    return GMI_OK;
}

gmi_status gmi_sim_secant_count(const gmi_sim *m, long long *count)
{
    SIM_ARG_CHECK(m != nullptr && count != nullptr, "gmi_sim_secant_count: null argument");
    *count = m->sec_count;
    return GMI_OK;
}

gmi_status gmi_sim_set_learned_jacobian(gmi_sim *m, const gmi_mlp *mlp, int rank, const gmi_learned_policy *policy)
{
    SIM_ARG_CHECK(m != nullptr, "gmi_sim_set_learned_jacobian: null simulation");
    GMI_CUDA_TRY(cudaSetDevice(m->solver->ctx->device));
    GMI_CUDA_TRY(cudaStreamSynchronize(sst(m)));
    if (mlp == nullptr) {
        m->mlp = nullptr;
        return GMI_OK;
    }
    const SimP &P = m->P;
    SIM_ARG_CHECK(rank == 2 || rank == 4 || rank == 8, "gmi_sim_set_learned_jacobian: rank must be 2, 4 or 8");
    SIM_ARG_CHECK(mlp->n_in == P.n6 && 2 * P.NS + 2 * P.n6 * rank <= mlp->n_out,
                  "gmi_sim_set_learned_jacobian: the network's widths do not fit 6 nseg inputs and this rank");
    SIM_ARG_CHECK(mlp->device == m->solver->ctx->device,
                  "gmi_sim_set_learned_jacobian: the network lives on another device");
    const size_t F = P.F, n6 = P.n6;
    if (!m->frames) {
        GMI_TRY(sim_alloc(m, &m->frames, 9 * F));
        GMI_TRY(sim_alloc_bytes(m, (void **)&m->phi, F * n6 * sizeof(float)));
        GMI_TRY(sim_alloc_bytes(m, (void **)&m->phi16, F * n6 * sizeof(__nv_bfloat16)));
    }
    if (!m->mlp || m->mlp->n_hidden != mlp->n_hidden || m->mlp->n_out != mlp->n_out || !m->O) {
        GMI_TRY(sim_alloc_bytes(m, (void **)&m->H1, F * mlp->n_hidden * sizeof(__nv_bfloat16)));
        GMI_TRY(sim_alloc_bytes(m, (void **)&m->H2, F * mlp->n_hidden * sizeof(__nv_bfloat16)));
        GMI_TRY(sim_alloc_bytes(m, (void **)&m->O, F * mlp->n_out * sizeof(float)));
    }
    GMI_TRY(ensure_snapshot(m));
    m->mlp = mlp;
    m->rank = rank;
    if (policy)
        m->policy = *policy;
    else
        gmi_learned_policy_init(&m->policy);
    return GMI_OK;
}

gmi_status gmi_sim_learned_policy(const gmi_sim *m, gmi_learned_policy *out)
{
    SIM_ARG_CHECK(m != nullptr && out != nullptr, "gmi_sim_learned_policy: null argument");
    *out = m->policy;
    return GMI_OK;
}

gmi_status gmi_sim_get_state(gmi_sim *m, int field, double *out_h)
{
    SIM_ARG_CHECK(m && out_h, "gmi_sim_get_state: null argument");
    const SimP &P = m->P;
    const double *src = nullptr;
    size_t count = 0;
    switch (field) {
        case GMI_STATE_SEG_X: src = P.x; count = 3 * (size_t)P.S; break;
        case GMI_STATE_SEG_Q: src = P.q; count = 4 * (size_t)P.S; break;
        case GMI_STATE_SEG_U: src = P.u; count = 3 * (size_t)P.S; break;
        case GMI_STATE_SEG_V: src = P.v; count = 6 * (size_t)P.S; break;
        case GMI_STATE_SEG_F: src = P.f; count = 6 * (size_t)P.S; break;
        case GMI_STATE_BODY_X: src = P.bx; count = 3 * (size_t)P.W; break;
        case GMI_STATE_BODY_Q: src = P.bq; count = 4 * (size_t)P.W; break;
        case GMI_STATE_BODY_U: src = P.bu; count = 3 * (size_t)P.W; break;
        case GMI_STATE_BODY_V: src = P.vb; count = 6 * (size_t)P.W; break;
        case GMI_STATE_LAMBDA: src = P.lam; count = 3 * (size_t)(P.NS - 1) * P.F; break;
        case GMI_STATE_TETHER: src = P.tl; count = 3 * (size_t)P.F; break;
        case GMI_STATE_CLAMP: src = P.cl; count = 3 * (size_t)P.F; break;
        case GMI_STATE_BLOB_F: src = m->solver->f_blobs; count = 3 * (size_t)m->solver->B; break;
        case GMI_STATE_SEG_F_INTERNAL: src = m->f_internal; count = 6 * (size_t)P.S; break;
        default: SIM_ARG_CHECK(false, "gmi_sim_get_state: unknown field");
    }
    GMI_CUDA_TRY(cudaSetDevice(m->solver->ctx->device));
    GMI_CUDA_TRY(cudaMemcpyAsync(out_h, src, count * sizeof(double), cudaMemcpyDeviceToHost, sst(m)));
    GMI_CUDA_TRY(cudaStreamSynchronize(sst(m)));
    return GMI_OK;
}


// ---------------------------------------------------------------------------
// Checkpoints in the reference's .backup layout (cilia_sim_main.cpp:370-381):
// per swimmer, each filament (filament.cpp:1595-1650: per segment q, x, xm1,
// xm2, u, um1; tether and clamp multipliers with their two previous values;
// the inextensibility multipliers with theirs), then the body
// (rigid_body.cpp:408-432: q, x, xm1, xm2, u, um1).
// ---------------------------------------------------------------------------

gmi_status gmi_sim_backup_count(const gmi_sim *m, long long *count)
{
    SIM_ARG_CHECK(m && count, "gmi_sim_backup_count: null argument");
    *count = (long long)m->P.W * (long long)per_swimmer_count(m->P);
    return GMI_OK;
}

gmi_status gmi_sim_export_backup(gmi_sim *m, double *out_h)
{
    SIM_ARG_CHECK(m && out_h, "gmi_sim_export_backup: null argument");
    GMI_CUDA_TRY(cudaSetDevice(m->solver->ctx->device));
    GMI_CUDA_TRY(cudaStreamSynchronize(sst(m)));
    BackupHost h;
    cudaStream_t st = sst(m);
    GMI_TRY(for_each_field(m->P, h, [st](double *d, std::vector<double> &v, size_t n) -> gmi_status {
        v.resize(n);
        GMI_CUDA_TRY(cudaMemcpyAsync(v.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        return GMI_OK;
    }));
    GMI_CUDA_TRY(cudaStreamSynchronize(st));
    size_t p = 0;
    walk_backup(m->P, h, [&](double &v) { out_h[p++] = v; });
    return GMI_OK;
}

gmi_status gmi_sim_import_backup(gmi_sim *m, const double *in_h)
{
    SIM_ARG_CHECK(m && in_h, "gmi_sim_import_backup: null argument");
    GMI_CUDA_TRY(cudaSetDevice(m->solver->ctx->device));
    GMI_CUDA_TRY(cudaStreamSynchronize(sst(m)));
    BackupHost h;
    GMI_TRY(for_each_field(m->P, h, [](double *, std::vector<double> &v, size_t n) -> gmi_status {
        v.assign(n, 0.0);
        return GMI_OK;
    }));
    size_t p = 0;
    walk_backup(m->P, h, [&](double &v) { v = in_h[p++]; });
    cudaStream_t st = sst(m);
    GMI_TRY(for_each_field(m->P, h, [st](double *d, std::vector<double> &v, size_t n) -> gmi_status {
        GMI_CUDA_TRY(cudaMemcpyAsync(d, v.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
        return GMI_OK;
    }));
    // q^{n-1} = q for segments and bodies (filament.cpp initial_setup and
    // rigid_body.cpp:71-100 read the backup this way); a fresh linear solver
    // starts from zero blob forces and body velocities
    GMI_CUDA_TRY(cudaMemcpyAsync(m->P.qm1, m->P.q, 4 * (size_t)m->P.S * sizeof(double), cudaMemcpyDeviceToDevice, st));
    GMI_CUDA_TRY(cudaMemcpyAsync(m->P.bqm1, m->P.bq, 4 * (size_t)m->P.W * sizeof(double), cudaMemcpyDeviceToDevice,
                                 st));
    GMI_CUDA_TRY(cudaMemsetAsync(m->solver->f_blobs, 0, 3 * (size_t)m->solver->B * sizeof(double), st));
    GMI_CUDA_TRY(cudaMemsetAsync(m->solver->v_bodies, 0, 6 * (size_t)m->P.W * sizeof(double), st));
    GMI_CUDA_TRY(cudaStreamSynchronize(st));
    m->prepared = false;  // the body reference matrices follow the restored state
    return GMI_OK;
}

}  // extern "C"
