// gmi_solver.cu -- device-resident mobility solver: the reference's
// rpy_mobility_solver state and the generic mobility_solver methods
// (read_positions_and_forces, assemble_rhs, apply_preconditioner,
// system_matrix_mult, solve_linear_system, compute_velocities,
// make_body_reference_matrices) with every vector operation on the GPU.
//
// Layout in HBM (FP64, the reference's host layouts so host<->device copies
// are single memcpys):
//   x_segs[3S] f_segs[6S] v_segs[6S]   x_blobs[3B] f_blobs[3B] v_blobs[3B] f_rep[3B]
//   bodies: x[3W] q[4W] (scalar first) f[6W] v[6W], R[9W] row-major,
//           rotated reference matrices ktk_rot[36W], mob_rot[36W] (column-major 6x6)
//   GMRES system of size n = 3B + 6W, blobs first (swimmer-major), then bodies;
//   Krylov basis Q[n x (m+1)] column-major, Hessenberg H[(m+1) x (m+1)] column-major.
// S = nswim*nfil*nseg segments, B = nswim*nblob blobs, W = nswim.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "gmi_context.hpp"
#include "gmi_pair_kernels.hpp"
#include "gmi_solver_device.cuh"
#include "gmi_solver_internal.hpp"
#include "gmi_gmres_cluster.hpp"

namespace gmi {

constexpr int kRedTpb = 256;      // threads of the reduction kernels
constexpr int kChunkRows = 1024;  // rows per block in dot-product partials

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
// Block-wide sum in a fixed order (result valid in thread 0).
template <int TPB> __device__ __forceinline__ double block_sum(double v, double *smem)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = threadIdx.x < TPB / 32 ? smem[threadIdx.x] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

// Rotation matrix of a unit quaternion (s, v0, v1, v2), row-major, with the
// reference's order of operations (quaternion.cpp:260-298).
__device__ __forceinline__ void quat_rot(const double *q, double *R)
{
    const double s = q[0], a = q[1], b = q[2], c = q[3];
    double R00 = 1.0, R11 = 1.0, R22 = 1.0;
    double t = 2.0 * a * a;
    R11 -= t; R22 -= t;
    t = 2.0 * b * b;
    R00 -= t; R22 -= t;
    t = 2.0 * c * c;
    R00 -= t; R11 -= t;
    t = 2.0 * a * b;
    double R10 = t, R01 = t;
    t = 2.0 * a * c;
    double R20 = t, R02 = t;
    t = 2.0 * b * c;
    double R12 = t, R21 = t;
    t = 2.0 * s * c;
    R10 += t; R01 -= t;
    t = 2.0 * s * b;
    R20 -= t; R02 += t;
    t = 2.0 * s * a;
    R21 += t; R12 -= t;
    R[0] = R00; R[1] = R01; R[2] = R02;
    R[3] = R10; R[4] = R11; R[5] = R12;
    R[6] = R20; R[7] = R21; R[8] = R22;
}

// ---------------------------------------------------------------------------
// body kernels
// ---------------------------------------------------------------------------
// R per swimmer and the 6x6 reference matrices rotated block by block,
// Q * block * Q^T (mobility_solver.cpp:660-677): (K^T K)^-1 and the body
// mobility as the reference has them, and K^T K itself (for the Arnoldi
// step's K^T z).  One thread per (swimmer, matrix, entry): each forms R
// itself and its entry's row of R * block, then the entry, with the
// operations of the whole-block product (a warp FP64 instruction costs the
// same on one lane as on 32, so the 108 entries of a swimmer take about as
// long as one).
__global__ void prepare_bodies_kernel(int W, const double *__restrict__ q, const double *__restrict__ ktk_ref,
                                      const double *__restrict__ mob_ref, const double *__restrict__ ktkf_ref,
                                      double *__restrict__ R, double *__restrict__ ktk_rot,
                                      double *__restrict__ mob_rot, double *__restrict__ ktkf_rot)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 108 * W) return;
    const int n = e / 108, m = (e % 108) / 36, rc = e % 36, r = rc % 6, c = rc / 6;
    double Rn[9];
    quat_rot(q + 4 * n, Rn);
    if (m == 0 && rc < 9) R[9 * n + rc] = Rn[rc];
    const double *src = m == 0 ? ktk_ref : (m == 1 ? mob_ref : ktkf_ref);
    double *dst = m == 0 ? ktk_rot : (m == 1 ? mob_rot : ktkf_rot);
    const double *A = src + 3 * (r / 3) + 6 * (3 * (c / 3));  // the block, column-major
    const int i = r % 3, j = c % 3;
    double T[3];  // row i of R A
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
        T[jj] = Rn[3 * i] * A[6 * jj] + Rn[3 * i + 1] * A[1 + 6 * jj] + Rn[3 * i + 2] * A[2 + 6 * jj];
    dst[36 * n + rc] = T[0] * Rn[3 * j] + T[1] * Rn[3 * j + 1] + T[2] * Rn[3 * j + 2];
}

// x_blob = X + R ref (rigid_body.cpp:334-352).
__global__ void blob_positions_kernel(int W, int nblob, const double *__restrict__ bx, const double *__restrict__ R,
                                      const double *__restrict__ refs, double *__restrict__ xb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * nblob) return;
    const int n = i / nblob, m = i % nblob;
    double d[3];
    rot_apply(R + 9 * n, refs + 3 * m, d);
    xb[3 * i] = bx[3 * n] + d[0];
    xb[3 * i + 1] = bx[3 * n + 1] + d[1];
    xb[3 * i + 2] = bx[3 * n + 2] + d[2];
}

// Per swimmer: sums[6n..] = (sum_m f_m, sum_m (R ref_m) x f_m) over its blobs.
// This is K^T f (mobility_solver.cpp:690-697, 921-940, 168-188), in two
// passes of kt_kernel: kKtBlobs blobs per CTA into part[(n gx + x) 6 + c],
// then the CTA partials added per (swimmer, component) in a fixed order.
constexpr int kKtBlobs = 128;

// Block sum of six per-thread values, in a fixed order: threads 0..5 write
// the totals to out[0..6).
template <int TPB> __device__ __forceinline__ void block_sum6(const double *v, double *out)
{
    __shared__ double red[TPB / 32][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const double t = warp_sum6_scatter(v);
    if ((lane & 3) == 0 && lane < 24) red[wid][lane >> 2] = t;
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < TPB / 32; ++w) s += red[w][threadIdx.x];
        out[threadIdx.x] = s;
    }
}

// body_f += sums (the blob repulsion's force and torque on each body).
__global__ void add_vec_kernel(int count, const double *__restrict__ a, double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) y[i] += a[i];
}

// rhs = [-v_blobs ; -body_f] (mobility_solver.cpp:363-419).
__global__ void assemble_rhs_kernel(int nb3, int nw6, const double *__restrict__ vb, const double *__restrict__ bf,
                                    double *__restrict__ rhs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nb3) rhs[i] = -vb[i];
    else if (i < nb3 + nw6) rhs[i] = -bf[i - nb3];
}

// Preconditioner, body part (mobility_solver.cpp:653-697):
// out_body = KTKinv_rot * b - mob_rot * in_body with b = -K^T in_blob.
__global__ void precond_body_kernel(int W, const double *__restrict__ sums, const double *__restrict__ in_body,
                                    const double *__restrict__ ktk_rot, const double *__restrict__ mob_rot,
                                    double *__restrict__ out_body)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= W) return;
    double b[6], u[6];
    for (int c = 0; c < 6; ++c) {
        b[c] = -sums[6 * n + c];
        u[c] = in_body[6 * n + c];
    }
    const double *Kt = ktk_rot + 36 * n, *Mb = mob_rot + 36 * n;
    for (int i = 0; i < 6; ++i) {
        double x = 0.0, y = 0.0;
        for (int j = 0; j < 6; ++j) {
            x += Kt[i + 6 * j] * b[j];
            y += Mb[i + 6 * j] * u[j];
        }
        out_body[6 * n + i] = x - y;
    }
}

// Preconditioner, blob part (mobility_solver.cpp:699-719):
// out_blob = Minv * (in_blob + U + Omega x (R ref)).  The reference scales
// the whole blob block by Minv inside its loop over swimmers
// (mobility_solver.cpp:718), so the blobs of swimmer n end up multiplied
// by Minv (W - n) times; this kernel reproduces that.
__global__ void precond_blob_kernel(int W, int nblob, const double *__restrict__ in_blob,
                                    const double *__restrict__ out_body, const double *__restrict__ R,
                                    const double *__restrict__ refs, double minv, double *__restrict__ out_blob)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * nblob) return;
    const int n = i / nblob, m = i % nblob;
    double d[3];
    rot_apply(R + 9 * n, refs + 3 * m, d);
    const double *U = out_body + 6 * n;
    double o0 = in_blob[3 * i] + U[0], o1 = in_blob[3 * i + 1] + U[1], o2 = in_blob[3 * i + 2] + U[2];
    o0 += U[4] * d[2] - U[5] * d[1];
    o1 += U[5] * d[0] - U[3] * d[2];
    o2 += U[3] * d[1] - U[4] * d[0];
    for (int k = n; k < W; ++k) {
        o0 *= minv;
        o1 *= minv;
        o2 *= minv;
    }
    out_blob[3 * i] = o0;
    out_blob[3 * i + 1] = o1;
    out_blob[3 * i + 2] = o2;
}

// System matrix, after the blob-blob apply (mobility_solver.cpp:905-960):
// out_blob = -(U + Omega x (R ref)) + (M_bb in_blob), out_body = -K^T in_blob.
__global__ void sysmult_finish_kernel(int W, int nblob, const double *__restrict__ mbb, const double *__restrict__ in_body,
                                      const double *__restrict__ sums, const double *__restrict__ R,
                                      const double *__restrict__ refs, double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nb = W * nblob;
    if (i < nb) {
        const int n = i / nblob, m = i % nblob;
        double d[3];
        rot_apply(R + 9 * n, refs + 3 * m, d);
        const double *U = in_body + 6 * n;
        out[3 * i] = -(U[0] - d[1] * U[5] + d[2] * U[4]) + mbb[3 * i];
        out[3 * i + 1] = -(U[1] - d[2] * U[3] + d[0] * U[5]) + mbb[3 * i + 1];
        out[3 * i + 2] = -(U[2] - d[0] * U[4] + d[1] * U[3]) + mbb[3 * i + 2];
    } else if (i < nb + 6 * W) {
        out[3 * nb + (i - nb)] = -sums[i - nb];
    }
}

// ---------------------------------------------------------------------------
// Krylov kernels
// ---------------------------------------------------------------------------
// partial[i * nchunks + c] = sum over rows of chunk c of Q[:, i] . w
__global__ void __launch_bounds__(kRedTpb) dot_partials_kernel(const double *__restrict__ Q, size_t ld,
                                                               const double *__restrict__ w, int n, int nchunks,
                                                               double *__restrict__ partial)
{
    __shared__ double red[32];
    const int c = blockIdx.x, i = blockIdx.y;
    const double *q = Q + ld * i;
    double a = 0.0;
    const int r0 = c * kChunkRows, r1 = min(n, r0 + kChunkRows);
    for (int r = r0 + threadIdx.x; r < r1; r += kRedTpb) a += q[r] * w[r];
    const double s = block_sum<kRedTpb>(a, red);
    if (threadIdx.x == 0) partial[(size_t)i * nchunks + c] = s;
}

// Classical Gram-Schmidt update: h_i = sum_c partial[i][c]; w -= sum_i h_i Q[:, i];
// block 0 adds h into the Hessenberg column (pass 0 stores, pass 1 adds).
__global__ void __launch_bounds__(kRedTpb) cgs_update_kernel(const double *__restrict__ Q, size_t ld, int k,
                                                             const double *__restrict__ partial, int nchunks,
                                                             double *__restrict__ w, int n, double *__restrict__ Hcol,
                                                             int pass)
{
    extern __shared__ double h[];
    for (int i = threadIdx.x; i < k; i += kRedTpb) {
        double s = 0.0;
        for (int c = 0; c < nchunks; ++c) s += partial[(size_t)i * nchunks + c];
        h[i] = s;
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int i = threadIdx.x; i < k; i += kRedTpb) Hcol[i] = pass == 0 ? h[i] : Hcol[i] + h[i];
    const int r = blockIdx.x * kRedTpb + threadIdx.x;
    if (r >= n) return;
    double acc = w[r];
    for (int i = 0; i < k; ++i) acc -= h[i] * Q[ld * i + r];
    w[r] = acc;
}

// q_out = w / ||w|| with ||w|| from the partials; block 0 stores the norm at *hval.
__global__ void normalize_kernel(const double *__restrict__ w, int n, const double *__restrict__ partial, int nchunks,
                                 double *__restrict__ q_out, double *__restrict__ hval)
{
    __shared__ double nrm;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int c = 0; c < nchunks; ++c) s += partial[c];
        nrm = sqrt(s);
        if (blockIdx.x == 0 && hval) *hval = nrm;
    }
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) q_out[r] = nrm > 0.0 ? w[r] / nrm : 0.0;
}

// One Givens step of solve_linear_system (mobility_solver.cpp:1189-1231) on
// column iter-1; writes |beta(iter)| / norm_rhs to *resid.
__global__ void givens_kernel(double *__restrict__ H, int ldh, double *__restrict__ beta, double *__restrict__ cs,
                              double *__restrict__ sn, int iter, double norm_rhs, double *__restrict__ resid)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double *col = H + (size_t)ldh * (iter - 1);
    for (int i = 1; i < iter; ++i) {
        const double t = cs[i - 1] * col[i - 1] + sn[i - 1] * col[i];
        col[i] = cs[i - 1] * col[i] - sn[i - 1] * col[i - 1];
        col[i - 1] = t;
    }
    const double hk = col[iter], hd = col[iter - 1];
    double c, s;
    if (hk == 0.0) {
        c = 1.0;
        s = 0.0;
    } else if (fabs(hk) > fabs(hd)) {
        const double t = hd / hk;
        s = (2.0 * (double)(hk > 0) - 1.0) / sqrt(1.0 + t * t);
        c = t * s;
    } else {
        const double t = hk / hd;
        c = (2.0 * (double)(hd > 0) - 1.0) / sqrt(1.0 + t * t);
        s = t * c;
    }
    cs[iter - 1] = c;
    sn[iter - 1] = s;
    col[iter - 1] = c * hd + s * hk;
    col[iter] = 0.0;
    beta[iter] = -s * beta[iter - 1];
    beta[iter - 1] = c * beta[iter - 1];
    *resid = fabs(beta[iter]) / norm_rhs;
}

// out = sum_i y_i Q[:, i], in the reference's column order (mobility_solver.cpp:1252-1255).
// (with ctl, k is the solve's iteration count on the device, ctl->k)
__global__ void combine_kernel(const double *__restrict__ Q, size_t ld, const double *__restrict__ y, int k, int n,
                               double *__restrict__ out, const GmresCtl *ctl)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    if (ctl != nullptr) k = ctl->k;
    double acc = 0.0;
    for (int i = 0; i < k; ++i) acc += y[i] * Q[ld * i + r];
    out[r] = acc;
}

__global__ void axpby_kernel(int n, double a, const double *__restrict__ x, double b, const double *__restrict__ y,
                             double *__restrict__ out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) out[r] = a * x[r] + b * y[r];
}

__global__ void scale_kernel(int n, const double *__restrict__ x, const double *__restrict__ s, double *__restrict__ out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) out[r] = x[r] / s[0];
}


// ---------------------------------------------------------------------------
// Device-controlled Arnoldi step (apply_preconditioner, system_matrix_mult,
// CGS2 orthogonalisation, Givens: mobility_solver.cpp:1162-1230).  The
// iteration count and the convergence flag live in a GmresCtl block on the
// device, so a step needs no host round trip and is replayed from a CUDA
// graph; once converged, every kernel of a replayed step returns at once.
//
// FP64 throughput per SM is low on this GPU, so every kernel spreads its
// rows over many CTAs and avoids FP64 shuffle trees.  Sums across CTAs (body
// moments, CGS projections, the norm) are finished by the last CTA to arrive
// (an atomic ticket; nobody waits), in a fixed order, so results are
// deterministic.  Projections use two levels: the last CTA of each group of
// kSGroup CTAs sums the group, the last group finisher sums the groups.
//   S1 (CTA per 32 blobs)   w -= Q h2 (the previous S4's second pass);
//                            q_{k-1} = w / ||w|| into Q; body moments;
//                            last CTA: body rows of q and z_body = U
//                            w_body = -K^T z of the coming z (linearity)
//   S2 (CTA per 64 blobs)   z_blob; records of z
//   pair kernel on the records -> mbb, or per-split partials
//   S3 (CTA per kSRows rows) w_blob = M_bb z - K z_body (adding the split
//                            partials); h1 = Q^T w; last: H col = h1
//   S4 (CTA per kSRows rows) w -= Q h1; h2 = Q^T w and ||w||^2; last: H col
//                            += h2, ||w - Q h2|| by Pythagoras, Givens, ctl
// ---------------------------------------------------------------------------
constexpr int kSBlobs = 64;   // blobs (threads) per CTA in S2
constexpr int kSRows = 32;    // rows per CTA in S3, S4
constexpr int kSTpb = 128;    // threads per CTA in S3, S4
constexpr int kSGroup = 16;   // CTAs per first-level group of the projection sums
constexpr int kFMaxK = 160;   // >= max_iter + 1
// layout of the step's scalar workspace (doubles)
constexpr int kHOff = 0;             // h[kFMaxK]: the last projections
constexpr int kNormOff = kFMaxK;     // ||w|| of the last step (or beta0 before the first)
constexpr int kStepScalars = kFMaxK + 8;

// ||x|| into *out in one launch: CTA c sums the squares of rows
// [c kChunkRows, (c + 1) kChunkRows) into partial[c] (as dot_partials_kernel
// would), and the last CTA to arrive adds the partials in chunk order.
__global__ void __launch_bounds__(kRedTpb) norm_kernel(const double *__restrict__ x, int n,
                                                       double *__restrict__ partial, double *__restrict__ out,
                                                       int *ticket)
{
    __shared__ double red[32];
    const int c = blockIdx.x;
    double a = 0.0;
    const int r0 = c * kChunkRows, r1 = min(n, r0 + kChunkRows);
    for (int r = r0 + threadIdx.x; r < r1; r += kRedTpb) a += x[r] * x[r];
    const double sum = block_sum<kRedTpb>(a, red);
    if (threadIdx.x == 0) partial[c] = sum;
    if (!last_cta(ticket, gridDim.x)) return;
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) t += __ldcg(partial + b);
        *out = sqrt(t);
    }
}

// K^T f per swimmer in one launch: each CTA's partial over its kKtBlobs
// blobs; then, in the last CTA to arrive, the partials added per swimmer
// (one warp per swimmer, lanes over the partials, a six-value warp sum).
__global__ void __launch_bounds__(kKtBlobs) kt_kernel(int W, int nblob, const double *__restrict__ R,
                                                      const double *__restrict__ refs,
                                                      const double *__restrict__ f, double *__restrict__ part,
                                                      double *__restrict__ sums, int *ticket)
{
    const int n = blockIdx.y, m = blockIdx.x * kKtBlobs + threadIdx.x, gx = gridDim.x;
    double a[6] = {0, 0, 0, 0, 0, 0};
    if (m < nblob) {
        const double *fm = f + 3 * ((size_t)n * nblob + m);
        double d[3];
        rot_apply(R + 9 * n, refs + 3 * m, d);
        a[0] = fm[0];
        a[1] = fm[1];
        a[2] = fm[2];
        a[3] = d[1] * fm[2] - d[2] * fm[1];
        a[4] = d[2] * fm[0] - d[0] * fm[2];
        a[5] = d[0] * fm[1] - d[1] * fm[0];
    }
    block_sum6<kKtBlobs>(a, part + ((size_t)n * gx + blockIdx.x) * 6);
    if (!last_cta(ticket, gx * gridDim.y)) return;
    const int lane = threadIdx.x & 31;
    for (int sw = threadIdx.x >> 5; sw < W; sw += kKtBlobs / 32) {
        double b[6] = {0, 0, 0, 0, 0, 0};
        for (int x = lane; x < gx; x += 32)
#pragma unroll
            for (int c = 0; c < 6; ++c) b[c] += __ldcg(part + ((size_t)sw * gx + x) * 6 + c);
        const double t = warp_sum6_scatter(b);
        if ((lane & 3) == 0 && lane < 24) sums[6 * sw + (lane >> 2)] = t;
    }
}

// Sum over the gx per-CTA 6-vectors of each swimmer (part[(n*gx + x)*6 + c])
// into sh[6n + c], in a fixed order, by whichever of two layouts issues
// fewer FP64 warp instructions: few swimmers take one warp each (the lanes
// stride over the partials, then a six-value warp sum); many swimmers take
// one thread per (swimmer, component), after a coalesced copy of the
// partials into shared memory (stage, kStageMax doubles) when they fit.
constexpr int kStageMax = 4096;
__device__ __forceinline__ void swimmer_sums(const double *part, int W, int gx, double *sh)
{
    __shared__ double stage[kStageMax];
    const int nw = blockDim.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = (W + nw - 1) / nw * (6 * ((gx + 31) / 32) + 9);
    const int per_thread = (6 * W + blockDim.x - 1) / blockDim.x * gx;
    if (per_warp < per_thread) {
        for (int n = threadIdx.x >> 5; n < W; n += nw) {
            double a[6] = {0, 0, 0, 0, 0, 0};
            for (int x = lane; x < gx; x += 32)
#pragma unroll
                for (int c = 0; c < 6; ++c) a[c] += __ldcg(part + ((size_t)n * gx + x) * 6 + c);
            const double t = warp_sum6_scatter(a);
            if ((lane & 3) == 0 && lane < 24) sh[6 * n + (lane >> 2)] = t;
        }
        __syncthreads();
        return;
    }
    const int total = 6 * W * gx;
    const bool staged = total <= kStageMax;
    if (staged)
        for (int e = threadIdx.x; e < total; e += blockDim.x) stage[e] = __ldcg(part + e);
    __syncthreads();
    for (int e = threadIdx.x; e < 6 * W; e += blockDim.x) {
        const int off = (e / 6) * gx * 6 + (e % 6);
        // four interleaved partial sums: GB300's FP64 adds have long latency
        double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
        int x = 0;
        if (staged) {
            for (; x + 3 < gx; x += 4) {
                t0 += stage[off + 6 * x];
                t1 += stage[off + 6 * (x + 1)];
                t2 += stage[off + 6 * (x + 2)];
                t3 += stage[off + 6 * (x + 3)];
            }
            for (; x < gx; ++x) t0 += stage[off + 6 * x];
        } else {
            for (; x + 3 < gx; x += 4) {
                t0 += __ldcg(part + off + 6 * (size_t)x);
                t1 += __ldcg(part + off + 6 * (size_t)(x + 1));
                t2 += __ldcg(part + off + 6 * (size_t)(x + 2));
                t3 += __ldcg(part + off + 6 * (size_t)(x + 3));
            }
            for (; x < gx; ++x) t0 += __ldcg(part + off + 6 * (size_t)x);
        }
        sh[e] = (t0 + t1) + (t2 + t3);
    }
    __syncthreads();
}

// S1: grid (ceil(nblob/kS1Blobs), W), kS1Tpb threads.  First the second
// CGS pass's update that the previous S4 left pending, w -= Q[:, 0..k-1) h2
// (h2 still in h): lane = blob, warp q takes the columns i = q mod 4, and
// the CTAs with the lowest linear indices also update the body rows, 32
// each.  Then q_{k-1} = w / ||w|| into Q and the body moments of q; the
// last CTA adds the moments per swimmer and forms the body rows of q and
// z_body.
constexpr int kS1Blobs = 32;
constexpr int kS1Tpb = 128;
__global__ void __launch_bounds__(kS1Tpb) s1_update_normalise_moments_kernel(
    int W, int nblob, double *__restrict__ Q, size_t ld, double *__restrict__ w,
    const double *__restrict__ R, const double *__restrict__ refs, const double *__restrict__ ktk_rot,
    const double *__restrict__ mob_rot, const double *__restrict__ ktkf_rot, double minv, double *__restrict__ z,
    double *__restrict__ part, const double *__restrict__ scal, int *ticket, const GmresCtl *ctl)
{
    pdl_wait_then_release();
    static_assert(kS1Tpb == 4 * 32 && kS1Blobs == 32, "S1: four warps over 32 blobs");
    if (ctl->done) return;
    __shared__ double hs[kFMaxK];
    __shared__ double up[4][3 * kS1Blobs];
    __shared__ double upb[4][32];
    const int n = blockIdx.y, lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nb = W * nblob;
    const int m = blockIdx.x * kS1Blobs + lane;
    const int kq = ctl->k, cnt = kq - 1;  // the pending update spans Q[:, 0..cnt)
    double *q = Q + ld * (size_t)(kq - 1);
    const double nrm = scal[kNormOff], inrm = 1.0 / nrm;
    for (int i = threadIdx.x; i < cnt; i += kS1Tpb) hs[i] = scal[kHOff + i];
    __syncthreads();
    const size_t row = 3 * ((size_t)n * nblob + m);
    double p0 = 0.0, p1 = 0.0, p2 = 0.0;
    if (m < nblob)
        for (int i = wid; i < cnt; i += 4) {
            const double *qi = Q + ld * i + row;
            p0 += hs[i] * qi[0];
            p1 += hs[i] * qi[1];
            p2 += hs[i] * qi[2];
        }
    up[wid][3 * lane] = p0;
    up[wid][3 * lane + 1] = p1;
    up[wid][3 * lane + 2] = p2;
    const int lin = blockIdx.y * gridDim.x + blockIdx.x, br = 32 * lin + lane;
    const bool body_cta = 32 * lin < 6 * W;
    if (body_cta) {
        double pb = 0.0;
        if (br < 6 * W)
            for (int i = wid; i < cnt; i += 4) pb += hs[i] * Q[ld * i + 3 * (size_t)nb + br];
        upb[wid][lane] = pb;
    }
    __syncthreads();
    if (body_cta && wid == 0 && br < 6 * W)
        w[3 * (size_t)nb + br] -= (upb[0][lane] + upb[1][lane]) + (upb[2][lane] + upb[3][lane]);
    double a[6] = {0, 0, 0, 0, 0, 0};
    if (wid == 0 && m < nblob) {
        double f[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int e = 3 * lane + c;
            f[c] = (w[row + c] - ((up[0][e] + up[1][e]) + (up[2][e] + up[3][e]))) * inrm;
            q[row + c] = f[c];
        }
        double d[3];
        rot_apply(R + 9 * n, refs + 3 * m, d);
        a[0] = f[0];
        a[1] = f[1];
        a[2] = f[2];
        a[3] = d[1] * f[2] - d[2] * f[1];
        a[4] = d[2] * f[0] - d[0] * f[2];
        a[5] = d[0] * f[1] - d[1] * f[0];
    }
    block_sum6<kS1Tpb>(a, part + ((size_t)n * gridDim.x + blockIdx.x) * 6);
    if (!last_cta(ticket, gridDim.x * gridDim.y)) return;
    extern __shared__ double sh[];  // 6 W moments of q, then 6 W of z_body
    double *zsh = sh + 6 * W;
    swimmer_sums(part, W, gridDim.x, sh);
    // body rows of q, and z_body = KTKinv_rot (-sums) - mob_rot q_body: one
    // thread per (swimmer, row), the products in two interleaved chains each
    for (int e = threadIdx.x; e < 6 * W; e += kS1Tpb) {
        const int sw = e / 6, i = e % 6;
        const double *sums = sh + 6 * sw, *wb = w + 3 * (size_t)nb + 6 * sw;
        q[3 * nb + e] = __ldcg(wb + i) * inrm;
        const double *Kt = ktk_rot + 36 * sw + i, *Mb = mob_rot + 36 * sw + i;
        double x0 = 0.0, x1 = 0.0, y0 = 0.0, y1 = 0.0;
#pragma unroll
        for (int j = 0; j < 6; j += 2) {
            x0 += Kt[6 * j] * (-sums[j]);
            x1 += Kt[6 * (j + 1)] * (-sums[j + 1]);
            y0 += Mb[6 * j] * __ldcg(wb + j);
            y1 += Mb[6 * (j + 1)] * __ldcg(wb + j + 1);
        }
        const double zb = (x0 + x1) - (y0 + y1) * inrm;
        z[3 * nb + e] = zb;
        zsh[e] = zb;
    }
    __syncthreads();  // every body row of w is read; z_body is complete
    // w_body = -K^T z for the blob block z = Minv^(W-n) (q + K z_body) that
    // S2 is about to form: by linearity -Minv^(W-n) (K^T q + (K^T K) z_body),
    // K^T q being the moments summed above (the reference sums K^T z over
    // the blobs of z, mobility_solver.cpp:921-940)
    for (int e = threadIdx.x; e < 6 * W; e += kS1Tpb) {
        const int sw = e / 6, i = e % 6;
        const double *Kf = ktkf_rot + 36 * sw + i, *zb = zsh + 6 * sw;
        double x0 = 0.0, x1 = 0.0;
#pragma unroll
        for (int j = 0; j < 6; j += 2) {
            x0 += Kf[6 * j] * zb[j];
            x1 += Kf[6 * (j + 1)] * zb[j + 1];
        }
        double v = sh[e] + (x0 + x1);
        for (int k = sw; k < W; ++k) v *= minv;
        w[3 * (size_t)nb + e] = -v;
    }
}

// S2: grid (ceil(nblob/kSBlobs), W), one thread per blob: the blob block of
// the preconditioner, z_blob = Minv^(W-n) (q + U + Omega x (R ref)), applied
// W - n times for swimmer n as the reference's loop does
// (mobility_solver.cpp:651-721), and the records of z for the pair kernel.
// (w_body = -K^T z was formed by S1 from the moments of q.)
__global__ void __launch_bounds__(kSBlobs) s2_precond_blobs_kernel(
    int W, int nblob, const double *__restrict__ Q, size_t ld, const double *__restrict__ R,
    const double *__restrict__ refs, double minv, const double *__restrict__ xb, double *__restrict__ z, void *rec,
    int f64, const GmresCtl *ctl)
{
    pdl_wait_then_release();
    if (ctl->done) return;
    const int n = blockIdx.y, m = blockIdx.x * kSBlobs + threadIdx.x, nb = W * nblob;
    if (m >= nblob) return;
    const double *in = Q + ld * (size_t)(ctl->k - 1);
    const double *U = z + 3 * nb + 6 * n;
    const size_t i = (size_t)n * nblob + m;
    double d[3];
    rot_apply(R + 9 * n, refs + 3 * m, d);
    double o[3] = {in[3 * i] + U[0], in[3 * i + 1] + U[1], in[3 * i + 2] + U[2]};
    o[0] += U[4] * d[2] - U[5] * d[1];
    o[1] += U[5] * d[0] - U[3] * d[2];
    o[2] += U[3] * d[1] - U[4] * d[0];
    for (int k = n; k < W; ++k) {
        o[0] *= minv;
        o[1] *= minv;
        o[2] *= minv;
    }
    z[3 * i] = o[0];
    z[3 * i + 1] = o[1];
    z[3 * i + 2] = o[2];
    pack_record(rec, (int)i, xb + 3 * i, o, f64);
}

// Column sums out[i * ostride] = sum over b < count of p[i * stride + b],
// i < k.  A column's terms go to G adjacent lanes (G the largest power of
// two, at most 32, with k G <= kSTpb), two interleaved chains per lane, and
// meet by shuffles, so the FP64 adds spread over every warp of the CTA
// whatever k is.  Fixed order: deterministic.
template <bool kCg>
__device__ __forceinline__ void sum_columns(const double *p, size_t stride, int count, int k, double *out,
                                            size_t ostride)
{
    int G = 1;
    while (G < 32 && k * (2 * G) <= kSTpb) G *= 2;
    const int t = threadIdx.x, g = t & (G - 1), c0 = t / G, cstep = kSTpb / G;
    for (int cb = 0; cb < k; cb += cstep) {
        const int i = cb + c0;
        double a0 = 0.0, a1 = 0.0;
        if (i < k) {
            const double *pi = p + (size_t)i * stride;
            int b = g;
            for (; b + G < count; b += 2 * G) {
                a0 += kCg ? __ldcg(pi + b) : pi[b];
                a1 += kCg ? __ldcg(pi + b + G) : pi[b + G];
            }
            if (b < count) a0 += kCg ? __ldcg(pi + b) : pi[b];
        }
        double sum = a0 + a1;
        for (int o = 1; o < G; o <<= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (i < k && g == 0) out[(size_t)i * ostride] = sum;
    }
}

// Projections of this CTA's rows (ws, kSRows of them) on Q[:, 0..k) into
// P[i*nblk + blk]: each column's rows split into G groups on adjacent lanes
// (the largest power of two with k G <= kSTpb), so every warp takes a share.
__device__ __forceinline__ void cta_projections(const double *__restrict__ Q, size_t ld, int row0, int rows, int k,
                                                const double *ws, double *__restrict__ P, int nblk)
{
    int G = 1;
    while (G < kSRows && k * (2 * G) <= kSTpb) G *= 2;
    const int per = kSRows / G, t = threadIdx.x, g = t & (G - 1), c0 = t / G, cstep = kSTpb / G;
    const int rb = g * per, re = min(rows, rb + per);
    for (int cb = 0; cb < k; cb += cstep) {
        const int i = cb + c0;
        double a0 = 0.0, a1 = 0.0;
        if (i < k) {
            const double *q = Q + ld * i + row0;
            int r = rb;
            for (; r + 1 < re; r += 2) {
                a0 += q[r] * ws[r];
                a1 += q[r + 1] * ws[r + 1];
            }
            if (r < re) a0 += q[r] * ws[r];
        }
        double sum = a0 + a1;
        for (int o = 1; o < G; o <<= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (i < k && g == 0) P[(size_t)i * nblk + blockIdx.x] = sum;
    }
}

// Two-level sum of the per-CTA projections into h[0..k); true in the CTA
// that finished it.  tickets[0] is the top level, tickets[1 + g] group g's.
__device__ __forceinline__ bool finish_projections(const double *P, int k, int nblk, double *G, int *tickets,
                                                   double *h)
{
    const int ngroups = (nblk + kSGroup - 1) / kSGroup, g = blockIdx.x / kSGroup;
    const int first = g * kSGroup, gsize = min(kSGroup, nblk - first);
    if (!last_cta(tickets + 1 + g, gsize)) return false;
    sum_columns<true>(P + first, nblk, gsize, k, G + g, ngroups);
    if (!last_cta(tickets, ngroups)) return false;
    sum_columns<true>(G, ngroups, ngroups, k, h, 1);
    __syncthreads();  // h[i] is written by column i's group lane, then read by thread i
    return true;
}

__device__ __forceinline__ void givens_step(double *__restrict__ H, int ldh, int iter, double nrm,
                                            double *__restrict__ beta, double *__restrict__ cs,
                                            double *__restrict__ sn, double *__restrict__ scal, GmresCtl *ctl);

// S3: blob rows of w, first CGS pass.  With splits > 1 the blob-blob pair
// sum left per-split partials (mpart[p * 3B + r]), which this kernel adds:
// warp q takes the splits p = q mod 4 for the CTA's 32 rows (one per lane).
__global__ void __launch_bounds__(kSTpb) s3_finish_project_kernel(
    int W, int nblob, const double *__restrict__ mbb, const double *__restrict__ mpart, int splits,
    const double *__restrict__ z, const double *__restrict__ R, const double *__restrict__ refs,
    double *__restrict__ w, const double *__restrict__ Q, size_t ld, int n, double *__restrict__ P,
    double *__restrict__ G, int *tickets, double *__restrict__ scal, double *__restrict__ H, int ldh,
    double *__restrict__ beta, double *__restrict__ cs, double *__restrict__ sn, GmresCtl *ctl, double eta2)
{
    pdl_wait_then_release();
    static_assert(kSTpb == 4 * kSRows && kSRows == 32, "S3's split sum: four warps over 32 rows");
    if (ctl->done) return;
    __shared__ double ws[kSRows];
    __shared__ double msum[4][kSRows];
    const int k = ctl->k, row0 = blockIdx.x * kSRows, nb3 = 3 * W * nblob;
    const int rows = min(kSRows, n - row0);
    if (splits > 1) {
        const int lr = threadIdx.x & 31, q = threadIdx.x >> 5, r = row0 + lr;
        double a0 = 0.0, a1 = 0.0;
        if (r < nb3) {
            int p = q;
            for (; p + 4 < splits; p += 8) {
                a0 += mpart[(size_t)p * nb3 + r];
                a1 += mpart[(size_t)(p + 4) * nb3 + r];
            }
            if (p < splits) a0 += mpart[(size_t)p * nb3 + r];
        }
        msum[q][lr] = a0 + a1;
        __syncthreads();
    }
    if (threadIdx.x < kSRows) {
        const int r = row0 + threadIdx.x;
        double v = 0.0;
        if (r < nb3) {
            const int i = r / 3, c = r % 3, sw = i / nblob, m = i % nblob;
            double d[3];
            rot_apply(R + 9 * sw, refs + 3 * m, d);
            const double *U = z + nb3 + 6 * sw;
            double kz;
            if (c == 0) kz = U[0] - d[1] * U[5] + d[2] * U[4];
            else if (c == 1) kz = U[1] - d[2] * U[3] + d[0] * U[5];
            else kz = U[2] - d[0] * U[4] + d[1] * U[3];
            const int t = threadIdx.x;
            const double mb = splits > 1 ? (msum[0][t] + msum[1][t]) + (msum[2][t] + msum[3][t]) : mbb[r];
            v = -kz + mb;
            w[r] = v;
        } else if (r < n) {
            v = w[r];
        }
        ws[threadIdx.x] = v;
    }
    __syncthreads();
    cta_projections(Q, ld, row0, rows, k, ws, P, gridDim.x);
    const bool dgks = eta2 > 0.0;
    if (dgks && threadIdx.x < 32) {  // ||w||^2 of the CTA's rows rides along as column k
        const double v = ws[threadIdx.x];
        const double a = warp_sum(v * v);
        if (threadIdx.x == 0) P[(size_t)k * gridDim.x + blockIdx.x] = a;
    }
    double *h = scal + kHOff;
    if (!finish_projections(P, dgks ? k + 1 : k, gridDim.x, G, tickets, h)) return;
    double *Hcol = H + (size_t)ldh * (k - 1);
    for (int i = threadIdx.x; i < k; i += kSTpb) Hcol[i] = h[i];
    // Conditional re-orthogonalisation (Daniel, Gragg, Kaufman and Stewart):
    // after one classical pass ||w - Q h||^2 = ||w||^2 - ||h||^2; when that
    // keeps at least eta^2 of ||w||^2 (eta = 1/sqrt 2: "twice is enough"),
    // w - Q h is orthogonal to Q to working precision and the difference
    // has not cancelled, so the second pass (S4) is skipped: its norm is
    // taken here and the Givens step runs in this CTA.  S1 then applies the
    // pending update w -= Q h with these first-pass coefficients.
    __shared__ double nrm_s;
    __shared__ int skip_s;
    if (threadIdx.x < 32) {
        int skip = 0;
        double nrm = 0.0;
        if (dgks) {
            double t = 0.0;
            for (int i = threadIdx.x; i < k; i += 32) t += h[i] * h[i];
            t = warp_sum(t);
            const double w2 = h[k], after = w2 - t;
            skip = (w2 > 0.0 && after >= eta2 * w2 && after < INFINITY) ? 1 : 0;
            nrm = skip ? sqrt(after) : 0.0;
        }
        if (threadIdx.x == 0) {
            nrm_s = nrm;
            skip_s = skip;
            ctl->pass2 = skip ? 0 : 1;
        }
    }
    __syncthreads();  // the H column is written; the decision is shared
    if (skip_s) givens_step(H, ldh, k, nrm_s, beta, cs, sn, scal, ctl);
}

// w -= Q h on this CTA's rows (rows go to ws): warp q takes the columns
// i = q mod 4 (lane = row, two interleaved chains), and the four partial
// products meet in shared memory.
__device__ __forceinline__ void cta_update(const double *__restrict__ Q, size_t ld, int row0, int rows, int k,
                                           const double *__restrict__ h, double *__restrict__ w, double *ws)
{
    static_assert(kSTpb == 4 * kSRows && kSRows == 32, "cta_update: four warps over 32 rows");
    __shared__ double hs[kFMaxK];
    __shared__ double up[4][kSRows];
    for (int i = threadIdx.x; i < k; i += kSTpb) hs[i] = h[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double p0 = 0.0, p1 = 0.0;
    if (lane < rows) {
        const double *q = Q + row0 + lane;
        int i = wid;
        for (; i + 4 < k; i += 8) {
            p0 += hs[i] * q[ld * i];
            p1 += hs[i + 4] * q[ld * (i + 4)];
        }
        if (i < k) p0 += hs[i] * q[ld * i];
    }
    up[wid][lane] = p0 + p1;
    __syncthreads();
    if (threadIdx.x < kSRows) {
        double v = 0.0;
        if (threadIdx.x < rows) {
            const int r = row0 + threadIdx.x;
            v = w[r] - ((up[0][lane] + up[1][lane]) + (up[2][lane] + up[3][lane]));
            w[r] = v;
        }
        ws[threadIdx.x] = v;
    }
    __syncthreads();
}

// The Givens step of solve_linear_system (mobility_solver.cpp:1189-1231) on
// H column iter-1, whose subdiagonal entry is nrm, run by the last CTA of
// S4 (all of its threads enter; warp 0 does the work): the previous
// rotations over the column, the new rotation, beta, the residual and the
// iteration control.  The H column and the rotations go to shared memory
// first, so the sequential parts read no global memory.
__device__ __forceinline__ void givens_step(double *__restrict__ H, int ldh, int iter, double nrm,
                                            double *__restrict__ beta, double *__restrict__ cs,
                                            double *__restrict__ sn, double *__restrict__ scal, GmresCtl *ctl)
{
    __shared__ double col[kFMaxK + 1], csh[kFMaxK], snh[kFMaxK];
    double *gcol = H + (size_t)ldh * (iter - 1);
    for (int i = threadIdx.x; i < iter; i += blockDim.x) {
        col[i] = gcol[i];
        if (i < iter - 1) {
            csh[i] = cs[i];
            snh[i] = sn[i];
        }
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    // The previous rotations over the new H column, as a warp scan: entry i
    // after rotation i is x_i = -s_{i-1} x_{i-1} + c_{i-1} col_i, a
    // first-order linear recurrence (x -> a x + b pairs, Kogge-Stone over 32
    // entries at a time); the rotated entries are c_{i-1} x_{i-1} + s_{i-1}
    // col_i.  (One thread's serial sweep costs ~64 cycles per FP64 step here.)
    double xin = 0.0;
    for (int base = 0; base < iter; base += 32) {
        const int i = base + lane;
        double aa = 1.0, bb = 0.0, cur = 0.0;
        if (i < iter) {
            cur = col[i];
            if (i == 0) {
                aa = 0.0;
                bb = cur;
            } else {
                aa = -snh[i - 1];
                bb = csh[i - 1] * cur;
            }
        }
        for (int o = 1; o < 32; o <<= 1) {
            const double ap = __shfl_up_sync(0xffffffffu, aa, o), bp = __shfl_up_sync(0xffffffffu, bb, o);
            if (lane >= o) {
                bb = fma(aa, bp, bb);
                aa = aa * ap;
            }
        }
        const double xi = fma(aa, xin, bb);
        double xm1 = __shfl_up_sync(0xffffffffu, xi, 1);
        if (lane == 0) xm1 = xin;
        if (i >= 1 && i < iter) col[i - 1] = csh[i - 1] * xm1 + snh[i - 1] * cur;
        xin = __shfl_sync(0xffffffffu, xi, 31);  // lanes past the column repeat its last entry
    }
    if (lane == 0) {
        scal[kNormOff] = nrm;
        const double hk = nrm, hd = xin;
        double c, s;
        if (hk == 0.0) {
            c = 1.0;
            s = 0.0;
        } else if (fabs(hk) > fabs(hd)) {  // the reference's scaled form; rsqrt saves a division
            const double u = hd / hk;
            s = (2.0 * (double)(hk > 0) - 1.0) * rsqrt(1.0 + u * u);
            c = u * s;
        } else {
            const double u = hk / hd;
            c = (2.0 * (double)(hd > 0) - 1.0) * rsqrt(1.0 + u * u);
            s = u * c;
        }
        cs[iter - 1] = c;
        sn[iter - 1] = s;
        col[iter - 1] = c * hd + s * hk;
        col[iter] = 0.0;
        beta[iter] = -s * beta[iter - 1];
        beta[iter - 1] = c * beta[iter - 1];
        const double resid = fabs(beta[iter]) * ctl->inv_norm_ref;
        ctl->resid = resid;
        const int replays = ++ctl->replays;
        // converged, at the cap, or NaN; the replay count bounds the loop even if k stalled
        const bool done = !(resid > ctl->tol) || iter >= ctl->max_iter || replays > ctl->max_iter;
        if (done)
            ctl->done = 1;
        else
            ctl->k = iter + 1;
    }
    __syncwarp();
    for (int i = lane; i <= iter; i += 32) gcol[i] = col[i];
}

// S4: second CGS pass.  w -= Q h1 (S3's projections), then h2 = Q^T w and,
// as one more projection column, ||w||^2.  The last CTA adds h2 to the H
// column and takes the new basis vector's norm as
// ||w - Q h2||^2 = ||w||^2 - ||h2||^2 (Q orthonormal; h2 is the second
// pass's correction, small next to w, so the difference keeps its
// precision), then runs the Givens step.  The update w -= Q h2 itself is
// left to the next S1, which touches every row anyway.
__global__ void __launch_bounds__(kSTpb) s4_project_norm_givens_kernel(
    const double *__restrict__ Q, size_t ld, int n, double *__restrict__ w, double *__restrict__ P,
    double *__restrict__ G, int *tickets, double *__restrict__ scal, double *__restrict__ H, int ldh,
    double *__restrict__ beta, double *__restrict__ cs, double *__restrict__ sn, GmresCtl *ctl)
{
    pdl_wait_then_release();
    if (ctl->done || ctl->pass2 == 0) return;  // converged, or S3 skipped the second pass
    __shared__ double ws[kSRows];
    __shared__ double nrm_s;
    const int k = ctl->k, row0 = blockIdx.x * kSRows, rows = min(kSRows, n - row0);
    double *h = scal + kHOff;
    cta_update(Q, ld, row0, rows, k, h, w, ws);
    cta_projections(Q, ld, row0, rows, k, ws, P, gridDim.x);
    if (threadIdx.x < 32) {  // kSRows == 32: one row per lane (zero past the last row)
        const double v = ws[threadIdx.x];
        const double a = warp_sum(v * v);
        if (threadIdx.x == 0) P[(size_t)k * gridDim.x + blockIdx.x] = a;
    }
    // h is overwritten only after every CTA has read it (all arrived)
    if (!finish_projections(P, k + 1, gridDim.x, G, tickets, h)) return;
    double *Hcol = H + (size_t)ldh * (k - 1);
    for (int i = threadIdx.x; i < k; i += kSTpb) Hcol[i] += h[i];
    if (threadIdx.x < 32) {
        double t = 0.0;
        for (int i = threadIdx.x; i < k; i += 32) t += h[i] * h[i];
        t = warp_sum(t);
        if (threadIdx.x == 0) nrm_s = sqrt(fmax(h[k] - t, 0.0));
    }
    __syncthreads();
    givens_step(H, ldh, k, nrm_s, beta, cs, sn, scal, ctl);
}

// Last node of the device-side loop's body: one thread decides whether the
// loop runs again.  It runs once per pass whatever the step kernels did, and
// its own pass count ends the loop after max_iter + 1 passes in any case.
__global__ void arnoldi_loop_guard_kernel(GmresCtl *ctl, cudaGraphConditionalHandle loop)
{
    pdl_wait_then_release();
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int passes = ++ctl->guard;
    const bool again = ctl->done == 0 && passes <= ctl->max_iter + 1;
    cudaGraphSetConditional(loop, again ? 1u : 0u);
}

// Back substitution y = H(0:iter, 0:iter)^-1 beta(0:iter)
// (mobility_solver.cpp:1236-1250) by one warp: column by column, the lanes
// update the remaining right-hand side, each row in the reference's order.
// The diagonal's reciprocals are taken up front, all lanes at once, so a
// column's step on the serial chain is one multiply and one FMA; the row
// blocks below the column (nothing left to update) are skipped warp-wide.
__global__ void backsolve_warp_kernel(const double *__restrict__ H, int ldh, const double *__restrict__ beta,
                                      int iter, double *__restrict__ y, const GmresCtl *ctl)
{
    constexpr int kPer = (kFMaxK + 31) / 32;
    __shared__ double b[kFMaxK], rd[kFMaxK];
    const int lane = threadIdx.x;
    if (ctl != nullptr) iter = min(ctl->k, kFMaxK - 1);  // the solve's count, read on the device
    for (int i = lane; i < iter; i += 32) {
        b[i] = beta[i];
        rd[i] = 1.0 / H[i + (size_t)ldh * i];
    }
    __syncwarp();
    // column j of H in registers (row i = lane + 32 q), the next one in flight
    double cur[kPer], nxt[kPer];
    const int j0 = iter - 1;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        const int i = lane + 32 * q;
        cur[q] = i < j0 ? H[i + (size_t)ldh * j0] : 0.0;
    }
    for (int j = j0; j >= 0; --j) {
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int i = lane + 32 * q;
            nxt[q] = (i < j - 1) ? H[i + (size_t)ldh * (j - 1)] : 0.0;
        }
        const double yj = b[j] * rd[j];
        const int qmax = (j - 1) >> 5;  // row blocks holding rows < j (-1 when j == 0)
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            if (q <= qmax) {
                const int i = lane + 32 * q;
                if (i < j) b[i] -= cur[q] * yj;
            }
        }
        if (lane == 0) y[j] = yj;
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kPer; ++q) cur[q] = nxt[q];
    }
}

}  // namespace gmi

namespace gmi {

static inline int grid_for(int n, int tpb = 256) { return (n + tpb - 1) / tpb; }

static gmi_status dalloc(gmi_solver *s, double **p, size_t count)
{
    if (count == 0) count = 1;
    cudaError_t e = dev_malloc(p, count * sizeof(double));
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e), "cudaMalloc", __FILE__, __LINE__);
        return GMI_ERR_CUDA;
    }
    s->allocs.push_back(*p);
    GMI_CUDA_TRY(cudaMemsetAsync(*p, 0, count * sizeof(double), s->ctx->stream));
    return GMI_OK;
}

static gmi_status halloc(double **p, size_t count)
{
    if (count == 0) count = 1;
    GMI_CUDA_TRY(host_alloc(p, count * sizeof(double), cudaHostAllocPortable));
    std::memset(*p, 0, count * sizeof(double));
    return GMI_OK;
}


static gmi_status launched(gmi_solver *s, int kernels = 1)
{
    s->ctx->launches += kernels;
    GMI_CUDA_TRY(cudaGetLastError());
    return GMI_OK;
}

static gmi_status read_scalar(gmi_solver *s, const double *d_ptr, double *out)
{
    GMI_CUDA_TRY(cudaMemcpyAsync(s->h_stage, d_ptr, sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    *out = s->h_stage[0];
    return GMI_OK;
}

static int nchunks_of(int n) { return (n + kChunkRows - 1) / kChunkRows; }

// ||x|| into s->scal[0] (device); no host sync.
static gmi_status device_norm(gmi_solver *s, const double *x, int n)
{
    const int nc = nchunks_of(n);
    norm_kernel<<<nc, kRedTpb, 0, s->ctx->stream>>>(x, n, s->partial, s->scal, s->aux_tickets);
    return launched(s);
}

static gmi_status prepare_bodies(gmi_solver *s)
{
    if (s->W == 0) return GMI_OK;
    prepare_bodies_kernel<<<grid_for(108 * s->W, 128), 128, 0, s->ctx->stream>>>(
        s->W, s->body_q, s->ktk_ref, s->mob_ref, s->ktkf_ref, s->R, s->ktk_rot, s->mob_rot, s->ktkf_rot);
    return launched(s);
}

// K^T of the blob block of `vec` into s->sums.
static gmi_status kt_sums(gmi_solver *s, const double *vec)
{
    const int gx = (s->cfg.nblob + kKtBlobs - 1) / kKtBlobs;
    kt_kernel<<<dim3(gx, s->W), kKtBlobs, 0, s->ctx->stream>>>(s->W, s->cfg.nblob, s->R, s->refs, vec, s->kt_part,
                                                              s->sums, s->aux_tickets + 1);
    return launched(s);
}

// out = P^-1 in (apply_preconditioner, right preconditioning)
static gmi_status apply_preconditioner(gmi_solver *s, const double *in, double *out)
{
    const int nb = s->B;
    GMI_TRY(kt_sums(s, in));
    precond_body_kernel<<<grid_for(s->W, 64), 64, 0, s->ctx->stream>>>(s->W, s->sums, in + 3 * nb, s->ktk_rot,
                                                                        s->mob_rot, out + 3 * nb);
    const double minv = 6.0 * kPi * s->cfg.mu * s->cfg.rblob;
    precond_blob_kernel<<<grid_for(nb), 256, 0, s->ctx->stream>>>(s->W, s->cfg.nblob, in, out + 3 * nb, s->R, s->refs,
                                                                  minv, out);
    return launched(s, 2);
}

// out = A in (system_matrix_mult): [M_bb, -K; -K^T, 0]
static gmi_status system_matrix_mult(gmi_solver *s, const double *in, double *out)
{
    const int nb = s->B;
    gmi_context *ctx = s->ctx;
    GMI_TRY(pack_records(ctx, s->x_blobs, in, 3, nb, ctx->rec_src));
    PairConsts k;
    fill_consts(k, s->cfg.rblob, s->cfg.rblob, s->cfg.rblob, s->cfg.mu);
    GMI_TRY(launch_pair(ctx, kBB, ctx->rec_src.ptr, 0, nb, ctx->rec_src.ptr, nb, k, s->mbb, 0));
    GMI_TRY(kt_sums(s, in));
    sysmult_finish_kernel<<<grid_for(nb + 6 * s->W), 256, 0, ctx->stream>>>(s->W, s->cfg.nblob, s->mbb, in + 3 * nb,
                                                                           s->sums, s->R, s->refs, out);
    return launched(s);
}

// CGS2 orthogonalisation of w against Q[:, 0..k-1]; H column receives the
// projections.  Then H(k, col) = ||w|| and Q[:, k] = w / ||w||.
static gmi_status orthonormalise(gmi_solver *s, double *w, int k, double *Hcol)
{
    const int n = s->n, nc = nchunks_of(n);
    const size_t ld = (size_t)n;
    for (int pass = 0; pass < 2; ++pass) {
        dot_partials_kernel<<<dim3(nc, k), kRedTpb, 0, s->ctx->stream>>>(s->Q, ld, w, n, nc, s->partial);
        cgs_update_kernel<<<grid_for(n, kRedTpb), kRedTpb, k * sizeof(double), s->ctx->stream>>>(
            s->Q, ld, k, s->partial, nc, w, n, Hcol, pass);
        GMI_TRY(launched(s, 2));
    }
    dot_partials_kernel<<<dim3(nc, 1), kRedTpb, 0, s->ctx->stream>>>(w, ld, w, n, nc, s->partial);
    normalize_kernel<<<grid_for(n), 256, 0, s->ctx->stream>>>(w, n, s->partial, nc, s->Q + ld * k, Hcol + k);
    return launched(s, 2);
}

// K^T K of one swimmer's blob references, column-major 6x6
// (mobility_solver.cpp:1697-1713): K maps (U, Omega) to U + Omega x r per blob.
static void ktk_from_refs(const double *refs, int nblob, double *KTK)
{
    for (int e = 0; e < 36; ++e) KTK[e] = 0.0;
    KTK[0] = KTK[7] = KTK[14] = (double)nblob;
    for (int m = 0; m < nblob; ++m) {
        const double *r = refs + 3 * m;
        // the reference's rcross(r) (matrix.cpp:665-679), row-major: rcross(r) b = b x r
        const double rc[9] = {0.0, r[2], -r[1], -r[2], 0.0, r[0], r[1], -r[0], 0.0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                KTK[i + 6 * (3 + j)] += rc[3 * i + j];
                KTK[(3 + i) + 6 * j] -= rc[3 * i + j];
                double rr = 0.0;
                for (int k = 0; k < 3; ++k) rr += rc[3 * i + k] * rc[3 * k + j];
                KTK[(3 + i) + 6 * (3 + j)] -= rr;
            }
    }
}

// A kernel launch of the Arnoldi step; with pdl, marked for programmatic
// dependent launch, so that it may start while the previous kernel finishes
// (each step kernel waits first, in pdl_wait_then_release).
template <typename... KArgs, typename... Args>
static cudaError_t launch_step(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                               cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// eta^2 of the conditional re-orthogonalisation in the device Arnoldi
// steps: the second Gram-Schmidt pass runs only when one pass kept less
// than eta^2 of ||w||^2, i.e. when the projection cancelled more than
// 1 - eta of the new vector's norm.  After one classical pass the new
// vector's loss of orthogonality to the basis is about eps / eta, so
// eta = 0.1 keeps it within ten rounding units per vector (far below what
// GMRES notices).  That is the default of the mixed-precision solve, which
// checks every result with an FP64-grade residual: measured on the swimmer
// workloads, eta = 0.1 and eta = 1/sqrt(2) give the same GMRES counts and
// the same velocities to the Broyden tolerance, and 0.1 skips the second
// pass far more often.  FP64 solves keep eta = 1/sqrt(2) (Daniel, Gragg,
// Kaufman and Stewart's "twice is enough" value): with 0.1 a 12-step FP64
// trajectory of a small swimmer drifted from the reference's own by 8e-4,
// with 1/sqrt(2) it matches it to 1e-9.  GMI_REORTH_ETA sets eta for both; 0 runs the
// second pass always.
double reorth_eta2(bool fp64)
{
    const char *env = std::getenv("GMI_REORTH_ETA");
    const double eta = env ? std::atof(env) : (fp64 ? 0.70710678118654752440 : 0.1);
    return eta > 0.0 ? eta * eta : 0.0;
}

// Sizes of the Arnoldi step's workspace inside s->partial and s->st_tickets.
struct StepLayout {
    int gx, nblk, ngroups;
    size_t doubles, tickets;
};

static StepLayout step_layout(int n, int nblob, int W)
{
    StepLayout L;
    L.gx = (nblob + kS1Blobs - 1) / kS1Blobs;  // S1's CTAs per swimmer (S2 has fewer)
    L.nblk = (n + kSRows - 1) / kSRows;
    L.ngroups = (L.nblk + kSGroup - 1) / kSGroup;
    L.doubles = (size_t)kFMaxK * (L.nblk + L.ngroups) + (size_t)W * L.gx * 6;
    L.tickets = 5 + 2 * (size_t)L.ngroups;
    return L;
}

// One device-controlled Arnoldi step (S1, S2, the blob-blob pair apply, S3,
// S4) enqueued on the solver stream; captured once per precision into
// s->graph[pidx].
static gmi_status enqueue_arnoldi_step(gmi_solver *s, cudaGraphConditionalHandle loop, bool use_loop)
{
    gmi_context *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const int nb = s->B, n = s->n, W = s->W, nblob = s->cfg.nblob, ldh = s->m + 1;
    const size_t ld = (size_t)n;
    const bool f64 = ctx->precision == GMI_FP64;
    const double minv = 6.0 * kPi * s->cfg.mu * s->cfg.rblob;
    const StepLayout L = step_layout(n, nblob, W);
    if (L.doubles > s->partial_count || L.tickets > s->st_ticket_count || s->m + 1 > kFMaxK || L.gx == 0 || W == 0) {
        set_last_error("Arnoldi step workspace smaller than the step needs", "enqueue_arnoldi_step", __FILE__,
                       __LINE__);
        return GMI_ERR_STATE;
    }
    double *P = s->partial, *G = P + (size_t)kFMaxK * L.nblk, *part = G + (size_t)kFMaxK * L.ngroups;
    int *tk = s->st_tickets;
    int *tk3 = tk + 2, *tk4 = tk3 + 1 + L.ngroups;
    const size_t wsm = 6 * (size_t)W * sizeof(double);
    const bool pdl = s->use_pdl;
    GMI_CUDA_TRY(launch_step(pdl, s1_update_normalise_moments_kernel, dim3(L.gx, W), dim3(kS1Tpb), 2 * wsm, st, W,
                             nblob, s->Q, ld, s->w, (const double *)s->R, (const double *)s->refs,
                             (const double *)s->ktk_rot, (const double *)s->mob_rot, (const double *)s->ktkf_rot,
                             minv, s->z, part, (const double *)s->st_scal, tk, (const GmresCtl *)s->ctl));
    GMI_CUDA_TRY(launch_step(pdl, s2_precond_blobs_kernel, dim3((nblob + kSBlobs - 1) / kSBlobs, W), dim3(kSBlobs),
                             0, st, W, nblob, (const double *)s->Q, ld, (const double *)s->R,
                             (const double *)s->refs, minv, (const double *)s->x_blobs, s->z, s->gm_rec,
                             f64 ? 1 : 0, (const GmresCtl *)s->ctl));
    ExplicitPairEnv env{};
    env.stream = st;
    env.partial = s->gm_partial;
    env.partial_bytes = s->gm_partial_bytes;
    env.err = ctx->d_err;
    env.wait_ns = ctx->wait_ns;
    env.encode_tiled = ctx->encode_tiled;
    env.sm_count = ctx->sm_count;
    if (nb <= kPairWarpMaxSources) {
        env.tpb = kPairWarpShapeTpb;  // warp per two target blobs
        env.tt = 2;
    } else {
        // FP32: the packed kernel, 64 targets per CTA with one source tile
        // per split (at 4096 blobs, in the time step of a 16,896-particle
        // swimmer: steps 0.6-1.1 ms faster than with 128, every step; 128 had
        // been faster with the kernels timed one at a time under a profiler);
        // FP64: smaller CTAs for small target sets
        const bool small = (long long)nb * 2 < (long long)ctx->sm_count * 256;
        env.tpb = (small || !f64) ? 64 : 128;
        env.tt = (small || !f64) ? 1 : 2;
    }
    // GMI_GM_PAIR="tpb,tt,splits" overrides the shape (0 keeps a field's choice)
    if (const char *gs = std::getenv("GMI_GM_PAIR")) {
        int a = 0, b = 0, c = 0;
        if (std::sscanf(gs, "%d,%d,%d", &a, &b, &c) == 3) {
            if (a > 0) env.tpb = a;
            if (b > 0) env.tt = b;
            env.max_splits = c > 0 ? c : 0;
        }
    }
    env.skip = &s->ctl->done;
    env.pdl = pdl ? 1 : 0;
    PairConsts k;
    fill_consts(k, s->cfg.rblob, s->cfg.rblob, s->cfg.rblob, s->cfg.mu);
    int splits = 1;
    env.splits_out = &splits;  // S3 adds the split partials
    GMI_TRY(launch_pair_into(env, kBB, f64, s->gm_rec, 0, nb, s->gm_rec, nb, k, s->mbb, 0));
    GMI_CUDA_TRY(launch_step(pdl, s3_finish_project_kernel, dim3(L.nblk), dim3(kSTpb), 0, st, W, nblob,
                             (const double *)s->mbb, (const double *)s->gm_partial, splits, (const double *)s->z,
                             (const double *)s->R, (const double *)s->refs, s->w, (const double *)s->Q, ld, n, P,
                             G, tk3, s->st_scal, s->H, ldh, s->beta, s->cs, s->sn, s->ctl, reorth_eta2(f64)));
    GMI_CUDA_TRY(launch_step(pdl, s4_project_norm_givens_kernel, dim3(L.nblk), dim3(kSTpb), 0, st,
                             (const double *)s->Q, ld, n, s->w, P, G, tk4, s->st_scal, s->H, ldh, s->beta, s->cs,
                             s->sn, s->ctl));
    if (use_loop)
        GMI_CUDA_TRY(launch_step(pdl, arnoldi_loop_guard_kernel, dim3(1), dim3(32), 0, st, s->ctl, loop));
    return GMI_OK;
}

// Arnoldi steps per pass of the device-side loop: 4 by default (against
// one: FP32C steps of a 16,896-particle swimmer 30.5 -> 30.0 ms, FP64 steps
// of a 962-particle one 27.9 -> 27.0 ms), GMI_GMRES_UNROLL (1..8) overrides.
static int gmres_loop_unroll()
{
    const char *e = std::getenv("GMI_GMRES_UNROLL");
    int u = e ? std::atoi(e) : 4;
    return u < 1 ? 1 : (u > 8 ? 8 : u);
}

// Capture the Arnoldi step into body (a conditional node's body graph, or a
// fresh graph when body is null).
static gmi_status capture_step(gmi_solver *s, cudaGraph_t body, cudaGraphConditionalHandle loop, bool use_loop,
                               cudaGraph_t *out)
{
    cudaStream_t st = s->ctx->stream;
    // no thread synchronises the device while this capture is open
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    if (body)
        GMI_CUDA_TRY(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    else
        GMI_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    // the device-side loop's body holds `unroll` steps and one guard: steps
    // after the last iteration return at once (every step kernel checks
    // ctl->done first), and the loop's per-pass cost is paid once per unroll
    gmi_status est = GMI_OK;
    const int unroll = use_loop ? gmres_loop_unroll() : 1;
    for (int u = 0; u < unroll && est == GMI_OK; ++u) est = enqueue_arnoldi_step(s, loop, use_loop && u == unroll - 1);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (est != GMI_OK) {
        if (g && !body) cudaGraphDestroy(g);
        return est;
    }
    GMI_CUDA_TRY(ce);
    *out = g;
    return GMI_OK;
}

// Capture the Arnoldi loop (a WHILE conditional node around one step, or the
// step alone where conditional nodes are unavailable) and instantiate it.
static gmi_status build_arnoldi_graph(gmi_solver *s, int pidx)
{
    cudaGraph_t g = nullptr;
    bool loops = false;
    size_t body_nodes = 0;
    // GMI_GMRES_DEVICE_LOOP=0 selects the host-replayed step graph (whose
    // kernels profilers can attribute one by one)
    const char *env = std::getenv("GMI_GMRES_DEVICE_LOOP");
    const bool want_loop = !(env && env[0] == '0');
    if (want_loop && cudaGraphCreate(&g, 0) == cudaSuccess) {
        cudaGraphConditionalHandle h{};
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cudaGraphNode_t node;
        bool ok = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
        if (ok) {
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
        }
        if (ok) {
            cudaGraph_t body = cp.conditional.phGraph_out[0], captured = nullptr;
            const gmi_status cst = capture_step(s, body, h, true, &captured);
            if (cst != GMI_OK) {
                cudaGraphDestroy(g);
                return cst;
            }
            cudaGraphGetNodes(body, nullptr, &body_nodes);
            loops = true;
        } else {
            cudaGraphDestroy(g);
            g = nullptr;
            cudaGetLastError();
        }
    }
    if (!loops) GMI_TRY(capture_step(s, nullptr, cudaGraphConditionalHandle{}, false, &g));
    const cudaError_t ie = cudaGraphInstantiate(&s->graph[pidx], g, 0);
    size_t cnt = body_nodes;  // launches per Arnoldi step
    if (!loops) cudaGraphGetNodes(g, nullptr, &cnt);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) s->graph[pidx] = nullptr;
    GMI_CUDA_TRY(ie);
    s->graph_nodes[pidx] = cnt;
    s->graph_loops[pidx] = loops;
    return GMI_OK;
}

// The whole Arnoldi loop as one graph: a WHILE conditional node whose body is
// one step; the norm kernel of the step clears the condition when the solve
// is done.  Falls back to a graph of one step, replayed in batches from the
// host, where conditional nodes are unavailable, and to launches without
// programmatic dependencies where a graph with them fails to build.
static gmi_status ensure_arnoldi_graph(gmi_solver *s, int pidx, size_t *nodes)
{
    cudaStream_t st = s->ctx->stream;
    if (st == nullptr || st == cudaStreamLegacy || st == cudaStreamPerThread) {
        set_last_error_msg("graph capture needs a non-default stream");
        return GMI_ERR_STATE;
    }
    if (s->graph[pidx] == nullptr) {
        const char *pdl_env = std::getenv("GMI_PDL");
        if (pdl_env && pdl_env[0] == '0') s->use_pdl = false;
        gmi_status gst = build_arnoldi_graph(s, pidx);
        if (gst != GMI_OK && s->use_pdl) {
            cudaGetLastError();
            s->use_pdl = false;
            gst = build_arnoldi_graph(s, pidx);
        }
        if (gst != GMI_OK) return gst;
    }
    *nodes = s->graph_nodes[pidx];
    return GMI_OK;
}

// Arnoldi/GMRES core of solve_linear_system (mobility_solver.cpp:1162-1350),
// right preconditioned, on A x = b with b in s->rhs and the initial guess in
// s->soln.  Stops when |beta(iter)| <= tol * norm_ref.  reject_warm_start
// applies the reference's rule that a warm start with a residual above
// ||b|| is replaced by zero (mobility_solver.cpp:1149-1156).  zero_start
// skips the initial residual apply (x0 = 0, r0 = b, ||b|| = norm_b).
static gmi_status gmres_run(gmi_solver *s, double norm_b, double norm_ref, double tol, bool reject_warm_start,
                            bool zero_start, int *iters_out, bool defer = false)
{
    const int n = s->n;
    const size_t ld = (size_t)n;
    cudaStream_t st = s->ctx->stream;
    *iters_out = 0;
    double beta0;
    if (zero_start) {
        GMI_CUDA_TRY(cudaMemcpyAsync(s->w, s->rhs, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
        beta0 = norm_b;
    } else {
        GMI_TRY(system_matrix_mult(s, s->soln, s->tmp));
        axpby_kernel<<<grid_for(n), 256, 0, st>>>(n, 1.0, s->rhs, -1.0, s->tmp, s->w);
        GMI_TRY(launched(s));
        GMI_TRY(device_norm(s, s->w, n));
        GMI_TRY(read_scalar(s, s->scal, &beta0));
        if (fabs(beta0) <= tol * norm_ref) {  // the initial guess is good enough
            s->gm_resid = fabs(beta0) / norm_ref;
            return GMI_OK;
        }
        if (reject_warm_start && fabs(beta0) > norm_b) {
            GMI_CUDA_TRY(cudaMemsetAsync(s->soln, 0, ld * sizeof(double), st));
            GMI_CUDA_TRY(cudaMemcpyAsync(s->w, s->rhs, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
            beta0 = norm_b;
        }
    }
    s->h_stage[0] = beta0;
    GMI_CUDA_TRY(cudaMemcpyAsync(s->beta, s->h_stage, sizeof(double), cudaMemcpyHostToDevice, st));
    const int max_iter = n < s->m ? n : s->m;
    const int ldh = s->m + 1;
    const int pidx = s->ctx->precision == GMI_FP64 ? 0 : 1;
    size_t nodes = 0;
    const bool cluster = s->use_cluster && max_iter >= 1 && cluster_gmres_usable(s);
    if (!cluster && s->use_graphs && ensure_arnoldi_graph(s, pidx, &nodes) != GMI_OK) s->use_graphs = false;
    // defer: the solve's control block is checked at the caller's next
    // synchronisation (gmres_finish_pending) instead of here, and the
    // epilogue reads the iteration count on the device
    bool deferred = false;
    if (cluster) {
        GmresCtl c{};
        c.k = 1;
        c.max_iter = max_iter;
        c.tol = tol;
        c.norm_ref = norm_ref;
        c.inv_norm_ref = 1.0 / norm_ref;
        *s->h_ctl = c;
        GMI_CUDA_TRY(cudaMemcpyAsync(s->ctl, s->h_ctl, sizeof c, cudaMemcpyHostToDevice, st));
        GMI_TRY(cluster_gmres_launch(s, beta0, norm_ref, tol, max_iter));
        if (defer) {
            deferred = true;
            s->ctl_pending_nodes = 0;
        } else {
            GMI_CUDA_TRY(cudaMemcpyAsync(s->h_ctl, s->ctl, sizeof c, cudaMemcpyDeviceToHost, st));
            GMI_CUDA_TRY(cudaStreamSynchronize(st));
            if (!s->h_ctl->done) {
                set_last_error_msg("cluster GMRES solve ended without completion");
                return GMI_ERR_STATE;
            }
        }
    }
    if (cluster || s->use_graphs) {
      if (!cluster) {
        // the first step normalises w = r0 by beta0 into Q[:, 0]
        GMI_CUDA_TRY(cudaMemcpyAsync(s->st_scal + kNormOff, s->h_stage, sizeof(double), cudaMemcpyHostToDevice, st));
        GmresCtl c{};
        c.k = 1;
        c.done = 0;
        c.max_iter = max_iter;
        c.replays = 0;
        c.guard = 0;
        c.tol = tol;
        c.norm_ref = norm_ref;
        c.inv_norm_ref = 1.0 / norm_ref;
        *s->h_ctl = c;
        GMI_CUDA_TRY(cudaMemcpyAsync(s->ctl, s->h_ctl, sizeof c, cudaMemcpyHostToDevice, st));
        int batch = 4, replayed = 0;
        if (s->graph_loops[pidx]) {
            GMI_CUDA_TRY(cudaGraphLaunch(s->graph[pidx], st));
            if (defer) {
                deferred = true;
                s->ctl_pending_nodes = (long long)nodes;
            } else {
                GMI_CUDA_TRY(cudaMemcpyAsync(s->h_ctl, s->ctl, sizeof c, cudaMemcpyDeviceToHost, st));
                GMI_CUDA_TRY(cudaStreamSynchronize(st));
                s->ctx->launches += (long long)s->h_ctl->guard * (long long)nodes;
                if (!s->h_ctl->done) {
                    set_last_error_msg("GMRES loop ended without completion");
                    return GMI_ERR_STATE;
                }
            }
        }
        for (; !s->graph_loops[pidx];) {
            for (int b = 0; b < batch; ++b) GMI_CUDA_TRY(cudaGraphLaunch(s->graph[pidx], st));
            replayed += batch;
            s->ctx->launches += (long long)batch * (long long)nodes;
            GMI_CUDA_TRY(cudaMemcpyAsync(s->h_ctl, s->ctl, sizeof c, cudaMemcpyDeviceToHost, st));
            GMI_CUDA_TRY(cudaStreamSynchronize(st));
            if (s->h_ctl->done) break;
            if (replayed > max_iter + 64) {
                set_last_error_msg("GMRES control block never signalled completion");
                return GMI_ERR_STATE;
            }
            batch = batch * 2 < 32 ? batch * 2 : 32;
        }
      }
        if (deferred) {
            backsolve_warp_kernel<<<1, 32, 0, st>>>(s->H, ldh, s->beta, 0, s->yv, s->ctl);
            combine_kernel<<<grid_for(n, 64), 64, 0, st>>>(s->Q, ld, s->yv, 0, n, s->tmp, s->ctl);
        } else {
            if (!std::isfinite(s->h_ctl->resid)) {
                set_last_error_msg("GMRES produced a non-finite residual");
                return GMI_ERR_NONFINITE;
            }
            s->gm_resid = s->h_ctl->resid;
            const int iter = s->h_ctl->k;
            backsolve_warp_kernel<<<1, 32, 0, st>>>(s->H, ldh, s->beta, iter, s->yv, nullptr);
            combine_kernel<<<grid_for(n, 64), 64, 0, st>>>(s->Q, ld, s->yv, iter, n, s->tmp, nullptr);
            *iters_out = iter;
        }
        GMI_TRY(launched(s, 2));
        GMI_TRY(apply_preconditioner(s, s->tmp, s->z));
        axpby_kernel<<<grid_for(n), 256, 0, st>>>(n, 1.0, s->soln, 1.0, s->z, s->soln);
        GMI_TRY(launched(s));
        if (deferred) {
            GMI_CUDA_TRY(cudaMemcpyAsync(s->h_ctl, s->ctl, sizeof(GmresCtl), cudaMemcpyDeviceToHost, st));
            s->ctl_pending = true;
        }
        return GMI_OK;
    }
    GMI_CUDA_TRY(cudaMemcpyAsync(s->scal, s->h_stage, sizeof(double), cudaMemcpyHostToDevice, st));
    scale_kernel<<<grid_for(n), 256, 0, st>>>(n, s->w, s->scal, s->Q);
    GMI_TRY(launched(s));
    for (int iter = 1; iter <= max_iter; ++iter) {
        GMI_TRY(apply_preconditioner(s, s->Q + ld * (iter - 1), s->z));
        GMI_TRY(system_matrix_mult(s, s->z, s->w));
        double *Hcol = s->H + (size_t)ldh * (iter - 1);
        GMI_TRY(orthonormalise(s, s->w, iter, Hcol));
        givens_kernel<<<1, 1, 0, st>>>(s->H, ldh, s->beta, s->cs, s->sn, iter, norm_ref, s->scal + 1);
        GMI_TRY(launched(s));
        double resid;
        GMI_TRY(read_scalar(s, s->scal + 1, &resid));
        if (!std::isfinite(resid)) {
            set_last_error_msg("GMRES produced a non-finite residual");
            return GMI_ERR_NONFINITE;
        }
        if (resid <= tol || iter == max_iter) {
            s->gm_resid = resid;
            backsolve_warp_kernel<<<1, 32, 0, st>>>(s->H, ldh, s->beta, iter, s->yv, nullptr);
            combine_kernel<<<grid_for(n, 64), 64, 0, st>>>(s->Q, ld, s->yv, iter, n, s->tmp, nullptr);
            GMI_TRY(launched(s, 2));
            GMI_TRY(apply_preconditioner(s, s->tmp, s->z));
            axpby_kernel<<<grid_for(n), 256, 0, st>>>(n, 1.0, s->soln, 1.0, s->z, s->soln);
            GMI_TRY(launched(s));
            *iters_out = iter;
            return GMI_OK;
        }
    }
    return GMI_OK;
}

// The checks of a deferred GMRES solve (gmres_run with defer), once the
// stream has been synchronised: completion, a finite residual, and its
// iteration count added to *iters.
static gmi_status gmres_finish_pending(gmi_solver *s, int *iters)
{
    if (!s->ctl_pending) return GMI_OK;
    s->ctl_pending = false;
    s->ctx->launches += (long long)s->h_ctl->guard * s->ctl_pending_nodes;
    if (!s->h_ctl->done) {
        set_last_error_msg("GMRES solve ended without completion");
        return GMI_ERR_STATE;
    }
    if (!std::isfinite(s->h_ctl->resid)) {
        set_last_error_msg("GMRES produced a non-finite residual");
        return GMI_ERR_NONFINITE;
    }
    s->gm_resid = s->h_ctl->resid;
    *iters += s->h_ctl->k;
    return GMI_OK;
}

static gmi_status store_solution(gmi_solver *s)
{
    const int nb = s->B;
    cudaStream_t st = s->ctx->stream;
    GMI_CUDA_TRY(cudaMemcpyAsync(s->f_blobs, s->soln, 3 * (size_t)nb * sizeof(double), cudaMemcpyDeviceToDevice, st));
    GMI_CUDA_TRY(cudaMemcpyAsync(s->v_bodies, s->soln + 3 * nb, 6 * (size_t)s->W * sizeof(double),
                                 cudaMemcpyDeviceToDevice, st));
    return GMI_OK;
}

// solve_linear_system (mobility_solver.cpp:970-1354) warm started from
// (f_blobs, v_bodies); the right-hand side must be in s->rhs.
//
// FP64 context: the reference algorithm as is.
// FP32C context: mixed-precision iterative refinement.  The residual
// b - A x is formed with the FP64-grade operator (the blob-blob sum in
// double-float arithmetic, the body terms in FP64); each correction solves
// A d = r by GMRES with the FP32C operator (FP64 Arnoldi, Givens and
// vectors) to the relative tolerance that would meet the target in one pass
// (kInnerMargin times it; GMI_INNER_MARGIN overrides), but not below
// kInnerTol; x += d.  This converges to the FP64 solution at the requested
// tolerance, which GMRES on the FP32C operator alone cannot (its answer is
// off by cond(A) times the operator's rounding).  kInnerTol sits somewhat
// below that rounding (~3e-7 of |A d|): GMRES's own residual estimate keeps
// falling there, and the deeper inner solves save more refinement restarts
// than they cost (the fewest total iterations on the 962- and 16,896-particle
// swimmers among floors from 1e-6 to 2e-8; GMI_INNER_TOL overrides it).  The
// margin is 1: on the same swimmers a margin of 0.3, 0.5, 0.7 or 1 gave the
// same velocities to the Broyden tolerance, and 1 the fewest GMRES
// iterations (225 against 267 per step on the 962-particle swimmer; the
// plain FP64 solve takes 210).  The iteration count returned is the sum of
// inner iterations.
static constexpr double kInnerTol = 1e-7;
static constexpr double kInnerMargin = 1.0;
static constexpr int kMaxRefinements = 12;

static gmi_status solve_linear_system(gmi_solver *s, int *iters_out)
{
    const int n = s->n, nb = s->B;
    const size_t ld = (size_t)n;
    const double tol = s->cfg.linear_tol;
    cudaStream_t st = s->ctx->stream;
    *iters_out = 0;
    s->last_rel_resid = 0.0;  // a zero right-hand side is solved exactly
    s->last_iters = 0;
    const int prec = s->ctx->precision;
    auto check_rhs = [&](double norm) -> gmi_status {
        if (!std::isfinite(norm)) {
            set_last_error_msg("non-finite right-hand side in the linear solve");
            return GMI_ERR_NONFINITE;
        }
        return GMI_OK;
    };
    GMI_TRY(device_norm(s, s->rhs, n));
    double norm_rhs = 0.0;
    if (prec == GMI_FP64) {
        GMI_TRY(read_scalar(s, s->scal, &norm_rhs));
        GMI_TRY(check_rhs(norm_rhs));
        if (norm_rhs == 0.0) {
            GMI_CUDA_TRY(cudaMemsetAsync(s->f_blobs, 0, 3 * (size_t)nb * sizeof(double), st));
            GMI_CUDA_TRY(cudaMemsetAsync(s->v_bodies, 0, 6 * (size_t)s->W * sizeof(double), st));
            return GMI_OK;
        }
    } else {
        // the mixed path reads ||b|| together with its first residual norm
        // (one host round trip for both), from scal[2]
        GMI_CUDA_TRY(cudaMemcpyAsync(s->scal + 2, s->scal, sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    GMI_CUDA_TRY(cudaMemcpyAsync(s->soln, s->f_blobs, 3 * (size_t)nb * sizeof(double), cudaMemcpyDeviceToDevice, st));
    GMI_CUDA_TRY(cudaMemcpyAsync(s->soln + 3 * nb, s->v_bodies, 6 * (size_t)s->W * sizeof(double),
                                 cudaMemcpyDeviceToDevice, st));
    if (prec == GMI_FP64) {
        int iters = 0;
        GMI_TRY(gmres_run(s, norm_rhs, norm_rhs, tol, true, false, &iters));
        *iters_out = iters;
        s->last_rel_resid = s->gm_resid;
        s->last_iters = iters;
        return store_solution(s);
    }
    // Mixed-precision refinement.  The residual of the warm start is formed
    // with the FP64-grade operator; after each correction delta (A delta ~ r,
    // so |A delta| ~ |r|) it is updated as r -= A delta with the FP32C
    // operator, whose error (~3e-7 |A delta|, i.e. ~3e-7 of a residual that is
    // already small against |b|) stays far below the tolerance.
    GMI_CUDA_TRY(cudaMemcpyAsync(s->b64, s->rhs, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
    int total = 0;
    gmi_status status = GMI_OK;
    // the blob-blob sum of this residual in double-float (FP64-grade, on the
    // FP32 pipe); GMI_REFINE_DF=0 takes the FP64 kernel instead
    const char *floor_env = std::getenv("GMI_INNER_TOL");  // the floor of the inner tolerance
    const double inner_floor = floor_env ? std::atof(floor_env) : kInnerTol;
    const char *margin_env = std::getenv("GMI_INNER_MARGIN");  // the inner target's margin
    const double inner_margin = margin_env ? std::atof(margin_env) : kInnerMargin;
    const char *df_env = std::getenv("GMI_REFINE_DF");
    s->ctx->precision = (df_env && df_env[0] == '0') ? GMI_FP64 : GMI_DF64;
    status = system_matrix_mult(s, s->soln, s->tmp);
    s->ctx->precision = prec;
    if (status != GMI_OK) return status;
    axpby_kernel<<<grid_for(n), 256, 0, st>>>(n, 1.0, s->b64, -1.0, s->tmp, s->rhs);
    GMI_TRY(launched(s));
    for (int outer = 0; outer < kMaxRefinements; ++outer) {
        if (outer > 0) {
            // r -= A delta (delta in s->z, the last correction)
            GMI_TRY(system_matrix_mult(s, s->z, s->tmp));
            axpby_kernel<<<grid_for(n), 256, 0, st>>>(n, 1.0, s->rhs, -1.0, s->tmp, s->rhs);
            GMI_TRY(launched(s));
        }
        GMI_TRY(device_norm(s, s->rhs, n));
        double beta;
        if (outer == 0) {  // ||r|| and ||b|| in one read
            GMI_CUDA_TRY(cudaMemcpyAsync(s->h_stage, s->scal, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
            GMI_CUDA_TRY(cudaStreamSynchronize(st));
            beta = s->h_stage[0];
            norm_rhs = s->h_stage[2];
            GMI_TRY(check_rhs(norm_rhs));
            if (norm_rhs == 0.0) {
                GMI_CUDA_TRY(cudaMemcpyAsync(s->rhs, s->b64, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
                GMI_CUDA_TRY(cudaMemsetAsync(s->f_blobs, 0, 3 * (size_t)nb * sizeof(double), st));
                GMI_CUDA_TRY(cudaMemsetAsync(s->v_bodies, 0, 6 * (size_t)s->W * sizeof(double), st));
                return GMI_OK;
            }
        } else {
            GMI_TRY(read_scalar(s, s->scal, &beta));
        }
        GMI_TRY(gmres_finish_pending(s, &total));  // the previous correction's solve
        if (!std::isfinite(beta)) {
            set_last_error_msg("non-finite residual in the refinement loop");
            return GMI_ERR_NONFINITE;
        }
        s->last_rel_resid = beta / norm_rhs;
        if (beta <= tol * norm_rhs) break;
        if (outer == 0 && beta > norm_rhs) {  // reject a poor warm start, as the reference does
            GMI_CUDA_TRY(cudaMemsetAsync(s->soln, 0, ld * sizeof(double), st));
            GMI_CUDA_TRY(cudaMemcpyAsync(s->rhs, s->b64, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
            beta = norm_rhs;
        }
        GMI_CUDA_TRY(cudaMemcpyAsync(s->xacc, s->soln, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
        GMI_CUDA_TRY(cudaMemsetAsync(s->soln, 0, ld * sizeof(double), st));
        const double want = inner_margin * tol * norm_rhs / beta;
        const double inner_tol = want > inner_floor ? want : inner_floor;
        int iters = 0;
        GMI_TRY(gmres_run(s, beta, beta, inner_tol, false, true, &iters, true));
        total += iters;  // zero when the solve is deferred (counted at the next synchronisation)
        // keep the correction for the residual update, then accumulate it
        GMI_CUDA_TRY(cudaMemcpyAsync(s->z, s->soln, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
        axpby_kernel<<<grid_for(n), 256, 0, st>>>(n, 1.0, s->xacc, 1.0, s->soln, s->soln);
        GMI_TRY(launched(s));
    }
    if (s->ctl_pending) {  // the refinement cap ended the loop after a solve
        GMI_CUDA_TRY(cudaStreamSynchronize(st));
        GMI_TRY(gmres_finish_pending(s, &total));
        // the residual after that last correction (the loop had no turn left
        // to check it): r -= A delta, as at the top of the loop
        GMI_TRY(system_matrix_mult(s, s->z, s->tmp));
        axpby_kernel<<<grid_for(n), 256, 0, st>>>(n, 1.0, s->rhs, -1.0, s->tmp, s->rhs);
        GMI_TRY(launched(s));
        GMI_TRY(device_norm(s, s->rhs, n));
        double beta = 0.0;
        GMI_TRY(read_scalar(s, s->scal, &beta));
        s->last_rel_resid = beta / norm_rhs;
    }
    GMI_CUDA_TRY(cudaMemcpyAsync(s->rhs, s->b64, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
    *iters_out = total;
    s->last_iters = total;
    return store_solution(s);
}

// read_positions_and_forces (mobility_solver.cpp:132-192) minus the host
// copies: segment arrays already on the device, body state staged.
static gmi_status positions_and_barrier(gmi_solver *s)
{
    gmi_context *ctx = s->ctx;
    GMI_TRY(prepare_bodies(s));
    if (s->B > 0) {
        blob_positions_kernel<<<grid_for(s->B), 256, 0, ctx->stream>>>(s->W, s->cfg.nblob, s->body_x, s->R, s->refs,
                                                                        s->x_blobs);
        GMI_TRY(launched(s));
    }
    BarrierLaunch a{};
    a.f_segs = s->f_segs;
    a.f_blobs_rep = s->f_rep;
    a.xs = s->x_segs;
    a.xb = s->x_blobs;
    a.S = s->S;
    a.B = s->B;
    a.start_seg = 0;
    a.num_segs = s->S;
    a.start_blob = 0;
    a.num_blobs = s->B;
    a.nseg = s->cfg.nseg;
    a.rseg = s->cfg.rseg;
    a.rblob = s->cfg.rblob;
    a.scale = s->cfg.repulsive_force_factor * s->cfg.end_force_magnitude;
    a.wall = s->cfg.wall;
    return launch_barrier(ctx, a);
}

static gmi_status stage_bodies(gmi_solver *s, const double *bx, const double *bq)
{
    const int W = s->W;
    if (W == 0) return GMI_OK;
    std::memcpy(s->h_stage + 8, bx, 3 * W * sizeof(double));
    std::memcpy(s->h_stage + 8 + 3 * W, bq, 4 * W * sizeof(double));
    GMI_CUDA_TRY(cudaMemcpyAsync(s->body_x, s->h_stage + 8, 3 * W * sizeof(double), cudaMemcpyHostToDevice,
                                 s->ctx->stream));
    GMI_CUDA_TRY(cudaMemcpyAsync(s->body_q, s->h_stage + 8 + 3 * W, 4 * W * sizeof(double), cudaMemcpyHostToDevice,
                                 s->ctx->stream));
    // the staging area is reused by the next call: make sure these copies have read it
    GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    return GMI_OK;
}

gmi_status solver_place_blobs(gmi_solver *s, const double *body_x, const double *body_q)
{
    GMI_TRY(stage_bodies(s, body_x, body_q));
    GMI_TRY(prepare_bodies(s));
    if (s->B > 0) {
        blob_positions_kernel<<<grid_for(s->B), 256, 0, s->ctx->stream>>>(s->W, s->cfg.nblob, s->body_x, s->R,
                                                                           s->refs, s->x_blobs);
        GMI_TRY(launched(s));
    }
    return GMI_OK;
}


static gmi_status seg_pair(gmi_solver *s, int kind)
{
    gmi_context *ctx = s->ctx;
    PairConsts k;
    if (kind == kSS) {
        GMI_TRY(pack_records(ctx, s->x_segs, s->f_segs, 6, s->S, ctx->rec_src));
        fill_consts(k, s->cfg.rseg, s->cfg.rseg, s->cfg.rseg, s->cfg.mu);
        return launch_pair(ctx, s->cfg.wall ? kSSWall : kSS, ctx->rec_src.ptr, 0, s->S, ctx->rec_src.ptr, s->S, k,
                           s->v_segs, 0);
    }
    if (kind == kBS) {
        GMI_TRY(pack_records(ctx, s->x_blobs, nullptr, 0, s->B, ctx->rec_tgt));
        GMI_TRY(pack_records(ctx, s->x_segs, s->f_segs, 6, s->S, ctx->rec_src));
        fill_consts(k, s->cfg.rseg, s->cfg.rseg, s->cfg.rblob, s->cfg.mu);
        return launch_pair(ctx, kBS, ctx->rec_tgt.ptr, 0, s->B, ctx->rec_src.ptr, s->S, k, s->v_blobs, 0);
    }
    if (kind == kSB) {
        GMI_TRY(pack_records(ctx, s->x_segs, nullptr, 0, s->S, ctx->rec_tgt));
        GMI_TRY(pack_records(ctx, s->x_blobs, s->f_blobs, 3, s->B, ctx->rec_src));
        fill_consts(k, s->cfg.rseg, s->cfg.rseg, s->cfg.rblob, s->cfg.mu);
        return launch_pair(ctx, kSB, ctx->rec_tgt.ptr, 0, s->S, ctx->rec_src.ptr, s->B, k, s->v_segs, 1);
    }
    GMI_TRY(pack_records(ctx, s->x_blobs, s->f_blobs, 3, s->B, ctx->rec_src));
    fill_consts(k, s->cfg.rblob, s->cfg.rblob, s->cfg.rblob, s->cfg.mu);
    return launch_pair(ctx, kBB, ctx->rec_src.ptr, 0, s->B, ctx->rec_src.ptr, s->B, k, s->v_blobs, 0);
}

static gmi_status h2d(gmi_solver *s, double *d, const double *h, size_t count)
{
    if (count == 0) return GMI_OK;
    GMI_CUDA_TRY(cudaMemcpyAsync(d, h, count * sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream));
    return GMI_OK;
}

static gmi_status d2h(gmi_solver *s, double *h, const double *d, size_t count)
{
    if (count == 0) return GMI_OK;
    GMI_CUDA_TRY(cudaMemcpyAsync(h, d, count * sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream));
    return GMI_OK;
}

// 6x6 inverse by Gauss-Jordan with partial pivoting (column-major), the
// reference's matrix::invert (LAPACK dgetrf + dgetri, matrix.cpp:538-571).
static bool invert6(const double *A, double *Ainv)
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
            if (std::fabs(M[r][c]) > std::fabs(M[p][c])) p = r;
        if (M[p][c] == 0.0) return false;
        if (p != c)
            for (int j = 0; j < 12; ++j) std::swap(M[c][j], M[p][j]);
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
        for (int j = 0; j < 6; ++j) Ainv[i + 6 * j] = M[i][6 + j];
    return true;
}

}  // namespace gmi

namespace gmi {

gmi_status solver_compute_velocities_device(gmi_solver *s, int *iters)
{
    const int W = s->W, B = s->B;
    cudaStream_t st = s->ctx->stream;
    *iters = 0;
    if (s->cfg.wall) {
        GMI_TRY(positions_and_barrier(s));
        return seg_pair(s, kSS);
    }
    GMI_TRY(positions_and_barrier(s));
    if (B > 0) {
        GMI_TRY(kt_sums(s, s->f_rep));
        add_vec_kernel<<<grid_for(6 * W), 256, 0, st>>>(6 * W, s->sums, s->body_f);
        GMI_TRY(launched(s));
    }
    GMI_TRY(seg_pair(s, kSS));
    GMI_TRY(seg_pair(s, kBS));
    assemble_rhs_kernel<<<grid_for(s->n), 256, 0, st>>>(3 * B, 6 * W, s->v_blobs, s->body_f, s->rhs);
    GMI_TRY(launched(s));
    GMI_TRY(solve_linear_system(s, iters));
    return seg_pair(s, kSB);
}

}  // namespace gmi

using namespace gmi;

#define GMI_ARG_CHECK(cond, msg)     \
    do {                             \
        if (!(cond)) {               \
            set_last_error_msg(msg); \
            return GMI_ERR_ARG;      \
        }                            \
    } while (0)

extern "C" {

gmi_status gmi_solver_destroy(gmi_solver *s)
{
    if (s == nullptr) return GMI_OK;
    if (s->ctx) {
        cudaSetDevice(s->ctx->device);
        cudaStreamSynchronize(s->ctx->stream);
    }
    for (int g = 0; g < 2; ++g)
        if (s->graph[g]) cudaGraphExecDestroy(s->graph[g]);
    prescribed_release(s);
    if (s->h_ctl) host_free(s->h_ctl);
    for (void *p : s->allocs) dev_free(p);
    double *hp[] = {s->h.v_segs_host, s->h.v_blobs_host, s->h.x_segs_host, s->h.x_blobs_host, s->h.f_segs_host,
                    s->h.f_blobs_host, s->h.f_blobs_repulsion_host, s->h_stage};
    for (double *p : hp)
        if (p) host_free(p);
    if (s->ctx) gmi_context_destroy(s->ctx);
    delete s;
    return GMI_OK;
}

gmi_status gmi_solver_create(const gmi_solver_config *cfg, gmi_solver **out)
{
    GMI_ARG_CHECK(cfg && out, "gmi_solver_create: null argument");
    *out = nullptr;
    GMI_ARG_CHECK(cfg->nswim >= 1 && cfg->nfil >= 0 && cfg->nseg >= 1 && cfg->nblob >= 0,
                  "gmi_solver_create: sizes must satisfy nswim >= 1, nfil >= 0, nseg >= 1, nblob >= 0");
    GMI_ARG_CHECK(cfg->mu > 0 && cfg->rseg > 0 && cfg->rblob > 0, "gmi_solver_create: mu and radii must be positive");
    GMI_ARG_CHECK(!cfg->wall || (cfg->nblob == 0 && cfg->nswim == 1),
                  "gmi_solver_create: the wall configuration has one swimmer and no blobs (config.hpp:222-226)");
    GMI_ARG_CHECK(cfg->wall || cfg->nblob > 0,
                  "gmi_solver_create: free-swimming bodies need blobs (the linear system is empty otherwise)");
    GMI_ARG_CHECK(cfg->precision == GMI_FP64 || cfg->precision == GMI_FP32C, "gmi_solver_create: bad precision");
    gmi_solver *s = new (std::nothrow) gmi_solver();
    GMI_ARG_CHECK(s != nullptr, "gmi_solver_create: out of host memory");
    s->cfg = *cfg;
    if (s->cfg.max_linear_iter <= 0) s->cfg.max_linear_iter = 150;
    if (s->cfg.max_linear_iter > kFMaxK - 1) {
        set_last_error_msg("gmi_solver_create: max_linear_iter above the supported 159");
        delete s;
        return GMI_ERR_ARG;
    }
    if (s->cfg.linear_tol <= 0) s->cfg.linear_tol = 1e-10;
    gmi_status st = gmi_context_create(cfg->device, &s->ctx);
    if (st != GMI_OK) {
        gmi_solver_destroy(s);
        return st;
    }
    s->ctx->precision = cfg->precision;
    s->W = cfg->nswim;
    s->S = cfg->nswim * cfg->nfil * cfg->nseg;
    s->B = cfg->nswim * cfg->nblob;
    s->n = cfg->wall ? 0 : 3 * s->B + 6 * s->W;
    s->m = s->cfg.max_linear_iter;
    const size_t S = s->S, B = s->B, W = s->W, n = s->n, m = s->m;
#define TRY_OR_DIE(expr)            \
    do {                            \
        st = (expr);                \
        if (st != GMI_OK) {         \
            gmi_solver_destroy(s);  \
            return st;              \
        }                           \
    } while (0)
    TRY_OR_DIE(halloc(&s->h.v_segs_host, 6 * S));
    TRY_OR_DIE(halloc(&s->h.v_blobs_host, 3 * B));
    TRY_OR_DIE(halloc(&s->h.x_segs_host, 3 * S));
    TRY_OR_DIE(halloc(&s->h.x_blobs_host, 3 * B));
    TRY_OR_DIE(halloc(&s->h.f_segs_host, 6 * S));
    TRY_OR_DIE(halloc(&s->h.f_blobs_host, 3 * B));
    TRY_OR_DIE(halloc(&s->h.f_blobs_repulsion_host, 3 * B));
    TRY_OR_DIE(halloc(&s->h_stage, 16 + 16 * W));
    TRY_OR_DIE(dalloc(s, &s->x_segs, 3 * S));
    TRY_OR_DIE(dalloc(s, &s->f_segs, 6 * S));
    TRY_OR_DIE(dalloc(s, &s->v_segs, 6 * S));
    TRY_OR_DIE(dalloc(s, &s->x_blobs, 3 * B));
    TRY_OR_DIE(dalloc(s, &s->f_blobs, 3 * B));
    TRY_OR_DIE(dalloc(s, &s->v_blobs, 3 * B));
    TRY_OR_DIE(dalloc(s, &s->f_rep, 3 * B));
    TRY_OR_DIE(dalloc(s, &s->body_x, 3 * W));
    TRY_OR_DIE(dalloc(s, &s->body_q, 4 * W));
    TRY_OR_DIE(dalloc(s, &s->body_f, 6 * W));
    TRY_OR_DIE(dalloc(s, &s->v_bodies, 6 * W));
    TRY_OR_DIE(dalloc(s, &s->R, 9 * W));
    TRY_OR_DIE(dalloc(s, &s->ktk_ref, 36));
    TRY_OR_DIE(dalloc(s, &s->mob_ref, 36));
    TRY_OR_DIE(dalloc(s, &s->ktk_rot, 36 * W));
    TRY_OR_DIE(dalloc(s, &s->mob_rot, 36 * W));
    TRY_OR_DIE(dalloc(s, &s->ktkf_ref, 36));
    TRY_OR_DIE(dalloc(s, &s->ktkf_rot, 36 * W));
    TRY_OR_DIE(dalloc(s, &s->refs, 3 * (size_t)cfg->nblob));
    TRY_OR_DIE(dalloc(s, &s->sums, 6 * W));
    TRY_OR_DIE(dalloc(s, &s->kt_part, 6 * W * (size_t)((cfg->nblob + kKtBlobs - 1) / kKtBlobs)));
    TRY_OR_DIE(dalloc(s, &s->scal, 8));
    double *aux_mem = nullptr;
    TRY_OR_DIE(dalloc(s, &aux_mem, 4));  // zeroed: tickets of norm_kernel and kt_kernel
    s->aux_tickets = reinterpret_cast<int *>(aux_mem);
    if (n > 0) {
        TRY_OR_DIE(dalloc(s, &s->rhs, n));
        TRY_OR_DIE(dalloc(s, &s->soln, n));
        TRY_OR_DIE(dalloc(s, &s->Q, n * (m + 1)));
        TRY_OR_DIE(dalloc(s, &s->H, (m + 1) * (m + 1)));
        TRY_OR_DIE(dalloc(s, &s->beta, m + 1));
        TRY_OR_DIE(dalloc(s, &s->cs, m));
        TRY_OR_DIE(dalloc(s, &s->sn, m));
        TRY_OR_DIE(dalloc(s, &s->yv, m + 1));
        TRY_OR_DIE(dalloc(s, &s->z, n));
        TRY_OR_DIE(dalloc(s, &s->w, n));
        TRY_OR_DIE(dalloc(s, &s->tmp, n));
        TRY_OR_DIE(dalloc(s, &s->b64, n));
        TRY_OR_DIE(dalloc(s, &s->xacc, n));
        TRY_OR_DIE(dalloc(s, &s->mbb, 3 * B));
        // partial serves the host loop's dot partials (two arrays of m + 1
        // columns over kChunkRows chunks) and the graph step's workspace.
        const StepLayout L = step_layout((int)n, cfg->nblob, (int)W);
        s->partial_count = std::max<size_t>(2 * ((size_t)nchunks_of((int)n) + n / 1024 + 1) * (m + 1), L.doubles);
        TRY_OR_DIE(dalloc(s, &s->partial, s->partial_count));
        TRY_OR_DIE(dalloc(s, &s->st_scal, kStepScalars));
        double *tk_mem = nullptr;
        s->st_ticket_count = L.tickets;
        TRY_OR_DIE(dalloc(s, &tk_mem, (L.tickets + 1) / 2));
        s->st_tickets = reinterpret_cast<int *>(tk_mem);
        double *ctl_mem = nullptr, *rec_mem = nullptr, *part_mem = nullptr;
        TRY_OR_DIE(dalloc(s, &ctl_mem, 8));
        s->ctl = reinterpret_cast<GmresCtl *>(ctl_mem);
        TRY_OR_DIE(dalloc(s, &rec_mem, 12 * B));
        s->gm_rec = rec_mem;
        const size_t max_splits = (B + 127) / 128 + 1;
        TRY_OR_DIE(dalloc(s, &part_mem, max_splits * 3 * B));
        s->gm_partial = part_mem;
        s->gm_partial_bytes = max_splits * 3 * B * sizeof(double);
        if (host_alloc(&s->h_ctl, sizeof(GmresCtl)) != cudaSuccess) {
            s->h_ctl = nullptr;
            set_last_error_msg("gmi_solver_create: pinned allocation failed");
            gmi_solver_destroy(s);
            return GMI_ERR_CUDA;
        }
    }
    // reference matrices start as identities (mobility_solver.cpp:85-88)
    double I6[36] = {0};
    for (int i = 0; i < 6; ++i) I6[i + 6 * i] = 1.0;
    TRY_OR_DIE(gmi_solver_set_body_reference_matrices(s, I6, I6));
    st = context_check_device_errors(s->ctx);
    if (st != GMI_OK) {
        gmi_solver_destroy(s);
        return st;
    }
#undef TRY_OR_DIE
    *out = s;
    return GMI_OK;
}

gmi_status gmi_solver_host_arrays(gmi_solver *s, gmi_host_arrays *out)
{
    GMI_ARG_CHECK(s && out, "gmi_solver_host_arrays: null argument");
    *out = s->h;
    return GMI_OK;
}

gmi_context *gmi_solver_context(gmi_solver *s) { return s ? s->ctx : nullptr; }

#define SOLVER_ENTRY(s)                                          \
    GMI_ARG_CHECK((s) != nullptr, "null solver");                \
    GMI_CUDA_TRY(cudaSetDevice((s)->ctx->device))

gmi_status gmi_solver_copy_segment_positions_to_device(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return h2d(s, s->x_segs, s->h.x_segs_host, 3 * (size_t)s->S);
}
gmi_status gmi_solver_copy_segment_forces_to_device(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return h2d(s, s->f_segs, s->h.f_segs_host, 6 * (size_t)s->S);
}
gmi_status gmi_solver_copy_blob_positions_to_device(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return h2d(s, s->x_blobs, s->h.x_blobs_host, 3 * (size_t)s->B);
}
gmi_status gmi_solver_copy_blob_forces_to_device(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return h2d(s, s->f_blobs, s->h.f_blobs_host, 3 * (size_t)s->B);
}
gmi_status gmi_solver_copy_interparticle_blob_forces_to_host(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return d2h(s, s->h.f_blobs_repulsion_host, s->f_rep, 3 * (size_t)s->B);
}
gmi_status gmi_solver_copy_blob_velocities_to_host(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return d2h(s, s->h.v_blobs_host, s->v_blobs, 3 * (size_t)s->B);
}
gmi_status gmi_solver_copy_segment_velocities_to_host(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return d2h(s, s->h.v_segs_host, s->v_segs, 6 * (size_t)s->S);
}
gmi_status gmi_solver_apply_interparticle_forces(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    BarrierLaunch a{};
    a.f_segs = s->f_segs;
    a.f_blobs_rep = s->f_rep;
    a.xs = s->x_segs;
    a.xb = s->x_blobs;
    a.S = s->S;
    a.B = s->B;
    a.num_segs = s->S;
    a.num_blobs = s->B;
    a.nseg = s->cfg.nseg;
    a.rseg = s->cfg.rseg;
    a.rblob = s->cfg.rblob;
    a.scale = s->cfg.repulsive_force_factor * s->cfg.end_force_magnitude;
    a.wall = s->cfg.wall;
    return launch_barrier(s->ctx, a);
}
gmi_status gmi_solver_wait_for_device(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return context_check_device_errors(s->ctx);
}
gmi_status gmi_solver_evaluate_segment_segment_mobility(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return seg_pair(s, kSS);
}
gmi_status gmi_solver_evaluate_segment_blob_mobility(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return seg_pair(s, kSB);
}
gmi_status gmi_solver_evaluate_blob_blob_mobility(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return seg_pair(s, kBB);
}
gmi_status gmi_solver_evaluate_blob_segment_mobility(gmi_solver *s)
{
    SOLVER_ENTRY(s);
    return seg_pair(s, kBS);
}

gmi_status gmi_solver_set_blob_references(gmi_solver *s, const double *refs)
{
    SOLVER_ENTRY(s);
    const int nblob = s->cfg.nblob;
    GMI_ARG_CHECK(nblob == 0 || refs != nullptr, "gmi_solver_set_blob_references: null references");
    if (nblob > 0) {
        GMI_CUDA_TRY(cudaMemcpyAsync(s->refs, refs, 3 * (size_t)nblob * sizeof(double), cudaMemcpyHostToDevice,
                                     s->ctx->stream));
    }
    double KTK[36];
    gmi::ktk_from_refs(refs, nblob, KTK);
    GMI_CUDA_TRY(cudaMemcpyAsync(s->ktkf_ref, KTK, sizeof KTK, cudaMemcpyHostToDevice, s->ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));  // KTK is a local
    s->refs_set = true;
    return GMI_OK;
}

gmi_status gmi_solver_set_body_reference_matrices(gmi_solver *s, const double *ktkinv, const double *mob)
{
    SOLVER_ENTRY(s);
    GMI_ARG_CHECK(ktkinv && mob, "gmi_solver_set_body_reference_matrices: null argument");
    // ordered on the solver stream: the kernels that rotate these matrices
    // (prepare_bodies) run on it; the legacy default stream would not be
    // ordered with a non-blocking solver stream
    GMI_CUDA_TRY(cudaMemcpyAsync(s->ktk_ref, ktkinv, 36 * sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream));
    GMI_CUDA_TRY(cudaMemcpyAsync(s->mob_ref, mob, 36 * sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));  // the caller's arrays may go away
    return GMI_OK;
}

gmi_status gmi_solver_get_v_bodies(gmi_solver *s, double *v)
{
    SOLVER_ENTRY(s);
    GMI_ARG_CHECK(v != nullptr, "gmi_solver_get_v_bodies: null output");
    GMI_CUDA_TRY(cudaMemcpyAsync(v, s->v_bodies, 6 * (size_t)s->W * sizeof(double), cudaMemcpyDeviceToHost,
                                 s->ctx->stream));
    return context_check_device_errors(s->ctx);
}

gmi_status gmi_solver_set_v_bodies(gmi_solver *s, const double *v)
{
    SOLVER_ENTRY(s);
    GMI_ARG_CHECK(v != nullptr, "gmi_solver_set_v_bodies: null input");
    GMI_CUDA_TRY(cudaMemcpyAsync(s->v_bodies, v, 6 * (size_t)s->W * sizeof(double), cudaMemcpyHostToDevice,
                                 s->ctx->stream));
    return context_check_device_errors(s->ctx);
}

gmi_status gmi_solver_compute_velocities(gmi_solver *s, const double *body_x, const double *body_q, double *body_f,
                                         int *num_gmres_iterations)
{
    SOLVER_ENTRY(s);
    const int W = s->W, S = s->S, B = s->B;
    GMI_ARG_CHECK(s->cfg.wall || (body_x && body_q && body_f), "gmi_solver_compute_velocities: null body state");
    GMI_ARG_CHECK(s->cfg.wall || B == 0 || s->refs_set,
                  "gmi_solver_compute_velocities: blob references not set (gmi_solver_set_blob_references)");
    int iters = 0;
    GMI_TRY(h2d(s, s->x_segs, s->h.x_segs_host, 3 * (size_t)S));
    GMI_TRY(h2d(s, s->f_segs, s->h.f_segs_host, 6 * (size_t)S));
    if (!s->cfg.wall) {
        GMI_TRY(stage_bodies(s, body_x, body_q));
        std::memcpy(s->h_stage + 8, body_f, 6 * W * sizeof(double));
        GMI_TRY(h2d(s, s->body_f, s->h_stage + 8, 6 * (size_t)W));
    }
    GMI_TRY(solver_compute_velocities_device(s, &iters));
    GMI_TRY(d2h(s, s->h.v_segs_host, s->v_segs, 6 * (size_t)S));
    if (!s->cfg.wall) {
        GMI_TRY(d2h(s, s->h.f_blobs_host, s->f_blobs, 3 * (size_t)B));
        GMI_TRY(d2h(s, s->h.x_blobs_host, s->x_blobs, 3 * (size_t)B));
        GMI_TRY(d2h(s, s->h.f_blobs_repulsion_host, s->f_rep, 3 * (size_t)B));
        GMI_TRY(d2h(s, s->h.v_blobs_host, s->v_blobs, 3 * (size_t)B));
        GMI_TRY(d2h(s, s->h_stage + 8, s->body_f, 6 * (size_t)W));
    }
    GMI_TRY(context_check_device_errors(s->ctx));
    if (!s->cfg.wall) std::memcpy(body_f, s->h_stage + 8, 6 * W * sizeof(double));
    if (num_gmres_iterations) *num_gmres_iterations = iters;
    if (s->strict && !s->cfg.wall && !(s->last_rel_resid <= s->cfg.linear_tol)) {
        set_last_error_msg("gmi_solver_compute_velocities: the linear solve stopped at its iteration cap above "
                           "the tolerance (results were written back; gmi_solver_last_linear_solve has the residual)");
        return GMI_ERR_NOT_CONVERGED;
    }
    return GMI_OK;
}

gmi_status gmi_solver_set_strict_convergence(gmi_solver *s, int strict)
{
    GMI_ARG_CHECK(s != nullptr, "gmi_solver_set_strict_convergence: null solver");
    s->strict = strict != 0;
    return GMI_OK;
}

gmi_status gmi_solver_last_linear_solve(const gmi_solver *s, int *iterations, double *relative_residual)
{
    GMI_ARG_CHECK(s != nullptr, "gmi_solver_last_linear_solve: null solver");
    if (iterations) *iterations = s->last_iters;
    if (relative_residual) *relative_residual = s->last_rel_resid;
    return GMI_OK;
}

gmi_status gmi_solver_make_body_reference_matrices(gmi_solver *s, const double *body_x, const double *body_q,
                                                   double *ktkinv_out, double *mob_out)
{
    SOLVER_ENTRY(s);
    GMI_ARG_CHECK(!s->cfg.wall, "gmi_solver_make_body_reference_matrices: not used with the wall configuration");
    GMI_ARG_CHECK(body_x && body_q, "gmi_solver_make_body_reference_matrices: null body state");
    GMI_ARG_CHECK(s->refs_set, "gmi_solver_make_body_reference_matrices: blob references not set");
    GMI_TRY(h2d(s, s->x_segs, s->h.x_segs_host, 3 * (size_t)s->S));
    GMI_TRY(h2d(s, s->f_segs, s->h.f_segs_host, 6 * (size_t)s->S));
    GMI_TRY(stage_bodies(s, body_x, body_q));
    return solver_make_body_reference_matrices_device(s, ktkinv_out, mob_out);
}

}  // extern "C"

namespace gmi {

gmi_status solver_make_body_reference_matrices_device(gmi_solver *s, double *ktkinv_out, double *mob_out)
{
    const int W = s->W, nblob = s->cfg.nblob;
    // (K^T K) from the references (mobility_solver.cpp:1697-1713), inverted on the host
    std::vector<double> refs(3 * (size_t)nblob);
    if (nblob > 0)
        GMI_CUDA_TRY(cudaMemcpyAsync(refs.data(), s->refs, refs.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                     s->ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    double KTK[36];
    ktk_from_refs(refs.data(), nblob, KTK);
    double KTKinv[36];
    if (!invert6(KTK, KTKinv)) {
        set_last_error_msg("K^T K is singular (are the blob references set?)");
        return GMI_ERR_NONFINITE;
    }
    double mob[36] = {0};
    for (int i = 0; i < 6; ++i) mob[i + 6 * i] = 1.0;
    GMI_TRY(gmi_solver_set_body_reference_matrices(s, KTKinv, mob));
    // all swimmers but the last moved far away (mobility_solver.cpp:1721-1731), restored after
    std::vector<double> bx0(3 * (size_t)W), bx;
    GMI_CUDA_TRY(cudaMemcpyAsync(bx0.data(), s->body_x, bx0.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                 s->ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    bx = bx0;
    const double shift = 1e10 * 2.2 * s->cfg.rseg * s->cfg.nseg;
    for (int n = 0; n < W - 1; ++n)
        for (int c = 0; c < 3; ++c) bx[3 * n + c] += shift;
    GMI_CUDA_TRY(cudaMemcpyAsync(s->body_x, bx.data(), bx.size() * sizeof(double), cudaMemcpyHostToDevice,
                                 s->ctx->stream));
    GMI_TRY(positions_and_barrier(s));
    for (int col = 0; col < 6; ++col) {
        GMI_CUDA_TRY(cudaMemsetAsync(s->rhs, 0, (size_t)s->n * sizeof(double), s->ctx->stream));
        s->h_stage[0] = -1.0;
        GMI_CUDA_TRY(cudaMemcpyAsync(s->rhs + (s->n - 1 - col), s->h_stage, sizeof(double), cudaMemcpyHostToDevice,
                                     s->ctx->stream));
        GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
        int iters = 0;
        GMI_TRY(solve_linear_system(s, &iters));
        GMI_CUDA_TRY(cudaMemcpyAsync(s->h_stage, s->v_bodies + 6 * (W - 1), 6 * sizeof(double),
                                     cudaMemcpyDeviceToHost, s->ctx->stream));
        GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
        for (int i = 0; i < 6; ++i) mob[i + 6 * (5 - col)] = s->h_stage[i];
        // the preconditioner of the next solve sees the updated column
        GMI_TRY(gmi_solver_set_body_reference_matrices(s, KTKinv, mob));
        GMI_TRY(prepare_bodies(s));
    }
    GMI_CUDA_TRY(cudaMemcpyAsync(s->body_x, bx0.data(), bx0.size() * sizeof(double), cudaMemcpyHostToDevice,
                                 s->ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    if (ktkinv_out) std::memcpy(ktkinv_out, KTKinv, sizeof KTKinv);
    if (mob_out) std::memcpy(mob_out, mob, sizeof mob);
    return context_check_device_errors(s->ctx);
}

}  // namespace gmi

