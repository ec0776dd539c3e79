// gmi_prescribed.cu -- mobility_solver::compute_velocities for cilia whose
// shapes are prescribed (CILIA_TYPE 3, mobility_solver.cpp:1362-1369), free
// bodies:
//
//   unknowns  x = [f_seg (3 per segment) | f_blob (3 per blob) | U (6 per body)
//                  | phase speeds (1 per filament, DYNAMIC_PHASE_EVOLUTION only)]
//   operator  (system_matrix_mult, mobility_solver.cpp:733-905)
//             seg:   M_ss f_seg + M_sb f_blob - (U + Omega x d_seg) [- phase_speed K]
//             blob:  M_bs f_seg + M_bb f_blob - (U + Omega x d_blob)
//             body:  -sum (f, d x f) over the body's segments and blobs
//             phase: -sum_k K_k . f_k over the filament's segments
//   rhs       (assemble_rhs, :211-310) with the phase speeds given: segment rows
//             phase_speed * vel_dir, the rest 0; with the phase speeds unknown:
//             phase rows -q (the generalised force of the beat at the
//             filament's phase, scaled by omega0 / 2 pi), the rest 0
//   precond.  (apply_preconditioner, :427-649) M ~ I / (6 pi mu a) per particle and
//             the body block through (K^T M^-1 K)^-1 (swimmer::make_precon_mat,
//             swimmer.cpp:929-1037), with the phase speeds unknown its Schur
//             complement form
// K is a filament's shape-velocity direction (vel_dir, 3 per segment).  All
// four pair sums run inside every GMRES iteration.  Segments carry no
// torques in this system (their forces are the unknowns).
#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "gmi_context.hpp"
#include "gmi_gmres.hpp"
#include "gmi_lie.cuh"
#include "gmi_pair_kernels.hpp"
#include "gmi_solver_device.cuh"
#include "gmi_solver_internal.hpp"


struct PrescribedWork {
    gmi::KrylovSpace K;
    int np = 0;
    bool dynamic = false;  // phase speeds among the unknowns
    double *vel_dir = nullptr, *phase = nullptr, *P6 = nullptr, *rhs = nullptr, *soln = nullptr, *f6 = nullptr;
    // phase speeds unknown: phases, natural frequencies, per filament
    // (|K|^2, sum K, sum d x K), the preconditioner's phase scratch, the
    // generalised-force table and the setter serial it was uploaded at
    double *phase_in = nullptr, *omega0 = nullptr, *fil7 = nullptr, *pph = nullptr, *table = nullptr;
    int ntable = 0;
    unsigned table_serial = 0;
    int *flag = nullptr;
};

namespace gmi {

namespace {

constexpr int kTpb = 256;

struct PSizes {
    int S, B, W, nseg_sw, nblob;  // nseg_sw: segments per swimmer
    int nseg, nfil;               // segments per filament, filaments per swimmer
    int F;                        // phase-speed unknowns: W * nfil, or 0 when the speeds are given
};

__device__ __forceinline__ void seg_arm(const PSizes &z, const double *xs, const double *bx, int m, int &sw,
                                        double *d)
{
    sw = m / z.nseg_sw;
    for (int c = 0; c < 3; ++c) d[c] = xs[3 * (size_t)m + c] - bx[3 * sw + c];
}
__device__ __forceinline__ void blob_arm(const PSizes &z, const double *R, const double *refs, int i, int &sw,
                                         double *d)
{
    sw = i / z.nblob;
    rot_apply(R + 9 * sw, refs + 3 * (i % z.nblob), d);
}

// CTA sum of N per-thread values in a fixed order; result valid in red[0..N) after the call
template <int N> __device__ void cta_sum(double *v, double (*red)[kTpb / 32])
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int e = 0; e < N; ++e) {
        const double t = warp_sum(v[e]);
        if (lane == 0) red[e][wid] = t;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double t = 0.0;
        for (int q = 0; q < kTpb / 32; ++q) t += red[threadIdx.x][q];
        red[threadIdx.x][0] = t;
    }
    __syncthreads();
}

// In-place inverse of a column-major 6x6 (Gauss-Jordan, partial pivoting);
// false if singular.
__device__ bool invert6(double *A)
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
        const double inv = 1.0 / M[c][c];
        for (int j = 0; j < 12; ++j) M[c][j] *= inv;
        for (int r = 0; r < 6; ++r) {
            if (r == c) continue;
            const double f = M[r][c];
            if (f != 0.0)
                for (int j = 0; j < 12; ++j) M[r][j] -= f * M[c][j];
        }
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) A[i + 6 * j] = M[i][6 + j];
    return true;
}

// Per filament f (one warp each): |K|^2, sum_k K_k and sum_k d_k x K_k, d_k
// the segment's arm from its body centre (swimmer::make_precon_mat,
// swimmer.cpp:974-1013, and the phase part of apply_preconditioner,
// mobility_solver.cpp:522-559, 566-597), stored as fil7[7 f + (0 | 1..3 | 4..6)].
__global__ void __launch_bounds__(kTpb) pk_fil_consts(PSizes z, const double *__restrict__ xs,
                                                      const double *__restrict__ bx,
                                                      const double *__restrict__ vel_dir, double *__restrict__ fil7)
{
    const int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (f >= z.F) return;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int k = lane; k < z.nseg; k += 32) {
        const int m = f * z.nseg + k;
        double d[3];
        int sw;
        seg_arm(z, xs, bx, m, sw, d);
        const double *K = vel_dir + 3 * (size_t)m;
        acc[0] += K[0] * K[0] + K[1] * K[1] + K[2] * K[2];
        for (int c = 0; c < 3; ++c) acc[1 + c] += K[c];
        acc[4] += d[1] * K[2] - d[2] * K[1];
        acc[5] += d[2] * K[0] - d[0] * K[2];
        acc[6] += d[0] * K[1] - d[1] * K[0];
    }
    for (int e = 0; e < 7; ++e) {
        const double t = warp_sum(acc[e]);
        if (lane == 0) fil7[7 * (size_t)f + e] = t;
    }
}

// (K^T M^-1 K)^-1 per swimmer, column-major (swimmer.cpp:929-1037):
// [[e I, sum m rc(d)], [-sum m rc(d), -sum m rc(d)^2]], e = sum of the
// mobility factors, rc the reference's rcross; with the phase speeds unknown
// (fil7 given) less m_seg C, C = sum over the swimmer's filaments of
// [[v1 v1^T, v1 v2^T], [v2 v1^T, v2 v2^T]] / |K|^2 (v1 = sum K, v2 = sum d x K);
// then inverted.
__global__ void __launch_bounds__(kTpb) pk_precon_mats(PSizes z, const double *__restrict__ xs,
                                                       const double *__restrict__ bx, const double *__restrict__ R,
                                                       const double *__restrict__ refs, double seg_mob,
                                                       double blob_mob, const double *__restrict__ fil7,
                                                       double *__restrict__ P6, int *flag)
{
    __shared__ double red[18][kTpb / 32];
    __shared__ double redc[27][kTpb / 32];
    const int n = blockIdx.x;
    double acc[18];
    for (int e = 0; e < 18; ++e) acc[e] = 0.0;
    for (int e = threadIdx.x; e < z.nseg_sw + z.nblob; e += kTpb) {
        double d[3], mob;
        int sw;
        if (e < z.nseg_sw) {
            seg_arm(z, xs, bx, n * z.nseg_sw + e, sw, d);
            mob = seg_mob;
        } else {
            blob_arm(z, R, refs, n * z.nblob + (e - z.nseg_sw), sw, d);
            mob = blob_mob;
        }
        const M3 rc = rcross(d), rc2 = m3_mul(rc, rc);
        for (int k = 0; k < 9; ++k) {
            acc[k] += mob * rc.a[k];
            acc[9 + k] += mob * rc2.a[k];
        }
    }
    cta_sum<18>(acc, red);
    if (fil7) {
        double c[27];  // v1 v1^T, v2 v1^T, v2 v2^T, row-major
        for (int e = 0; e < 27; ++e) c[e] = 0.0;
        for (int i = threadIdx.x; i < z.nfil; i += kTpb) {
            const double *g = fil7 + 7 * ((size_t)n * z.nfil + i);
            const double inv = 1.0 / g[0];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    c[3 * a + b] += g[1 + a] * g[1 + b] * inv;
                    c[9 + 3 * a + b] += g[4 + a] * g[1 + b] * inv;
                    c[18 + 3 * a + b] += g[4 + a] * g[4 + b] * inv;
                }
        }
        cta_sum<27>(c, redc);
    }
    if (threadIdx.x != 0) return;
    double A[36];
    const double eye = (double)z.nseg_sw * seg_mob + (double)z.nblob * blob_mob;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double tr = red[3 * i + j][0], br = red[9 + 3 * i + j][0];
            A[i + 6 * j] = i == j ? eye : 0.0;
            A[i + 6 * (3 + j)] = tr;
            A[(3 + i) + 6 * j] = -tr;
            A[(3 + i) + 6 * (3 + j)] = -br;
        }
    if (fil7)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                A[i + 6 * j] -= seg_mob * redc[3 * i + j][0];
                A[(3 + i) + 6 * j] -= seg_mob * redc[9 + 3 * i + j][0];
                A[i + 6 * (3 + j)] -= seg_mob * redc[9 + 3 * j + i][0];
                A[(3 + i) + 6 * (3 + j)] -= seg_mob * redc[18 + 3 * i + j][0];
            }
    if (!invert6(A)) atomicOr(flag, 1);
    for (int k = 0; k < 36; ++k) P6[36 * n + k] = A[k];
}

// f6 = (f, 0) per segment from the 3-per-segment unknowns
__global__ void pk_expand(int S, const double *__restrict__ in, double *__restrict__ f6)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= S) return;
    for (int c = 0; c < 3; ++c) {
        f6[6 * (size_t)m + c] = in[3 * (size_t)m + c];
        f6[6 * (size_t)m + 3 + c] = 0.0;
    }
}

// the preconditioner's phase speed of filament f: pph_f / m_seg - (v1 . U +
// v2 . Omega) / |K|^2 (mobility_solver.cpp:564-597), U the body's
// preconditioned rows
__device__ __forceinline__ double precond_phase(const double *g, double pph, double seg_mob, const double *U)
{
    const double t = g[1] * U[0] + g[2] * U[1] + g[3] * U[2] + g[4] * U[3] + g[5] * U[4] + g[6] * U[5];
    return pph / seg_mob - t / g[0];
}

// particle rows: out = base - s (U + Omega x d), base = v (operator) or a (in + U + Omega x d) (preconditioner).
// With the phase speeds unknown (z.F > 0) the segment rows also take
// -phase_speed K (operator, mobility_solver.cpp:831-866) or + m_seg phi K
// (preconditioner, :606-634), and in the preconditioner the threads past the
// particles write its phase rows.
template <bool PRECOND>
__global__ void pk_rows(PSizes z, const double *__restrict__ in, const double *__restrict__ vsegs,
                        const double *__restrict__ vblobs, const double *__restrict__ xs, const double *__restrict__ bx,
                        const double *__restrict__ R, const double *__restrict__ refs, double seg_mob, double blob_mob,
                        const double *__restrict__ Uall, const double *__restrict__ vel_dir,
                        const double *__restrict__ fil7, const double *__restrict__ pph, double *__restrict__ out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t poff = 3 * (size_t)(z.S + z.B) + 6 * (size_t)z.W;
    if (PRECOND && p >= z.S + z.B) {
        const int f = p - z.S - z.B;
        if (f < z.F)
            out[poff + f] = precond_phase(fil7 + 7 * (size_t)f, pph[f], seg_mob, Uall + 6 * (f / z.nfil));
        return;
    }
    if (p >= z.S + z.B) return;
    double d[3];
    int sw;
    const bool seg = p < z.S;
    if (seg)
        seg_arm(z, xs, bx, p, sw, d);
    else
        blob_arm(z, R, refs, p - z.S, sw, d);
    const double *U = Uall + 6 * sw;
    const double k[3] = {U[0] + U[4] * d[2] - U[5] * d[1], U[1] + U[5] * d[0] - U[3] * d[2],
                         U[2] + U[3] * d[1] - U[4] * d[0]};
    double phi = 0.0;  // the filament's phase-speed term
    if (z.F && seg) {
        const int f = p / z.nseg;
        phi = PRECOND ? seg_mob * precond_phase(fil7 + 7 * (size_t)f, pph[f], seg_mob, U) : in[poff + f];
    }
    const size_t r = 3 * (size_t)p;
    for (int c = 0; c < 3; ++c) {
        const double K = z.F && seg ? vel_dir[r + c] : 0.0;
        if (PRECOND) {
            const double mob = seg ? seg_mob : blob_mob;
            out[r + c] = mob * in[r + c] + mob * k[c] + phi * K;
        } else {
            const double v = seg ? vsegs[6 * (size_t)p + c] : vblobs[3 * (size_t)(p - z.S) + c];
            out[r + c] = v - k[c] - phi * K;
        }
    }
}

// phase rows, one warp per filament: dot = sum_k K_k . in_k over its
// segments; the operator writes -dot (mobility_solver.cpp:831-866), the
// preconditioner pph = (-in_phase - m_seg dot) / |K|^2 (:518-556)
template <bool PRECOND>
__global__ void __launch_bounds__(kTpb) pk_phase_rows(PSizes z, const double *__restrict__ in,
                                                      const double *__restrict__ vel_dir,
                                                      const double *__restrict__ fil7, double seg_mob,
                                                      double *__restrict__ out)
{
    const int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (f >= z.F) return;
    const size_t r0 = 3 * (size_t)f * z.nseg;
    double dot = 0.0;
    for (int r = lane; r < 3 * z.nseg; r += 32) dot += vel_dir[r0 + r] * in[r0 + r];
    dot = warp_sum(dot);
    if (lane) return;
    const size_t poff = 3 * (size_t)(z.S + z.B) + 6 * (size_t)z.W;
    if (PRECOND)
        out[f] = (-in[poff + f] - seg_mob * dot) / fil7[7 * (size_t)f];
    else
        out[poff + f] = -dot;
}

// body rows, one CTA per swimmer: t = sum over its segments and blobs of
// (s f, d x s f) with s = mob (preconditioner) or 1 (operator); operator
// out_body = -t; preconditioner out_body = P6 (-in_body - t), where with the
// phase speeds unknown t also holds sum over the swimmer's filaments of
// pph (v1, v2) (mobility_solver.cpp:556-563)
template <bool PRECOND>
__global__ void __launch_bounds__(kTpb) pk_body(PSizes z, const double *__restrict__ in, const double *__restrict__ xs,
                                                const double *__restrict__ bx, const double *__restrict__ R,
                                                const double *__restrict__ refs, double seg_mob, double blob_mob,
                                                const double *__restrict__ P6, const double *__restrict__ fil7,
                                                const double *__restrict__ pph, double *__restrict__ out)
{
    __shared__ double red[6][kTpb / 32];
    const int n = blockIdx.x;
    const size_t uoff = 3 * (size_t)(z.S + z.B);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int e = threadIdx.x; e < z.nseg_sw + z.nblob; e += kTpb) {
        double d[3];
        int sw, p;
        if (e < z.nseg_sw) {
            p = n * z.nseg_sw + e;
            seg_arm(z, xs, bx, p, sw, d);
        } else {
            p = z.S + n * z.nblob + (e - z.nseg_sw);
            blob_arm(z, R, refs, p - z.S, sw, d);
        }
        const double sc = PRECOND ? (e < z.nseg_sw ? seg_mob : blob_mob) : 1.0;
        const double f[3] = {sc * in[3 * (size_t)p], sc * in[3 * (size_t)p + 1], sc * in[3 * (size_t)p + 2]};
        acc[0] += f[0];
        acc[1] += f[1];
        acc[2] += f[2];
        acc[3] += d[1] * f[2] - d[2] * f[1];
        acc[4] += d[2] * f[0] - d[0] * f[2];
        acc[5] += d[0] * f[1] - d[1] * f[0];
    }
    if (PRECOND && z.F)
        for (int i = threadIdx.x; i < z.nfil; i += kTpb) {
            const size_t f = (size_t)n * z.nfil + i;
            const double *g = fil7 + 7 * f;
            for (int j = 0; j < 6; ++j) acc[j] += pph[f] * g[1 + j];
        }
    cta_sum<6>(acc, red);
    if (threadIdx.x != 0) return;
    if (!PRECOND) {
        for (int j = 0; j < 6; ++j) out[uoff + 6 * n + j] = -red[j][0];
        return;
    }
    double b[6];
    for (int j = 0; j < 6; ++j) b[j] = -in[uoff + 6 * n + j] - red[j][0];
    const double *A = P6 + 36 * n;
    for (int i = 0; i < 6; ++i) {
        double t = 0.0;
        for (int j = 0; j < 6; ++j) t += A[i + 6 * j] * b[j];
        out[uoff + 6 * n + i] = t;
    }
}

// segment rows of the right-hand side: phase_speed * vel_dir; zero elsewhere
__global__ void pk_rhs(int np, int S3, int nseg3, const double *__restrict__ vel_dir,
                       const double *__restrict__ phase, double *__restrict__ rhs)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= np) return;
    rhs[r] = r < S3 ? phase[r / nseg3] * vel_dir[r] : 0.0;
}

// The generalised force of the beat at phase phi from a table of n >= 2
// samples over one period, by the reference's cubic Hermite rule with its
// end-point differences (mobility_solver.cpp:221-282).
__host__ __device__ inline double hermite_generalised_force(const double *t, int n, double phi)
{
    double x = 0.5 * phi / kPi;
    x -= floor(x);
    x *= n;
    const int lo = (int)x;
    if (lo == n) return t[0];
    const int hi = lo == n - 1 ? 0 : lo + 1;
    const double dlo = lo == 0 ? t[1] - t[0] : 0.5 * (t[hi] - t[lo - 1]);
    const double dhi = hi == 0 ? t[0] - t[n - 1] : 0.5 * (t[hi == n - 1 ? 0 : hi + 1] - t[lo]);
    const double s = x - lo, s2 = s * s, s3 = s2 * s;
    return t[lo] * (2.0 * s3 - 3.0 * s2 + 1.0) + dlo * (s3 - 2.0 * s2 + s) + t[hi] * (3.0 * s2 - 2.0 * s3) +
           dhi * (s3 - s2);
}

// the right-hand side with the phase speeds unknown: -q omega0 / (2 pi) in
// the phase rows (mobility_solver.cpp:284-296), zero elsewhere
__global__ void pk_rhs_dynamic(int np, size_t poff, const double *__restrict__ table, int ntable,
                               const double *__restrict__ phase, const double *__restrict__ omega0,
                               double *__restrict__ rhs)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= np) return;
    if ((size_t)r < poff) {
        rhs[r] = 0.0;
        return;
    }
    const size_t f = r - poff;
    rhs[r] = -(hermite_generalised_force(table, ntable, phase[f]) * (0.5 * omega0[f] / kPi));
}

// solution -> f_segs (forces, zero torques), f_blobs, v_bodies
__global__ void pk_store(PSizes z, const double *__restrict__ x, double *__restrict__ f6, double *__restrict__ fb,
                         double *__restrict__ vb)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < z.S) {
        for (int c = 0; c < 3; ++c) {
            f6[6 * (size_t)p + c] = x[3 * (size_t)p + c];
            f6[6 * (size_t)p + 3 + c] = 0.0;
        }
    } else if (p < z.S + z.B) {
        for (int c = 0; c < 3; ++c) fb[3 * (size_t)(p - z.S) + c] = x[3 * (size_t)p + c];
    } else if (p < z.S + z.B + z.W) {
        const int n = p - z.S - z.B;
        for (int j = 0; j < 6; ++j) vb[6 * n + j] = x[3 * (size_t)(z.S + z.B) + 6 * n + j];
    }
}

inline int blocks(int n) { return (n + kTpb - 1) / kTpb; }

gmi_status dalloc0(double **p, size_t n, cudaStream_t st)
{
    GMI_CUDA_TRY(dev_malloc(p, (n ? n : 1) * sizeof(double)));
    GMI_CUDA_TRY(cudaMemsetAsync(*p, 0, (n ? n : 1) * sizeof(double), st));
    return GMI_OK;
}

void release_work(PrescribedWork *pw)
{
    krylov_free(pw->K);
    for (double *p : {pw->vel_dir, pw->phase, pw->P6, pw->rhs, pw->soln, pw->f6, pw->phase_in, pw->omega0, pw->fil7,
                      pw->pph, pw->table})
        if (p) dev_free(p);
    if (pw->flag) dev_free(pw->flag);
    delete pw;
}

// The workspace for solves with the phase speeds given (dynamic false) or
// unknown; a solve of the other kind than the last one starts a new one
// (and with it a cold start).
gmi_status ensure_work(gmi_solver *s, bool dynamic)
{
    if (s->prescribed && s->prescribed->dynamic == dynamic) return GMI_OK;
    if (s->prescribed) {
        GMI_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
        release_work(s->prescribed);
        s->prescribed = nullptr;
    }
    PrescribedWork *pw = new (std::nothrow) PrescribedWork();
    if (!pw) {
        set_last_error_msg("prescribed cilia: out of host memory");
        return GMI_ERR_ARG;
    }
    s->prescribed = pw;
    pw->dynamic = dynamic;
    cudaStream_t st = s->ctx->stream;
    const size_t S = s->S, B = s->B, W = s->W, F = (size_t)s->W * s->cfg.nfil;
    pw->np = (int)(3 * S + 3 * B + 6 * W + (dynamic ? F : 0));
    GMI_TRY(krylov_alloc(pw->K, pw->np, s->m, st));
    GMI_TRY(dalloc0(&pw->vel_dir, 3 * S, st));
    GMI_TRY(dalloc0(&pw->phase, F, st));
    GMI_TRY(dalloc0(&pw->P6, 36 * W, st));
    GMI_TRY(dalloc0(&pw->rhs, pw->np, st));
    GMI_TRY(dalloc0(&pw->soln, pw->np, st));
    GMI_TRY(dalloc0(&pw->f6, 6 * S, st));
    if (dynamic) {
        GMI_TRY(dalloc0(&pw->phase_in, F, st));
        GMI_TRY(dalloc0(&pw->omega0, F, st));
        GMI_TRY(dalloc0(&pw->fil7, 7 * F, st));
        GMI_TRY(dalloc0(&pw->pph, F, st));
    }
    double *fl = nullptr;
    GMI_TRY(dalloc0(&fl, 1, st));
    pw->flag = reinterpret_cast<int *>(fl);
    return GMI_OK;
}

// One prescribed-cilia solve.  phase_speed: the given speeds, or with
// dynamic the initial guess of the unknown ones (the reference passes
// omega0, filament.cpp:841); speed_out (dynamic only): the solved speeds;
// phase, omega0: the filaments' phases and natural frequencies (dynamic only).
gmi_status prescribed_solve(gmi_solver *s, const double *body_x, const double *body_q, const double *vel_dir,
                            const double *phase_speed, double *speed_out, const double *phase, const double *omega0,
                            bool dynamic, int *gmres_iters, const char *who)
{
    if (s->cfg.wall || s->B == 0 || !s->refs_set) {
        set_last_error_msg((std::string(who) + ": free-swimming bodies with blob references").c_str());
        return GMI_ERR_ARG;
    }
    if (dynamic && s->gen_force_refs.size() < 2) {
        set_last_error_msg(
            (std::string(who) + ": no generalised-force table (gmi_solver_set_generalised_force_refs)").c_str());
        return GMI_ERR_ARG;
    }
    gmi_context *ctx = s->ctx;
    GMI_CUDA_TRY(cudaSetDevice(ctx->device));
    GMI_TRY(ensure_work(s, dynamic));
    PrescribedWork *pw = s->prescribed;
    cudaStream_t st = ctx->stream;
    const int S = s->S, B = s->B, W = s->W, F = W * s->cfg.nfil, nseg = s->cfg.nseg;
    const PSizes z{S, B, W, s->cfg.nfil * nseg, s->cfg.nblob, nseg, s->cfg.nfil, dynamic ? F : 0};
    const double seg_mob = 6.0 * kPi * s->cfg.mu * s->cfg.rseg, blob_mob = 6.0 * kPi * s->cfg.mu * s->cfg.rblob;
    const size_t uoff = 3 * (size_t)(S + B), poff = uoff + 6 * (size_t)W;
    // segment positions from the caller's host array, shapes, phase speeds, bodies
    GMI_CUDA_TRY(cudaMemcpyAsync(s->x_segs, s->h.x_segs_host, 3 * (size_t)S * sizeof(double), cudaMemcpyHostToDevice,
                                 st));
    GMI_CUDA_TRY(cudaMemcpyAsync(pw->vel_dir, vel_dir, 3 * (size_t)S * sizeof(double), cudaMemcpyHostToDevice, st));
    if (dynamic) {
        if (pw->table_serial != s->gen_force_serial || !pw->table) {
            if (pw->table) dev_free(pw->table);
            pw->table = nullptr;
            GMI_TRY(dalloc0(&pw->table, s->gen_force_refs.size(), st));
            GMI_CUDA_TRY(cudaMemcpyAsync(pw->table, s->gen_force_refs.data(), s->gen_force_refs.size() * sizeof(double),
                                         cudaMemcpyHostToDevice, st));
            // the host vector may change once the call returns
            GMI_CUDA_TRY(cudaStreamSynchronize(st));
            pw->ntable = (int)s->gen_force_refs.size();
            pw->table_serial = s->gen_force_serial;
        }
        GMI_CUDA_TRY(cudaMemcpyAsync(pw->phase_in, phase, (size_t)F * sizeof(double), cudaMemcpyHostToDevice, st));
        GMI_CUDA_TRY(cudaMemcpyAsync(pw->omega0, omega0, (size_t)F * sizeof(double), cudaMemcpyHostToDevice, st));
        // the phase-speed part of the warm start (mobility_solver.cpp:1094-1113)
        GMI_CUDA_TRY(cudaMemcpyAsync(pw->soln + poff, phase_speed, (size_t)F * sizeof(double), cudaMemcpyHostToDevice,
                                     st));
    } else {
        GMI_CUDA_TRY(cudaMemcpyAsync(pw->phase, phase_speed, (size_t)F * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    GMI_TRY(solver_place_blobs(s, body_x, body_q));
    GMI_CUDA_TRY(cudaMemsetAsync(pw->flag, 0, sizeof(int), st));
    const int warp_blocks = (int)((32 * (size_t)F + kTpb - 1) / kTpb);
    if (dynamic) {
        pk_fil_consts<<<warp_blocks, kTpb, 0, st>>>(z, s->x_segs, s->body_x, pw->vel_dir, pw->fil7);
        ctx->launches++;
    }
    pk_precon_mats<<<W, kTpb, 0, st>>>(z, s->x_segs, s->body_x, s->R, s->refs, seg_mob, blob_mob,
                                       dynamic ? pw->fil7 : nullptr, pw->P6, pw->flag);
    if (dynamic)
        pk_rhs_dynamic<<<blocks(pw->np), kTpb, 0, st>>>(pw->np, poff, pw->table, pw->ntable, pw->phase_in, pw->omega0,
                                                        pw->rhs);
    else
        pk_rhs<<<blocks(pw->np), kTpb, 0, st>>>(pw->np, 3 * S, 3 * nseg, pw->vel_dir, pw->phase, pw->rhs);
    ctx->launches += 2;
    GMI_CUDA_TRY(cudaGetLastError());

    PairConsts kss, ksb, kbb;
    fill_consts(kss, s->cfg.rseg, s->cfg.rseg, s->cfg.rseg, s->cfg.mu);
    fill_consts(ksb, s->cfg.rseg, s->cfg.rseg, s->cfg.rblob, s->cfg.mu);
    fill_consts(kbb, s->cfg.rblob, s->cfg.rblob, s->cfg.rblob, s->cfg.mu);
    DeviceApply matvec = [&](const double *in, double *out) -> gmi_status {
        pk_expand<<<blocks(S), kTpb, 0, st>>>(S, in, pw->f6);
        ctx->launches++;
        // segments with their forces; M_ss onto segments, M_bs onto blobs
        GMI_TRY(pack_records(ctx, s->x_segs, pw->f6, 6, S, ctx->rec_src));
        GMI_TRY(launch_pair(ctx, kSS, ctx->rec_src.ptr, 0, S, ctx->rec_src.ptr, S, kss, s->v_segs, 0));
        GMI_TRY(pack_records(ctx, s->x_blobs, nullptr, 0, B, ctx->rec_tgt));
        GMI_TRY(launch_pair(ctx, kBS, ctx->rec_tgt.ptr, 0, B, ctx->rec_src.ptr, S, ksb, s->v_blobs, 0));
        // blobs with their forces; M_bb onto blobs, M_sb onto segments
        GMI_TRY(pack_records(ctx, s->x_blobs, in + 3 * (size_t)S, 3, B, ctx->rec_src));
        GMI_TRY(launch_pair(ctx, kBB, ctx->rec_src.ptr, 0, B, ctx->rec_src.ptr, B, kbb, s->v_blobs, 1));
        GMI_TRY(pack_records(ctx, s->x_segs, nullptr, 0, S, ctx->rec_tgt));
        GMI_TRY(launch_pair(ctx, kSB, ctx->rec_tgt.ptr, 0, S, ctx->rec_src.ptr, B, ksb, s->v_segs, 1));
        pk_rows<false><<<blocks(S + B), kTpb, 0, st>>>(z, in, s->v_segs, s->v_blobs, s->x_segs, s->body_x, s->R,
                                                       s->refs, seg_mob, blob_mob, in + uoff, pw->vel_dir, pw->fil7,
                                                       nullptr, out);
        pk_body<false><<<W, kTpb, 0, st>>>(z, in, s->x_segs, s->body_x, s->R, s->refs, seg_mob, blob_mob, pw->P6,
                                           nullptr, nullptr, out);
        ctx->launches += 2;
        if (dynamic) {
            pk_phase_rows<false><<<warp_blocks, kTpb, 0, st>>>(z, in, pw->vel_dir, pw->fil7, seg_mob, out);
            ctx->launches++;
        }
        GMI_CUDA_TRY(cudaGetLastError());
        return GMI_OK;
    };
    DeviceApply precond = [&](const double *in, double *out) -> gmi_status {
        if (dynamic) {
            pk_phase_rows<true><<<warp_blocks, kTpb, 0, st>>>(z, in, pw->vel_dir, pw->fil7, seg_mob, pw->pph);
            ctx->launches++;
        }
        pk_body<true><<<W, kTpb, 0, st>>>(z, in, s->x_segs, s->body_x, s->R, s->refs, seg_mob, blob_mob, pw->P6,
                                          pw->fil7, pw->pph, out);
        pk_rows<true><<<blocks(S + B + z.F), kTpb, 0, st>>>(z, in, nullptr, nullptr, s->x_segs, s->body_x, s->R,
                                                            s->refs, seg_mob, blob_mob, out + uoff, pw->vel_dir,
                                                            pw->fil7, pw->pph, out);
        ctx->launches += 2;
        GMI_CUDA_TRY(cudaGetLastError());
        return GMI_OK;
    };
    int iters = 0;
    GMI_TRY(krylov_gmres(ctx, pw->K, precond, matvec, pw->rhs, pw->soln, s->cfg.linear_tol, &iters));
    pk_store<<<blocks(S + B + W), kTpb, 0, st>>>(z, pw->soln, s->f_segs, s->f_blobs, s->v_bodies);
    ctx->launches++;
    GMI_CUDA_TRY(cudaGetLastError());
    GMI_CUDA_TRY(cudaMemcpyAsync(s->h.f_segs_host, s->f_segs, 6 * (size_t)S * sizeof(double), cudaMemcpyDeviceToHost,
                                 st));
    GMI_CUDA_TRY(cudaMemcpyAsync(s->h.f_blobs_host, s->f_blobs, 3 * (size_t)B * sizeof(double),
                                 cudaMemcpyDeviceToHost, st));
    if (dynamic)
        GMI_CUDA_TRY(cudaMemcpyAsync(speed_out, pw->soln + poff, (size_t)F * sizeof(double), cudaMemcpyDeviceToHost,
                                     st));
    int flag = 0;
    GMI_CUDA_TRY(cudaMemcpyAsync(&flag, pw->flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    GMI_CUDA_TRY(cudaStreamSynchronize(st));
    GMI_TRY(context_check_device_errors(ctx));
    if (flag) {
        set_last_error_msg((std::string(who) + ": singular body preconditioner matrix").c_str());
        return GMI_ERR_NONFINITE;
    }
    if (gmres_iters) *gmres_iters = iters;
    return GMI_OK;
}

}  // namespace

void prescribed_release(gmi_solver *s)
{
    if (!s->prescribed) return;
    release_work(s->prescribed);
    s->prescribed = nullptr;
}

}  // namespace gmi

using namespace gmi;

extern "C" gmi_status gmi_solver_compute_velocities_prescribed(gmi_solver *s, const double *body_x,
                                                               const double *body_q, const double *vel_dir,
                                                               const double *phase_speed, int *gmres_iters)
{
    if (!s || !body_x || !body_q || !vel_dir || !phase_speed) {
        set_last_error_msg("gmi_solver_compute_velocities_prescribed: null argument");
        return GMI_ERR_ARG;
    }
    return prescribed_solve(s, body_x, body_q, vel_dir, phase_speed, nullptr, nullptr, nullptr, false, gmres_iters,
                            "gmi_solver_compute_velocities_prescribed");
}

extern "C" gmi_status gmi_solver_set_generalised_force_refs(gmi_solver *s, const double *refs, int count)
{
    if (!s || (!refs && count > 0) || count < 0 || count == 1) {
        set_last_error_msg("gmi_solver_set_generalised_force_refs: bad table (count 0 clears, else >= 2 samples)");
        return GMI_ERR_ARG;
    }
    for (int i = 0; i < count; ++i)
        if (!std::isfinite(refs[i])) {
            set_last_error_msg("gmi_solver_set_generalised_force_refs: non-finite sample");
            return GMI_ERR_ARG;
        }
    try {
        s->gen_force_refs.assign(refs, refs + count);
    } catch (...) {
        set_last_error_msg("gmi_solver_set_generalised_force_refs: out of host memory");
        return GMI_ERR_ARG;
    }
    ++s->gen_force_serial;
    return GMI_OK;
}

extern "C" gmi_status gmi_solver_compute_velocities_prescribed_dynamic(gmi_solver *s, const double *body_x,
                                                                       const double *body_q, const double *vel_dir,
                                                                       const double *phase, const double *omega0,
                                                                       double *phase_speed, int *gmres_iters)
{
    if (!s || !body_x || !body_q || !vel_dir || !phase || !omega0 || !phase_speed) {
        set_last_error_msg("gmi_solver_compute_velocities_prescribed_dynamic: null argument");
        return GMI_ERR_ARG;
    }
    return prescribed_solve(s, body_x, body_q, vel_dir, phase_speed, phase_speed, phase, omega0, true, gmres_iters,
                            "gmi_solver_compute_velocities_prescribed_dynamic");
}
