// gmi_gmres.cu -- device-resident GMRES over operator callbacks.
#include <cmath>

#include "gmi_gmres.hpp"
#include "gmi_solver_device.cuh"

namespace gmi {

namespace {

constexpr int kTpb = 256;
constexpr int kRows = 1024;  // rows per CTA of the dot-product partials

int chunks(int n) { return (n + kRows - 1) / kRows; }
int grid(int n, int tpb = kTpb) { return (n + tpb - 1) / tpb; }

// partial[i * nc + c] = sum over chunk c of Q[:, i] . v
__global__ void __launch_bounds__(kTpb) kdots(const double *__restrict__ Q, size_t ld, const double *__restrict__ v,
                                              int n, int nc, double *__restrict__ partial)
{
    __shared__ double red[kTpb / 32];
    const int c = blockIdx.x, i = blockIdx.y, r0 = c * kRows, r1 = min(n, r0 + kRows);
    const double *q = Q + ld * i;
    double t = 0.0;
    for (int r = r0 + threadIdx.x; r < r1; r += kTpb) t += q[r] * v[r];
    t = warp_sum(t);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q2 = 0; q2 < kTpb / 32; ++q2) s += red[q2];
        partial[(size_t)i * nc + c] = s;
    }
}

// h[i] = sum of the partials; H column (=, or += on the second pass); w -= Q h
__global__ void kcgs(const double *__restrict__ Q, size_t ld, int k, const double *__restrict__ partial, int nc,
                     double *__restrict__ w, int n, double *__restrict__ Hcol, int pass)
{
    extern __shared__ double h[];
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < nc; ++c) s += partial[(size_t)i * nc + c];
        h[i] = s;
        if (blockIdx.x == 0) Hcol[i] = pass == 0 ? s : Hcol[i] + s;
    }
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double v = w[r];
    for (int i = 0; i < k; ++i) v -= h[i] * Q[ld * i + r];
    w[r] = v;
}

// ||v|| into out[0]
__global__ void knorm(const double *__restrict__ partial, int nc, double *__restrict__ out)
{
    double s = 0.0;
    for (int c = 0; c < nc; ++c) s += partial[c];
    out[0] = sqrt(s);
}

// q = w / ||w|| (||w|| in nrm[0]); H(k, k-1) = ||w||
__global__ void knormalize(const double *__restrict__ w, int n, const double *__restrict__ nrm, double *__restrict__ q,
                           double *__restrict__ Hentry)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0 && Hentry) *Hentry = nrm[0];
    if (r < n) q[r] = w[r] / nrm[0];
}

// Givens step on H column iter-1 (mobility_solver.cpp:1191-1228); out[0] = |beta(iter)| / norm_ref
__global__ void kgivens(double *__restrict__ H, int ldh, double *__restrict__ beta, double *__restrict__ cs,
                        double *__restrict__ sn, int iter, double norm_ref, double *__restrict__ out)
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
    out[0] = fabs(beta[iter]) / norm_ref;
}

// y = H(0:iter, 0:iter)^-1 beta(0:iter), one warp, each row in the
// reference's order (mobility_solver.cpp:1236-1250)
__global__ void kbacksolve(const double *__restrict__ H, int ldh, const double *__restrict__ beta, int iter,
                           double *__restrict__ y)
{
    extern __shared__ double b[];
    for (int i = threadIdx.x; i < iter; i += 32) b[i] = beta[i];
    __syncwarp();
    for (int j = iter - 1; j >= 0; --j) {
        const double yj = b[j] / H[j + (size_t)ldh * j];
        for (int i = threadIdx.x; i < j; i += 32) b[i] -= H[i + (size_t)ldh * j] * yj;
        if (threadIdx.x == 0) y[j] = yj;
        __syncwarp();
    }
}

// out = Q(:, 0:k) y
__global__ void kcombine(const double *__restrict__ Q, size_t ld, const double *__restrict__ y, int k, int n,
                         double *__restrict__ out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double acc = 0.0;
    for (int i = 0; i < k; ++i) acc += y[i] * Q[ld * i + r];
    out[r] = acc;
}

// out = a x + b y
__global__ void kaxpby(int n, double a, const double *__restrict__ x, double b, const double *__restrict__ y,
                       double *__restrict__ out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) out[r] = a * x[r] + b * y[r];
}

gmi_status dev_alloc(double **p, size_t count, cudaStream_t st)
{
    GMI_CUDA_TRY(dev_malloc(p, (count ? count : 1) * sizeof(double)));
    GMI_CUDA_TRY(cudaMemsetAsync(*p, 0, (count ? count : 1) * sizeof(double), st));
    return GMI_OK;
}

// ||v|| to the host (one synchronisation)
gmi_status norm_host(gmi_context *ctx, KrylovSpace &K, const double *v, double *out)
{
    const int nc = chunks(K.n);
    kdots<<<dim3(nc, 1), kTpb, 0, ctx->stream>>>(v, (size_t)K.n, v, K.n, nc, K.partial);
    knorm<<<1, 1, 0, ctx->stream>>>(K.partial, nc, K.scal);
    ctx->launches += 2;
    GMI_CUDA_TRY(cudaGetLastError());
    GMI_CUDA_TRY(cudaMemcpyAsync(K.h_scal, K.scal, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *out = K.h_scal[0];
    return GMI_OK;
}

}  // namespace

gmi_status krylov_alloc(KrylovSpace &K, int n, int m, cudaStream_t st)
{
    krylov_free(K);
    K.n = n;
    K.m = m;
    const size_t N = (size_t)n, M = (size_t)m;
    gmi_status e = GMI_OK;
    if ((e = dev_alloc(&K.Q, N * (M + 1), st)) != GMI_OK || (e = dev_alloc(&K.H, (M + 1) * (M + 1), st)) != GMI_OK ||
        (e = dev_alloc(&K.beta, M + 1, st)) != GMI_OK || (e = dev_alloc(&K.cs, M, st)) != GMI_OK ||
        (e = dev_alloc(&K.sn, M, st)) != GMI_OK || (e = dev_alloc(&K.yv, M + 1, st)) != GMI_OK ||
        (e = dev_alloc(&K.w, N, st)) != GMI_OK || (e = dev_alloc(&K.z, N, st)) != GMI_OK ||
        (e = dev_alloc(&K.tmp, N, st)) != GMI_OK ||
        (e = dev_alloc(&K.partial, (size_t)chunks(n) * (M + 1), st)) != GMI_OK ||
        (e = dev_alloc(&K.scal, 4, st)) != GMI_OK) {
        krylov_free(K);
        return e;
    }
    if (host_alloc(&K.h_scal, 4 * sizeof(double)) != cudaSuccess) {
        K.h_scal = nullptr;
        krylov_free(K);
        set_last_error_msg("krylov_alloc: pinned allocation failed");
        return GMI_ERR_CUDA;
    }
    return GMI_OK;
}

void krylov_free(KrylovSpace &K)
{
    for (double **p : {&K.Q, &K.H, &K.beta, &K.cs, &K.sn, &K.yv, &K.w, &K.z, &K.tmp, &K.partial, &K.scal}) {
        if (*p) dev_free(*p);
        *p = nullptr;
    }
    if (K.h_scal) host_free(K.h_scal);
    K.h_scal = nullptr;
    K.n = K.m = 0;
}

gmi_status krylov_gmres(gmi_context *ctx, KrylovSpace &K, const DeviceApply &precond, const DeviceApply &matvec,
                        const double *rhs, double *soln, double tol, int *iters)
{
    cudaStream_t st = ctx->stream;
    const int n = K.n, ldh = K.m + 1, nc = chunks(n);
    const size_t ld = (size_t)n;
    *iters = 0;
    double norm_rhs = 0.0;
    GMI_TRY(norm_host(ctx, K, rhs, &norm_rhs));
    if (!std::isfinite(norm_rhs)) {
        set_last_error_msg("non-finite right-hand side in the linear solve");
        return GMI_ERR_NONFINITE;
    }
    if (norm_rhs == 0.0) {  // the solution is zero (mobility_solver.cpp:1005-1060)
        GMI_CUDA_TRY(cudaMemsetAsync(soln, 0, ld * sizeof(double), st));
        return GMI_OK;
    }
    // r0 = rhs - A x0; reject a warm start whose residual exceeds ||rhs||
    GMI_TRY(matvec(soln, K.tmp));
    kaxpby<<<grid(n), kTpb, 0, st>>>(n, 1.0, rhs, -1.0, K.tmp, K.w);
    ctx->launches++;
    double beta0 = 0.0;
    GMI_TRY(norm_host(ctx, K, K.w, &beta0));
    if (beta0 <= tol * norm_rhs) return GMI_OK;
    if (beta0 > norm_rhs) {
        GMI_CUDA_TRY(cudaMemsetAsync(soln, 0, ld * sizeof(double), st));
        GMI_CUDA_TRY(cudaMemcpyAsync(K.w, rhs, ld * sizeof(double), cudaMemcpyDeviceToDevice, st));
        beta0 = norm_rhs;
    }
    K.h_scal[1] = beta0;
    GMI_CUDA_TRY(cudaMemcpyAsync(K.beta, K.h_scal + 1, sizeof(double), cudaMemcpyHostToDevice, st));
    GMI_CUDA_TRY(cudaMemcpyAsync(K.scal, K.h_scal + 1, sizeof(double), cudaMemcpyHostToDevice, st));
    knormalize<<<grid(n), kTpb, 0, st>>>(K.w, n, K.scal, K.Q, nullptr);
    ctx->launches++;
    const int max_iter = n < K.m ? n : K.m;
    for (int iter = 1; iter <= max_iter; ++iter) {
        GMI_TRY(precond(K.Q + ld * (iter - 1), K.z));
        GMI_TRY(matvec(K.z, K.w));
        double *Hcol = K.H + (size_t)ldh * (iter - 1);
        for (int pass = 0; pass < 2; ++pass) {  // classical Gram-Schmidt, twice
            kdots<<<dim3(nc, iter), kTpb, 0, st>>>(K.Q, ld, K.w, n, nc, K.partial);
            kcgs<<<grid(n), kTpb, iter * sizeof(double), st>>>(K.Q, ld, iter, K.partial, nc, K.w, n, Hcol, pass);
            ctx->launches += 2;
        }
        kdots<<<dim3(nc, 1), kTpb, 0, st>>>(K.w, ld, K.w, n, nc, K.partial);
        knorm<<<1, 1, 0, st>>>(K.partial, nc, K.scal);
        knormalize<<<grid(n), kTpb, 0, st>>>(K.w, n, K.scal, K.Q + ld * iter, Hcol + iter);
        kgivens<<<1, 1, 0, st>>>(K.H, ldh, K.beta, K.cs, K.sn, iter, norm_rhs, K.scal + 1);
        ctx->launches += 4;
        GMI_CUDA_TRY(cudaGetLastError());
        GMI_CUDA_TRY(cudaMemcpyAsync(K.h_scal + 2, K.scal + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
        GMI_CUDA_TRY(cudaStreamSynchronize(st));
        const double resid = K.h_scal[2];
        if (!std::isfinite(resid)) {
            set_last_error_msg("GMRES produced a non-finite residual");
            return GMI_ERR_NONFINITE;
        }
        if (resid <= tol || iter == max_iter) {
            kbacksolve<<<1, 32, iter * sizeof(double), st>>>(K.H, ldh, K.beta, iter, K.yv);
            kcombine<<<grid(n, 64), 64, 0, st>>>(K.Q, ld, K.yv, iter, n, K.tmp);
            ctx->launches += 2;
            GMI_TRY(precond(K.tmp, K.z));
            kaxpby<<<grid(n), kTpb, 0, st>>>(n, 1.0, soln, 1.0, K.z, soln);
            ctx->launches++;
            GMI_CUDA_TRY(cudaGetLastError());
            *iters = iter;
            return GMI_OK;
        }
    }
    return GMI_OK;
}

}  // namespace gmi
