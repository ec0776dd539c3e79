// gmi_seeding.cu -- repulsive seeding of points on the unit sphere: the
// reference's blob seeding and uniform filament seeding
// (repulsive_blob_seeding, seeding.cu:13-160; the UNIFORM_SEEDING branch of
// repulsive_filament_seeding, seeding.cu:233-389), whose GPU path runs the
// force kernel seeding_repulsion_step (cuda_functions.cu:1159-1250).
//
// Start: a spiral of n points, z_m = 2 m / (n - 1) - 1 (z = -1 for n = 1),
// the azimuth advanced by 3.6 / (r sqrt n) from one point to the next
// (r = sqrt(1 - z^2)) and 0 at the two poles.  Step: every point moves by
// the sum over the others of 5 (2 - d) (x_i - x_j) / d, d = |x_i - x_j|,
// and is put back on the unit sphere; the relaxation stops once no
// coordinate moved by more than 1e-4.
//
// On the device: one thread per point sums its force over the others in
// index order (sources staged through shared memory in tiles), FP64; one
// update kernel renormalises and takes the largest move (the bit patterns
// of non-negative doubles order like their values, so an integer atomicMax
// finds it).  The host reads that one word per step.
#include <cmath>
#include <cstring>
#include <vector>

#include "gmi_context.hpp"

namespace gmi {

constexpr int kSeedTpb = 128;
constexpr double kSeedMove = 1e-4;  // seeding.cu:67

__global__ void __launch_bounds__(kSeedTpb) seed_force_kernel(const double *__restrict__ X, int N,
                                                              double *__restrict__ F)
{
    __shared__ double sx[kSeedTpb], sy[kSeedTpb], sz[kSeedTpb];
    const int i = blockIdx.x * kSeedTpb + threadIdx.x;
    double xi = 0.0, yi = 0.0, zi = 0.0, fx = 0.0, fy = 0.0, fz = 0.0;
    if (i < N) {
        xi = X[3 * i];
        yi = X[3 * i + 1];
        zi = X[3 * i + 2];
    }
    for (int j0 = 0; j0 < N; j0 += kSeedTpb) {
        const int j = j0 + threadIdx.x;
        if (j < N) {
            sx[threadIdx.x] = X[3 * j];
            sy[threadIdx.x] = X[3 * j + 1];
            sz[threadIdx.x] = X[3 * j + 2];
        }
        __syncthreads();
        if (i < N) {
            const int jn = min(kSeedTpb, N - j0);
            for (int t = 0; t < jn; ++t) {
                if (j0 + t == i) continue;
                const double dx = xi - sx[t], dy = yi - sy[t], dz = zi - sz[t];
                const double d = sqrt(dx * dx + dy * dy + dz * dz);
                const double inv = 1.0 / d;
                const double mag = 5.0 * (2.0 - d);
                fx += mag * dx * inv;
                fy += mag * dy * inv;
                fz += mag * dz * inv;
            }
        }
        __syncthreads();
    }
    if (i < N) {
        F[3 * i] = fx;
        F[3 * i + 1] = fy;
        F[3 * i + 2] = fz;
    }
}

__global__ void __launch_bounds__(kSeedTpb) seed_update_kernel(const double *__restrict__ X,
                                                               const double *__restrict__ F, int N,
                                                               double *__restrict__ Xn,
                                                               unsigned long long *__restrict__ max_move)
{
    __shared__ double red[kSeedTpb / 32];
    const int i = blockIdx.x * kSeedTpb + threadIdx.x;
    double mv = 0.0;
    if (i < N) {
        double p[3];
        for (int c = 0; c < 3; ++c) p[c] = __dadd_rn(X[3 * i + c], F[3 * i + c]);
        // the host update's arithmetic in its written order, no contraction
        const double nrm =
            sqrt(__dadd_rn(__dadd_rn(__dmul_rn(p[0], p[0]), __dmul_rn(p[1], p[1])), __dmul_rn(p[2], p[2])));
        for (int c = 0; c < 3; ++c) {
            p[c] /= nrm;
            mv = fmax(mv, fabs(p[c] - X[3 * i + c]));
            Xn[3 * i + c] = p[c];
        }
        if (!(fabs(p[0]) + fabs(p[1]) + fabs(p[2]) < INFINITY)) mv = INFINITY;  // coincident points
    }
    for (int o = 16; o > 0; o >>= 1) mv = fmax(mv, __shfl_xor_sync(0xffffffffu, mv, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mv;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = red[0];
        for (int w = 1; w < kSeedTpb / 32; ++w) m = fmax(m, red[w]);
        atomicMax(max_move, (unsigned long long)__double_as_longlong(m));
    }
}

// The spiral start (seeding.cu:23-43).
static void seed_spiral(int n, double *x)
{
    double phi = 0.0;
    for (int m = 0; m < n; ++m) {
        const double z = (n == 1) ? -1.0 : 2.0 * m / double(n - 1) - 1.0;
        const double r = std::sqrt(1.0 - z * z);
        if (m == 0 || m == n - 1)
            phi = 0.0;
        else
            phi += 3.6 / (r * std::sqrt((double)n));
        x[3 * m] = r * std::cos(phi);
        x[3 * m + 1] = r * std::sin(phi);
        x[3 * m + 2] = z;
    }
}

}  // namespace gmi

using namespace gmi;

extern "C" gmi_status gmi_seed_sphere_repulsive(int device, int n, int max_steps, double *refs_out_h, int *steps_out)
{
    if (n < 1 || max_steps < 1 || refs_out_h == nullptr) {
        set_last_error_msg("gmi_seed_sphere_repulsive: n and max_steps must be positive, refs_out_h non-null");
        return GMI_ERR_ARG;
    }
    GMI_CUDA_TRY(cudaSetDevice(device));
    std::vector<double> h(3 * (size_t)n);
    seed_spiral(n, h.data());
    cudaStream_t st = nullptr;
    GMI_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    double *X = nullptr, *Xn = nullptr, *F = nullptr;
    unsigned long long *mm = nullptr, *mh = nullptr;
    gmi_status status = GMI_OK;
    int steps = 0;
    auto fail = [&](cudaError_t e, const char *what) {
        set_last_error(cudaGetErrorString(e), what, __FILE__, __LINE__);
        status = GMI_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = dev_malloc(&X, 3 * (size_t)n * sizeof(double))) != cudaSuccess ||
        (e = dev_malloc(&Xn, 3 * (size_t)n * sizeof(double))) != cudaSuccess ||
        (e = dev_malloc(&F, 3 * (size_t)n * sizeof(double))) != cudaSuccess ||
        (e = dev_malloc(&mm, sizeof(unsigned long long))) != cudaSuccess ||
        (e = host_alloc(&mh, sizeof(unsigned long long))) != cudaSuccess) {
        fail(e, "allocation");
    }
    if (status == GMI_OK &&
        (e = cudaMemcpyAsync(X, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        fail(e, "cudaMemcpyAsync");
    const int grid = (n + kSeedTpb - 1) / kSeedTpb;
    bool converged = false;
    while (status == GMI_OK && steps < max_steps) {
        cudaMemsetAsync(mm, 0, sizeof(unsigned long long), st);
        seed_force_kernel<<<grid, kSeedTpb, 0, st>>>(X, n, F);
        seed_update_kernel<<<grid, kSeedTpb, 0, st>>>(X, F, n, Xn, mm);
        cudaMemcpyAsync(mh, mm, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) {
            fail(e, "seeding step");
            break;
        }
        ++steps;
        std::swap(X, Xn);
        double move = 0.0;
        std::memcpy(&move, mh, sizeof move);
        if (!(move < INFINITY)) {
            set_last_error_msg("gmi_seed_sphere_repulsive: coincident points (non-finite move)");
            status = GMI_ERR_NONFINITE;
            break;
        }
        if (move <= kSeedMove) {
            converged = true;
            break;
        }
    }
    if (status == GMI_OK &&
        (e = cudaMemcpyAsync(refs_out_h, X, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        fail(e, "cudaMemcpyAsync");
    if (status == GMI_OK && (e = cudaStreamSynchronize(st)) != cudaSuccess) fail(e, "cudaStreamSynchronize");
    if (X) dev_free(X);
    if (Xn) dev_free(Xn);
    if (F) dev_free(F);
    if (mm) dev_free(mm);
    if (mh) host_free(mh);
    cudaStreamDestroy(st);
    if (steps_out) *steps_out = steps;
    if (status == GMI_OK && !converged) {
        set_last_error_msg("gmi_seed_sphere_repulsive: not settled within max_steps");
        return GMI_ERR_NOT_CONVERGED;
    }
    return status;
}
