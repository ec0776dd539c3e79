/*
 * ref_kernels_driver.cpp -- C entry points that run the reference's own
 * kernels (cuda_functions.cu, compiled for the CPU through ref_cpu_shim.h)
 * over every target.  TEST INFRASTRUCTURE ONLY: used to pin the oracle
 * restatement (rpy_oracle.c) and to generate the golden fixtures.
 *
 * Launch shape: blockDim = 1, one block per target, blocks spread over host
 * threads with OpenMP.  The reference's grid-stride loop then visits target
 * i = blockIdx.x once, exactly as a <<<n, 1>>> launch would.
 */
#include "ref_cpu_shim.h"
#include "ref_kernels_config.h"

#include "cuda_functions.hpp"

thread_local ref_dim3 threadIdx = {0, 0, 0};
thread_local ref_dim3 blockIdx = {0, 0, 0};
thread_local ref_dim3 blockDim = {1, 1, 1};
thread_local ref_dim3 gridDim = {1, 1, 1};

int ref_nswim = 1, ref_nfil = 1, ref_nseg = 1, ref_nblob = 0;
double ref_rseg = 1.0, ref_rblob = 1.0, ref_mu = 1.0;
double ref_repulsive_force_factor = 1.0, ref_end_force_magnitude = 1.0;

template <class F>
static void launch(int nblocks, F &&body)
{
#pragma omp parallel for schedule(dynamic, 8)
    for (int b = 0; b < nblocks; ++b) {
        threadIdx = {0, 0, 0};
        blockIdx = {b, 0, 0};
        blockDim = {1, 1, 1};
        gridDim = {nblocks, 1, 1};
        body();
    }
}

extern "C" {

/* nseg_per_fil * nfil * nswim = S segments, nblob * nswim = B blobs. */
void ref_set_problem(int nswim, int nfil, int nseg, int nblob, double rseg, double rblob,
                     double mu, double repulsive_force_factor, double end_force_magnitude)
{
    ref_nswim = nswim;
    ref_nfil = nfil;
    ref_nseg = nseg;
    ref_nblob = nblob;
    ref_rseg = rseg;
    ref_rblob = rblob;
    ref_mu = mu;
    ref_repulsive_force_factor = repulsive_force_factor;
    ref_end_force_magnitude = end_force_magnitude;
}

int ref_is_wall_build(void) { return REF_WALL; }

void ref_mss(double *v, const double *f, const double *x)
{
    const int n = ref_nswim * ref_nfil * ref_nseg;
    launch(n, [&] { Mss_mult(v, f, x, 0, n); });
}

void ref_mbb(double *v, const double *f, const double *x)
{
    const int n = ref_nswim * ref_nblob;
    launch(n, [&] { Mbb_mult(v, f, x, 0, n); });
}

void ref_msb(double *v, const double *fb, const double *xs, const double *xb)
{
    const int n = ref_nswim * ref_nfil * ref_nseg;
    launch(n, [&] { Msb_mult(v, fb, xs, xb, 0, n); });
}

void ref_mbs(double *v, const double *fs, const double *xb, const double *xs)
{
    const int n = ref_nswim * ref_nblob;
    launch(n, [&] { Mbs_mult(v, fs, xb, xs, 0, n); });
}

void ref_barrier(double *fs, double *fbrep, const double *xs, const double *xb)
{
    const int S = ref_nswim * ref_nfil * ref_nseg;
    const int B = ref_nswim * ref_nblob;
    const int n = S > B ? S : B;
    launch(n, [&] { barrier_forces(fs, fbrep, xs, xb, 0, S, 0, B); });
}

} /* extern "C" */
