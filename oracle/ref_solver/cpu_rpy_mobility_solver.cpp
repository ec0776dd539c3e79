/*
 * cpu_rpy_mobility_solver.cpp -- see cpu_rpy_mobility_solver.hpp.
 * Mirrors rpy_mobility_solver.cu:14-311 on one "GPU" that is the host.
 * TEST INFRASTRUCTURE ONLY.
 */
#include <algorithm>
#include <cstring>

#include "ref_cpu_shim.h"
#include "config.hpp"
#include "cuda_functions.hpp"
#include "cpu_rpy_mobility_solver.hpp"

thread_local ref_dim3 threadIdx = {0, 0, 0};
thread_local ref_dim3 blockIdx = {0, 0, 0};
thread_local ref_dim3 blockDim = {1, 1, 1};
thread_local ref_dim3 gridDim = {1, 1, 1};

// <<<n, 1>>>: one single-thread block per target, spread over host threads.
template <class F> static void launch(int nblocks, F &&body)
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

static const int S_TOT = NSWIM * NFIL * NSEG;
static const int B_TOT = NSWIM * NBLOB;

rpy_mobility_solver::rpy_mobility_solver() {}
rpy_mobility_solver::~rpy_mobility_solver() {}

void rpy_mobility_solver::allocate_host_memory()
{
    v_segs_host = new double[6 * S_TOT + 1];
    v_blobs_host = new double[3 * B_TOT + 1];
    x_segs_host = new double[3 * S_TOT + 1];
    x_blobs_host = new double[3 * B_TOT + 1];
    f_segs_host = new double[6 * S_TOT + 1];
    f_blobs_host = new double[3 * B_TOT + 1];
    f_blobs_repulsion_host = new double[3 * B_TOT + 1];
}

void rpy_mobility_solver::allocate_device_memory()
{
    v_segs_dev = new double[6 * S_TOT + 1];
    v_blobs_dev = new double[3 * B_TOT + 1];
    x_segs_dev = new double[3 * S_TOT + 1];
    x_blobs_dev = new double[3 * B_TOT + 1];
    f_segs_dev = new double[6 * S_TOT + 1];
    f_blobs_dev = new double[3 * B_TOT + 1];
    f_blobs_repulsion_dev = new double[3 * B_TOT + 1];
}

void rpy_mobility_solver::free_host_memory()
{
    delete[] v_segs_host; delete[] v_blobs_host; delete[] x_segs_host; delete[] x_blobs_host;
    delete[] f_segs_host; delete[] f_blobs_host; delete[] f_blobs_repulsion_host;
}

void rpy_mobility_solver::free_device_memory()
{
    delete[] v_segs_dev; delete[] v_blobs_dev; delete[] x_segs_dev; delete[] x_blobs_dev;
    delete[] f_segs_dev; delete[] f_blobs_dev; delete[] f_blobs_repulsion_dev;
}

void rpy_mobility_solver::copy_segment_positions_to_device() { std::memcpy(x_segs_dev, x_segs_host, 3 * S_TOT * sizeof(double)); }
void rpy_mobility_solver::copy_segment_forces_to_device() { std::memcpy(f_segs_dev, f_segs_host, 6 * S_TOT * sizeof(double)); }
void rpy_mobility_solver::copy_blob_positions_to_device() { std::memcpy(x_blobs_dev, x_blobs_host, 3 * B_TOT * sizeof(double)); }
void rpy_mobility_solver::copy_blob_forces_to_device() { std::memcpy(f_blobs_dev, f_blobs_host, 3 * B_TOT * sizeof(double)); }
void rpy_mobility_solver::copy_interparticle_blob_forces_to_host() { std::memcpy(f_blobs_repulsion_host, f_blobs_repulsion_dev, 3 * B_TOT * sizeof(double)); }
void rpy_mobility_solver::copy_blob_velocities_to_host() { std::memcpy(v_blobs_host, v_blobs_dev, 3 * B_TOT * sizeof(double)); }
void rpy_mobility_solver::copy_segment_velocities_to_host() { std::memcpy(v_segs_host, v_segs_dev, 6 * S_TOT * sizeof(double)); }

void rpy_mobility_solver::apply_interparticle_forces()
{
    const int n = std::max(S_TOT, B_TOT);
    launch(n, [&] { barrier_forces(f_segs_dev, f_blobs_repulsion_dev, x_segs_dev, x_blobs_dev, 0, S_TOT, 0, B_TOT); });
}

void rpy_mobility_solver::wait_for_device() {}

void rpy_mobility_solver::evaluate_segment_segment_mobility()
{
    launch(S_TOT, [&] { Mss_mult(v_segs_dev, f_segs_dev, x_segs_dev, 0, S_TOT); });
}

void rpy_mobility_solver::evaluate_segment_blob_mobility()
{
    launch(S_TOT, [&] { Msb_mult(v_segs_dev, f_blobs_dev, x_segs_dev, x_blobs_dev, 0, S_TOT); });
}

void rpy_mobility_solver::evaluate_blob_blob_mobility()
{
    launch(B_TOT, [&] { Mbb_mult(v_blobs_dev, f_blobs_dev, x_blobs_dev, 0, B_TOT); });
}

void rpy_mobility_solver::evaluate_blob_segment_mobility()
{
    launch(B_TOT, [&] { Mbs_mult(v_blobs_dev, f_segs_dev, x_blobs_dev, x_segs_dev, 0, B_TOT); });
}
