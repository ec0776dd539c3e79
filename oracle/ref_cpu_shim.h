/*
 * ref_cpu_shim.h -- lets the reference's CUDA kernel source
 * (cuda_functions.cu, read where it lies in the reference tree) compile as
 * plain C++ for the CPU.  TEST INFRASTRUCTURE ONLY: the product never
 * includes this header.
 *
 * Execution model: every kernel is launched with blockDim.x == 1 and one
 * block per target (THREADS_PER_BLOCK is 1 in ref_kernels_config.h), so
 * each block's __syncthreads() is a no-op and its shared-memory tile holds a
 * single source.  The per-target summation order is then the reference's
 * own (sources in index order), and the pair arithmetic is the reference's
 * own source text, in FP64.  Blocks may run on different host threads: the
 * built-in index variables and the __shared__ arrays are thread_local.
 *
 * This header must be force-included (-include) before the reference file,
 * together with ref_kernels_config.h, whose include guard replaces the
 * reference's config.hpp.
 */
#ifndef GMI_REF_CPU_SHIM_H
#define GMI_REF_CPU_SHIM_H

#include <cmath>
#include <cstdlib>
#include <algorithm>

using std::abs;
using std::fmin;
using std::sqrt;

struct ref_dim3 {
    int x, y, z;
};

extern thread_local ref_dim3 threadIdx;
extern thread_local ref_dim3 blockIdx;
extern thread_local ref_dim3 blockDim;
extern thread_local ref_dim3 gridDim;

#define __global__
#define __device__
#define __host__
#define __shared__ static thread_local
#define __syncthreads() ((void)0)

#endif
