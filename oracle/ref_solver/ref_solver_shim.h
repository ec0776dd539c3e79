/*
 * ref_solver_shim.h -- force-included before every reference source in the
 * CPU build of the reference's own simulator (build_ref_solver.py).
 * TEST INFRASTRUCTURE ONLY.
 *
 *  - std::random_device (filament.cpp's initial perturbation) becomes a
 *    default-seeded std::minstd_rand, so runs are reproducible;
 *  - std::setprecision(n) in the reference's writers becomes 17 digits, so
 *    the .dat/.backup files carry full FP64 state;
 *  - rpy_mobility_solver (rpy_mobility_solver.hpp, CUDA) is replaced by the
 *    CPU class in cpu_rpy_mobility_solver.hpp through its include guard.
 */
#ifndef GMI_REF_SOLVER_SHIM_H
#define GMI_REF_SOLVER_SHIM_H

#include <iomanip>
#include <random>

#define random_device minstd_rand
#define setprecision(n) setprecision(17)

#include "cpu_rpy_mobility_solver.hpp"

#endif
