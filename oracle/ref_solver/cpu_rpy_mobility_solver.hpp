/*
 * cpu_rpy_mobility_solver.hpp -- a CPU stand-in for the reference's CUDA
 * rpy_mobility_solver (rpy_mobility_solver.hpp:15-63), with the same 15
 * overrides of mobility_solver.hpp:25-44.  Host and "device" arrays are plain
 * heap arrays; the evaluate_* / barrier calls run the reference's own kernels
 * (cuda_functions.cu, compiled for the CPU through ../ref_cpu_shim.h) with
 * one-thread blocks.  TEST INFRASTRUCTURE ONLY.
 */
#ifndef MY_RPY_MOBILITY_SOLVER_HEADER_INCLUDED
#define MY_RPY_MOBILITY_SOLVER_HEADER_INCLUDED

#include "mobility_solver.hpp"

class rpy_mobility_solver : public mobility_solver {
public:
    void free_host_memory();
    void free_device_memory();
    void allocate_host_memory();
    void allocate_device_memory();

    void copy_segment_positions_to_device();
    void copy_segment_forces_to_device();
    void copy_blob_positions_to_device();
    void copy_blob_forces_to_device();

    void copy_interparticle_blob_forces_to_host();
    void copy_blob_velocities_to_host();
    void copy_segment_velocities_to_host();

    void apply_interparticle_forces();
    void wait_for_device();
    void evaluate_segment_segment_mobility();
    void evaluate_segment_blob_mobility();
    void evaluate_blob_blob_mobility();
    void evaluate_blob_segment_mobility();

    double *v_segs_dev, *v_blobs_dev, *x_segs_dev, *x_blobs_dev, *f_segs_dev, *f_blobs_dev, *f_blobs_repulsion_dev;

    ~rpy_mobility_solver();
    rpy_mobility_solver();
};

#endif
