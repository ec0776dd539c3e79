// gb300_mobility_solver.hpp -- the reference-side binding of libgmi.
//
// A drop-in backend for the reference simulator's abstract mobility_solver
// (mobility_solver.hpp:18-102), to be compiled inside the reference tree
// next to rpy_mobility_solver.hpp.  It implements the 15 pure virtuals by
// forwarding to the C ABI in include/gmi.h, and points the base class's
// host arrays (v_segs_host, x_segs_host, ...) at the solver's pinned arrays,
// which the reference's filaments and bodies write in place
// (cilia_sim_main.cpp:141-144).  The reference's own host GMRES then runs
// unchanged on top of the GB300 kernels.
//
// compute_velocities_on_device() and make_body_reference_matrices_on_device()
// are the device-resident fast path (GMRES, preconditioner and the K, K^T
// products on the GPU).  mobility_solver::compute_velocities is not virtual in
// the reference, so the driver calls these two in place of
// mobility.compute_velocities / mobility.make_body_reference_matrices
// (cilia_sim_main.cpp:159, 216, 292).
#ifndef GB300_MOBILITY_SOLVER_HEADER_INCLUDED
#define GB300_MOBILITY_SOLVER_HEADER_INCLUDED

#include <vector>

#include "gmi.h"
#include "mobility_solver.hpp"

class swimmer;

class gb300_mobility_solver : public mobility_solver {
public:
    // the base class's pure virtuals (mobility_solver.hpp:25-44)
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

    // device-resident generic methods
    void compute_velocities_on_device(std::vector<swimmer> &swimmers, int &num_gmres_iterations, const int nt);
    void make_body_reference_matrices_on_device(std::vector<swimmer> &swimmers);

    // GMI_FP64 reproduces the reference's arithmetic; GMI_FP32C is the
    // mixed-precision mode.  Set before initialise().
    int precision = GMI_FP64;
    gmi_solver *solver = nullptr;

    ~gb300_mobility_solver();
    gb300_mobility_solver();

private:
    bool blob_refs_set = false;
    bool gen_force_refs_set = false;
#if PRESCRIBED_CILIA
    void compute_velocities_prescribed_on_device(std::vector<swimmer> &swimmers, int &num_gmres_iterations);
#endif
    void check(gmi_status st, const char *what) const;
    void ensure_blob_references(const std::vector<swimmer> &swimmers);
};

#endif
