// gb300_mobility_solver.cpp -- see gb300_mobility_solver.hpp.
//
// Compiled inside the reference tree (it includes the reference's config.hpp,
// mobility_solver.hpp, swimmer.hpp) and linked against libgmi.so.
#include "gb300_mobility_solver.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "config.hpp"
#include "swimmer.hpp"

gb300_mobility_solver::gb300_mobility_solver() {}
gb300_mobility_solver::~gb300_mobility_solver() {}

void gb300_mobility_solver::check(gmi_status st, const char *what) const
{
    if (st != GMI_OK) {
        // the reference has no error channel on these void methods; stop loudly
        std::fprintf(stderr, "gb300_mobility_solver: %s failed (status %d): %s\n", what, (int)st, gmi_last_error());
        std::exit(EXIT_FAILURE);
    }
}

// allocate_host_memory + allocate_device_memory (rpy_mobility_solver.cu:55-115):
// one gmi_solver owns both the pinned host arrays and the device state.
void gb300_mobility_solver::allocate_host_memory()
{
    gmi_solver_config cfg;
    std::memset(&cfg, 0, sizeof cfg);
    cfg.nswim = NSWIM;
    cfg.nfil = NFIL;
    cfg.nseg = NSEG;
    cfg.nblob = NBLOB;
    cfg.mu = MU;
    cfg.rseg = RSEG;
    cfg.rblob = RBLOB;
#if defined(REPULSIVE_FORCE_FACTOR) && defined(END_FORCE_MAGNITUDE)
    cfg.repulsive_force_factor = REPULSIVE_FORCE_FACTOR;
    cfg.end_force_magnitude = END_FORCE_MAGNITUDE;
#else
    // prescribed-shape cilia define no barrier (mobility_solver.cpp:152-163
    // skips it); the solver's defaults stand in, unused
    cfg.repulsive_force_factor = 2.0;
    cfg.end_force_magnitude = 1.0;
#endif
    cfg.wall = INFINITE_PLANE_WALL;
#if USE_GMRES_FOR_LINEAR_SYSTEM
    cfg.max_linear_iter = MAX_LINEAR_SYSTEM_ITER;
    cfg.linear_tol = LINEAR_SYSTEM_TOL;
#endif
    cfg.precision = precision;
    cfg.device = 0;
    check(gmi_solver_create(&cfg, &solver), "gmi_solver_create");
    gmi_host_arrays h;
    check(gmi_solver_host_arrays(solver, &h), "gmi_solver_host_arrays");
    v_segs_host = h.v_segs_host;
    v_blobs_host = h.v_blobs_host;
    x_segs_host = h.x_segs_host;
    x_blobs_host = h.x_blobs_host;
    f_segs_host = h.f_segs_host;
    f_blobs_host = h.f_blobs_host;
    f_blobs_repulsion_host = h.f_blobs_repulsion_host;
}

void gb300_mobility_solver::allocate_device_memory() {}

void gb300_mobility_solver::free_host_memory()
{
    gmi_solver_destroy(solver);
    solver = nullptr;
}

void gb300_mobility_solver::free_device_memory() {}

void gb300_mobility_solver::copy_segment_positions_to_device()
{
    check(gmi_solver_copy_segment_positions_to_device(solver), "copy_segment_positions_to_device");
}
void gb300_mobility_solver::copy_segment_forces_to_device()
{
    check(gmi_solver_copy_segment_forces_to_device(solver), "copy_segment_forces_to_device");
}
void gb300_mobility_solver::copy_blob_positions_to_device()
{
    check(gmi_solver_copy_blob_positions_to_device(solver), "copy_blob_positions_to_device");
}
void gb300_mobility_solver::copy_blob_forces_to_device()
{
    check(gmi_solver_copy_blob_forces_to_device(solver), "copy_blob_forces_to_device");
}
void gb300_mobility_solver::copy_interparticle_blob_forces_to_host()
{
    check(gmi_solver_copy_interparticle_blob_forces_to_host(solver), "copy_interparticle_blob_forces_to_host");
}
void gb300_mobility_solver::copy_blob_velocities_to_host()
{
    check(gmi_solver_copy_blob_velocities_to_host(solver), "copy_blob_velocities_to_host");
}
void gb300_mobility_solver::copy_segment_velocities_to_host()
{
    check(gmi_solver_copy_segment_velocities_to_host(solver), "copy_segment_velocities_to_host");
}
void gb300_mobility_solver::apply_interparticle_forces()
{
    check(gmi_solver_apply_interparticle_forces(solver), "apply_interparticle_forces");
}
void gb300_mobility_solver::wait_for_device() { check(gmi_solver_wait_for_device(solver), "wait_for_device"); }
void gb300_mobility_solver::evaluate_segment_segment_mobility()
{
    check(gmi_solver_evaluate_segment_segment_mobility(solver), "evaluate_segment_segment_mobility");
}
void gb300_mobility_solver::evaluate_segment_blob_mobility()
{
    check(gmi_solver_evaluate_segment_blob_mobility(solver), "evaluate_segment_blob_mobility");
}
void gb300_mobility_solver::evaluate_blob_blob_mobility()
{
    check(gmi_solver_evaluate_blob_blob_mobility(solver), "evaluate_blob_blob_mobility");
}
void gb300_mobility_solver::evaluate_blob_segment_mobility()
{
    check(gmi_solver_evaluate_blob_segment_mobility(solver), "evaluate_blob_segment_mobility");
}

// Gathers the body state the device solve needs from the swimmers.
static void gather_bodies(const std::vector<swimmer> &swimmers, std::vector<double> &x, std::vector<double> &q,
                          std::vector<double> &f)
{
    const size_t W = swimmers.size();
    x.resize(3 * W);
    q.resize(4 * W);
    f.resize(6 * W);
    for (size_t n = 0; n < W; ++n) {
        const rigid_body &b = swimmers[n].body;
        for (int c = 0; c < 3; ++c) x[3 * n + c] = b.x[c];
        q[4 * n] = b.q.scalar_part;
        for (int c = 0; c < 3; ++c) q[4 * n + 1 + c] = b.q.vector_part[c];
        for (int c = 0; c < 6; ++c) f[6 * n + c] = swimmers[n].f(c);
    }
}

// The swimmers are identical (cilia_sim_main.cpp:154): swimmer 0's blob
// references serve all of them.
void gb300_mobility_solver::ensure_blob_references(const std::vector<swimmer> &swimmers)
{
    if (blob_refs_set || NBLOB == 0) return;
    check(gmi_solver_set_blob_references(solver, &swimmers[0].body.blob_references[0]),
          "gmi_solver_set_blob_references");
    blob_refs_set = true;
}

// mobility_solver::compute_velocities (mobility_solver.cpp:1358-1402) with the
// linear solve on the device.  Like the reference it adds the blob repulsion
// to each swimmer's force/torque (mobility_solver.cpp:166-188) and leaves the
// solution in f_blobs_host and v_bodies.
void gb300_mobility_solver::compute_velocities_on_device(std::vector<swimmer> &swimmers, int &num_gmres_iterations,
                                                         const int nt)
{
    (void)nt;
#if PRESCRIBED_CILIA
    compute_velocities_prescribed_on_device(swimmers, num_gmres_iterations);
    return;
#endif
    ensure_blob_references(swimmers);
    std::vector<double> x, q, f;
    gather_bodies(swimmers, x, q, f);
    check(gmi_solver_compute_velocities(solver, x.data(), q.data(), f.data(), &num_gmres_iterations),
          "gmi_solver_compute_velocities");
    for (size_t n = 0; n < swimmers.size(); ++n)
        for (int c = 0; c < 6; ++c) swimmers[n].f(c) = f[6 * n + c];
#if !USE_BROYDEN_FOR_EVERYTHING
    if (v_bodies.num_rows == 6 * NSWIM)
        check(gmi_solver_get_v_bodies(solver, &v_bodies.data[0]), "gmi_solver_get_v_bodies");
#endif
}

#if PRESCRIBED_CILIA
// mobility_solver::compute_velocities for prescribed-shape cilia
// (mobility_solver.cpp:1362-1369): the filaments' shape-velocity directions
// and phase speeds go to the device solve; the segment forces land in
// f_segs_host, the blob forces in f_blobs_host, the body velocities in
// v_bodies.  With DYNAMIC_PHASE_EVOLUTION the phase speeds are unknowns: the
// generalised-force table the base class read (mobility_solver.cpp:37-65) is
// handed over once, and the solved speeds are written back to the filaments
// (mobility_solver.cpp:1306-1320).
void gb300_mobility_solver::compute_velocities_prescribed_on_device(std::vector<swimmer> &swimmers,
                                                                    int &num_gmres_iterations)
{
    ensure_blob_references(swimmers);
    std::vector<double> x, q, f;
    gather_bodies(swimmers, x, q, f);
    const size_t F = swimmers.size() * NFIL;
    std::vector<double> vel_dir(3 * NSEG * F), speed(F), phase(F), omega0(F);
    for (size_t n = 0; n < swimmers.size(); ++n)
        for (int i = 0; i < NFIL; ++i) {
            const filament &fil = swimmers[n].filaments[i];
            const size_t k = n * NFIL + i;
            for (int m = 0; m < 3 * NSEG; ++m) vel_dir[3 * NSEG * k + m] = fil.vel_dir[m];
            speed[k] = fil.phase_speed;
            phase[k] = fil.phase;
            omega0[k] = fil.omega0;
        }
#if DYNAMIC_PHASE_EVOLUTION
    if (!gen_force_refs_set) {
        check(gmi_solver_set_generalised_force_refs(solver, gen_force_refs.data(), (int)gen_force_refs.size()),
              "gmi_solver_set_generalised_force_refs");
        gen_force_refs_set = true;
    }
    check(gmi_solver_compute_velocities_prescribed_dynamic(solver, x.data(), q.data(), vel_dir.data(), phase.data(),
                                                           omega0.data(), speed.data(), &num_gmres_iterations),
          "gmi_solver_compute_velocities_prescribed_dynamic");
    for (size_t n = 0; n < swimmers.size(); ++n)
        for (int i = 0; i < NFIL; ++i) swimmers[n].filaments[i].phase_speed = speed[n * NFIL + i];
#else
    check(gmi_solver_compute_velocities_prescribed(solver, x.data(), q.data(), vel_dir.data(), speed.data(),
                                                   &num_gmres_iterations),
          "gmi_solver_compute_velocities_prescribed");
#endif
    if (v_bodies.num_rows == 6 * NSWIM)
        check(gmi_solver_get_v_bodies(solver, &v_bodies.data[0]), "gmi_solver_get_v_bodies");
}
#endif

// mobility_solver::make_body_reference_matrices (mobility_solver.cpp:1693-1771)
// on the device; the matrices land in the base class's members.
void gb300_mobility_solver::make_body_reference_matrices_on_device(std::vector<swimmer> &swimmers)
{
#if !USE_BROYDEN_FOR_EVERYTHING
    ensure_blob_references(swimmers);
    std::vector<double> x, q, f;
    gather_bodies(swimmers, x, q, f);
    double ktk[36], mob[36];
    check(gmi_solver_make_body_reference_matrices(solver, x.data(), q.data(), ktk, mob),
          "gmi_solver_make_body_reference_matrices");
    for (int i = 0; i < 36; ++i) {
        KTKinv_reference.data[i] = ktk[i];
        body_mobility_reference.data[i] = mob[i];
    }
#else
    (void)swimmers;
#endif
}
