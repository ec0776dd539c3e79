/*
 * gmi.h -- C ABI of the GB300 mobility library (libgmi.so).
 *
 * The library is a drop-in for the GPU half of the reference's
 * rpy_mobility_solver (rpy_mobility_solver.{hpp,cu}) and for the generic
 * mobility_solver methods that consume it (mobility_solver.cpp).  Every entry
 * point takes plain pointers and sizes, returns a gmi_status, and never
 * exits the process.  Device pointers are marked _d; host pointers _h.
 *
 * Precision: GMI_FP64 evaluates the pair sums in FP64 like the reference;
 * GMI_FP32C evaluates them in FP32 with double-float source positions and
 * compensated (two-sum) accumulation, and returns FP64 results; GMI_DF64
 * (blob-blob only) carries every step of the pair formula as a double-float
 * (hi, lo) FP32 pair, FP64-grade accuracy on the FP32 pipe.
 */
#ifndef GMI_H
#define GMI_H

#if defined(__GNUC__)
#define GMI_API __attribute__((visibility("default")))
#else
#define GMI_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gmi_status {
    GMI_OK = 0,
    GMI_ERR_ARG = 1,            /* bad size, null pointer, unsupported option */
    GMI_ERR_CUDA = 2,           /* a CUDA runtime call failed (see gmi_last_error) */
    GMI_ERR_DEVICE_TIMEOUT = 3, /* a kernel's bounded wait gave up; results invalid */
    GMI_ERR_NONFINITE = 4,      /* NaN/Inf met where the reference would diverge */
    GMI_ERR_NOT_CONVERGED = 5,  /* an iterative solve hit its iteration cap */
    GMI_ERR_STATE = 6           /* call out of order (e.g. solve before setup) */
} gmi_status;

typedef enum gmi_precision {
    GMI_FP64 = 0,  /* reference arithmetic */
    GMI_FP32C = 1, /* FP32 pair math, compensated accumulation, FP64 I/O */
    GMI_DF64 = 2   /* double-float (FP32 hi/lo pairs) pair math, ~1e-13, FP64 I/O;
                      gmi_Mbb_mult only (other pair sums return GMI_ERR_ARG) */
} gmi_precision;

/* Message describing the last failure on the calling thread ("" if none). */
GMI_API const char *gmi_last_error(void);
/* Library version: major*10000 + minor*100 + patch. */
GMI_API int gmi_version(void);

/* ------------------------------------------------------------------------
 * Context: one GPU, one CUDA stream, scratch memory that grows on demand,
 * the launch-shape cache of the autotuner, and a device error word.
 * (The reference keeps the equivalent state in rpy_mobility_solver's
 * members, rpy_mobility_solver.hpp:45-58.)
 *
 * Threads: separate contexts (and the solvers and simulations built on
 * them) may be driven from separate host threads at once; the library
 * serialises graph captures with device-wide synchronising allocations and
 * only ever raises a kernel's shared-memory limit.  One handle must not be
 * used from two threads at once.
 * ---------------------------------------------------------------------- */
typedef struct gmi_context gmi_context;

GMI_API gmi_status gmi_context_create(int device, gmi_context **out);
GMI_API gmi_status gmi_context_destroy(gmi_context *ctx);
/* Use an existing cudaStream_t (passed as void*); NULL selects the context's
 * own non-blocking stream.  For the legacy default stream pass
 * cudaStreamLegacy ((void*)1): work there is ordered with the caller's
 * default-stream copies. */
GMI_API gmi_status gmi_context_set_stream(gmi_context *ctx, void *cuda_stream);
GMI_API gmi_status gmi_context_set_precision(gmi_context *ctx, int precision);
GMI_API int gmi_context_precision(const gmi_context *ctx);
/* Block until the context's stream drains; reports device-side errors
 * (bounded-wait timeouts) recorded since the last call.
 * Replaces rpy_mobility_solver::wait_for_device (rpy_mobility_solver.cu:230-239). */
GMI_API gmi_status gmi_context_synchronize(gmi_context *ctx);
/* Number of library kernels launched on this context so far. */
GMI_API long long gmi_context_launch_count(const gmi_context *ctx);
/* Deadline of the pair kernels' bounded waits on their source tiles, in
 * nanoseconds of the GPU's global timer: a wait that runs past it makes the
 * kernel record a timeout and return, and the next synchronising call
 * reports GMI_ERR_DEVICE_TIMEOUT.  0 restores the default (2 s); otherwise
 * 1 us .. 60 s.  A launch captured in a CUDA graph keeps the deadline it was
 * captured with.  The reference's kernels have no waits to bound. */
GMI_API gmi_status gmi_context_set_wait_deadline(gmi_context *ctx, long long nanoseconds);
/* Check of the bounded-wait machinery: one CTA waits, through the pair
 * kernels' bounded wait and the context's deadline, on an mbarrier that
 * expects two arrivals.  withhold_arrival 0: both arrive, GMI_OK.
 * withhold_arrival 1: one never arrives, the wait gives up at the deadline
 * and the call returns GMI_ERR_DEVICE_TIMEOUT; the context stays usable.
 * Synchronises the context stream.  No counterpart in the reference. */
GMI_API gmi_status gmi_context_check_bounded_wait(gmi_context *ctx, int withhold_arrival);

/* ------------------------------------------------------------------------
 * Pair sums on device arrays, in the reference's layouts (FP64, AoS):
 *   X segs [3*S], F segs [6*S] = (f, tau), V segs [6*S] = (v, omega)
 *   X blobs [3*B], F blobs [3*B], V blobs [3*B]
 * Targets are [start, start+num) of their set; V is indexed from `start`
 * (V[0] belongs to target `start`), as in the reference kernels.  All
 * calls are asynchronous on the context stream.
 * ---------------------------------------------------------------------- */

/* V = M_ss F: segment <- segment, free space.  Replaces Mss_mult
 * (cuda_functions.cu:246-425, launched at rpy_mobility_solver.cu:241-255). */
GMI_API gmi_status gmi_Mss_mult(gmi_context *ctx, double *V_d, const double *F_d, const double *X_d,
                        int start_seg, int num_segs, int total_segs, double rseg, double mu);

/* V = M_ss F above a no-slip wall at z = 0 (Swan & Brady); a = mu = 1 as in
 * the reference.  Replaces the INFINITE_PLANE_WALL Mss_mult
 * (cuda_functions.cu:10-242). */
GMI_API gmi_status gmi_Mss_mult_wall(gmi_context *ctx, double *V_d, const double *F_d, const double *X_d,
                             int start_seg, int num_segs, int total_segs);

/* V = M_bb F: blob <- blob.  Replaces Mbb_mult (cuda_functions.cu:429-539,
 * launched at rpy_mobility_solver.cu:277-291). */
GMI_API gmi_status gmi_Mbb_mult(gmi_context *ctx, double *V_d, const double *F_d, const double *X_d,
                        int start_blob, int num_blobs, int total_blobs, double rblob, double mu);

/* V += M_sb F_blobs: segment <- blob (accumulates, as the reference).
 * Replaces Msb_mult (cuda_functions.cu:541-694, rpy_mobility_solver.cu:259-273). */
GMI_API gmi_status gmi_Msb_mult(gmi_context *ctx, double *V_d, const double *F_blobs_d, const double *Xs_d,
                        const double *Xb_d, int start_seg, int num_segs, int total_segs,
                        int total_blobs, double rseg, double rblob, double mu);

/* V = M_bs F_segs: blob <- segment (overwrites).  Replaces Mbs_mult
 * (cuda_functions.cu:697-863, rpy_mobility_solver.cu:295-309). */
GMI_API gmi_status gmi_Mbs_mult(gmi_context *ctx, double *V_d, const double *F_segs_d, const double *Xb_d,
                        const double *Xs_d, int start_blob, int num_blobs, int total_blobs,
                        int total_segs, double rseg, double rblob, double mu);

/* Allocation-free form of gmi_Mss_mult, for callers that cannot call
 * cudaMalloc: programs that fix their device-memory budget at start-up and
 * hand it all to their own allocator, or that cannot accept the device-wide
 * synchronisation cudaMalloc/cudaFree imply.  It needs no gmi_context:
 * scratch comes from a 16 MiB array compiled into the library, which every
 * GPU that loads the library holds until process exit.  Limit:
 * total_segs <= 32768 (larger problems return GMI_ERR_ARG).  precision is a
 * gmi_precision; cuda_stream a cudaStream_t (NULL = legacy default stream).
 * The first call in each CUDA context (the device's primary context, or a
 * context the caller made current) looks up the array's device address in
 * that context; make it before any stream capture.  All calls share the
 * array, so calls that overlap on the GPU race.  Returns when V is complete.
 * No counterpart in the reference. */
GMI_API gmi_status gmi_Mss_mult_noalloc(double *V_d, const double *F_d, const double *X_d, int start_seg,
                                        int num_segs, int total_segs, double rseg, double mu, int precision,
                                        void *cuda_stream);

/* Short-range barrier forces.  Segment targets ADD into f_segs[6*i+0..2];
 * blob targets OVERWRITE f_blobs_repulsion[3*(i-start_blob)..] (skipped when
 * wall != 0, as with the reference's prescribed wall bodies).  Segments
 * i, j of one filament (nseg per filament) with |i-j| <= 1 do not repel.
 * force_scale = REPULSIVE_FORCE_FACTOR * END_FORCE_MAGNITUDE.
 * Replaces barrier_forces (cuda_functions.cu:961-1157,
 * rpy_mobility_solver.cu:207-228). */
GMI_API gmi_status gmi_barrier_forces(gmi_context *ctx, double *f_segs_d, double *f_blobs_repulsion_d,
                              const double *x_segs_d, const double *x_blobs_d, int start_seg,
                              int num_segs, int start_blob, int num_blobs, int total_segs,
                              int total_blobs, int nseg_per_filament, double rseg, double rblob,
                              double force_scale, int wall);

/* Autotuner: time the candidate launch shapes of one pair kernel for the
 * given sizes on the context's GPU and keep the fastest for later calls.
 * kind: 0 = ss, 1 = ss wall, 2 = bb, 3 = sb, 4 = bs. */
GMI_API gmi_status gmi_autotune(gmi_context *ctx, int kind, int num_targets, int num_sources);
/* The launch shape the context will use for this kernel and size:
 * threads per CTA, targets per thread, source splits (0 = automatic).
 * Returns GMI_ERR_STATE if the size was never tuned (defaults apply). */
GMI_API gmi_status gmi_tuned_shape(const gmi_context *ctx, int kind, int num_targets, int num_sources,
                                   int *threads_per_cta, int *targets_per_thread, int *source_splits);
/* Sources one thread takes per step in that shape: 2 for the packed FP32
 * kernel (two sources per f32x2 instruction), 1 otherwise.  Same return
 * convention as gmi_tuned_shape. */
GMI_API gmi_status gmi_tuned_sources_per_step(const gmi_context *ctx, int kind, int num_targets, int num_sources,
                                              int *sources_per_step);
/* Pin the launch shape of one pair kernel and size (what gmi_autotune would
 * store).  threads_per_cta / targets_per_thread: a tiled shape (64, 128 or
 * 256 threads; 1, 2 or 4 targets as the kernel table has them) or 32 for the
 * warp-per-target kernel (1 or 2 targets per warp); source_splits 0 =
 * automatic; sources_per_step 2 (packed) needs FP32 and kind != 1.
 * GMI_ERR_ARG for a shape that has no kernel. */
GMI_API gmi_status gmi_set_shape(gmi_context *ctx, int kind, int num_targets, int num_sources, int threads_per_cta,
                                 int targets_per_thread, int source_splits, int sources_per_step);

/* ------------------------------------------------------------------------
 * Mobility solver: the device-resident replacement of the reference's
 * rpy_mobility_solver plus the generic mobility_solver methods that drive it
 * (mobility_solver.hpp:18-102).  One solver couples nswim swimmers, each a
 * rigid body of nblob blobs with nfil filaments of nseg segments, exactly as
 * the reference's NSWIM/NFIL/NSEG/NBLOB macros do (config.hpp:95-98).
 * ---------------------------------------------------------------------- */
typedef struct gmi_solver gmi_solver;

typedef struct gmi_solver_config {
    int nswim, nfil, nseg, nblob;       /* NSWIM NFIL NSEG NBLOB */
    double mu, rseg, rblob;             /* MU RSEG RBLOB */
    double repulsive_force_factor;      /* REPULSIVE_FORCE_FACTOR */
    double end_force_magnitude;         /* END_FORCE_MAGNITUDE */
    int wall;                           /* INFINITE_PLANE_WALL (then nblob = 0) */
    int max_linear_iter;                /* MAX_LINEAR_SYSTEM_ITER (<= 0: 150) */
    double linear_tol;                  /* LINEAR_SYSTEM_TOL (<= 0: 1e-10) */
    int precision;                      /* pair-sum precision, gmi_precision */
    int device;
} gmi_solver_config;

/* The solver-owned pinned host arrays the filament and body code reads and
 * writes in place (mobility_solver.hpp:54-60; allocated with
 * cudaHostAlloc(..., cudaHostAllocPortable) as rpy_mobility_solver.cu:65-71). */
typedef struct gmi_host_arrays {
    double *v_segs_host;            /* [6*S] */
    double *v_blobs_host;           /* [3*B] */
    double *x_segs_host;            /* [3*S] */
    double *x_blobs_host;           /* [3*B] */
    double *f_segs_host;            /* [6*S] */
    double *f_blobs_host;           /* [3*B] */
    double *f_blobs_repulsion_host; /* [3*B] */
} gmi_host_arrays;

/* allocate_host_memory + allocate_device_memory + mobility_solver::initialise
 * (rpy_mobility_solver.cu:55-115, mobility_solver.cpp:22-130): zeroes the
 * blob forces (the first GMRES warm start) and v_bodies. */
GMI_API gmi_status gmi_solver_create(const gmi_solver_config *cfg, gmi_solver **out);
/* free_host_memory + free_device_memory (rpy_mobility_solver.cu:14-53). */
GMI_API gmi_status gmi_solver_destroy(gmi_solver *s);
GMI_API gmi_status gmi_solver_host_arrays(gmi_solver *s, gmi_host_arrays *out);
/* The solver's context (pair kernels, stream, precision). */
GMI_API gmi_context *gmi_solver_context(gmi_solver *s);

/* The 15 per-backend operations of mobility_solver.hpp:25-44, asynchronous
 * on the solver stream like the reference's cudaMemcpyAsync/launches
 * (rpy_mobility_solver.cu:119-311). */
GMI_API gmi_status gmi_solver_copy_segment_positions_to_device(gmi_solver *s);
GMI_API gmi_status gmi_solver_copy_segment_forces_to_device(gmi_solver *s);
GMI_API gmi_status gmi_solver_copy_blob_positions_to_device(gmi_solver *s);
GMI_API gmi_status gmi_solver_copy_blob_forces_to_device(gmi_solver *s);
GMI_API gmi_status gmi_solver_copy_interparticle_blob_forces_to_host(gmi_solver *s);
GMI_API gmi_status gmi_solver_copy_blob_velocities_to_host(gmi_solver *s);
GMI_API gmi_status gmi_solver_copy_segment_velocities_to_host(gmi_solver *s);
GMI_API gmi_status gmi_solver_apply_interparticle_forces(gmi_solver *s);
GMI_API gmi_status gmi_solver_wait_for_device(gmi_solver *s);
GMI_API gmi_status gmi_solver_evaluate_segment_segment_mobility(gmi_solver *s);
GMI_API gmi_status gmi_solver_evaluate_segment_blob_mobility(gmi_solver *s);
GMI_API gmi_status gmi_solver_evaluate_blob_blob_mobility(gmi_solver *s);
GMI_API gmi_status gmi_solver_evaluate_blob_segment_mobility(gmi_solver *s);

/* Blob positions in the body frame, shared by all swimmers (the reference's
 * rigid_body::blob_references, rigid_body.cpp:184-237), 3*nblob values. */
GMI_API gmi_status gmi_solver_set_blob_references(gmi_solver *s, const double *blob_references_h);

/* mobility_solver::make_body_reference_matrices (mobility_solver.cpp:1693-1771):
 * (K^T K)^-1 from the blob references and the 6x6 body mobility of the last
 * swimmer from six GMRES solves with the other swimmers moved 1e10*DL*NSEG
 * away.  body_x_h[3*nswim], body_q_h[4*nswim] (scalar part first); the
 * segment positions/forces are read from the host arrays.  Outputs (may be
 * NULL): the two 6x6 matrices, column-major like the reference's matrix. */
GMI_API gmi_status gmi_solver_make_body_reference_matrices(gmi_solver *s, const double *body_x_h,
                                                           const double *body_q_h, double *ktkinv_h,
                                                           double *body_mobility_h);
/* Install reference matrices computed elsewhere (e.g. restored state). */
GMI_API gmi_status gmi_solver_set_body_reference_matrices(gmi_solver *s, const double *ktkinv_h,
                                                          const double *body_mobility_h);

/* mobility_solver::compute_velocities (mobility_solver.cpp:1358-1402) with
 * every step on the device: copies x_segs_host/f_segs_host in, blob
 * positions from (body_x_h, body_q_h), barrier forces (the blob part is
 * added into body_f_h[6*nswim] as read_positions_and_forces does,
 * mobility_solver.cpp:166-188), M_ss, M_bs, the right-hand side, GMRES for
 * the blob forces and body velocities, M_sb; then v_segs_host,
 * f_blobs_host, x_blobs_host, f_blobs_repulsion_host and v_blobs_host are
 * written back and the call returns when they are valid.
 * num_gmres_iterations may be NULL. */
GMI_API gmi_status gmi_solver_compute_velocities(gmi_solver *s, const double *body_x_h, const double *body_q_h,
                                                 double *body_f_h, int *num_gmres_iterations);

/* mobility_solver::compute_velocities for prescribed-shape cilia (CILIA_TYPE 3;
 * mobility_solver.cpp:1362-1369 with assemble_rhs :211-310, the preconditioner
 * :427-649, system_matrix_mult :733-905 and swimmer::make_precon_mat,
 * swimmer.cpp:929-1037), free bodies, phases at the caller's speeds: solves
 * for the segment forces, blob forces and body velocities that move the
 * segments (x_segs_host, filled by the caller) at phase_speed[F] times
 * vel_dir[3*S] (the filaments' shape-velocity directions) while the bodies
 * swim force- and torque-free.  Results: f_segs_host (forces; torques 0),
 * f_blobs_host, and the body velocities (gmi_solver_get_v_bodies).  Each
 * solve warm-starts from the previous one; no barrier forces (as the
 * reference). */
GMI_API gmi_status gmi_solver_compute_velocities_prescribed(gmi_solver *s, const double *body_x_h,
                                                            const double *body_q_h, const double *vel_dir_h,
                                                            const double *phase_speed_h, int *gmres_iters);

/* The generalised-force table of the prescribed beat, which the reference's
 * mobility_solver constructor reads from its reference file
 * (mobility_solver.cpp:37-65; written by a WRITE_GENERALISED_FORCES run,
 * cilia_sim_main.cpp:184-246): count samples of sum_k vel_dir_k . f_k of one
 * cilium over one beat period, sample j at phase 2 pi j / count.  count >= 2;
 * count 0 clears the table.  The solver keeps its own copy. */
GMI_API gmi_status gmi_solver_set_generalised_force_refs(gmi_solver *s, const double *refs_h, int count);

/* gmi_solver_compute_velocities_prescribed with the phase speeds among the
 * unknowns (DYNAMIC_PHASE_EVOLUTION; mobility_solver.cpp:219-296, :518-634,
 * :831-866, :1031-1113, :1306-1320; swimmer.cpp:974-1023): each filament's
 * segments move at phase_speed times its vel_dir, and its generalised force
 * sum_k vel_dir_k . f_k equals the table's value at phase[f] (cubic Hermite
 * interpolation) times omega0[f] / (2 pi).  phase_speed_h[F]: on entry the
 * initial guess (the reference uses omega0, filament.cpp:841), on return the
 * solved speeds.  Needs gmi_solver_set_generalised_force_refs first.  The
 * other results are those of gmi_solver_compute_velocities_prescribed; a
 * solve of the other kind than the last one starts cold. */
GMI_API gmi_status gmi_solver_compute_velocities_prescribed_dynamic(gmi_solver *s, const double *body_x_h,
                                                                    const double *body_q_h, const double *vel_dir_h,
                                                                    const double *phase_h, const double *omega0_h,
                                                                    double *phase_speed_h, int *gmres_iters);

/* The last linear solve (GMRES, or in FP32C the mixed-precision refinement):
 * its GMRES iterations and its relative residual |b - A x| / |b| (GMRES's
 * estimate in FP64; the FP64-grade refinement residual in FP32C).  Either
 * pointer may be NULL.  No counterpart in the reference. */
GMI_API gmi_status gmi_solver_last_linear_solve(const gmi_solver *s, int *iterations, double *relative_residual);
/* strict != 0: gmi_solver_compute_velocities returns GMI_ERR_NOT_CONVERGED
 * when the linear solve stopped at max_linear_iter (or, in FP32C, at the
 * refinement cap) with its residual above linear_tol; the results are still
 * written back.  0 (the default) keeps the reference's behaviour, which
 * accepts the capped solve silently (mobility_solver.cpp:1234). */
GMI_API gmi_status gmi_solver_set_strict_convergence(gmi_solver *s, int strict);

/* v_bodies after the last solve: 6*nswim values (U, Omega per swimmer). */
GMI_API gmi_status gmi_solver_get_v_bodies(gmi_solver *s, double *v_bodies_h);
GMI_API gmi_status gmi_solver_set_v_bodies(gmi_solver *s, const double *v_bodies_h);

/* ------------------------------------------------------------------------
 * Implicit time step on the device: the reference's main loop
 * (cilia_sim_main.cpp:205-343) with Broyden's method (broyden_solver.cpp),
 * the swimmer/filament/segment/body state updates and forces (swimmer.cpp,
 * filament.cpp, segment.cpp, rigid_body.cpp), the approximate inverse
 * Jacobian (filament.cpp:1222-1539, swimmer.cpp:329-845) and the residual
 * (mobility_solver.cpp:1404-1689), for free-swimming spherical bodies with
 * end-force-driven filaments (CILIA_TYPE 0) and the GMRES linear solve.
 * ---------------------------------------------------------------------- */
typedef struct gmi_sim gmi_sim;

typedef struct gmi_sim_config {
    gmi_solver_config mobility;   /* sizes, radii, viscosity, barrier scale, GMRES, precision, device */
    double kb, kt;                /* KB, KT */
    double dt;                    /* DT */
    int num_euler_steps;          /* NUM_EULER_STEPS (<= 0: 1) */
    int max_broyden_iter;         /* MAX_BROYDEN_ITER (<= 0: 100) */
    double tol;                   /* TOL (<= 0: 1e-4) */
    double jacobian_confidence;   /* JACOBIAN_CONFIDENCE_FACTOR (<= 0: 0.1) */
    double body_radius;           /* R_OVER_L*DL*NSEG: sphere radius in the approximate Jacobian (swimmer.cpp:607) */
} gmi_sim_config;

/* State fields readable with gmi_sim_get_state (FP64, reference layouts). */
typedef enum gmi_state_field {
    GMI_STATE_SEG_X = 0,  /* [3*S] segment positions */
    GMI_STATE_SEG_Q = 1,  /* [4*S] segment quaternions (scalar first) */
    GMI_STATE_SEG_U = 2,  /* [3*S] segment Lie-algebra updates */
    GMI_STATE_SEG_V = 3,  /* [6*S] segment velocities of the last solve */
    GMI_STATE_SEG_F = 4,  /* [6*S] segment forces/torques of the last solve (before barrier) */
    GMI_STATE_BODY_X = 5, /* [3*W] */
    GMI_STATE_BODY_Q = 6, /* [4*W] */
    GMI_STATE_BODY_U = 7, /* [3*W] */
    GMI_STATE_BODY_V = 8, /* [6*W] body velocities of the last solve */
    GMI_STATE_LAMBDA = 9, /* [3*(nseg-1)*F] inextensibility multipliers */
    GMI_STATE_TETHER = 10, /* [3*F] */
    GMI_STATE_CLAMP = 11,  /* [3*F] */
    GMI_STATE_BLOB_F = 12, /* [3*B] blob forces of the last solve */
    GMI_STATE_SEG_F_INTERNAL = 13 /* [6*S] segment forces without the barrier
                                     (the reference's f_segs_host) */
} gmi_state_field;

/* swimmer::initial_setup for free-swimming spheres (swimmer.cpp:169-230,
 * rigid_body.cpp:184-213, filament.cpp:60-81, 265-323): blob_refs[3*nblob]
 * (body frame, scaled), fil_refs[3*nfil] (filament base relative to the body
 * centre, scaled; the filament stands along it), body_x0[3*nswim];
 * perturb1/perturb2[3*F] (or NULL) are added to segments 4 and 12 at step 0
 * (filament.cpp:1181-1196).
 * With cfg->mobility.wall set: filaments on the infinite no-slip wall z = 0
 * (INFINITE_PLANE_WALL, swimmer.cpp:68-110): nswim = 1, nblob = 0,
 * blob_refs and body_x0 may be NULL, fil_refs are the base points and every
 * filament stands along +z; no body unknowns, no linear solve. */
GMI_API gmi_status gmi_sim_create(const gmi_sim_config *cfg, const double *blob_refs, const double *fil_refs,
                                  const double *body_x0, const double *perturb1, const double *perturb2,
                                  gmi_sim **out);
GMI_API gmi_status gmi_sim_destroy(gmi_sim *sim);
GMI_API gmi_solver *gmi_sim_solver(gmi_sim *sim);
/* make_body_reference_matrices on the initial state (cilia_sim_main.cpp:159-165);
 * body_mobility_out (36, column-major) may be NULL. */
GMI_API gmi_status gmi_sim_prepare(gmi_sim *sim, double *body_mobility_out);
/* Time step nt (0-based): Broyden until the residual meets tol.  Returns
 * GMI_ERR_NOT_CONVERGED / GMI_ERR_NONFINITE where the reference stops. */
GMI_API gmi_status gmi_sim_step(gmi_sim *sim, int nt, int *broyden_iters, int *gmres_iters_total);
/* Drive the filaments by a prescribed preferred-curvature beat through the
 * reference's strain_twist hook (filament::body_frame_moment,
 * filament.cpp:1104-1106, which the reference leaves at zero,
 * swimmer.cpp:92, 210): time step nt solves with
 *     strain_twist_f = (0, amplitude sin(2 pi (nt + 1) dt / period + phase_f), 0)
 * (phases_h: one per filament).  end_force_scale multiplies the end force
 * (0: the beat alone drives the filaments); the barrier keeps its scale
 * (repulsive_force_factor * end_force_magnitude).  An extension: the
 * reference has no time-dependent preferred curvature. */
GMI_API gmi_status gmi_sim_set_beat(gmi_sim *sim, double amplitude, double period, const double *phases_h,
                                    double end_force_scale);
GMI_API gmi_status gmi_sim_get_state(gmi_sim *sim, int field, double *out_h);

/* Checkpoints in the reference's .backup layout (replaces the state part of
 * cilia_sim_main.cpp:370-381 and :29-77; filament.cpp:1595-1650;
 * rigid_body.cpp:408-432): per swimmer, NFIL filaments of 9 + 28*NSEG values
 * (per segment q, x, xm1, xm2, u, um1; tether and clamp multipliers and their
 * two previous values; the inextensibility multipliers and theirs), then the
 * body (q, x, xm1, xm2, u, um1: 19 values).  The step number that the file
 * starts with is the caller's.  Import sets q^{n-1} = q, zeroes the linear
 * solver's warm start, and requires gmi_sim_prepare again, as the reference's
 * restart does. */
GMI_API gmi_status gmi_sim_backup_count(const gmi_sim *sim, long long *count);
GMI_API gmi_status gmi_sim_export_backup(gmi_sim *sim, double *out_h);
GMI_API gmi_status gmi_sim_import_backup(gmi_sim *sim, const double *in_h);

/* ------------------------------------------------------------------------
 * Learned initial inverse Jacobian (no counterpart in the reference, which
 * starts every time step's Broyden solve from JACOBIAN_CONFIDENCE_FACTOR
 * times the approximate inverse of swimmer::jacobian_inv_mult,
 * broyden_solver.cpp:26-68, swimmer.cpp:690-845).
 *
 * A 3-layer MLP (n_in -> n_hidden -> n_hidden -> n_out, ReLU, bf16 weights
 * and activations, FP32 accumulation on the tensor cores) maps a filament's
 * shape in its local frame (phi: per segment, the position relative to the
 * base over the filament length and the tangent, 6 nseg values) to a
 * per-filament initial inverse Jacobian
 *     H0 d = sigma (.) (conf Jinv d) + U (V^T d)
 * (sigma: one scale per 3-vector, U, V: 6 nseg x rank), fitted to the secant
 * pairs (change of the Broyden error, update) of plain Broyden runs.
 * ---------------------------------------------------------------------- */
typedef struct gmi_mlp gmi_mlp;

/* Widths are positive multiples of 8; weights Kaiming-uniform from seed, the
 * last layer scaled down so that the untrained network is close to the plain
 * method (sigma = 1, U V^T = 0). */
GMI_API gmi_status gmi_mlp_create(int device, int n_in, int n_hidden, int n_out, unsigned long long seed,
                                  gmi_mlp **out);
GMI_API gmi_status gmi_mlp_destroy(gmi_mlp *m);
/* FP32 master parameters, flat: W1 [n_hidden x n_in] b1 W2 b2 W3 [n_out x
 * n_hidden] b3, each segment starting at offsets6[l] (row-major W). */
GMI_API gmi_status gmi_mlp_param_count(const gmi_mlp *m, long long *count);
GMI_API gmi_status gmi_mlp_param_offsets(const gmi_mlp *m, long long *offsets6);
GMI_API gmi_status gmi_mlp_get_params(gmi_mlp *m, float *params_h, long long count);
GMI_API gmi_status gmi_mlp_set_params(gmi_mlp *m, const float *params_h, long long count);
/* O [batch x n_out] (FP32, device) of X [batch x n_in] (FP32, device;
 * rounded to bf16 on input).  Synchronous. */
GMI_API gmi_status gmi_mlp_forward(gmi_mlp *m, const float *X_d, int batch, float *O_d);
/* Gradients of the last gmi_mlp_forward's batch for upstream dO [batch x
 * n_out] (FP32, device), in the flat parameter layout (grad_h may be NULL).
 * Synchronous. */
GMI_API gmi_status gmi_mlp_backward(gmi_mlp *m, const float *dO_d, int batch, float *grad_h);
/* Mean secant-pair loss of records [nrec x (n_in + 18 nseg)] (FP32, device;
 * layout phi | d | b | t, see gmi_sim_set_secant_buffer) for a head of the
 * given rank (2, 4 or 8; n_in = 6 nseg, n_out >= 2 nseg + 12 nseg rank).
 * O_scratch_d holds min(nrec, 4096) x n_out floats; dO_d (nrec x n_out, or
 * NULL) receives the gradient of the mean over each chunk of 4096. */
GMI_API gmi_status gmi_mlp_secant_loss(gmi_mlp *m, const float *records_d, long long nrec, int nseg, int rank,
                                       float *O_scratch_d, double *mean_loss, float *dO_d);
/* Adam on the secant-pair loss: steps minibatches of batch records drawn
 * with replacement (a counter-based hash of seed and the step).  loss_h
 * (steps floats, or NULL) receives each step's minibatch loss. */
GMI_API gmi_status gmi_mlp_train_secant(gmi_mlp *m, const float *records_d, long long nrec, int nseg, int rank,
                                        int steps, int batch, float lr, unsigned long long seed, float *loss_h);
GMI_API long long gmi_mlp_launch_count(const gmi_mlp *m);

/* When a time step uses the learned H0 and when it falls back to the plain
 * one.  Plain host logic (no GPU), the same the time step runs.
 * Modes: 0 calibrating (the first calibration_steps steps are plain, their
 * mean Broyden count is the yardstick), 1 learned, 2 fell back (plain from
 * then on).  A learned step gets at most
 *     cap = ceil(cap_factor * plain mean) + 2
 * Broyden iterations; one that does not converge within it (or diverges) is
 * a regression: the step is restarted from its initial guess with the plain
 * H0.  max_regressions regressions, or a mean learned count above
 * (1 + margin) * plain mean over the last window learned steps, end the
 * learned mode. */
typedef struct gmi_learned_policy {
    int calibration_steps;  /* default 3 */
    int window;             /* default 8 */
    int max_regressions;    /* default 2 */
    double margin;          /* default 0.05 */
    double cap_factor;      /* default 2 */
    /* state, written by gmi_learned_policy_record */
    int mode;
    int steps_plain, steps_learned, regressions;
    double plain_iters_sum;
    int recent[64];         /* Broyden counts of the last learned steps (ring) */
    int recent_count;
} gmi_learned_policy;

GMI_API void gmi_learned_policy_init(gmi_learned_policy *p);
GMI_API int gmi_learned_policy_use_learned(const gmi_learned_policy *p);
GMI_API int gmi_learned_policy_iteration_cap(const gmi_learned_policy *p, int max_broyden_iter);
GMI_API void gmi_learned_policy_record(gmi_learned_policy *p, int used_learned, int converged, int broyden_iters);

/* Collect secant pairs: every Broyden iteration of a plain step appends one
 * record per filament, [phi (6 nseg) | d | b | t (6 nseg each)] in FP32, to
 * records_d (device, capacity records; NULL stops collecting), while room
 * is left.  d: the change of the filament's Broyden error over the
 * iteration; b: conf Jinv d (the plain initial inverse Jacobian applied to
 * it); t: the filament's update of that iteration; all in the filament's
 * local frame (e3 along the filament's base direction). */
GMI_API gmi_status gmi_sim_set_secant_buffer(gmi_sim *sim, float *records_d, long long capacity);
GMI_API gmi_status gmi_sim_secant_count(const gmi_sim *sim, long long *count);
/* Jacobian probes for the records of gmi_sim_set_secant_buffer: every step
 * whose Broyden solve iterates first applies probes_per_step (0..64) random
 * updates v = -conf Jinv r from its initial guess (r: normal samples scaled
 * per row by the size of the step's error), evaluates the error there and
 * appends one record per filament, [phi | d = e(x + v) - e(x) | conf Jinv d
 * | v], restoring the state after each probe.  secant_pairs = 0 leaves the
 * Broyden iterations' own records out.  No counterpart in the reference. */
GMI_API gmi_status gmi_sim_set_jacobian_probes(gmi_sim *sim, int probes_per_step, unsigned long long seed,
                                               int secant_pairs);
/* Use the network's H0 (mlp NULL: the plain method) under policy (NULL:
 * defaults).  The network is read, not modified; several simulations may
 * share one.  rank is the head's rank (2, 4 or 8); n_in must be 6 nseg. */
GMI_API gmi_status gmi_sim_set_learned_jacobian(gmi_sim *sim, const gmi_mlp *mlp, int rank,
                                                const gmi_learned_policy *policy);
/* The policy's state after the steps so far. */
GMI_API gmi_status gmi_sim_learned_policy(const gmi_sim *sim, gmi_learned_policy *out);

/* Repulsive seeding of n points on the unit sphere, the reference's blob
 * seeding and uniform filament seeding (repulsive_blob_seeding,
 * seeding.cu:13-160, and seeding.cu:233-389 with UNIFORM_SEEDING; force
 * kernel seeding_repulsion_step, cuda_functions.cu:1159-1250): a spiral
 * start, then steps that move every point by the sum of 5 (2 - d) times
 * the unit separation from every other point and put it back on the
 * sphere, until no coordinate moves by more than 1e-4.  refs_out_h
 * receives 3 n coordinates (the reference writes them to sphere<n>.seed);
 * steps_out (may be NULL) the steps taken.  GMI_ERR_NOT_CONVERGED after
 * max_steps steps, GMI_ERR_NONFINITE for coincident points. */
GMI_API gmi_status gmi_seed_sphere_repulsive(int device, int n, int max_steps, double *refs_out_h, int *steps_out);

/* Measured FMA-pipe throughput (FLOP/s, FMA = 2) of this GPU for
 * precision GMI_FP32C (FP32 pipe) or GMI_FP64 (FP64 pipe): the roofline
 * denominator of the pair kernels, which are bound by that pipe.  No
 * counterpart in the reference. */
GMI_API gmi_status gmi_measure_fma_peak(gmi_context *ctx, int precision, double *flops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* GMI_H */
