/*
 * ref_kernels_config.h -- configuration used to compile the reference's
 * cuda_functions.cu for the CPU checker.  TEST INFRASTRUCTURE ONLY.
 *
 * It defines the reference config's include guard (config.hpp:5-6), so the
 * reference's own config.hpp is skipped, and supplies the macros that
 * cuda_functions.cu reads.  The problem sizes and radii, compile-time
 * constants in the reference (config.hpp:95-103), become run-time variables
 * here so one build serves every test size; the derived macros keep the
 * reference's definitions (config.hpp:183-200, 222-226).  Flags that select
 * code by preprocessor (#if) stay compile-time: REF_WALL=1 builds the
 * Swan-Brady wall variant, REF_WALL=0 the free-space solver with a free
 * rigid body.
 */
#ifndef MY_CONFIG_HEADER_INCLUDED
#define MY_CONFIG_HEADER_INCLUDED

extern int ref_nswim, ref_nfil, ref_nseg, ref_nblob;
extern double ref_rseg, ref_rblob, ref_mu;
extern double ref_repulsive_force_factor, ref_end_force_magnitude;

#ifndef REF_WALL
#define REF_WALL 0
#endif

#define THREADS_PER_BLOCK 1

#define NSWIM ref_nswim
#define NFIL ref_nfil
#define NSEG ref_nseg
#define NBLOB ref_nblob
#define MU ref_mu
#define RSEG ref_rseg
#define RBLOB ref_rblob
#define REPULSIVE_FORCE_FACTOR ref_repulsive_force_factor
#define END_FORCE_MAGNITUDE ref_end_force_magnitude

#define PI 3.14159265358979323846264338327950288
#define DL (2.2 * RSEG)
#define NTOTAL (NSWIM * (NFIL * NSEG + NBLOB))

#define INFINITE_PLANE_WALL REF_WALL
#define PRESCRIBED_BODY_VELOCITIES REF_WALL
#define PRESCRIBED_CILIA 0
#define NO_CILIA_SQUIRMER 0
#define USE_BROYDEN_FOR_EVERYTHING 0

#endif
