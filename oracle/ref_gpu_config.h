/*
 * ref_gpu_config.h -- configuration used to compile the reference's
 * cuda_functions.cu for the GPU (sm_103a), as its own build does: every size
 * is a compile-time macro (config.hpp:95-103), so each problem size is its
 * own build (REF_N sources, one swimmer of one "filament" of REF_N segments
 * and REF_N blobs), and the launch shape is the reference's default
 * THREADS_PER_BLOCK 64 (config.hpp:135).  TEST INFRASTRUCTURE ONLY: the
 * product never includes this header.
 *
 * It defines the reference config's include guard (config.hpp:5-6), so the
 * reference's own config.hpp is skipped, and supplies the macros that
 * cuda_functions.cu reads, with the reference's definitions of the derived
 * ones (config.hpp:183-200, 222-226).
 */
#ifndef MY_CONFIG_HEADER_INCLUDED
#define MY_CONFIG_HEADER_INCLUDED

#ifndef REF_N
#error "REF_N (the number of particles of this build) is required"
#endif

#define THREADS_PER_BLOCK 64

#define NSWIM 1
#define NFIL 1
#define NSEG REF_N
#define NBLOB REF_N
#define MU 1.0
#define RSEG 1.0
#define RBLOB 1.0
#define REPULSIVE_FORCE_FACTOR 2.0
#define END_FORCE_MAGNITUDE 1.0

#define PI 3.14159265358979323846264338327950288
#define DL (2.2 * RSEG)
#define NTOTAL (NSWIM * (NFIL * NSEG + NBLOB))

#define INFINITE_PLANE_WALL 0
#define PRESCRIBED_BODY_VELOCITIES 0
#define PRESCRIBED_CILIA 0
#define NO_CILIA_SQUIRMER 0
#define USE_BROYDEN_FOR_EVERYTHING 0

#endif
