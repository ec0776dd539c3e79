/*
 * seeding_stub.cpp -- the reference's seeding functions (seeding.cu:13-389)
 * are only reached when no sphereN.seed file is present; the CPU build
 * always supplies the files, so these stop loudly.  TEST INFRASTRUCTURE ONLY.
 */
#include <cstdio>
#include <cstdlib>

void repulsive_blob_seeding(double *const)
{
    std::fprintf(stderr, "ref solver: blob seed file missing\n");
    std::exit(2);
}

void repulsive_filament_seeding(double *const)
{
    std::fprintf(stderr, "ref solver: filament seed file missing\n");
    std::exit(2);
}
