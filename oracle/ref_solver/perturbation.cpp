/*
 * perturbation.cpp -- prints the two initial force perturbations the
 * reference gives every filament (filament.cpp:292-313) once its
 * std::random_device is the default-seeded std::minstd_rand of
 * ref_solver_shim.h.  Usage: perturbation <END_FORCE_MAGNITUDE>.
 * TEST INFRASTRUCTURE ONLY.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

int main(int argc, char **argv)
{
    const double efm = argc > 1 ? std::atof(argv[1]) : 1.0;
    const double pMag = 0.01 * efm;
    std::minstd_rand rd{};
    std::mt19937 gen{rd()};
    std::normal_distribution<double> d(0, 1);
    double dir1[3] = {d(gen), d(gen), d(gen)};
    const double n1 = std::sqrt(dir1[0] * dir1[0] + dir1[1] * dir1[1] + dir1[2] * dir1[2]);
    double dir2[3] = {d(gen), d(gen), d(gen)};
    const double n2 = std::sqrt(dir2[0] * dir2[0] + dir2[1] * dir2[1] + dir2[2] * dir2[2]);
    std::printf("%.17g %.17g %.17g\n", pMag * dir1[0] / n1, pMag * dir1[1] / n1, pMag * dir1[2] / n1);
    std::printf("%.17g %.17g %.17g\n", pMag * dir2[0] / n2, pMag * dir2[1] / n2, pMag * dir2[2] / n2);
    return 0;
}
