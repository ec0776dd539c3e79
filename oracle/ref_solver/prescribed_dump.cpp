// prescribed_dump.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A driver for the reference's own prescribed-shape cilia build (CILIA_TYPE
// 3), linked with its unmodified sources in place of cilia_sim_main.cpp.  It
// takes the steps cilia_sim_main.cpp:205-343 takes for this simulation type
// (swimmer initial guesses, forces_and_torques, compute_velocities, explicit
// body update, end_of_step) and, around every compute_velocities call, writes
// what the mobility solver receives and returns:
//   step, GMRES iterations, then per swimmer the body x and q; per segment
//   its position and shape-velocity direction (filament vel_dir); per
//   filament its phase, natural frequency omega0 and phase speed (with
//   DYNAMIC_PHASE_EVOLUTION the solver's initial guess); after the solve
//   the segment forces, blob forces, body velocities and, per filament, the
//   phase speed the solve left (phase_speed_out).
// One line per item, "<name> <values...>", in prescribed_dump.txt.
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <vector>

#include "swimmer.hpp"
#include "rpy_mobility_solver.hpp"
#include "config.hpp"

static void put(std::ofstream &f, const char *name, const double *v, int n)
{
    f << name;
    for (int i = 0; i < n; ++i) f << " " << v[i];
    f << "\n";
}

int main()
{
    std::ofstream out("prescribed_dump.txt");
    out << std::scientific << std::setprecision(17);
    rpy_mobility_solver mobility;
    mobility.initialise();
    std::vector<swimmer> swimmers(NSWIM);
    double *none = nullptr;
    for (int n = 0; n < NSWIM; n++)
        swimmers[n].initial_setup(n, none, &mobility.x_segs_host[3 * n * NFIL * NSEG],
                                  &mobility.f_segs_host[6 * n * NFIL * NSEG], &mobility.f_blobs_host[3 * n * NBLOB]);
    for (int nt = 0; nt < TOTAL_TIME_STEPS; nt++) {
        for (int i = 0; i < NSWIM; i++) {
            swimmers[i].initial_guess(nt);
            swimmers[i].forces_and_torques(nt);
        }
        out << "step " << nt << "\n";
        for (int n = 0; n < NSWIM; n++) {
            const swimmer &sw = swimmers[n];
            const double q[4] = {sw.body.q.scalar_part, sw.body.q.vector_part[0], sw.body.q.vector_part[1],
                                 sw.body.q.vector_part[2]};
            put(out, "body_x", sw.body.x, 3);
            put(out, "body_q", q, 4);
            for (int i = 0; i < NFIL; i++) {
                put(out, "vel_dir", sw.filaments[i].vel_dir.data(), 3 * NSEG);
                put(out, "phase_speed", &sw.filaments[i].phase_speed, 1);
                put(out, "phase", &sw.filaments[i].phase, 1);
                put(out, "omega0", &sw.filaments[i].omega0, 1);
            }
        }
        put(out, "x_segs", mobility.x_segs_host, 3 * NSWIM * NFIL * NSEG);
        int iters = 0;
        mobility.compute_velocities(swimmers, iters, nt);
        const double di = iters;
        put(out, "gmres_iters", &di, 1);
        put(out, "f_segs", mobility.f_segs_host, 6 * NSWIM * NFIL * NSEG);
        put(out, "f_blobs", mobility.f_blobs_host, 3 * NSWIM * NBLOB);
        put(out, "v_bodies", &mobility.v_bodies.data[0], 6 * NSWIM);
        for (int n = 0; n < NSWIM; n++)
            for (int i = 0; i < NFIL; i++) put(out, "phase_speed_out", &swimmers[n].filaments[i].phase_speed, 1);
        for (int n = 0; n < NSWIM; n++) {  // explicit body update, as cilia_sim_main.cpp:218-232
            swimmer &sw = swimmers[n];
            for (int c = 0; c < 3; c++) {
                sw.body.x[c] += DT * mobility.v_bodies(6 * n + c);
                sw.body.u[c] = DT * mobility.v_bodies(6 * n + 3 + c);
            }
            sw.body.q = lie_exp(sw.body.u) * sw.body.qm1;
        }
        for (int i = 0; i < NSWIM; i++) swimmers[i].end_of_step(nt);
    }
    return 0;
}
