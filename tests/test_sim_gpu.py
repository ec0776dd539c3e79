"""The device time step against the reference's own simulator.

tests/golden/sim_small_swimmer.npz was produced by the reference's unmodified
cilia_sim_main.cpp and solver classes compiled for the CPU
(tests/golden/make_golden_sim.py): one free-swimming sphere of 162 blobs with
4 end-force-driven filaments of 20 segments, 12 steps (Euler, then BDF2 with
both multiplier-extrapolation stages).  Every step is compared: Broyden
iteration count, segment quaternions, body position and orientation, segment
and body velocities.  Differences come from GMRES (CGS2 vs MGS Arnoldi,
tolerance 1e-10), the approximate-Jacobian inverse (Gauss-Jordan vs LAPACK)
and summation order, so state agrees to ~1e-12 and velocities to the GMRES tolerance (~1e-9)
when the Broyden iteration counts agree, which they must, step by step.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu

TRAJ_TOL = 1e-10
VEL_TOL = 1e-7


def test_trajectory_matches_reference(gmi_lib):
    from generic_mobility_interface_class_gb300.sim import Simulation
    g = load_golden("small_swimmer", prefix="sim_")
    sim = Simulation.from_golden(g)
    sim.prepare()
    nsteps = g["seg_q"].shape[0]
    for nt in range(nsteps):
        biters, giters = sim.step(nt)
        assert biters == int(g["broyden_iters"][nt]), (nt, biters, int(g["broyden_iters"][nt]))
        q = sim.state("seg_q").ravel()
        assert rel_err(q, g["seg_q"][nt]) < TRAJ_TOL, nt
        bx, bq = sim.state("body_x").ravel(), sim.state("body_q").ravel()
        assert np.max(np.abs(bx - g["body_state"][nt][:3])) < TRAJ_TOL * 10, nt
        assert np.max(np.abs(bq - g["body_state"][nt][3:])) < TRAJ_TOL, nt
        assert rel_err(sim.state("seg_v").ravel(), g["seg_v"][nt]) < VEL_TOL, nt
        assert rel_err(sim.state("body_v").ravel(), g["body_v"][nt]) < VEL_TOL, nt
    sim.close()
