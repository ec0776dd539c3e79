"""Golden trajectories from the reference's own simulator run on the CPU.

Builds cilia_sim_main.cpp and the rest of the reference (unmodified, from
the reference tree) with oracle/ref_solver/build_ref_solver.py, runs a case,
and stores its inputs (blob and filament references, the initial force
perturbations) and its per-step output (segment quaternions, body state,
segment and body velocities, Broyden iteration counts, final backup) in
sim_<case>.npz.  The fixtures are committed; the tests never need the tree.

    python tests/golden/make_golden_sim.py small_swimmer
    python tests/golden/make_golden_sim.py small_swimmer --restart 4

With --restart N the reference is run again from the first run's final
.backup for N more steps (its INITIAL_CONDITIONS_TYPE 1 path), and the
restart's inputs and steps go to sim_<case>_restart.npz.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_solver import build_ref_solver as brs  # noqa: E402


def parse_dat(path, skip_cols=1):
    rows = [np.array(ln.split()[skip_cols:], dtype=np.float64) for ln in open(path) if ln.strip()]
    return np.stack(rows)


def collect(case, restart_steps=0):
    """Run the case (and the restart) and return (fixture name, arrays); main
    saves them."""
    if restart_steps:
        first, rundir = brs.run_restart(case, restart_steps)
    else:
        rundir = brs.run_case(case)
    spec = dict(brs.COMMON)
    spec.update({k: v for k, v in brs.CASES[case].items() if k.isupper()})
    cfg = open(os.path.join(os.path.dirname(rundir), "config.hpp")).read()

    def macro(name):
        m = re.search(r"#define[ \t]+" + name + r"[ \t]+([^\n/]*)", cfg)
        return m.group(1).strip()

    nseg, nfil, nblob = int(spec["NSEG"]), int(spec["NFIL"]), int(spec["NBLOB"])
    nswim = int(spec["NSWIM"])
    DL = 2.2 * float(spec["RSEG"])
    kb = float(macro("KB"))
    dimless = float(macro("DIMENSIONLESS_FORCE"))
    efm = dimless * kb / (DL * DL * nseg * nseg)
    steps_per_period = float(macro("STEPS_PER_PERIOD"))
    dt = eval(spec.get("DT", f"(36.3833/{steps_per_period})"))
    r_over_l = eval(spec["R_OVER_L"])
    # perturbations: the reference's generator, compiled here
    exe = os.path.join(os.path.dirname(rundir), "perturbation")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", os.path.join(ROOT, "oracle", "ref_solver", "perturbation.cpp"),
                    "-o", exe], check=True)
    p = np.array([ln.split() for ln in subprocess.run([exe, repr(efm)], capture_output=True, text=True,
                                                       check=True).stdout.split("\n") if ln.strip()], dtype=float)
    # The reference writes its reference-position files at the default stream
    # precision (6 digits); rebuild the exact values the way it does: unit
    # seeds times Rsphere (rigid_body.cpp:200, 231) and times
    # R_OVER_L*L + 1.05*(0.5*DL + RBLOB) for the filament bases (swimmer.cpp:172, 199).
    out = subprocess.run(["cat", os.path.join(rundir, "stdout.txt")], capture_output=True, text=True).stdout
    broyden = [int(m) for m in re.findall(r"Completed step \d+/\d+ in (\d+) Broyden iterations", out)]
    L = DL * nseg
    wall = brs.is_wall(case)
    if wall:
        # filaments on the wall: the reference's rectangular grid, no body
        nswim, nblob = 1, 0
        blob_refs = np.zeros((0, 3))
        fil_refs = brs.wall_filament_bases(nfil, nseg, DL)
    else:
        blobs, fils = brs.seeds(case)
        blob_refs = blobs * (r_over_l * DL * nseg)
        fil_refs = fils * (r_over_l * L + 1.05 * (0.5 * DL + float(spec["RBLOB"])))
        chk_b = parse_dat(os.path.join(rundir, "test_blob_references.dat"), 0).reshape(-1, 3)
        assert np.allclose(chk_b, blob_refs, rtol=1e-5, atol=1e-5)
    chk_f = parse_dat(os.path.join(rundir, "test_fil_references.dat"), 0).reshape(-1, 3)
    assert np.allclose(chk_f, fil_refs, rtol=1e-5, atol=1e-5)

    # swimmer n starts at x = n * 3 (R + L) (rigid_body.cpp, SPHEROID_BODIES)
    body_x0 = np.zeros((nswim, 3))
    body_x0[:, 0] = np.arange(nswim) * 3.0 * (r_over_l * DL * nseg + L)
    def dat(name, ncols):
        path = os.path.join(rundir, name)
        if os.path.exists(path):
            return parse_dat(path)
        return np.zeros((len(broyden), ncols))  # not written for the wall (mobility_solver.cpp:1786-1879)

    data = dict(
        wall=int(wall), nswim=nswim, body_x0=body_x0, nfil=nfil, nseg=nseg, nblob=nblob, kb=kb, kt=float(macro("KT")), dt=dt, end_force_magnitude=efm,
        repulsive_force_factor=float(macro("REPULSIVE_FORCE_FACTOR")), rseg=float(spec["RSEG"]),
        rblob=float(spec["RBLOB"]), mu=float(spec["MU"]), body_radius=r_over_l * DL * nseg,
        tol=float(macro("TOL")), linear_tol=float(macro("LINEAR_SYSTEM_TOL")),
        max_linear_iter=int(macro("MAX_LINEAR_SYSTEM_ITER")),
        blob_refs=blob_refs, fil_refs=fil_refs,
        perturbation1=p[0], perturbation2=p[1],
        seg_q=parse_dat(os.path.join(rundir, "test_seg_states.dat")),
        body_state=dat("test_body_states.dat", 7 * nswim),
        seg_v=parse_dat(os.path.join(rundir, "test_seg_vels.dat")),
        body_v=dat("test_body_vels.dat", 6 * nswim),
        blob_f=dat("test_blob_forces.dat", 3 * nblob * nswim),
        broyden_iters=np.array(broyden),
        backup=parse_dat(os.path.join(rundir, "test.backup")),
    )
    nsteps = data["seg_q"].shape[0]
    keep = np.arange(nsteps) if nsteps <= 20 else np.unique(np.r_[np.arange(0, nsteps, 10), nsteps - 1])
    for key in ("seg_q", "body_state", "seg_v", "body_v", "blob_f"):
        data[key] = data[key][keep]
    data["steps"] = keep
    name = f"sim_{case}"
    if restart_steps:
        # the restart began from the first run's final backup: the steps here
        # are nt_start .. nt_start + restart_steps - 1
        with open(os.path.join(first, "test.backup")) as fh:
            tok = fh.read().split()
        data["nt_start"] = int(tok[0])
        data["backup_in"] = np.array(tok[1:], dtype=np.float64)
        data["steps"] = keep + int(tok[0])
        name += "_restart"
    return name, data


def main(case, restart_steps=0):
    name, data = collect(case, restart_steps)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **data)
    print(case, {k: np.shape(v) for k, v in data.items() if np.ndim(v)})


if __name__ == "__main__":
    # python tests/golden/make_golden_sim.py <case> [--restart N]
    args = sys.argv[1:]
    n_restart = int(args[args.index("--restart") + 1]) if "--restart" in args else 0
    main(args[0] if args and not args[0].startswith("--") else "small_swimmer", n_restart)
