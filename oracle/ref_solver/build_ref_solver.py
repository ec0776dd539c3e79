"""Build and run the reference's own simulator on the CPU.  TEST INFRASTRUCTURE ONLY.

The reference's unmodified host sources (cilia_sim_main.cpp, mobility_solver.cpp,
broyden_solver.cpp, swimmer.cpp, filament.cpp, rigid_body.cpp, segment.cpp,
quaternion.cpp, matrix.cpp) and its kernels (cuda_functions.cu, compiled as C++
through ../ref_cpu_shim.h) are compiled from where they lie in the reference
tree.  Each case gets a config.hpp derived from the reference's own config.hpp
by replacing the values of named #define lines; it is written to the build
directory under oracle/_ref and force-included, so its include guard keeps the
reference's copy out.  ref_solver_shim.h makes the run reproducible and
full-precision and swaps the CUDA rpy_mobility_solver for a CPU one.

    python oracle/ref_solver/build_ref_solver.py <case> [--run]

Outputs (oracle/_ref/solver_<case>/run): the reference's .dat and .backup files,
written every step with 17 significant digits, and stdout with the Broyden
iteration counts.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
sys.path.insert(0, ROOT)
from oracle import reference_dir  # noqa: E402

REF = reference_dir()


def _scipy_libs() -> str:
    """The directory of the OpenBLAS that scipy's wheel bundles (the LAPACK
    behind lapack_shim.c): ``scipy.libs`` beside the installed package."""
    import scipy
    return os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(scipy.__file__))), "scipy.libs")


SCIPY_LIBS = _scipy_libs()

REF_CPP = ["cilia_sim_main.cpp", "matrix.cpp", "quaternion.cpp", "segment.cpp", "filament.cpp", "broyden_solver.cpp",
           "rigid_body.cpp", "swimmer.cpp", "mobility_solver.cpp"]

# Values common to every case: free-swimming instability-driven cilia on a
# spherical body with the RPY mobility and GMRES, written every step.
COMMON = dict(CILIA_TYPE="0", BODY_OR_SURFACE_TYPE="2", MOBILITY_TYPE="1", SOLVER_TYPE="1",
              INITIAL_CONDITIONS_TYPE="0", THREADS_PER_BLOCK="1", SAVES_PER_PERIOD="STEPS_PER_PERIOD",
              NSWIM="1", MU="1.0", RSEG="1.0")

CASES = {
    # small swimmer: 4 filaments x 20 segments on 162 blobs
    "small_swimmer": dict(NFIL="4", NSEG="20", NBLOB="162", R_OVER_L="0.25", RBLOB="1.0", KB="1800.0",
                          KT="1800.0", TOTAL_TIME_STEPS="12", nblob_subdiv=2, fil_subdiv=1, seed=5),
    # two identical swimmers (the reference places swimmer n at x = 3 n (R + L),
    # rigid_body.cpp SPHEROID_BODIES branch): the multi-swimmer paths
    "two_swimmers": dict(NSWIM="2", NFIL="4", NSEG="20", NBLOB="162", R_OVER_L="0.25", RBLOB="1.0", KB="1800.0",
                         KT="1800.0", TOTAL_TIME_STEPS="8", nblob_subdiv=2, fil_subdiv=1, seed=7),
    # filaments on an infinite no-slip wall (INFINITE_PLANE_WALL): a 3 x 3
    # rectangular grid of 20-segment filaments, Swan-Brady wall mobility, no
    # rigid body and no linear solve
    # prescribed-shape cilia (CILIA_TYPE 3, the coral-larvae beat fit, phases
    # advancing at constant speed): the solver's prescribed-motion system
    "prescribed": dict(CILIA_TYPE="3", NFIL="4", NSEG="20", NBLOB="162", R_OVER_L="0.25", RBLOB="1.0",
                       TOTAL_TIME_STEPS="3", DYNAMIC_PHASE_EVOLUTION="false", nblob_subdiv=2, fil_subdiv=1, seed=5),
    # the reference's generalised-force table for that beat: its own main
    # built with WRITE_GENERALISED_FORCES (config.hpp:259-266 makes that one
    # swimmer with one cilium over one period, phase 0, omega0 = 2 pi), which
    # writes sum_k vel_dir_k . f_k of the cilium after every step
    # (cilia_sim_main.cpp:184-246)
    "prescribed_table": dict(CILIA_TYPE="3", NFIL="1", NSEG="20", NBLOB="162", R_OVER_L="0.25", RBLOB="1.0",
                             TOTAL_TIME_STEPS="STEPS_PER_PERIOD", DYNAMIC_PHASE_EVOLUTION="false",
                             WRITE_GENERALISED_FORCES="true", nblob_subdiv=2, fil_subdiv=1, seed=5),
    # phase speeds solved with the forces (DYNAMIC_PHASE_EVOLUTION): the
    # "prescribed" swimmer driven by that table
    "prescribed_dynamic": dict(CILIA_TYPE="3", NFIL="4", NSEG="20", NBLOB="162", R_OVER_L="0.25", RBLOB="1.0",
                               TOTAL_TIME_STEPS="4", DYNAMIC_PHASE_EVOLUTION="true", nblob_subdiv=2, fil_subdiv=1,
                               seed=5),
    "wall_filaments": dict(BODY_OR_SURFACE_TYPE="0", NFIL="9", NSEG="20", NBLOB="0", R_OVER_L="0.25",
                           RBLOB="1.0", TOTAL_TIME_STEPS="10", seed=3),
    # BASELINE config 1 geometry: sphere of radius 10a, 642 blobs (icosphere 3),
    # 16 filaments x 20 segments at random icosphere vertices, GMRES tol 1e-8,
    # Broyden tol 1e-4, 100 steps.  The prescribed preferred-curvature beat of
    # that config is not a reference feature; the filaments are driven by the
    # reference's end force at its default stiffness and time step (with
    # KB = KT = 1 and dt = 1/300 the extrapolated guess already meets the
    # tolerance and Broyden never iterates).
    "config1": dict(NFIL="16", NSEG="20", NBLOB="642", R_OVER_L="(10.0/44.0)", RBLOB="1.0",
                    LINEAR_SYSTEM_TOL="1e-8", TOTAL_TIME_STEPS="100", nblob_subdiv=3, fil_subdiv=3, seed=2026),
}


def config_text(overrides: dict) -> str:
    text = open(os.path.join(REF, "config.hpp")).read()
    for key, val in overrides.items():
        pat = re.compile(r"(#define[ \t]+" + re.escape(key) + r"[ \t]+)([^\n]*)")
        text, n = pat.subn(lambda m: m.group(1) + val, text)
        if n == 0:
            raise KeyError(f"config.hpp has no #define {key}")
    return text


def build(case: str, overrides: dict | None = None, tag: str = "", driver: str | None = None) -> str:
    spec = dict(COMMON)
    spec.update({k: v for k, v in CASES[case].items() if k.isupper()})
    spec.update(overrides or {})
    out = os.path.join(ORACLE, "_ref", f"solver_{case}{tag}")
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(out, "config.hpp"), "w") as fh:
        fh.write(config_text(spec))
    exe = os.path.join(out, "cilia_cpu")
    inc = ["-I" + out, "-I" + HERE, "-I" + ORACLE, "-I" + REF]
    base = ["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-std=c++17", "-w", *inc,
            "-include", os.path.join(out, "config.hpp")]
    jobs = []
    for f in REF_CPP:
        if driver and f == "cilia_sim_main.cpp":
            # a test driver takes the place of the reference's main
            f_src = os.path.join(HERE, driver)
            jobs.append(base + ["-include", os.path.join(HERE, "ref_solver_shim.h"), "-I" + REF, "-c", f_src,
                                "-o", os.path.join(out, driver + ".o")])
            continue
        jobs.append(base + ["-include", os.path.join(HERE, "ref_solver_shim.h"), "-c", os.path.join(REF, f),
                            "-o", os.path.join(out, f + ".o")])
    jobs.append(base + ["-c", os.path.join(HERE, "cpu_rpy_mobility_solver.cpp"),
                        "-o", os.path.join(out, "cpu_rpy_mobility_solver.o")])
    jobs.append(base + ["-c", os.path.join(HERE, "seeding_stub.cpp"), "-o", os.path.join(out, "seeding_stub.o")])
    jobs.append(base + ["-include", os.path.join(ORACLE, "ref_cpu_shim.h"), "-x", "c++", "-c",
                        os.path.join(REF, "cuda_functions.cu"), "-o", os.path.join(out, "cuda_functions.o")])
    jobs.append(["gcc", "-O2", "-c", os.path.join(HERE, "lapack_shim.c"), "-o", os.path.join(out, "lapack_shim.o")])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(" ".join(cmd) + "\n" + r.stderr)

    with ThreadPoolExecutor(8) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(out, f) for f in os.listdir(out) if f.endswith(".o")]
    blas = [f for f in os.listdir(SCIPY_LIBS) if f.startswith("libscipy_openblas")][0]
    run(["g++", "-fopenmp", *objs, "-o", exe, os.path.join(SCIPY_LIBS, blas), "-Wl,-rpath," + SCIPY_LIBS])
    return exe


def is_wall(case: str) -> bool:
    return CASES[case].get("BODY_OR_SURFACE_TYPE", COMMON["BODY_OR_SURFACE_TYPE"]) == "0"


def wall_filament_bases(nfil: int, nseg: int, dl: float = 2.2):
    """The reference's rectangular grid of filament bases on the wall
    (swimmer.cpp:68-110, RECTANGULAR_SEEDING): step 1.4 L, height DL / 2."""
    import math
    import numpy as np
    L = dl * nseg
    gx = int(math.sqrt(float(nfil)))
    gy = max(1, int(math.ceil(nfil / float(gx))))
    step = 1.4 * L
    im, jm = 0.5 * (gx - 1.0), 0.5 * (gy - 1.0)
    out = np.zeros((nfil, 3))
    for i in range(gx):
        for j in range(gy):
            f = j + i * gy
            if f < nfil:
                out[f] = [(i - im) * step, (j - jm) * step, 0.5 * dl]
    return out


def seeds(case: str):
    """Unit-sphere seeds: blobs on an icosphere, filaments at random icosphere vertices."""
    import numpy as np
    sys.path.insert(0, ROOT)
    from generic_mobility_interface_class_gb300 import seeding
    spec = CASES[case]
    nblob, nfil = int(spec["NBLOB"]), int(spec["NFIL"])
    blobs = seeding.icosphere(spec["nblob_subdiv"])[:nblob]
    verts = seeding.icosphere(spec["fil_subdiv"])
    rng = np.random.default_rng(spec["seed"])
    fils = verts[rng.choice(len(verts), nfil, replace=False)]
    return blobs, fils


def run_case(case: str, exe: str | None = None) -> str:
    import numpy as np
    exe = exe or build(case)
    rundir = os.path.join(os.path.dirname(exe), "run")
    os.makedirs(rundir, exist_ok=True)
    for f in os.listdir(rundir):
        os.remove(os.path.join(rundir, f))
    spec = CASES[case]
    if not is_wall(case):  # spheres read their seeds; the wall seeds a grid itself
        blobs, fils = seeds(case)
        assert spec["NBLOB"] != spec["NFIL"]
        np.savetxt(os.path.join(rundir, f"sphere{spec['NBLOB']}.seed"), blobs.ravel()[None, :], fmt="%.17g")
        np.savetxt(os.path.join(rundir, f"sphere{spec['NFIL']}.seed"), fils.ravel()[None, :], fmt="%.17g")
    r = subprocess.run([exe], cwd=rundir, capture_output=True, text=True)
    with open(os.path.join(rundir, "stdout.txt"), "w") as fh:
        fh.write(r.stdout)
    if r.returncode != 0:
        raise RuntimeError(r.stderr + r.stdout[-2000:])
    return rundir


GEN_FORCE_FILE = "coral_larvae_reference_generalised_forces.dat"  # filament.cpp:1666-1674, SHAPE_SEQUENCE 2


def generalised_force_table() -> str:
    """Run the "prescribed_table" case (the reference's own main) and return
    the path of the generalised-force file it wrote."""
    rundir = run_case("prescribed_table")
    return os.path.join(rundir, GEN_FORCE_FILE)


def run_prescribed_dump(case: str) -> str:
    """Build the case with prescribed_dump.cpp as its driver, run it, and
    return the path of its dump (see prescribed_dump.cpp).  A case with
    DYNAMIC_PHASE_EVOLUTION reads the generalised-force table, which the
    "prescribed_table" case writes first."""
    import shutil
    table = generalised_force_table() if CASES[case].get("DYNAMIC_PHASE_EVOLUTION") == "true" else None
    exe = build(case, tag="_dump", driver="prescribed_dump.cpp")
    rundir = os.path.join(os.path.dirname(exe), "run")
    os.makedirs(rundir, exist_ok=True)
    for f in os.listdir(rundir):
        os.remove(os.path.join(rundir, f))
    if table:
        shutil.copy(table, rundir)
    blobs, fils = seeds(case)
    spec = CASES[case]
    import numpy as np
    np.savetxt(os.path.join(rundir, f"sphere{spec['NBLOB']}.seed"), blobs.ravel()[None, :], fmt="%.17g")
    np.savetxt(os.path.join(rundir, f"sphere{spec['NFIL']}.seed"), fils.ravel()[None, :], fmt="%.17g")
    r = subprocess.run([exe], cwd=rundir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr + r.stdout[-2000:])
    return os.path.join(rundir, "prescribed_dump.txt")


def run_restart(case: str, extra_steps: int) -> tuple[str, str]:
    """Run the case, then the reference restarting from its final backup
    (INITIAL_CONDITIONS_TYPE 1, cilia_sim_main.cpp:29-77) for extra_steps
    more steps.  Returns (first run dir, restart run dir)."""
    import shutil
    first = run_case(case)
    total = int(CASES[case]["TOTAL_TIME_STEPS"]) + extra_steps
    exe = build(case, {"INITIAL_CONDITIONS_TYPE": "1", "TOTAL_TIME_STEPS": str(total)}, tag="_restart")
    rundir = os.path.join(os.path.dirname(exe), "run")
    os.makedirs(rundir, exist_ok=True)
    for f in os.listdir(rundir):
        os.remove(os.path.join(rundir, f))
    for f in os.listdir(first):
        if f.endswith(".seed") or f.endswith(".backup"):
            shutil.copy(os.path.join(first, f), rundir)
    r = subprocess.run([exe], cwd=rundir, capture_output=True, text=True)
    with open(os.path.join(rundir, "stdout.txt"), "w") as fh:
        fh.write(r.stdout)
    if r.returncode != 0:
        raise RuntimeError(r.stderr + r.stdout[-2000:])
    return first, rundir


if __name__ == "__main__":
    case = sys.argv[1]
    exe = build(case)
    print(exe)
    if "--run" in sys.argv:
        print(run_case(case, exe))
