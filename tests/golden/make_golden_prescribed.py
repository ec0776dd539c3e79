"""Golden linear solves of prescribed-shape cilia from the reference's own code.

Builds the reference's unmodified sources for CILIA_TYPE 3 (its coral-larvae
beat fit, phases at constant speed) with oracle/ref_solver/prescribed_dump.cpp
as the driver (oracle/ref_solver/build_ref_solver.py run_prescribed_dump), and
stores, for every step, what mobility_solver::compute_velocities received
(segment positions, shape-velocity directions, phase speeds, body state) and
returned (segment forces, blob forces, body velocities, GMRES iterations) in
prescribed.npz.

With the case "prescribed_dynamic" the phase speeds are unknowns of the
solve (DYNAMIC_PHASE_EVOLUTION): the reference's own main first writes its
generalised-force table over one beat period (case "prescribed_table"), and
prescribed_dynamic.npz also holds that table, the phases and natural
frequencies each solve received and the phase speeds it returned.

    python tests/golden/make_golden_prescribed.py [prescribed|prescribed_dynamic]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_solver import build_ref_solver as brs  # noqa: E402

PER_FILAMENT = ("vel_dir", "phase_speed", "phase", "omega0", "phase_speed_out")


def collect(case: str = "prescribed") -> dict:
    """Run the case and return the fixture's arrays (main saves them)."""
    path = brs.run_prescribed_dump(case)
    spec = dict(brs.COMMON)
    spec.update({k: v for k, v in brs.CASES[case].items() if k.isupper()})
    nfil, nseg, nblob = int(spec["NFIL"]), int(spec["NSEG"]), int(spec["NBLOB"])
    steps = []
    cur = None
    for ln in open(path):
        tok = ln.split()
        if not tok:
            continue
        if tok[0] == "step":
            cur = {k: [] for k in PER_FILAMENT}
            steps.append(cur)
            continue
        vals = np.array(tok[1:], dtype=np.float64)
        if tok[0] in PER_FILAMENT:
            cur[tok[0]].append(vals)
        else:
            cur[tok[0]] = vals
    dl = 2.2 * float(spec["RSEG"])
    r_over_l = eval(spec["R_OVER_L"])
    blobs, _ = brs.seeds(case)
    data = dict(
        nfil=nfil, nseg=nseg, nblob=nblob, rseg=float(spec["RSEG"]), rblob=float(spec["RBLOB"]), mu=float(spec["MU"]),
        blob_refs=blobs * (r_over_l * dl * nseg), linear_tol=1e-10, max_linear_iter=150,
        body_x=np.stack([s["body_x"] for s in steps]), body_q=np.stack([s["body_q"] for s in steps]),
        x_segs=np.stack([s["x_segs"] for s in steps]),
        vel_dir=np.stack([np.concatenate(s["vel_dir"]) for s in steps]),
        phase_speed=np.stack([np.concatenate(s["phase_speed"]) for s in steps]),
        gmres_iters=np.array([int(s["gmres_iters"][0]) for s in steps]),
        f_segs=np.stack([s["f_segs"] for s in steps]), f_blobs=np.stack([s["f_blobs"] for s in steps]),
        v_bodies=np.stack([s["v_bodies"] for s in steps]))
    if spec.get("DYNAMIC_PHASE_EVOLUTION") == "true":
        table = np.array(open(os.path.join(os.path.dirname(path), brs.GEN_FORCE_FILE)).read().split(), np.float64)
        assert int(table[0]) == len(table) - 1
        data.update(gen_force_refs=table[1:],
                    phase=np.stack([np.concatenate(s["phase"]) for s in steps]),
                    omega0=np.stack([np.concatenate(s["omega0"]) for s in steps]),
                    phase_speed_out=np.stack([np.concatenate(s["phase_speed_out"]) for s in steps]))
    return data


def main(case: str = "prescribed"):
    data = collect(case)
    np.savez_compressed(os.path.join(HERE, f"{case}.npz"), **data)
    print({k: np.shape(v) for k, v in data.items() if np.ndim(v)})


if __name__ == "__main__":
    main(*sys.argv[1:2])
