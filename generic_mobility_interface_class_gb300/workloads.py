"""Seeded free-swimmer workloads for the device time step.

Each function returns the keyword arguments of ``sim.Simulation``: one
spherical body covered by blobs, with straight filaments standing on it and
driven by the reference's instability end force (the INSTABILITY_CILIA
branch of config.hpp:236-242):

* end force   F = DIMENSIONLESS_FORCE * KB / (DL^2 NSEG^2), DIMENSIONLESS_FORCE 220;
* time step   dt = 36.3833 / STEPS_PER_PERIOD, STEPS_PER_PERIOD 300;
* repulsion   REPULSIVE_FORCE_FACTOR 2;
* stiffness   KB = KT = 1800 (config.hpp:105-106);
* perturbation per filament: 0.01 F along two random unit directions
  (filament.cpp:344-360), drawn here from the workload's seed.

Geometry follows the reference's seeding conventions: blob references are
the unit seeds scaled to the body radius R (rigid_body.cpp:214-220), filament
bases are the unit seeds scaled to R + 1.05 (DL/2 + RBLOB) (swimmer.cpp:179-199),
with DL = 2.2 RSEG (config.hpp:204).

* ``config1``: R = 10a, 642 blobs on an icosphere (3 subdivisions), 16
  filaments of 20 segments at seeded random icosphere vertices.
* ``config3``: R = 40a, 4096 Fibonacci-lattice blobs, 640 filaments of 20
  segments at seeded random surface points (rejection below an angular
  separation that keeps neighbouring bases 2 DL apart).

The prescribed preferred-curvature beat and metachronal phase lag of the
benchmark's description are not reference features; the filaments here beat
through the reference's own end-force instability.
"""
from __future__ import annotations

import numpy as np

from . import seeding

DIMENSIONLESS_FORCE = 220.0
STEPS_PER_PERIOD = 300


def instability_parameters(nseg: int, rseg: float = 1.0, kb: float = 1800.0, kt: float = 1800.0) -> dict:
    dl = 2.2 * rseg
    return dict(kb=kb, kt=kt, end_force_magnitude=DIMENSIONLESS_FORCE * kb / (dl * dl * nseg * nseg),
                dt=36.3833 / STEPS_PER_PERIOD, repulsive_force_factor=2.0)


def _perturbations(rng, nfil: int, magnitude: float):
    d1 = rng.normal(size=(nfil, 3))
    d2 = rng.normal(size=(nfil, 3))
    d1 *= magnitude / np.linalg.norm(d1, axis=1, keepdims=True)
    d2 *= magnitude / np.linalg.norm(d2, axis=1, keepdims=True)
    return d1, d2


def free_swimmer(blob_seeds, fil_seeds, radius: float, nseg: int, seed: int, rseg: float = 1.0, rblob: float = 1.0,
                 tol: float = 1e-4, linear_tol: float = 1e-8, max_linear_iter: int = 150) -> dict:
    blob_seeds = np.asarray(blob_seeds, dtype=np.float64)
    fil_seeds = np.asarray(fil_seeds, dtype=np.float64)
    nfil = fil_seeds.shape[0]
    dl = 2.2 * rseg
    phys = instability_parameters(nseg, rseg)
    p1, p2 = _perturbations(np.random.default_rng(seed + 17), nfil, 0.01 * phys["end_force_magnitude"])
    return dict(nfil=nfil, nseg=nseg, nblob=blob_seeds.shape[0], blob_refs=radius * blob_seeds,
                fil_refs=fil_seeds * (radius + 1.05 * (0.5 * dl + rblob)), perturbation1=p1, perturbation2=p2,
                mu=1.0, rseg=rseg, rblob=rblob, body_radius=radius, tol=tol, linear_tol=linear_tol,
                max_linear_iter=max_linear_iter, **phys)


def random_surface_points(n: int, min_angle: float, seed: int) -> np.ndarray:
    """n unit vectors, uniform on the sphere, each at least min_angle (radians)
    from every earlier one (random sequential addition)."""
    rng = np.random.default_rng(seed)
    cmax = np.cos(min_angle)
    pts = np.empty((n, 3))
    k = 0
    for _ in range(10000):
        cand = rng.normal(size=(4 * n, 3))
        cand /= np.linalg.norm(cand, axis=1, keepdims=True)
        for c in cand:
            if k == 0 or np.max(pts[:k] @ c) < cmax:
                pts[k] = c
                k += 1
                if k == n:
                    return pts
    raise RuntimeError("random_surface_points: could not place every point")


def config1(seed: int = 2026) -> dict:
    verts = seeding.icosphere(3)
    rng = np.random.default_rng(seed)
    fils = verts[rng.choice(len(verts), 16, replace=False)]
    return free_swimmer(verts, fils, radius=10.0, nseg=20, seed=seed)


def config3(seed: int = 2026) -> dict:
    radius, nseg = 40.0, 20
    base = radius + 1.05 * (0.5 * 2.2 + 1.0)
    fils = random_surface_points(640, 2.0 * 2.2 / base, seed)
    return free_swimmer(seeding.fibonacci_sphere(4096), fils, radius=radius, nseg=nseg, seed=seed)


WORKLOADS = {
    "config1": ("1 swimmer, R=10a, 642 icosphere blobs, 16 x 20 segments (962 particles)", config1),
    "config3": ("1 swimmer, R=40a, 4096 Fibonacci blobs, 640 x 20 segments (16,896 particles)", config3),
}


def main(argv=None) -> None:
    """Run a seeded workload through the device time step and print, per
    step, the Broyden and GMRES iteration counts and the wall time:

        python -m generic_mobility_interface_class_gb300.workloads config3 --precision fp32c --steps 3
    """
    import argparse
    import time

    from . import build
    from ._lib import GMI_FP32C, GMI_FP64
    from .sim import Simulation

    p = argparse.ArgumentParser(prog="python -m generic_mobility_interface_class_gb300.workloads")
    p.add_argument("workload", choices=sorted(WORKLOADS))
    p.add_argument("--precision", choices=["fp64", "fp32c"], default="fp32c")
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--device", type=int, default=0)
    args = p.parse_args(argv)
    build.build()
    desc, make = WORKLOADS[args.workload]
    sim = Simulation(**make(), precision=GMI_FP32C if args.precision == "fp32c" else GMI_FP64, device=args.device)
    t0 = time.perf_counter()
    sim.prepare()
    print(f"{args.workload} ({desc}), {args.precision}: prepare {1e3 * (time.perf_counter() - t0):.1f} ms", flush=True)
    for nt in range(args.steps):
        t0 = time.perf_counter()
        b, g = sim.step(nt)
        print(f"step {nt}: {b} Broyden iterations, {g} GMRES iterations, {1e3 * (time.perf_counter() - t0):.1f} ms",
              flush=True)
    sim.close()


if __name__ == "__main__":
    main()
