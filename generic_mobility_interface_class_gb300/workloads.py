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
* ``config4``: 64 independent swimmers of uneven size (radius 10a-40a,
  642-4096 blobs, 16-512 filaments, fewer where the surface holds fewer),
  a list of keyword sets for ``batch.SwimmerBatch``.
* ``config5``: R = 100a, 10,242 icosphere blobs (5 subdivisions), 8000
  filaments of 20 segments on a Fibonacci lattice (170,242 particles).

``config1_beat`` and ``config3_beat`` drive the same geometries the way the
benchmark describes them instead: a prescribed sinusoidal preferred-curvature
beat (period 1, a random phase per filament for config 1, the metachronal
lag 2 pi (azimuth / 2 pi) 4 for config 3), KB = KT = 1, dt = 1/300, no end
force.  The beat is not a reference feature; it enters through the
reference's own preferred-curvature hook (strain_twist,
filament.cpp:1104-1106; gmi_sim_set_beat).
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
                 tol: float = 1e-4, linear_tol: float = 1e-8, max_linear_iter: int = 150, kb: float = 1800.0,
                 kt: float = 1800.0) -> dict:
    blob_seeds = np.asarray(blob_seeds, dtype=np.float64)
    fil_seeds = np.asarray(fil_seeds, dtype=np.float64)
    nfil = fil_seeds.shape[0]
    dl = 2.2 * rseg
    phys = instability_parameters(nseg, rseg, kb, kt)
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


def max_filaments(radius: float, rseg: float = 1.0, rblob: float = 1.0, fill: float = 0.6) -> int:
    """How many filament bases random sequential addition places on a body
    of this radius with neighbouring bases 2 DL apart, as a fraction fill of
    the jamming count (0.547 of the sphere covered by disks of radius DL)."""
    dl = 2.2 * rseg
    base = radius + 1.05 * (0.5 * dl + rblob)
    return int(fill * 0.547 * 4.0 * np.pi * base * base / (np.pi * dl * dl))


def config4(seed: int = 2026, nswim: int = 64, radius=(10.0, 40.0), blobs=(642, 4096), filaments=(16, 512),
            nseg: int = 20) -> list[dict]:
    """Independent swimmers of uneven size, one ``Simulation`` keyword set
    each.  Per swimmer, from the seed: the radius uniform in ``radius``;
    Fibonacci-lattice blobs, their count growing linearly with the radius
    across ``blobs``; a filament count log-uniform in ``filaments``, capped by
    ``max_filaments`` so that the bases keep 2 DL apart (a 10a sphere holds
    40 of them); bases at random surface points."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(radius[0], radius[1], size=nswim)
    f = np.exp(rng.uniform(np.log(filaments[0]), np.log(filaments[1]), size=nswim))
    span = max(radius[1] - radius[0], 1e-300)
    out = []
    for i in range(nswim):
        nblob = int(round(blobs[0] + (blobs[1] - blobs[0]) * (r[i] - radius[0]) / span))
        nfil = max(1, min(int(round(f[i])), max_filaments(r[i])))
        base = r[i] + 1.05 * (0.5 * 2.2 + 1.0)
        fils = random_surface_points(nfil, 2.0 * 2.2 / base, seed + 1000 * (i + 1))
        out.append(free_swimmer(seeding.fibonacci_sphere(nblob), fils, radius=float(r[i]), nseg=nseg,
                                seed=seed + 1000 * (i + 1)))
    return out


def config5(seed: int = 2026) -> dict:
    """R = 100a, 10,242 icosphere blobs (5 subdivisions), 8000 filaments of
    20 segments (170,242 particles), driven by the instability end force.
    8000 bases do not fit at 2 DL apart on this sphere (about 2,800 do), so
    they sit on a Fibonacci lattice, about 4a (1.8 DL) apart."""
    return free_swimmer(seeding.icosphere(5), seeding.fibonacci_sphere(8000), radius=100.0, nseg=20, seed=seed)


# ---- the prescribed preferred-curvature beat ---------------------------------
# KB = KT = 1, dt = 1/300, period 1; the preferred bending curvature
# amplitude sin(2 pi t + phase), with amplitude pi / (2 L) (a quarter turn
# over the filament length L = NSEG DL); no end force (the barrier keeps the
# instability workloads' scale for KB = 1).  An extension of the reference
# through its strain_twist hook (filament.cpp:1104-1106).
BEAT_PERIOD = 1.0


def beat_swimmer(blob_seeds, fil_seeds, radius: float, nseg: int, seed: int, phases) -> dict:
    kw = free_swimmer(blob_seeds, fil_seeds, radius, nseg, seed, kb=1.0, kt=1.0)
    kw["dt"] = BEAT_PERIOD / STEPS_PER_PERIOD
    length = nseg * 2.2 * kw["rseg"]
    kw["beat"] = dict(amplitude=np.pi / (2.0 * length), period=BEAT_PERIOD,
                      phases=np.asarray(phases, dtype=np.float64), end_force_scale=0.0)
    return kw


def config1_beat(seed: int = 2026) -> dict:
    """config1's geometry driven by the beat, a random phase per filament."""
    verts = seeding.icosphere(3)
    rng = np.random.default_rng(seed)
    fils = verts[rng.choice(len(verts), 16, replace=False)]
    phases = np.random.default_rng(seed + 5).uniform(0.0, 2.0 * np.pi, size=16)
    return beat_swimmer(verts, fils, radius=10.0, nseg=20, seed=seed, phases=phases)


def config3_beat(seed: int = 2026) -> dict:
    """config3's geometry driven by the beat with the metachronal phase lag
    2 pi (azimuth / 2 pi) 4, the azimuth of each filament's base."""
    radius, nseg = 40.0, 20
    base = radius + 1.05 * (0.5 * 2.2 + 1.0)
    fils = random_surface_points(640, 2.0 * 2.2 / base, seed)
    azimuth = np.mod(np.arctan2(fils[:, 1], fils[:, 0]), 2.0 * np.pi)
    phases = 2.0 * np.pi * (azimuth / (2.0 * np.pi)) * 4.0
    return beat_swimmer(seeding.fibonacci_sphere(4096), fils, radius=radius, nseg=nseg, seed=seed, phases=phases)


WORKLOADS = {
    "config1": ("1 swimmer, R=10a, 642 icosphere blobs, 16 x 20 segments (962 particles)", config1),
    "config3": ("1 swimmer, R=40a, 4096 Fibonacci blobs, 640 x 20 segments (16,896 particles)", config3),
    "config5": ("1 swimmer, R=100a, 10,242 icosphere blobs, 8000 x 20 segments (170,242 particles)", config5),
    "config1_beat": ("config1 geometry, preferred-curvature beat (random phases), KB=KT=1, dt=1/300", config1_beat),
    "config3_beat": ("config3 geometry, preferred-curvature beat (metachronal lag 4 x azimuth), KB=KT=1, dt=1/300",
                     config3_beat),
}

# Workloads of independent swimmers (a list of Simulation keyword sets), run
# by batch.SwimmerBatch.
BATCH_WORKLOADS = {
    "config4": ("64 independent swimmers, R ~ U[10a, 40a], 642-4096 Fibonacci blobs, 16-512 (log-uniform, "
                "capped by the surface) x 20 segments", config4),
}


def main(argv=None) -> None:
    """Run a seeded workload through the device time step and print, per
    step, the Broyden and GMRES iteration counts and the wall time:

        python -m generic_mobility_interface_class_gb300.workloads config3 --precision fp32c --steps 3
        python -m generic_mobility_interface_class_gb300.workloads config4 --swimmers 64 --steps 3
        python -m generic_mobility_interface_class_gb300.workloads config4 --steps 3 --no-barrier
    """
    import argparse
    import time

    from . import build
    from ._lib import GMI_FP32C, GMI_FP64
    from .batch import SwimmerBatch
    from .sim import Simulation

    p = argparse.ArgumentParser(prog="python -m generic_mobility_interface_class_gb300.workloads")
    p.add_argument("workload", choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS))
    p.add_argument("--precision", choices=["fp64", "fp32c"], default="fp32c")
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--device", type=int, default=0)
    p.add_argument("--swimmers", type=int, default=64, help="swimmers of a batch workload")
    p.add_argument("--threads", type=int, default=None, help="host threads of a batch workload (default: one each)")
    p.add_argument("--per-swimmer", action="store_true",
                   help="batch workloads: also print each swimmer's Broyden and GMRES iterations per step")
    p.add_argument("--profile-from", type=int, default=None,
                   help="bracket steps from this one to the last with cudaProfilerStart/Stop, so that a profiler "
                        "started with --profile-from-start off captures only those steps")
    p.add_argument("--no-barrier", action="store_true",
                   help="batch workloads: after step 0, run the remaining steps with SwimmerBatch.run (no "
                        "batch-wide barrier between steps) and print their total time")
    args = p.parse_args(argv)
    build.build()
    prec = GMI_FP32C if args.precision == "fp32c" else GMI_FP64
    if args.workload in BATCH_WORKLOADS:
        desc, make = BATCH_WORKLOADS[args.workload]
        t0 = time.perf_counter()
        sim = SwimmerBatch(make(nswim=args.swimmers), precision=prec, device=args.device, threads=args.threads)
        sim.prepare()
    else:
        desc, make = WORKLOADS[args.workload]
        t0 = time.perf_counter()
        sim = Simulation(**make(), precision=prec, device=args.device)
        sim.prepare()
    print(f"{args.workload} ({desc}), {args.precision}: prepare {1e3 * (time.perf_counter() - t0):.1f} ms", flush=True)
    batch = isinstance(sim, SwimmerBatch)
    profiling = False
    for nt in range(args.steps):
        if args.profile_from is not None and nt == args.profile_from:
            import torch
            torch.cuda.synchronize()
            torch.cuda.profiler.start()
            profiling = True
        if batch and args.no_barrier and nt == 1:
            t0 = time.perf_counter()
            runs = sim.run(args.steps - 1, nt)
            ms = 1e3 * (time.perf_counter() - t0)
            b = sum(x[0] for r in runs for x in r)
            g = sum(x[1] for r in runs for x in r)
            n = args.steps - 1
            print(f"steps 1-{n}, no barrier: {len(runs)} swimmers, {b} Broyden and {g} GMRES iterations in all, "
                  f"{ms:.1f} ms ({ms / n:.1f} ms per batch step)", flush=True)
            break
        t0 = time.perf_counter()
        it = sim.step(nt)
        ms = 1e3 * (time.perf_counter() - t0)
        if isinstance(it, list):
            b, g = sum(x[0] for x in it), sum(x[1] for x in it)
            print(f"step {nt}: {len(it)} swimmers, {b} Broyden and {g} GMRES iterations in all, {ms:.1f} ms",
                  flush=True)
            if args.per_swimmer:
                print("  per swimmer (Broyden, GMRES): " + " ".join(f"{x[0]},{x[1]}" for x in it), flush=True)
        else:
            print(f"step {nt}: {it[0]} Broyden iterations, {it[1]} GMRES iterations, {ms:.1f} ms", flush=True)
    if profiling:
        import torch
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    sim.close()


if __name__ == "__main__":
    main()
