"""Seeded synthetic geometries for the benchmark and test workloads.

The reference seeds blobs and filament bases by a repulsive relaxation on
the unit sphere (seeding.cu:13-389), or reads them from sphereN.seed files.
The workloads here instead use deterministic constructions:

* ``icosphere(k)``: vertices of a k-times subdivided icosahedron on the unit
  sphere (642 vertices for k = 3, 10242 for k = 5);
* ``fibonacci_sphere(n)``: the Fibonacci lattice of n points;
* ``random_cube(n, min_sep, phi, a)``: n points uniform in a cube sized for
  volume fraction phi of spheres of radius a, with rejection below min_sep;
* ``radial_filaments``: straight filaments standing on a sphere.

All randomness comes from ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import math

import numpy as np


def icosphere(subdivisions: int) -> np.ndarray:
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache: dict[tuple[int, int], int] = {}

        def mid(i: int, j: int) -> int:
            key = (min(i, j), max(i, j))
            if key not in cache:
                m = verts[i] + verts[j]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        new_faces = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    return np.array(verts)


def fibonacci_sphere(n: int) -> np.ndarray:
    k = np.arange(n, dtype=np.float64)
    z = 1.0 - (2.0 * k + 1.0) / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = k * math.pi * (3.0 - math.sqrt(5.0))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def cube_side(n: int, phi: float = 0.05, a: float = 1.0) -> float:
    return (n * (4.0 / 3.0) * math.pi * a ** 3 / phi) ** (1.0 / 3.0)


def random_cube(n: int, min_sep: float = 2.2, phi: float = 0.05, a: float = 1.0, seed: int = 2026) -> np.ndarray:
    """n points uniform in the cube of side cube_side(n, phi, a); any point
    closer than min_sep to an earlier accepted point is redrawn."""
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    L = cube_side(n, phi, a)
    pts = rng.uniform(0.0, L, size=(n, 3))
    for _ in range(200):
        pairs = cKDTree(pts).query_pairs(min_sep, output_type="ndarray")
        if len(pairs) == 0:
            return pts
        bad = np.unique(pairs.max(axis=1))
        pts[bad] = rng.uniform(0.0, L, size=(len(bad), 3))
    raise RuntimeError("random_cube: rejection did not converge")


def overlapping_cloud(n: int, L: float, seed: int = 7) -> np.ndarray:
    """Uniform points with no rejection (exercises the overlapping branches)."""
    return np.random.default_rng(seed).uniform(0.0, L, size=(n, 3))


def radial_filaments(base_dirs: np.ndarray, base_radius: float, nseg: int, dl: float = 2.2) -> np.ndarray:
    """Segment positions (nfil*nseg, 3) of straight filaments along the unit
    directions base_dirs, first segment at base_radius (the reference's
    straight initial state, filament.cpp:283-295)."""
    d = base_dirs / np.linalg.norm(base_dirs, axis=1, keepdims=True)
    s = base_radius + dl * np.arange(nseg, dtype=np.float64)
    return (d[:, None, :] * s[None, :, None]).reshape(-1, 3)


def repulsive_sphere(n: int, device: int = 0, max_steps: int = 100000) -> np.ndarray:
    """The reference's repulsive seeding of n points on the unit sphere
    (seeding.cu:13-160), run on the GPU by gmi_seed_sphere_repulsive; the
    (n, 3) unit vectors the reference caches as sphere<n>.seed."""
    import ctypes

    from . import _lib
    out = np.zeros((n, 3))
    steps = ctypes.c_int()
    _lib.check(_lib.load().gmi_seed_sphere_repulsive(device, n, max_steps, out.ctypes.data_as(ctypes.c_void_p),
                                                       ctypes.byref(steps)))
    return out
