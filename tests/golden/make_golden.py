"""Generate the golden pair-sum fixtures from the reference's own kernels.

Runs cuda_functions.cu (Mss_mult free and wall, Mbb_mult, Msb_mult,
Mbs_mult, barrier_forces), compiled for the CPU by `make -C oracle ref`, on
small seeded inputs and stores inputs and outputs in pairs_<case>.npz.
Needs the reference tree (GMI_REFERENCE_DIR, or a ``reference`` directory
beside the repository);
the fixtures it writes are committed, so the tests never need the tree.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import rpy  # noqa: E402
from generic_mobility_interface_class_gb300 import seeding  # noqa: E402

# (name, nswim, nfil, nseg, nblob, rseg, rblob, mu, rff, efm, layout)
CASES = [
    ("overlap_equal", 1, 4, 6, 40, 1.0, 1.0, 1.0, 2.0, 3.5, "cloud"),
    ("overlap_unequal", 2, 3, 5, 20, 1.0, 1.4, 1.3, 2.0, 1.25, "cloud"),
    ("blob_bigger_inner", 1, 2, 4, 12, 0.6, 1.5, 0.8, 1.0, 2.0, "tight"),
    ("swimmer_sphere", 1, 6, 10, 162, 1.0, 1.0, 1.0, 2.0, 0.4, "swimmer"),
    ("single_particle", 1, 1, 1, 1, 1.0, 1.0, 1.0, 1.0, 1.0, "cloud"),
]
WALL_CASES = [
    ("wall_filaments", 4, 5, 2.0, 3.0),
    ("wall_near", 3, 4, 2.0, 12.0),
]


def make_inputs(rng, S, B, layout, nfil, nseg):
    if layout == "cloud":
        L = 2.0 * (S + B) ** (1.0 / 3.0)
        xs = rng.uniform(0, L, (S, 3))
        xb = rng.uniform(0, L, (B, 3))
    elif layout == "tight":
        xs = rng.uniform(0, 2.0, (S, 3))
        xb = rng.uniform(0, 2.0, (B, 3))
    else:  # a sphere of blobs (icosphere level 2) with radial filaments
        R = 8.0
        xb = R * seeding.icosphere(2)[:B]
        dirs = seeding.icosphere(1)[rng.choice(42, nfil, replace=False)]
        xs = seeding.radial_filaments(dirs, R + 2.1, nseg)
        xs += 0.3 * rng.normal(size=xs.shape)
    fs = rng.normal(size=(S, 6))
    fb = rng.normal(size=(B, 3))
    v_in = rng.normal(size=(S, 6))
    return xs, xb, fs, fb, v_in


def main():
    rpy.build(with_reference=True)
    rng = np.random.default_rng(2026)
    for name, nswim, nfil, nseg, nblob, rs, rb, mu, rff, efm, layout in CASES:
        S, B = nswim * nfil * nseg, nswim * nblob
        xs, xb, fs, fb, v_in = make_inputs(rng, S, B, layout, nfil, nseg)
        R = rpy.RefKernels(nswim, nfil, nseg, nblob, rs, rb, mu, rff, efm)
        fs_bar, fb_rep = R.barrier(xs, xb, fs)
        out = dict(
            nswim=nswim, nfil=nfil, nseg=nseg, nblob=nblob, rseg=rs, rblob=rb, mu=mu,
            force_scale=rff * efm, wall=0,
            xs=xs, xb=xb, fs=fs, fb=fb, v_in=v_in,
            v_ss=R.mss(xs, fs), v_bb=R.mbb(xb, fb), v_sb=R.msb(xs, xb, fb, v_in), v_bs=R.mbs(xb, xs, fs),
            fs_barrier=fs_bar, fb_repulsion=fb_rep,
        )
        np.savez_compressed(os.path.join(HERE, f"pairs_{name}.npz"), **out)
        print(name, S, B)
    for name, nfil, nseg, rff, zmax in WALL_CASES:
        S = nfil * nseg
        xs = rng.uniform(0, 8.0, (S, 3))
        xs[:, 2] = rng.uniform(0.6, zmax, S)
        fs = rng.normal(size=(S, 6))
        efm = 1.7
        R = rpy.RefKernels(1, nfil, nseg, 0, 1.0, 1.0, 1.0, rff, efm, wall=True)
        fs_bar, _ = R.barrier(xs, np.zeros((0, 3)), fs)
        np.savez_compressed(os.path.join(HERE, f"pairs_{name}.npz"),
                            nswim=1, nfil=nfil, nseg=nseg, nblob=0, rseg=1.0, rblob=1.0, mu=1.0,
                            force_scale=rff * efm, wall=1, xs=xs, fs=fs, v_ss=R.mss(xs, fs), fs_barrier=fs_bar)
        print(name, S)


if __name__ == "__main__":
    main()
