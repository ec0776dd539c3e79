"""The CPU oracle (oracle/rpy_oracle.c) against the reference's own kernels.

Two pins: the committed golden fixtures (made by tests/golden/make_golden.py
from cuda_functions.cu compiled for the CPU), and, where the reference tree
is present, fresh random inputs run through the reference kernels directly.
"""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, golden_cases, load_golden, rel_err

FREE = [c for c in golden_cases() if not c.startswith("wall")]
WALL = [c for c in golden_cases() if c.startswith("wall")]


@pytest.mark.parametrize("case", FREE)
def test_oracle_matches_golden_free(case, oracle_built):
    rpy = oracle_built
    g = load_golden(case)
    rs, rb, mu = float(g["rseg"]), float(g["rblob"]), float(g["mu"])
    assert rel_err(rpy.mss(g["xs"], g["fs"], rs, mu), g["v_ss"]) < 1e-13
    assert rel_err(rpy.mbb(g["xb"], g["fb"], rb, mu), g["v_bb"]) < 1e-13
    assert rel_err(rpy.msb(g["xs"], g["xb"], g["fb"], rs, rb, mu, v_in=g["v_in"]), g["v_sb"]) < 1e-13
    assert rel_err(rpy.mbs(g["xb"], g["xs"], g["fs"], rs, rb, mu), g["v_bs"]) < 1e-13
    fs, fb = rpy.barrier(g["xs"], g["xb"], g["fs"], int(g["nseg"]), rs, rb, float(g["force_scale"]))
    np.testing.assert_array_equal(fs, g["fs_barrier"])
    np.testing.assert_array_equal(fb, g["fb_repulsion"])


@pytest.mark.parametrize("case", WALL)
def test_oracle_matches_golden_wall(case, oracle_built):
    rpy = oracle_built
    g = load_golden(case)
    # the reference writes its wall constants with 15 significant digits
    assert rel_err(rpy.mss_wall(g["xs"], g["fs"]), g["v_ss"]) < 1e-13
    fs, _ = rpy.barrier(g["xs"], np.zeros((0, 3)), g["fs"], int(g["nseg"]), 1.0, 1.0,
                        float(g["force_scale"]), wall=True)
    np.testing.assert_array_equal(fs, g["fs_barrier"])


def test_golden_exercises_every_branch():
    """The fixtures cover near and far fields and all three unequal-radius
    branches (r > a_s + a_b, |a_s - a_b| < r <= a_s + a_b, r <= |a_s - a_b|)."""
    seen = set()
    for case in FREE:
        g = load_golden(case)
        rs, rb = float(g["rseg"]), float(g["rblob"])
        d_ss = np.linalg.norm(g["xs"][:, None] - g["xs"][None], axis=-1)
        d_sb = np.linalg.norm(g["xs"][:, None] - g["xb"][None], axis=-1)
        if np.any((d_ss > 0) & (d_ss <= 2 * rs)):
            seen.add("ss_near")
        if np.any(d_ss > 2 * rs):
            seen.add("ss_far")
        if np.any(d_sb > rs + rb):
            seen.add("sb_far")
        if np.any((d_sb > abs(rs - rb)) & (d_sb <= rs + rb)):
            seen.add("sb_mid")
        if np.any(d_sb <= abs(rs - rb)):
            seen.add("sb_inner")
    assert seen == {"ss_near", "ss_far", "sb_far", "sb_mid", "sb_inner"}


def test_oracle_target_slices(oracle_built):
    rpy = oracle_built
    g = load_golden("swimmer_sphere")
    full = rpy.mss(g["xs"], g["fs"])
    part = rpy.mss(g["xs"], g["fs"], targets=(7, 20))
    np.testing.assert_array_equal(part, full[7:27])
    fullb = rpy.mbb(g["xb"], g["fb"])
    np.testing.assert_array_equal(rpy.mbb(g["xb"], g["fb"], targets=(100, 62)), fullb[100:])


def test_oracle_against_reference_kernels_random(oracle_built):
    rpy = oracle_built
    if not rpy.have_reference_kernels():
        pytest.skip("reference kernels not built (reference tree absent)")
    rng = np.random.default_rng(11)
    for nswim, nfil, nseg, nblob, rs, rb in [(1, 5, 7, 33, 1.0, 1.0), (3, 2, 4, 9, 1.1, 0.7)]:
        S, B = nswim * nfil * nseg, nswim * nblob
        L = 1.8 * (S + B) ** (1 / 3)
        xs, xb = rng.uniform(0, L, (S, 3)), rng.uniform(0, L, (B, 3))
        fs, fb = rng.normal(size=(S, 6)), rng.normal(size=(B, 3))
        R = rpy.RefKernels(nswim, nfil, nseg, nblob, rs, rb, 0.9, 2.0, 1.1)
        assert rel_err(rpy.mss(xs, fs, rs, 0.9), R.mss(xs, fs)) < 1e-13
        assert rel_err(rpy.mbb(xb, fb, rb, 0.9), R.mbb(xb, fb)) < 1e-13
        v0 = rng.normal(size=(S, 6))
        assert rel_err(rpy.msb(xs, xb, fb, rs, rb, 0.9, v_in=v0), R.msb(xs, xb, fb, v0)) < 1e-13
        assert rel_err(rpy.mbs(xb, xs, fs, rs, rb, 0.9), R.mbs(xb, xs, fs)) < 1e-13
        a, b = rpy.barrier(xs, xb, fs, nseg, rs, rb, 2.2)
        c, d = R.barrier(xs, xb, fs)
        np.testing.assert_array_equal(a, c)
        np.testing.assert_array_equal(b, d)


def test_self_mobility_known_answer(oracle_built):
    """A lone particle: v = F/(6 pi mu a), omega = T/(8 pi mu a^3)."""
    rpy = oracle_built
    a, mu = 1.3, 0.7
    f = np.array([[1.0, -2.0, 0.5, 0.3, 0.2, -0.1]])
    v = rpy.mss(np.zeros((1, 3)), f, a, mu)[0]
    np.testing.assert_allclose(v[:3], f[0, :3] / (6 * np.pi * mu * a), rtol=1e-15)
    np.testing.assert_allclose(v[3:], f[0, 3:] / (8 * np.pi * mu * a ** 3), rtol=1e-15)


def test_mobility_symmetry(oracle_built):
    """M_ij = M_ji^T for the 6x6 free-space segment mobility (far and near)."""
    rpy = oracle_built
    for sep in (3.7, 1.4):
        x = np.array([[0.0, 0.0, 0.0], [sep * 0.6, sep * 0.8, 0.0]])
        M = np.zeros((12, 12))
        for c in range(12):
            f = np.zeros((2, 6))
            f.flat[c] = 1.0
            M[:, c] = rpy.mss(x, f).ravel()
        np.testing.assert_allclose(M, M.T, atol=1e-15)
        assert np.all(np.linalg.eigvalsh(M) > 0)


@pytest.mark.parametrize("case", ["prescribed", "prescribed_dynamic"])
def test_prescribed_system_restatement_against_reference_solutions(case, oracle_built):
    """The dense restatement of the prescribed-cilia system
    (oracle/mobility_dense.py prescribed_system) holds the reference's own
    solutions: |A x - b| / |b| at the GMRES tolerance (1e-10) for every step of
    both golden cases, with the phase speeds given and with them solved for
    (whose b is the interpolated generalised-force table alone)."""
    from oracle import mobility_dense as md
    g = load_golden(case, prefix="")
    nfil, nseg = int(g["nfil"]), int(g["nseg"])
    S = nfil * nseg
    for k in range(len(g["gmres_iters"])):
        x = [g["f_segs"][k].reshape(S, 6)[:, :3].ravel(), g["f_blobs"][k], g["v_bodies"][k]]
        if case == "prescribed_dynamic":
            x.append(g["phase_speed_out"][k])
            kw = dict(table=g["gen_force_refs"], phase=g["phase"][k], omega0=g["omega0"][k])
        else:
            kw = dict(phase_speed=g["phase_speed"][k])
        Ax, b = md.prescribed_system(np.concatenate(x), g["x_segs"][k], g["body_x"][k], g["body_q"][k],
                                     g["blob_refs"], g["vel_dir"][k], nfil, nseg, float(g["rseg"]),
                                     float(g["rblob"]), float(g["mu"]), **kw)
        assert np.linalg.norm(Ax - b) / np.linalg.norm(b) < 2e-10, (case, k)


def test_generalised_force_interpolation_edges():
    """The table interpolation hits the samples at phases 2 pi j / n, wraps
    over the period (phase + 2 pi, negative phases) and runs from sample
    n - 1 back to sample 0 near 2 pi; with samples of a smooth periodic
    function it is close to that function between the samples."""
    from oracle.mobility_dense import generalised_force
    n = 300
    ph = 2 * np.pi * np.arange(n) / n
    table = 3.0 + np.cos(ph) + 0.5 * np.sin(2 * ph)
    assert np.allclose(generalised_force(table, ph), table, rtol=0, atol=1e-12)
    assert np.allclose(generalised_force(table, ph + 2 * np.pi), table, rtol=0, atol=1e-12)
    assert np.allclose(generalised_force(table, ph - 4 * np.pi), table, rtol=0, atol=1e-12)
    mid = 2 * np.pi * (np.arange(n) + 0.37) / n
    exact = 3.0 + np.cos(mid) + 0.5 * np.sin(2 * mid)
    got = generalised_force(table, mid)
    assert np.max(np.abs(got[1:-1] - exact[1:-1])) < 1e-6
    # the first and last intervals take one-sided differences at sample 0
    assert abs(got[0] - exact[0]) < 1e-4 and abs(got[-1] - exact[-1]) < 1e-4
    # the last interval runs back to sample 0
    assert min(table[-1], table[0]) - 1e-3 <= generalised_force(table, [2 * np.pi - 1e-9])[0] <= \
        max(table[-1], table[0]) + 1e-3


@pytest.mark.parametrize("case", ["prescribed", "prescribed_dynamic"])
def test_prescribed_fixtures_regenerate_from_the_reference(case):
    """tests/golden/<case>.npz is what the reference's own builds produce:
    its CILIA_TYPE 3 simulator driven by oracle/ref_solver/prescribed_dump.cpp
    (and, for the solved phase speeds, the generalised-force table its own
    WRITE_GENERALISED_FORCES run writes), rebuilt and rerun here; every array
    matches the committed fixture exactly.  Skipped without the reference
    tree."""
    from oracle import reference_dir
    if not os.path.isfile(os.path.join(reference_dir(), "mobility_solver.cpp")):
        pytest.skip("reference tree not present")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden_prescribed as mg
    fresh = mg.collect(case)
    want = load_golden(case, prefix="")
    assert sorted(fresh) == sorted(want)
    for k in want:
        assert np.array_equal(np.asarray(fresh[k]), want[k]), k


@pytest.mark.parametrize("case", ["small_swimmer", "two_swimmers", "wall_filaments"])
def test_trajectory_fixtures_regenerate_from_the_reference(case):
    """tests/golden/sim_<case>.npz is the reference's own simulator,
    rebuilt from its unmodified sources and rerun here
    (tests/golden/make_golden_sim.py): every committed array matches the
    fresh run exactly.  (The generator has since added a few scalar keys the
    older fixtures do not carry.)  Skipped without the reference tree."""
    from oracle import reference_dir
    if not os.path.isfile(os.path.join(reference_dir(), "mobility_solver.cpp")):
        pytest.skip("reference tree not present")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden_sim as mg
    name, fresh = mg.collect(case)
    want = load_golden(name, prefix="")
    assert set(want) <= set(fresh)
    for k in want:
        assert np.array_equal(np.asarray(fresh[k]), want[k]), k
