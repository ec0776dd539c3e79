"""The reference's .backup and .dat text formats (host code, no GPU)."""
import numpy as np
import pytest

from conftest import load_golden

from generic_mobility_interface_class_gb300 import formats


def test_backup_text_is_the_references():
    # std::scientific with setprecision(10), the completed-step count first
    # (cilia_sim_main.cpp:370-381)
    assert formats.format_backup(12, [1.5, -2e-3, 0.0]) == "12 1.5000000000e+00 -2.0000000000e-03 0.0000000000e+00 \n"
    nt, v = formats.parse_backup("12 1.5000000000e+00 -2.0000000000e-03 \n")
    assert nt == 12 and np.array_equal(v, [1.5, -2e-3])


@pytest.mark.parametrize("case", ["small_swimmer", "two_swimmers", "wall_filaments", "config1"])
def test_backup_length_matches_reference_files(case):
    g = load_golden(case, prefix="sim_")
    nswim = int(g["nswim"]) if "nswim" in g else 1
    assert g["backup"].shape[1] == formats.backup_count(nswim, int(g["nfil"]), int(g["nseg"]))


def test_backup_round_trip(tmp_path):
    v = np.random.default_rng(1).normal(size=2295) * 10.0 ** np.random.default_rng(2).integers(-8, 3, size=2295)
    path = str(tmp_path / "x.backup")
    formats.write_backup(path, 7, v, digits=17)
    nt, back = formats.read_backup(path)
    assert nt == 7 and np.array_equal(back, v)
    formats.write_backup(path, 7, v)  # the reference's 10 digits
    assert np.max(np.abs(formats.read_backup(path)[1] - v) / np.maximum(np.abs(v), 1e-300)) < 6e-11


def test_dat_files(tmp_path):
    prefix = str(tmp_path / "run")
    q = np.arange(8.0).reshape(2, 4)
    formats.write_step_data(prefix, 0, q, np.zeros((1, 3)), [[1.0, 0, 0, 0]], np.ones((2, 6)), np.ones((2, 6)),
                            body_v=np.zeros(6), blob_f=np.zeros(9))
    formats.write_step_data(prefix, 1, q, np.zeros((1, 3)), [[1.0, 0, 0, 0]], np.ones((2, 6)), np.ones((2, 6)))
    labels, rows = formats.read_dat(prefix + "_seg_states.dat")
    assert list(labels) == [1, 2] and np.array_equal(rows[0], q.ravel())  # nt + 1 (cilia_sim_main.cpp:346)
    labels, rows = formats.read_dat(prefix + "_seg_vels.dat")
    assert list(labels) == [0, 1]  # nt (mobility_solver.cpp:1781-1795)
    labels, rows = formats.read_dat(prefix + "_body_states.dat")
    assert np.array_equal(rows[0], [0, 0, 0, 1, 0, 0, 0])  # x then q (rigid_body.cpp:402-406)
    assert list(formats.read_dat(prefix + "_body_vels.dat")[0]) == [0]
