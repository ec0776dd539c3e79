"""Checkpoints and time series in the reference's formats, through the
device time step: the exported state after 12 steps against the reference's
own .backup, an import/export round trip, and a restart from the reference's
backup against the reference's own restart (tests/golden/make_golden_sim.py
--restart: INITIAL_CONDITIONS_TYPE 1, cilia_sim_main.cpp:29-77)."""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu


def _sim(g, **kw):
    from generic_mobility_interface_class_gb300.sim import Simulation
    return Simulation.from_golden(g, **kw)


def test_backup_after_12_steps_matches_reference(gmi_lib):
    g = load_golden("small_swimmer", prefix="sim_")
    sim = _sim(g)
    sim.prepare()
    for nt in range(12):
        sim.step(nt)
    got = sim.export_backup()
    sim.close()
    # the reference prints 10 significant digits; the trajectories agree to ~1e-12
    assert got.shape == g["backup"][0].shape
    assert rel_err(got, g["backup"][0]) < 1e-9


def test_backup_import_export_round_trip(gmi_lib):
    g = load_golden("small_swimmer", prefix="sim_")
    sim = _sim(g)
    sim.import_backup(g["backup"][0])
    assert np.array_equal(sim.export_backup(), g["backup"][0])
    sim.close()


def test_restart_matches_reference_restart(gmi_lib, tmp_path):
    g = load_golden("small_swimmer_restart", prefix="sim_")
    sim = _sim(g)
    path = str(tmp_path / "in.backup")
    from generic_mobility_interface_class_gb300 import formats
    formats.write_backup(path, int(g["nt_start"]), g["backup_in"], digits=17)
    nt0 = sim.read_backup(path)
    assert nt0 == int(g["nt_start"])
    sim.prepare()
    for k, nt in enumerate(range(nt0, nt0 + len(g["broyden_iters"]))):
        b, _ = sim.step(nt)
        assert b == int(g["broyden_iters"][k]), (nt, b)
        assert rel_err(sim.state("seg_q").ravel(), g["seg_q"][k]) < 1e-10
        assert rel_err(sim.state("seg_v").ravel(), g["seg_v"][k]) < 1e-7
        assert rel_err(sim.state("body_v").ravel(), g["body_v"][k]) < 1e-7
    sim.close()


def test_dat_writer_against_reference_series(gmi_lib, tmp_path):
    """The first two steps written as the reference's .dat files and read
    back: labels and values of the reference's own series."""
    from generic_mobility_interface_class_gb300 import formats
    g = load_golden("small_swimmer", prefix="sim_")
    sim = _sim(g)
    sim.prepare()
    prefix = str(tmp_path / "run")
    for nt in range(2):
        sim.step(nt)
        sim.write_step_data(prefix, nt)
    sim.close()
    labels, q = formats.read_dat(prefix + "_seg_states.dat")
    assert list(labels) == [1, 2]
    assert rel_err(q, g["seg_q"][:2]) < 1e-9
    labels, v = formats.read_dat(prefix + "_seg_vels.dat")
    assert list(labels) == [0, 1]
    assert rel_err(v, g["seg_v"][:2]) < 1e-7
    _, bs = formats.read_dat(prefix + "_body_states.dat")
    assert np.max(np.abs(bs - g["body_state"][:2])) < 1e-9
    _, fb = formats.read_dat(prefix + "_blob_forces.dat")
    assert rel_err(fb, g["blob_f"][:2]) < 1e-6
