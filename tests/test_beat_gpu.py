"""The prescribed preferred-curvature beat (gmi_sim_set_beat), an extension
through the reference's strain_twist hook (filament.cpp:1104-1106).

* A beat of zero amplitude with the end force kept is the plain time step,
  bit for bit.
* The beat-driven config-1 workload (KB = KT = 1, dt = 1/300): FP32C pair
  sums with FP64 solves against the FP64 path after 30 steps, at the
  benchmark's error target (swimmer velocity within 1e-5 relative), and the
  beat turns the filaments' segments.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def run(kw, steps, precision):
    from generic_mobility_interface_class_gb300.sim import Simulation
    sim = Simulation(**kw, precision=precision)
    sim.prepare()
    counts = [sim.step(nt) for nt in range(steps)]
    out = {f: sim.state(f) for f in ("seg_x", "seg_q", "body_v", "seg_v", "body_x")}
    sim.close()
    return counts, out


def test_zero_amplitude_beat_is_the_plain_step(gmi_lib):
    from generic_mobility_interface_class_gb300 import workloads
    kw = workloads.config1()
    plain, s0 = run(kw, 4, 1)
    kw = dict(kw, beat=dict(amplitude=0.0, period=1.0, phases=np.zeros(16), end_force_scale=1.0))
    beat, s1 = run(kw, 4, 1)
    assert beat == plain
    for f in s0:
        np.testing.assert_array_equal(s1[f], s0[f])


def test_beat_driven_config1_fp32c_against_fp64(gmi_lib):
    from generic_mobility_interface_class_gb300 import workloads
    kw = workloads.config1_beat()
    steps = 30
    c64, s64 = run(kw, steps, 0)
    c32, s32 = run(kw, steps, 1)
    assert [c[0] for c in c32] == [c[0] for c in c64]  # the same Broyden counts
    ev = np.linalg.norm(s32["body_v"] - s64["body_v"]) / np.linalg.norm(s64["body_v"])
    es = np.linalg.norm(s32["seg_v"] - s64["seg_v"]) / np.linalg.norm(s64["seg_v"])
    assert ev < 1e-5 and es < 1e-5, (ev, es)
    # the beat turns every filament's segments (at KB = 1 slowly: the
    # preferred-curvature moment is ~KB A ~ 0.04 against a rotational drag
    # of 8 pi), and the body moves
    om = np.linalg.norm(s64["seg_v"][:, 3:].reshape(16, 20, 3), axis=2)
    assert np.all(om.max(axis=1) > 1e-5), om.max(axis=1)
    assert np.all(np.isfinite(s64["seg_q"]))
    assert np.linalg.norm(s64["body_v"][0]) > 0.0
