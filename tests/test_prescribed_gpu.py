"""Prescribed-shape cilia: the linear solves of mobility_solver::compute_velocities
(CILIA_TYPE 3) against the reference's own, step by step.

tests/golden/prescribed.npz comes from the reference's unmodified sources
built for CILIA_TYPE 3 (its coral-larvae beat fit, phases at constant speed,
one sphere of 162 blobs with 4 x 20-segment cilia) and driven by
oracle/ref_solver/prescribed_dump.cpp, which records what the mobility solver
received and returned at every step (tests/golden/make_golden_prescribed.py).
Each solve here gets the same segment positions, shape-velocity directions,
phase speeds and body state, warm-starts from the previous solve as the
reference does, and must return the same segment forces, blob forces and
body velocities to the GMRES tolerance (1e-10).
"""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu

SOLVE_TOL = 1e-7  # GMRES stops at a relative residual of 1e-10 on both sides


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32c"])
def test_prescribed_solves_match_reference(gmi_lib, precision):
    from generic_mobility_interface_class_gb300.solver import MobilitySolver
    g = load_golden("prescribed", prefix="")
    nfil, nseg, nblob = int(g["nfil"]), int(g["nseg"]), int(g["nblob"])
    s = MobilitySolver(nswim=1, nfil=nfil, nseg=nseg, nblob=nblob, mu=float(g["mu"]), rseg=float(g["rseg"]),
                       rblob=float(g["rblob"]), linear_tol=float(g["linear_tol"]),
                       max_linear_iter=int(g["max_linear_iter"]), precision=precision)
    s.set_blob_references(g["blob_refs"])
    S = nfil * nseg
    tol = SOLVE_TOL if precision == 0 else 1e-4
    for k in range(len(g["gmres_iters"])):
        s.x_segs_host[:] = g["x_segs"][k].reshape(S, 3)
        it = s.compute_velocities_prescribed(g["vel_dir"][k].reshape(S, 3), g["phase_speed"][k],
                                             g["body_x"][k].reshape(1, 3), g["body_q"][k].reshape(1, 4))
        fs = np.array(s.f_segs_host[:, :3])
        want_fs = g["f_segs"][k].reshape(S, 6)[:, :3]
        assert rel_err(fs, want_fs) < tol, (k, rel_err(fs, want_fs))
        assert np.all(np.array(s.f_segs_host[:, 3:]) == 0.0)
        assert rel_err(np.array(s.f_blobs_host), g["f_blobs"][k].reshape(nblob, 3)) < tol, k
        assert rel_err(s.v_bodies().ravel(), g["v_bodies"][k]) < tol, k
        if precision == 0:
            assert abs(it - int(g["gmres_iters"][k])) <= 3, (k, it, int(g["gmres_iters"][k]))
    s.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32c"])
def test_prescribed_dynamic_solves_match_reference(gmi_lib, precision):
    """Phase speeds among the unknowns (DYNAMIC_PHASE_EVOLUTION):
    tests/golden/prescribed_dynamic.npz holds the reference's generalised-force
    table (its own WRITE_GENERALISED_FORCES run over one beat period) and four
    solves of the same swimmer driven by it.  Each solve here gets that
    table, the step's phases, natural frequencies, shapes and body state, and
    omega0 as the phase speeds' initial guess (as the reference); it must
    return the same forces, body velocities and phase speeds.  A static solve
    after the dynamic ones starts cold and still matches its own golden."""
    from generic_mobility_interface_class_gb300.solver import MobilitySolver
    g = load_golden("prescribed_dynamic", prefix="")
    nfil, nseg, nblob = int(g["nfil"]), int(g["nseg"]), int(g["nblob"])
    s = MobilitySolver(nswim=1, nfil=nfil, nseg=nseg, nblob=nblob, mu=float(g["mu"]), rseg=float(g["rseg"]),
                       rblob=float(g["rblob"]), linear_tol=float(g["linear_tol"]),
                       max_linear_iter=int(g["max_linear_iter"]), precision=precision)
    s.set_blob_references(g["blob_refs"])
    s.set_generalised_force_refs(g["gen_force_refs"])
    S = nfil * nseg
    tol = SOLVE_TOL if precision == 0 else 1e-4
    for k in range(len(g["gmres_iters"])):
        s.x_segs_host[:] = g["x_segs"][k].reshape(S, 3)
        it, speeds = s.compute_velocities_prescribed_dynamic(
            g["vel_dir"][k].reshape(S, 3), g["phase"][k], g["omega0"][k], phase_speed=g["phase_speed"][k],
            body_x=g["body_x"][k].reshape(1, 3), body_q=g["body_q"][k].reshape(1, 4))
        assert rel_err(speeds, g["phase_speed_out"][k]) < tol, (k, speeds, g["phase_speed_out"][k])
        want_fs = g["f_segs"][k].reshape(S, 6)[:, :3]
        assert rel_err(np.array(s.f_segs_host[:, :3]), want_fs) < tol, k
        assert np.all(np.array(s.f_segs_host[:, 3:]) == 0.0)
        assert rel_err(np.array(s.f_blobs_host), g["f_blobs"][k].reshape(nblob, 3)) < tol, k
        assert rel_err(s.v_bodies().ravel(), g["v_bodies"][k]) < tol, k
        if precision == 0:
            assert abs(it - int(g["gmres_iters"][k])) <= 3, (k, it, int(g["gmres_iters"][k]))
    st = load_golden("prescribed", prefix="")
    s.x_segs_host[:] = st["x_segs"][0].reshape(S, 3)
    s.compute_velocities_prescribed(st["vel_dir"][0].reshape(S, 3), st["phase_speed"][0],
                                    st["body_x"][0].reshape(1, 3), st["body_q"][0].reshape(1, 4))
    assert rel_err(s.v_bodies().ravel(), st["v_bodies"][0]) < tol
    s.close()


def _two_swimmers(g, k, phase_shift=0.7):
    """The golden swimmer of step k and a copy 3 (R + L) further along x (the
    reference's spacing of swimmers, rigid_body.cpp), its phases shifted."""
    nfil, nseg = int(g["nfil"]), int(g["nseg"])
    L = 2.2 * float(g["rseg"]) * nseg
    R = np.linalg.norm(g["blob_refs"], axis=1).max()
    shift = np.array([3.0 * (R + L), 0.0, 0.0])
    xs0 = g["x_segs"][k].reshape(-1, 3)
    return dict(xs=np.concatenate([xs0, xs0 + shift]),
                bx=np.stack([g["body_x"][k], g["body_x"][k] + shift]),
                bq=np.stack([g["body_q"][k], g["body_q"][k]]),
                vd=np.concatenate([g["vel_dir"][k], g["vel_dir"][k]]).reshape(-1, 3),
                phase=np.concatenate([g["phase"][k], g["phase"][k] + phase_shift]),
                omega0=np.concatenate([g["omega0"][k], g["omega0"][k]]), nfil=nfil, nseg=nseg)


def test_prescribed_dynamic_two_swimmers_against_oracle(gmi_lib, oracle_built):
    """Two swimmers with the phase speeds solved for: the golden geometry and
    a copy 3 (R + L) away with its phases shifted.  The solution satisfies
    the restated system (oracle/mobility_dense.py prescribed_system, pinned
    to the reference's own solutions) to the GMRES tolerance, and matches
    its dense solve.  With several swimmers the reference's preconditioner
    treats the phase rows differently (its block operations over all
    swimmers' phase rows sit inside the loop over swimmers); the system and
    its solution are the same."""
    from generic_mobility_interface_class_gb300.solver import MobilitySolver
    from oracle import mobility_dense as md
    g = load_golden("prescribed_dynamic", prefix="")
    t = _two_swimmers(g, 0)
    nfil, nseg, nblob = t["nfil"], t["nseg"], int(g["nblob"])
    rseg, rblob, mu = float(g["rseg"]), float(g["rblob"]), float(g["mu"])
    s = MobilitySolver(nswim=2, nfil=nfil, nseg=nseg, nblob=nblob, mu=mu, rseg=rseg, rblob=rblob,
                       linear_tol=1e-10, max_linear_iter=150)
    s.set_blob_references(g["blob_refs"])
    s.set_generalised_force_refs(g["gen_force_refs"])
    s.x_segs_host[:] = t["xs"]
    it, speeds = s.compute_velocities_prescribed_dynamic(t["vd"], t["phase"], t["omega0"], body_x=t["bx"],
                                                         body_q=t["bq"])
    x = np.concatenate([np.array(s.f_segs_host[:, :3]).ravel(), np.array(s.f_blobs_host).ravel(),
                        s.v_bodies().ravel(), speeds])
    s.close()
    args = (t["xs"], t["bx"], t["bq"], g["blob_refs"], t["vd"], nfil, nseg, rseg, rblob, mu)
    kw = dict(table=g["gen_force_refs"], phase=t["phase"], omega0=t["omega0"])
    Ax, b = md.prescribed_system(x, *args, **kw)
    assert np.linalg.norm(Ax - b) / np.linalg.norm(b) < 1e-9, it
    n = len(x)
    A = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        A[:, j] = md.prescribed_system(e, *args, **kw)[0]
    xd = np.linalg.solve(A, b)
    assert rel_err(x, xd) < 1e-6
    assert rel_err(speeds, xd[-2 * nfil:]) < 1e-7
    # the two swimmers' phase speeds differ (their phases do)
    assert np.abs(speeds[:nfil] - speeds[nfil:]).max() > 1e-3


def test_prescribed_dynamic_needs_a_table(gmi_lib):
    from generic_mobility_interface_class_gb300._lib import GmiError
    from generic_mobility_interface_class_gb300.solver import MobilitySolver
    g = load_golden("prescribed_dynamic", prefix="")
    nfil, nseg, nblob = int(g["nfil"]), int(g["nseg"]), int(g["nblob"])
    s = MobilitySolver(nswim=1, nfil=nfil, nseg=nseg, nblob=nblob)
    s.set_blob_references(g["blob_refs"])
    S = nfil * nseg
    s.x_segs_host[:] = g["x_segs"][0].reshape(S, 3)
    args = (g["vel_dir"][0].reshape(S, 3), g["phase"][0], g["omega0"][0])
    with pytest.raises(GmiError):
        s.compute_velocities_prescribed_dynamic(*args)
    with pytest.raises(GmiError):
        s.set_generalised_force_refs([1.0])
    with pytest.raises(GmiError):
        s.set_generalised_force_refs([1.0, np.nan])
    s.set_generalised_force_refs(g["gen_force_refs"])
    s.set_generalised_force_refs([])
    with pytest.raises(GmiError):
        s.compute_velocities_prescribed_dynamic(*args)
    s.close()


def test_prescribed_rejects_the_wall(gmi_lib):
    from generic_mobility_interface_class_gb300._lib import GmiError
    from generic_mobility_interface_class_gb300.solver import MobilitySolver
    s = MobilitySolver(nswim=1, nfil=1, nseg=4, nblob=0, wall=True)
    with pytest.raises(GmiError):
        s.compute_velocities_prescribed(np.zeros((4, 3)), np.ones(1))
    s.close()
