"""Failure paths on the GPU, none of which faults, traps or hangs the GPU.

* A bounded wait that runs out: the check kernel waits on an mbarrier whose
  second arrival is withheld (a flag nothing sets); with a short deadline
  the wait gives up, the call reports GMI_ERR_DEVICE_TIMEOUT, and the
  context keeps working.
* Non-finite input: a NaN in the host segment forces makes the mobility
  solve report GMI_ERR_NONFINITE (the reference would carry the NaN on).
* A capped linear solve: with max_linear_iter = 2 the reference accepts the
  unconverged GMRES answer silently (mobility_solver.cpp:1234); so does
  this solver by default, and it reports the residual; in strict mode it
  returns GMI_ERR_NOT_CONVERGED.
"""
import time

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture
def own_ctx(gmi_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from generic_mobility_interface_class_gb300.mobility import Context
    ctx = Context(0)
    yield ctx
    ctx.close()


def test_bounded_wait_gives_up_and_context_survives(own_ctx, oracle_built):
    from generic_mobility_interface_class_gb300._lib import GmiError
    ctx = own_ctx
    ctx.set_wait_deadline(2_000_000)  # 2 ms
    ctx.check_bounded_wait(False)  # both arrivals: completes
    t0 = time.perf_counter()
    with pytest.raises(GmiError) as e:
        ctx.check_bounded_wait(True)
    took = time.perf_counter() - t0
    assert e.value.status == 3  # GMI_ERR_DEVICE_TIMEOUT
    assert took < 1.0, took  # gave up at the short deadline, not at the 2 s default
    # the error is reported once; the context keeps working
    ctx.synchronize()
    ctx.check_bounded_wait(False)
    rpy = oracle_built
    from generic_mobility_interface_class_gb300 import seeding
    x = seeding.random_cube(600, seed=4)
    f = np.random.default_rng(4).normal(size=(600, 6))
    ctx.set_wait_deadline(0)
    got = ctx.mss(torch.as_tensor(x, device="cuda"), torch.as_tensor(f, device="cuda")).cpu().numpy()
    ctx.synchronize()
    assert rel_err(got, rpy.mss(x, f)) < 1e-10


def test_wait_deadline_range(own_ctx):
    from generic_mobility_interface_class_gb300._lib import GmiError
    for bad in (-1, 10, 61_000_000_000):
        with pytest.raises(GmiError):
            own_ctx.set_wait_deadline(bad)
    own_ctx.set_wait_deadline(0)
    own_ctx.set_wait_deadline(1000)


def _solver(precision, max_linear_iter=150, linear_tol=1e-8):
    from test_solver_gpu import swimmer_geometry
    from generic_mobility_interface_class_gb300.solver import MobilitySolver
    nfil, nseg = 4, 10
    refs, bx, bq, xs, fs, bf = swimmer_geometry(1, nfil, nseg)
    s = MobilitySolver(nswim=1, nfil=nfil, nseg=nseg, nblob=refs.shape[0], repulsive_force_factor=1.0,
                       end_force_magnitude=1.5, precision=precision, max_linear_iter=max_linear_iter,
                       linear_tol=linear_tol)
    s.set_blob_references(refs)
    s.x_segs_host[:] = xs
    s.f_segs_host[:] = fs
    s.make_body_reference_matrices(bx, bq)
    return s, bx, bq, bf


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32c"])
def test_nan_force_reports_nonfinite(gmi_lib, prec):
    from generic_mobility_interface_class_gb300._lib import GmiError
    s, bx, bq, bf = _solver(prec)
    try:
        s.f_segs_host[7, 2] = np.nan
        with pytest.raises(GmiError) as e:
            s.compute_velocities(bx, bq, bf)
        assert e.value.status == 4  # GMI_ERR_NONFINITE
    finally:
        s.close()


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32c"])
def test_capped_linear_solve(gmi_lib, prec):
    from generic_mobility_interface_class_gb300._lib import GmiError
    tol = 1e-8
    s, bx, bq, bf = _solver(prec, max_linear_iter=2, linear_tol=tol)
    try:
        # the reference's behaviour: the capped answer is accepted
        it, _ = s.compute_velocities(bx, bq, bf)
        iters, resid = s.last_linear_solve()
        assert iters == it and resid > tol
    finally:
        s.close()
    # strict: the same capped solve is reported, its results still written back
    s, bx, bq, bf = _solver(prec, max_linear_iter=2, linear_tol=tol)
    try:
        s.set_strict_convergence(True)
        with pytest.raises(GmiError) as e:
            s.compute_velocities(bx, bq, bf)
        assert e.value.status == 5  # GMI_ERR_NOT_CONVERGED
        assert s.last_linear_solve()[1] > tol
        assert np.all(np.isfinite(s.v_segs_host)) and np.any(s.v_segs_host != 0.0)
    finally:
        s.close()
    # with room to converge, strict mode passes and the residual meets tol
    s, bx, bq, bf = _solver(prec, linear_tol=tol)
    try:
        s.set_strict_convergence(True)
        s.compute_velocities(bx, bq, bf)
        assert s.last_linear_solve()[1] <= tol
    finally:
        s.close()
