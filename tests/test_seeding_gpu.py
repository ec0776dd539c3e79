"""Repulsive seeding on the unit sphere (gmi_seed_sphere_repulsive), the
reference's blob and uniform filament seeding (seeding.cu:13-160, 233-389).

Against the reference's own GPU path: its seeding_repulsion_step kernel
(cuda_functions.cu:1159-1250, built for sm_103a, oracle/ref_gpu.py) with
its host update restated in numpy, from the same spiral start.  The points
and the number of relaxation steps agree; the points are unit vectors and
no two coincide.  Skipped where the reference cubins were not built.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n", [642, 1500])
def test_seeding_matches_the_reference_kernel(gmi_lib, n):
    from generic_mobility_interface_class_gb300 import _lib
    from oracle import ref_gpu
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not ref_gpu.available(16384):
        pytest.skip("reference cubins not built")
    import ctypes
    got = np.zeros((n, 3))
    steps = ctypes.c_int()
    _lib.check(_lib.load().gmi_seed_sphere_repulsive(0, n, 100000, got.ctypes.data_as(ctypes.c_void_p),
                                                       ctypes.byref(steps)))
    k = ref_gpu.RefKernels(16384)
    want, want_steps = k.seed_sphere(n)
    k.close()
    assert abs(steps.value - want_steps) <= 1, (steps.value, want_steps)
    assert np.abs(got - want).max() < 1e-6
    np.testing.assert_allclose(np.linalg.norm(got, axis=1), 1.0, atol=1e-14)
    d = np.linalg.norm(got[:, None, :] - got[None, :, :], axis=2)
    np.fill_diagonal(d, np.inf)
    # quasi-uniform: the nearest neighbour distance is close to its mean
    nn = d.min(axis=1)
    assert nn.min() > 0.5 * nn.mean()
