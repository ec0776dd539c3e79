"""The reference's own CUDA kernels, built for sm_103a from its
cuda_functions.cu (make -C oracle ref-gpu) and run on this GPU through the
driver API (oracle/ref_gpu.py), against this library's FP64 and FP32C pair
sums and the CPU oracle, on the microbenchmark's N = 16,384 cube.  Skipped
where the cubins were not built (they need the reference tree at build
time)."""
import numpy as np
import pytest

from conftest import per_target_rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

N = 16384


@pytest.fixture(scope="module")
def ref_kernels(gmi_lib):
    from oracle import ref_gpu
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not ref_gpu.available(N):
        pytest.skip("reference cubins not built")
    k = ref_gpu.RefKernels(N)
    yield k
    k.close()


def cube(seed=2026):
    from generic_mobility_interface_class_gb300 import seeding
    x = seeding.random_cube(N, min_sep=2.2, phi=0.05, a=1.0, seed=seed)
    f = np.random.default_rng(seed + 1).normal(size=(N, 6))
    return x, f


def test_reference_cuda_mss_against_this_library_and_the_oracle(ref_kernels, oracle_built):
    from generic_mobility_interface_class_gb300.mobility import Context
    x, f = cube()
    X = torch.as_tensor(x, device="cuda")
    F = torch.as_tensor(f, device="cuda")
    V = torch.empty((N, 6), dtype=torch.float64, device="cuda")
    ref_kernels.mss(V, F, X)
    torch.cuda.synchronize()
    v_ref = V.cpu().numpy()
    # the CPU oracle on a slice of targets
    want = oracle_built.mss(x, f, targets=(1000, 256))
    assert per_target_rel(v_ref[1000:1256], want)[0] < 1e-12
    with Context(0) as ctx:
        ctx.set_precision(0)
        v64 = ctx.mss(X, F).cpu().numpy()
        ctx.set_precision(1)
        v32 = ctx.mss(X, F).cpu().numpy()
        ctx.synchronize()
    assert per_target_rel(v64, v_ref)[0] < 1e-10
    assert per_target_rel(v32, v_ref)[0] < 2e-5


def test_reference_cuda_mbb_against_this_library(ref_kernels):
    from generic_mobility_interface_class_gb300.mobility import Context
    x, f = cube(7)
    X = torch.as_tensor(x, device="cuda")
    F = torch.as_tensor(np.ascontiguousarray(f[:, :3]), device="cuda")
    # the reference writes the targets of [start, start + num) from V's first row
    V = torch.empty((5000, 3), dtype=torch.float64, device="cuda")
    ref_kernels.mbb(V, F, X, start=100, num=5000)
    torch.cuda.synchronize()
    with Context(0) as ctx:
        got = ctx.mbb(X, F, start=100, num=5000).cpu().numpy()
        ctx.synchronize()
    assert per_target_rel(got, V.cpu().numpy())[0] < 1e-10
