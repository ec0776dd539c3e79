"""GPU parity of the segment mobility apply at the microbenchmark's sizes.

The apply benchmark runs N = 16,384 ... 131,072 particles in a cube at volume
fraction 0.05 with rejection below 2.2a, f and tau ~ N(0,1) (the 6-dof
Mss_mult formula, cuda_functions.cu:246-425).  These tests compare the CUDA
path through the C ABI with the FP64 CPU oracle on those same inputs:

* N = 16,384: every target (2.7e8 pairs);
* N = 131,072: 1,024 targets in eight slices spread over the index range,
  so several target CTAs and every source split of the tiled kernels are
  covered, with the default launch shape and with the autotuned one (the
  shape the benchmark times).

Errors are per target (|v_i - v_i^oracle| / |v_i^oracle| for v and omega
separately) as well as max-normalised.  Bounds: FP64 1e-10 per target;
FP32C 2e-5 per target and 2e-6 max-normalised.
"""
import numpy as np
import pytest

from conftest import per_target_rel, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FP64_PER_TARGET = 1e-10
FP32C_PER_TARGET = 2e-5
FP32C_GLOBAL = 2e-6


def T(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def cube_inputs(n, seed):
    from generic_mobility_interface_class_gb300 import seeding
    x = seeding.random_cube(n, min_sep=2.2, phi=0.05, a=1.0, seed=seed)
    f = np.random.default_rng(seed + 1).normal(size=(n, 6))
    return x, f


def slices(n, count=8, width=128):
    """count target slices of width, spread evenly over [0, n), the last
    ending at n."""
    starts = np.linspace(0, n - width, count).astype(int)
    return [(int(s), width) for s in starts]


@pytest.fixture
def own_ctx(gmi_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from generic_mobility_interface_class_gb300.mobility import Context
    ctx = Context(0)
    yield ctx
    ctx.close()


def check(got, want, prec):
    pt_max, pt_rms = per_target_rel(got, want)
    g = rel_err(got, want)
    if prec == 0:
        assert pt_max < FP64_PER_TARGET, (pt_max, pt_rms, g)
    else:
        assert pt_max < FP32C_PER_TARGET, (pt_max, pt_rms, g)
        assert g < FP32C_GLOBAL, (pt_max, pt_rms, g)
    return pt_max


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32c"])
def test_n16384_every_target(own_ctx, oracle_built, prec):
    rpy = oracle_built
    n = 16384
    x, f = cube_inputs(n, 2026)
    want = rpy.mss(x, f)
    own_ctx.set_precision(prec)
    got = own_ctx.mss(T(x), T(f)).cpu().numpy()
    own_ctx.synchronize()
    check(got, want, prec)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32c"])
def test_n131072_target_slices(own_ctx, oracle_built, prec):
    rpy = oracle_built
    n = 131072
    x, f = cube_inputs(n, 2026)
    sl = slices(n)
    want = np.concatenate([rpy.mss(x, f, targets=s) for s in sl])
    own_ctx.set_precision(prec)
    xd, fd = T(x), T(f)
    shapes = ["default"]
    if prec == 1:
        shapes.append("autotuned")
    for shape in shapes:
        if shape == "autotuned":
            own_ctx.autotune(0, n, n)
            assert own_ctx.tuned_shape(0, n, n)[3]
        v = own_ctx.mss(xd, fd).cpu().numpy()
        own_ctx.synchronize()
        got = np.concatenate([v[s:s + w] for s, w in sl])
        check(got, want, prec)


def test_n131072_pinned_benchmark_shape(own_ctx, oracle_built):
    """The launch shape the microbenchmark's traffic capture pins (256
    threads, one target each, 8 source splits, two sources per packed step)
    and the scalar kernel with the same split count."""
    rpy = oracle_built
    n = 131072
    x, f = cube_inputs(n, 2026)
    sl = slices(n, count=4)
    want = np.concatenate([rpy.mss(x, f, targets=s) for s in sl])
    own_ctx.set_precision(1)
    xd, fd = T(x), T(f)
    for per_step in (2, 1):
        own_ctx.set_shape(0, n, n, 256, 1, 8, per_step)
        v = own_ctx.mss(xd, fd).cpu().numpy()
        own_ctx.synchronize()
        check(np.concatenate([v[s:s + w] for s, w in sl]), want, 1)
