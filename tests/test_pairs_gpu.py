"""GPU parity of the pair sums through the C ABI.

FP64 results must match the reference (golden fixtures from the reference's
own kernels, and the CPU oracle at larger sizes) to 1e-10 relative; FP32C
results carry a stated error bound against the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FP64_TOL = 1e-10      # spec bound for the FP64 path
FP32C_TOL = 2e-6      # max |v - v64| / max |v64| for the compensated FP32 path
DF64_TOL = 1e-12      # the same for the double-float blob-blob sum
FREE = [c for c in golden_cases() if not c.startswith("wall")]
WALL = [c for c in golden_cases() if c.startswith("wall")]


def T(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def N(t):
    return t.detach().cpu().numpy()


@pytest.fixture(params=[0, 1], ids=["fp64", "fp32c"])
def prec_ctx(request, gpu_ctx):
    gpu_ctx.set_precision(request.param)
    yield gpu_ctx, (FP64_TOL if request.param == 0 else FP32C_TOL)
    gpu_ctx.set_precision(0)


@pytest.mark.parametrize("case", FREE)
def test_pairs_match_golden(case, prec_ctx):
    ctx, tol = prec_ctx
    g = load_golden(case)
    rs, rb, mu = float(g["rseg"]), float(g["rblob"]), float(g["mu"])
    xs, xb, fs, fb = T(g["xs"]), T(g["xb"]), T(g["fs"]), T(g["fb"])
    assert rel_err(N(ctx.mss(xs, fs, rs, mu)), g["v_ss"]) < tol
    assert rel_err(N(ctx.mbb(xb, fb, rb, mu)), g["v_bb"]) < tol
    v = T(g["v_in"])
    ctx.msb(xs, xb, fb, v, rs, rb, mu)
    assert rel_err(N(v), g["v_sb"]) < tol
    assert rel_err(N(ctx.mbs(xb, xs, fs, rs, rb, mu)), g["v_bs"]) < tol
    ctx.synchronize()


@pytest.mark.parametrize("case", FREE)
def test_barrier_matches_golden(case, gpu_ctx):
    g = load_golden(case)
    fs = T(g["fs"])
    fb = gpu_ctx.barrier(T(g["xs"]), T(g["xb"]), fs, int(g["nseg"]), float(g["rseg"]), float(g["rblob"]),
                         float(g["force_scale"]))
    gpu_ctx.synchronize()
    assert rel_err(N(fs), g["fs_barrier"]) < 1e-14
    assert rel_err(N(fb), g["fb_repulsion"]) < 1e-14


@pytest.mark.parametrize("case", WALL)
def test_wall_matches_golden(case, prec_ctx):
    ctx, tol = prec_ctx
    g = load_golden(case)
    assert rel_err(N(ctx.mss_wall(T(g["xs"]), T(g["fs"]))), g["v_ss"]) < tol
    fs = T(g["fs"])
    ctx.barrier(T(g["xs"]), torch.zeros((0, 3), dtype=torch.float64, device="cuda"), fs, int(g["nseg"]),
                1.0, 1.0, float(g["force_scale"]), wall=True)
    ctx.synchronize()
    assert rel_err(N(fs), g["fs_barrier"]) < 1e-14


def _swimmer_cloud(nblob, nfil, nseg, R, seed):
    """Blobs on a Fibonacci sphere of radius R and nfil filaments of nseg
    segments (spacing 2.2) standing out of it in random directions, jittered
    so that segments of nearby filaments and base segments and blobs come
    within the barrier's reach."""
    rng = np.random.default_rng(seed)
    k = np.arange(nblob) + 0.5
    polar, az = np.arccos(1 - 2 * k / nblob), np.pi * (1 + 5 ** 0.5) * k
    xb = R * np.stack([np.cos(az) * np.sin(polar), np.sin(az) * np.sin(polar), np.cos(polar)], 1)
    d = rng.normal(size=(nfil, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = R + 1.1 + 2.2 * np.arange(nseg)
    xs = (d[:, None, :] * r[None, :, None] + 0.3 * rng.normal(size=(nfil, nseg, 3))).reshape(-1, 3)
    return xs, xb


@pytest.mark.parametrize("cells", ["1", "0"], ids=["cell_list", "all_pairs"])
def test_barrier_swimmer_against_oracle(gpu_ctx, oracle_built, monkeypatch, cells):
    """The barrier at the config-3 shape (4096 blobs, 640 x 20 segments), by
    the cell list and by the all-pairs kernel, against the oracle (which adds
    each target's pairs in ascending source order, as the reference)."""
    rpy = oracle_built
    monkeypatch.setenv("GMI_BARRIER_CELLS", cells)
    xs, xb = _swimmer_cloud(4096, 640, 20, 40.0, seed=3)
    fs = np.random.default_rng(4).normal(size=(len(xs), 6))
    want_s, want_b = rpy.barrier(xs, xb, fs, 20, 1.0, 1.0, 2.5)
    assert np.count_nonzero(np.abs(want_s - fs).sum(1)) > 100 and np.count_nonzero(want_b.any(1)) > 100
    got = T(fs)
    fb = gpu_ctx.barrier(T(xs), T(xb), got, 20, 1.0, 1.0, 2.5)
    gpu_ctx.synchronize()
    assert rel_err(N(got), want_s) < 1e-14
    assert rel_err(N(fb), want_b) < 1e-14


def test_barrier_cell_overflow_against_oracle(gpu_ctx, oracle_built, monkeypatch):
    """A cluster of 64 blobs inside a unit ball: each of them has more
    candidates than the cell kernel keeps, so the overflow kernel finishes
    them; the rest take the cell list."""
    rpy = oracle_built
    monkeypatch.setenv("GMI_BARRIER_CELLS", "1")
    rng = np.random.default_rng(9)
    xs, xb = _swimmer_cloud(2048, 100, 20, 25.0, seed=8)
    ball = rng.normal(size=(64, 3))
    ball *= (rng.uniform(size=(64, 1)) ** (1 / 3)) / np.linalg.norm(ball, axis=1, keepdims=True)
    xb = np.concatenate([xb, ball + np.array([0.0, 0.0, 60.0])])
    fs = rng.normal(size=(len(xs), 6))
    want_s, want_b = rpy.barrier(xs, xb, fs, 20, 1.0, 1.0, 1.5)
    got = T(fs)
    fb = gpu_ctx.barrier(T(xs), T(xb), got, 20, 1.0, 1.0, 1.5)
    gpu_ctx.synchronize()
    assert rel_err(N(got), want_s) < 1e-14
    assert rel_err(N(fb), want_b) < 1e-14
    assert np.abs(want_b[-64:]).max() > 0


@pytest.mark.parametrize("case", WALL)
def test_wall_barrier_cell_list(case, gpu_ctx, monkeypatch):
    monkeypatch.setenv("GMI_BARRIER_CELLS", "1")
    g = load_golden(case)
    fs = T(g["fs"])
    gpu_ctx.barrier(T(g["xs"]), torch.zeros((0, 3), dtype=torch.float64, device="cuda"), fs, int(g["nseg"]),
                    1.0, 1.0, float(g["force_scale"]), wall=True)
    gpu_ctx.synchronize()
    assert rel_err(N(fs), g["fs_barrier"]) < 1e-14


@pytest.mark.parametrize("case", FREE)
def test_barrier_cell_list_matches_golden(case, gpu_ctx, monkeypatch):
    monkeypatch.setenv("GMI_BARRIER_CELLS", "1")
    g = load_golden(case)
    fs = T(g["fs"])
    fb = gpu_ctx.barrier(T(g["xs"]), T(g["xb"]), fs, int(g["nseg"]), float(g["rseg"]), float(g["rblob"]),
                         float(g["force_scale"]))
    gpu_ctx.synchronize()
    assert rel_err(N(fs), g["fs_barrier"]) < 1e-14
    assert rel_err(N(fb), g["fb_repulsion"]) < 1e-14


def test_larger_against_oracle(prec_ctx, oracle_built):
    """Thousands of particles (the warp-per-target kernel, at most 4096
    sources); random cube with rejection (config-2 shape)."""
    from generic_mobility_interface_class_gb300 import seeding
    ctx, tol = prec_ctx
    rpy = oracle_built
    n = 3001
    x = seeding.random_cube(n, seed=5)
    f = np.random.default_rng(5).normal(size=(n, 6))
    want = rpy.mss(x, f)
    got = N(ctx.mss(T(x), T(f)))
    assert rel_err(got, want) < tol
    wantb = rpy.mbb(x, f[:, :3])
    assert rel_err(N(ctx.mbb(T(x), T(f[:, :3]))), wantb) < tol


def test_tiled_kernel_against_oracle(prec_ctx, oracle_built):
    """More than 4096 sources (the TMA-tiled kernel): several tiles, several
    source splits, a ragged last tile; every pair kind, including the
    unequal-radius segment/blob couplings."""
    from generic_mobility_interface_class_gb300 import seeding
    ctx, tol = prec_ctx
    rpy = oracle_built
    n = 5003
    x = seeding.random_cube(n, seed=11)
    f = np.random.default_rng(11).normal(size=(n, 6))
    assert rel_err(N(ctx.mss(T(x), T(f))), rpy.mss(x, f)) < tol
    assert rel_err(N(ctx.mbb(T(x), T(f[:, :3]))), rpy.mbb(x, f[:, :3])) < tol
    # 700 segments against 5003 blobs (radii 1 and 1.4, all three branches
    # occur in a dense cloud) and 700 blobs against 5003 segments
    xs = x[:700] + 0.37
    v_in = np.random.default_rng(12).normal(size=(700, 6))
    v = T(v_in)
    ctx.msb(T(xs), T(x), T(f[:, :3]), v, a_seg=1.0, a_blob=1.4)
    want = rpy.msb(xs, x, f[:, :3], a_seg=1.0, a_blob=1.4, v_in=v_in)
    assert rel_err(N(v), want) < tol
    got = N(ctx.mbs(T(xs), T(x), T(f), a_seg=1.0, a_blob=1.4))
    assert rel_err(got, rpy.mbs(xs, x, f, a_seg=1.0, a_blob=1.4)) < tol


TILED_SHAPES = [(128, 1), (128, 2), (256, 1), (256, 2), (128, 4), (64, 1), (64, 2)]
PACKED_SHAPES = [(64, 1), (64, 2), (128, 1), (128, 2), (256, 1)]


@pytest.fixture
def own_ctx(gmi_lib):
    """A context of its own: pinned shapes and precision stay in this test."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from generic_mobility_interface_class_gb300.mobility import Context
    ctx = Context(0)
    yield ctx
    ctx.close()


@pytest.mark.parametrize("splits", [0, 3, 9])
@pytest.mark.parametrize("per_step,tpb,tt", [(1, *s) for s in TILED_SHAPES] + [(2, *s) for s in PACKED_SHAPES])
def test_every_tiled_shape_against_oracle(own_ctx, oracle_built, per_step, tpb, tt, splits):
    """Every entry of the tiled-kernel table, scalar (one source per thread
    step) and packed (two sources per f32x2 step), pinned with set_shape, on
    an odd source count (a ragged last tile whose last source has no
    partner) and with forced source splits (9: one tile per split, where the
    packed kernel runs in half its shared memory): all four free-space kinds
    against the FP64 oracle at the FP32C bound."""
    from generic_mobility_interface_class_gb300 import seeding
    rpy = oracle_built
    ctx = own_ctx
    ctx.set_precision(1)
    n, ns = 1031, 301
    x = seeding.random_cube(n, seed=23)
    f = np.random.default_rng(23).normal(size=(n, 6))
    xs = x[:ns] + 0.37
    for kind, nt, nsrc in [(0, n, n), (2, n, n), (3, ns, n), (4, ns, n)]:
        ctx.set_shape(kind, nt, nsrc, tpb, tt, splits, per_step)
        assert ctx.tuned_sources_per_step(kind, nt, nsrc) == per_step
    assert rel_err(N(ctx.mss(T(x), T(f))), rpy.mss(x, f)) < FP32C_TOL
    assert rel_err(N(ctx.mbb(T(x), T(f[:, :3]))), rpy.mbb(x, f[:, :3])) < FP32C_TOL
    v_in = np.random.default_rng(24).normal(size=(ns, 6))
    v = T(v_in)
    ctx.msb(T(xs), T(x), T(f[:, :3]), v, a_seg=1.0, a_blob=1.4)
    assert rel_err(N(v), rpy.msb(xs, x, f[:, :3], a_seg=1.0, a_blob=1.4, v_in=v_in)) < FP32C_TOL
    got = N(ctx.mbs(T(xs), T(x), T(f), a_seg=1.0, a_blob=1.4))
    assert rel_err(got, rpy.mbs(xs, x, f, a_seg=1.0, a_blob=1.4)) < FP32C_TOL


def test_set_shape_rejects_missing_kernels(own_ctx):
    """No packed kernel in FP64 or for the wall kind; no 64 x 4 entry."""
    from generic_mobility_interface_class_gb300._lib import GmiError
    ctx = own_ctx
    ctx.set_precision(0)
    with pytest.raises(GmiError):
        ctx.set_shape(0, 100, 100, 128, 2, 0, 2)
    ctx.set_precision(1)
    with pytest.raises(GmiError):
        ctx.set_shape(1, 100, 100, 128, 2, 0, 2)
    with pytest.raises(GmiError):
        ctx.set_shape(0, 100, 100, 64, 4, 0, 1)
    ctx.set_shape(0, 100, 100, 32, 2, 0, 1)
    assert ctx.tuned_shape(0, 100, 100)[:2] == (32, 2)


def test_target_slices_and_accumulate(gpu_ctx, oracle_built):
    rpy = oracle_built
    g = load_golden("swimmer_sphere")
    xs, fs = T(g["xs"]), T(g["fs"])
    part = N(gpu_ctx.mss(xs, fs, start=7, num=20))
    assert rel_err(part, g["v_ss"][7:27]) < FP64_TOL
    # Msb accumulates onto the caller's array for a target slice only
    v = T(g["v_in"][10:40])
    gpu_ctx.msb(xs, T(g["xb"]), T(g["fb"]), v, start=10, num=30)
    assert rel_err(N(v), g["v_sb"][10:40]) < FP64_TOL


def test_empty_sources_and_targets(gpu_ctx):
    z3 = torch.zeros((0, 3), dtype=torch.float64, device="cuda")
    xs = T(np.array([[0.0, 0.0, 0.0], [3.0, 0.0, 0.0]]))
    v = T(np.ones((2, 6)))
    gpu_ctx.msb(xs, z3, z3, v)  # no blobs: V unchanged
    gpu_ctx.synchronize()
    np.testing.assert_array_equal(N(v), np.ones((2, 6)))
    out = gpu_ctx.mbs(z3, xs, T(np.ones((2, 6))))  # no blob targets
    assert out.shape == (0, 3)
    vb = gpu_ctx.mbs(T(np.zeros((3, 3))), z3, torch.zeros((0, 6), dtype=torch.float64, device="cuda"))
    gpu_ctx.synchronize()
    np.testing.assert_array_equal(N(vb), np.zeros((3, 3)))


def test_autotune_keeps_results(gpu_ctx, oracle_built):
    rpy = oracle_built
    from generic_mobility_interface_class_gb300 import seeding
    n = 2048
    x = seeding.random_cube(n, seed=9)
    f = np.random.default_rng(9).normal(size=(n, 6))
    want = rpy.mss(x, f)
    for prec, tol in ((0, FP64_TOL), (1, FP32C_TOL)):
        gpu_ctx.set_precision(prec)
        gpu_ctx.autotune(0, n, n)
        assert rel_err(N(gpu_ctx.mss(T(x), T(f))), want) < tol
    gpu_ctx.set_precision(0)


def test_fp32c_is_translation_robust(gpu_ctx, oracle_built):
    """Double-float positions: shifting the whole cloud far from the origin
    keeps the FP32C error at its bound."""
    rpy = oracle_built
    g = load_golden("swimmer_sphere")
    xs = g["xs"] + np.array([1.0e4, -2.5e4, 3.3e3])
    want = rpy.mss(xs, g["fs"])
    gpu_ctx.set_precision(1)
    got = N(gpu_ctx.mss(T(xs), T(g["fs"])))
    gpu_ctx.set_precision(0)
    assert rel_err(got, want) < FP32C_TOL


@pytest.mark.parametrize("n", [901, 2048, 3001, 5003])
def test_double_float_blob_blob_against_oracle(own_ctx, oracle_built, n):
    """GMI_DF64: the blob-blob sum in double-float arithmetic against the
    FP64 oracle (near and far pairs, the self term; up to 2048 sources the
    warp-per-target kernel, above it several tiles and source splits), also
    with the cloud far from the origin, a target slice, and accumulation;
    the other pair sums refuse the precision."""
    from generic_mobility_interface_class_gb300 import GmiError, seeding
    rpy = oracle_built
    x = seeding.random_cube(n, seed=7)
    f = np.random.default_rng(7).normal(size=(n, 3))
    own_ctx.set_precision(2)
    for shift in (np.zeros(3), np.array([1.0e3, -2.5e3, 3.3e2])):
        xs = x + shift
        want = rpy.mbb(xs, f)
        assert rel_err(N(own_ctx.mbb(T(xs), T(f))), want) < DF64_TOL
    want = rpy.mbb(x, f)
    got = N(own_ctx.mbb(T(x), T(f), start=100, num=700))
    assert rel_err(got, want[100:800]) < DF64_TOL
    with pytest.raises(GmiError):
        own_ctx.mss(T(x), T(np.zeros((n, 6))))
    own_ctx.synchronize()
