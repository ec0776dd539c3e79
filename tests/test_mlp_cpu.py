"""The learned initial inverse Jacobian without a GPU: the FP64 oracle of the
network and of the secant-pair loss against finite differences, its bf16
rounding against torch's, and the fall-back policy of the library (plain host
code, called through the C ABI)."""
import ctypes

import numpy as np
import pytest

from oracle import mlp as om


def small_net(seed=0, n_in=16, hidden=8, n_out=24):
    rng = np.random.default_rng(seed)
    sizes = [hidden * n_in, hidden, hidden * hidden, hidden, n_out * hidden, n_out]
    offsets, o = [], 0
    for s in sizes:
        offsets.append(o)
        o += (s + 7) // 8 * 8
    p = rng.normal(size=o) * 0.5
    return p, offsets, (n_in, hidden, n_out)


def test_backward_matches_finite_differences():
    p, off, (ni, nh, no) = small_net()
    rng = np.random.default_rng(1)
    X = rng.normal(size=(5, ni))
    G = rng.normal(size=(5, no))  # loss = sum(G * O)

    def loss(q):
        O, _ = om.forward(om.unpack(q, ni, nh, no, off), X, rounded=False)
        return float((G * O).sum())

    O, cache = om.forward(om.unpack(p, ni, nh, no, off), X, rounded=False)
    g = om.pack(om.backward(cache, G, rounded=False), p.size, off)
    idx = rng.choice(p.size, 40, replace=False)
    h = 1e-6
    for i in idx:
        q1, q2 = p.copy(), p.copy()
        q1[i] += h
        q2[i] -= h
        fd = (loss(q1) - loss(q2)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_secant_head_matches_finite_differences():
    nseg, rank = 2, 2
    n6 = 6 * nseg
    rng = np.random.default_rng(3)
    n_out = 2 * nseg + 2 * n6 * rank
    O = rng.normal(size=(3, n_out)) * 0.5
    O[0, 0] = 3.5  # one clamped log-scale: zero gradient there
    rec = rng.normal(size=(3, 4 * n6))
    loss, dO = om.secant_head(O, rec, nseg, rank)
    assert dO[0, 0] == 0.0

    def mean_loss(o):
        return float(om.secant_head(o, rec, nseg, rank)[0].mean())

    h = 1e-6
    for r in range(3):
        for c in range(n_out):
            if r == 0 and c == 0:
                continue
            o1, o2 = O.copy(), O.copy()
            o1[r, c] += h
            o2[r, c] -= h
            fd = (mean_loss(o1) - mean_loss(o2)) / (2 * h)
            assert abs(fd - dO[r, c]) <= 1e-6 * max(1.0, abs(fd)), (r, c, fd, dO[r, c])


def test_secant_head_is_exact_for_the_plain_start():
    """sigma = 1 and U V^T = 0 give H0 d = b: a record whose update is b has
    zero loss."""
    nseg, rank = 3, 4
    n6 = 6 * nseg
    rng = np.random.default_rng(5)
    rec = rng.normal(size=(4, 4 * n6))
    rec[:, 3 * n6:] = rec[:, 2 * n6:3 * n6]
    O = np.zeros((4, 2 * nseg + 2 * n6 * rank))
    loss, _ = om.secant_head(O, rec, nseg, rank)
    assert np.all(loss == 0.0)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.normal(size=4000) * 10.0 ** rng.integers(-30, 30, size=4000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.01171875, 3.0e38, 1e-40]])
    want = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(om.bf16(x), want)


# ---- the fall-back policy ------------------------------------------------------
@pytest.fixture(scope="module")
def lib():
    from generic_mobility_interface_class_gb300 import _lib, build
    build.build()
    return _lib.load()


def policy(lib, **kw):
    from generic_mobility_interface_class_gb300._lib import LearnedPolicy
    p = LearnedPolicy()
    lib.gmi_learned_policy_init(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_policy_defaults_and_calibration(lib):
    p = policy(lib)
    assert (p.calibration_steps, p.window, p.max_regressions, p.margin, p.cap_factor) == (3, 8, 2, 0.05, 2.0)
    pr = ctypes.byref(p)
    assert lib.gmi_learned_policy_iteration_cap(pr, 100) == 100  # no plain steps yet: the library's cap
    for it in (6, 5, 7):
        assert lib.gmi_learned_policy_use_learned(pr) == 0
        lib.gmi_learned_policy_record(pr, 0, 1, it)
    assert p.mode == 1 and lib.gmi_learned_policy_use_learned(pr) == 1
    assert lib.gmi_learned_policy_iteration_cap(pr, 100) == 2 * 6 + 2  # ceil(2 x mean 6) + 2
    assert lib.gmi_learned_policy_iteration_cap(pr, 9) == 9


def test_policy_falls_back_after_regressions(lib):
    """A learned step that misses its cap is a regression; the second one
    ends the learned mode for good."""
    p = policy(lib, calibration_steps=1)
    pr = ctypes.byref(p)
    lib.gmi_learned_policy_record(pr, 0, 1, 6)
    lib.gmi_learned_policy_record(pr, 1, 0, 14)  # missed the cap: restarted plain
    lib.gmi_learned_policy_record(pr, 0, 1, 6)
    assert p.mode == 1 and p.regressions == 1
    lib.gmi_learned_policy_record(pr, 1, 1, 4)
    lib.gmi_learned_policy_record(pr, 1, 0, 14)
    assert p.mode == 2 and p.regressions == 2
    assert lib.gmi_learned_policy_use_learned(pr) == 0
    lib.gmi_learned_policy_record(pr, 0, 1, 6)
    assert p.mode == 2  # no way back


def test_policy_falls_back_when_counts_regress(lib):
    """Converged learned steps whose mean Broyden count over the window
    exceeds (1 + margin) x the plain mean end the learned mode."""
    p = policy(lib, calibration_steps=2, window=4, margin=0.1)
    pr = ctypes.byref(p)
    lib.gmi_learned_policy_record(pr, 0, 1, 10)
    lib.gmi_learned_policy_record(pr, 0, 1, 10)
    for it in (8, 9, 10):
        lib.gmi_learned_policy_record(pr, 1, 1, it)
        assert p.mode == 1
    lib.gmi_learned_policy_record(pr, 1, 1, 11)  # window mean 9.5 <= 11: keeps going
    assert p.mode == 1
    for it in (12, 12, 12):
        lib.gmi_learned_policy_record(pr, 1, 1, it)
    assert p.mode == 2  # window mean 12 > 11


def test_policy_without_calibration_starts_learned(lib):
    p = policy(lib, calibration_steps=0)
    pr = ctypes.byref(p)
    assert lib.gmi_learned_policy_use_learned(pr) == 1
    assert lib.gmi_learned_policy_iteration_cap(pr, 50) == 50
    lib.gmi_learned_policy_record(pr, 1, 1, 7)
    assert p.mode == 1 and p.steps_learned == 1
