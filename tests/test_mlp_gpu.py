"""The learned initial inverse Jacobian on the GPU.

* The network's tensor-core forward and backward (bf16 operands, FP32
  accumulation) against the FP64 oracle with the same bf16 rounding points
  (oracle/mlp.py): the only difference left is FP32 against FP64
  accumulation, so the outputs and gradients agree to ~1e-3 of their scale.
* The secant-pair loss and its gradient against the oracle's.
* Training on the GPU reduces the loss of records with a known answer.
* In the time step: a network whose output is the plain start (sigma = 1,
  U V^T = 0) reproduces the plain trajectory bit for bit; a bad network is
  caught by the policy, every learned attempt restarted plain, and the
  trajectory again equals the plain one; secant pairs are collected.
"""
import numpy as np
import pytest

from oracle import mlp as om

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FWD_TOL = 2e-3   # max |O - O_oracle| / max |O_oracle|
GRAD_TOL = 5e-3  # the same per parameter block


@pytest.fixture
def net(gmi_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from generic_mobility_interface_class_gb300.learned import LearnedJacobian
    n = LearnedJacobian(nseg=20, seed=11)
    yield n
    n.close()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def layers64(net):
    return [(W.astype(np.float64), b.astype(np.float64)) for W, b in net.layers()]


def test_forward_and_backward_match_oracle(net):
    rng = np.random.default_rng(5)
    # a network with an output layer of ordinary size, so that every output matters
    p = net.params()
    W3, _ = net.layers(p)[2]
    W3 *= 20.0
    net.set_params(p)
    X = rng.normal(size=(300, net.n_in)).astype(np.float32)
    O = net.forward(torch.as_tensor(X, device="cuda")).cpu().numpy()
    O64, cache = om.forward(layers64(net), X)
    assert rel(O, O64) < FWD_TOL
    dO = (rng.normal(size=O.shape) / 300.0).astype(np.float32)
    g = net.backward(torch.as_tensor(dO, device="cuda"))
    go = om.pack(om.backward(cache, dO), net.nparam, net.offsets)
    for l in range(6):
        a, b = net.offsets[l], (net.offsets[l + 1] if l < 5 else net.nparam)
        assert rel(g[a:b], go[a:b]) < GRAD_TOL, (l, rel(g[a:b], go[a:b]))


def test_secant_loss_matches_oracle(net):
    rng = np.random.default_rng(6)
    n6 = 6 * net.nseg
    rec = rng.normal(size=(700, 4 * n6)).astype(np.float32)
    recd = torch.as_tensor(rec, device="cuda")
    loss, dO = net.loss(recd, with_grad=True)
    O = net.forward(torch.as_tensor(np.ascontiguousarray(rec[:, :n6]), device="cuda")).cpu().numpy()
    lo, do = om.secant_head(O.astype(np.float64), rec, net.nseg, net.rank)
    assert abs(loss - lo.mean()) <= 1e-5 * lo.mean()
    assert rel(dO.cpu().numpy(), do) < 1e-4


def test_training_fits_a_known_operator(net):
    """Records whose update is 3 b (sigma = 3 everywhere): training drives
    the loss down by more than a factor of ten, and the fitted scales
    approach 3."""
    rng = np.random.default_rng(8)
    n6 = 6 * net.nseg
    n = 4000
    rec = np.zeros((n, 4 * n6), dtype=np.float32)
    rec[:, :n6] = rng.normal(size=(n, n6))
    rec[:, n6:2 * n6] = rng.normal(size=(n, n6))
    rec[:, 2 * n6:3 * n6] = rng.normal(size=(n, n6))
    rec[:, 3 * n6:] = 3.0 * rec[:, 2 * n6:3 * n6]
    recd = torch.as_tensor(rec, device="cuda")
    before = net.loss(recd)
    losses = net.train(recd, steps=600, batch=256, lr=2e-3)
    after = net.loss(recd)
    assert np.all(np.isfinite(losses))
    assert after < before / 10, (before, after)
    O = net.forward(torch.as_tensor(np.ascontiguousarray(rec[:64, :n6]), device="cuda")).cpu().numpy()
    sig = np.exp(np.clip(O[:, :2 * net.nseg], -3, 3))
    assert abs(np.median(sig) - 3.0) < 0.3


# ---- in the time step ---------------------------------------------------------
def small_swimmer(**kw):
    from generic_mobility_interface_class_gb300 import seeding, workloads
    verts = seeding.icosphere(2)
    rng = np.random.default_rng(3)
    fils = seeding.icosphere(1)[rng.choice(42, 6, replace=False)]
    args = workloads.free_swimmer(verts, fils, radius=8.0, nseg=20, seed=3)
    args.update(kw)
    return args


def run(kw, steps, net=None, policy=None, precision=1, records=None):
    from generic_mobility_interface_class_gb300.sim import Simulation
    sim = Simulation(**kw, precision=precision)
    sim.prepare()
    if net is not None:
        sim.set_learned_jacobian(net, policy)
    if records is not None:
        sim.set_secant_buffer(records)
    counts = [sim.step(nt) for nt in range(steps)]
    out = {f: sim.state(f) for f in ("seg_q", "seg_x", "body_x", "body_q", "body_v", "seg_v")}
    pol = sim.learned_policy()
    nrec = sim.secant_count()
    sim.close()
    return counts, out, pol, nrec


def zero_net(net, log_scale=0.0):
    """Every weight zero; the log-scale biases set to log_scale: sigma =
    exp(log_scale), U = V = 0."""
    p = np.zeros(net.nparam, dtype=np.float32)
    b3 = net.offsets[5]
    p[b3:b3 + 2 * net.nseg] = log_scale
    net.set_params(p)


def test_plain_start_network_reproduces_the_plain_trajectory(net):
    from generic_mobility_interface_class_gb300.learned import default_policy
    kw = small_swimmer()
    plain, s0, _, _ = run(kw, 6)
    zero_net(net)
    learned, s1, pol, _ = run(kw, 6, net, default_policy(calibration_steps=0))
    assert pol.mode == 1 and pol.steps_learned == 6 and pol.regressions == 0
    assert learned == plain
    for f in s0:
        np.testing.assert_array_equal(s1[f], s0[f])


def test_bad_network_falls_back_to_the_plain_trajectory(net):
    """sigma = exp(-3): every learned step is twenty times too timid and
    misses its cap of 3 iterations (cap_factor 0.01), so it is restarted
    plain from its initial guess; after two such regressions the policy
    stops trying.  The state after every step is the
    plain method's, bit for bit."""
    from generic_mobility_interface_class_gb300.learned import default_policy
    kw = small_swimmer()
    plain, s0, _, _ = run(kw, 7)
    zero_net(net, log_scale=-3.0)
    pol_in = default_policy(calibration_steps=2, cap_factor=0.01)
    learned, s1, pol, _ = run(kw, 7, net, pol_in)
    assert pol.mode == 2 and pol.regressions == 2 and pol.steps_learned == 2
    # the restarted steps did more Broyden iterations (attempt + plain), the others the same
    assert [c[0] for c in learned[:2]] == [c[0] for c in plain[:2]]
    assert sum(c[0] for c in learned) > sum(c[0] for c in plain)
    for f in s0:
        np.testing.assert_array_equal(s1[f], s0[f])


def test_nonfinite_network_falls_back_to_the_plain_trajectory(net):
    """A network whose U outputs are NaN makes the first learned update
    non-finite, so the state goes non-finite and the step's next linear solve
    meets a non-finite right-hand side.  That is a divergence of the learned
    attempt: the step is restarted plain from its initial guess, and after
    two such regressions the policy stops trying.  The trajectory is the
    plain method's, bit for bit."""
    from generic_mobility_interface_class_gb300.learned import default_policy
    kw = small_swimmer()
    plain, s0, _, _ = run(kw, 5)
    zero_net(net)
    p = net.params()
    b3 = net.offsets[5]
    p[b3 + 2 * net.nseg:b3 + 2 * net.nseg + 6 * net.nseg * net.rank] = np.nan  # U
    net.set_params(p)
    learned, s1, pol, _ = run(kw, 5, net, default_policy(calibration_steps=0))
    assert pol.mode == 2 and pol.regressions == 2 and pol.steps_learned == 2
    assert [c[1] > 0 for c in learned] == [True] * 5
    for f in s0:
        np.testing.assert_array_equal(s1[f], s0[f])


def test_jacobian_probes_leave_the_trajectory_unchanged(gmi_lib):
    """Probe records (gmi_sim_set_jacobian_probes): each iterating step
    appends probes x filaments records of finite, non-zero d, b and t, and
    the state is restored after every probe, so the trajectory is the one
    without probes, bit for bit."""
    from generic_mobility_interface_class_gb300.learned import record_length
    from generic_mobility_interface_class_gb300.sim import Simulation
    kw = small_swimmer()
    plain, s0, _, _ = run(kw, 3)
    rec = torch.zeros((2000, record_length(20)), dtype=torch.float32, device="cuda")
    sim = Simulation(**kw, precision=1)
    sim.prepare()
    sim.set_secant_buffer(rec)
    sim.set_jacobian_probes(3, seed=5, secant_pairs=False)
    counts = [sim.step(nt) for nt in range(3)]
    s1 = {f: sim.state(f) for f in s0}
    nrec = sim.secant_count()
    sim.close()
    assert [c[0] for c in counts] == [c[0] for c in plain]
    for f in s0:
        np.testing.assert_array_equal(s1[f], s0[f])
    iterating = sum(1 for c in plain if c[0] > 0)
    assert nrec == 3 * 6 * iterating
    r = rec[:nrec].cpu().numpy()
    assert np.all(np.isfinite(r))
    n6 = 120
    for k in (1, 2, 3):
        assert np.all(np.linalg.norm(r[:, k * n6:(k + 1) * n6], axis=1) > 0)
    # the probes of one step differ from one another
    assert not np.array_equal(r[0, 3 * n6:], r[6, 3 * n6:])


def test_secant_pairs_are_collected(gmi_lib):
    from generic_mobility_interface_class_gb300.learned import record_length
    kw = small_swimmer()
    rec = torch.zeros((5000, record_length(20)), dtype=torch.float32, device="cuda")
    counts, _, _, nrec = run(kw, 3, records=rec)
    iters = sum(c[0] for c in counts)
    assert nrec == 6 * iters  # one record per filament and Broyden iteration
    r = rec[:nrec].cpu().numpy()
    assert np.all(np.isfinite(r))
    n6 = 120
    # features: the base segment sits at the origin of its local frame, the
    # first tangent is close to the local e3 of a filament that starts radially
    assert np.all(r[:, 0:3] == 0.0)
    assert np.all(np.linalg.norm(r[:, 3:6], axis=1) > 0.99)
    # d (the change of the error), b and t are not all zero
    for k in (1, 2, 3):
        assert np.all(np.linalg.norm(r[:, k * n6:(k + 1) * n6], axis=1) > 0)
