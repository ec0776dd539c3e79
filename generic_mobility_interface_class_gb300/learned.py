"""The learned initial inverse Jacobian (gmi_mlp_*, gmi_sim_set_learned_jacobian).

The reference starts each time step's Broyden solve from
JACOBIAN_CONFIDENCE_FACTOR times the approximate inverse Jacobian of
swimmer::jacobian_inv_mult (broyden_solver.cpp:26-68, swimmer.cpp:690-845),
which models each segment's hydrodynamics by its self-mobility alone.
``LearnedJacobian`` is a 3-layer MLP (width 256, bf16 weights, FP32
accumulation, trained and run by the library's own tensor-core kernels) that
maps a filament's shape in its local frame to a per-filament correction of
that start,

    H0 d = sigma (.) (conf Jinv d) + U (V^T d),

fitted to the secant pairs (the change of the Broyden error over an
iteration, the update that caused it) that plain Broyden runs produce.  The
time step uses it under a policy that falls back to the plain start whenever
the Broyden counts regress (``_lib.LearnedPolicy``, include/gmi.h).

    net = LearnedJacobian(nseg=20)
    records = collect_secant_pairs(workloads.config3(), steps=20, capacity=50_000)
    losses = net.train(records, steps=2000)
    sim.set_learned_jacobian(net)
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import GMI_FP32C, LearnedPolicy, check

HIDDEN = 256
RANK = 4


def head_outputs(nseg: int, rank: int) -> int:
    """Outputs of the secant head: 2 nseg log-scales, then U and V (6 nseg x rank each)."""
    return 2 * nseg + 12 * nseg * rank


def record_length(nseg: int) -> int:
    """Floats per secant-pair record: phi, d, b, t (6 nseg each)."""
    return 24 * nseg


def default_policy(**kw) -> LearnedPolicy:
    p = LearnedPolicy()
    _lib.load().gmi_learned_policy_init(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class LearnedJacobian:
    """gmi_mlp: n_in = 6 nseg -> hidden -> hidden -> head_outputs(nseg, rank)
    rounded up to a multiple of 8."""

    def __init__(self, nseg: int = 20, hidden: int = HIDDEN, rank: int = RANK, device: int = 0, seed: int = 2026):
        self.lib = _lib.load()
        self.nseg, self.hidden, self.rank, self.device = nseg, hidden, rank, device
        self.n_in = 6 * nseg
        self.n_out = (head_outputs(nseg, rank) + 7) // 8 * 8
        h = ctypes.c_void_p()
        check(self.lib.gmi_mlp_create(device, self.n_in, hidden, self.n_out, seed, ctypes.byref(h)))
        self.handle = h
        n = ctypes.c_longlong()
        check(self.lib.gmi_mlp_param_count(self.handle, ctypes.byref(n)))
        self.nparam = n.value
        off = (ctypes.c_longlong * 6)()
        check(self.lib.gmi_mlp_param_offsets(self.handle, off))
        self.offsets = list(off)

    # -- parameters ---------------------------------------------------------
    def params(self) -> np.ndarray:
        out = np.zeros(self.nparam, dtype=np.float32)
        check(self.lib.gmi_mlp_get_params(self.handle, out.ctypes.data_as(ctypes.c_void_p), self.nparam))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparam:
            raise ValueError(f"expected {self.nparam} parameters, got {p.size}")
        check(self.lib.gmi_mlp_set_params(self.handle, p.ctypes.data_as(ctypes.c_void_p), self.nparam))

    def layers(self, p=None):
        """[(W1, b1), (W2, b2), (W3, b3)] as numpy views of the flat array."""
        p = self.params() if p is None else p
        shapes = [(self.hidden, self.n_in), (self.hidden, self.hidden), (self.n_out, self.hidden)]
        out = []
        for l, (r, c) in enumerate(shapes):
            w0, b0 = self.offsets[2 * l], self.offsets[2 * l + 1]
            out.append((p[w0:w0 + r * c].reshape(r, c), p[b0:b0 + r]))
        return out

    def save(self, path) -> None:
        np.savez(path, params=self.params(), nseg=self.nseg, hidden=self.hidden, rank=self.rank)

    @classmethod
    def load(cls, path, device: int = 0) -> "LearnedJacobian":
        d = np.load(path)
        net = cls(nseg=int(d["nseg"]), hidden=int(d["hidden"]), rank=int(d["rank"]), device=device)
        net.set_params(d["params"])
        return net

    # -- device calls (torch float32 CUDA tensors) ---------------------------
    def forward(self, X):
        import torch
        out = torch.empty((X.shape[0], self.n_out), dtype=torch.float32, device=X.device)
        check(self.lib.gmi_mlp_forward(self.handle, ctypes.c_void_p(X.data_ptr()), X.shape[0],
                                       ctypes.c_void_p(out.data_ptr())))
        return out

    def backward(self, dO) -> np.ndarray:
        """Flat FP32 gradients of the last forward's batch for upstream dO."""
        g = np.zeros(self.nparam, dtype=np.float32)
        check(self.lib.gmi_mlp_backward(self.handle, ctypes.c_void_p(dO.data_ptr()), dO.shape[0],
                                        g.ctypes.data_as(ctypes.c_void_p)))
        return g

    def loss(self, records, with_grad: bool = False):
        """Mean secant-pair loss over records; with_grad also returns the
        gradient with respect to the output rows (per chunk of 4096)."""
        import torch
        n = records.shape[0]
        scratch = torch.empty((min(n, 4096), self.n_out), dtype=torch.float32, device=records.device)
        dO = torch.empty((n, self.n_out), dtype=torch.float32, device=records.device) if with_grad else None
        v = ctypes.c_double()
        check(self.lib.gmi_mlp_secant_loss(self.handle, ctypes.c_void_p(records.data_ptr()), n, self.nseg, self.rank,
                                           ctypes.c_void_p(scratch.data_ptr()), ctypes.byref(v),
                                           ctypes.c_void_p(dO.data_ptr()) if with_grad else None))
        return (v.value, dO) if with_grad else v.value

    def train(self, records, steps: int = 2000, batch: int = 512, lr: float = 1e-3, seed: int = 7) -> np.ndarray:
        """Adam on the secant-pair loss; returns the per-step minibatch loss."""
        losses = np.zeros(steps, dtype=np.float32)
        check(self.lib.gmi_mlp_train_secant(self.handle, ctypes.c_void_p(records.data_ptr()), records.shape[0],
                                            self.nseg, self.rank, steps, batch, ctypes.c_float(lr), seed,
                                            losses.ctypes.data_as(ctypes.c_void_p)))
        return losses

    @property
    def launches(self) -> int:
        return int(self.lib.gmi_mlp_launch_count(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gmi_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def collect_secant_pairs(sim_kwargs: dict, steps: int, capacity: int, precision: int = GMI_FP32C, device: int = 0,
                         first_step: int = 0, probes: int = 0, secant_pairs: bool = True, seed: int = 0):
    """Run the plain method for ``steps`` time steps and return the secant-pair
    records it produced (a float32 CUDA tensor, at most ``capacity`` rows):
    the Broyden iterations' own pairs (``secant_pairs``) and ``probes``
    random-direction Jacobian probes per iterating step."""
    import torch

    from .sim import Simulation
    nseg = int(sim_kwargs["nseg"])
    rec = torch.zeros((capacity, record_length(nseg)), dtype=torch.float32, device=f"cuda:{device}")
    sim = Simulation(**sim_kwargs, precision=precision, device=device)
    try:
        sim.prepare()
        sim.set_secant_buffer(rec)
        if probes or not secant_pairs:
            sim.set_jacobian_probes(probes, seed, secant_pairs)
        for nt in range(first_step, first_step + steps):
            sim.step(nt)
            if sim.secant_count() >= capacity:
                break
        torch.cuda.synchronize()
        n = sim.secant_count()
        sim.set_secant_buffer(None)
    finally:
        sim.close()
    return rec[:n].clone()
