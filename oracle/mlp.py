"""FP64 numpy restatement of the learned initial inverse Jacobian's network
and secant-pair loss (csrc/gmi_mlp.cu).  TEST INFRASTRUCTURE ONLY.

The library computes in bf16 with FP32 accumulation; this oracle computes
in FP64 and, with ``rounded=True``, rounds to bf16 (round to nearest even)
at exactly the points the library stores bf16 values: the input X, the
hidden activations H1, H2, the upstream gradient dO and the hidden
gradients dZ2, dZ1.  The remaining difference is FP32 against FP64
accumulation.  With ``rounded=False`` it is the exact FP64 network, whose
gradients the finite-difference tests check.

There is no counterpart in the reference: the reference has no learned
component.  Its Broyden start is conf * Jinv (broyden_solver.cpp:26-68);
the head below adds the network's correction to it.
"""
from __future__ import annotations

import numpy as np


def bf16(x) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float64).astype(np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    bias = 0x7FFF + ((u >> 16) & 1)
    r = ((u + bias) & 0xFFFF0000).astype(np.uint32)
    nan = np.isnan(f)
    out = r.view(np.float32).astype(np.float64)
    out[nan] = np.nan
    return out


def unpack(p, n_in, hidden, n_out, offsets):
    """[(W1, b1), (W2, b2), (W3, b3)] from the flat parameter array."""
    p = np.asarray(p, dtype=np.float64)
    shapes = [(hidden, n_in), (hidden, hidden), (n_out, hidden)]
    out = []
    for l, (r, c) in enumerate(shapes):
        w0, b0 = offsets[2 * l], offsets[2 * l + 1]
        out.append((p[w0:w0 + r * c].reshape(r, c), p[b0:b0 + r]))
    return out


def forward(layers, X, rounded=True):
    """Returns (O, cache); layers hold FP64 copies of the FP32 master weights."""
    rnd = bf16 if rounded else (lambda a: np.asarray(a, dtype=np.float64))
    (W1, b1), (W2, b2), (W3, b3) = layers
    W1r, W2r, W3r = rnd(W1), rnd(W2), rnd(W3)
    X0 = rnd(X)
    H1 = rnd(np.maximum(X0 @ W1r.T + b1, 0.0))
    H2 = rnd(np.maximum(H1 @ W2r.T + b2, 0.0))
    O = H2 @ W3r.T + b3
    return O, (X0, H1, H2, W1r, W2r, W3r)


def backward(cache, dO, rounded=True):
    """Gradients [(dW1, db1), (dW2, db2), (dW3, db3)] for upstream dO."""
    rnd = bf16 if rounded else (lambda a: np.asarray(a, dtype=np.float64))
    X0, H1, H2, W1r, W2r, W3r = cache
    d3 = rnd(dO)
    dW3, db3 = d3.T @ H2, d3.sum(axis=0)
    d2 = rnd((d3 @ W3r) * (H2 > 0))
    dW2, db2 = d2.T @ H1, d2.sum(axis=0)
    d1 = rnd((d2 @ W2r) * (H1 > 0))
    dW1, db1 = d1.T @ X0, d1.sum(axis=0)
    return [(dW1, db1), (dW2, db2), (dW3, db3)]


def pack(grads, nparam, offsets):
    g = np.zeros(nparam)
    for l, (dW, db) in enumerate(grads):
        g[offsets[2 * l]:offsets[2 * l] + dW.size] = dW.ravel()
        g[offsets[2 * l + 1]:offsets[2 * l + 1] + db.size] = db
    return g


def secant_head(O, records, nseg, rank, batch=None):
    """Per-record loss |sigma b + U V^T d - t|^2 / |t|^2 and dL/dO of the
    batch mean (batch = the divisor of the mean, default len(O)).
    records: [n x 24 nseg] (phi | d | b | t)."""
    O = np.asarray(O, dtype=np.float64)
    R = np.asarray(records, dtype=np.float64)
    n6, nblk = 6 * nseg, 2 * nseg
    B = O.shape[0] if batch is None else batch
    d, b, t = R[:, n6:2 * n6], R[:, 2 * n6:3 * n6], R[:, 3 * n6:4 * n6]
    s_raw = O[:, :nblk]
    s = np.clip(s_raw, -3.0, 3.0)
    sig = np.repeat(np.exp(s), 3, axis=1)
    U = O[:, nblk:nblk + n6 * rank].reshape(-1, n6, rank)
    V = O[:, nblk + n6 * rank:nblk + 2 * n6 * rank].reshape(-1, n6, rank)
    y = np.einsum("nir,ni->nr", V, d)
    pred = sig * b + np.einsum("nir,nr->ni", U, y)
    e = pred - t
    T = (t * t).sum(axis=1) + 1e-30
    loss = (e * e).sum(axis=1) / T
    gp = 2.0 * e / (T[:, None] * B)
    dO = np.zeros_like(O)
    inside = (s_raw > -3.0) & (s_raw < 3.0)
    dO[:, :nblk] = (gp * b).reshape(-1, nblk, 3).sum(axis=2) * np.exp(s) * inside
    dy = np.einsum("nir,ni->nr", U, gp)
    dO[:, nblk:nblk + n6 * rank] = np.einsum("ni,nr->nir", gp, y).reshape(-1, n6 * rank)
    dO[:, nblk + n6 * rank:nblk + 2 * n6 * rank] = np.einsum("ni,nr->nir", d, dy).reshape(-1, n6 * rank)
    return loss, dO
