"""Dense FP64 restatement of the reference's mobility solve.  TEST
INFRASTRUCTURE ONLY.

compute_velocities() follows mobility_solver::compute_velocities
(mobility_solver.cpp:1358-1402) step by step, but solves the saddle-point
system [M_bb, -K; -K^T, 0] [f; V] = [-M_bs F_s; -F_body]
(assemble_rhs :361-419, system_matrix_mult :905-962) with a dense LU
instead of GMRES, so it checks the GMRES answer independently of the
Krylov method and the preconditioner.  M_bb is assembled column by column
from the pinned pair-sum oracle (oracle/rpy.py).
"""
from __future__ import annotations

import numpy as np

from . import rpy


def rot_mat(q):
    """quaternion::rot_mat (quaternion.cpp:260-298), q = (s, v0, v1, v2)."""
    s, a, b, c = q
    return np.array([[1 - 2 * (b * b + c * c), 2 * (a * b - s * c), 2 * (a * c + s * b)],
                     [2 * (a * b + s * c), 1 - 2 * (a * a + c * c), 2 * (b * c - s * a)],
                     [2 * (a * c - s * b), 2 * (b * c + s * a), 1 - 2 * (a * a + b * b)]])


def blob_positions(body_x, body_q, refs):
    """rigid_body::blob_positions (rigid_body.cpp:334-352) for every swimmer."""
    out = []
    for x, q in zip(body_x, body_q):
        out.append(x[None, :] + refs @ rot_mat(q).T)
    return np.concatenate(out, axis=0) if out else np.zeros((0, 3))


def k_matrix(body_q, refs):
    """K: body velocity (U, Omega) of every swimmer -> blob velocities
    U + Omega x (R ref)  (mobility_solver.cpp:944-950)."""
    W, nblob = len(body_q), len(refs)
    K = np.zeros((3 * W * nblob, 6 * W))
    for n, q in enumerate(body_q):
        d = refs @ rot_mat(q).T
        for m in range(nblob):
            r = 3 * (n * nblob + m)
            K[r:r + 3, 6 * n:6 * n + 3] = np.eye(3)
            dx, dy, dz = d[m]
            K[r:r + 3, 6 * n + 3:6 * n + 6] = np.array([[0, dz, -dy], [-dz, 0, dx], [dy, -dx, 0]])
    return K


def mbb_matrix(xb, a, mu):
    B = xb.shape[0]
    M = np.zeros((3 * B, 3 * B))
    for k in range(3 * B):
        e = np.zeros((B, 3))
        e.flat[k] = 1.0
        M[:, k] = rpy.mbb(xb, e, a, mu).ravel()
    return M


def saddle_matrix(xb, body_q, refs, a_blob, mu):
    """[M_bb, -K; -K^T, 0] (system_matrix_mult, mobility_solver.cpp:905-962)."""
    Mbb = mbb_matrix(xb, a_blob, mu)
    K = k_matrix(body_q, refs)
    nb, nw = Mbb.shape[0], K.shape[1]
    A = np.zeros((nb + nw, nb + nw))
    A[:nb, :nb] = Mbb
    A[:nb, nb:] = -K
    A[nb:, :nb] = -K.T
    return A


def saddle_solve(xb, body_q, refs, rhs, a_blob, mu, A=None):
    A = saddle_matrix(xb, body_q, refs, a_blob, mu) if A is None else A
    nb = A.shape[0] - 6 * len(np.asarray(body_q).reshape(-1, 4))
    sol = np.linalg.solve(A, rhs)
    return sol[:nb].reshape(-1, 3), sol[nb:].reshape(-1, 6)


def compute_velocities(xs, fs, body_x, body_q, body_f, refs, nseg, rseg=1.0, rblob=1.0, mu=1.0, force_scale=1.0):
    body_x = np.asarray(body_x, dtype=np.float64).reshape(-1, 3)
    body_q = np.asarray(body_q, dtype=np.float64).reshape(-1, 4)
    refs = np.asarray(refs, dtype=np.float64).reshape(-1, 3)
    xb = blob_positions(body_x, body_q, refs)
    fs2, frep = rpy.barrier(xs, xb, fs, nseg, rseg, rblob, force_scale)
    bf = np.array(body_f, dtype=np.float64).reshape(-1, 6).copy()
    nblob = refs.shape[0]
    for n, q in enumerate(body_q):
        fr = frep[n * nblob:(n + 1) * nblob]
        d = refs @ rot_mat(q).T
        bf[n, :3] += fr.sum(axis=0)
        bf[n, 3:] += np.cross(d, fr).sum(axis=0)
    v_segs = rpy.mss(xs, fs2, rseg, mu)
    v_blobs = rpy.mbs(xb, xs, fs2, rseg, rblob, mu)
    rhs = np.concatenate([-v_blobs.ravel(), -bf.ravel()])
    A = saddle_matrix(xb, body_q, refs, rblob, mu)
    f_blobs, v_bodies = saddle_solve(xb, body_q, refs, rhs, rblob, mu, A=A)
    v_segs = rpy.msb(xs, xb, f_blobs, rseg, rblob, mu, v_in=v_segs)
    return dict(v_segs=v_segs, f_blobs=f_blobs, v_bodies=v_bodies, body_f=bf, f_rep=frep, x_blobs=xb,
                v_blobs_bs=v_blobs, A=A, rhs=rhs)


def ktk_inverse(refs):
    """(K^T K)^-1 of one body (mobility_solver.cpp:1697-1716)."""
    K = k_matrix(np.array([[1.0, 0, 0, 0]]), np.asarray(refs).reshape(-1, 3))
    return np.linalg.inv(K.T @ K)


def body_mobility_reference(xb_last, refs, body_q_last, a_blob, mu):
    """6x6 body mobility of a lone body: V = N F with F the force/torque on
    it (mobility_solver.cpp:1733-1741 solve rhs = -e_k in the body rows)."""
    refs = np.asarray(refs).reshape(-1, 3)
    nb = 3 * refs.shape[0]
    N = np.zeros((6, 6))
    for col in range(6):
        rhs = np.zeros(nb + 6)
        rhs[nb + 5 - col] = -1.0
        _, vb = saddle_solve(xb_last, np.asarray(body_q_last).reshape(1, 4), refs, rhs, a_blob, mu)
        N[:, 5 - col] = vb[0]
    return N


def generalised_force(table, phase):
    """The generalised force of the prescribed beat at each phase: the
    reference's cubic Hermite interpolation of its table over one period,
    with its one-sided difference at sample 0 (mobility_solver.cpp:219-280)."""
    t = np.asarray(table, dtype=np.float64)
    n = len(t)
    out = []
    for phi in np.atleast_1d(np.asarray(phase, dtype=np.float64)):
        x = 0.5 * phi / np.pi
        x -= np.floor(x)
        x *= n
        lo = int(x)
        if lo == n:
            out.append(t[0])
            continue
        hi = 0 if lo == n - 1 else lo + 1
        dlo = t[1] - t[0] if lo == 0 else 0.5 * (t[hi] - t[lo - 1])
        dhi = t[0] - t[n - 1] if hi == 0 else 0.5 * (t[0 if hi == n - 1 else hi + 1] - t[lo])
        s = x - lo
        out.append(t[lo] * (2 * s ** 3 - 3 * s ** 2 + 1) + dlo * (s ** 3 - 2 * s ** 2 + s) +
                   t[hi] * (3 * s ** 2 - 2 * s ** 3) + dhi * (s ** 3 - s ** 2))
    return np.array(out)


def prescribed_system(x, xs, body_x, body_q, refs, vel_dir, nfil, nseg, rseg=1.0, rblob=1.0, mu=1.0,
                      phase_speed=None, table=None, phase=None, omega0=None):
    """(A x, b) of the prescribed-shape cilia system (CILIA_TYPE 3):
    system_matrix_mult (mobility_solver.cpp:733-905) and assemble_rhs
    (:211-310) for free bodies.  x = [f_seg (S,3) | f_blob (B,3) | (U, Omega)
    (W,6) | phase speeds (F,) when table is given].  With phase_speed given
    (the speeds prescribed) the segment rows of b are phase_speed * vel_dir;
    with table, phase and omega0 given (DYNAMIC_PHASE_EVOLUTION) the phase
    speeds are unknowns: their rows of A x are -sum_k K_k . f_k, the segment
    rows take -phase_speed K, and b's phase rows are -q omega0 / (2 pi)."""
    body_x = np.asarray(body_x, dtype=np.float64).reshape(-1, 3)
    body_q = np.asarray(body_q, dtype=np.float64).reshape(-1, 4)
    refs = np.asarray(refs, dtype=np.float64).reshape(-1, 3)
    xs = np.asarray(xs, dtype=np.float64).reshape(-1, 3)
    K = np.asarray(vel_dir, dtype=np.float64).reshape(-1, 3)
    W, S, nblob = len(body_x), len(xs), len(refs)
    dynamic = table is not None
    F = W * nfil if dynamic else 0
    B = W * nblob
    x = np.asarray(x, dtype=np.float64)
    fs = x[:3 * S].reshape(S, 3)
    fb = x[3 * S:3 * (S + B)].reshape(B, 3)
    U = x[3 * (S + B):3 * (S + B) + 6 * W].reshape(W, 6)
    ps = x[3 * (S + B) + 6 * W:]
    xb = blob_positions(body_x, body_q, refs)
    fs6 = np.concatenate([fs, np.zeros_like(fs)], axis=1)
    v_segs = rpy.msb(xs, xb, fb, rseg, rblob, mu, v_in=rpy.mss(xs, fs6, rseg, mu))[:, :3]
    v_blobs = rpy.mbs(xb, xs, fs6, rseg, rblob, mu) + rpy.mbb(xb, fb, rblob, mu)
    sw_seg = np.arange(S) // (nfil * nseg)
    sw_blob = np.arange(B) // nblob
    d_seg = xs - body_x[sw_seg]
    d_blob = xb - body_x[sw_blob]
    rows_seg = v_segs - U[sw_seg, :3] - np.cross(U[sw_seg, 3:], d_seg)
    rows_blob = v_blobs - U[sw_blob, :3] - np.cross(U[sw_blob, 3:], d_blob)
    body = np.zeros((W, 6))
    for n in range(W):
        body[n, :3] = -fs[sw_seg == n].sum(0) - fb[sw_blob == n].sum(0)
        body[n, 3:] = -np.cross(d_seg[sw_seg == n], fs[sw_seg == n]).sum(0) - \
            np.cross(d_blob[sw_blob == n], fb[sw_blob == n]).sum(0)
    b = np.zeros(3 * (S + B) + 6 * W + F)
    fil = np.arange(S) // nseg
    if dynamic:
        rows_seg = rows_seg - ps[fil][:, None] * K
        phase_rows = -np.einsum("fkc,fkc->f", K.reshape(F, nseg, 3), fs.reshape(F, nseg, 3))
        b[3 * (S + B) + 6 * W:] = -generalised_force(table, phase) * (0.5 * np.asarray(omega0) / np.pi)
    else:
        phase_rows = np.zeros(0)
        b[:3 * S] = (np.asarray(phase_speed, dtype=np.float64)[fil][:, None] * K).ravel()
    Ax = np.concatenate([rows_seg.ravel(), rows_blob.ravel(), body.ravel(), phase_rows])
    return Ax, b
