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
