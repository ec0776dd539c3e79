"""The barrier's cell list finds every pair its FP32 screen accepts.

barrier_cell_kernel (csrc/gmi_pair_kernels.cu) searches only the 27 cells
around a target.  That is complete if every pair the FP32 screen accepts
lies in adjacent cells: the cell width is the widest screen cutoff plus the
screen's rounding margin, times 1.01, and cell coordinates are
floor(x / h) in FP32.  This test restates that arithmetic (FP32 offsets
from the first particle, the extent, the margin, the fused squared
distance) in numpy and checks the claim on clouds built to stress it:
pairs placed just inside the cutoff, far from the origin, at every
orientation.
"""
import numpy as np

F = np.float32


def fmaf(a, b, c):
    """FP32 fused multiply-add: the product of two FP32 values is exact in
    FP64, so one rounding of the FP64 sum to FP32 reproduces it (up to a
    double rounding that no test point here comes near)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F)


def screen_and_cells(x, cut):
    """FP32 screen positions (offsets from the first particle), the squared
    screen cutoff with the margin, and every particle's cell."""
    p0 = x[0]
    s = (x - p0).astype(F)
    extent = F(np.abs(s).max())
    margin = F(1.0e-6) * extent
    c = F(cut) + margin
    inv_h = F(1.0) / ((F(cut) + margin) * F(1.01))
    cells = np.floor(s * inv_h).astype(np.int64)
    return s, c * c, cells


def accepted_pairs(s, c2):
    """Pairs (i, j) the screen accepts: fma(dx, dx, fma(dy, dy, dz dz)) < c2."""
    out = []
    for i in range(len(s)):
        d = s[i][None, :] - s  # FP32 differences
        d2 = fmaf(d[:, 0], d[:, 0], fmaf(d[:, 1], d[:, 1], d[:, 2] * d[:, 2]))
        for j in np.nonzero(d2 < c2)[0]:
            if j != i:
                out.append((i, j))
    return out


def check_cloud(x, cut):
    s, c2, cells = screen_and_cells(x, cut)
    pairs = accepted_pairs(s, c2)
    assert pairs, "the cloud must contain accepted pairs"
    for i, j in pairs:
        assert np.all(np.abs(cells[i] - cells[j]) <= 1), (i, j, cells[i], cells[j])
    return len(pairs)


def test_pairs_at_the_cutoff_far_from_the_origin():
    """Pairs at 0.999-1.001 of the cutoff in random orientations, the cloud
    offset by up to 1000 cutoffs (coarse FP32 offsets)."""
    rng = np.random.default_rng(1)
    cut = float(F(1.1 * 2.0) * F(1.001))
    for offset in (0.0, 37.5, 1000.0):
        a = rng.uniform(-offset * cut - 50, offset * cut + 50, size=(300, 3))
        u = rng.normal(size=(300, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        b = a + u * cut * rng.uniform(0.999, 1.001, size=(300, 1))
        x = np.concatenate([a, b]) + offset * cut
        check_cloud(x, cut)


def test_dense_cloud_and_cell_boundaries():
    """A dense cloud, and pairs straddling cell boundaries along each axis."""
    rng = np.random.default_rng(2)
    cut = float(F(1.1 * 2.0) * F(1.001))
    x = rng.uniform(0, 20, size=(400, 3))
    assert check_cloud(x, cut) > 100
    h = cut * 1.01
    base = rng.integers(-50, 50, size=(200, 3)) * h
    d = np.zeros((200, 3))
    d[np.arange(200), rng.integers(0, 3, 200)] = cut * 0.9995
    x = np.concatenate([base - 1e-7, base - 1e-7 + d])
    check_cloud(x, cut)
