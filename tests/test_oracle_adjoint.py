"""The oracle's adjoints (the CPU checkers of the adjoint skeletons) against
FP64 central finite differences of the oracle's own forward functions."""
import numpy as np
import pytest


def fd(loss, x, j, h=0.5):
    xp, xm = x.copy(), x.copy()
    xp.flat[j] += h
    xm.flat[j] -= h
    return (loss(xp) - loss(xm)) / (float(xp.flat[j]) - float(xm.flat[j]))


@pytest.mark.parametrize("shape", [(23, 31), (1, 17), (12, 2)])
@pytest.mark.parametrize("padding", [0, 1])
def test_stencil_adjoint_matches_fd(orc, shape, padding):
    rows, cols = shape
    R = 3
    img = orc.uniform_f32(rows * cols, 1, 0.0, 255.0).reshape(rows, cols)
    g = orc.uniform_f32(rows * cols, 2, -1.0, 1.0).reshape(rows, cols)
    w = orc.uniform_f32((2 * R + 1) ** 2, 3, -1.0, 1.0)
    g64 = g.astype(np.float64)
    loss = lambda v: float((g64 * orc.stencil_f64(v, R, w, padding, 0.0)).sum())
    adj = orc.stencil_adjoint_f64(g, R, w, padding)
    for j in range(rows * cols):  # every pixel: edges and corners included
        assert abs(fd(loss, img, j) - adj.flat[j]) <= 1e-6 * max(1.0, abs(adj.flat[j])), j


@pytest.mark.parametrize("inclusive", [False, True])
def test_reverse_scan_is_scan_adjoint(orc, inclusive):
    n = 1000
    x = orc.uniform_f32(n, 4, -1.0, 1.0)
    g = orc.uniform_f32(n, 5, -1.0, 1.0)
    g64 = g.astype(np.float64)
    loss = lambda v: float(np.dot(g64, orc.scan_f64(v, inclusive=inclusive)))
    adj = orc.scan_f64(g, inclusive=inclusive, reverse=True)
    for j in range(0, n, 37):
        assert abs(fd(loss, x, j) - adj[j]) <= 1e-9 * max(1.0, abs(adj[j]))
