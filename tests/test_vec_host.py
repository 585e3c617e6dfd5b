"""The host's row-wise 3-vector helpers (vortexpanel_gpu/_vec.py) give numpy's own results bit for bit: cross3 as
np.cross, norm3 as np.linalg.norm(axis=1), scatter_add as np.add.at from zeros (vector and row weights, repeated
indices in any order)."""
import numpy as np

from vortexpanel_gpu._vec import cross3, dot3, norm3, scatter_add


def test_cross_norm_dot_match_numpy():
    rng = np.random.default_rng(3)
    a = rng.standard_normal((5000, 3)) * 10.0 ** rng.uniform(-8, 8, (5000, 1))
    b = rng.standard_normal((5000, 3))
    assert np.array_equal(cross3(a, b), np.cross(a, b))
    assert np.array_equal(norm3(a), np.linalg.norm(a, axis=1))
    assert np.array_equal(dot3(a, b), a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1] + a[:, 2] * b[:, 2])


def test_scatter_add_matches_add_at():
    rng = np.random.default_rng(4)
    idx = rng.integers(0, 300, (4000, 3))
    w = rng.standard_normal(idx.size) * 10.0 ** rng.uniform(-6, 6, idx.size)
    ref = np.zeros(310)
    np.add.at(ref, idx.ravel(), w)
    assert np.array_equal(scatter_add(310, idx, w), ref)
    rows = rng.standard_normal((idx.shape[0] * 3, 3))
    ref = np.zeros((300, 3))
    for k in range(3):
        np.add.at(ref, idx[:, k], rows[k * idx.shape[0]:(k + 1) * idx.shape[0]])
    assert np.array_equal(scatter_add(300, idx.T, rows), ref)
