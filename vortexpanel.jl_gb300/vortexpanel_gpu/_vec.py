"""Row-wise 3-vector arithmetic for the host side of a step (n x 3 float arrays), written out by component: numpy's
generic cross, norm and unbuffered add.at carry a per-call overhead that dominated the host part of a 25k-triangle
step. Each returns the same values, bit for bit, as the numpy call it replaces: the same products and sums in the
same order."""
from __future__ import annotations

import numpy as np


def cross3(a, b):
    """np.cross(a, b) of n x 3 arrays"""
    a0, a1, a2 = a[:, 0], a[:, 1], a[:, 2]
    b0, b1, b2 = b[:, 0], b[:, 1], b[:, 2]
    out = np.empty((a.shape[0], 3))
    out[:, 0] = a1 * b2 - a2 * b1
    out[:, 1] = a2 * b0 - a0 * b2
    out[:, 2] = a0 * b1 - a1 * b0
    return out


def dot3(a, b):
    """the row-wise dot product of n x 3 arrays, summed in component order"""
    return a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1] + a[:, 2] * b[:, 2]


def norm3(a):
    """np.linalg.norm(a, axis=1) of an n x 3 array"""
    return np.sqrt(dot3(a, a))


def scatter_add(n, idx, w):
    """out[idx[i]] += w[i] over i in order from zeros(n), as np.add.at does (w: a vector, or rows of an array)"""
    idx = np.asarray(idx).ravel()
    if w.ndim == 1:
        return np.bincount(idx, weights=w, minlength=n)
    out = np.empty((n, w.shape[1]))
    for d in range(w.shape[1]):
        out[:, d] = np.bincount(idx, weights=w[:, d], minlength=n)
    return out
