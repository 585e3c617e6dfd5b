"""assemble's external velocity field (src/assembly/assemble.jl:423-427), the host part of b (api.external_rhs), on
the CPU: the 7-point Radon rule (rules.jl:76-92) is exact to degree 5, so a constant and a linear field give the
closed-form integrals -∫ψ_a n·u dA of the hat, onering and dual test functions."""
import math

import numpy as np
import pytest

from vortexpanel_gpu import api, meshes


def test_radon7_degree_five():
    lam, w = api.radon7()
    assert abs(w.sum() - 1) < 1e-15 and np.abs(lam.sum(1) - 1).max() < 1e-15
    for p, q, r in ((1, 0, 0), (2, 1, 0), (1, 1, 1), (3, 0, 2), (5, 0, 0), (2, 2, 1)):
        exact = 2 * math.factorial(p) * math.factorial(q) * math.factorial(r) / math.factorial(p + q + r + 2)
        assert abs(w @ (lam[:, 0] ** p * lam[:, 1] ** q * lam[:, 2] ** r) / exact - 1) < 1e-13


@pytest.fixture(scope="module")
def sphere():
    g, dm = meshes.sphere_case(1)
    return g, dm, api.build_elements(g)


def test_constant_field(sphere):
    g, dm, els = sphere
    U0 = np.array([0.3, -1.0, 0.5])
    for test, per_corner in (("hat", 1 / 3), ("onering", 1.0), ("dual", 1 / 3)):
        b = api.external_rhs(els, dm, lambda X: np.broadcast_to(U0, X.shape), test)
        ref = np.zeros(dm.nslot)
        np.add.at(ref, dm.corner_slot, -np.repeat(((els.n @ U0) * els.area * per_corner)[:, None], 3, axis=1))
        if test == "dual":  # the dual cells' areas are not a third each; only the total is
            assert abs(b.sum() - ref.sum()) < 1e-13 * np.abs(ref).sum()
        else:
            assert np.abs(b - ref).max() < 1e-14 * np.abs(ref).max()


def test_linear_field(sphere):
    g, dm, els = sphere
    M = np.array([[0.2, -0.1, 0.4], [0.0, 0.3, -0.2], [0.5, 0.1, -0.3]])
    c = np.array([0.1, 0.2, -0.3])
    b = api.external_rhs(els, dm, lambda X: X @ M.T + c, "hat")
    # hat: -∫λ_a (u·n) dA with u·n linear, ∫λ_a λ_b dA = A (1 + δ_ab) / 12
    corners = els.corners.reshape(-1, 3, 3)
    un = np.einsum("tkd,td->tk", corners @ M.T + c, els.n)
    rows = -(els.area[:, None] / 12) * (un.sum(1)[:, None] + un)
    ref = np.zeros(dm.nslot)
    np.add.at(ref, dm.corner_slot, rows)
    assert np.abs(b - ref).max() < 1e-14 * np.abs(ref).max()


def test_test_weights():
    lam, _ = api.radon7()
    assert np.array_equal(api.test_weights("hat", lam), lam)
    d = api.test_weights("dual", lam)
    assert np.abs(d.sum(1) - 1).max() < 1e-15 and np.allclose(d[0], 1 / 3)  # the centre's tie is shared
    with pytest.raises(ValueError):
        api.test_weights("box", lam)
