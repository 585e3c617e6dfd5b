"""The oracle pinned to the reference's known answers (CPU, no GPU): the quadrature rules
(test/elements/test_elements.jl:8-47), the sphere's exact doublet, its surface velocity and the system diagnostics
(test/assembly/test_sphere.jl:34-55), the Carlson integrals of the ellipsoid (test/assembly/test_ellipsoid.jl:30-33),
and the Kutta-Joukowski and Trefftz loads of an elliptic loading (test/post/test_forces.jl:25-49). The reference
stores no golden arrays; these are the values and bounds its own tests assert."""
import math

import numpy as np
import pytest

from vortexpanel_gpu import meshes


def mono(a, b, c):
    """integral over the triangle of l1^a l2^b l3^c dA / A"""
    return 2 * math.factorial(a) * math.factorial(b) * math.factorial(c) / math.factorial(a + b + c + 2)


def integ(lam, w, f):
    return float(sum(wi * f(l) for l, wi in zip(lam, w)))


def test_gauss_legendre_and_graded(oracle):
    for n in (1, 2, 5, 9):
        x, w = oracle.rule1d("gauss", n)
        for k in range(2 * n):
            assert abs(np.sum(w * x ** k) - 1 / (k + 1)) <= 1e-14
    x, w = oracle.rule1d("graded", levels=6, ratio=0.15, order=3)
    assert abs(w.sum() - 1) < 1e-14
    assert abs(np.sum(w * np.log(x)) + 1) <= 1e-6


@pytest.mark.parametrize("n,degree", [(1, 1), (3, 2), (6, 4), (7, 5)])
def test_triangle_rules(oracle, n, degree):
    lam, w = oracle.rule("triangle", n)
    assert abs(w.sum() - 1) < 1e-14
    for a in range(degree + 1):
        for b in range(degree + 1 - a):
            for c in range(degree + 1 - a - b):
                assert abs(integ(lam, w, lambda l: l[0] ** a * l[1] ** b * l[2] ** c) - mono(a, b, c)) <= 1e-14


def test_graded_rules(oracle):
    e, v, s = oracle.rule("edge"), oracle.rule("vertex"), oracle.rule("self")
    for lam, w in (e, v, s):
        assert abs(w.sum() - 1) < 1e-13
        assert (lam > 0).all() and np.allclose(lam.sum(axis=1), 1, atol=1e-14)
        assert abs(integ(lam, w, lambda l: l[0] ** 2 * l[1] * l[2]) / mono(2, 1, 1) - 1) <= 1e-12
    assert abs(integ(*e, lambda l: math.log(l[2])) / -1.5 - 1) <= 1e-6
    assert abs(integ(*v, lambda l: math.log(1 - l[0])) / -0.5 - 1) <= 1e-6
    assert abs(integ(*s, lambda l: math.log(l[0]) + math.log(l[1]) + math.log(l[2])) / -4.5 - 1) <= 1e-6
    errs = [abs(integ(*oracle.rule("edge", levels=L), lambda l: math.log(l[2])) + 1.5) for L in (2, 4, 6)]
    assert errs[2] < errs[1] < errs[0]
    for k in range(3):
        assert abs(integ(*oracle.rule("edge", k=k), lambda l: math.log(l[(k + 2) % 3])) / -1.5 - 1) <= 1e-6
        assert abs(integ(*oracle.rule("vertex", k=k), lambda l: math.log(1 - l[k])) / -0.5 - 1) <= 1e-6


@pytest.fixture(scope="module")
def sphere2(oracle):
    V = np.array([1.0, 0.3, -0.2])
    V /= np.linalg.norm(V)
    g, dm = meshes.sphere_case(2)
    sig = oracle.source_strengths(g, V)
    A, b, stats = oracle.assemble(g, dm, sig, V)
    sol = oracle.solve_galerkin(dm, A, b)
    return g, dm, V, A, b, stats, sol


def test_sphere_exact_doublet(oracle, sphere2):
    g, dm, V, A, b, stats, sol = sphere2
    node_of_slot = np.zeros(dm.nslot, int)
    node_of_slot[dm.corner_slot.ravel()] = g.tris.ravel()
    mu_ex = g.x[node_of_slot] @ V / 2
    err = sol["mu"] - mu_ex
    err -= np.sum(dm.slot_area * err) / np.sum(dm.slot_area)
    muL2 = math.sqrt(np.sum(dm.slot_area * err ** 2) / np.sum(dm.slot_area)) / 0.5
    assert muL2 < 3e-3 and np.abs(err).max() / 0.5 < 1e-2
    els = oracle.elements(g)
    ug = oracle.gradient_velocity(g, dm, sol["mu"], V, els=els)
    cp = oracle.pressure_coefficient(ug, V)
    c = els["centroid"] / np.linalg.norm(els["centroid"], axis=1)[:, None]
    cpex = 1 - 9 / 4 * (1 - (c @ V) ** 2)
    assert math.sqrt(np.sum(els["area"] * (cp - cpex) ** 2) / np.sum(els["area"])) < 0.025


def test_sphere_surface_velocity(oracle, sphere2):
    # the two velocity routes agree and the leak is O(h) (test_sphere.jl:19-32,40): singularity sums at the centroids
    # (Post.jl:32-64) against the doublet gradient
    g, dm, V, A, b, stats, sol = sphere2
    els = oracle.elements(g)
    u = oracle.surface_velocity(g, dm, oracle.source_strengths(g, V), sol["mu"], V)
    ug = oracle.gradient_velocity(g, dm, sol["mu"], V, els=els)
    n = els["n"]
    rms = lambda v: math.sqrt(np.sum(els["area"] * v ** 2) / np.sum(els["area"]))  # noqa: E731
    c = els["centroid"] / np.linalg.norm(els["centroid"], axis=1)[:, None]
    cpex = 1 - 9 / 4 * (1 - (c @ V) ** 2)
    assert rms(oracle.pressure_coefficient(u, V) - cpex) < 0.08
    tang = u - np.einsum("ij,ij->i", u, n)[:, None] * n
    assert np.linalg.norm(tang - ug, axis=1).max() < 0.05
    assert rms(np.einsum("ij,ij->i", u, n)) < 0.045


def test_sphere_system_diagnostics(oracle, sphere2):
    g, dm, V, A, b, stats, sol = sphere2
    c = oracle.consistency(dm, A, b)
    assert c["rows"] < 1e-12 and c["columns"] < 1e-5 and c["rhs"] < 1e-12
    assert abs(sol["lam"][0]) < 1e-14 and sol["residual"] < 1e-12
    shifted = oracle.solve_galerkin(dm, A, b + 1e-3)
    assert abs(shifted["lam"][0] - 1e-3) < 1e-9
    assert sol["cond"] < 1e3
    assert stats["pairs"]["self"] == g.ntri and sum(stats["pairs"].values()) == g.ntri ** 2


def test_carlson_and_ellipsoid_factors(oracle):
    assert abs(oracle.carlson_rd(0.0, 2.0, 1.0) - 1.7972103521034) < 1e-12
    assert abs(oracle.carlson_rd(2.0, 3.0, 4.0) - 0.16510527294261) < 1e-13
    for axes in ((3.0, 1.0, 1.0), (1.0, 2.0, 3.0), (1.0, 1.0, 1.0)):
        assert abs(oracle.ellipsoid_factors(*axes).sum() - 2) < 1e-12


def _straight_te(y):
    x = np.stack([np.zeros(len(y)), np.asarray(y), np.zeros(len(y))], axis=1)
    return meshes.WakeTE(np.arange(len(y), dtype=np.int32), x, [np.arange(len(y))], [False])


def test_kutta_joukowski_and_trefftz(oracle):
    wte = _straight_te(np.linspace(-1.0, 1.0, 9))
    V = np.array([2.0, 0.0, 0.0])
    assert np.allclose(oracle.kutta_joukowski_force(wte, np.full(9, 0.8), V), [0.0, 0.0, 2 * 0.8 * 2.0 / 2.0],
                       rtol=1e-14, atol=1e-15)
    b, c = 2.0, 0.5
    AR = b / c
    V = np.array([1.0, 0.0, 0.0])

    def ratio(n):
        y = np.array([-b / 2 * math.cos(math.pi * k / n) for k in range(n + 1)])
        mu = np.sqrt(np.maximum(0.0, 1 - (2 * y / b) ** 2))
        w = _straight_te(y)
        CL = oracle.kutta_joukowski_force(w, mu, V)[2] / (b * c)
        CD = oracle.trefftz_drag(w, mu, V) / (b * c)
        return CD / (CL ** 2 / (math.pi * AR))

    assert abs(ratio(160) - 1) < 0.01
    assert abs(ratio(160) - 1) < abs(ratio(40) - 1) < abs(ratio(10) - 1)
    y = np.array([-math.cos(math.pi * k / 40) for k in range(41)])
    mu = np.sqrt(np.maximum(0.0, 1 - y ** 2))
    d5 = np.array([math.cos(math.radians(5)), 0.0, math.sin(math.radians(5))])
    assert abs(oracle.trefftz_drag(_straight_te(y), mu, d5) / oracle.trefftz_drag(_straight_te(y), mu, V) - 1) < 1e-12
