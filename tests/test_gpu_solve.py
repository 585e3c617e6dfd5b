"""Parity of the GPU bordered solve (vp_factorize / vp_solve / vp_solve_system through the C ABI) with the oracle,
which solves the same bordered system with LAPACK (dgetrf, dgecon) as the reference does (src/assembly/solve.jl)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sphere(vp, oracle):
    g, dm = vp.meshes.sphere_case(2)
    V = np.array([1.0, 0.3, -0.2])
    V /= np.linalg.norm(V)
    els = vp.build_elements(g)
    sig = vp.source_strengths(els, V)
    A, b, _ = vp.assemble(g, dm, els, sig, V)
    ref = oracle.solve_galerkin(dm, A.download(), b)
    return g, dm, V, els, sig, A, b, ref


@pytest.fixture(scope="module")
def wing(vp, oracle):
    w = vp.meshes.wing(12, 8, aspect=4.0)
    wake = vp.meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
    W = vp.meshes.wake_rows(w.dm, wake.te)
    a = np.radians(5.0)
    V = np.array([np.cos(a), 0.0, np.sin(a)])
    els = vp.build_elements(w.g)
    sig = vp.source_strengths(els, V)
    A, b, _ = vp.assemble(w.g, w.dm, els, sig, V, wake=wake)
    ref = oracle.solve_galerkin(w.dm, A.download(), b, W=W)
    return w, wake, W, V, els, sig, A, b, ref


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sphere_solve(vp, sphere, precision):
    g, dm, V, els, sig, A, b, ref = sphere
    s = vp.solve_galerkin(dm, A, b, precision=precision)
    scale = np.max(np.abs(ref["q"]))
    assert np.max(np.abs(s["q"] - ref["q"])) < 1e-11 * scale
    assert abs(s["lam"][0] - ref["lam"][0]) < 1e-12
    assert s["residual"] < 1e-12
    assert abs(s["cond"] / ref["cond"] - 1) < 0.05


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wing_solve_and_loads(vp, oracle, wing, precision):
    w, wake, W, V, els, sig, A, b, ref = wing
    F = vp.factorize_galerkin(w.dm, A, W=W, precision=precision)
    s = vp.solve_galerkin(F, b)
    scale = np.max(np.abs(ref["q"]))
    assert np.max(np.abs(s["q"] - ref["q"])) < 1e-10 * scale
    mu_w = w.dm.K @ s["q"]
    mu_w_ref = w.dm.K @ ref["q"]
    S = w.span * w.chord
    eL = np.array([-np.sin(np.radians(5)), 0, np.cos(np.radians(5))])
    cp = vp.pressure_coefficient(vp.gradient_velocity(els, w.dm, s["mu"], V), V)
    oels = oracle.elements(w.g)
    cp_ref = oracle.pressure_coefficient(oracle.gradient_velocity(w.g, w.dm, ref["mu"], V, oels), V)
    CL = vp.pressure_force(els, cp)[0] @ eL / S
    CL_ref = oracle.pressure_force(oels, cp_ref)[0] @ eL / S
    assert abs(CL - CL_ref) < 1e-10
    CDi = vp.trefftz_drag(w.dm.wake_te, mu_w, V) / S
    CDi_ref = oracle.trefftz_drag(w.dm.wake_te, mu_w_ref, V) / S
    assert abs(CDi - CDi_ref) < 1e-12
    assert CL > 0.1 and CDi > 0


def test_many_rhs(vp, oracle, wing):
    w, wake, W, V, els, sig, A, b, ref = wing
    F = vp.factorize_galerkin(w.dm, A, W=W)
    B = np.stack([b, 2 * b, b + 1e-3], axis=1)
    s = vp.solve_galerkin(F, B)
    r = oracle.solve_factored(ref["F"], B)
    assert np.max(np.abs(s["q"] - r["q"])) < 1e-10 * np.max(np.abs(r["q"]))
    assert np.max(np.abs(s["lam"] - r["lam"])) < 1e-10


def test_incompatible_rhs(vp, sphere):
    # λ takes up an incompatible right hand side (test_sphere.jl:50-51)
    g, dm, V, els, sig, A, b, ref = sphere
    F = vp.factorize_galerkin(dm, A)
    s = vp.solve_galerkin(F, b + 1e-3)
    assert abs(s["lam"][0] - 1e-3) < 1e-9


def test_dimension_mismatch(vp, wing):
    w, wake, W, V, els, sig, A, b, ref = wing
    with pytest.raises(ValueError):
        vp.factorize_galerkin(w.dm, A)  # A has wake columns, W missing


def test_external_field_end_to_end(vp, sphere):
    # a uniform external velocity U0 through assemble(..., external=) equals the freestream V + U0: the device b plus
    # the host's 7-point term (exact for a constant field on hat functions), and the solution of either
    g, dm, V, els, sig, A, b, ref = sphere
    U0 = np.array([0.2, -0.1, 0.05])
    sig2 = vp.source_strengths(els, V + U0)
    A1, b1, _ = vp.assemble(g, dm, els, sig2, V, external=lambda X: np.tile(U0, (len(X), 1)))
    A2, b2, _ = vp.assemble(g, dm, els, sig2, V + U0)
    assert np.max(np.abs(b1 - b2)) < 1e-13 * np.max(np.abs(b2))
    s1 = vp.solve_galerkin(vp.factorize_galerkin(dm, A1), b1)
    s2 = vp.solve_galerkin(dm, A2, b2)
    assert np.max(np.abs(s1["q"] - s2["q"])) < 1e-11 * np.max(np.abs(s2["q"]))
