"""The post-processing reductions on the GPU (vp_consistency, vp_surface_loads, vp_pressure_force, vp_wake_loads
through the C ABI) against the oracle's restatement of consistency (src/assembly/solve.jl:111-115), the gradient route
(src/post/Post.jl:72-84), the pressure force, Kutta-Joukowski and Trefftz (src/post/forces.jl:11-81), on the same
inputs. FP64 on both sides; the sums run in other orders, so agreement is to rounding (1e-12 of the scale)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

V0 = np.array([1.0, 0.3, -0.2]) / np.linalg.norm([1.0, 0.3, -0.2])


@pytest.fixture(scope="module")
def sphere(vp):
    g, dm = vp.meshes.sphere_case(2)
    els = vp.build_elements(g)
    A, b, _ = vp.assemble(g, dm, els, vp.source_strengths(els, V0), V0)
    return g, dm, els, A, b


@pytest.fixture(scope="module")
def wing(vp):
    w = vp.meshes.wing(10, 6, aspect=4.0)
    wake = vp.meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
    W = vp.meshes.wake_rows(w.dm, wake.te)
    a = math.radians(5.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    els = vp.build_elements(w.g)
    A, b, _ = vp.assemble(w.g, w.dm, els, vp.source_strengths(els, V), V, wake=wake)
    return w, wake, W, V, els, A, b


def _close(a, b, rel=1e-12, floor=1e-15):
    return abs(a - b) <= rel * abs(b) + floor


def test_consistency_sphere(vp, oracle, sphere):
    # the reference's bounds on icosphere(2) (test/assembly/test_sphere.jl:44-47), and the oracle's values
    g, dm, els, A, b = sphere
    c = vp.consistency(dm, A)
    co = oracle.consistency(dm, A.download(), b)
    assert c["rows"] < 1e-12 and c["columns"] < 1e-5 and c["rhs"] < 1e-12
    assert _close(c["columns"], co["columns"], 1e-9)
    assert abs(c["rows"] - co["rows"]) < 1e-14 and abs(c["rhs"] - co["rhs"]) < 1e-15


def test_consistency_wing_with_wake_rows(vp, oracle, wing):
    w, wake, W, V, els, A, b = wing
    c = vp.consistency(w.dm, A, W=W)
    co = oracle.consistency(w.dm, A.download(), b, W=W)
    for k in ("rows", "columns", "rhs"):
        assert _close(c[k], co[k], 1e-9, 1e-15), (k, c[k], co[k])
    with pytest.raises(ValueError):
        vp.consistency(w.dm, A)  # wake columns without W
    c2 = vp.consistency(w.dm, A, W=W)
    assert c2 == c  # fixed summation order: bit-identical


def test_surface_loads(vp, oracle, wing):
    w, wake, W, V, els, A, b = wing
    rng = np.random.default_rng(3)
    mu = 0.3 * rng.standard_normal(w.dm.nslot)
    dmu = 0.1 * rng.standard_normal(w.dm.nslot)
    origin = np.array([0.25, 0.0, 0.0])
    r = vp.surface_loads(els, w.dm, mu, V, dmudt=dmu, origin=origin)
    oe = oracle.elements(w.g)
    u = oracle.gradient_velocity(w.g, w.dm, mu, V, els=oe)
    cp = oracle.pressure_coefficient(u, V, dmu[w.dm.corner_slot].mean(axis=1))
    F, M = oracle.pressure_force(oe, cp, origin)
    assert np.max(np.abs(r["u"] - u)) <= 1e-13 * np.max(np.abs(u))
    assert np.max(np.abs(r["cp"] - cp)) <= 1e-13 * np.max(np.abs(cp))
    assert np.max(np.abs(r["F"] - F)) <= 1e-12 * np.max(np.abs(F)) and np.max(np.abs(r["M"] - M)) <= 1e-12 * np.max(np.abs(M))
    # steady: gradient_velocity alone, and pressure_force of a given cp
    u0 = vp.gradient_velocity(els, w.dm, mu, V)
    assert np.max(np.abs(u0 - u)) <= 1e-13 * np.max(np.abs(u))
    cp0 = oracle.pressure_coefficient(u, V)
    F0, M0 = vp.pressure_force(els, cp0)
    Fo, Mo = oracle.pressure_force(oe, cp0)
    assert np.max(np.abs(F0 - Fo)) <= 1e-12 * np.max(np.abs(Fo)) and np.max(np.abs(M0 - Mo)) <= 1e-12 * np.max(np.abs(Mo))


def test_wake_loads(vp, oracle, wing):
    w, wake, W, V, els, A, b = wing
    wte = w.dm.wake_te
    rng = np.random.default_rng(4)
    muw = np.sin(np.linspace(0, math.pi, len(wte.node))) + 0.05 * rng.standard_normal(len(wte.node))
    F, D = vp.wake_loads(wte, muw, V)
    Fo = oracle.kutta_joukowski_force(wte, muw, V)
    Do = oracle.trefftz_drag(wte, muw, V)
    assert np.max(np.abs(F - Fo)) <= 1e-13 * np.max(np.abs(Fo))
    assert _close(D, Do, 1e-12)
    # a closed line (a ring), where every node's trailing vortex takes the last strip as its "before"
    th = np.linspace(0, 2 * math.pi, 13)[:-1]
    ring = vp.meshes.WakeTE(np.arange(12), np.stack([np.zeros(12), np.cos(th), np.sin(th)], axis=1), [np.arange(12)],
                            [True])
    mur = 1 + 0.3 * np.cos(th) + 0.1 * np.sin(2 * th)
    F, D = vp.wake_loads(ring, mur, V)
    assert np.max(np.abs(F - oracle.kutta_joukowski_force(ring, mur, V))) <= 1e-13
    assert _close(D, oracle.trefftz_drag(ring, mur, V), 1e-12)


def test_loads_errors(vp, wing):
    w, wake, W, V, els, A, b = wing
    with pytest.raises(ValueError):
        vp.surface_loads(els, w.dm, np.zeros(3), V)
    with pytest.raises(ValueError):
        vp.wake_loads(w.dm.wake_te, np.zeros(len(w.dm.wake_te.node)), np.zeros(3))
