"""The explicit parts of the adjoint gradients (host code, no GPU): the derivatives of CL of the gradient route
(Post.jl:72-84, forces.jl:11-20) and of CDi of the Trefftz plane (forces.jl:53-81) with respect to the doublet
values, the node coordinates and alpha, against central finite differences of the oracle's restatement of the
loads."""
import math

import numpy as np
import pytest

import oracle as O
from vortexpanel_gpu import meshes
from vortexpanel_gpu.adjoint import cdi_trefftz, cl_pressure


@pytest.fixture(scope="module")
def small_wing():
    return meshes.wing(10, 6, aspect=6.0)


def _cl(w, x, mu, a):
    g = meshes.Geometry(x, w.g.tris)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    eL = np.array([-math.sin(a), 0.0, math.cos(a)])
    els = O.elements(g)
    cp = O.pressure_coefficient(O.gradient_velocity(g, w.dm, mu, V, els=els), V)
    return float(O.pressure_force(els, cp)[0] @ eL / (w.span * w.chord))


def test_cl_explicit_derivatives(small_wing):
    w = small_wing
    rng = np.random.default_rng(2)
    mu = rng.standard_normal(w.dm.nslot) * 0.3
    a = math.radians(4.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    dV = np.array([-math.sin(a), 0.0, math.cos(a)])
    CL, dmu, gx, dal = cl_pressure(w.g, w.dm, mu, V, dV, dV.copy(), -V, w.span * w.chord)
    assert abs(CL - _cl(w, w.g.x, mu, a)) <= 1e-13
    h = 1e-6
    for i in rng.choice(w.dm.nslot, 6, replace=False):
        e = np.zeros_like(mu)
        e[i] = h
        fd = (_cl(w, w.g.x, mu + e, a) - _cl(w, w.g.x, mu - e, a)) / (2 * h)
        assert abs(dmu[i] - fd) <= 1e-7 * max(1.0, abs(fd))
    for n in rng.choice(w.g.nnode, 6, replace=False):
        for k in range(3):
            xp, xm = w.g.x.copy(), w.g.x.copy()
            xp[n, k] += h
            xm[n, k] -= h
            fd = (_cl(w, xp, mu, a) - _cl(w, xm, mu, a)) / (2 * h)
            assert abs(gx[n, k] - fd) <= 1e-6 * max(1.0, np.abs(gx).max())
    fd = (_cl(w, w.g.x, mu, a + h) - _cl(w, w.g.x, mu, a - h)) / (2 * h)
    assert abs(dal - fd) <= 1e-7


def test_cdi_explicit_derivatives(small_wing):
    w = small_wing
    wte = w.dm.wake_te
    rng = np.random.default_rng(3)
    muw = np.sin(np.linspace(0, math.pi, len(wte.node))) + 0.1 * rng.standard_normal(len(wte.node))
    S = w.span * w.chord
    a = math.radians(6.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    dV = np.array([-math.sin(a), 0.0, math.cos(a)])

    def cdi(X, mu, al):
        t = meshes.WakeTE(wte.node, X, wte.lines, wte.closed)
        VV = np.array([math.cos(al), 0.0, math.sin(al)])
        return O.trefftz_drag(t, mu, VV) / S

    CDi, dmu, gx, dal = cdi_trefftz(wte, muw, V, dV, S)
    assert abs(CDi - cdi(wte.x, muw, a)) <= 1e-13 * max(1.0, abs(CDi))
    h = 1e-6
    for i in range(len(muw)):
        e = np.zeros_like(muw)
        e[i] = h
        fd = (cdi(wte.x, muw + e, a) - cdi(wte.x, muw - e, a)) / (2 * h)
        assert abs(dmu[i] - fd) <= 1e-7 * max(1.0, np.abs(dmu).max())
    for n in range(len(muw)):
        for k in range(3):
            xp, xm = wte.x.copy(), wte.x.copy()
            xp[n, k] += h
            xm[n, k] -= h
            fd = (cdi(xp, muw, a) - cdi(xm, muw, a)) / (2 * h)
            assert abs(gx[n, k] - fd) <= 1e-6 * max(1.0, np.abs(gx).max())
    fd = (cdi(wte.x, muw, a + h) - cdi(wte.x, muw, a - h)) / (2 * h)
    assert abs(dal - fd) <= 1e-7 * max(1.0, abs(dal))
