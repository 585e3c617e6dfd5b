"""The derivative oracle (the C++ oracle's assembly on forward-mode dual numbers, the bordered solve and the loads
on jets) pinned the way the reference pins its derivatives (test/kernels/test_kernels.jl:127-148): the source
kernel's Jacobian is divergence- and curl-free off the triangle and its vertex derivatives agree with central
differences at 1e-7; and the whole wing pipeline's directional derivatives agree with central differences of the
FP64 oracle itself."""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import dual_oracle  # noqa: E402
import oracle  # noqa: E402
import wingcase  # noqa: E402

from vortexpanel_gpu import meshes  # noqa: E402


def _tri():
    rng = np.random.default_rng(7)
    a, b, c = rng.standard_normal((3, 3))
    return a, b, c


def test_source_velocity_jacobian_is_div_and_curl_free():
    a, b, c = _tri()
    n = np.cross(b - a, c - a)
    n /= np.linalg.norm(n)
    cen = (a + b + c) / 3
    diam = max(np.linalg.norm(b - a), np.linalg.norm(c - b), np.linalg.norm(a - c))
    nu1 = np.cross(c - b, n)
    nu1 /= np.linalg.norm(nu1)
    nu3 = np.cross(b - a, n)
    nu3 /= np.linalg.norm(nu3)
    pts = [cen + 0.05 * diam * n, b + 0.02 * diam * (n + nu1) / np.linalg.norm(n + nu1),
           cen + 30 * diam * (n + nu3) / np.linalg.norm(n + nu3)]
    for x in pts:
        w, Jm = dual_oracle.source_velocity_jacobian(a, b, c, x)
        w0 = oracle.source_velocity(a, b, c, x)
        assert np.allclose(w, w0, rtol=0, atol=1e-15 * np.linalg.norm(w0))
        s = np.linalg.norm(Jm)
        assert abs(np.trace(Jm)) < 1e-12 * s and np.linalg.norm(Jm - Jm.T) < 1e-12 * s


def test_source_velocity_vertex_derivative_against_differences():
    a, b, c = _tri()
    n = np.cross(b - a, c - a)
    n /= np.linalg.norm(n)
    diam = max(np.linalg.norm(b - a), np.linalg.norm(c - b), np.linalg.norm(a - c))
    x0 = (a + b + c) / 3 + 0.3 * diam * n
    _, Jm = dual_oracle.source_velocity_jacobian(a, b, c, x0, wrt="a", far=math.inf)
    h = 1e-6
    Jfd = np.stack([(oracle.source_velocity(a + h * e, b, c, x0, far=math.inf) -
                     oracle.source_velocity(a - h * e, b, c, x0, far=math.inf)) / (2 * h) for e in np.eye(3)], axis=1)
    assert np.allclose(Jm, Jfd, rtol=1e-7, atol=1e-7 * np.abs(Jfd).max())


def _oracle_loads(w, wake, W, a):
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    eL = np.array([-math.sin(a), 0.0, math.cos(a)])
    A, b, _ = oracle.assemble(w.g, w.dm, oracle.source_strengths(w.g, V), V, wake=wake)
    s = oracle.solve_galerkin(w.dm, A, b, W)
    els = oracle.elements(w.g)
    cp = oracle.pressure_coefficient(oracle.gradient_velocity(w.g, w.dm, s["mu"], V, els), V)
    F, _ = oracle.pressure_force(els, cp)
    S = w.span * w.chord
    return F @ eL / S, oracle.trefftz_drag(w.dm.wake_te, w.dm.K @ s["q"], V) / S


def test_wing_tangents_against_oracle_differences():
    """the dual pipeline on a small jittered wing with its rigid wake: CL and CDi equal the oracle's, and their
    derivatives along single node coordinates (a trailing edge node among them, whose wake rows move with it) and
    alpha agree with central differences of the oracle, step 1e-6"""
    w = wingcase.jittered(meshes.wing(8, 5, aspect=6.0))
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
    W = meshes.wake_rows(w.dm, wake.te)
    a = math.radians(5.0)
    rng = np.random.default_rng(1)
    nodes = [(int(n), int(rng.integers(3))) for n in rng.choice(wingcase.clear_nodes(w.g), 3, replace=False)]
    nodes.append((int(w.dm.wake_te.node[len(w.dm.wake_te.node) // 2]), 0))
    # the trailing edge node at the tip, across the wake's plane: points of the tip cap lie in the first wake sheet's
    # plane, where the solid angle's value takes the in-plane branch and its derivative the off-plane formula's
    te = w.dm.wake_te.node
    nodes.append((int(te[np.argmin(w.g.x[te, 1])]), 2))
    dirs = []
    for n, c in nodes:
        dx = np.zeros((w.g.nnode, 3))
        dx[n, c] = 1.0
        dirs.append((dx, 0.0))
    dirs.append((np.zeros((w.g.nnode, 3)), 1.0))
    CL, CDi, dCL, dCDi = dual_oracle.wing_loads_tangent(w, wake, W, a, dirs)
    CL0, CDi0 = _oracle_loads(w, wake, W, a)
    assert abs(CL - CL0) < 1e-12 and abs(CDi - CDi0) < 1e-13
    h = 1e-6
    for k, (dx, da) in enumerate(dirs):
        p = _oracle_loads(*wingcase.moved(w, wake, w.g.x + h * dx), W, a + h * da)
        m = _oracle_loads(*wingcase.moved(w, wake, w.g.x - h * dx), W, a - h * da)
        for i, d in enumerate((dCL[k], dCDi[k])):
            fd = (p[i] - m[i]) / (2 * h)
            assert abs(d - fd) <= 1e-6 * max(abs(fd), 1e-3), (k, i, d, fd)
