"""Adjoint gradients through the C ABI (vp_solve_transposed, vp_adjoint) against central finite differences of the
GPU's FP64 forward path (assemble + factorize + solve + loads), step 1e-6 chord, on a small lifting wing with its
rigid wake: dCL/dx and dCDi/dx at seeded random nodes, trailing edge and tip nodes among them, and d/dalpha."""
import math

import numpy as np
import pytest
import wingcase

from vortexpanel_gpu import api, meshes
from vortexpanel_gpu.adjoint import wing_gradients

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    w = wingcase.jittered(meshes.wing(12, 6, aspect=6.0))
    ang = wingcase.corner_angles(w.g)
    # no corner within 0.01 degrees of a switch of the vertex rule (90, and 150 for corner_angle = 75), wedges present
    assert np.abs(ang - 90).min() > 1e-2 and np.abs(ang - 150).min() > 1e-2 and (ang > 90.5).any()
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
    W = meshes.wake_rows(w.dm, wake.te)
    return w, wake, W


_moved = wingcase.moved
_loads = wingcase.loads


def _nodes(w):
    rng = np.random.default_rng(1)
    te = int(w.dm.wake_te.node[len(w.dm.wake_te.node) // 2])
    tip = int(np.argmax(w.g.x[:, 1]))
    return sorted(set(rng.choice(w.g.nnode, 6, replace=False).tolist()) | {te, tip})


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gradients_against_finite_differences(case, precision):
    w, wake, W = case
    a = math.radians(5.0)
    out = wing_gradients(w, wake, W, a, precision=precision)
    CL0, CDi0 = _loads(w, wake, W, a)
    assert abs(out["CL"] - CL0) <= 1e-6 and abs(out["CDi"] - CDi0) <= 1e-6
    h = 1e-6 * w.chord
    for name, k in (("CL", 0), ("CDi", 1)):
        grad = out["d" + name + "_dx"]
        scale = np.abs(grad).max()
        for n in _nodes(w):
            for c in range(3):
                xp, xm = w.g.x.copy(), w.g.x.copy()
                xp[n, c] += h
                xm[n, c] -= h
                fp = _loads(*_moved(w, wake, xp), W, a)[k]
                fm = _loads(*_moved(w, wake, xm), W, a)[k]
                fd = (fp - fm) / (2 * h)
                assert abs(grad[n, c] - fd) <= 1e-5 * scale, (name, precision, n, c, grad[n, c], fd, scale)
        fd = (_loads(w, wake, W, a + 1e-6)[k] - _loads(w, wake, W, a - 1e-6)[k]) / 2e-6
        da = out["d" + name + "_dalpha"]
        assert abs(da - fd) <= 1e-5 * max(abs(fd), 1e-3), (name, precision, da, fd)


def test_mixed_gradients_match_fp64(case):
    w, wake, W = case
    a = math.radians(3.0)
    g64 = wing_gradients(w, wake, W, a, precision="fp64")
    g32 = wing_gradients(w, wake, W, a, precision="mixed")
    for name in ("CL", "CDi"):
        d = g64["d" + name + "_dx"]
        assert np.abs(g32["d" + name + "_dx"] - d).max() <= 1e-5 * np.abs(d).max(), name
        assert abs(g32["d" + name + "_dalpha"] - g64["d" + name + "_dalpha"]) <= 1e-5 * abs(g64["d" + name + "_dalpha"])


def test_transposed_solve(case):
    """M' xi = g through vp_solve_transposed: xi' (M q) = g' q for the solved q of any right hand side"""
    from vortexpanel_gpu.adjoint import solve_transposed
    w, wake, W = case
    V = np.array([1.0, 0.0, 0.1])
    els = api.build_elements(w.g)
    A, b, _ = api.assemble(w.g, w.dm, els, api.source_strengths(els, V), V, wake=wake)
    for precision in ("fp64", "mixed"):
        F = api.factorize_galerkin(w.dm, A, W=W, precision=precision)
        rng = np.random.default_rng(4)
        g = rng.standard_normal(w.dm.nq)
        g -= g.mean()  # orthogonal to the body's constant mode
        xi = solve_transposed(F, g)
        q = api.solve_galerkin(F, b)["q"]
        # [g; 0]' [q; lambda] = [xi; eta]' M [q; lambda] = xi' (C' b)
        assert abs(g @ q - xi @ (w.dm.C.T @ b)) <= 1e-9 * np.abs(g).sum() * np.abs(q).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pair_derivatives_reproducible(precision):
    """The adjoint's sums scattered from many warps (test side, source side, node derivatives, d/dalpha) are
    order-independent fixed-point totals: two runs on the same input agree bit for bit. A 3k-triangle wing, so that
    each triangle's sums gather contributions from many CTAs."""
    from vortexpanel_gpu.adjoint import pair_derivatives
    w = meshes.wing(40, 20, aspect=8.0)
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=2.0)
    a = math.radians(5.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    dV = np.array([-math.sin(a), 0.0, math.cos(a)])
    els = api.build_elements(w.g)
    sig = api.source_strengths(els, V)
    rng = np.random.default_rng(7)
    nu = rng.standard_normal((w.dm.nslot, 2))
    mu = rng.standard_normal(w.dm.nslot + wake.x.shape[0])
    opts = api.AssemblyOptions(precision=precision)
    runs = [pair_derivatives(w.g, w.dm, sig, V, dV, nu, mu, opts=opts, wake=wake)[:3] for _ in range(3)]
    for r in runs[1:]:
        for x0, x1 in zip(runs[0], r):
            x0, x1 = np.asarray(x0), np.asarray(x1)
            assert np.isfinite(x0).all()
            assert np.array_equal(x0.view(np.uint64), x1.view(np.uint64))
