"""The GPU adjoint against the derivative oracle on the 1,356-triangle coarsening of the headline wing (AR 8, NACA
0012, 20 x 16 panels per side, ladder caps, rigid wake 2.5 spans long, alpha 5 deg; nodes moved by up to 2% of their
shortest edge). The oracle carries forward-mode dual numbers through its assembly and exact tangents through the
bordered solve and the loads, as ForwardDiff does in the reference's tests (test/kernels/test_kernels.jl:127-148).

Directions: single node coordinates drawn with seed 1 (a trailing edge node and a tip node among them), dense random
directions over every node (seed 2), and alpha. The FP64 gradients agree within 1e-7: a single coordinate relative
to max|grad|, a dense direction relative to sum |grad_i v_i|, alpha relative to its own size. The mixed gradients
are held to 1e-5 on the same scales."""
import math
import os
import sys

import numpy as np
import pytest
import wingcase

from vortexpanel_gpu import meshes
from vortexpanel_gpu.adjoint import wing_gradients

pytestmark = pytest.mark.gpu

ALPHA = math.radians(5.0)


@pytest.fixture(scope="module")
def coarse():
    w = wingcase.jittered_rel(meshes.wing(20, 16, aspect=8.0), 0.02, seed=20)
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=2.5)
    W = meshes.wake_rows(w.dm, wake.te)
    assert w.g.ntri == 1356
    return w, wake, W


@pytest.fixture(scope="module")
def dual(oracle, coarse):
    sys.path.insert(0, os.path.dirname(oracle.__file__))
    import dual_oracle

    w, wake, W = coarse
    rng = np.random.default_rng(1)
    te = int(w.dm.wake_te.node[len(w.dm.wake_te.node) // 3])
    tip = int(np.argmax(w.g.x[:, 1]))
    nodes = sorted(set(rng.choice(w.g.nnode, 8, replace=False).tolist()) | {te, tip})
    singles = [(n, int(rng.integers(3))) for n in nodes]
    dense = np.random.default_rng(2).standard_normal((5, w.g.nnode, 3))
    dirs, kinds = [], []
    for n, c in singles:
        dx = np.zeros((w.g.nnode, 3))
        dx[n, c] = 1.0
        dirs.append((dx, 0.0))
        kinds.append(("node", n, c))
    for k, v in enumerate(dense):
        dirs.append((v, 0.0))
        kinds.append(("dense", k, None))
    dirs.append((np.zeros((w.g.nnode, 3)), 1.0))
    kinds.append(("alpha", None, None))
    nd = dual_oracle.nd_max()
    CL = CDi = None
    dCL, dCDi = [], []
    for i0 in range(0, len(dirs), nd):
        CL, CDi, a, b = dual_oracle.wing_loads_tangent(w, wake, W, ALPHA, dirs[i0:i0 + nd])
        dCL += a.tolist()
        dCDi += b.tolist()
    return dirs, kinds, CL, CDi, np.array(dCL), np.array(dCDi)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_against_dual_oracle(coarse, dual, precision):
    w, wake, W = coarse
    dirs, kinds, CL, CDi, dCL, dCDi = dual
    g = wing_gradients(w, wake, W, ALPHA, precision=precision)
    tol = 1e-7 if precision == "fp64" else 1e-5
    assert abs(g["CL"] - CL) <= (1e-10 if precision == "fp64" else 1e-6)
    assert abs(g["CDi"] - CDi) <= (1e-11 if precision == "fp64" else 1e-6)
    worst = {}
    for name, ref in (("CL", dCL), ("CDi", dCDi)):
        grad = g["d" + name + "_dx"]
        scale = np.abs(grad).max()
        for (dx, da), kind, r in zip(dirs, kinds, ref):
            got = float(np.sum(grad * dx) + g["d" + name + "_dalpha"] * da)
            if kind[0] == "node":
                s = scale
            elif kind[0] == "dense":
                s = float(np.sum(np.abs(grad * dx)))
            else:
                s = abs(r)
            e = abs(got - r) / s
            worst[(name, kind[0])] = max(worst.get((name, kind[0]), 0.0), e)
            assert e <= tol, (precision, name, kind, got, r, e)
    print(f"adjoint ({precision}) vs dual oracle, worst relative error by kind:", worst)
