"""The timed workload against the oracle: the 25,532-triangle wing (AR 8, NACA 0012, 112 x 56 full-cosine panels per
side, ladder caps, rigid wake 2.5 spans long, alpha 5 deg), through the C ABI.

  - Row samples of A and b: the oracle assembles the rows of every slot of a set of sample triangles (trailing edge,
    tip cap, leading edge, and random ones with seed 1), complete because all of those slots' triangles are among its
    test triangles; FP64 within 1e-10 of each row's largest entry, mixed within 5e-5.
  - The solve: the oracle's LAPACK solve (dgetrf) of the GPU's FP64 A against the GPU's solve, FP64 and mixed, in q,
    and CL (pressure route) and CDi (Trefftz) from the oracle's loads against the device's.
  - The adjoint: central finite differences of the FP64 forward, step 1e-6 chord, at 32 nodes drawn with seed 1 (one
    coordinate each) and in alpha, against the FP64 and mixed gradients. The wing's nodes are first moved by up to 2%
    of their shortest edge, and the drawn nodes are among those whose corners are clear of the vertex rule's switch.
"""
import math

import numpy as np
import pytest
import wingcase

from vortexpanel_gpu import api, meshes
from vortexpanel_gpu.adjoint import wing_gradients

pytestmark = pytest.mark.gpu

ALPHA = math.radians(5.0)
V = np.array([math.cos(ALPHA), 0.0, math.sin(ALPHA)])


@pytest.fixture(scope="module")
def w25():
    w = meshes.wing(112, 56, aspect=8.0)
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=2.5)
    W = meshes.wake_rows(w.dm, wake.te)
    assert w.g.ntri == 25532
    return w, wake, W


def _sample_slots(w):
    """slots of sample triangles: nearest to the trailing edge at mid-span and at the tip, the tip cap, the leading
    edge, and 24 drawn with seed 1; and every triangle that has one of them as a corner"""
    c = w.g.x[w.g.tris].mean(axis=1)
    half = w.span / 2
    seeds = [int(np.argmin(np.linalg.norm(c - p, axis=1))) for p in
             (np.array([w.chord, 0.3, 0.0]), np.array([w.chord, half, 0.0]), np.array([0.5 * w.chord, half, 0.0]),
              np.array([0.0, -1.0, 0.0]), np.array([0.5 * w.chord, -half, 0.01]))]
    seeds += np.random.default_rng(1).choice(w.g.ntri, 24, replace=False).tolist()
    slots = np.unique(w.dm.corner_slot[seeds].ravel())
    tests = np.flatnonzero(np.isin(w.dm.corner_slot, slots).any(axis=1))
    return slots, tests


@pytest.fixture(scope="module")
def oracle_rows(oracle, w25):
    w, wake, W = w25
    slots, tests = _sample_slots(w)
    sig = oracle.source_strengths(w.g, V)
    Ao, bo, _ = oracle.assemble(w.g, w.dm, sig, V, wake=wake, tests=tests)
    return slots, Ao[slots], bo[slots]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_row_samples_match_oracle(w25, oracle_rows, precision):
    w, wake, W = w25
    slots, Ao, bo = oracle_rows
    els = api.build_elements(w.g)
    A, b, st = api.assemble(w.g, w.dm, els, api.source_strengths(els, V), V, wake=wake,
                            opts=api.AssemblyOptions(precision=precision))
    rows = np.stack([A.download_rows(int(s), int(s) + 1)[0][0] for s in slots])
    scale = np.maximum(np.abs(Ao).max(axis=1, keepdims=True), 1e-300)
    err = float(np.max(np.abs(rows - Ao) / scale))
    berr = float(np.max(np.abs(b[slots] - bo)) / np.abs(bo).max())
    tol = 1e-10 if precision == "fp64" else 5e-5
    assert err < tol and berr < tol, (precision, err, berr)
    assert len(slots) > 60 and sum(st["pairs"].values()) == w.g.ntri * (w.g.ntri + len(wake.tris) + len(wake.filaments))


@pytest.fixture(scope="module")
def oracle_solve(oracle, w25):
    """the oracle's LAPACK solve of the GPU's FP64 A, and its loads"""
    w, wake, W = w25
    els = api.build_elements(w.g)
    A, b, _ = api.assemble(w.g, w.dm, els, api.source_strengths(els, V), V, wake=wake)
    Ah = A.download()
    del A
    ref = oracle.solve_galerkin(w.dm, Ah, b, W=W)
    del Ah
    oe = oracle.elements(w.g)
    cp = oracle.pressure_coefficient(oracle.gradient_velocity(w.g, w.dm, ref["mu"], V, els=oe), V)
    S = w.span * w.chord
    eL = np.array([-math.sin(ALPHA), 0.0, math.cos(ALPHA)])
    CL = float(oracle.pressure_force(oe, cp)[0] @ eL / S)
    CDi = float(oracle.trefftz_drag(w.dm.wake_te, w.dm.K @ ref["q"], V) / S)
    return ref["q"], CL, CDi


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_and_loads_match_oracle(w25, oracle_solve, precision):
    w, wake, W = w25
    q_ref, CL_ref, CDi_ref = oracle_solve
    els = api.build_elements(w.g)
    opts = api.AssemblyOptions(precision=precision)
    A, b, _ = api.assemble(w.g, w.dm, els, api.source_strengths(els, V), V, wake=wake, opts=opts)
    s = api.solve_galerkin(api.factorize_galerkin(w.dm, A, W=W, precision=precision), b)
    CL, CDi = wingcase.loads(w, wake, W, ALPHA, precision=precision)
    qerr = float(np.max(np.abs(s["q"] - q_ref)) / np.abs(q_ref).max())
    if precision == "fp64":
        assert qerr < 1e-9 and abs(CL - CL_ref) < 1e-10 and abs(CDi - CDi_ref) < 1e-11, (qerr, CL - CL_ref, CDi - CDi_ref)
    else:
        assert qerr < 1e-5 and abs(CL - CL_ref) < 1e-6 and abs(CDi - CDi_ref) < 1e-6, (qerr, CL - CL_ref, CDi - CDi_ref)


def test_adjoint_against_finite_differences(w25):
    w, wake, W = w25
    w = wingcase.jittered_rel(w, 0.02, seed=20)
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=2.5)
    W = meshes.wake_rows(w.dm, wake.te)
    g64 = wing_gradients(w, wake, W, ALPHA, precision="fp64")
    g32 = wing_gradients(w, wake, W, ALPHA, precision="mixed")
    nodes = np.random.default_rng(1).choice(wingcase.clear_nodes(w.g), 32, replace=False)
    coords = np.random.default_rng(1).integers(0, 3, 32)
    h = 1e-6 * w.chord
    fd = {"CL": [], "CDi": []}
    for n, c in zip(nodes, coords):
        xp, xm = w.g.x.copy(), w.g.x.copy()
        xp[n, c] += h
        xm[n, c] -= h
        fp = wingcase.loads(*wingcase.moved(w, wake, xp), W, ALPHA)
        fm = wingcase.loads(*wingcase.moved(w, wake, xm), W, ALPHA)
        fd["CL"].append((fp[0] - fm[0]) / (2 * h))
        fd["CDi"].append((fp[1] - fm[1]) / (2 * h))
    fa = [(p - m) / 2e-6 for p, m in zip(wingcase.loads(w, wake, W, ALPHA + 1e-6), wingcase.loads(w, wake, W, ALPHA - 1e-6))]
    report = {}
    for k, name in enumerate(("CL", "CDi")):
        f = np.array(fd[name])
        for tag, gr in (("fp64", g64), ("mixed", g32)):
            grad = gr["d" + name + "_dx"]
            scale = np.abs(grad).max()
            e = float(np.max(np.abs(grad[nodes, coords] - f)) / scale)
            ea = abs(gr["d" + name + "_dalpha"] - fa[k]) / max(abs(fa[k]), 1e-3)
            report[(name, tag)] = (e, ea)
    print("adjoint vs FD at 25k (rel to max|grad|, rel in alpha):", report)
    for key, (e, ea) in report.items():
        assert e <= 1e-5 and ea <= 1e-5, (key, e, ea)
