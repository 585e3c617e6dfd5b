"""The angle-of-attack sweep of the lifting wing with batched right hand sides, on the GPU through the C ABI: AR 8
NACA 0012, 80 x 40 panels per side (13,116 triangles), rigid wake 2.5 spans, one factorization and 64 right hand
sides for alpha in [-4, 12] deg, CL by pressure (src/post/forces.jl:11-20) and CDi by Trefftz (forces.jl:53-81).
Against the oracle's golden values (tests/golden/make_golden.py --sweep), though the bordered matrix's condition
number is 7.7e5:
- FP64 to 1e-11 in CL and 1e-12 in CDi (measured 3.5e-14 and 2.7e-15);
- mixed precision to 1e-6 in both, the bar of the mixed path (measured 1.0e-7 and 7.6e-9)."""
import math
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import make_golden  # noqa: E402


@pytest.fixture(scope="module")
def sweep(vp):
    d = np.load(os.path.join(HERE, make_golden.SWEEP + ".npz"))
    w, wake, W, alpha = make_golden.sweep_case()
    assert np.array_equal(alpha, d["alpha"])
    els = vp.build_elements(w.g)
    S = w.span * w.chord
    out = {}
    for precision in ("fp64", "mixed"):
        opts = vp.AssemblyOptions(precision=precision)
        A, bx, _ = vp.assemble(w.g, w.dm, els, vp.source_strengths(els, [1.0, 0, 0]), [1.0, 0, 0], wake=wake,
                               opts=opts)
        _, bz, _ = vp.assemble(w.g, w.dm, els, vp.source_strengths(els, [0, 0, 1.0]), [0, 0, 1.0], wake=wake,
                               opts=opts)
        F = vp.factorize_galerkin(w.dm, A, W=W, precision=precision)
        s = vp.solve_galerkin(F, make_golden.sweep_rhs(bx, bz, alpha))
        CL, CDi = [], []
        for k, a in enumerate(alpha):
            V = np.array([math.cos(a), 0.0, math.sin(a)])
            mu = w.dm.C @ s["q"][:, k]
            cp = vp.pressure_coefficient(vp.gradient_velocity(els, w.dm, mu, V), V)
            CL.append(vp.pressure_force(els, cp)[0] @ np.array([-math.sin(a), 0.0, math.cos(a)]) / S)
            CDi.append(vp.trefftz_drag(w.dm.wake_te, w.dm.K @ s["q"][:, k], V) / S)
        out[precision] = (np.array(CL), np.array(CDi), F.cond)
        del A, F
    return d, out


@pytest.mark.parametrize("precision,tol_cl,tol_cdi", [("fp64", 1e-11, 1e-12), ("mixed", 1e-6, 1e-6)])
def test_sweep_matches_golden(sweep, precision, tol_cl, tol_cdi):
    d, out = sweep
    CL, CDi, cond = out[precision]
    dcl, dcdi = np.abs(CL - d["CL"]).max(), np.abs(CDi - d["CDi"]).max()
    print(f"{precision}: max |dCL| {dcl:.3e}, max |dCDi| {dcdi:.3e}, cond {cond:.4e} (oracle {float(d['cond']):.4e})")
    assert dcl < tol_cl
    assert dcdi < tol_cdi
    assert abs(cond / float(d["cond"]) - 1) < 0.05


def test_sweep_physics(sweep):
    # lift slope near the lifting-line value 2 pi AR / (AR + 2) = 5.03 per radian; induced drag near elliptic
    d, out = sweep
    CL, CDi, _ = out["mixed"]
    slope = np.polyfit(d["alpha"], CL, 1)[0]
    assert 4.5 < slope < 5.3
    assert np.all(np.diff(CL) > 0)
    k = np.argmin(np.abs(d["alpha"] - math.radians(8.0)))
    assert 0.95 < CDi[k] * math.pi * 8.0 / CL[k] ** 2 < 1.1
