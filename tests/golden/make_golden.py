"""Generates the golden fixtures of tests/golden/ with the CPU oracle (oracle/), with the reference's default
AssemblyOptions:
- the assembled A and b of the unit icosphere at subdivision 1 (non-lifting, V∞ = (1, 0.3, -0.2)/|.|) and of a small
  lifting wing (6 x 3 panels per side, AR 4) with its rigid wake;
- with --sweep, the angle-of-attack sweep of the lifting wing with batched right hand sides: AR 8 NACA 0012,
  80 x 40 panels per side, rigid wake 2.5 spans along +x, one LAPACK factorization and 64 right hand sides for alpha
  uniformly in [-4, 12] deg (b is linear in V∞: b(alpha) = cos(alpha) b_x + sin(alpha) b_z), CL by pressure and CDi
  by Trefftz (about a minute on 8 cores).
The reference itself (Julia) cannot run here; the fixtures pin the GPU path and later oracle builds to these values.

    python tests/golden/make_golden.py [--sweep]
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "vortexpanel.jl_gb300"), os.path.join(ROOT, "oracle")]

import oracle  # noqa: E402
from vortexpanel_gpu import meshes  # noqa: E402


def cases():
    V = np.array([1.0, 0.3, -0.2])
    V /= np.linalg.norm(V)
    g, dm = meshes.sphere_case(1)
    yield "icosphere1", g, dm, V, None
    w = meshes.wing(6, 3, aspect=4.0)
    a = math.radians(5.0)
    Vw = np.array([math.cos(a), 0.0, math.sin(a)])
    yield "wing6x3", w.g, w.dm, Vw, meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)


SWEEP = "wing80x40_alpha_sweep"


def sweep_case():
    """the wing, its rigid wake and wake rows, and the 64 angles of attack (radians) of the sweep"""
    w = meshes.wing(80, 40, aspect=8.0)
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=2.5)
    return w, wake, meshes.wake_rows(w.dm, wake.te), np.radians(np.linspace(-4.0, 12.0, 64))


def sweep_rhs(bx, bz, alpha):
    """the right hand sides of every angle (columns) from those of V∞ = x and V∞ = z"""
    return np.cos(alpha)[None, :] * bx[:, None] + np.sin(alpha)[None, :] * bz[:, None]


def sweep():
    w, wake, W, alpha = sweep_case()
    A, bx, _ = oracle.assemble(w.g, w.dm, oracle.source_strengths(w.g, [1.0, 0, 0]), [1.0, 0, 0], wake=wake)
    _, bz, _ = oracle.assemble(w.g, w.dm, oracle.source_strengths(w.g, [0, 0, 1.0]), [0, 0, 1.0], wake=wake)
    F = oracle.factorize_galerkin(w.dm, A, W)
    B = sweep_rhs(bx, bz, alpha)
    els = oracle.elements(w.g)
    S = w.span * w.chord
    CL, CDi = [], []
    for k, a in enumerate(alpha):
        s = oracle.solve_factored(F, B[:, k])
        V = np.array([math.cos(a), 0.0, math.sin(a)])
        cp = oracle.pressure_coefficient(oracle.gradient_velocity(w.g, w.dm, s["mu"], V, els), V)
        CL.append(oracle.pressure_force(els, cp)[0] @ np.array([-math.sin(a), 0.0, math.cos(a)]) / S)
        CDi.append(oracle.trefftz_drag(w.dm.wake_te, w.dm.K @ s["q"], V) / S)
    np.savez_compressed(os.path.join(HERE, SWEEP + ".npz"), alpha=alpha, CL=np.array(CL), CDi=np.array(CDi),
                        cond=F.cond)
    print(SWEEP, w.g.ntri, "triangles, cond", F.cond)


def main():
    oracle.build()
    if "--sweep" in sys.argv:
        sweep()
        return
    for name, g, dm, V, wake in cases():
        sig = oracle.source_strengths(g, V)
        A, b, _ = oracle.assemble(g, dm, sig, V, wake=wake)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), A=A, b=b, V=V)
        print(name, A.shape)


if __name__ == "__main__":
    main()
