"""surface_velocity (src/post/Post.jl:32-64) on the GPU against the oracle's restatement, on the icosphere at
subdivision 2 (body sheets and sources, the own sheet's side-1 limit) and on a small lifting wing with its rigid wake
(wake sheets and tip filaments too): FP64 within 1e-10 of the largest velocity, mixed within 1e-5."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sphere(vp, oracle):
    V = np.array([1.0, 0.3, -0.2]) / np.linalg.norm([1.0, 0.3, -0.2])
    g, dm = vp.meshes.sphere_case(2)
    sig = oracle.source_strengths(g, V)
    A, b, _ = oracle.assemble(g, dm, sig, V)
    mu = oracle.solve_galerkin(dm, A, b)["mu"]
    return g, dm, V, sig, mu, None, None


def _wing(vp, oracle):
    w = vp.meshes.wing(6, 3, aspect=4.0)
    wake = vp.meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
    W = vp.meshes.wake_rows(w.dm, wake.te)
    a = math.radians(5.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    sig = oracle.source_strengths(w.g, V)
    A, b, _ = oracle.assemble(w.g, w.dm, sig, V, wake=wake)
    q = oracle.solve_galerkin(w.dm, A, b, W=W)["q"]
    return w.g, w.dm, V, sig, w.dm.C @ q, wake, W @ q


@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_surface_velocity_matches_oracle(vp, oracle, case):
    g, dm, V, sig, mu, wake, mu_w = (_sphere if case == "sphere" else _wing)(vp, oracle)
    if wake is not None:
        assert len(wake.tris) > 0 and len(wake.filaments) > 0
    ref = oracle.surface_velocity(g, dm, sig, mu, V, wake=wake, mu_wake=mu_w)
    els = vp.build_elements(g)
    scale = np.abs(ref).max()
    for precision, tol in (("fp64", 1e-10), ("mixed", 1e-5)):
        u = vp.surface_velocity(els, dm, sig, mu, V, wake=wake, mu_wake=mu_w, precision=precision)
        err = np.abs(u - ref).max() / scale
        print(f"{case} {precision}: max |du| / max |u| {err:.3e}")
        assert err < tol


def test_surface_velocity_needs_wake_doublets(vp):
    w = vp.meshes.wing(4, 2, aspect=4.0)
    wake = vp.meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
    els = vp.build_elements(w.g)
    with pytest.raises(ValueError):
        vp.surface_velocity(els, w.dm, np.zeros(w.g.ntri), np.zeros(w.dm.nslot), [1.0, 0, 0], wake=wake)
