"""The free wake on the GPU, modeled on the reference's tests (test/freewake/test_freewake.jl:42-76, 130-160) on the
generated wing: the trailing edge panel with the other rows as explicit elements reproduces the implicit rigid wake,
explicit_rhs equals the assembled columns times their doublets, the blob and body velocity kernels match direct
sums, an impulsive start with a prescribed wake keeps Kelvin's theorem, and the free wake stays bounded with a lift
close to the prescribed wake's."""
import dataclasses
import math

import numpy as np
import pytest

from vortexpanel_gpu import api, meshes
from vortexpanel_gpu import freewake as fw

pytestmark = pytest.mark.gpu

ALPHA = math.radians(5.0)
V = np.array([math.cos(ALPHA), 0.0, math.sin(ALPHA)])
LIFT = np.array([-math.sin(ALPHA), 0.0, math.cos(ALPHA)])


@pytest.fixture(scope="module")
def wing():
    return meshes.wing(12, 8, aspect=6.0)


def test_explicit_rows_reproduce_the_rigid_wake(wing):
    w = wing
    g, dm = w.g, w.dm
    els = api.build_elements(g)
    sig = api.source_strengths(els, V)
    wf = meshes.build_wake(g, dm, V, length=1.0)
    A, b, _ = api.assemble(g, dm, els, sig, V, wake=wf)
    ref = api.solve_galerkin(dm, A, b, W=meshes.wake_rows(dm, wf.te))
    muw = dm.K @ ref["q"]
    te = meshes.te_panel(g, dm, V, length=wf.rows[1])
    At, bt, _ = api.assemble(g, dm, els, sig, V, wake=te)
    F = api.factorize_galerkin(dm, At, W=meshes.wake_rows(dm, te.te))
    topo = fw.Topology.of(dm)
    n = topo.nte
    st = fw.FreeWakeState(n)
    for j in range(1, len(wf.rows)):
        st.x.append(wf.x[j * n:(j + 1) * n].copy())
        st.mu.append(muw.copy())
    st.mu_line = muw.copy()
    rhs = fw.explicit_rhs(g, dm, fw.vortex_elements(st, topo), np.zeros((0, 7)))
    s = api.solve_galerkin(F, bt + rhs)
    assert np.abs(dm.K @ s["q"] - muw).max() < 1e-12 * np.abs(muw).max()
    assert np.abs(s["q"] - ref["q"]).max() < 1e-12 * np.abs(ref["q"]).max()
    cols = At.download()[:, dm.nslot:] @ muw[te.te]
    e = fw.rigid_elements(te, muw)
    assert np.abs(fw.explicit_rhs(g, dm, e, np.zeros((0, 7))) + cols).max() < 1e-13 * np.abs(cols).max()


def test_blob_velocities():
    rng = np.random.default_rng(1)
    blobs = np.hstack([rng.uniform(-1, 1, (700, 3)), 1e-2 * rng.standard_normal((700, 3)), rng.uniform(0.02, 0.1, (700, 1))])
    X = rng.uniform(-1.2, 1.2, (300, 3))
    r = X[:, None, :] - blobs[None, :, :3]
    d2 = (r * r).sum(-1) + blobs[None, :, 6] ** 2
    ref = (np.cross(np.broadcast_to(blobs[None, :, 3:6], r.shape), r) / (4 * math.pi * d2 * np.sqrt(d2))[..., None]).sum(1)
    u64 = fw.blob_velocities(blobs, X)
    u32 = fw.blob_velocities(blobs, X, precision="mixed")
    scale = np.abs(ref).max()
    assert np.abs(u64 - ref).max() < 1e-13 * scale
    assert np.abs(u32 - ref).max() < 1e-5 * scale


def test_body_velocity(wing, oracle):
    g = wing.g
    rng = np.random.default_rng(2)
    sig = rng.standard_normal(g.ntri)
    gam = rng.standard_normal((g.ntri, 3))
    X = np.array([[1.3, 0.1, 0.2], [1.05, -2.0, 0.01], [3.0, 1.0, -0.5], [0.5, 0.0, 0.3], [8.0, 0.5, 1.0]])
    ref = np.zeros_like(X)
    for t, (a, b, c) in enumerate(g.x[g.tris]):
        for i, x in enumerate(X):
            wv = oracle.source_velocity(a, b, c, x, far=10.0)
            ref[i] += sig[t] * wv + np.cross(gam[t], wv)
    u64 = fw.body_velocity(g, sig, gam, X)
    u32 = fw.body_velocity(g, sig, gam, X, precision="mixed")
    scale = np.abs(ref).max()
    assert np.abs(u64 - ref).max() < 1e-12 * scale
    assert np.abs(u32 - ref).max() < 1e-5 * scale


def test_impulsive_start(wing):
    w = wing
    dt = meshes.te_panel_size(w.g, w.dm)
    S = w.span * w.chord
    sim = fw.FreeWakeSim(w.g, w.dm, V, fw.FreeWakeOptions(dt=dt, max_rows=4, advection="freestream"))
    hist = sim.run(12)
    st = sim.state
    for k in range(len(st.x) - 1):
        assert np.allclose(st.x[k + 1][3], sim.edge[3] + (k + 1) * dt * V, rtol=0, atol=1e-12)
    assert all(np.linalg.norm(r["Omega"]) < 1e-12 for r in hist)
    kj = [r["F_kj"] @ LIFT / S for r in hist]
    assert kj[0] < kj[4] < kj[8] < kj[11]
    assert len(st.particles) > 0 and st.conversions == 12 - 4
    free = fw.FreeWakeSim(w.g, w.dm, V, fw.FreeWakeOptions(dt=dt, max_rows=4))
    fh = free.run(12)
    assert all(r["umax"] < 3 * np.linalg.norm(V) for r in fh)
    assert abs((fh[-1]["F_kj"] @ LIFT / S) / kj[-1] - 1) < 0.03


def test_mixed_run_matches_fp64(wing):
    w = wing
    dt = meshes.te_panel_size(w.g, w.dm)
    runs = {}
    for prec in ("fp64", "mixed"):
        sim = fw.FreeWakeSim(w.g, w.dm, V, fw.FreeWakeOptions(dt=dt, max_rows=3),
                             assembly=api.AssemblyOptions(precision=prec))
        runs[prec] = sim.run(6)
    S = w.span * w.chord
    for a, b in zip(runs["fp64"], runs["mixed"]):
        assert abs((a["F_kj"] - b["F_kj"]) @ LIFT / S) < 1e-6
        # the pressure route's unsteady term divides the step's change of the doublets by dt
        assert abs((a["F_pressure"] - b["F_pressure"]) @ LIFT / S) < 1e-5
