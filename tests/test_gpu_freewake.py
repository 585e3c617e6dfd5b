"""The free wake on the GPU, modeled on the reference's tests (test/freewake/test_freewake.jl:42-76, 130-160) on the
generated wing, and the device-resident FreeWakeSim against the oracle's FreeWakeSim (the reference's bookkeeping in
numpy with the oracle's kernels) step for step:
  - the trailing edge panel with the other rows as explicit elements reproduces the implicit rigid wake, and
    explicit_rhs equals the assembled columns times their doublets;
  - the blob and body velocity kernels match direct sums;
  - every record (loads, moments, counts) and the state (node rows, particles) match the oracle's after 10 steps in
    FP64 within 1e-9 of their scale, with conversion, merging (merge_rows = 2) and deletion, for each core rule;
  - an impulsive start with a prescribed wake keeps Kelvin's theorem; a free wake stays bounded with a lift close to
    the prescribed wake's; the mixed run stays within 1e-6 of FP64; a checkpoint continues bit-identically."""
import math

import freewake_oracle as OF
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


def _sources(e, blobs):
    """the oracle's WakeElements as the product's ExplicitSources"""
    return fw.ExplicitSources(np.array([np.concatenate(t) for t in e.sheets]).reshape(-1, 9),
                              np.array(e.sheet_mu, float).reshape(-1, 3),
                              np.array([np.concatenate(s) for s in e.segments]).reshape(-1, 6),
                              np.array(e.segment_g, float).reshape(-1, 2), np.asarray(blobs, float).reshape(-1, 7))


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
    topo = OF.Topology.of(dm)
    n = topo.nte
    st = OF.FreeWakeState(n)
    for j in range(1, len(wf.rows)):
        st.x.append(wf.x[j * n:(j + 1) * n].copy())
        st.mu.append(muw.copy())
    st.mu_line = muw.copy()
    rhs = fw.explicit_rhs(g, dm, _sources(OF.vortex_elements(st, topo), np.zeros((0, 7))))
    s = api.solve_galerkin(F, bt + rhs)
    assert np.abs(dm.K @ s["q"] - muw).max() < 1e-12 * np.abs(muw).max()
    assert np.abs(s["q"] - ref["q"]).max() < 1e-12 * np.abs(ref["q"]).max()
    cols = At.download()[:, dm.nslot:] @ muw[te.te]
    e = OF.rigid_elements(te, muw)
    assert np.abs(fw.explicit_rhs(g, dm, _sources(e, np.zeros((0, 7)))) + cols).max() < 1e-13 * np.abs(cols).max()


def test_explicit_rhs_matches_oracle(wing, oracle):
    # sheets, filaments and particles (near ones among them) against the oracle's explicit_rhs
    w = wing
    topo = OF.Topology.of(w.dm)
    wf = meshes.build_wake(w.g, w.dm, V, rows=0.04 * np.arange(6))
    n = topo.nte
    st = OF.FreeWakeState(n)
    rng = np.random.default_rng(5)
    for j in range(6):
        st.x.append(wf.x[j * n:(j + 1) * n] + 1e-3 * rng.standard_normal((n, 3)))
        st.mu.append(np.sin(np.linspace(0.2, 3.0, n)) + 0.05 * rng.standard_normal(n))
    e = OF.vortex_elements(st, topo)
    blobs = np.hstack([rng.uniform([0.9, -3, -0.3], [3.0, 3, 0.3], (300, 3)), 1e-2 * rng.standard_normal((300, 3)),
                       np.full((300, 1), 0.05)])
    ref = OF.explicit_rhs(w.g, w.dm, e, blobs)
    for prec, tol in (("fp64", 1e-10), ("mixed", 2e-6)):
        got = fw.explicit_rhs(w.g, w.dm, _sources(e, blobs), opts=api.AssemblyOptions(precision=prec))
        assert np.abs(got - ref).max() < tol * np.abs(ref).max(), prec


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
    ref = OF.body_velocity(g, sig, gam, X)
    u64 = fw.body_velocity(g, sig, gam, X)
    u32 = fw.body_velocity(g, sig, gam, X, precision="mixed")
    scale = np.abs(ref).max()
    assert np.abs(u64 - ref).max() < 1e-12 * scale
    assert np.abs(u32 - ref).max() < 1e-5 * scale


CASES = {
    "auto": dict(max_rows=3),
    "merge_delete": dict(max_rows=2, merge_rows=2, delete_beyond=0.12),
    "scaled": dict(max_rows=3, core="scaled", merge_rows="auto"),
    "fixed": dict(max_rows=2, core=0.05),
}


@pytest.mark.parametrize("case", list(CASES))
def test_device_sim_matches_oracle(wing, oracle, case):
    w = wing
    dt = meshes.te_panel_size(w.g, w.dm)
    kw = CASES[case]
    sim = fw.FreeWakeSim(w.g, w.dm, V, fw.FreeWakeOptions(dt=dt, **kw), capacity=64)  # grows as it goes
    ref = OF.FreeWakeSim(w.g, w.dm, V, OF.FreeWakeOptions(dt=dt, **kw))
    assert sim.keep_rows == ref.keep_rows and sim.merge == ref.merge
    for _ in range(10):
        a, b = sim.step(), ref.step()
        assert (a["n"], a["rows"], a["particles"]) == (b["n"], b["rows"], b["particles"]), (case, a["n"])
        for k in ("F_pressure", "M_pressure", "F_kj", "Omega", "I", "mu_w"):
            s = max(np.abs(b[k]).max(), 1e-3)
            assert np.abs(a[k] - b[k]).max() < 1e-9 * s, (case, a["n"], k, a[k], b[k])
        if a["n"] > 0:
            assert np.abs(a["F_impulse"] - b["F_impulse"]).max() < 1e-7 * max(np.abs(b["F_impulse"]).max(), 1e-3)
        assert abs(a["lam"] - b["lam"]) < 1e-12 and abs(a["umax"] - b["umax"]) < 1e-9 * b["umax"]
    st, so = sim.state, ref.state
    assert len(st.x) == len(so.x) and st.conversions == so.conversions
    assert np.abs(np.array(st.x) - np.array(so.x)).max() < 1e-11
    assert np.abs(st.particles - so.particles).max() < 1e-10 * max(1.0, np.abs(so.particles).max())
    assert np.array_equal(st.tag, so.tag) and np.array_equal(st.group, so.group)
    assert np.array_equal(st.batch_rows, so.batch_rows)
    assert np.abs(sim.cp - ref.cp).max() < 1e-9 * np.abs(ref.cp).max()
    if case == "merge_delete":  # the deletion limit removed particles: the downstream ones are gone
        d = V / np.linalg.norm(V)
        assert so.conversions > 0 and (so.particles[:, :3] @ d).max() <= (sim.edge @ d).max() + 0.12 * sim.te.span


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


def test_checkpoint_restore_continues(wing, tmp_path):
    w = wing
    dt = meshes.te_panel_size(w.g, w.dm)
    opts = fw.FreeWakeOptions(dt=dt, max_rows=2, merge_rows=2)
    a = fw.FreeWakeSim(w.g, w.dm, V, opts)
    a.run(5)
    ck = a.checkpoint()
    np.savez(tmp_path / "wake.npz", **ck["state"])
    tail = [a.step() for _ in range(3)]
    b = fw.FreeWakeSim(w.g, w.dm, V, opts)
    with np.load(tmp_path / "wake.npz") as d:
        b.restore({"state": {k: d[k] for k in d.files}, "history": ck["history"]})
    assert b.n == 5 and len(b.history) == 5
    for ra in tail:
        rb = b.step()
        for k in ("F_pressure", "F_kj", "F_impulse", "Omega", "I", "mu_w"):
            assert np.array_equal(ra[k], rb[k]), k
        assert (ra["rows"], ra["particles"]) == (rb["rows"], rb["particles"])
    with pytest.raises(ValueError):
        bad = dict(ck["state"])
        bad["mu"] = np.zeros(w.dm.nslot + 1)
        b.restore({"state": bad, "history": []})
