"""The free wake's oracle bookkeeping (no GPU), pinned to the reference's tests: core radii and sheet vorticity
(test/freewake/test_freewake.jl:15-40), and conversion of panel rows into particles conserving the total vorticity and
its first moment (:80-98), merging conserving the total vorticity (:100-128), on wake rows built from the generated
wing with seeded doublets. The product's option checks and the core of its set-up (first particles, merged batches)
against the oracle's CoreRule."""
import math

import numpy as np
import pytest

import freewake_oracle as fw

from vortexpanel_gpu import api, meshes
from vortexpanel_gpu import freewake as pfw


def test_core_radius():
    V = np.array([1.0, 0.0, 0.0])
    o = np.zeros(3)
    auto = fw.CoreRule(fw.FreeWakeOptions(dt=0.1), V)
    for w, l in ((0.25, 0.06), (0.25, 0.006), (0.02, 0.06)):
        assert math.isclose(auto.tri(o, o + [w, 0, 0], o + [w, l, 0]), 1.5 * math.hypot(w, l) / 2, rel_tol=1e-14)
    assert math.isclose(auto.seg(o, np.array([0.2, 0, 0])), 1.5 * 0.1, rel_tol=1e-14)
    assert fw.CoreRule(fw.FreeWakeOptions(dt=0.1, core=0.05), V).seg(o, np.array([1.0, 0, 0])) == 0.05
    scaled = fw.CoreRule(fw.FreeWakeOptions(dt=0.1, core="scaled"), V)
    assert math.isclose(scaled.tri(o, np.array([0.25, 0, 0]), np.array([0.25, 0.006, 0])),
                        max(1.5 * math.sqrt(0.25 * 0.006), 0.1), rel_tol=1e-14)


def test_sheet_vorticity():
    p, q, r = np.array([0.1, 0.0, 0.2]), np.array([1.0, 0.3, -0.1]), np.array([0.4, 0.9, 0.3])
    mu = np.array([0.7, -0.2, 1.1])
    g = meshes.Geometry(np.array([p, q, r]), np.array([[0, 1, 2]], np.int32))
    els = api.build_elements(g)
    gam = sum(mu[k] * els.gam[k][0] for k in range(3))
    assert np.allclose(fw.sheet_vorticity(p, q, r, mu), gam * els.area[0], rtol=1e-14, atol=1e-15)


def test_options():
    for F in (fw.FreeWakeOptions, pfw.FreeWakeOptions):
        with pytest.raises(ValueError):
            F(dt=0.0).check()
        with pytest.raises(ValueError):
            F(dt=0.1, advection="x").check()
        with pytest.raises(ValueError):
            F(dt=0.1, core=-1.0).check()
        with pytest.raises(NotImplementedError):
            F(dt=0.1, te_direction="bisector").check()


@pytest.mark.parametrize("core", ["auto", "scaled", 0.05])
def test_product_core_of_quad_matches_oracle(core):
    V = np.array([0.9, 0.0, 0.2])
    o = np.zeros(3)
    ref = fw.CoreRule(fw.FreeWakeOptions(dt=0.02, core=core), V)
    params = pfw.core_params(pfw.FreeWakeOptions(dt=0.02, core=core), V)
    for w, l in ((0.25, 0.06), (0.02, 0.3), (0.1, 0.0)):
        assert math.isclose(pfw.core_of_quad(params, w, l), ref.tri(o, o + [w, 0, 0], o + [w, l, 0]), rel_tol=1e-15)


def test_product_topology_matches_oracle():
    w = meshes.wing(10, 6, aspect=6.0)
    a, b = fw.Topology.of(w.dm), pfw.Topology.of(w.dm)
    assert (a.nte, a.segments, a.first_nodes, a.last_nodes) == (b.nte, b.strips, b.first_nodes, b.last_nodes)


def _state(w, nrow=6, seed=3):
    """a free wake state on the rows of a rigid wake, with seeded doublets per row and a starting mu_line of zero"""
    dm = w.dm
    wake = meshes.build_wake(w.g, dm, (1.0, 0.0, 0.1), rows=0.05 * np.arange(nrow + 1))
    topo = fw.Topology.of(dm)
    n = topo.nte
    st = fw.FreeWakeState(n, len(topo.segments))
    rng = np.random.default_rng(seed)
    for j in range(nrow + 1):
        st.x.append(wake.x[j * n:(j + 1) * n].copy() + 1e-3 * rng.standard_normal((n, 3)))
        st.mu.append(np.sin(np.linspace(0.1, 3.0, n)) + 0.1 * rng.standard_normal(n))
    return st, topo


def _moments(st, topo, core):
    b = np.vstack([fw.free_wake_blobs(fw.vortex_elements(st, topo), core), st.particles])
    Om, I = fw.vorticity_moments(b)
    return Om, I, np.abs(b[:, 3:6]).sum(), (np.linalg.norm(b[:, :3], axis=1) * np.linalg.norm(b[:, 3:6], axis=1)).sum()


@pytest.mark.parametrize("tip", ["zero", "free"])
def test_conversion_conserves_vorticity_and_impulse(tip):
    w = meshes.wing(10, 6, aspect=6.0)
    st, topo = _state(w)
    core = fw.CoreRule(fw.FreeWakeOptions(dt=0.05), np.array([1.0, 0, 0]))
    Om0, I0, sO, sI = _moments(st, topo, core)
    for _ in range(3):
        fw.convert_oldest(st, topo, core)
        Om, I, _, _ = _moments(st, topo, core)
        assert np.linalg.norm(Om - Om0) < 1e-14 * sO
        assert np.linalg.norm(I - I0) < 1e-14 * sI
    assert st.conversions == 3 and len(st.x) == 4


def test_merging_conserves_vorticity():
    w = meshes.wing(10, 6, aspect=6.0)
    st, topo = _state(w, nrow=8)
    core = fw.CoreRule(fw.FreeWakeOptions(dt=0.05), np.array([1.0, 0, 0]))
    merge = [3] * len(topo.segments)
    merged = False
    for _ in range(4):
        Om0, I0, sO, _ = _moments(st, topo, core)
        pending = int((st.tag > 0).sum())
        n0 = len(st.particles)
        fw.convert_oldest(st, topo, core, merge)
        Om, I, _, _ = _moments(st, topo, core)
        assert np.linalg.norm(Om - Om0) < 1e-14 * sO
        assert np.linalg.norm(I - I0) < 2e-2 * np.linalg.norm(I0)
        if int((st.tag > 0).sum()) < pending:
            merged = True
            assert len(st.particles) < n0 + 2 * len(topo.segments) + 4
    assert merged


def test_state_checkpoint_round_trip(tmp_path):
    # the wake state through named arrays and an .npz file, then on with the same conversions as the original
    w = meshes.wing(10, 6, aspect=6.0)
    st, topo = _state(w, nrow=8)
    core = fw.CoreRule(fw.FreeWakeOptions(dt=0.05), np.array([1.0, 0, 0]))
    merge = [3] * len(topo.segments)
    fw.convert_oldest(st, topo, core, merge)
    np.savez(tmp_path / "wake.npz", **st.to_arrays())
    with np.load(tmp_path / "wake.npz") as d:
        back = fw.FreeWakeState.from_arrays({k: d[k] for k in d.files})
    for _ in range(3):
        fw.convert_oldest(st, topo, core, merge)
        fw.convert_oldest(back, topo, core, merge)
    assert len(back.x) == len(st.x) and back.conversions == st.conversions
    assert all(np.array_equal(a, b) for a, b in zip(back.x, st.x))
    assert all(np.array_equal(a, b) for a, b in zip(back.mu, st.mu))
    for k in ("particles", "mu_line", "tag", "group", "batch_rows", "batch_length", "batch_width"):
        assert np.array_equal(getattr(back, k), getattr(st, k)), k
