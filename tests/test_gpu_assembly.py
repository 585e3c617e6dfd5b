"""Parity of the GPU assembly (vp_assemble through the C ABI) with the CPU oracle on the same meshes.

FP64: every entry of A and b within 1e-10 of the row's largest |entry| (the oracle and the GPU round the
near-singular evaluations differently: the GPU forms the offsets to the source's corners from the test triangle's
corners, the oracle from absolute points); per-tier pair and point counts identical. VP_MIXED: A within 5e-5 of the
row scale (FP32 far and near tiers), b within 5e-5 of its scale.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _row_rel(A, B):
    s = np.maximum(np.abs(B).max(axis=1, keepdims=True), 1e-300)
    return float(np.max(np.abs(A - B) / s))


def _case_sphere(m, level=2):
    g, dm = m.sphere_case(level)
    return g, dm, None


def _case_wing(m, nc=10, ns=6):
    w = m.wing(nc, ns, aspect=4.0)
    wake = m.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
    return w.g, w.dm, wake


def _case_ellipsoid(m):
    g, dm = m.ellipsoid_case(n=5, axes=(3.0, 1.0, 1.0), jitter=0.2, slivers=(4, 0.05), seed=3)
    return g, dm, None


CASES = {"sphere2": _case_sphere, "wing": _case_wing, "ellipsoid": _case_ellipsoid}


@pytest.fixture(scope="module")
def systems(vp, oracle):
    out = {}
    m = vp.meshes
    for name, mk in CASES.items():
        g, dm, wake = mk(m)
        V = np.array([np.cos(np.radians(5)), 0.1, np.sin(np.radians(5))])
        els = vp.build_elements(g)
        sig = vp.source_strengths(els, V)
        Ao, bo, so = oracle.assemble(g, dm, sig, V, wake=wake)
        out[name] = (g, dm, wake, V, els, sig, Ao, bo, so)
    return out


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_matches_oracle(vp, systems, name):
    g, dm, wake, V, els, sig, Ao, bo, so = systems[name]
    A, b, st = vp.assemble(g, dm, els, sig, V, wake=wake)
    Ag = A.download()
    assert Ag.shape == Ao.shape
    assert _row_rel(Ag, Ao) < 1e-10
    assert np.max(np.abs(b - bo)) < 1e-10 * np.max(np.abs(bo))
    assert st["pairs"] == so["pairs"]
    assert st["points"] == so["points"]


def test_tiers_present(systems):
    # the cases exercise every tier: contact at the wake's first row and the slivers, wide corners, filaments
    seen = set()
    for name in CASES:
        so = systems[name][8]
        seen |= {k for k, v in so["pairs"].items() if v > 0}
    assert seen == {"self", "edge", "vertex", "contact", "near", "far"}


def test_deterministic(vp, systems):
    g, dm, wake, V, els, sig, *_ = systems["wing"]
    A1, b1, _ = vp.assemble(g, dm, els, sig, V, wake=wake)
    A2, b2, _ = vp.assemble(g, dm, els, sig, V, wake=wake)
    assert np.array_equal(A1.download(), A2.download()) and np.array_equal(b1, b2)


@pytest.mark.parametrize("test", ["onering", "dual"])
def test_test_weights(vp, oracle, systems, test):
    g, dm, wake, V, els, sig, *_ = systems["sphere2"]
    Ao, bo, _ = oracle.assemble(g, dm, sig, V, test=test)
    A, b, _ = vp.assemble(g, dm, els, sig, V, opts=vp.AssemblyOptions(test=test))
    assert _row_rel(A.download(), Ao) < 1e-10
    assert np.max(np.abs(b - bo)) < 1e-10 * np.max(np.abs(bo))


def test_options_match_oracle(vp, oracle, systems):
    g, dm, wake, V, els, sig, *_ = systems["sphere2"]
    kw = dict(far_ratio=8.0, near_ratio=4.0, near_depth=5, touch_levels=10, touch_order=4, kernel_far=1e300)
    Ao, bo, so = oracle.assemble(g, dm, sig, V, **kw)
    A, b, st = vp.assemble(g, dm, els, sig, V, opts=vp.AssemblyOptions(**kw))
    assert _row_rel(A.download(), Ao) < 1e-10
    assert st["points"] == so["points"]


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_close_to_fp64(vp, systems, name):
    g, dm, wake, V, els, sig, Ao, bo, so = systems[name]
    A, b, st = vp.assemble(g, dm, els, sig, V, wake=wake, opts=vp.AssemblyOptions(precision="mixed"))
    assert _row_rel(A.download(), Ao) < 5e-5
    assert np.max(np.abs(b - bo)) < 5e-5 * np.max(np.abs(bo))
    assert st["pairs"] == so["pairs"]


def test_errors(vp):
    g, dm = vp.meshes.sphere_case(1)
    els = vp.build_elements(g)
    V = np.array([1.0, 0, 0])
    with pytest.raises(ValueError):
        vp.assemble(g, dm, els, vp.source_strengths(els, V), V, opts=vp.AssemblyOptions(test="box"))
    bad = vp.meshes.Geometry(g.x.copy(), g.tris.copy())
    bad.x[bad.tris[0, 1]] = bad.x[bad.tris[0, 0]]  # collapse a triangle
    with pytest.raises(ValueError):
        vp.assemble(bad, dm, els, vp.source_strengths(els, V), V)
    with pytest.raises(ValueError):
        vp.assemble(g, dm, els, np.zeros(3), V)
