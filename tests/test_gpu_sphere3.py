"""The plain method on the unit icosphere at subdivision 3 (642 nodes, 1,280 triangles), FP64, no wake, V∞ along a
generic direction, prescribed sources σ = -n·V∞, hat test weights, default tiers, through the C ABI:
  - A, b, the pair and point counts against the oracle on the same mesh;
  - μ and Cp against the exact flow, μ = V∞·x/2 and Cp = 1 - (9/4) sin²θ, at the reference's bounds and orders
    (test/assembly/test_sphere.jl:9-55): second order in μ and first order in Cp from icosphere(2) to icosphere(3);
  - the system diagnostics on the device: row sums < 1e-12, column sums < 1e-5, b sums < 1e-12, λ < 1e-14,
    residual < 1e-12;
  - the mixed path within 1e-6 of FP64 in μ."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

V = np.array([1.0, 0.3, -0.2]) / np.linalg.norm([1.0, 0.3, -0.2])


def _solve(vp, level, precision="fp64"):
    g, dm = vp.meshes.sphere_case(level)
    els = vp.build_elements(g)
    sig = vp.source_strengths(els, V)
    A, b, st = vp.assemble(g, dm, els, sig, V, opts=vp.AssemblyOptions(precision=precision))
    s = vp.solve_galerkin(dm, A, b, precision=precision)
    node_of_slot = np.zeros(dm.nslot, int)
    node_of_slot[dm.corner_slot.ravel()] = g.tris.ravel()
    err = s["mu"] - g.x[node_of_slot] @ V / 2
    err -= np.sum(dm.slot_area * err) / np.sum(dm.slot_area)  # the null space: compared without the mean
    muL2 = math.sqrt(np.sum(dm.slot_area * err ** 2) / np.sum(dm.slot_area)) / 0.5
    cp = vp.surface_loads(els, dm, s["mu"], V)["cp"]
    c = els.centroid / np.linalg.norm(els.centroid, axis=1)[:, None]
    cpex = 1 - 9 / 4 * (1 - (c @ V) ** 2)
    cpL2 = math.sqrt(np.sum(els.area * (cp - cpex) ** 2) / np.sum(els.area))
    return dict(g=g, dm=dm, els=els, sig=sig, A=A, b=b, st=st, s=s, muL2=muL2, mumax=np.abs(err).max() / 0.5,
                cpL2=cpL2)


@pytest.fixture(scope="module")
def s2(vp):
    return _solve(vp, 2)


@pytest.fixture(scope="module")
def s3(vp):
    return _solve(vp, 3)


def test_icosphere3_matches_oracle(vp, oracle, s3):
    g, dm = s3["g"], s3["dm"]
    assert g.ntri == 1280 and g.nnode == 642
    Ao, bo, so = oracle.assemble(g, dm, s3["sig"], V)
    Ag = s3["A"].download()
    scale = np.maximum(np.abs(Ao).max(axis=1, keepdims=True), 1e-300)
    assert np.max(np.abs(Ag - Ao) / scale) < 1e-10
    assert np.max(np.abs(s3["b"] - bo)) < 1e-10 * np.abs(bo).max()
    assert s3["st"]["pairs"] == so["pairs"] and s3["st"]["points"] == so["points"]
    ref = oracle.solve_galerkin(dm, Ao, bo)
    assert np.max(np.abs(s3["s"]["q"] - ref["q"])) < 1e-10 * np.abs(ref["q"]).max()


def test_icosphere3_exact_flow(s2, s3):
    assert s2["muL2"] < 3e-3 and s2["mumax"] < 1e-2 and s2["cpL2"] < 0.025
    assert s3["muL2"] < s2["muL2"] and s3["cpL2"] < s2["cpL2"]
    assert s2["muL2"] / s3["muL2"] > 3.5  # second order
    assert s2["cpL2"] / s3["cpL2"] > 1.7  # first order


def test_icosphere3_diagnostics(vp, s3):
    c = vp.consistency(s3["dm"], s3["A"])
    assert c["rows"] < 1e-12 and c["columns"] < 1e-5 and c["rhs"] < 1e-12
    s = s3["s"]
    assert abs(s["lam"][0]) < 1e-14 and s["residual"] < 1e-12 and s["cond"] < 1e3
    st = s3["st"]
    assert st["pairs"]["self"] == 1280 and sum(st["pairs"].values()) == 1280 ** 2


def test_icosphere3_mixed(vp, s3):
    m = _solve(vp, 3, "mixed")
    assert np.max(np.abs(m["s"]["mu"] - s3["s"]["mu"])) < 1e-6 * np.abs(s3["s"]["mu"]).max()
    assert abs(m["muL2"] - s3["muL2"]) < 1e-6
