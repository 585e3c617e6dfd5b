"""Ellipsoids in uniform flow against the exact solution (the reference's test/assembly/test_ellipsoid.jl and
validation/common/exact_flows.jl), through the C ABI, in FP64 and in mixed precision.

- The reference's triaxial body on a scaled cube_sphere(6): μ error below its bound 5e-3 (test_ellipsoid.jl:66), and
  the GPU's μ equal to the oracle's on the same mesh (FP64 1e-10, mixed 1e-6 of the doublet scale).
- The 3:1:1 ellipsoid of the mixed-precision workload, cube_sphere(32) with jitter 0.2 and 10 slivers (12,288
  triangles), at 5° incidence: mixed and FP64 agree in μ (1e-5 of the doublet scale) and in Cp, and both meet the
  exact flow as the oracle does on this mesh (μ L2 1.70e-4, Cp L2 7.0e-3; bounds 2e-4 and 7.5e-3).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VE = np.array([1.0, 0.3, -0.2]) / np.linalg.norm([1.0, 0.3, -0.2])


def _solve(vp, g, dm, V, precision):
    els = vp.build_elements(g)
    sig = vp.source_strengths(els, V)
    A, b, stats = vp.assemble(g, dm, els, sig, V, opts=vp.AssemblyOptions(precision=precision))
    s = vp.solve_galerkin(dm, A, b, precision=precision)
    cp = vp.pressure_coefficient(vp.gradient_velocity(els, dm, s["mu"], V), V)
    return s, cp, els


def _errors(flow, g, dm, mu, cp, centroid, area):
    """μ L2 error over the slots without the mean (the closed body's null space) / the doublet scale; Cp L2 error
    at the centroids (test_ellipsoid.jl:21-26)"""
    err = mu - flow.exact_doublet(g.x)
    err = err - np.sum(dm.slot_area * err) / np.sum(dm.slot_area)
    muL2 = math.sqrt(np.sum(dm.slot_area * err ** 2) / np.sum(dm.slot_area)) / flow.doublet_scale()
    cpe = cp - flow.exact_cp(centroid)
    return muL2, math.sqrt(np.sum(area * cpe ** 2) / np.sum(area))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_triaxial_against_exact_flow_and_oracle(vp, oracle, precision):
    m = vp.meshes
    X, F = m.cube_sphere(6, split=False)
    X, F = m.scale_nodes((X, F), (2.0, 1.0, 0.5))
    g = m.Geometry(X, m.split_quads(X, F), name="triaxial cube_sphere(6)")
    dm = m.closed_body_dofmap(g)
    flow = oracle.EllipsoidFlow((2.0, 1.0, 0.5), VE)
    s, cp, els = _solve(vp, g, dm, VE, precision)
    oels = oracle.elements(g)
    muL2, _ = _errors(flow, g, dm, s["mu"], cp, oels["centroid"], oels["area"])
    print(f"triaxial cube_sphere(6) {precision}: mu L2 error {muL2:.4e}, cond {s['cond']:.1f}")
    assert muL2 < 5e-3
    A, b, _ = oracle.assemble(g, dm, oracle.source_strengths(g, VE), VE)
    ref = oracle.solve_galerkin(dm, A, b)
    d = ref["mu"] - s["mu"]
    d -= np.sum(dm.slot_area * d) / np.sum(dm.slot_area)
    print(f"triaxial {precision} vs oracle: max |dmu| / scale {np.max(np.abs(d)) / flow.doublet_scale():.3e}")
    assert np.max(np.abs(d)) < (1e-10 if precision == "fp64" else 1e-6) * flow.doublet_scale()
    assert s["cond"] < 1e3


@pytest.fixture(scope="module")
def ellipsoid311(vp, oracle):
    g, dm = vp.meshes.ellipsoid_case(32)
    a = math.radians(5.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    flow = oracle.EllipsoidFlow((3.0, 1.0, 1.0), V)
    oels = oracle.elements(g)
    out = {}
    for precision in ("fp64", "mixed"):
        s, cp, _ = _solve(vp, g, dm, V, precision)
        out[precision] = (s, cp, _errors(flow, g, dm, s["mu"], cp, oels["centroid"], oels["area"]))
    return g, dm, flow, out


def test_mixed_ellipsoid_matches_fp64(ellipsoid311):
    g, dm, flow, out = ellipsoid311
    (s64, cp64, _), (s32, cp32, _) = out["fp64"], out["mixed"]
    d = s32["mu"] - s64["mu"]
    d -= np.sum(dm.slot_area * d) / np.sum(dm.slot_area)
    print(f"ellipsoid 3:1:1 mixed vs FP64: max |dmu| / scale {np.max(np.abs(d)) / flow.doublet_scale():.3e}, "
          f"max |dCp| {np.max(np.abs(cp32 - cp64)):.3e}; mu, Cp L2 errors: FP64 {out['fp64'][2]}, mixed {out['mixed'][2]}")
    assert g.ntri == 12288
    assert np.max(np.abs(d)) < 1e-5 * flow.doublet_scale()
    assert np.max(np.abs(cp32 - cp64)) < 1e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ellipsoid_against_exact_flow(ellipsoid311, precision):
    _, _, _, out = ellipsoid311
    s, _, (muL2, cpL2) = out[precision]
    assert muL2 < 2e-4
    assert cpL2 < 7.5e-3
    assert s["residual"] < 1e-12
