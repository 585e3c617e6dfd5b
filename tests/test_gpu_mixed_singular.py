"""Mixed precision on the near-singular blocks alone: the entries of A whose row and column slots share a triangle
(self, edge-touching and vertex-touching pairs, and the contact pairs at the thin trailing edge, every pair of them
evaluated with the guarded FP32 kernel or, where the guard refuses, in FP64) against the FP64 path, on a lifting wing
with its wake and on the sphere. The FP32 guard sends a point to FP64 near a source edge seen at a small angle or near
the source's plane; the bound here is what the guard is set to keep."""
import math

import numpy as np
import pytest

from vortexpanel_gpu import api, meshes

pytestmark = pytest.mark.gpu


def _neighbour_mask(dm, ncols):
    """(row slot, column slot) pairs of slots that are corners of one triangle"""
    n = dm.nslot
    M = np.zeros((n, ncols), bool)
    cs = dm.corner_slot
    for a in range(3):
        for b in range(3):
            M[cs[:, a], cs[:, b]] = True
    return M


@pytest.mark.parametrize("case", ["wing", "sphere"])
def test_near_singular_entries_mixed_vs_fp64(case):
    a = math.radians(5.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    if case == "wing":
        w = meshes.wing(24, 12, aspect=8.0)
        g, dm = w.g, w.dm
        wake = meshes.build_wake(g, dm, (1.0, 0.0, 0.0), length=1.0)
    else:
        g, dm = meshes.sphere_case(3)
        wake = None
    els = api.build_elements(g)
    sig = api.source_strengths(els, V)
    A64, b64, s64 = api.assemble(g, dm, els, sig, V, wake=wake, opts=api.AssemblyOptions(precision="fp64"))
    A32, b32, s32 = api.assemble(g, dm, els, sig, V, wake=wake, opts=api.AssemblyOptions(precision="mixed"))
    D64, D32 = A64.download(), A32.download()
    M = _neighbour_mask(dm, D64.shape[1])
    scale = np.abs(D64).max(axis=1, keepdims=True)
    rel = np.where(M, np.abs(D32 - D64) / scale, 0.0)
    print(f"{case}: near-singular entries {int(M.sum())}, largest error {rel.max():.2e} of the row's largest entry, "
          f"FP64 points {s32['points_fp64']} of {sum(s32['points'].values())}")
    assert rel.max() <= 2e-5
