"""vp_assemble_batch: an uneven batch of lifting wings (different panel counts, aspect ratios and wakes, and a closed
body among them) assembled in shared launches gives every system the A, b and tier counts that vp_assemble gives it
alone with the same far tile, bit for bit, in FP64 and in mixed precision, for every far tile the library has."""
import math

import numpy as np
import pytest

from vortexpanel_gpu import _lib, api, meshes

pytestmark = pytest.mark.gpu


def _cases():
    a = math.radians(4.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    out = []
    for nc, ns, ar in ((10, 6, 4.0), (16, 10, 12.0), (6, 4, 8.0), (12, 12, 6.0)):
        w = meshes.wing(nc, ns, aspect=ar)
        wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
        els = api.build_elements(w.g)
        out.append((w.g, w.dm, api.source_strengths(els, V), V, wake))
    g, dm = meshes.sphere_case(2)
    out.append((g, dm, api.source_strengths(api.build_elements(g), V), V, None))
    return out


@pytest.mark.parametrize("precision,tile", [("fp64", 1), ("fp64", 2), ("fp64", 4), ("mixed", 2), ("mixed", 4),
                                            ("mixed", 8)])
def test_batch_equals_single_systems(precision, tile):
    cases = _cases()
    opts = api.AssemblyOptions(precision=precision)
    ctx = api.default_context()
    code = _lib.VP_MIXED if precision == "mixed" else _lib.VP_FP64
    default = _lib.load().vp_get_far_tile(ctx.h, code)
    _lib.check(ctx.h, _lib.load().vp_set_far_tile(ctx.h, code, tile))
    try:
        batch = api.assemble_batch(cases, opts=opts, tune=False)
        single = [api.assemble(g, dm, api.build_elements(g), sig, V, opts=opts, wake=wake, tune=False)
                  for g, dm, sig, V, wake in cases]
    finally:
        _lib.check(ctx.h, _lib.load().vp_set_far_tile(ctx.h, code, default))
    assert len(batch) == len(cases)
    for (g, dm, sig, V, wake), (Ab, bb, sb), (A1, b1, s1) in zip(cases, batch, single):
        assert Ab.shape == A1.shape
        assert np.array_equal(Ab.download(), A1.download()), (precision, g.ntri)
        assert np.array_equal(bb, b1)
        assert sb["pairs"] == s1["pairs"] and sb["points"] == s1["points"]
        assert sb["points_fp64"] == s1["points_fp64"]


def test_far_tiles_agree():
    """the far tier's tiles sum the same pairs in another grouping: A agrees to rounding across tiles"""
    g, dm, sig, V, wake = _cases()[1]
    ctx = api.default_context()
    for precision, tiles, tol in (("fp64", (1, 4), 1e-13), ("mixed", (2, 8), 1e-6)):
        code = _lib.VP_MIXED if precision == "mixed" else _lib.VP_FP64
        default = _lib.load().vp_get_far_tile(ctx.h, code)
        As = []
        try:
            for t in tiles:
                _lib.check(ctx.h, _lib.load().vp_set_far_tile(ctx.h, code, t))
                A, b, _ = api.assemble(g, dm, api.build_elements(g), sig, V, wake=wake, tune=False,
                                       opts=api.AssemblyOptions(precision=precision))
                As.append(A.download())
        finally:
            _lib.check(ctx.h, _lib.load().vp_set_far_tile(ctx.h, code, default))
        assert np.abs(As[0] - As[1]).max() <= tol * np.abs(As[0]).max(), precision
