"""vp_eval_points_static, the variant of vp_eval_points for callers that cannot allocate device memory while they run
(a host whose memory sits in its own pool, a loop that cannot afford cudaMalloc's synchronisation). It stages through a
fixed device array. It is checked against vp_eval_points on the same inputs: two calls in a row with different inputs
and modes, so that nothing left in the array from one call reaches the next, and the size limit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(rng, n):
    a = rng.standard_normal((n, 3))
    b = a + rng.standard_normal((n, 3))
    c = a + rng.standard_normal((n, 3))
    tri = np.concatenate([a, b, c], axis=1)
    x = (a + b + c) / 3 + rng.uniform(0.3, 30.0, (n, 1)) * rng.standard_normal((n, 3))
    m = rng.standard_normal((n, 3))
    return tri, x, m


def test_static_matches_allocating_entry(vp):
    api = vp.api
    rng = np.random.default_rng(11)
    # first call: the full size, reverse mode (widest output); second: fewer points, velocity only, FP32
    tri, x, m = _case(rng, api.STATIC_POINTS_MAX)
    got = api.eval_points_static(1, tri, x, m, kernel_far=10.0)
    ref = api.eval_points(1, tri, x, m, kernel_far=10.0)
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
    tri2, x2, _ = _case(rng, 333)
    got2 = api.eval_points_static(0, tri2, x2, kernel_far=10.0, precision="mixed")
    ref2 = api.eval_points(0, tri2, x2, kernel_far=10.0, precision="mixed")
    assert np.allclose(got2, ref2, rtol=1e-6, atol=1e-7 * np.abs(ref2).max())
    # the filament form, a third call
    rows = np.concatenate([tri2[:, :6], rng.standard_normal((333, 2)), np.zeros((333, 1))], axis=1)
    got3 = api.eval_points_static(2, rows, x2, tri2[:, 6:9])
    ref3 = api.eval_points(2, rows, x2, tri2[:, 6:9])
    assert np.allclose(got3, ref3, rtol=1e-12, atol=1e-14 * np.abs(ref3).max())


def test_static_call_allocates_nothing(vp):
    # after a first call (which looks up the array's address), further calls leave the device's free memory as it was
    torch = pytest.importorskip("torch")
    api = vp.api
    tri, x, m = _case(np.random.default_rng(5), api.STATIC_POINTS_MAX)
    api.eval_points_static(1, tri, x, m)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for mode in (0, 1, 2, 1):
        api.eval_points_static(mode, tri, x, m)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)


def test_static_rejects_oversize_and_bad_precision(vp):
    api = vp.api
    tri, x, _ = _case(np.random.default_rng(1), api.STATIC_POINTS_MAX + 1)
    with pytest.raises(ValueError, match="above"):
        api.eval_points_static(0, tri, x)
    ctx = api.default_context()
    out = np.zeros((4, 3))
    t4, x4 = np.ascontiguousarray(tri[:4]), np.ascontiguousarray(x[:4])
    code = vp._lib.load().vp_eval_points_static(ctx.h, 0, 7, 4, t4.ctypes.data_as(vp._lib.D),
                                               x4.ctypes.data_as(vp._lib.D), None, 0, 10.0,
                                               out.ctypes.data_as(vp._lib.D))
    assert code == vp._lib.VP_ERR_ARG
