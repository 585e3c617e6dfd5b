"""The host side of surface_velocity (vortexpanel_gpu.api) on the CPU: the own sheet's side-1 limit, the wake
sheets' strengths and the filament rows around the GPU sums. The two device sums are replaced here by the oracle's
scalar kernels (the test's stand-in for the GPU, which the -m gpu tests run), and the composition must equal the
oracle's restatement of Post.surface_velocity (src/post/Post.jl:32-64) to rounding."""
import math

import numpy as np
import pytest

from vortexpanel_gpu import api, meshes


@pytest.fixture
def cpu_sums(monkeypatch, oracle):
    def sheets(ctx, precision, corners, sigma, gamma, X, kernel_far):
        U = np.zeros_like(X)
        for s in range(len(corners)):
            a, b, c = corners[s, 0:3], corners[s, 3:6], corners[s, 6:9]
            for i, x in enumerate(X):
                w = oracle.source_velocity(a, b, c, x, side=0, far=kernel_far)
                U[i] += sigma[s] * w + np.cross(gamma[s], w)
        return U

    def filaments(mode, rows, xs, m, precision="fp64", ctx=None):
        assert mode == 2
        out = np.zeros((len(rows), 10))
        for i in range(len(rows)):
            va, vb = oracle.segment_velocity(rows[i, 0:3], rows[i, 3:6], xs[i])
            out[i, 0] = rows[i, 6] * (va @ m[i]) + rows[i, 7] * (vb @ m[i])
        return out

    monkeypatch.setattr(api, "_sheet_velocity", sheets)
    monkeypatch.setattr(api, "eval_points", filaments)
    monkeypatch.setattr(api, "default_context", lambda: None)


def test_closed_body(oracle, cpu_sums):
    V = np.array([1.0, 0.3, -0.2]) / np.linalg.norm([1.0, 0.3, -0.2])
    g, dm = meshes.sphere_case(1)
    sig = oracle.source_strengths(g, V)
    mu = np.random.default_rng(3).standard_normal(dm.nslot)
    ref = oracle.surface_velocity(g, dm, sig, mu, V)
    u = api.surface_velocity(api.build_elements(g), dm, sig, mu, V)
    assert np.abs(u - ref).max() < 1e-13 * np.abs(ref).max()


def test_wing_with_wake(oracle, cpu_sums):
    w = meshes.wing(4, 2, aspect=4.0)
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)
    a = math.radians(4.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    sig = oracle.source_strengths(w.g, V)
    rng = np.random.default_rng(4)
    mu, mu_w = rng.standard_normal(w.dm.nslot), rng.standard_normal(wake.nwake)
    ref = oracle.surface_velocity(w.g, w.dm, sig, mu, V, wake=wake, mu_wake=mu_w)
    u = api.surface_velocity(api.build_elements(w.g), w.dm, sig, mu, V, wake=wake, mu_wake=mu_w)
    assert np.abs(u - ref).max() < 1e-13 * np.abs(ref).max()
    with pytest.raises(ValueError):
        api.surface_velocity(api.build_elements(w.g), w.dm, sig, mu, V, wake=wake)
