"""The device kernels at single points (vp_eval_points through the C ABI) against the oracle: the source-triangle
velocity in FP64 and FP32 (the reference's own sample points, test/kernels/test_kernels.jl:20-44, and its FP32 test
rtol 1e-4, :141-147), and the reverse-mode derivatives of the adjoint against central finite differences of the
oracle's FP64 kernel (the reference checks its vertex derivatives against finite differences to 1e-7, :135-140)."""
import math

import numpy as np
import pytest

from test_oracle_kernels import SHAPES, place, sample_points, tri_data

pytestmark = pytest.mark.gpu


def _points():
    tris, xs, sides, labels = [], [], [], []
    for name, abc in SHAPES.items():
        a, b, c = (place(p) for p in abc)
        t = tri_data(a, b, c)
        for label, x, side in sample_points(t):
            tris.append(np.concatenate([a, b, c]))
            xs.append(x)
            sides.append(side)
            labels.append((name, label))
    return np.array(tris), np.array(xs), sides, labels


def test_velocity_fp64_and_fp32(vp, oracle):
    tris, xs, sides, labels = _points()
    for side in (-1, 0, 1):
        idx = [i for i, s in enumerate(sides) if s == side]
        w = vp.api.eval_points(0, tris[idx], xs[idx], side=side, kernel_far=math.inf)
        w32 = vp.api.eval_points(0, tris[idx], xs[idx], side=side, kernel_far=10.0, precision="mixed")
        for j, i in enumerate(idx):
            t = tris[i].reshape(3, 3)
            ref = oracle.source_velocity(t[0], t[1], t[2], xs[i], side=side, far=math.inf)
            name, label = labels[i]
            rtol = 1e-7 if "1e-8" in label else 1e-11
            assert np.linalg.norm(w[j] - ref) <= 1e-13 + rtol * np.linalg.norm(ref), (name, label, w[j], ref)
            # FP32 on the same rounded input, away from the log-singular edges and corners
            if label in ("far", "near above", "near below", "in-plane outside"):
                ref10 = oracle.source_velocity(t[0], t[1], t[2], xs[i], side=side, far=10.0)
                assert np.linalg.norm(w32[j] - ref10) <= 1e-4 * np.linalg.norm(ref10), (name, label)


def test_far_field_switch(vp, oracle):
    tris, xs, sides, labels = _points()
    idx = [i for i, l in enumerate(labels) if l[1] == "far"]
    w = vp.api.eval_points(0, tris[idx], xs[idx], kernel_far=10.0)
    for j, i in enumerate(idx):
        t = tris[i].reshape(3, 3)
        ref = oracle.source_velocity(t[0], t[1], t[2], xs[i], far=10.0)
        assert np.linalg.norm(w[j] - ref) <= 1e-13 * np.linalg.norm(ref)


def _s(oracle, t, x, m, far):
    return oracle.source_velocity(t[0], t[1], t[2], x, far=far) @ m


@pytest.mark.parametrize("far", [math.inf, 10.0])
def test_reverse_mode_against_fd(vp, oracle, far):
    rng = np.random.default_rng(3)
    tris, xs, ms = [], [], []
    for name, abc in SHAPES.items():
        a, b, c = (place(p) for p in abc)
        t = tri_data(a, b, c)
        for dist in (0.3, 1.5, 15.0, 40.0):
            u = rng.standard_normal(3)
            u /= np.linalg.norm(u)
            tris.append(np.concatenate([a, b, c]))
            xs.append(t["c"] + dist * t["diam"] * u + 0.05 * t["diam"] * t["n"])
            ms.append(rng.standard_normal(3))
    tris, xs, ms = np.array(tris), np.array(xs), np.array(ms)
    out = vp.api.eval_points(1, tris, xs, ms, kernel_far=far)
    for i in range(len(xs)):
        t = tris[i].reshape(3, 3)
        s = _s(oracle, t, xs[i], ms[i], far)
        # the exact form loses digits to cancellation far from the triangle (about 1e-12 relative at 40 diameters)
        assert abs(out[i, 0] - s) <= (1e-10 if far == math.inf else 1e-12) * (abs(s) + 1e-300)
        if far == math.inf and i % 4 >= 2:
            # the exact form 15 and 40 diameters away: its rounding (about 1e-13 of |w||m| for the sliver) over the
            # FD step is above the tolerance; the multipole form (far = 10) is the one used there
            continue
        h = 1e-6 * np.linalg.norm(t[1] - t[0])
        scale = max(np.abs(out[i, 1:]).max(), 1e-300)
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            fd = (_s(oracle, t, xs[i] + e, ms[i], far) - _s(oracle, t, xs[i] - e, ms[i], far)) / (2 * h)
            assert abs(out[i, 1 + k] - fd) <= 1e-5 * scale, ("x", i, k, out[i, 1 + k], fd)
        for a in range(3):
            for k in range(3):
                tp, tm = t.copy(), t.copy()
                tp[a, k] += h
                tm[a, k] -= h
                # the multipole switch is kept where the central point has it
                fd = (_s(oracle, tp, xs[i], ms[i], far) - _s(oracle, tm, xs[i], ms[i], far)) / (2 * h)
                assert abs(out[i, 4 + 3 * a + k] - fd) <= 1e-5 * scale, ("v", i, a, k, out[i, 4 + 3 * a + k], fd)


def test_filament_reverse_mode(vp, oracle):
    rng = np.random.default_rng(5)
    a, b = np.array([0.2, -0.3, 0.1]), np.array([1.1, 0.4, -0.2])
    rows, xs, ns = [], [], []
    for x in (np.array([0.5, 0.8, 0.3]), np.array([-1.0, 0.2, 0.0]), np.array([3.0, -2.0, 1.0]),
              (a + b) / 2 + np.array([0.0, 0.0, 0.05])):
        ca, cb = rng.standard_normal(2)
        rows.append(np.concatenate([a, b, [ca, cb, 0.0]]))
        xs.append(x)
        ns.append(rng.standard_normal(3))
    rows, xs, ns = np.array(rows), np.array(xs), np.array(ns)
    out = vp.api.eval_points(2, rows, xs, ns)

    def s(aa, bb, x, ca, cb, n):
        va, vb = oracle.segment_velocity(aa, bb, x)
        return ca * (va @ n) + cb * (vb @ n)

    h = 1e-6
    for i in range(len(xs)):
        ca, cb = rows[i, 6], rows[i, 7]
        s0 = s(a, b, xs[i], ca, cb, ns[i])
        assert abs(out[i, 0] - s0) <= 1e-12 * abs(s0)
        scale = np.abs(out[i, 1:]).max()
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            assert abs(out[i, 1 + k] - (s(a, b, xs[i] + e, ca, cb, ns[i]) - s(a, b, xs[i] - e, ca, cb, ns[i])) / (2 * h)) \
                <= 1e-5 * scale
            assert abs(out[i, 4 + k] - (s(a + e, b, xs[i], ca, cb, ns[i]) - s(a - e, b, xs[i], ca, cb, ns[i])) / (2 * h)) \
                <= 1e-5 * scale
            assert abs(out[i, 7 + k] - (s(a, b + e, xs[i], ca, cb, ns[i]) - s(a, b - e, xs[i], ca, cb, ns[i])) / (2 * h)) \
                <= 1e-5 * scale
