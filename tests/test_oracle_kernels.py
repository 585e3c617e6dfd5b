"""The oracle's kernels against independent referees, as the reference pins its own kernels
(test/kernels/test_kernels.jl, test/kernels/reference.jl, test/kernels/test_segment.jl, test/kernels/test_blob.jl):
a polar quadrature about the point's projection with analytic radial integrals (adaptive in the angle), and adaptive
cubature over the Duffy square. The referees are restated here in numpy/scipy."""
import math

import numpy as np
import pytest
from scipy.integrate import quad, quad_vec


def _rot():
    a = np.array([0.3, -0.7, 0.65])
    a /= np.linalg.norm(a)
    th = 1.1
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + math.sin(th) * K + (1 - math.cos(th)) * K @ K


ROT = _rot()
SHIFT = np.array([0.4, -1.2, 2.5])
SHAPES = {
    "equilateral": ((0.0, 0, 0), (1.0, 0, 0), (0.5, math.sqrt(3) / 2, 0)),
    "right": ((0.0, 0, 0), (1.0, 0, 0), (0.0, 1, 0)),
    "sliver": ((0.0, 0, 0), (1.0, 0, 0), (0.5, 0.01, 0)),
    "skewed": ((0.0, 0, 0), (1.0, 0, 0), (1.9, 0.08, 0)),
}


def place(p):
    return ROT @ np.asarray(p, float) + SHIFT


def tri_data(a, b, c):
    n = np.cross(b - a, c - a)
    n /= np.linalg.norm(n)
    lens = [np.linalg.norm(b - a), np.linalg.norm(c - b), np.linalg.norm(a - c)]
    nu = [np.cross(b - a, n) / lens[0], np.cross(c - b, n) / lens[1], np.cross(a - c, n) / lens[2]]
    return dict(v=(a, b, c), n=n, c=(a + b + c) / 3, diam=max(lens), nu=nu)


def ray_interval(q, e):
    lo, hi = 0.0, math.inf
    for k in range(3):
        a, b = q[k], q[(k + 1) % 3]
        t = b - a
        nu = np.array([t[1], -t[0]])
        c0, c1 = -nu @ a, nu @ e
        if abs(c1) < 1e-300:
            if c0 > 0:
                return None
        elif c1 > 0:
            hi = min(hi, -c0 / c1)
        else:
            lo = max(lo, -c0 / c1)
    return (lo, hi) if lo < hi else None


def w_polar(a, b, c, x, side=0):
    """Polar-quadrature referee of w(x) (test/kernels/reference.jl:31-62)"""
    n = np.cross(b - a, c - a)
    n /= np.linalg.norm(n)
    e1 = (b - a) / np.linalg.norm(b - a)
    e2 = np.cross(n, e1)
    z = (x - a) @ n
    size = max(np.linalg.norm(b - a), np.linalg.norm(c - b), np.linalg.norm(a - c))
    if abs(z) <= 1e-12 * size:
        z = 0.0
    p = x - z * n
    q = [np.array([(y - p) @ e1, (y - p) @ e2]) for y in (a, b, c)]
    Z = abs(z)

    def integrand(th):
        e = np.array([math.cos(th), math.sin(th)])
        iv = ray_interval(q, e)
        if iv is None:
            return np.zeros(3)
        r1, r2 = iv
        if Z > 0:
            F = lambda r: math.asinh(r / Z) - r / math.sqrt(r * r + Z * Z)  # noqa: E731
            tang = -(F(r2) - F(r1))
            normal = z * (1 / math.sqrt(r1 * r1 + Z * Z) - 1 / math.sqrt(r2 * r2 + Z * Z))
        else:
            tang = -math.log(r2) if r1 == 0 else -math.log(r2 / r1)
            normal = float(side) if r1 == 0 else 0.0
        return np.array([tang * e[0], tang * e[1], normal])

    br = sorted(set([0.0] + [math.atan2(v[1], v[0]) % (2 * math.pi) for v in q] + [2 * math.pi]))
    I = np.zeros(3)
    for k in range(len(br) - 1):
        I += quad_vec(integrand, br[k], br[k + 1], epsrel=1e-13, epsabs=0, limit=2000)[0]
    return (I[0] * e1 + I[1] * e2 + I[2] * n) / (4 * math.pi)


def w_cubature(a, b, c, x):
    """Adaptive cubature referee over the Duffy square (test/kernels/reference.jl:64-75)"""
    A2 = np.linalg.norm(np.cross(b - a, c - a))

    def inner(u):
        def f(v):
            y = a + u * (b - a) + u * v * (c - b)
            r = x - y
            return (A2 * u) * r / np.linalg.norm(r) ** 3

        return quad_vec(f, 0, 1, epsrel=1e-12, epsabs=0)[0]

    return quad_vec(inner, 0, 1, epsrel=1e-11, epsabs=0)[0] / (4 * math.pi)


def sample_points(t):
    a, b = t["v"][0], t["v"][1]
    n, h = t["n"], t["diam"]
    nu1 = t["nu"][0]
    mid = (a + b) / 2
    bis = (t["nu"][0] + t["nu"][1]) / np.linalg.norm(t["nu"][0] + t["nu"][1])
    ub = (b - a) / np.linalg.norm(b - a)
    d = ROT @ np.array([1.0, 2.0, 0.5])
    d /= np.linalg.norm(d)
    dd = nu1 + 0.4 * ub
    dd /= np.linalg.norm(dd)
    nb = n + bis
    nb /= np.linalg.norm(nb)
    return [
        ("far", t["c"] + 20 * h * d, 0), ("near above", t["c"] + 0.1 * h * n, 0),
        ("near below", t["c"] - 0.1 * h * n + 0.2 * h * ub, 0), ("very near", t["c"] + 1e-6 * h * n, 0),
        ("in-plane inside, side +1", t["c"], 1), ("in-plane inside, side -1", t["c"], -1),
        ("in-plane inside, principal value", t["c"] + 0.1 * h * ub, 0),
        ("in-plane outside", t["c"] + 2 * h * dd, 0), ("in-plane on an edge's extension", b + 0.5 * (b - a), 0),
        ("edge-adjacent above", mid + 1e-3 * h * n, 0), ("edge-adjacent, 1e-8 above", mid + 1e-8 * h * n, 0),
        ("edge-adjacent in-plane inside", mid - 1e-3 * h * nu1, 1),
        ("edge-adjacent in-plane outside", mid + 1e-3 * h * nu1, 0),
        ("vertex-adjacent above", b + 1e-3 * h * nb, 0), ("vertex-adjacent in-plane outside", b + 1e-3 * h * bis, 0),
    ]


@pytest.mark.parametrize("shape", list(SHAPES))
def test_closed_form_against_polar_quadrature(oracle, shape):
    a, b, c = (place(p) for p in SHAPES[shape])
    t = tri_data(a, b, c)
    for label, x, side in sample_points(t):
        w = oracle.source_velocity(a, b, c, x, side=side, far=math.inf)
        r = w_polar(a, b, c, x, side=side)
        rtol = 1e-7 if label == "edge-adjacent, 1e-8 above" else 1e-9
        assert np.linalg.norm(w - r) <= 1e-13 + rtol * np.linalg.norm(r), (shape, label, w, r)


@pytest.mark.parametrize("shape", list(SHAPES))
def test_closed_form_against_cubature(oracle, shape):
    a, b, c = (place(p) for p in SHAPES[shape])
    t = tri_data(a, b, c)
    n, h = t["n"], t["diam"]
    u2 = n + t["nu"][1]
    u2 /= np.linalg.norm(u2)
    u3 = n - t["nu"][2]
    u3 /= np.linalg.norm(u3)
    for x in (t["c"] + 0.5 * h * n, t["c"] - 2 * h * u2, b + 0.2 * h * u3):
        w = oracle.source_velocity(a, b, c, x, far=math.inf)
        r = w_cubature(a, b, c, x)
        assert np.linalg.norm(w - r) <= 1e-10 * np.linalg.norm(r)


@pytest.mark.parametrize("shape", list(SHAPES))
def test_limits_on_the_plane(oracle, shape):
    a, b, c = (place(p) for p in SHAPES[shape])
    t = tri_data(a, b, c)
    n = t["n"]
    up, down, pv = (oracle.source_velocity(a, b, c, t["c"], side=s) for s in (1, -1, 0))
    assert abs(up @ n - 0.5) < 1e-12 and abs(down @ n + 0.5) < 1e-12 and abs(pv @ n) < 1e-14
    assert np.allclose(up - down, n, rtol=1e-12, atol=1e-14)
    near = oracle.source_velocity(a, b, c, t["c"] + 1e-9 * t["diam"] * n)
    assert np.linalg.norm(up - near) <= 1e-6 * np.linalg.norm(near)
    assert abs(oracle.inplane_fraction(a, b, c, (a + b) / 2) - 0.5) < 1e-12
    al = math.acos((c - a) @ (b - a) / (np.linalg.norm(c - a) * np.linalg.norm(b - a)))
    assert abs(oracle.inplane_fraction(a, b, c, a) - al / (2 * math.pi)) < 1e-12
    assert abs(oracle.source_velocity(a, b, c, t["c"] + 3 * t["diam"] * t["nu"][0], side=1) @ n) < 1e-15


@pytest.mark.parametrize("shape", list(SHAPES))
def test_far_field(oracle, shape):
    a, b, c = (place(p) for p in SHAPES[shape])
    t = tri_data(a, b, c)
    for u in (np.array([1.0, 0.2, -0.3]), np.array([-0.4, 1.0, 0.9]), t["n"]):
        u = u / np.linalg.norm(u)
        x = t["c"] + 10 * t["diam"] * u
        ex = oracle.source_velocity_exact(a, b, c, x)
        assert np.linalg.norm(oracle.source_velocity_far(a, b, c, x) - ex) / np.linalg.norm(ex) < 5e-6
        x2 = t["c"] + 20 * t["diam"] * u
        ex2 = oracle.source_velocity_exact(a, b, c, x2)
        assert np.linalg.norm(oracle.source_velocity_far(a, b, c, x2) - ex2) / np.linalg.norm(ex2) < 5e-7
        assert np.array_equal(oracle.source_velocity(a, b, c, x2), oracle.source_velocity_far(a, b, c, x2))


def test_consistency_and_gauss_flux(oracle):
    a, b, c = (place(p) for p in SHAPES["skewed"])
    t = tri_data(a, b, c)
    for label, x, side in sample_points(t):
        if label == "far":
            continue
        rtol = 1e-7 if label == "edge-adjacent, 1e-8 above" else 1e-12
        w1 = oracle.source_velocity(a, c, b, x, side=-side, far=math.inf)
        w2 = oracle.source_velocity(a, b, c, x, side=side, far=math.inf)
        assert np.linalg.norm(w1 - w2) <= 1e-14 + rtol * np.linalg.norm(w2), label
    L = 1.5 * t["diam"]
    xg, wg = np.polynomial.legendre.leggauss(24)
    xg, wg = L * xg, L * wg
    flux = 0.0
    for axis in range(3):
        i, j = [k for k in range(3) if k != axis]
        for s in (-1.0, 1.0):
            for xi, wi in zip(xg, wg):
                for xj, wj in zip(xg, wg):
                    p = np.zeros(3)
                    p[axis], p[i], p[j] = s * L, xi, xj
                    flux += wi * wj * s * oracle.source_velocity(a, b, c, t["c"] + p)[axis]
    area = 0.5 * np.linalg.norm(np.cross(b - a, c - a))
    assert abs(flux - area) < 1e-10 * area
    with pytest.raises(ValueError):
        oracle.source_velocity(a, b, a + 2 * (b - a), t["c"] + t["n"])


def test_vertex_derivatives_against_fd(oracle):
    a, b, c = (place(p) for p in SHAPES["sliver"])
    t = tri_data(a, b, c)
    x0 = t["c"] + 0.3 * t["diam"] * t["n"]
    h = 1e-6
    J = np.zeros((3, 3))
    for k in range(3):
        e = np.zeros(3)
        e[k] = h
        J[:, k] = (oracle.source_velocity(a + e, b, c, x0, far=math.inf) -
                   oracle.source_velocity(a - e, b, c, x0, far=math.inf)) / (2 * h)
    # divergence and curl of w vanish off the triangle: the x-Jacobian is symmetric and traceless
    Jx = np.zeros((3, 3))
    for k in range(3):
        e = np.zeros(3)
        e[k] = h
        Jx[:, k] = (oracle.source_velocity(a, b, c, x0 + e) - oracle.source_velocity(a, b, c, x0 - e)) / (2 * h)
    assert abs(np.trace(Jx)) < 1e-6 * np.linalg.norm(Jx) and np.linalg.norm(Jx - Jx.T) < 1e-6 * np.linalg.norm(Jx)
    assert np.all(np.isfinite(J))


def test_sheet_jump(oracle):
    a, b, c = (place(p) for p in SHAPES["equilateral"])
    t = tri_data(a, b, c)
    g = 2.0 * (b - a) / np.linalg.norm(b - a) - 0.7 * t["nu"][0]
    up = np.cross(g, oracle.source_velocity(a, b, c, t["c"], side=1))
    dn = np.cross(g, oracle.source_velocity(a, b, c, t["c"], side=-1))
    assert np.allclose(up - dn, np.cross(g, t["n"]), rtol=1e-12, atol=1e-14)


def _segment_quad(a, b, x, Ga, Gb):
    e = b - a

    def f(s):
        y = a + s * e
        return (Ga * (1 - s) + Gb * s) * np.cross(e, x - y) / np.linalg.norm(x - y) ** 3

    return quad_vec(f, 0, 1, epsrel=1e-12, epsabs=0)[0] / (4 * math.pi)


def test_segment_linear_strength(oracle):
    a, b = np.array([0.2, -0.3, 0.1]), np.array([1.1, 0.4, -0.2])
    off = np.cross(b - a, [0.0, 0.0, 1.0])
    off /= np.linalg.norm(off)
    for x in (np.array([0.5, 0.8, 0.3]), np.array([-1.0, 0.2, 0.0]), (a + b) / 2 + 1e-3 * off, a + 1e-3 * off,
              np.array([30.0, -20.0, 10.0])):
        va, vb = oracle.segment_velocity(a, b, x)
        ra = _segment_quad(a, b, x, 1.0, 0.0)
        rb = _segment_quad(a, b, x, 0.0, 1.0)
        assert np.linalg.norm(va - ra) <= 1e-9 * np.linalg.norm(ra)
        assert np.linalg.norm(vb - rb) <= 1e-9 * np.linalg.norm(rb)


def test_segment_constant_strength(oracle):
    L, d = 1e4, 0.3
    va, vb = oracle.segment_velocity(np.array([-L, 0.0, 0]), np.array([L, 0.0, 0]), np.array([0.0, d, 0]))
    assert np.allclose(va + vb, [0, 0, 1 / (2 * math.pi * d)], rtol=1e-6)
    a, b = np.array([0.2, -0.3, 0.1]), np.array([1.1, 0.4, -0.2])
    assert np.linalg.norm(sum(oracle.segment_velocity(a, b, a + 2 * (b - a)))) < 1e-14
    assert not np.any(oracle.segment_velocity(a, b, (a + b) / 2)[0])


def test_blob(oracle):
    xp, al, dl = np.array([0.1, -0.2, 0.3]), np.array([0.4, 1.0, -0.7]), 0.05
    for r in (20 * dl, 100 * dl):
        u = np.array([0.3, -0.5, 0.8])
        x = xp + r * u / np.linalg.norm(u)
        pv = np.cross(al, x - xp) / (4 * math.pi * np.linalg.norm(x - xp) ** 3)
        assert np.linalg.norm(oracle.blob_velocity(x, xp, al, dl) - pv) <= 2 * (dl / r) ** 2 * np.linalg.norm(pv)
    assert not np.any(oracle.blob_velocity(xp, xp, al, dl))
