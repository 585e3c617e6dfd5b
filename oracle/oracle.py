"""Python face of the CPU oracle. TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
bench's CPU-baseline leg, never by the product path.

The pair integrals and the assembly loop are the C++ restatement in vp_oracle.cpp. The dense linear algebra is the
reference's own third-party boundary, LAPACK (src/assembly/solve.jl:54-55 calls ``lu`` = dgetrf and
``LAPACK.gecon!``), reached here through scipy's LAPACK bindings; the DOF-map reduction (src/dofmap/system.jl), the
bordered system (src/assembly/solve.jl:15-115), the loads (src/post/Post.jl:19-23,72-84, src/post/forces.jl:11-81) and
the exact ellipsoid flow (validation/common/exact_flows.jl) are restated below in numpy.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libvp_oracle.so")
TIERS = ("self", "edge", "vertex", "contact", "near", "far")

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the C++ restatement (g++, OpenMP) into oracle/_build/libvp_oracle.so"""
    src = os.path.join(HERE, "vp_oracle.cpp")
    hdrs = [os.path.join(HERE, h) for h in ("vp_oracle.hpp", "vp_dual.hpp")]
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(map(os.path.getmtime, [src] + hdrs)):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


class _Opts(ctypes.Structure):
    _fields_ = [("test", ctypes.c_int), ("far_ratio", ctypes.c_double), ("far_points", ctypes.c_int),
                ("near_points", ctypes.c_int), ("near_ratio", ctypes.c_double), ("near_depth", ctypes.c_int),
                ("touch_levels", ctypes.c_int), ("touch_ratio", ctypes.c_double), ("touch_order", ctypes.c_int),
                ("corner_angle", ctypes.c_double), ("contact_rel", ctypes.c_double), ("kernel_far", ctypes.c_double)]


DEFAULTS = dict(test="hat", far_ratio=3.0, far_points=3, near_points=7, near_ratio=1.5, near_depth=3, touch_levels=6,
                touch_ratio=0.15, touch_order=3, corner_angle=75.0, contact_rel=0.1, kernel_far=10.0)
_TEST = {"hat": 0, "onering": 1, "dual": 2}


def options(**kw) -> _Opts:
    d = dict(DEFAULTS)
    d.update(kw)
    if d["test"] not in _TEST:
        raise ValueError(f"test must be hat, onering or dual, not {d['test']}")
    o = _Opts()
    for k, _ in _Opts._fields_:
        setattr(o, k, _TEST[d[k]] if k == "test" else d[k])
    return o


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
            D = ctypes.POINTER(ctypes.c_double)
            I = ctypes.POINTER(ctypes.c_int)
            L = ctypes.POINTER(ctypes.c_longlong)
            _lib.vpo_source_velocity.argtypes = [D, D, ctypes.c_int, ctypes.c_double, ctypes.c_double, D]
            _lib.vpo_source_velocity_parts.argtypes = [D, D, ctypes.c_int, D]
            _lib.vpo_inplane_fraction.argtypes = [D, D, ctypes.c_double]
            _lib.vpo_inplane_fraction.restype = ctypes.c_double
            _lib.vpo_segment_velocity.argtypes = [D, D, D, D, D]
            _lib.vpo_blob_velocity.argtypes = [D, D, D, ctypes.c_double, D]
            _lib.vpo_rule.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_int, D, D, ctypes.c_int]
            _lib.vpo_rule1d.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, D, D,
                                        ctypes.c_int]
            _lib.vpo_pair_rule.argtypes = [ctypes.POINTER(_Opts), D, D, I, ctypes.c_int, ctypes.c_int, ctypes.c_int, D,
                                           D, ctypes.c_int, I]
            _lib.vpo_pair_block.argtypes = [D, D, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, D, D]
            _lib.vpo_assemble.argtypes = [ctypes.POINTER(_Opts), ctypes.c_int, D, ctypes.c_int, I, I, ctypes.c_int,
                                          ctypes.c_int, I, D, D, ctypes.c_int, D, ctypes.c_int, I, ctypes.c_int, I,
                                          ctypes.c_int, ctypes.c_int, D, D, L, L, ctypes.c_int]
            _lib.vpo_assemble_list.argtypes = [ctypes.POINTER(_Opts), ctypes.c_int, D, ctypes.c_int, I, I, ctypes.c_int,
                                               ctypes.c_int, I, D, D, ctypes.c_int, D, ctypes.c_int, I, ctypes.c_int, I,
                                               ctypes.c_int, I, D, D, L, L, ctypes.c_int]
        return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


# ---- kernels -------------------------------------------------------------------------------------------------------

def source_velocity(a, b, c, x, side=0, far=10.0, plane_tol=1e-12):
    abc, pa = _d(np.concatenate([a, b, c]))
    xx, px = _d(x)
    w, pw = _d(np.zeros(3))
    if lib().vpo_source_velocity(pa, px, side, far, plane_tol, pw) != 0:
        raise ValueError("degenerate triangle")
    return w


def source_velocity_exact(a, b, c, x):
    abc, pa = _d(np.concatenate([a, b, c]))
    xx, px = _d(x)
    w, pw = _d(np.zeros(3))
    lib().vpo_source_velocity_parts(pa, px, 0, pw)
    return w


def source_velocity_far(a, b, c, x):
    abc, pa = _d(np.concatenate([a, b, c]))
    xx, px = _d(x)
    w, pw = _d(np.zeros(3))
    lib().vpo_source_velocity_parts(pa, px, 1, pw)
    return w


def inplane_fraction(a, b, c, x, tol=1e-12):
    abc, pa = _d(np.concatenate([a, b, c]))
    xx, px = _d(x)
    return lib().vpo_inplane_fraction(pa, px, tol)


def segment_velocity(a, b, x):
    A, pa = _d(a)
    B, pb = _d(b)
    X, px = _d(x)
    va, pva = _d(np.zeros(3))
    vb, pvb = _d(np.zeros(3))
    lib().vpo_segment_velocity(pa, pb, px, pva, pvb)
    return va, vb


def blob_velocity(x, xp, al, delta):
    X, px = _d(x)
    P, pp = _d(xp)
    A, pa = _d(al)
    u, pu = _d(np.zeros(3))
    lib().vpo_blob_velocity(px, pp, pa, float(delta), pu)
    return u


# ---- rules ---------------------------------------------------------------------------------------------------------

def rule(kind, n=0, levels=6, ratio=0.15, order=3, k=0):
    """kind: 'triangle' (n points), 'edge', 'vertex', 'self'; k rotates corner 0 to corner k"""
    kid = {"triangle": 0, "edge": 1, "vertex": 2, "self": 3}[kind]
    m = lib().vpo_rule(kid, n, levels, ratio, order, k, None, None, 0)
    lam, pl = _d(np.zeros((m, 3)))
    w, pw = _d(np.zeros(m))
    lib().vpo_rule(kid, n, levels, ratio, order, k, pl, pw, m)
    return lam, w


def rule1d(kind, n=0, levels=6, ratio=0.15, order=3):
    kid = {"gauss": 0, "graded": 1, "graded_both": 2}[kind]
    m = lib().vpo_rule1d(kid, n, levels, ratio, order, None, None, 0)
    x, px = _d(np.zeros(m))
    w, pw = _d(np.zeros(m))
    lib().vpo_rule1d(kid, n, levels, ratio, order, px, pw, m)
    return x, w


def pair_rule(T, S, shared=(0, 0, 0), same=False, mode="body", depth_extra=0, **kw):
    """(tier name, lam, w) of the rule for test triangle T (3x3 corners) and source S (triangle, or 2x3 segment ends
    with mode='segment'; mode='wake' for a wake triangle)"""
    o = options(**kw)
    Tx, pT = _d(np.asarray(T, float).ravel())
    Sx, pS = _d(np.asarray(S, float).ravel())
    sh, psh = _i(np.asarray(shared, np.int32))
    md = {"body": 0, "wake": 1, "segment": 2}[mode]
    tier = ctypes.c_int(-1)
    m = lib().vpo_pair_rule(ctypes.byref(o), pT, pS, psh, int(same), md, depth_extra, None, None, 0, ctypes.byref(tier))
    if m < 0:
        raise ValueError("degenerate triangle")
    lam, pl = _d(np.zeros((m, 3)))
    w, pw = _d(np.zeros(m))
    lib().vpo_pair_rule(ctypes.byref(o), pT, pS, psh, int(same), md, depth_extra, pl, pw, m, ctypes.byref(tier))
    return TIERS[tier.value], lam, w


def pair_block(T, S, lam, w, sigma=0.0, test="hat", side=0, kernel_far=10.0):
    Tx, pT = _d(np.asarray(T, float).ravel())
    Sx, pS = _d(np.asarray(S, float).ravel())
    L, pl = _d(lam)
    W, pw = _d(w)
    blk, pb = _d(np.zeros(9))
    rb, pr = _d(np.zeros(3))
    lib().vpo_pair_block(pT, pS, pl, pw, len(W), sigma, _TEST[test], side, kernel_far, pb, pr)
    return blk.reshape(3, 3), rb


# ---- assembly ------------------------------------------------------------------------------------------------------

def source_strengths(g, V):
    """sigma = -V.n of every triangle (assemble.jl:364)"""
    x, t = g.x, g.tris
    n = np.cross(x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]])
    n /= np.linalg.norm(n, axis=1)[:, None]
    return -n @ np.asarray(V, float)


def assemble(g, dm, sigma, V, wake=None, rows=None, tests=None, nthreads=0, **kw):
    """A (nslot x (nslot + nwake)), b (nslot) and the per-tier pair and point counts (assemble.jl:377-447).
    ``rows = (t0, t1)`` assembles only the rows of test triangles t0..t1-1 (a sample for timing); ``tests`` (an array
    of triangle indices) only those test triangles' rows, so that the rows of every slot whose triangles are all
    among them are complete."""
    o = options(**kw)
    x, px = _d(g.x)
    tris, pt = _i(g.tris)
    cs, pc = _i(dm.corner_slot)
    tp, ptp = _i(g.touch_pairs.reshape(-1, 2) if len(g.touch_pairs) else np.zeros((1, 2)))
    sg, ps = _d(sigma)
    VV, pV = _d(V)
    if wake is not None:
        wx, pwx = _d(wake.x)
        wt, pwt = _i(wake.tris if len(wake.tris) else np.zeros((1, 3)))
        wf, pwf = _i(wake.filaments if len(wake.filaments) else np.zeros((1, 2)))
        nw, nwt, nf = wake.x.shape[0], len(wake.tris), len(wake.filaments)
    else:
        wx, pwx = _d(np.zeros(3))
        wt, pwt = _i(np.zeros(3))
        wf, pwf = _i(np.zeros(2))
        nw = nwt = nf = 0
    ncols = dm.nslot + nw
    A, pA = _d(np.zeros((dm.nslot, ncols)))
    b, pb = _d(np.zeros(dm.nslot))
    P = np.zeros(6, np.int64)
    Q = np.zeros(6, np.int64)
    LL = ctypes.POINTER(ctypes.c_longlong)
    if tests is not None:
        tl, ptl = _i(np.asarray(tests, np.int32))
        r = lib().vpo_assemble_list(ctypes.byref(o), g.nnode, px, g.ntri, pt, pc, dm.nslot, len(g.touch_pairs), ptp,
                                    ps, pV, nw, pwx, nwt, pwt, nf, pwf, len(tl), ptl, pA, pb, P.ctypes.data_as(LL),
                                    Q.ctypes.data_as(LL), nthreads)
    else:
        t0, t1 = (0, g.ntri) if rows is None else rows
        r = lib().vpo_assemble(ctypes.byref(o), g.nnode, px, g.ntri, pt, pc, dm.nslot, len(g.touch_pairs), ptp, ps, pV,
                               nw, pwx, nwt, pwt, nf, pwf, t0, t1, pA, pb, P.ctypes.data_as(LL), Q.ctypes.data_as(LL),
                               nthreads)
    if r != 0:
        raise ValueError("degenerate triangle")
    return A, b, {"pairs": dict(zip(TIERS, P.tolist())), "points": dict(zip(TIERS, Q.tolist()))}


# ---- bordered system and LAPACK solve (src/assembly/solve.jl, src/dofmap/system.jl) ----------------------------------

def reduce_system(dm, A, b, W=None):
    """(C' A [C; W], C' b) (system.jl:141-145)"""
    Cf = dm.C if W is None else sp.vstack([dm.C, W]).tocsr()
    if A.shape != (dm.nslot, Cf.shape[0]):
        raise ValueError(f"A is {A.shape}, expected ({dm.nslot}, {Cf.shape[0]})")
    return np.asarray(dm.C.T @ np.asarray(Cf.T @ A.T).T), dm.C.T @ b


def bordered_rows(dm):
    """(e, c) of every body (system.jl:156-165)"""
    rows = []
    for bi, qs in enumerate(dm.body_q):
        e = np.zeros(dm.nq)
        e[np.asarray(qs, dtype=np.int64)] = 1
        c = dm.C.T @ (dm.slot_area * (dm.slot_body == bi + 1))
        rows.append((e, np.asarray(c).ravel()))
    return rows


def bordered_matrix(dm, A, W=None):
    """The bordered matrix and the scales of its border columns (solve.jl:23-38)"""
    Ar, _ = reduce_system(dm, A, np.zeros(dm.nslot), W)
    rows = bordered_rows(dm)
    nq, nb = dm.nq, len(rows)
    M = np.zeros((nq + nb, nq + nb))
    M[:nq, :nq] = Ar
    scale = np.sum(np.abs(np.diag(Ar))) / nq
    se = np.zeros(nb)
    for k, (e, c) in enumerate(rows):
        se[k] = scale / np.linalg.norm(e)
        M[:nq, nq + k] = se[k] * e
        M[nq + k, :nq] = c * (scale / np.linalg.norm(c))
    return M, se


def bordered_rhs(dm, b):
    return np.concatenate([dm.C.T @ b, np.zeros(len(dm.body_closed))])


class Factorization:
    """GalerkinFactorization (solve.jl:65-72) over LAPACK dgetrf"""

    def __init__(self, dm, M, se):
        self.lu = sla.lu_factor(M, check_finite=False)
        rcond, info = sla.lapack.dgecon(self.lu[0], np.linalg.norm(M, 1), norm="1")
        self.cond = 1.0 / rcond
        self.se, self.C, self.nq, self.nb, self.M = se, dm.C, dm.nq, len(se), M


def factorize_galerkin(dm, A, W=None):
    M, se = bordered_matrix(dm, A, W)
    return Factorization(dm, M, se)


def solve_factored(F, b):
    """solve_galerkin(F, b) (solve.jl:95-99); b may hold several right hand sides as columns"""
    rhs = np.concatenate([F.C.T @ b, np.zeros((F.nb,) + b.shape[1:])])
    x = sla.lu_solve(F.lu, rhs, check_finite=False)
    q = x[:F.nq]
    return dict(q=q, mu=F.C @ q, lam=(F.se * x[F.nq:].T).T if b.ndim > 1 else F.se * x[F.nq:], cond=F.cond)


def solve_galerkin(dm, A, b, W=None):
    """(q, mu, lambda, cond, residual) (solve.jl:51-59)"""
    F = factorize_galerkin(dm, A, W)
    rhs = bordered_rhs(dm, b)
    x = sla.lu_solve(F.lu, rhs, check_finite=False)
    q = x[:dm.nq]
    res = np.linalg.norm(F.M @ x - rhs) / np.linalg.norm(rhs)
    return dict(q=q, mu=dm.C @ q, lam=F.se * x[dm.nq:], cond=F.cond, residual=res, x=x, F=F)


def consistency(dm, A, b, W=None):
    """Row, column and right hand side sum defects (solve.jl:111-115)"""
    Cf = dm.C if W is None else sp.vstack([dm.C, W]).tocsr()
    ACf = np.asarray((Cf.T @ A.T).T)
    nA = np.max(np.sum(np.abs(ACf), axis=1))
    return dict(rows=np.max(np.abs(ACf.sum(axis=1))) / nA, columns=np.max(np.abs(ACf.sum(axis=0))) / nA,
                rhs=abs(b.sum()) / np.sum(np.abs(b)))


# ---- loads (src/post/Post.jl, src/post/forces.jl) ------------------------------------------------------------------

def elements(g):
    x, t = g.x, g.tris
    a, b, c = x[t[:, 0]], x[t[:, 1]], x[t[:, 2]]
    nA = np.cross(b - a, c - a)
    A2 = np.linalg.norm(nA, axis=1)
    n = nA / A2[:, None]
    e = [c - b, a - c, b - a]
    gradl = [np.cross(n, ek) / A2[:, None] for ek in e]
    gam = [-ek / A2[:, None] for ek in e]
    return dict(n=n, area=A2 / 2, centroid=(a + b + c) / 3, gradl=gradl, gam=gam)


def surface_velocity(g, dm, sigma, mu, V, wake=None, mu_wake=None, kernel_far=10.0):
    """Velocity on the fluid side at every centroid from the singularities (Post.jl:32-64): V∞ + Σ σ_s w_s + γ_s × w_s
    with the own sheet at side 1, plus the wake's sheets (Post.jl:49-51) and tip filaments (Post.jl:52-55).
    Scalar loops over (point, source): small meshes only."""
    els = elements(g)
    V = np.asarray(V, float)
    m = np.asarray(mu)[dm.corner_slot]
    gam = sum(m[:, k:k + 1] * els["gam"][k] for k in range(3))
    X = g.x[g.tris]
    wsheets, wfil = [], []
    if wake is not None:
        mw = np.asarray(mu_wake, float)
        for t in wake.tris:
            a, b, c = wake.x[t[0]], wake.x[t[1]], wake.x[t[2]]
            A2 = np.linalg.norm(np.cross(b - a, c - a))
            e = [c - b, a - c, b - a]
            wsheets.append((a, b, c, sum(mw[t[k]] * (-e[k] / A2) for k in range(3))))
        for fa, fb in wake.filaments:
            wfil.append((wake.x[fa], wake.x[fb], mw[fa], mw[fb]))
    u = np.zeros((g.ntri, 3))
    for t in range(g.ntri):
        x = els["centroid"][t]
        acc = V.copy()
        for s in range(g.ntri):
            w = source_velocity(X[s, 0], X[s, 1], X[s, 2], x, side=1 if s == t else 0, far=kernel_far)
            acc += sigma[s] * w + np.cross(gam[s], w)
        for a, b, c, gw in wsheets:
            acc += np.cross(gw, source_velocity(a, b, c, x, far=kernel_far))
        for a, b, ma, mb in wfil:
            va, vb = segment_velocity(a, b, x)
            acc += ma * va + mb * vb
        u[t] = acc
    return u


def gradient_velocity(g, dm, mu, V, els=None):
    """V - (V.n)n + grad mu per triangle (Post.jl:72-73)"""
    els = els or elements(g)
    V = np.asarray(V, float)
    m = mu[dm.corner_slot]
    grad = sum(m[:, k:k + 1] * els["gradl"][k] for k in range(3))
    n = els["n"]
    return V - (n @ V)[:, None] * n + grad


def pressure_coefficient(u, V, dmudt=None):
    V = np.asarray(V, float)
    s = np.einsum("ij,ij->i", u, u)
    if dmudt is not None:
        s = s + 2 * dmudt
    return 1 - s / (V @ V)


def pressure_force(els, cp, origin=np.zeros(3)):
    f = -(cp * els["area"])[:, None] * els["n"]
    return f.sum(axis=0), np.cross(els["centroid"] - origin, f).sum(axis=0)


def te_segments(wte):
    out = []
    for line, closed in zip(wte.lines, wte.closed):
        m = len(line)
        for i in range(m if closed else m - 1):
            out.append((line[i], line[(i + 1) % m]))
    return out


def kutta_joukowski_force(wte, mu_w, V):
    V = np.asarray(V, float)
    G = np.zeros(3)
    for a, b in te_segments(wte):
        G += (mu_w[a] + mu_w[b]) / 2 * (wte.x[b] - wte.x[a])
    return 2 / (V @ V) * np.cross(V, G)


def trefftz_drag(wte, mu_w, V):
    """Induced drag in units of q (forces.jl:53-81)"""
    V = np.asarray(V, float)
    d = V / np.linalg.norm(V)

    def P(x):
        return x - (x @ d) * d

    vort, strips = [], []
    for line, closed in zip(wte.lines, wte.closed):
        m = len(line)
        nseg = m if closed else m - 1
        G = [(mu_w[line[i]] + mu_w[line[(i + 1) % m]]) / 2 for i in range(nseg)]
        for i in range(m):
            before = G[i - 1] if i > 0 else (G[nseg - 1] if closed else 0.0)
            after = G[i] if i < nseg else 0.0
            vort.append((P(wte.x[line[i]]), after - before))
        for i in range(nseg):
            strips.append((P(wte.x[line[i]]), P(wte.x[line[(i + 1) % m]]), G[i]))
    D = 0.0
    for a, b, Gk in strips:
        c, l = (a + b) / 2, np.linalg.norm(b - a)
        n = np.cross(d, (b - a) / l)
        v = np.zeros(3)
        for p, dG in vort:
            r = c - p
            v += dG / (4 * math.pi) * np.cross(d, r) / (r @ r)
        D += Gk * (n @ v) * l
    return 2 * D / (V @ V)


# ---- the exact ellipsoid flow (validation/common/exact_flows.jl:12-86) ----------------------------------------------

def carlson_rd(x, y, z):
    x0, y0, z0 = float(x), float(y), float(z)
    A0 = (x0 + y0 + 3 * z0) / 5
    Q = (np.spacing(A0) / 4) ** (-1 / 6) * max(abs(A0 - x0), abs(A0 - y0), abs(A0 - z0))
    x, y, z, A = x0, y0, z0, A0
    s, f = 0.0, 1.0
    while f * Q >= abs(A):
        lam = math.sqrt(x) * math.sqrt(y) + math.sqrt(x) * math.sqrt(z) + math.sqrt(y) * math.sqrt(z)
        s += f / (math.sqrt(z) * (z + lam))
        f /= 4
        x, y, z, A = (x + lam) / 4, (y + lam) / 4, (z + lam) / 4, (A + lam) / 4
    X, Y = f * (A0 - x0) / A, f * (A0 - y0) / A
    Z = -(X + Y) / 3
    e2, e3 = X * Y - 6 * Z**2, (3 * X * Y - 8 * Z**2) * Z
    e4, e5 = 3 * (X * Y - Z**2) * Z**2, X * Y * Z**3
    series = 1 - 3 * e2 / 14 + e3 / 6 + 9 * e2**2 / 88 - 3 * e4 / 22 - 9 * e2 * e3 / 52 + 3 * e5 / 26
    return f * A ** (-1.5) * series + 3 * s


def ellipsoid_factors(a, b, c):
    k = 2 * a * b * c / 3
    return np.array([k * carlson_rd(b**2, c**2, a**2), k * carlson_rd(c**2, a**2, b**2),
                     k * carlson_rd(a**2, b**2, c**2)])


class EllipsoidFlow:
    def __init__(self, axes, V):
        self.axes = np.asarray(axes, float)
        self.V = np.asarray(V, float)
        self.factors = ellipsoid_factors(*self.axes)
        self.kmu = self.factors / (2 - self.factors) * self.V
        self.k = 2 * self.V / (2 - self.factors)

    def surface_point(self, p):
        return p / np.sqrt(np.sum((p / self.axes) ** 2, axis=-1, keepdims=True))

    def surface_normal(self, x):
        n = x / self.axes**2
        return n / np.linalg.norm(n, axis=-1, keepdims=True)

    def exact_doublet(self, x):
        return x @ self.kmu

    def doublet_scale(self):
        return np.linalg.norm(self.kmu * self.axes)

    def exact_velocity(self, p):
        n = self.surface_normal(self.surface_point(p))
        return self.k - (n @ self.k)[..., None] * n

    def exact_cp(self, p):
        u = self.exact_velocity(p)
        return 1 - np.sum(u * u, axis=-1) / (self.V @ self.V)
