"""The reference's Julia API for the Galerkin hot path, over the GPU library.

Same names, argument meaning and errors as VortexPanel.jl:
  assemble(g, dm, els, σ, V∞; opts, wake) -> A, b, stats      src/assembly/assemble.jl:377-447
  factorize_galerkin(dm, A; W) -> GalerkinFactorization          src/assembly/solve.jl:81-87
  solve_galerkin(F, b) -> (q, μ, λ, cond)                        src/assembly/solve.jl:95-99
  solve_galerkin(dm, A, b; W) -> (q, μ, λ, cond, residual)       src/assembly/solve.jl:51-59
  source_strengths(els, V∞)                                      src/assembly/assemble.jl:364
and the loads the hot path's outputs feed (src/post/Post.jl:19-23,72-84; src/post/forces.jl:11-81).

``A`` stays on the GPU (a ``DeviceSystem``); ``np.asarray(A)`` or ``A.download()`` copies it to the host like the
reference's Matrix. ArgumentError maps to ValueError, SingularException to ``SingularError``.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, fields

import numpy as np
import scipy.sparse as sp

from . import _lib, autotune
from ._lib import D, I, check, default_context, load
from ._vec import cross3, norm3

TIER_NAMES = ("self", "edge", "vertex", "contact", "near", "far")


@dataclass
class AssemblyOptions:
    """AssemblyOptions (assemble.jl:26-41) plus the arithmetic: precision = 'fp64' (every integral, the LU and the
    solve in FP64) or 'mixed' (FP32 far and near tiers, FP64 touching and contact tiers, FP32 LU refined with FP64
    residuals)."""
    test: str = "hat"
    far_ratio: float = 3.0
    far_points: int = 3
    near_points: int = 7
    near_ratio: float = 1.5
    near_depth: int = 3
    touch_levels: int = 6
    touch_ratio: float = 0.15
    touch_order: int = 3
    corner_angle: float = 75.0
    contact_rel: float = 0.1
    kernel_far: float = 10.0
    precision: str = "fp64"
    threaded: bool = True  # accepted for compatibility; the GPU path is always parallel

    def c_struct(self) -> _lib.vp_assembly_options:
        tests = {"hat": 0, "onering": 1, "dual": 2}
        if self.test not in tests:
            raise ValueError(f"test must be :hat, :onering or :dual, not {self.test}")
        precs = {"fp64": _lib.VP_FP64, "mixed": _lib.VP_MIXED}
        if self.precision not in precs:
            raise ValueError(f"precision must be 'fp64' or 'mixed', not {self.precision}")
        o = _lib.vp_assembly_options()
        for f in fields(self):
            if f.name in ("threaded",):
                continue
            v = getattr(self, f.name)
            if f.name == "test":
                v = tests[v]
            elif f.name == "precision":
                v = precs[v]
            setattr(o, f.name, v)
        return o


def _dp(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(D)


def _ip(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(I)


# ---- elements (src/elements/flat_triangle.jl) -------------------------------------------------------------------------

@dataclass
class Elements:
    """The FlatTriangle fields of every triangle, as arrays: n, area, centroid, diam, gradλ (3 x ntri x 3), γ, and the
    corners (ntri x 9)"""
    n: np.ndarray
    area: np.ndarray
    centroid: np.ndarray
    diam: np.ndarray
    gradl: list
    gam: list
    corners: np.ndarray = None


def build_elements(g) -> Elements:
    x, t = g.x, g.tris
    a, b, c = x[t[:, 0]], x[t[:, 1]], x[t[:, 2]]
    nA = cross3(b - a, c - a)
    A2 = norm3(nA)
    if np.any(~(A2 > 0)):
        raise ValueError(f"degenerate triangle {int(np.argmin(A2))}")
    n = nA / A2[:, None]
    e = [c - b, a - c, b - a]
    diam = np.maximum.reduce([norm3(b - a), norm3(c - b), norm3(a - c)])
    return Elements(n, A2 / 2, (a + b + c) / 3, diam, [cross3(n, ek) / A2[:, None] for ek in e],
                    [-ek / A2[:, None] for ek in e], np.ascontiguousarray(np.concatenate([a, b, c], axis=1)))


def source_strengths(els: Elements, V, V_body=None) -> np.ndarray:
    """σ = -(V∞ - V_body)·n (assemble.jl:364)"""
    V = np.asarray(V, float)
    if V_body is not None:
        V = V - np.asarray(V_body, float)
    return -(els.n @ V)


# ---- assembly ----------------------------------------------------------------------------------------------------------

class DeviceSystem:
    """The assembled A (nslot x (nslot + nwake)) and b, resident on the GPU"""

    def __init__(self, ctx, handle, nslot, ncols):
        self.ctx, self.h, self.nslot, self.ncols = ctx, handle, nslot, ncols

    @property
    def shape(self):
        return (self.nslot, self.ncols)

    def download(self):
        A = np.zeros((self.nslot, self.ncols))
        check(self.ctx.h, load().vp_system_download(self.ctx.h, self.h, A.ctypes.data_as(D), None))
        return A

    def download_rows(self, r0, r1):
        """rows [r0, r1) of A and of b"""
        A = np.zeros((r1 - r0, self.ncols))
        b = np.zeros(r1 - r0)
        check(self.ctx.h, load().vp_system_download_rows(self.ctx.h, self.h, r0, r1, A.ctypes.data_as(D),
                                                         b.ctypes.data_as(D)))
        return A, b

    def rhs(self):
        b = np.zeros(self.nslot)
        check(self.ctx.h, load().vp_system_download(self.ctx.h, self.h, None, b.ctypes.data_as(D)))
        return b

    def __array__(self, dtype=None, copy=None):
        A = self.download()
        return A if dtype is None else A.astype(dtype)

    def __del__(self):
        if getattr(self, "h", None):
            try:
                load().vp_system_free(self.h)
            except Exception:
                pass
            self.h = None


def radon7():
    """The 7-point degree-5 triangle rule of Radon (rules.jl:76-92, n = 7): barycentrics (7 x 3), weights (sum 1)"""
    s = math.sqrt(15.0)
    a, b = (6 - s) / 21, (6 + s) / 21
    lam = [(1 / 3, 1 / 3, 1 / 3)]
    for p in (a, b):
        lam += [(1 - 2 * p, p, p), (p, 1 - 2 * p, p), (p, p, 1 - 2 * p)]
    w = [9 / 40] + [(155 - s) / 1200] * 3 + [(155 + s) / 1200] * 3
    return np.array(lam), np.array(w)


def test_weights(test, lam):
    """ψ at barycentrics lam (n x 3) (assemble.jl:52-58): hat λ, onering 1, dual the indicator of the largest λ
    (ties shared)"""
    lam = np.asarray(lam, float)
    if test == "hat":
        return lam.copy()
    if test == "onering":
        return np.ones_like(lam)
    if test == "dual":
        ind = (np.abs(lam - lam.max(axis=1, keepdims=True)) < 1e-12).astype(float)
        return ind / ind.sum(axis=1, keepdims=True)
    raise ValueError(f"test must be :hat, :onering or :dual, not {test}")


def external_rhs(els: Elements, dm, external, test="hat"):
    """The external velocity field's part of b (assemble.jl:423-427): -∫ψ_a n·u_ext dA over every test triangle
    by the 7-point rule, added into the slots. `external` maps points (n x 3) to velocities (n x 3)."""
    lam, w = radon7()
    X = np.einsum("qk,tkd->tqd", lam, els.corners.reshape(-1, 3, 3))
    U = np.asarray(external(X.reshape(-1, 3)), float).reshape(X.shape)
    un = np.einsum("tqd,td->tq", U, els.n)
    rows = -np.einsum("q,t,tq,qa->ta", w, els.area, un, test_weights(test, lam))
    b = np.zeros(dm.nslot)
    np.add.at(b, dm.corner_slot, rows)
    return b


def assemble(g, dm, els, sigma, V, opts: AssemblyOptions = None, external=None, wake=None, ctx=None, tune=True):
    """A, b and stats (assemble.jl:377-447). A is a DeviceSystem; b and stats are on the host. `external`, if given,
    is a velocity field (e.g. particles), a function of points (n x 3) returning velocities (n x 3): its part of b is
    added on the host (external_rhs) to the b of the device, which then differs from A.rhs(). With `tune`, the far
    tier's tile is the autotuner's choice for the mesh's size (autotune.py, the committed sweep)."""
    opts = opts or AssemblyOptions()
    ctx = ctx or default_context()
    if tune:
        autotune.apply(ctx, opts.precision, g.ntri)
    o = opts.c_struct()
    x, px = _dp(g.x)
    tr, pt = _ip(g.tris)
    cs, pc = _ip(dm.corner_slot)
    tp = np.asarray(g.touch_pairs, np.int32).reshape(-1, 2)
    tpp, ptp = _ip(tp if len(tp) else np.zeros((1, 2), np.int32))
    sg, ps = _dp(sigma)
    if sg.shape != (g.ntri,):
        raise ValueError(f"σ has {sg.shape[0]} entries, expected {g.ntri}")
    VV, pV = _dp(V)
    if wake is not None:
        wx, pwx = _dp(wake.x)
        wt, pwt = _ip(wake.tris if len(wake.tris) else np.zeros((1, 3)))
        wf, pwf = _ip(wake.filaments if len(wake.filaments) else np.zeros((1, 2)))
        nw, nwt, nf = wake.x.shape[0], len(wake.tris), len(wake.filaments)
    else:
        wx = wt = wf = None
        pwx, pwt, pwf = None, None, None
        nw = nwt = nf = 0
    h = ctypes.c_void_p()
    st = _lib.vp_assembly_stats()
    check(ctx.h, load().vp_assemble(ctx.h, ctypes.byref(o), g.nnode, px, g.ntri, pt, pc, dm.nslot, len(tp), ptp, ps, pV,
                                    nw, pwx, nwt, pwt, nf, pwf, ctypes.byref(h), ctypes.byref(st)))
    A = DeviceSystem(ctx, h, dm.nslot, dm.nslot + nw)
    stats = {"pairs": dict(zip(TIER_NAMES, list(st.pairs))), "points": dict(zip(TIER_NAMES, list(st.points))),
             "time": st.time_ms / 1e3, "points_fp64": st.points_fp64}
    b = A.rhs()
    if external is not None:
        b = b + external_rhs(els, dm, external, opts.test)
    return A, b, stats


def assemble_batch(cases, opts: AssemblyOptions = None, ctx=None, tune=True):
    """assemble for a batch of independent bodies of uneven sizes in shared launches (vp_assemble_batch): cases is a
    list of (g, dm, sigma, V, wake or None); returns a list of (A, b, stats) as assemble gives them with the same far
    tile, A and b the same bit for bit. One options set (and precision) and one far tile (with `tune`, the
    autotuner's choice for the largest body) for the whole batch."""
    opts = opts or AssemblyOptions()
    ctx = ctx or default_context()
    if tune:
        autotune.apply(ctx, opts.precision, max(c[0].ntri for c in cases))
    o = opts.c_struct()
    keep = []
    ins = (_lib.vp_assembly_input * len(cases))()
    shapes = []
    for k, (g, dm, sigma, V, wake) in enumerate(cases):
        x, px = _dp(g.x)
        tr, pt = _ip(g.tris)
        cs, pc = _ip(dm.corner_slot)
        tp = np.asarray(g.touch_pairs, np.int32).reshape(-1, 2)
        tpp, ptp = _ip(tp if len(tp) else np.zeros((1, 2), np.int32))
        sg, ps = _dp(sigma)
        if sg.shape != (g.ntri,):
            raise ValueError(f"case {k}: σ has {sg.shape[0]} entries, expected {g.ntri}")
        VV, pV = _dp(V)
        keep += [x, tr, cs, tpp, sg, VV]
        it = ins[k]
        it.nnode, it.x, it.ntri, it.tris, it.corner_slot, it.nslot = g.nnode, px, g.ntri, pt, pc, dm.nslot
        it.ntouch, it.touch_pairs, it.sigma, it.vinf = len(tp), ptp, ps, pV
        nw = 0
        if wake is not None:
            wx, pwx = _dp(wake.x)
            wt, pwt = _ip(wake.tris if len(wake.tris) else np.zeros((1, 3)))
            wf, pwf = _ip(wake.filaments if len(wake.filaments) else np.zeros((1, 2)))
            keep += [wx, wt, wf]
            nw = wake.x.shape[0]
            it.nwnode, it.wx, it.nwtri, it.wtris, it.nfil, it.fil = nw, pwx, len(wake.tris), pwt, len(wake.filaments), pwf
        shapes.append((dm.nslot, dm.nslot + nw))
    hs = (ctypes.c_void_p * len(cases))()
    sts = (_lib.vp_assembly_stats * len(cases))()
    check(ctx.h, load().vp_assemble_batch(ctx.h, ctypes.byref(o), len(cases), ins, hs, sts))
    out = []
    for k, (nr, nc) in enumerate(shapes):
        A = DeviceSystem(ctx, ctypes.c_void_p(hs[k]), nr, nc)
        st = sts[k]
        stats = {"pairs": dict(zip(TIER_NAMES, list(st.pairs))), "points": dict(zip(TIER_NAMES, list(st.points))),
                 "time": st.time_ms / 1e3, "points_fp64": st.points_fp64}
        out.append((A, A.rhs(), stats))
    return out


# ---- the bordered solve ------------------------------------------------------------------------------------------------

class GalerkinFactorization:
    """The LU of the bordered system on the GPU (solve.jl:65-72)"""

    def __init__(self, ctx, handle, dm, precision):
        self.ctx, self.h, self.dm, self.precision = ctx, handle, dm, precision
        n = ctypes.c_int()
        c = ctypes.c_double()
        check(ctx.h, load().vp_factor_info(handle, ctypes.byref(n), ctypes.byref(c)))
        self.n, self.cond = n.value, c.value
        self.nq, self.nb = dm.nq, len(dm.body_closed)

    def __del__(self):
        if getattr(self, "h", None):
            try:
                load().vp_factor_free(self.h)
            except Exception:
                pass
            self.h = None


def _csr_parts(M):
    M = sp.csr_matrix(M)
    p, pp = _ip(M.indptr)
    c, pc = _ip(M.indices if M.nnz else np.zeros(1))
    v, pv = _dp(M.data if M.nnz else np.zeros(1))
    return (p, c, v), (pp, pc, pv)


def factorize_galerkin(dm, A: DeviceSystem, W=None, precision=None, ctx=None) -> GalerkinFactorization:
    """Factor the bordered matrix of C' A [C; W] once, for many right hand sides (solve.jl:81-87)"""
    ctx = ctx or A.ctx
    precision = precision or "fp64"
    prec = {"fp64": _lib.VP_FP64, "mixed": _lib.VP_MIXED}[precision]
    keepC, (cp, cc, cv) = _csr_parts(dm.C)
    nw = 0 if W is None else W.shape[0]
    if A.ncols != dm.nslot + nw:
        raise ValueError(f"A is {A.shape}, expected ({dm.nslot}, {dm.nslot + nw})")
    if W is not None:
        keepW, (wp, wc, wv) = _csr_parts(W)
    else:
        wp = wc = wv = None
    qb, pqb = _ip(dm.q_body)
    sa, psa = _dp(dm.slot_area)
    sb, psb = _ip(dm.slot_body)
    h = ctypes.c_void_p()
    cond = ctypes.c_double()
    check(ctx.h, load().vp_factorize(ctx.h, A.h, prec, dm.nq, cp, cc, cv, nw, wp, wc, wv, len(dm.body_closed), pqb, psa,
                                     psb, ctypes.byref(h), ctypes.byref(cond)))
    return GalerkinFactorization(ctx, h, dm, precision)


def solve_galerkin(*args, W=None, precision=None, ctx=None):
    """solve_galerkin(F, b) (solve.jl:95-99) or solve_galerkin(dm, A, b; W) (solve.jl:51-59). b may hold several right
    hand sides as columns."""
    if isinstance(args[0], GalerkinFactorization):
        F, b = args
        b = np.asarray(b, float)
        nrhs = 1 if b.ndim == 1 else b.shape[1]
        bb, pb = _dp(b.reshape(F.dm.nslot, nrhs).T.copy().ravel())  # column-major
        q = np.zeros(F.nq * nrhs)
        lam = np.zeros(max(F.nb, 1) * nrhs)
        check(F.ctx.h, load().vp_solve(F.ctx.h, F.h, nrhs, pb, q.ctypes.data_as(D), lam.ctypes.data_as(D)))
        q = q.reshape(nrhs, F.nq).T
        lam = lam[:F.nb * nrhs].reshape(nrhs, F.nb).T
        if b.ndim == 1:
            q, lam = q[:, 0], lam[:, 0]
        return dict(q=q, mu=F.dm.C @ q, lam=lam, cond=F.cond)
    dm, A, b = args
    F = factorize_galerkin(dm, A, W=W, precision=precision, ctx=ctx)
    res = ctypes.c_double()
    q = np.zeros(dm.nq)
    lam = np.zeros(max(F.nb, 1))
    if np.array_equal(np.asarray(b), A.rhs()):
        check(F.ctx.h, load().vp_solve_system(F.ctx.h, F.h, A.h, q.ctypes.data_as(D), lam.ctypes.data_as(D),
                                              ctypes.byref(res)))
        residual = res.value
    else:
        s = solve_galerkin(F, b)
        q, lam = s["q"], s["lam"]
        residual = float("nan")
    return dict(q=q, mu=dm.C @ q, lam=lam[:F.nb], cond=F.cond, residual=residual, F=F)


# ---- loads (src/post/Post.jl, src/post/forces.jl) ------------------------------------------------------------------

def element_values(dm, mu):
    return np.asarray(mu)[dm.corner_slot]


def sheet_strengths(els: Elements, dm, mu):
    """γ = Σ_b μ_b γ_b of every triangle (Post.jl:19-23)"""
    m = element_values(dm, mu)
    return sum(m[:, k:k + 1] * els.gam[k] for k in range(3))


def _sheet_velocity(ctx, precision, corners, sigma, gamma, X, kernel_far):
    """Σ σ_s w_s + γ_s × w_s of the triangles (corners n x 9) at the points X, on the GPU (vp_body_velocity)"""
    c = np.ascontiguousarray(corners, dtype=np.float64)
    sg = np.ascontiguousarray(sigma, dtype=np.float64)
    gm = np.ascontiguousarray(gamma, dtype=np.float64)
    x = np.ascontiguousarray(X, dtype=np.float64)
    U = np.zeros_like(x)
    prec = {"fp64": _lib.VP_FP64, "mixed": _lib.VP_MIXED}[precision]
    check(ctx.h, load().vp_body_velocity(ctx.h, prec, len(c), c.ctypes.data_as(D), sg.ctypes.data_as(D),
                                        gm.ctypes.data_as(D), kernel_far, len(x), x.ctypes.data_as(D),
                                        U.ctypes.data_as(D)))
    return U


def surface_velocity(els: Elements, dm, sigma, mu, V, wake=None, mu_wake=None, kernel_far=10.0, precision="fp64",
                     ctx=None):
    """Velocity on the fluid side at every triangle's centroid from the singularities (Post.jl:32-64):
    V∞ + Σ σ_s w_s + Σ γ_s × w_s, the triangle's own sheet taken on the side its normal points to, plus, with a
    `wake` and the doublets of its nodes `mu_wake` (W q), the wake's sheets and tip filaments. The sums run on the
    GPU: the sheets through vp_body_velocity, which takes every sheet at side 0 (at its own centroid, in its plane);
    the side-1 limit of the own sheet adds ½σn + ½γ × n. The filaments go through vp_eval_points (mode 2, one
    evaluation per centroid and filament)."""
    ctx = ctx or default_context()
    V = np.asarray(V, float)
    sigma = np.asarray(sigma, float)
    gam = sheet_strengths(els, dm, mu)
    X = els.centroid
    u = V + _sheet_velocity(ctx, precision, els.corners, sigma, gam, X, kernel_far)
    u += 0.5 * (sigma[:, None] * els.n + np.cross(gam, els.n))
    if wake is not None:
        if mu_wake is None:
            raise ValueError("surface_velocity with a wake needs mu_wake, the doublets of its nodes")
        mw = np.asarray(mu_wake, float)
        if len(wake.tris):
            wc = wake.x[wake.tris]  # (nwtri, 3, 3)
            wa, wb, wcc = wc[:, 0], wc[:, 1], wc[:, 2]
            A2 = np.linalg.norm(np.cross(wb - wa, wcc - wa), axis=1)[:, None]
            e = [wcc - wb, wa - wcc, wb - wa]
            gw = sum(mw[wake.tris[:, k]][:, None] * (-e[k] / A2) for k in range(3))
            u += _sheet_velocity(ctx, precision, wc.reshape(-1, 9), np.zeros(len(wc)), gw, X, kernel_far)
        if len(wake.filaments):
            nt, nf = len(X), len(wake.filaments)
            fa, fb = wake.x[wake.filaments[:, 0]], wake.x[wake.filaments[:, 1]]
            rows = np.zeros((nf, 9))
            rows[:, 0:3], rows[:, 3:6] = fa, fb
            rows[:, 6], rows[:, 7] = mw[wake.filaments[:, 0]], mw[wake.filaments[:, 1]]
            rows = np.tile(rows, (nt, 1))
            xs = np.repeat(X, nf, axis=0)
            for k in range(3):
                m = np.zeros((nt * nf, 3))
                m[:, k] = 1.0
                s = eval_points(2, rows, xs, m, precision=precision, ctx=ctx)[:, 0]
                u[:, k] += s.reshape(nt, nf).sum(axis=1)
    return u


def surface_loads(els: Elements, dm, mu, V, dmudt=None, origin=(0.0, 0.0, 0.0), ctx=None):
    """The gradient route in one FP64 pass on the GPU (vp_surface_loads): u = V∞ - (V∞·n)n + ∇μ per triangle
    (Post.jl:72-73), Cp = 1 - (|u|² + 2 ∂μ/∂t)/|V∞|² with the element mean of the slot values dmudt (Post.jl:82-84),
    and the force and moment -Σ Cp A n, Σ (c - origin) × (-Cp A n) (forces.jl:11-20). Returns a dict u, cp, F, M."""
    ctx = ctx or default_context()
    c, pc = _dp(els.corners)
    cs, pcs = _ip(dm.corner_slot)
    m, pm = _dp(mu)
    if m.shape != (dm.nslot,):
        raise ValueError(f"μ has {m.shape[0]} entries, expected {dm.nslot}")
    dd, pdd = (None, None) if dmudt is None else _dp(dmudt)
    VV, pV = _dp(V)
    o, po = _dp(origin)
    nt = c.shape[0]
    u, cp, F, M = np.zeros((nt, 3)), np.zeros(nt), np.zeros(3), np.zeros(3)
    check(ctx.h, load().vp_surface_loads(ctx.h, nt, pc, pcs, dm.nslot, pm, pdd, pV, po, u.ctypes.data_as(D),
                                         cp.ctypes.data_as(D), F.ctypes.data_as(D), M.ctypes.data_as(D)))
    return dict(u=u, cp=cp, F=F, M=M)


def gradient_velocity(els: Elements, dm, mu, V, ctx=None):
    """V∞ - (V∞·n)n + ∇μ on every triangle (Post.jl:72-73), FP64 on the GPU"""
    return surface_loads(els, dm, mu, V, ctx=ctx)["u"]


def pressure_coefficient(u, V, dmudt=None):
    """1 - (|u|² + 2 ∂μ/∂t)/|V∞|² at given velocities (Post.jl:82-84); surface_loads gives it from μ on the GPU"""
    V = np.asarray(V, float)
    s = np.einsum("ij,ij->i", np.asarray(u, float), np.asarray(u, float))
    if dmudt is not None:
        s = s + 2 * np.asarray(dmudt)
    return 1 - s / (V @ V)


def pressure_force(els: Elements, cp, origin=(0.0, 0.0, 0.0), ctx=None):
    """Force and moment about origin, in units of q∞, of a Cp constant on each triangle (forces.jl:11-20), FP64 on the
    GPU (vp_pressure_force)"""
    ctx = ctx or default_context()
    c, pc = _dp(els.corners)
    cc, pcc = _dp(cp)
    if cc.shape != (c.shape[0],):
        raise ValueError(f"cp has {cc.shape[0]} entries, expected {c.shape[0]}")
    o, po = _dp(origin)
    F, M = np.zeros(3), np.zeros(3)
    check(ctx.h, load().vp_pressure_force(ctx.h, c.shape[0], pc, pcc, po, F.ctypes.data_as(D), M.ctypes.data_as(D)))
    return F, M


def wake_loads(wte, mu_w, V, ctx=None):
    """(F_kj, D_trefftz): kutta_joukowski_force and trefftz_drag (forces.jl:34-39,53-81) of the trailing edge
    doublets mu_w, in units of q∞, FP64 on the GPU (vp_wake_loads)"""
    ctx = ctx or default_context()
    x, px = _dp(wte.x)
    mw, pmw = _dp(mu_w)
    if mw.shape != (x.shape[0],):
        raise ValueError(f"μ_w has {mw.shape[0]} entries, expected {x.shape[0]}")
    lines = [np.asarray(L, np.int32) for L in wte.lines]
    ptr, pptr = _ip(np.concatenate([[0], np.cumsum([len(L) for L in lines])]) if lines else np.zeros(1))
    nodes, pnodes = _ip(np.concatenate(lines) if lines else np.zeros(1))
    closed, pclosed = _ip(np.asarray([bool(c) for c in wte.closed], np.int32) if lines else np.zeros(1))
    VV, pV = _dp(V)
    F, Dv = np.zeros(3), ctypes.c_double()
    check(ctx.h, load().vp_wake_loads(ctx.h, x.shape[0], px, len(lines), pptr, pnodes, pclosed, pmw, pV,
                                      F.ctypes.data_as(D), ctypes.byref(Dv)))
    return F, Dv.value


def kutta_joukowski_force(wte, mu_w, V, ctx=None):
    """(2/|V∞|²) V∞ × ∫μ_w dl along the trailing edge lines (forces.jl:34-39), FP64 on the GPU"""
    return wake_loads(wte, mu_w, V, ctx=ctx)[0]


def trefftz_drag(wte, mu_w, V, ctx=None):
    """Induced drag in the Trefftz plane, in units of q∞ (forces.jl:53-81), FP64 on the GPU"""
    return wake_loads(wte, mu_w, V, ctx=ctx)[1]


def consistency(dm, A: DeviceSystem, b=None, W=None, ctx=None):
    """Row, column and right hand side sum defects of A [C; W] (solve.jl:111-115), FP64 on the GPU
    (vp_consistency). b defaults to the device's own; a host b given here (an external field's) enters the rhs
    defect."""
    ctx = ctx or A.ctx
    keepC, (cp, cc, cv) = _csr_parts(dm.C)
    nw = 0 if W is None else W.shape[0]
    if A.ncols != dm.nslot + nw:
        raise ValueError(f"A is {A.shape}, expected ({dm.nslot}, {dm.nslot + nw})")
    if W is not None:
        keepW, (wp, wc, wv) = _csr_parts(W)
    else:
        wp = wc = wv = None
    out = np.zeros(3)
    check(ctx.h, load().vp_consistency(ctx.h, A.h, dm.nq, cp, cc, cv, nw, wp, wc, wv, out.ctypes.data_as(D)))
    res = dict(rows=float(out[0]), columns=float(out[1]), rhs=float(out[2]))
    if b is not None:
        bb = np.asarray(b, float)
        if not np.array_equal(bb, A.rhs()):
            res["rhs"] = float(abs(bb.sum()) / np.abs(bb).sum())
    return res


# ---- diagnostics -----------------------------------------------------------------------------------------------------

def eval_points(mode, tri, x, m=None, side=0, kernel_far=10.0, precision="fp64", ctx=None):
    """The device kernels at points (vp_eval_points): mode 0 velocity w, 1 s = w·m with its x and corner
    derivatives, 2 the filament's (see include/vortexpanel_gpu.h)"""
    ctx = ctx or default_context()
    tri = np.ascontiguousarray(np.asarray(tri, float).reshape(-1, 9))
    n = tri.shape[0]
    x = np.ascontiguousarray(np.asarray(x, float).reshape(n, 3))
    nout = {0: 3, 1: 13, 2: 10}[mode]
    out = np.zeros((n, nout))
    mm = None if m is None else np.ascontiguousarray(np.asarray(m, float).reshape(n, 3))
    prec = {"fp64": _lib.VP_FP64, "mixed": _lib.VP_MIXED}[precision]
    check(ctx.h, load().vp_eval_points(ctx.h, mode, prec, n, tri.ctypes.data_as(D), x.ctypes.data_as(D),
                                       None if mm is None else mm.ctypes.data_as(D), side, kernel_far,
                                       out.ctypes.data_as(D)))
    return out


STATIC_POINTS_MAX = 2048  # VP_STATIC_POINTS_MAX in include/vortexpanel_gpu.h


def eval_points_static(mode, tri, x, m=None, side=0, kernel_far=10.0, precision="fp64", ctx=None):
    """eval_points through vp_eval_points_static: no device allocation, at most STATIC_POINTS_MAX points a call;
    calls that overlap in time on one device race on its staging array"""
    ctx = ctx or default_context()
    tri = np.ascontiguousarray(np.asarray(tri, float).reshape(-1, 9))
    n = tri.shape[0]
    x = np.ascontiguousarray(np.asarray(x, float).reshape(n, 3))
    out = np.zeros((n, {0: 3, 1: 13, 2: 10}[mode]))
    mm = None if m is None else np.ascontiguousarray(np.asarray(m, float).reshape(n, 3))
    prec = {"fp64": _lib.VP_FP64, "mixed": _lib.VP_MIXED}[precision]
    check(ctx.h, load().vp_eval_points_static(ctx.h, mode, prec, n, tri.ctypes.data_as(D), x.ctypes.data_as(D),
                                              None if mm is None else mm.ctypes.data_as(D), side, kernel_far,
                                              out.ctypes.data_as(D)))
    return out
