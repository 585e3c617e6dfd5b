"""Derivative oracle of the lifting wing's loads. TEST INFRASTRUCTURE ONLY: the tests use it as the checker of the
GPU adjoint; nothing in the product imports it.

The reference checks derivatives with ForwardDiff (test/kernels/test_kernels.jl:127-148). Here the C++ oracle's
templated assembly runs on forward-mode dual numbers (vpo_dual_assemble: A, b and the elements along up to
`vpo_dual_nd()` directions at once, tiers and pieces taken at the value), and the steps after it carry their tangents
exactly: the bordered solve (solve.jl:15-42, 51-59) by q' = M^-1 (r' - M' x), and the loads (Post.jl:72-73,
forces.jl:11-81) on jets, arrays of values with their derivatives.

A direction is (dx, dalpha): a tangent of every node position (nnode x 3) and of the angle of attack. The rigid
wake's nodes move with their trailing edge nodes (a wake node's tangent is its trailing edge node's), and the
freestream is (cos a, 0, sin a), as the product's gradients define them.
"""
import ctypes
import math

import numpy as np
import scipy.linalg as sla

import oracle


class J:
    """a jet: value v (shape S) and derivatives d (nd x S)"""

    __slots__ = ("v", "d")

    def __init__(self, v, d):
        self.v = np.asarray(v, float)
        self.d = np.asarray(d, float)

    @staticmethod
    def const(v, nd):
        v = np.asarray(v, float)
        return J(v, np.zeros((nd,) + v.shape))

    def _lift(self, o):
        o = o if isinstance(o, J) else J.const(o, self.d.shape[0])
        r = max(self.v.ndim, o.v.ndim)
        return o._rank(r)

    def _rank(self, r):
        """the same jet with leading unit axes up to rank r (numpy's broadcasting of the values, applied to the
        derivatives behind their direction axis)"""
        k = r - self.v.ndim
        if k <= 0:
            return self
        return J(self.v.reshape((1,) * k + self.v.shape), self.d.reshape(self.d.shape[:1] + (1,) * k + self.v.shape))

    def _pair(self, o):
        o = self._lift(o)
        return self._rank(o.v.ndim), o

    def __add__(self, o):
        a, o = self._pair(o)
        return J(a.v + o.v, a.d + o.d)

    __radd__ = __add__

    def __sub__(self, o):
        a, o = self._pair(o)
        return J(a.v - o.v, a.d - o.d)

    def __rsub__(self, o):
        return self._lift(o) - self

    def __neg__(self):
        return J(-self.v, -self.d)

    def __mul__(self, o):
        a, o = self._pair(o)
        return J(a.v * o.v, a.d * o.v + a.v * o.d)

    __rmul__ = __mul__

    def __truediv__(self, o):
        a, o = self._pair(o)
        q = a.v / o.v
        return J(q, (a.d - q * o.d) / o.v)

    def __rtruediv__(self, o):
        return self._lift(o) / self

    def __getitem__(self, k):
        k = k if isinstance(k, tuple) else (k,)
        return J(self.v[k], self.d[(slice(None),) + k])

    def col(self):
        """a trailing axis of length 1, for broadcasting against 3-vectors"""
        return J(self.v[..., None], self.d[..., None])


def jdot(a, b):
    p = a * b
    return J(p.v.sum(axis=-1), p.d.sum(axis=-1))


def jcross(a, b):
    return J(np.cross(a.v, b.v), np.cross(a.d, b.v) + np.cross(a.v, b.d))


def jsqrt(a):
    s = np.sqrt(a.v)
    return J(s, a.d / (2 * s))


def jsum(a, axis=0):
    return J(a.v.sum(axis=axis), a.d.sum(axis=axis + 1))


def nd_max():
    return int(oracle.lib().vpo_dual_nd())


def dual_assemble(g, dm, V, dV, dx, wake=None, dwx=None, nthreads=0, **kw):
    """A ((1 + nd) x nslot x ncols), b ((1 + nd) x nslot) and per triangle (area, n, gradl) ((1 + nd) x ntri x 13)
    of assemble (assemble.jl:377-447) with sigma = -n.V, along the nd directions dx (nd x nnode x 3), dwx (nd x nwnode
    x 3), dV (nd x 3)"""
    L = oracle.lib()
    nd = len(dx)
    if nd > nd_max():
        raise ValueError(f"at most {nd_max()} directions per pass")
    if not hasattr(L, "_dual_set"):
        D = ctypes.POINTER(ctypes.c_double)
        I = ctypes.POINTER(ctypes.c_int)
        LL = ctypes.POINTER(ctypes.c_longlong)
        L.vpo_dual_assemble.argtypes = [ctypes.c_void_p, ctypes.c_int, D, D, ctypes.c_int, I, I, ctypes.c_int,
                                        ctypes.c_int, I, D, D, ctypes.c_int, D, D, ctypes.c_int, I, ctypes.c_int, I,
                                        ctypes.c_int, D, D, D, LL, LL, ctypes.c_int]
        L.vpo_dual_assemble.restype = ctypes.c_int
        L._dual_set = True
    o = oracle.options(**kw)
    x, px = oracle._d(g.x)
    dxa, pdx = oracle._d(np.asarray(dx, float).reshape(nd, g.nnode, 3) if nd else np.zeros(3))
    tris, pt = oracle._i(g.tris)
    cs, pc = oracle._i(dm.corner_slot)
    tp, ptp = oracle._i(g.touch_pairs.reshape(-1, 2) if len(g.touch_pairs) else np.zeros((1, 2)))
    VV, pV = oracle._d(V)
    dVa, pdV = oracle._d(np.asarray(dV, float).reshape(nd, 3) if nd else np.zeros(3))
    if wake is not None:
        wx, pwx = oracle._d(wake.x)
        dwa, pdw = oracle._d(np.asarray(dwx, float).reshape(nd, len(wake.x), 3) if nd else np.zeros(3))
        wt, pwt = oracle._i(wake.tris if len(wake.tris) else np.zeros((1, 3)))
        wf, pwf = oracle._i(wake.filaments if len(wake.filaments) else np.zeros((1, 2)))
        nw, nwt, nf = wake.x.shape[0], len(wake.tris), len(wake.filaments)
    else:
        wx, pwx = oracle._d(np.zeros(3))
        dwa, pdw = oracle._d(np.zeros(3))
        wt, pwt = oracle._i(np.zeros(3))
        wf, pwf = oracle._i(np.zeros(2))
        nw = nwt = nf = 0
    ncols = dm.nslot + nw
    A, pA = oracle._d(np.zeros((1 + nd, dm.nslot, ncols)))
    b, pb = oracle._d(np.zeros((1 + nd, dm.nslot)))
    E, pE = oracle._d(np.zeros((1 + nd, g.ntri, 13)))
    P = np.zeros(6, np.int64)
    Q = np.zeros(6, np.int64)
    LLp = ctypes.POINTER(ctypes.c_longlong)
    r = L.vpo_dual_assemble(ctypes.byref(o), g.nnode, px, pdx, g.ntri, pt, pc, dm.nslot, len(g.touch_pairs), ptp, pV,
                            pdV, nw, pwx, pdw, nwt, pwt, nf, pwf, nd, pA, pb, pE, P.ctypes.data_as(LLp),
                            Q.ctypes.data_as(LLp), nthreads)
    if r != 0:
        raise ValueError(f"vpo_dual_assemble failed ({r})")
    return A, b, E, {"pairs": dict(zip(oracle.TIERS, P.tolist())), "points": dict(zip(oracle.TIERS, Q.tolist()))}


def _bordered_tangent(dm, A, dA, area, darea, W):
    """the bordered matrix M (solve.jl:23-38) and its tangents along the directions of dA, darea: Ar = C'A[C; W] is
    linear in A; the border's scale sum|diag Ar|/nq and area rows c = C'(slot area of the body) follow the
    geometry"""
    M, se = oracle.bordered_matrix(dm, A, W)
    nq = dm.nq
    Ar = M[:nq, :nq]
    rows = oracle.bordered_rows(dm)
    scale = np.sum(np.abs(np.diag(Ar))) / nq
    out = []
    for k in range(len(dA)):
        dAr, _ = oracle.reduce_system(dm, dA[k], np.zeros(dm.nslot), W)
        dscale = np.sum(np.sign(np.diag(Ar)) * np.diag(dAr)) / nq
        dslot = np.zeros(dm.nslot)
        for c in range(3):
            np.add.at(dslot, dm.corner_slot[:, c], darea[k] / 3.0)
        dM = np.zeros_like(M)
        dM[:nq, :nq] = dAr
        for j, (e, c) in enumerate(rows):
            dM[:nq, nq + j] = dscale / np.linalg.norm(e) * e
            dc = np.asarray(dm.C.T @ (dslot * (dm.slot_body == j + 1))).ravel()
            nc = np.linalg.norm(c)
            dM[nq + j, :nq] = dc * (scale / nc) + c * (dscale / nc) - c * (scale * (c @ dc) / nc**3)
        out.append(dM)
    return M, out


def _trefftz(wte_lines, wte_closed, X, mu_w, V):
    """trefftz_drag (forces.jl:53-81) on jets: X (nte x 3), mu_w (nte) and V (3)"""
    d = V / jsqrt(jdot(V, V))

    def P(x):
        return x - jdot(x, d) * d

    vort, strips = [], []
    for line, closed in zip(wte_lines, wte_closed):
        m = len(line)
        nseg = m if closed else m - 1
        G = [(mu_w[line[i]] + mu_w[line[(i + 1) % m]]) / 2 for i in range(nseg)]
        for i in range(m):
            before = G[i - 1] if i > 0 else (G[nseg - 1] if closed else 0.0)
            after = G[i] if i < nseg else 0.0
            vort.append((P(X[line[i]]), after - before))
        for i in range(nseg):
            strips.append((P(X[line[i]]), P(X[line[(i + 1) % m]]), G[i]))
    D = 0.0
    for a, b, Gk in strips:
        c, l = (a + b) / 2, jsqrt(jdot(b - a, b - a))
        n = jcross(d, (b - a) / l)
        v = 0.0
        for p, dG in vort:
            r = c - p
            v = v + dG / (4 * math.pi) * jcross(d, r) / jdot(r, r)
        D = D + Gk * jdot(n, v) * l
    return 2 * D / jdot(V, V)


def wing_loads_tangent(w, wake, W, a, dirs, nthreads=0):
    """CL (pressure route, Post.jl:72-84) and CDi (Trefftz, forces.jl:53-81) of wing w with rigid wake `wake`
    (rows along +x from the trailing edge) at angle of attack a, and their derivatives along dirs = [(dx, dalpha),
    ...]: returns (CL, CDi, dCL (nd), dCDi (nd))"""
    nd = len(dirs)
    g, dm = w.g, w.dm
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    dV = np.array([da * np.array([-math.sin(a), 0.0, math.cos(a)]) for _, da in dirs])
    dx = np.array([np.asarray(x, float) for x, _ in dirs])
    wte = dm.wake_te
    wnode = wte.node[wake.te]  # the body node each wake node follows
    dwx = dx[:, wnode, :]
    A, b, E, _ = dual_assemble(g, dm, V, dV, dx, wake=wake, dwx=dwx, nthreads=nthreads)
    area, darea = E[0, :, 0], E[1:, :, 0]
    M, dM = _bordered_tangent(dm, A[0], A[1:], area, darea, W)
    lu = sla.lu_factor(M)
    rhs = oracle.bordered_rhs(dm, b[0])
    xs = sla.lu_solve(lu, rhs)
    dxs = np.array([sla.lu_solve(lu, oracle.bordered_rhs(dm, b[1 + k]) - dM[k] @ xs) for k in range(nd)])
    q, dq = xs[:dm.nq], dxs[:, :dm.nq]
    mu = J(dm.C @ q, np.array([dm.C @ dq[k] for k in range(nd)]))
    # the pressure route: u = V - (V.n) n + sum_k mu_k gradl_k (Post.jl:72-73), cp = 1 - u.u / V.V, F = -sum cp A n
    Vj = J(V, dV)
    n = J(E[0, :, 1:4], E[1:, :, 1:4])
    Aj = J(area, darea)
    u = Vj - jdot(n, Vj).col() * n
    for k in range(3):
        gl = J(E[0, :, 4 + 3 * k:7 + 3 * k], E[1:, :, 4 + 3 * k:7 + 3 * k])
        u = u + mu[dm.corner_slot[:, k]].col() * gl
    cp = 1.0 - jdot(u, u) / jdot(Vj, Vj)
    F = jsum(-(cp * Aj).col() * n, axis=0)
    eL = J(np.array([-math.sin(a), 0.0, math.cos(a)]),
           np.array([da * np.array([-math.cos(a), 0.0, -math.sin(a)]) for _, da in dirs]))
    S = w.span * w.chord
    CL = jdot(F, eL) / S
    # Trefftz drag of mu_w = K q at the trailing edge nodes
    mw = J(dm.K @ q, np.array([dm.K @ dq[k] for k in range(nd)]))
    X = J(g.x[wte.node], dx[:, wte.node, :])
    CDi = _trefftz(wte.lines, wte.closed, X, mw, Vj) / S
    return float(CL.v), float(CDi.v), CL.d.copy(), CDi.d.copy()


def source_velocity_jacobian(a, b, c, x, wrt="x", far=10.0):
    """source_velocity (source_triangle.jl:134-138) of triangle abc at x and its Jacobian (row: component of w,
    column: coordinate of x, or of vertex a with wrt='a') on dual numbers"""
    L = oracle.lib()
    D = ctypes.POINTER(ctypes.c_double)
    L.vpo_dual_source_velocity.argtypes = [D, D, ctypes.c_int, ctypes.c_double, D, D]
    L.vpo_dual_source_velocity.restype = ctypes.c_int
    abc, pabc = oracle._d(np.concatenate([a, b, c]))
    xx, px = oracle._d(x)
    w, pw = oracle._d(np.zeros(3))
    Jm, pJ = oracle._d(np.zeros((3, 3)))
    if L.vpo_dual_source_velocity(pabc, px, 0 if wrt == "x" else 1, far, pw, pJ) != 0:
        raise ValueError("degenerate triangle")
    return w, Jm
