"""Adjoint gradients of the wing loads through the GPU path: dCL/dx, dCDi/dx (all body nodes) and d/dalpha.

The reference obtains derivatives with ForwardDiff duals through its Julia assembly and solve; the GPU path uses the
discrete adjoint of the same equations instead. With the reduced bordered system M q = r (factorize_galerkin) and an
objective J(x, q):

    dJ/dx = dJ/dx|_q - xi' (dM/dx q - dr/dx),    M' [xi; eta] = [dJ/dq; 0],

where the pair-integral part, xi' (dM/dx q - dr/dx) = d/dx [nu' (A mu - b)] with nu = C xi (row values) and
mu = [C q; W q] (column values), is computed on the GPU by vp_adjoint from the pairs' rules (vp_gradient.cu), and
the transposed solve reuses the LU (vp_solve_transposed). The border (one zero-mean row per closed body) adds
nothing: the objectives here do not change when a constant is added to a body's doublet, so eta = 0, and the
multipliers lambda vanish for the compatible right hand sides of a closed body.

The objectives are the reference's loads: CL = F·e_L / S with F = -sum Cp n A of the gradient route
(Post.jl:72-84, forces.jl:11-20) and CDi = D / S of the Trefftz plane (forces.jl:53-81), each with its explicit
derivative written out below (reverse mode by hand). The wake nodes are taken to move with their trailing edge
nodes (rigid wake rows at fixed offsets along a fixed direction).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import D, check, load
from ._vec import cross3, norm3, scatter_add
from .api import (AssemblyOptions, _dp, _ip, assemble, build_elements, default_context, factorize_galerkin,
                  solve_galerkin, source_strengths)


def solve_transposed(F, g):
    """xi of M' [xi; eta] = [g; 0] with the factors F (g: nq, or nq x k)"""
    g = np.asarray(g, float)
    k = 1 if g.ndim == 1 else g.shape[1]
    gg = np.ascontiguousarray(g.reshape(F.nq, k).T).ravel()
    xi = np.zeros(F.nq * k)
    check(F.ctx.h, load().vp_solve_transposed(F.ctx.h, F.h, k, gg.ctypes.data_as(D), xi.ctypes.data_as(D)))
    xi = xi.reshape(k, F.nq).T
    return xi[:, 0] if g.ndim == 1 else xi


def pair_derivatives(g, dm, sigma, V, dV, nu, mu, opts: AssemblyOptions = None, wake=None, ctx=None):
    """d/dx, d/dwx and d/dalpha of nu' (A(x) mu - b(x)) (vp_adjoint) for one adjoint vector nu (nslot) or two
    (nslot x 2, one pass); returns (grad_x, grad_wx, dalpha, stats), with a leading axis of 2 for two vectors"""
    opts = opts or AssemblyOptions()
    ctx = ctx or default_context()
    o = opts.c_struct()
    x, px = _dp(g.x)
    tr, pt = _ip(g.tris)
    cs, pc = _ip(dm.corner_slot)
    tp = np.asarray(g.touch_pairs, np.int32).reshape(-1, 2)
    tpp, ptp = _ip(tp if len(tp) else np.zeros((1, 2), np.int32))
    sg, ps = _dp(sigma)
    VV, pV = _dp(V)
    dVV, pdV = _dp(dV)
    if wake is not None:
        wx, pwx = _dp(wake.x)
        wt, pwt = _ip(wake.tris if len(wake.tris) else np.zeros((1, 3)))
        wf, pwf = _ip(wake.filaments if len(wake.filaments) else np.zeros((1, 2)))
        nw, nwt, nf = wake.x.shape[0], len(wake.tris), len(wake.filaments)
    else:
        wx = wt = wf = None
        pwx, pwt, pwf = None, None, None
        nw = nwt = nf = 0
    nu = np.asarray(nu, float)
    single = nu.ndim == 1
    nv = nu.reshape(dm.nslot, -1)
    k = nv.shape[1]
    if k not in (1, 2):
        raise ValueError("one or two adjoint vectors")
    nuu, pnu = _dp(nv.T.copy().ravel())
    muu, pmu = _dp(mu)
    if muu.shape != (dm.nslot + nw,):
        raise ValueError("mu must have one value per column")
    gx = np.zeros((k, g.nnode, 3))
    gw = np.zeros((k, max(nw, 1), 3))
    dal = np.zeros(k)
    st = _lib.vp_assembly_stats()
    check(ctx.h, load().vp_adjoint(ctx.h, ctypes.byref(o), g.nnode, px, g.ntri, pt, pc, dm.nslot, len(tp), ptp, ps, pV,
                                   nw, pwx, nwt, pwt, nf, pwf, k, pnu, pmu, pdV, gx.ctypes.data_as(D),
                                   gw.ctypes.data_as(D), dal.ctypes.data_as(D), ctypes.byref(st)))
    gw = gw[:, :nw]
    if single:
        return gx[0], gw[0], float(dal[0]), st
    return gx, gw, dal, st


# ---- objectives with their explicit derivatives ------------------------------------------------------------------------

def cl_pressure(g, dm, mu_slot, V, dV, eL, deL, S):
    """CL = F·e_L / S, F = -sum Cp A n, Cp = 1 - |u|^2/|V|^2, u = V - (V·n)n + grad mu (gradient route, Post.jl:72-84,
    forces.jl:11-20). Returns CL, dCL/dmu (slots), dCL/dx at fixed mu (nnode x 3), dCL/dalpha at fixed mu."""
    x, t = g.x, g.tris
    a, b, c = x[t[:, 0]], x[t[:, 1]], x[t[:, 2]]
    nA = cross3(b - a, c - a)
    A2 = norm3(nA)
    n = nA / A2[:, None]
    e = [c - b, a - c, b - a]
    m = np.asarray(mu_slot)[dm.corner_slot]
    G = sum(m[:, k:k + 1] * e[k] for k in range(3))
    i2 = 1.0 / A2 ** 2
    gmu = cross3(nA, G) * i2[:, None]
    Vn = n @ V
    u = V - Vn[:, None] * n + gmu
    V2 = V @ V
    uu = np.einsum("ij,ij->i", u, u)
    cp = 1 - uu / V2
    nAe = nA @ eL
    CL = float(-(cp * nAe).sum() / (2 * S))
    # reverse
    cp_b = -nAe / (2 * S)
    nA_b = -(cp / (2 * S))[:, None] * eL
    u_b = (cp_b * (-2 / V2))[:, None] * u
    n_b = -Vn[:, None] * u_b - np.einsum("ij,ij->i", u_b, n)[:, None] * V
    G_b = cross3(u_b, nA) * i2[:, None]
    trip = np.einsum("ij,ij->i", u_b, gmu)  # u_b·(nA x G) / |nA|^2
    nA_b += cross3(G, u_b) * i2[:, None] - (2 * trip * i2)[:, None] * nA
    m_b = np.stack([np.einsum("ij,ij->i", G_b, e[k]) for k in range(3)], axis=1)
    dmu = scatter_add(dm.nslot, dm.corner_slot, m_b.ravel())
    xa_b, xb_b, xc_b = np.zeros_like(a), np.zeros_like(a), np.zeros_like(a)
    # e_0 = c - b, e_1 = a - c, e_2 = b - a
    for k, (p, q) in enumerate(((2, 1), (0, 2), (1, 0))):
        eb = m[:, k:k + 1] * G_b
        (xa_b, xb_b, xc_b)[p][:] += eb
        (xa_b, xb_b, xc_b)[q][:] -= eb
    nA_b += (n_b - np.einsum("ij,ij->i", n_b, n)[:, None] * n) / A2[:, None]
    u1, u2 = b - a, c - a
    u1_b, u2_b = cross3(u2, nA_b), cross3(nA_b, u1)
    xb_b += u1_b
    xc_b += u2_b
    xa_b -= u1_b + u2_b
    gx = scatter_add(len(x), t.T, np.concatenate([xa_b, xb_b, xc_b]))
    # alpha: V and e_L
    V_b = (u_b - np.einsum("ij,ij->i", u_b, n)[:, None] * n).sum(axis=0) + (cp_b * 2 * uu / V2 ** 2).sum() * V
    Fv = -(cp[:, None] * nA).sum(axis=0) / 2
    dal = float(V_b @ dV + (Fv / S) @ deL)
    return CL, dmu, gx, dal


def _trefftz_parts(wte):
    """per line: segments (i, i+1) and the vortex at every line point with its before / after segments"""
    seg_a, seg_b, vort, before, after = [], [], [], [], []
    for line, closed in zip(wte.lines, wte.closed):
        line = np.asarray(line)
        m = len(line)
        nseg = m if closed else m - 1
        s0 = len(seg_a)
        for i in range(nseg):
            seg_a.append(line[i])
            seg_b.append(line[(i + 1) % m])
        for i in range(m):
            vort.append(line[i])
            before.append(s0 + (i - 1 if i > 0 else nseg - 1) if (i > 0 or closed) else -1)
            after.append(s0 + i if i < nseg else -1)
    return (np.array(seg_a, int), np.array(seg_b, int), np.array(vort, int), np.array(before, int),
            np.array(after, int))


def cdi_trefftz(wte, mu_w, V, dV, S):
    """CDi = D / S with D the Trefftz-plane induced drag in units of q∞ (forces.jl:53-81). Returns CDi, dCDi/dmu_w,
    dCDi/dx of the trailing edge points (nte x 3) and dCDi/dalpha at fixed mu_w."""
    sa, sb, pv, bef, aft = _trefftz_parts(wte)
    if len(sa) == 0:
        return 0.0, np.zeros(len(mu_w)), np.zeros_like(wte.x), 0.0
    mu_w = np.asarray(mu_w, float)
    Vn = np.linalg.norm(V)
    d = V / Vn
    X = wte.x
    P = X - (X @ d)[:, None] * d
    Gs = (mu_w[sa] + mu_w[sb]) / 2
    Gpad = np.append(Gs, 0.0)
    dG = Gpad[aft] - Gpad[bef]
    ua = P[sb] - P[sa]
    cc = (P[sa] + P[sb]) / 2
    r = cc[:, None, :] - P[pv][None, :, :]
    r2 = np.einsum("kpi,kpi->kp", r, r)
    ur = np.einsum("ki,kpi->kp", ua, r)
    h = ur / r2 / (4 * math.pi)
    Dsum = float(Gs @ h @ dG)
    k2 = 2 / (V @ V) / S
    CDi = k2 * Dsum
    # reverse
    Gs_b = k2 * (h @ dG)
    dG_b = k2 * (Gs @ h)
    h_b = k2 * np.outer(Gs, dG) / (4 * math.pi)
    ua_b = np.einsum("kp,kpi->ki", h_b / r2, r)
    r_b = (h_b / r2)[:, :, None] * ua[:, None, :] - (2 * h_b * ur / r2 ** 2)[:, :, None] * r
    cc_b = r_b.sum(axis=1)
    P_b = np.zeros_like(P)
    np.add.at(P_b, pv, -r_b.sum(axis=0))
    np.add.at(P_b, sa, -ua_b + cc_b / 2)
    np.add.at(P_b, sb, ua_b + cc_b / 2)
    x_b = P_b - (P_b @ d)[:, None] * d
    d_b = -((P_b @ d)[:, None] * X + (X @ d)[:, None] * P_b).sum(axis=0)
    mu_b = np.zeros(len(mu_w))
    Gpad_b = np.zeros(len(Gs) + 1)
    np.add.at(Gpad_b, aft, dG_b)
    np.add.at(Gpad_b, bef, -dG_b)
    Gs_b = Gs_b + Gpad_b[:-1]
    np.add.at(mu_b, sa, Gs_b / 2)
    np.add.at(mu_b, sb, Gs_b / 2)
    dd = (dV - (dV @ d) * d) / Vn
    dal = float(d_b @ dd - CDi * 2 * (V @ dV) / (V @ V))
    return CDi, mu_b, x_b, dal


# ---- the whole pipeline ------------------------------------------------------------------------------------------------

def wing_gradients(w, wake, W, alpha, precision="mixed", opts=None, ctx=None, timings=None):
    """CL and CDi of a wing with its rigid wake at angle of attack alpha (radians, |V∞| = 1, lift direction
    e_L = (-sin a, 0, cos a), reference area span x chord) and their gradients with respect to every body node (nnode x
    3) and alpha, through the GPU assembly, factorization, solve and adjoint. Returns a dict."""
    import time
    ctx = ctx or default_context()
    opts = opts or AssemblyOptions(precision=precision)
    g, dm = w.g, w.dm
    V = np.array([math.cos(alpha), 0.0, math.sin(alpha)])
    dV = np.array([-math.sin(alpha), 0.0, math.cos(alpha)])
    eL = dV.copy()
    deL = -V
    S = w.span * w.chord
    t0 = time.perf_counter()
    els = build_elements(g)
    sig = source_strengths(els, V)
    A, b, stats = assemble(g, dm, els, sig, V, wake=wake, opts=opts, ctx=ctx)
    F = factorize_galerkin(dm, A, W=W, precision=precision, ctx=ctx)
    s = solve_galerkin(F, b)
    del A
    q = s["q"]
    mu_slot = dm.C @ q
    mu_w = dm.K @ q
    mu_cols = np.concatenate([mu_slot, W @ q]) if W is not None else mu_slot
    t1 = time.perf_counter()
    CL, dCL_dmu, gCL, aCL = cl_pressure(g, dm, mu_slot, V, dV, eL, deL, S)
    CDi, dCDi_dmuw, gCDi_te, aCDi = cdi_trefftz(dm.wake_te, mu_w, V, dV, S)
    gCDi = np.zeros_like(g.x)
    np.add.at(gCDi, dm.wake_te.node, gCDi_te)
    xi = solve_transposed(F, np.stack([dm.C.T @ dCL_dmu, dm.K.T @ dCDi_dmuw], axis=1))
    del F
    out = dict(CL=CL, CDi=CDi, q=q, stats=stats, cond=s["cond"])
    nu = np.stack([dm.C @ xi[:, 0], dm.C @ xi[:, 1]], axis=1)
    fx, fw, fa, st = pair_derivatives(g, dm, sig, V, dV, nu, mu_cols, opts=opts, wake=wake, ctx=ctx)
    out["adjoint_points"] = dict(zip(("self", "edge", "vertex", "contact", "near", "far"), list(st.points)))
    out["adjoint_points_fp64"] = st.points_fp64
    for name, gx, al, k in (("CL", gCL, aCL, 0), ("CDi", gCDi, aCDi, 1)):
        grad = gx - fx[k]
        if wake is not None and fw.shape[1]:
            np.add.at(grad, dm.wake_te.node[wake.te], -fw[k])
        out["d" + name + "_dx"] = grad
        out["d" + name + "_dalpha"] = al - fa[k]
    if timings is not None:
        timings["forward"] = t1 - t0
        timings["adjoint"] = time.perf_counter() - t1
    return out
