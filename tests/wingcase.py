"""Helpers of the wing tests: the jittered wing (no corner at a switch of the vertex rule), moved copies with their
rigid wake, and the FP64 forward loads through the public API."""
import dataclasses
import math

import numpy as np

from vortexpanel_gpu import api, meshes


def corner_angles(g):
    x, t = g.x, g.tris
    out = []
    for k in range(3):
        u = x[t[:, (k + 1) % 3]] - x[t[:, k]]
        v = x[t[:, (k + 2) % 3]] - x[t[:, k]]
        c = np.einsum("ij,ij->i", u, v) / (np.linalg.norm(u, axis=1) * np.linalg.norm(v, axis=1))
        out.append(np.degrees(np.arccos(np.clip(c, -1, 1))))
    return np.concatenate(out)


def jittered(w, amount=2e-3, seed=20):
    """The wing with its nodes moved in x and y by up to `amount` chords: the extruded wing's quads have corners of
    exactly 90 degrees, where the vertex rule switches from one piece to wedges (assemble.jl:102-125), so that the
    discrete loads jump under a rounding-level move and finite differences across the switch mean nothing"""
    rng = np.random.default_rng(seed)
    x = w.g.x.copy()
    x[:, :2] += rng.uniform(-amount, amount, (len(x), 2)) * w.chord
    w = dataclasses.replace(w, g=dataclasses.replace(w.g, x=x))
    te = w.dm.wake_te
    return dataclasses.replace(w, dm=dataclasses.replace(w.dm, wake_te=meshes.WakeTE(te.node, x[te.node].copy(),
                                                                                      te.lines, te.closed)))


def moved(w, wake, x):
    """the wing with its nodes at x; the wake rows keep their offsets from the trailing edge nodes"""
    wte = w.dm.wake_te
    te = meshes.WakeTE(wte.node, x[wte.node].copy(), wte.lines, wte.closed)
    d = np.array([1.0, 0.0, 0.0])
    wk = dataclasses.replace(wake, x=te.x[wake.te] + wake.rows[wake.row][:, None] * d)
    return dataclasses.replace(w, g=dataclasses.replace(w.g, x=x), dm=dataclasses.replace(w.dm, wake_te=te)), wk


def loads(w, wake, W, a, precision="fp64"):
    """CL (pressure route) and CDi (Trefftz) of the wing at angle of attack a through assemble, factorize, solve"""
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    eL = np.array([-math.sin(a), 0.0, math.cos(a)])
    els = api.build_elements(w.g)
    sig = api.source_strengths(els, V)
    opts = api.AssemblyOptions(precision=precision)
    A, b, _ = api.assemble(w.g, w.dm, els, sig, V, wake=wake, opts=opts)
    s = api.solve_galerkin(api.factorize_galerkin(w.dm, A, W=W, precision=precision), b)
    del A
    S = w.span * w.chord
    F = api.surface_loads(els, w.dm, s["mu"], V)["F"]
    return float(F @ eL / S), float(api.trefftz_drag(w.dm.wake_te, w.dm.K @ s["q"], V) / S)


def jittered_rel(w, rel=0.02, seed=20):
    """The wing with each node moved in x and y by up to `rel` times its shortest edge (meshes with cosine spacing
    have edges far shorter than a fixed jitter near the leading and trailing edges)"""
    x, t = w.g.x, w.g.tris
    h = np.full(len(x), np.inf)
    for a, b in ((0, 1), (1, 2), (2, 0)):
        L = np.linalg.norm(x[t[:, b]] - x[t[:, a]], axis=1)
        np.minimum.at(h, t[:, a], L)
        np.minimum.at(h, t[:, b], L)
    rng = np.random.default_rng(seed)
    x = x.copy()
    x[:, :2] += rng.uniform(-rel, rel, (len(x), 2)) * h[:, None]
    w = dataclasses.replace(w, g=dataclasses.replace(w.g, x=x))
    te = w.dm.wake_te
    return dataclasses.replace(w, dm=dataclasses.replace(w.dm, wake_te=meshes.WakeTE(te.node, x[te.node].copy(),
                                                                                      te.lines, te.closed)))


def clear_nodes(g, margin=0.05, switches=(90.0, 150.0)):
    """nodes whose triangles' corners all lie more than `margin` degrees from a switch of the vertex rule's wedge
    count (assemble.jl:102-125): a move of one of them by a finite-difference step changes no rule"""
    t = g.tris
    ang = corner_angles(g).reshape(3, -1).T  # (ntri, 3)
    bad_tri = np.zeros(len(t), bool)
    for s in switches:
        bad_tri |= (np.abs(ang - s) <= margin).any(axis=1)
    bad = np.zeros(g.nnode, bool)
    for k in range(3):
        bad[t[bad_tri, k]] = True
    return np.flatnonzero(~bad)
