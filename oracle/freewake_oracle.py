"""The free wake's reference restatement: TEST INFRASTRUCTURE ONLY, the checker of the GPU's device-resident
simulation (imported by tests/ and the bench's CPU leg, never by the product path).

FreeWakeSim, step!, run! (src/freewake/step.jl) over the state, vortex elements, conversion and merging of
src/freewake/state.jl, restated in numpy with the reference's data structures (node rows as lists, particles as an
array), and with the oracle's kernels for the work that scales: explicit_rhs (src/assembly/explicit.jl:31-85),
body_velocity (src/post/Post.jl:92-112) and blob_velocities (step.jl:176-187) from the C++ restatement, the body with
its trailing edge panel assembled by the oracle and solved with LAPACK, and the loads of oracle.py.

Blobs are arrays of 7 columns: position (3), strength alpha (3), core delta.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

import oracle as O

# ---- options and core rule (state.jl:1-92) ----------------------------------------------------------------------------


@dataclass
class FreeWakeOptions:
    """FreeWakeOptions (state.jl:25-48): dt; te_len (None: 0.3 |V∞| dt); te_direction ('freestream'); max_rows
    ('auto' or >= 0); merge_rows (1, 'auto' or > 1); core ('auto', 'scaled' or a radius); overlap, core_factor,
    core_floor; advection ('free' or 'freestream'); delete_beyond (spans)."""
    dt: float
    te_len: float | None = None
    te_direction: str = "freestream"
    max_rows: int | str = "auto"
    merge_rows: int | str = 1
    core: str | float = "auto"
    overlap: float = 1.5
    core_factor: float = 1.5
    core_floor: float | None = None
    advection: str = "free"
    delete_beyond: float = math.inf

    def check(self):
        if not self.dt > 0:
            raise ValueError("dt must be positive")
        if not (self.max_rows == "auto" or (isinstance(self.max_rows, int) and self.max_rows >= 0)):
            raise ValueError("max_rows must be 'auto' or at least 0")
        if not (self.merge_rows == "auto" or (isinstance(self.merge_rows, int) and self.merge_rows >= 1)):
            raise ValueError("merge_rows must be 'auto' or at least 1")
        if self.advection not in ("free", "freestream"):
            raise ValueError(f"advection must be 'free' or 'freestream', not {self.advection}")
        if self.te_direction == "bisector":
            raise NotImplementedError("te_direction = 'bisector' needs the trailing edge bisectors, which this DOF map "
                                      "does not carry; use 'freestream'")
        if self.te_direction != "freestream":
            raise ValueError("te_direction must be 'freestream' or 'bisector'")
        if not (self.core in ("auto", "scaled") or (isinstance(self.core, (int, float)) and self.core > 0)):
            raise ValueError(f"core must be 'auto', 'scaled' or a positive number, not {self.core}")
        if not (self.overlap > 0 and self.core_factor > 0):
            raise ValueError("overlap and core_factor must be positive")
        return self


class CoreRule:
    """CoreRule (state.jl:64-92): the core of a triangle's particle (p, q, r) or of a filament's blobs (a, b)"""

    def __init__(self, o: FreeWakeOptions, V):
        self.floor = float(o.core_floor if o.core_floor is not None else np.linalg.norm(V) * o.dt)
        self.overlap, self.factor = float(o.overlap), float(o.core_factor)
        self.mode = "fixed" if isinstance(o.core, (int, float)) else o.core
        self.value = float(o.core) if self.mode == "fixed" else 0.0

    def tri(self, p, q, r):
        if self.mode == "fixed":
            return self.value
        if self.mode == "auto":
            return self.overlap * max(np.linalg.norm(q - p), np.linalg.norm(r - q), np.linalg.norm(p - r)) / 2
        return max(self.factor * math.sqrt(np.linalg.norm(np.cross(q - p, r - p))), self.floor)

    def seg(self, a, b):
        if self.mode == "fixed":
            return self.value
        if self.mode == "auto":
            return self.overlap * np.linalg.norm(b - a) / 2
        return max(self.factor * np.linalg.norm(b - a) / 2, self.floor)


@dataclass
class Topology:
    """Strips (A, B) of neighbouring wake trailing edge nodes and the end nodes of open lines (state.jl:99-121)"""
    nte: int
    segments: list
    first_nodes: list
    last_nodes: list

    @staticmethod
    def of(dm):
        wte = dm.wake_te
        segs, firsts, lasts = [], [], []
        for line, closed in zip(wte.lines, wte.closed):
            line = [int(v) for v in line]
            m = len(line)
            segs += [(line[i], line[i + 1]) for i in range(m - 1)]
            if closed:
                segs.append((line[m - 1], line[0]))
            else:
                firsts.append(line[0])
                lasts.append(line[m - 1])
        return Topology(len(wte.node), segs, firsts, lasts)


# ---- state and vortex elements (state.jl:132-369) ----------------------------------------------------------------------


@dataclass
class FreeWakeState:
    """Node rows x from the newest to the oldest, the doublets mu they were shed with, mu_line, particles (N x 7),
    conversions and the merge bookkeeping (state.jl:132-147)"""
    nte: int
    nstrips: int = 0
    x: list = field(default_factory=list)
    mu: list = field(default_factory=list)
    mu_line: np.ndarray = None
    particles: np.ndarray = None
    conversions: int = 0
    tag: np.ndarray = None
    group: np.ndarray = None
    batch_rows: np.ndarray = None
    batch_length: np.ndarray = None
    batch_width: np.ndarray = None

    def __post_init__(self):
        self.mu_line = np.zeros(self.nte)
        self.particles = np.zeros((0, 7))
        self.tag = np.zeros(0, int)
        self.group = np.zeros(0, np.int8)
        self.batch_rows = np.zeros(self.nstrips, int)
        self.batch_length = np.zeros(self.nstrips)
        self.batch_width = np.zeros(self.nstrips)

    def keep_particles(self, keep):
        self.particles = self.particles[keep]
        self.tag = self.tag[keep]
        self.group = self.group[keep]

    def to_arrays(self) -> dict:
        """the state as named arrays (a checkpoint; the reference keeps it in memory only)"""
        nr = len(self.x)
        return {"nte": np.array(self.nte), "nstrips": np.array(self.nstrips),
                "x": np.array(self.x).reshape(nr, self.nte, 3), "mu": np.array(self.mu).reshape(nr, self.nte),
                "mu_line": self.mu_line, "particles": self.particles, "conversions": np.array(self.conversions),
                "tag": self.tag, "group": self.group, "batch_rows": self.batch_rows,
                "batch_length": self.batch_length, "batch_width": self.batch_width}

    @classmethod
    def from_arrays(cls, d) -> "FreeWakeState":
        st = cls(int(d["nte"]), int(d["nstrips"]))
        st.x = [np.array(r, float) for r in d["x"]]
        st.mu = [np.array(r, float) for r in d["mu"]]
        st.conversions = int(d["conversions"])
        for k in ("mu_line", "particles", "tag", "group", "batch_rows", "batch_length", "batch_width"):
            setattr(st, k, np.array(d[k]))
        return st


def _nondegenerate(p, q, r):
    return np.linalg.norm(np.cross(q - p, r - p)) > 1e-12 * max((q - p) @ (q - p), (r - p) @ (r - p), (r - q) @ (r - q))


class WakeElements:
    """Triangles (corners, corner doublets; the nondegenerate ones also as sheets for the right hand side) and filament
    segments with their end circulations (state.jl:162-200)"""

    def __init__(self):
        self.corners, self.corner_mu, self.sheets, self.sheet_mu, self.segments, self.segment_g = [], [], [], [], [], []

    def add_sheet(self, p, q, r, mp, mq, mr):
        self.corners.append((p, q, r))
        self.corner_mu.append((mp, mq, mr))
        if _nondegenerate(p, q, r):
            self.sheets.append((p, q, r))
            self.sheet_mu.append((mp, mq, mr))

    def add_segment(self, a, b, ga, gb):
        self.segments.append((a, b))
        self.segment_g.append((ga, gb))


def panel_row(e, st, topo, i):
    """sheets and tip sides of the panel row between node rows i and i + 1 (state.jl:203-218), 0-based"""
    x0, x1, m0, m1 = st.x[i], st.x[i + 1], st.mu[i], st.mu[i + 1]
    for A, B in topo.segments:
        e.add_sheet(x0[A], x1[A], x0[B], m0[A], m1[A], m0[B])
        e.add_sheet(x1[A], x1[B], x0[B], m1[A], m1[B], m0[B])
    for k in topo.first_nodes:
        e.add_segment(x1[k], x0[k], m1[k], m0[k])
    for k in topo.last_nodes:
        e.add_segment(x0[k], x1[k], m0[k], m1[k])


def far_end(e, st, topo, i):
    """the far end filament along node row i, B -> A, strength mu - mu_line (state.jl:221-230)"""
    x, mu = st.x[i], st.mu[i]
    for A, B in topo.segments:
        gA, gB = mu[A] - st.mu_line[A], mu[B] - st.mu_line[B]
        if gA == 0 and gB == 0:
            continue
        e.add_segment(x[B], x[A], gB, gA)


def vortex_elements(st: FreeWakeState, topo: Topology):
    """the free wake's vortex elements (state.jl:241-253)"""
    e = WakeElements()
    nr = len(st.x)
    for i in range(nr - 1):
        panel_row(e, st, topo, i)
    if nr >= 1:
        for A, B in topo.segments:
            e.add_segment(st.x[0][A], st.x[0][B], st.mu[0][A], st.mu[0][B])
        far_end(e, st, topo, nr - 1)
    return e


def rigid_elements(w, mu_w):
    """vortex elements of a rigid wake with the doublets mu_w of its trailing edge nodes (state.jl:256-265)"""
    e = WakeElements()
    mn = np.asarray(mu_w)[w.te]
    for t in w.tris:
        e.add_sheet(w.x[t[0]], w.x[t[1]], w.x[t[2]], mn[t[0]], mn[t[1]], mn[t[2]])
    for a, b in w.filaments:
        e.add_segment(w.x[a], w.x[b], mn[a], mn[b])
    return e


def sheet_vorticity(p, q, r, mu):
    """gamma A = sum over edges of (mu_a + mu_b)/2 (x_b - x_a) (state.jl:272)"""
    return ((mu[0] + mu[1]) * (q - p) + (mu[1] + mu[2]) * (r - q) + (mu[2] + mu[0]) * (p - r)) / 2


_GS = 1 / (2 * math.sqrt(3))


def segment_blobs(a, b, ga, gb, delta):
    """two blobs at the 2-point Gauss positions of a filament (blob.jl:31-38)"""
    out = []
    for xi in (0.5 - _GS, 0.5 + _GS):
        al = (((1 - xi) * ga + xi * gb) / 2) * (b - a)
        out.append(np.concatenate([a + xi * (b - a), al, [delta]]))
    return out


def free_wake_blobs(e: WakeElements, core: CoreRule):
    """blob representation of vortex elements (state.jl:275-295)"""
    rows = []
    for (p, q, r), mu in zip(e.corners, e.corner_mu):
        rows.append(np.concatenate([(p + q + r) / 3, sheet_vorticity(p, q, r, mu), [core.tri(p, q, r)]]))
    for (a, b), (ga, gb) in zip(e.segments, e.segment_g):
        rows += segment_blobs(a, b, ga, gb, core.seg(a, b))
    return np.array(rows).reshape(-1, 7)


def convert_oldest(st: FreeWakeState, topo: Topology, core: CoreRule, merge=None):
    """convert the oldest panel row into particles (state.jl:300-343); returns the number created"""
    nr = len(st.x)
    if nr < 2:
        return 0
    e = WakeElements()
    panel_row(e, st, topo, nr - 2)
    far_end(e, st, topo, nr - 1)
    blobs = free_wake_blobs(e, core)
    tag, group = np.zeros(len(blobs), int), np.zeros(len(blobs), np.int8)
    if merge is not None:
        up, down = st.x[nr - 2], st.x[nr - 1]
        for s, (A, B) in enumerate(topo.segments):
            k = merge[s]
            if k <= 1:
                continue
            m = k - st.batch_rows[s]
            for h, (u, v) in enumerate(((1 / 3, 1 / 3), (2 / 3, 2 / 3))):
                tag[2 * s + h] = s + 1
                group[2 * s + h] = 1 if u + (m - 1 + v) / k < 1 else 2
            st.batch_rows[s] += 1
            st.batch_length[s] += (np.linalg.norm(down[A] - up[A]) + np.linalg.norm(down[B] - up[B])) / 2
            st.batch_width[s] = np.linalg.norm(up[B] - up[A])
    st.particles = np.vstack([st.particles, blobs])
    st.tag = np.concatenate([st.tag, tag])
    st.group = np.concatenate([st.group, group])
    st.mu_line = st.mu[nr - 2].copy()
    st.x.pop()
    st.mu.pop()
    st.conversions += 1
    if merge is not None:
        for s in range(len(topo.segments)):
            if merge[s] > 1 and st.batch_rows[s] >= merge[s]:
                merge_strip(st, s, core)
    return len(blobs)


def merge_strip(st: FreeWakeState, s: int, core: CoreRule):
    """merge strip s's batch into one particle pair (state.jl:352-373)"""
    idx = np.flatnonzero(st.tag == s + 1)
    o = np.zeros(3)
    delta = core.tri(o, o + np.array([st.batch_width[s], 0, 0]), o + np.array([st.batch_width[s], st.batch_length[s], 0]))
    merged = []
    for g in (1, 2):
        sel = idx[st.group[idx] == g]
        if len(sel) == 0:
            continue
        al = st.particles[sel, 3:6].sum(axis=0)
        w = np.linalg.norm(st.particles[sel, 3:6], axis=1)
        x = (w[:, None] * st.particles[sel, :3]).sum(axis=0) / w.sum() if w.sum() > 0 else st.particles[sel, :3].mean(axis=0)
        merged.append(np.concatenate([x, al, [delta]]))
    st.keep_particles(st.tag != s + 1)
    if merged:
        st.particles = np.vstack([st.particles, np.array(merged)])
        st.tag = np.concatenate([st.tag, np.zeros(len(merged), int)])
        st.group = np.concatenate([st.group, np.zeros(len(merged), np.int8)])
    st.batch_rows[s] = 0
    st.batch_length[s] = 0.0


def vorticity_moments(blobs):
    """total vorticity and impulse of a set of blobs (state.jl:381-385)"""
    b = np.asarray(blobs).reshape(-1, 7)
    return b[:, 3:6].sum(axis=0), np.cross(b[:, :3], b[:, 3:6]).sum(axis=0) / 2


# ---- the oracle's kernels ---------------------------------------------------------------------------------------------

def _lib():
    lib = O.lib()
    if not getattr(lib, "_fw_bound", False):
        D = ctypes.POINTER(ctypes.c_double)
        I = ctypes.POINTER(ctypes.c_int)
        lib.vpo_explicit_rhs.argtypes = [ctypes.POINTER(O._Opts), D, ctypes.c_int, I, I, ctypes.c_int, D, D,
                                         ctypes.c_int, D, D, ctypes.c_int, D, D, ctypes.c_int]
        lib.vpo_body_velocity.argtypes = [D, ctypes.c_int, D, D, ctypes.c_double, ctypes.c_int, D, D, ctypes.c_int]
        lib.vpo_blob_velocities.argtypes = [ctypes.c_int, D, ctypes.c_int, D, D, ctypes.c_int]
        lib._fw_bound = True
    return lib


def explicit_rhs(g, dm, e: WakeElements, blobs, nthreads=0, **kw):
    """-int psi_i n.u dA of the known sheets, filaments and particles per slot (explicit.jl:31-85)"""
    o = O.options(**kw)
    x, px = O._d(g.x)
    tr, pt = O._i(g.tris)
    cs, pc = O._i(dm.corner_slot)
    sx, psx = O._d(np.array([np.concatenate(t) for t in e.sheets]).reshape(-1, 9) if e.sheets else np.zeros((1, 9)))
    sm, psm = O._d(np.array(e.sheet_mu, float).reshape(-1, 3) if e.sheets else np.zeros((1, 3)))
    fx, pfx = O._d(np.array([np.concatenate(s) for s in e.segments]).reshape(-1, 6) if e.segments else np.zeros((1, 6)))
    fg, pfg = O._d(np.array(e.segment_g, float).reshape(-1, 2) if e.segments else np.zeros((1, 2)))
    b = np.asarray(blobs, float).reshape(-1, 7)
    bb, pb = O._d(b if len(b) else np.zeros((1, 7)))
    rhs, prhs = O._d(np.zeros(dm.nslot))
    if _lib().vpo_explicit_rhs(ctypes.byref(o), px, g.ntri, pt, pc, len(e.sheets), psx, psm, len(e.segments), pfx,
                               pfg, len(b), pb, prhs, nthreads) != 0:
        raise ValueError("degenerate triangle")
    return rhs


def body_velocity(g, sigma, gamma, X, kernel_far=10.0, nthreads=0):
    """sigma_s w_s + gamma_s x w_s of the body's triangles at the points X (Post.jl:92-112)"""
    c, pc = O._d(g.x[g.tris].reshape(-1, 9))
    sg, ps = O._d(sigma)
    gm, pg = O._d(np.asarray(gamma, float).reshape(-1, 3))
    xx, px = O._d(np.asarray(X, float).reshape(-1, 3))
    U, pU = O._d(np.zeros_like(xx))
    if _lib().vpo_body_velocity(pc, g.ntri, ps, pg, kernel_far, len(xx), px, pU, nthreads) != 0:
        raise ValueError("degenerate triangle")
    return U


def blob_velocities(blobs, X, nthreads=0):
    """velocity of the blobs at every point of X (step.jl:176-187)"""
    b, pb = O._d(np.asarray(blobs, float).reshape(-1, 7) if len(blobs) else np.zeros((1, 7)))
    xx, px = O._d(np.asarray(X, float).reshape(-1, 3))
    U, pU = O._d(np.zeros_like(xx))
    _lib().vpo_blob_velocities(len(np.asarray(blobs).reshape(-1, 7)), pb, len(xx), px, pU, nthreads)
    return U


# ---- the simulation (step.jl) ----------------------------------------------------------------------------------------

def _corner_slot_values(dm, mu):
    return np.asarray(mu)[dm.corner_slot]


def sheet_strengths(els, dm, mu):
    """the vortex sheet gamma of every triangle: sum_b mu_b gamma_b (Post.jl:19-23), from oracle.elements"""
    m = _corner_slot_values(dm, mu)
    return sum(m[:, k:k + 1] * els["gam"][k] for k in range(3))


class FreeWakeSim:
    """FreeWakeSim(g, dm, V; opts, assembly) (step.jl:8-58) with step() and run(n) (step.jl:113-216), on the oracle"""

    def __init__(self, g, dm, V, opts: FreeWakeOptions, nthreads=0, **assembly):
        from vortexpanel_gpu import meshes
        opts.check()
        self.g, self.dm, self.V = g, dm, np.asarray(V, float)
        self.opts, self.kw, self.nthreads = opts, assembly, nthreads
        self.kernel_far = assembly.get("kernel_far", 10.0)
        self.els = O.elements(g)
        self.sigma = O.source_strengths(g, self.V)
        te_len = opts.te_len if opts.te_len is not None else 0.3 * np.linalg.norm(self.V) * opts.dt
        self.te = meshes.te_panel(g, dm, self.V, length=te_len)
        A, self.b0, _ = O.assemble(g, dm, self.sigma, self.V, wake=self.te, nthreads=nthreads, **assembly)
        self.F = O.factorize_galerkin(dm, A, W=meshes.wake_rows(dm, self.te.te))
        del A
        self.topo = Topology.of(dm)
        nte = self.topo.nte
        self.edge = self.te.x[nte:2 * nte].copy()
        self.core = CoreRule(opts, self.V)
        row = np.linalg.norm(self.V) * opts.dt
        if opts.max_rows == "auto":
            self.keep_rows = rows_for_distance(self.core, self.edge, self.topo, 3, self.te.rows[1], row)
        else:
            self.keep_rows = int(opts.max_rows)
        widths = [np.linalg.norm(self.edge[B] - self.edge[A]) for A, B in self.topo.segments]
        if opts.merge_rows == "auto":
            self.merge = [max(1, int(round(w / row))) for w in widths]
        elif opts.merge_rows == 1:
            self.merge = None
        else:
            self.merge = [int(opts.merge_rows)] * len(widths)
        self.state = FreeWakeState(nte, len(self.topo.segments))
        self.n, self.t = 0, 0.0
        self.mu = np.zeros(dm.nslot)
        self.mu_w = np.zeros(nte)
        self.cp = np.zeros(g.ntri)
        self.I_prev = np.zeros(3)
        self.history = []

    def _te_blobs(self, mu_w):
        return free_wake_blobs(rigid_elements(self.te, mu_w), self.core)

    def step(self):
        """one time step in MESA's order (step.jl:113-146); returns the step's record"""
        st, o, dm = self.state, self.opts, self.dm
        we = vortex_elements(st, self.topo)
        rhs = explicit_rhs(self.g, dm, we, st.particles, nthreads=self.nthreads, **self.kw)
        sol = O.solve_factored(self.F, self.b0 + rhs)
        mu_w = dm.K @ sol["q"]
        loads = self._loads(sol, mu_w, we)
        if not st.x:
            st.x.append(self.edge.copy())
            st.mu.append(mu_w.copy())
        X = np.vstack(st.x + [st.particles[:, :3]])
        U = self._velocities(sol, mu_w, we, X)
        nrow = sum(len(r) for r in st.x)
        k = 0
        for r in st.x:
            r += o.dt * U[k:k + len(r)]
            k += len(r)
        st.particles[:, :3] += o.dt * U[nrow:]
        st.x.insert(0, self.edge.copy())
        st.mu.insert(0, mu_w.copy())
        while len(st.x) - 1 > self.keep_rows:
            convert_oldest(st, self.topo, self.core, self.merge)
        if math.isfinite(o.delete_beyond):
            d = self.V / np.linalg.norm(self.V)
            limit = (self.edge @ d).max() + o.delete_beyond * self.te.span
            st.keep_particles(st.particles[:, :3] @ d <= limit)
        rec = dict(n=self.n, t=self.t, **loads, rows=len(st.x) - 1, particles=len(st.particles),
                   lam=float(np.atleast_1d(sol["lam"])[0]) if np.size(sol["lam"]) else 0.0,
                   umax=float(np.linalg.norm(U, axis=1).max()) if len(U) else 0.0)
        self.history.append(rec)
        self.mu, self.mu_w = sol["mu"], mu_w
        self.n += 1
        self.t += o.dt
        return rec

    def _loads(self, sol, mu_w, we):
        """the loads of the solved state (step.jl:149-163)"""
        dm, els, V = self.dm, self.els, self.V
        u = O.gradient_velocity(self.g, dm, sol["mu"], V, els=els)
        dmu = np.zeros(dm.nslot) if self.n == 0 else (sol["mu"] - self.mu) / self.opts.dt
        cp = O.pressure_coefficient(u, V, _corner_slot_values(dm, dmu).mean(axis=1))
        self.cp = cp
        Fp, Mp = O.pressure_force(els, cp)
        Fkj = O.kutta_joukowski_force(dm.wake_te, mu_w, V)
        gam = sheet_strengths(els, dm, sol["mu"])
        body = np.hstack([els["centroid"], gam * els["area"][:, None], np.zeros((len(els["area"]), 1))])
        blobs = np.vstack([body, self._te_blobs(mu_w), free_wake_blobs(we, self.core), self.state.particles])
        Om, I = vorticity_moments(blobs)
        Fimp = np.full(3, np.nan) if self.n == 0 else -(2 / (V @ V)) * (I - self.I_prev) / self.opts.dt
        self.I_prev = I
        return dict(mu_w=mu_w, F_pressure=Fp, M_pressure=Mp, F_kj=Fkj, F_impulse=Fimp, Omega=Om, I=I)

    def _velocities(self, sol, mu_w, we, X):
        """V + the body (exact kernels) + every wake element as blobs at the points X (step.jl:166-173)"""
        V = self.V
        if self.opts.advection == "freestream":
            return np.tile(V, (len(X), 1))
        gam = sheet_strengths(self.els, self.dm, sol["mu"])
        ub = body_velocity(self.g, self.sigma, gam, X, kernel_far=self.kernel_far, nthreads=self.nthreads)
        blobs = np.vstack([self._te_blobs(mu_w), free_wake_blobs(we, self.core), self.state.particles])
        uw = blob_velocities(blobs, X, nthreads=self.nthreads)
        return V + ub + uw

    def run(self, nsteps, progress=None):
        """take nsteps steps (step.jl:205-216); returns the history"""
        for _ in range(nsteps):
            rec = self.step()
            if progress is not None:
                progress(self, rec)
        return self.history


def first_core(core, edge, topo, row):
    """the core of the widest strip's first particles (step.jl:68-73)"""
    w = max(np.linalg.norm(edge[B] - edge[A]) for A, B in topo.segments)
    o = np.zeros(3)
    return core.tri(o, o + np.array([w, 0, 0]), o + np.array([w, row, 0]))


def rows_for_distance(core, edge, topo, cores, te_len, row):
    """the fewest rows that create the first particles at least `cores` cores behind the trailing edge
    (step.jl:80-82)"""
    return max(0, math.ceil((cores * first_core(core, edge, topo, row) - te_len) / row - 0.5))
