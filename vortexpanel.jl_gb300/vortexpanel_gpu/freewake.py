"""Free wake with vortex particles: FreeWakeSim, step!, run! (src/freewake/step.jl) as a simulation resident on the GPU.

The host resolves the options as the reference does (te_len, max_rows, merge_rows, the core rule, delete_beyond;
src/freewake/state.jl:25-92, step.jl:35-58), builds the trailing edge panel, assembles the body with it and factors
the bordered matrix once (assemble, factorize_galerkin). vp_freewake_create then takes the body, the factors, the DOF
map and the wake's topology, and every step (vp_freewake_step) runs on the device with no allocation: the free wake's
elements, explicit_rhs through the assembly's tiers, the solve, the loads, the velocities (body kernels and the blob
N-body sum), forward Euler, shedding, conversion of the oldest row into particles with merging, and deletion. The
host receives the step's record.

The one-shot entries blob_velocities, body_velocity and explicit_rhs evaluate the same kernels on host arrays.
Blobs are arrays of 7 columns: position (3), strength alpha (3), core delta.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib, api, meshes
from ._lib import D, I, check, load

# ---- options (state.jl:25-48) and their resolution ---------------------------------------------------------------


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
        """check_options (state.jl:50-60): ValueError for the reference's ArgumentError"""
        if not self.dt > 0:
            raise ValueError("dt must be positive")
        if self.max_rows != "auto" and not (isinstance(self.max_rows, int) and self.max_rows >= 0):
            raise ValueError("max_rows must be 'auto' or at least 0")
        if self.merge_rows != "auto" and not (isinstance(self.merge_rows, int) and self.merge_rows >= 1):
            raise ValueError("merge_rows must be 'auto' or at least 1")
        if self.advection not in ("free", "freestream"):
            raise ValueError(f"advection must be 'free' or 'freestream', not {self.advection}")
        if self.te_direction == "bisector":
            raise NotImplementedError("te_direction = 'bisector' needs the trailing edge bisectors, which this DOF map "
                                      "does not carry; use 'freestream'")
        if self.te_direction != "freestream":
            raise ValueError("te_direction must be 'freestream' or 'bisector'")
        if isinstance(self.core, str):
            if self.core not in ("auto", "scaled"):
                raise ValueError(f"core must be 'auto', 'scaled' or a positive number, not {self.core}")
        elif not self.core > 0:
            raise ValueError(f"core must be 'auto', 'scaled' or a positive number, not {self.core}")
        if not (self.overlap > 0 and self.core_factor > 0):
            raise ValueError("overlap and core_factor must be positive")
        return self


_CORE_MODES = {"auto": 0, "scaled": 1}


def core_params(o: FreeWakeOptions, V):
    """the CoreRule (state.jl:64-92) as (mode, overlap, factor, floor, value): mode 0 auto, 1 scaled, 2 fixed; the
    floor defaults to |V∞| dt"""
    floor = float(o.core_floor if o.core_floor is not None else np.linalg.norm(V) * o.dt)
    if isinstance(o.core, str):
        return _CORE_MODES[o.core], float(o.overlap), float(o.core_factor), floor, 0.0
    return 2, float(o.overlap), float(o.core_factor), floor, float(o.core)


def core_of_quad(params, width, length):
    """the rule's core of a triangle of a width x length quad: (w,0,0), (w,l,0) from the origin, as the reference
    sizes the first particles and merged batches (step.jl:68-73, state.jl:360)"""
    mode, overlap, factor, floor, value = params
    if mode == 2:
        return value
    if mode == 0:
        return overlap * max(width, length, math.hypot(width, length)) / 2
    return max(factor * math.sqrt(width * length), floor)


@dataclass
class Topology:
    """the wake's strips (A, B) of neighbouring trailing edge nodes (closed lines wrap around) and the end nodes of
    open lines (state.jl:99-121)"""
    nte: int
    strips: list
    first_nodes: list
    last_nodes: list

    @staticmethod
    def of(dm):
        wte = dm.wake_te
        strips, firsts, lasts = [], [], []
        for line, closed in zip(wte.lines, wte.closed):
            line = [int(v) for v in line]
            strips += list(zip(line[:-1], line[1:]))
            if closed:
                strips.append((line[-1], line[0]))
            else:
                firsts.append(line[0])
                lasts.append(line[-1])
        return Topology(len(wte.node), strips, firsts, lasts)


# ---- one-shot device entries ---------------------------------------------------------------------------------------

_PREC = {"fp64": _lib.VP_FP64, "mixed": _lib.VP_MIXED}


@dataclass
class ExplicitSources:
    """ExplicitSources (explicit.jl:10-18) as arrays: sheets (n x 9 corners) with their corner doublets (n x 3),
    filament segments (n x 6 ends) with their end circulations (n x 2), and blobs (n x 7)"""
    sheets: np.ndarray = field(default_factory=lambda: np.zeros((0, 9)))
    sheet_mu: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    segments: np.ndarray = field(default_factory=lambda: np.zeros((0, 6)))
    segment_gamma: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))
    blobs: np.ndarray = field(default_factory=lambda: np.zeros((0, 7)))


def blob_velocities(blobs, X, precision="fp64", ctx=None):
    """velocity of the blobs at every point of X (step.jl:176-187), on the GPU"""
    ctx = ctx or api.default_context()
    b = np.ascontiguousarray(np.asarray(blobs, float).reshape(-1, 7))
    x = np.ascontiguousarray(np.asarray(X, float).reshape(-1, 3))
    U = np.zeros_like(x)
    check(ctx.h, load().vp_blob_velocities(ctx.h, _PREC[precision], len(b), b.ctypes.data_as(D), len(x),
                                          x.ctypes.data_as(D), U.ctypes.data_as(D)))
    return U


def body_velocity(g, sigma, gamma, X, kernel_far=10.0, precision="fp64", ctx=None):
    """sigma_s w_s + gamma_s x w_s of the body's triangles at the points X (Post.jl:92-112), on the GPU"""
    ctx = ctx or api.default_context()
    c = np.ascontiguousarray(g.x[g.tris].reshape(-1, 9))
    sg = np.ascontiguousarray(np.asarray(sigma, float))
    gm = np.ascontiguousarray(np.asarray(gamma, float).reshape(-1, 3))
    x = np.ascontiguousarray(np.asarray(X, float).reshape(-1, 3))
    U = np.zeros_like(x)
    check(ctx.h, load().vp_body_velocity(ctx.h, _PREC[precision], len(c), c.ctypes.data_as(D), sg.ctypes.data_as(D),
                                        gm.ctypes.data_as(D), kernel_far, len(x), x.ctypes.data_as(D),
                                        U.ctypes.data_as(D)))
    return U


def explicit_rhs(g, dm, src: ExplicitSources, opts: api.AssemblyOptions = None, ctx=None):
    """-int psi_i n.u dA of known sheets, filaments and particles per slot (explicit.jl:31-85), on the GPU"""
    opts = opts or api.AssemblyOptions()
    ctx = ctx or api.default_context()
    o = opts.c_struct()
    x, px = api._dp(g.x)
    tr, pt = api._ip(g.tris)
    cs, pc = api._ip(dm.corner_slot)
    sx, psx = api._dp(np.asarray(src.sheets, float).reshape(-1, 9))
    sm, psm = api._dp(np.asarray(src.sheet_mu, float).reshape(-1, 3))
    fx, pfx = api._dp(np.asarray(src.segments, float).reshape(-1, 6))
    fg, pfg = api._dp(np.asarray(src.segment_gamma, float).reshape(-1, 2))
    b, pb = api._dp(np.asarray(src.blobs, float).reshape(-1, 7))
    rhs = np.zeros(dm.nslot)
    check(ctx.h, load().vp_explicit_rhs(ctx.h, ctypes.byref(o), g.nnode, px, g.ntri, pt, pc, dm.nslot, len(sx), psx,
                                       psm, len(fx), pfx, pfg, len(b), pb, rhs.ctypes.data_as(D)))
    return rhs


# ---- the device-resident simulation ----------------------------------------------------------------------------------

vp_freewake_setup, vp_freewake_record, vp_freewake_counts = (_lib.vp_freewake_setup, _lib.vp_freewake_record,
                                                              _lib.vp_freewake_counts)


@dataclass
class WakeState:
    """the device state as host arrays (FreeWakeState, state.jl:132-147): node rows x and their doublets mu, newest
    first, mu_line, particles (N x 7), conversions, and the merge bookkeeping"""
    x: list
    mu: list
    mu_line: np.ndarray
    particles: np.ndarray
    conversions: int
    tag: np.ndarray
    group: np.ndarray
    batch_rows: np.ndarray
    batch_length: np.ndarray
    batch_width: np.ndarray


class FreeWakeSim:
    """FreeWakeSim(g, dm, V∞; opts, assembly) (step.jl:35-58) with step() and run(n) (step.jl:113-216). The state lives
    on the GPU; `state` copies it to the host. `capacity` sizes the particle arrays up front (they grow by
    reallocation between steps when a step could overflow them)."""

    def __init__(self, g, dm, V, opts: FreeWakeOptions, assembly: api.AssemblyOptions = None, ctx=None,
                 capacity: int = 4096):
        opts.check()
        self.g, self.dm, self.V = g, dm, np.asarray(V, float)
        self.opts = opts
        self.assembly = assembly or api.AssemblyOptions()
        self.ctx = ctx or api.default_context()
        self.precision = self.assembly.precision
        self.els = api.build_elements(g)
        self.sigma = api.source_strengths(self.els, self.V)
        te_len = opts.te_len if opts.te_len is not None else 0.3 * np.linalg.norm(self.V) * opts.dt
        self.te = meshes.te_panel(g, dm, self.V, length=te_len)
        A, self.b0, _ = api.assemble(g, dm, self.els, self.sigma, self.V, opts=self.assembly, wake=self.te, ctx=self.ctx)
        self.F = api.factorize_galerkin(dm, A, W=meshes.wake_rows(dm, self.te.te), precision=self.precision,
                                        ctx=self.ctx)
        del A
        self.topo = Topology.of(dm)
        nte = self.topo.nte
        self.edge = np.ascontiguousarray(self.te.x[nte:2 * nte])  # the panel's downstream edge (its row 1)
        self.core = core_params(opts, self.V)
        row = np.linalg.norm(self.V) * opts.dt
        widths = [float(np.linalg.norm(self.edge[B] - self.edge[A])) for A, B in self.topo.strips]
        if opts.max_rows == "auto":  # rows_for_distance(3, ...) (step.jl:80-82)
            first = core_of_quad(self.core, max(widths), row)
            self.keep_rows = max(0, math.ceil((3 * first - self.te.rows[1]) / row - 0.5))
        else:
            self.keep_rows = int(opts.max_rows)
        if opts.merge_rows == "auto":
            self.merge = [max(1, int(round(w / row))) for w in widths]
        elif opts.merge_rows == 1:
            self.merge = None
        else:
            self.merge = [int(opts.merge_rows)] * len(widths)
        d = self.V / np.linalg.norm(self.V)
        delete = float((self.edge @ d).max() + opts.delete_beyond * self.te.span) if math.isfinite(
            opts.delete_beyond) else math.inf
        self.history = []
        self._create(delete, capacity)

    def _create(self, delete_limit, capacity):
        g, dm, o = self.g, self.dm, self.opts
        keep = []  # arrays the set-up points into, alive for the call

        def dp(a):
            a = np.ascontiguousarray(np.asarray(a, float))
            keep.append(a)
            return a.ctypes.data_as(D)

        def ip(a):
            a = np.ascontiguousarray(np.asarray(a, np.int32))
            if a.size == 0:
                a = np.zeros(1, np.int32)
            keep.append(a)
            return a.ctypes.data_as(I)

        s = vp_freewake_setup()
        s.dt, s.keep_rows = float(o.dt), int(self.keep_rows)
        s.core_mode, s.overlap, s.core_factor, s.core_floor, s.core_value = self.core
        s.advection = 0 if o.advection == "free" else 1
        s.delete_limit = delete_limit
        s.assembly = self.assembly.c_struct()
        s.nnode, s.x, s.ntri, s.tris, s.corner_slot = g.nnode, dp(g.x), g.ntri, ip(g.tris), ip(dm.corner_slot)
        s.nslot, s.sigma, s.vinf, s.factor, s.b0 = dm.nslot, dp(self.sigma), dp(self.V), self.F.h, dp(self.b0)
        C, K = dm.C.tocsr(), dm.K.tocsr()
        s.nq, s.C_rowptr, s.C_col, s.C_val = dm.nq, ip(C.indptr), ip(C.indices), dp(C.data if C.nnz else [0.0])
        s.nte, s.K_rowptr, s.K_col, s.K_val = self.topo.nte, ip(K.indptr), ip(K.indices), dp(K.data if K.nnz else [0.0])
        wte = dm.wake_te
        lines = [np.asarray(L, np.int32) for L in wte.lines]
        s.te_x = dp(wte.x)
        s.nline = len(lines)
        s.line_ptr = ip(np.concatenate([[0], np.cumsum([len(L) for L in lines])]))
        s.line_nodes = ip(np.concatenate(lines) if lines else [])
        s.line_closed = ip([int(bool(c)) for c in wte.closed])
        s.nstrip, s.strips = len(self.topo.strips), ip(np.asarray(self.topo.strips).reshape(-1))
        s.nfirst, s.first_nodes = len(self.topo.first_nodes), ip(self.topo.first_nodes)
        s.nlast, s.last_nodes = len(self.topo.last_nodes), ip(self.topo.last_nodes)
        s.edge = dp(self.edge)
        te = self.te
        s.npw, s.pw_x, s.pw_te = len(te.x), dp(te.x), ip(te.te)
        s.npt, s.pt_tris = len(te.tris), ip(np.asarray(te.tris).reshape(-1))
        s.npf, s.pf = len(te.filaments), ip(np.asarray(te.filaments).reshape(-1))
        s.merge = ip(self.merge) if self.merge is not None else None
        s.particle_capacity = int(capacity)
        h = ctypes.c_void_p()
        check(self.ctx.h, load().vp_freewake_create(self.ctx.h, ctypes.byref(s), ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            try:
                load().vp_freewake_free(self.h)
            except Exception:
                pass
            self.h = None

    # -- the steps --
    def counts(self):
        c = vp_freewake_counts()
        check(self.ctx.h, load().vp_freewake_info(self.h, ctypes.byref(c)))
        return c

    @property
    def n(self):
        return self.counts().n

    @property
    def t(self):
        return self.counts().t

    def step(self):
        """step!(sim) (step.jl:113-146): one time step on the GPU; returns its record"""
        r = vp_freewake_record()
        check(self.ctx.h, load().vp_freewake_step(self.h, ctypes.byref(r)))
        mu_w = np.zeros(self.topo.nte)
        check(self.ctx.h, load().vp_freewake_get_state(self.h, None, None, None, None, None, None, None, None, None,
                                                       None, mu_w.ctypes.data_as(D), None))
        rec = dict(n=r.n, t=r.t, mu_w=mu_w, F_pressure=np.array(r.F_pressure), M_pressure=np.array(r.M_pressure),
                   F_kj=np.array(r.F_kj), F_impulse=np.array(r.F_impulse), Omega=np.array(r.Omega), I=np.array(r.I),
                   rows=r.rows, particles=r.particles, lam=r.lam, umax=r.umax)
        self.history.append(rec)
        return rec

    def run(self, nsteps, progress=None):
        """run!(sim, n) (step.jl:205-216): take nsteps steps; returns the history"""
        for _ in range(nsteps):
            rec = self.step()
            if progress is not None:
                progress(self, rec)
        return self.history

    # -- the state on the host --
    def _get(self):
        c = self.counts()
        nte, ns = self.topo.nte, len(self.topo.strips)
        a = dict(rows_x=np.zeros((c.nrows, nte, 3)), rows_mu=np.zeros((c.nrows, nte)), mu_line=np.zeros(nte),
                 particles=np.zeros((c.nparticles, 7)), tag=np.zeros(c.nparticles, np.int32),
                 group=np.zeros(c.nparticles, np.int8), batch_rows=np.zeros(ns, np.int32), batch_length=np.zeros(ns),
                 batch_width=np.zeros(ns), mu=np.zeros(self.dm.nslot), mu_w=np.zeros(nte), cp=np.zeros(self.g.ntri))
        ptr = {k: (v.ctypes.data_as(I) if v.dtype == np.int32 else
                   v.ctypes.data_as(ctypes.POINTER(ctypes.c_byte)) if v.dtype == np.int8 else v.ctypes.data_as(D))
               for k, v in a.items()}
        check(self.ctx.h, load().vp_freewake_get_state(
            self.h, ptr["rows_x"], ptr["rows_mu"], ptr["mu_line"], ptr["particles"], ptr["tag"], ptr["group"],
            ptr["batch_rows"], ptr["batch_length"], ptr["batch_width"], ptr["mu"], ptr["mu_w"], ptr["cp"]))
        return c, a

    @property
    def state(self) -> WakeState:
        c, a = self._get()
        return WakeState(x=list(a["rows_x"]), mu=list(a["rows_mu"]), mu_line=a["mu_line"], particles=a["particles"],
                         conversions=c.conversions, tag=a["tag"], group=a["group"], batch_rows=a["batch_rows"],
                         batch_length=a["batch_length"], batch_width=a["batch_width"])

    @property
    def mu(self):
        return self._get()[1]["mu"]

    @property
    def cp(self):
        """the pressure coefficient of the last step"""
        return self._get()[1]["cp"]

    def checkpoint(self) -> dict:
        """the simulation's evolving state as named arrays, and its history: restore() on a FreeWakeSim of the same
        body, options and assembly continues from it"""
        c, a = self._get()
        a.update(n=np.array(c.n), t=np.array(c.t), nrows=np.array(c.nrows), conversions=np.array(c.conversions),
                 I_prev=np.array(c.I_prev))
        return {"state": a, "history": list(self.history)}

    def restore(self, ckpt: dict):
        a = ckpt["state"]
        nte = self.topo.nte
        if a["rows_x"].shape[1:] != (nte, 3) or a["mu"].shape != (self.dm.nslot,):
            raise ValueError("the checkpoint is of another wing or DOF map")
        c = vp_freewake_counts()
        c.n, c.t, c.nrows = int(a["n"]), float(a["t"]), int(a["nrows"])
        c.nparticles, c.conversions = len(a["particles"]), int(a["conversions"])
        for z in range(3):
            c.I_prev[z] = float(a["I_prev"][z])
        arr = {k: np.ascontiguousarray(v) for k, v in a.items()}
        tag = np.ascontiguousarray(arr["tag"], np.int32)
        group = np.ascontiguousarray(arr["group"], np.int8)
        brows = np.ascontiguousarray(arr["batch_rows"], np.int32)
        part = np.ascontiguousarray(arr["particles"], float).reshape(-1, 7)
        check(self.ctx.h, load().vp_freewake_set_state(
            self.h, ctypes.byref(c), arr["rows_x"].ctypes.data_as(D), arr["rows_mu"].ctypes.data_as(D),
            arr["mu_line"].ctypes.data_as(D), part.ctypes.data_as(D), tag.ctypes.data_as(I),
            group.ctypes.data_as(ctypes.POINTER(ctypes.c_byte)), brows.ctypes.data_as(I),
            arr["batch_length"].ctypes.data_as(D), arr["batch_width"].ctypes.data_as(D), arr["mu"].ctypes.data_as(D),
            arr["mu_w"].ctypes.data_as(D), arr["cp"].ctypes.data_as(D)))
        self.history = list(ckpt["history"])
