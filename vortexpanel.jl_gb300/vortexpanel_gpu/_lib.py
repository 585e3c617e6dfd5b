"""ctypes binding of libvortexpanel_gpu.so (include/vortexpanel_gpu.h). There is no CPU fallback: if the library
cannot be loaded or no CUDA device is present, every call raises."""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)
F32 = ctypes.POINTER(ctypes.c_float)

VP_OK, VP_ERR_ARG, VP_ERR_DEGENERATE, VP_ERR_SINGULAR, VP_ERR_NOCONV, VP_ERR_TIMEOUT, VP_ERR_CUDA, VP_ERR_NOMEM = range(8)
VP_FP64, VP_MIXED = 0, 1


class vp_assembly_options(ctypes.Structure):
    _fields_ = [("test", ctypes.c_int), ("far_ratio", ctypes.c_double), ("far_points", ctypes.c_int),
                ("near_points", ctypes.c_int), ("near_ratio", ctypes.c_double), ("near_depth", ctypes.c_int),
                ("touch_levels", ctypes.c_int), ("touch_ratio", ctypes.c_double), ("touch_order", ctypes.c_int),
                ("corner_angle", ctypes.c_double), ("contact_rel", ctypes.c_double), ("kernel_far", ctypes.c_double),
                ("precision", ctypes.c_int)]


class vp_assembly_stats(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_longlong * 6), ("points", ctypes.c_longlong * 6), ("time_ms", ctypes.c_double),
                ("points_fp64", ctypes.c_longlong)]


class vp_freewake_setup(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("keep_rows", ctypes.c_int), ("core_mode", ctypes.c_int),
                ("overlap", ctypes.c_double), ("core_factor", ctypes.c_double), ("core_floor", ctypes.c_double),
                ("core_value", ctypes.c_double), ("advection", ctypes.c_int), ("delete_limit", ctypes.c_double),
                ("assembly", vp_assembly_options), ("nnode", ctypes.c_int), ("x", D), ("ntri", ctypes.c_int),
                ("tris", I), ("corner_slot", I), ("nslot", ctypes.c_int), ("sigma", D), ("vinf", D),
                ("factor", ctypes.c_void_p), ("b0", D), ("nq", ctypes.c_int), ("C_rowptr", I), ("C_col", I),
                ("C_val", D), ("nte", ctypes.c_int), ("K_rowptr", I), ("K_col", I), ("K_val", D), ("te_x", D),
                ("nline", ctypes.c_int), ("line_ptr", I), ("line_nodes", I), ("line_closed", I),
                ("nstrip", ctypes.c_int), ("strips", I), ("nfirst", ctypes.c_int), ("first_nodes", I),
                ("nlast", ctypes.c_int), ("last_nodes", I), ("edge", D), ("npw", ctypes.c_int), ("pw_x", D),
                ("pw_te", I), ("npt", ctypes.c_int), ("pt_tris", I), ("npf", ctypes.c_int), ("pf", I), ("merge", I),
                ("particle_capacity", ctypes.c_int)]


class vp_freewake_record(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("t", ctypes.c_double), ("F_pressure", ctypes.c_double * 3),
                ("M_pressure", ctypes.c_double * 3), ("F_kj", ctypes.c_double * 3), ("F_impulse", ctypes.c_double * 3),
                ("Omega", ctypes.c_double * 3), ("I", ctypes.c_double * 3), ("rows", ctypes.c_int),
                ("particles", ctypes.c_int), ("lam", ctypes.c_double), ("umax", ctypes.c_double)]


class vp_freewake_counts(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("t", ctypes.c_double), ("nrows", ctypes.c_int), ("nparticles", ctypes.c_int),
                ("conversions", ctypes.c_int), ("I_prev", ctypes.c_double * 3)]


class vp_assembly_input(ctypes.Structure):
    _fields_ = [("nnode", ctypes.c_int), ("x", D), ("ntri", ctypes.c_int), ("tris", I), ("corner_slot", I),
                ("nslot", ctypes.c_int), ("ntouch", ctypes.c_int), ("touch_pairs", I), ("sigma", D), ("vinf", D),
                ("nwnode", ctypes.c_int), ("wx", D), ("nwtri", ctypes.c_int), ("wtris", I), ("nfil", ctypes.c_int),
                ("fil", I)]


B8 = ctypes.POINTER(ctypes.c_byte)

# (name, restype, argtypes) of every entry point declared in include/vortexpanel_gpu.h
SIGNATURES = [
    ("vp_default_options", None, [ctypes.POINTER(vp_assembly_options)]),
    ("vp_ctx_create", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    ("vp_ctx_destroy", None, [ctypes.c_void_p]),
    ("vp_last_error", ctypes.c_char_p, [ctypes.c_void_p]),
    ("vp_assemble", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(vp_assembly_options), ctypes.c_int, D, ctypes.c_int, I, I, ctypes.c_int,
      ctypes.c_int, I, D, D, ctypes.c_int, D, ctypes.c_int, I, ctypes.c_int, I, ctypes.POINTER(ctypes.c_void_p),
      ctypes.POINTER(vp_assembly_stats)]),
    ("vp_set_far_tile", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    ("vp_get_far_tile", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("vp_assemble_batch", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(vp_assembly_options), ctypes.c_int, ctypes.POINTER(vp_assembly_input),
      ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(vp_assembly_stats)]),
    ("vp_system_shape", ctypes.c_int, [ctypes.c_void_p, I, I]),
    ("vp_system_download", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, D, D]),
    ("vp_system_download_rows", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, D, D]),
    ("vp_system_free", None, [ctypes.c_void_p]),
    ("vp_factorize", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, I, I, D, ctypes.c_int, I, I, D, ctypes.c_int, I, D,
      I, ctypes.POINTER(ctypes.c_void_p), D]),
    ("vp_solve", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, D, D, D]),
    ("vp_solve_system", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, D, D, D]),
    ("vp_phase_times", ctypes.c_int, [ctypes.c_void_p, D, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    ("vp_transfer_bytes", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                         ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    ("vp_eval_points", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, D, D, D, ctypes.c_int,
                                      ctypes.c_double, D]),
    ("vp_eval_points_static", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, D, D, D,
                                             ctypes.c_int, ctypes.c_double, D]),
    ("vp_solve_transposed", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, D, D]),
    ("vp_adjoint", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(vp_assembly_options), ctypes.c_int, D, ctypes.c_int, I, I, ctypes.c_int,
      ctypes.c_int, I, D, D, ctypes.c_int, D, ctypes.c_int, I, ctypes.c_int, I, ctypes.c_int, D, D, D, D, D, D,
      ctypes.POINTER(vp_assembly_stats)]),
    ("vp_blob_velocities", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, D, ctypes.c_int, D, D]),
    ("vp_body_velocity", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, D, D, D, ctypes.c_double,
                                        ctypes.c_int, D, D]),
    ("vp_explicit_rhs", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(vp_assembly_options), ctypes.c_int, D,
                                       ctypes.c_int, I, I, ctypes.c_int, ctypes.c_int, D, D, ctypes.c_int, D, D,
                                       ctypes.c_int, D, D]),
    ("vp_consistency", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, I, I, D, ctypes.c_int, I, I, D,
                                      D]),
    ("vp_surface_loads", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, D, I, ctypes.c_int, D, D, D, D, D, D, D, D]),
    ("vp_pressure_force", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, D, D, D, D, D]),
    ("vp_wake_loads", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, D, ctypes.c_int, I, I, I, D, D, D, D]),
    ("vp_freewake_create", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(vp_freewake_setup),
                                          ctypes.POINTER(ctypes.c_void_p)]),
    ("vp_freewake_step", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(vp_freewake_record)]),
    ("vp_freewake_info", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(vp_freewake_counts)]),
    ("vp_freewake_get_state", ctypes.c_int, [ctypes.c_void_p, D, D, D, D, I, B8, I, D, D, D, D, D]),
    ("vp_freewake_set_state", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(vp_freewake_counts), D, D, D, D, I, B8,
                                             I, D, D, D, D, D]),
    ("vp_freewake_free", None, [ctypes.c_void_p]),
    ("vp_gemm_sub_f32", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, F32, ctypes.c_int,
                                       F32, ctypes.c_int, F32, ctypes.c_int]),
    ("vp_factor_info", ctypes.c_int, [ctypes.c_void_p, I, D]),
    ("vp_factor_free", None, [ctypes.c_void_p]),
]

_lock = threading.Lock()
_lib = None


class VPError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[vp status {code}] {msg}")
        self.code = code


class SingularError(VPError):
    """The reference's LinearAlgebra.SingularException"""


def load(build_if_missing: bool = True):
    """The loaded library; builds it first (nvcc, sm_103a) when it is missing or stale and nvcc is available"""
    global _lib
    with _lock:
        if _lib is None:
            if build_if_missing and not _build.up_to_date():
                _build.build()
            if not os.path.exists(_build.LIB):
                raise RuntimeError(f"libvortexpanel_gpu.so is not built ({_build.LIB}); run build() first")
            lib = ctypes.CDLL(_build.LIB)
            for name, res, args in SIGNATURES:
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            _lib = lib
        return _lib


def check(ctx, code):
    if code == VP_OK:
        return
    msg = load().vp_last_error(ctx).decode() if ctx else ""
    if code in (VP_ERR_ARG, VP_ERR_DEGENERATE):
        raise ValueError(f"[vp status {code}] {msg}")
    if code == VP_ERR_SINGULAR:
        raise SingularError(code, msg)
    raise VPError(code, msg)


class Context:
    """A device context (stream, cuBLAS handle) of the library"""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        code = self.lib.vp_ctx_create(device, ctypes.byref(h))
        if code != VP_OK:
            raise VPError(code, f"cannot create a context on CUDA device {device} (no GPU, or the driver failed)")
        self.h = h
        self.device = device

    PHASES = ("setup", "classify", "far", "near", "reduce", "lu", "cond", "solve", "adj_setup", "adj_far", "adj_near",
              "adj_solve", "wake", "near_pairs", "adj_pairs", "wake_rhs", "wake_vel")

    def phase_times(self, reset=False):
        """Device milliseconds per phase since the last reset, and the number of the library's kernel launches"""
        ms = (ctypes.c_double * len(self.PHASES))()
        n = ctypes.c_longlong()
        check(self.h, self.lib.vp_phase_times(self.h, ms, len(self.PHASES), ctypes.byref(n), int(reset)))
        return dict(zip(self.PHASES, list(ms))), n.value

    def transfer_bytes(self, reset=False):
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        check(self.h, self.lib.vp_transfer_bytes(self.h, ctypes.byref(a), ctypes.byref(b), int(reset)))
        return a.value, b.value

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            try:
                self.lib.vp_ctx_destroy(h)
            except Exception:
                pass
            self.h = None


_default = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default
