"""The C ABI (no GPU): every function include/vortexpanel_gpu.h declares is exported by the built library, and the
Python binding declares a signature for each, with the prototype's number of arguments."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "vortexpanel_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vp_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    from vortexpanel_gpu import _build, _lib
    path = _build.build(verbose=False)
    lib = ctypes.CDLL(path)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(names) <= bound | {"vp_default_options", "vp_ctx_create", "vp_ctx_destroy", "vp_last_error"}, \
        sorted(set(names) - bound)


def _prototypes():
    """name -> number of parameters of every function prototype in the header"""
    src = open(os.path.join(ROOT, "include", "vortexpanel_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    out = {}
    for name, params in re.findall(r"\b(vp_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        p = params.strip()
        out[name] = 0 if p in ("", "void") else p.count(",") + 1
    return out


def test_bindings_match_the_header_arity():
    # every ctypes signature takes as many arguments as the header's prototype
    from vortexpanel_gpu import _lib
    protos = _prototypes()
    assert len(protos) >= 20
    bad = [(n, len(args), protos[n]) for n, _, args in _lib.SIGNATURES if n in protos and len(args) != protos[n]]
    assert not bad, bad


def test_static_points_limit_matches_the_header():
    # the Python layer's limit is the header's VP_STATIC_POINTS_MAX
    from vortexpanel_gpu import api
    src = open(os.path.join(ROOT, "include", "vortexpanel_gpu.h")).read()
    m = re.search(r"#define\s+VP_STATIC_POINTS_MAX\s+(\d+)", src)
    assert m and int(m.group(1)) == api.STATIC_POINTS_MAX
