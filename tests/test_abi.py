"""The C ABI (no GPU): every function include/vortexpanel_gpu.h declares is exported by the built library, and the
Python binding declares a signature for each."""
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
