"""The tensor-core GEMM of the mixed-precision LU's trailing updates (vp_gemm_sub_f32 through the C ABI: C -= A B,
FP32 column-major, each operand split into three bf16 pieces, six tcgen05 products accumulated in FP32 in TMEM)
against the FP64 product of the same FP32 inputs. FP32-class accuracy: its error is within 3x that of an FP32 GEMM
of the same inputs (numpy's, FP32 accumulation) and within 1e-5 of max |A||B|; a plain bf16 product (2^-8 per term)
or a two-piece split (2^-16) would be hundreds of times worse per term. Ragged sizes, leading dimensions larger than
the rows, and k below, at and above one 64-wide slice. And the bordered LU with the tensor cores against the same LU
on cuBLAS SGEMM: the refined solutions agree to FP64 rounding."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _gemm(vp, A, B, C, lda=None, ldb=None, ldc=None):
    m, k = A.shape
    n = B.shape[1]
    lda, ldb, ldc = lda or m, ldb or k, ldc or m
    a = np.zeros((k, lda), np.float32)
    a[:, :m] = A.T
    b = np.zeros((n, ldb), np.float32)
    b[:, :k] = B.T
    c = np.zeros((n, ldc), np.float32)
    c[:, :m] = C.T
    F = ctypes.POINTER(ctypes.c_float)
    ctx = vp.default_context()
    vp._lib.check(ctx.h, vp._lib.load().vp_gemm_sub_f32(ctx.h, m, n, k, a.ctypes.data_as(F), lda, b.ctypes.data_as(F),
                                                         ldb, c.ctypes.data_as(F), ldc))
    return c[:, :m].T


@pytest.mark.parametrize("m,n,k,pad", [(128, 128, 64, 0), (300, 260, 200, 7), (1000, 520, 700, 0), (256, 384, 40, 3),
                                       (129, 1000, 1300, 1)])
def test_tensor_core_gemm_is_fp32_class(vp, m, n, k, pad):
    rng = np.random.default_rng(m + 7 * n + 13 * k)
    A = rng.standard_normal((m, k)).astype(np.float32)
    B = (rng.standard_normal((k, n)) * np.exp(rng.uniform(-3, 3, (k, 1)))).astype(np.float32)
    C = rng.standard_normal((m, n)).astype(np.float32)
    got = _gemm(vp, A, B, C, lda=m + pad, ldb=k + pad, ldc=m + pad).astype(np.float64)
    ref = C.astype(np.float64) - A.astype(np.float64) @ B.astype(np.float64)
    scale = (np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)).max()
    err = np.abs(got - ref).max() / scale
    err32 = np.abs((C - A @ B).astype(np.float64) - ref).max() / scale  # an FP32 GEMM's error on the same inputs
    assert err < 3 * err32 + 1e-9 and err < 1e-5, (err, err32)
    # the padded leading dimensions' extra rows of C are untouched: only the m x n block changes
    assert np.isfinite(got).all()


def test_lu_with_tensor_cores_matches_cublas(vp, tmp_path):
    """the icosphere(3) system (order 643: its top-level updates run on the tensor cores) factored in mixed precision
    with and without the tensor-core GEMM, in a child process for the second (the switch is read per call)"""
    code = ("import sys, numpy as np; sys.path[:0] = [%r, %r]; import vortexpanel_gpu as vp\n"
            "g, dm = vp.meshes.sphere_case(3); V = np.array([1.0, 0.3, -0.2]); V /= np.linalg.norm(V)\n"
            "els = vp.build_elements(g); A, b, _ = vp.assemble(g, dm, els, vp.source_strengths(els, V), V)\n"
            "s = vp.solve_galerkin(dm, A, b, precision='mixed'); np.save(sys.argv[1], s['q'])\n") % (
        os.path.join(ROOT, "vortexpanel.jl_gb300"), ROOT)
    out = {}
    for flag in ("1", "0"):
        path = str(tmp_path / f"q{flag}.npy")
        env = dict(os.environ, VP_LU_TENSOR_CORES=flag)
        subprocess.run([sys.executable, "-c", code, path], check=True, env=env, timeout=600)
        out[flag] = np.load(path)
    q1, q0 = out["1"], out["0"]
    assert np.abs(q1 - q0).max() < 1e-12 * np.abs(q0).max()
