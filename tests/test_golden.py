"""The committed golden fixtures (tests/golden/, made by tests/golden/make_golden.py from the oracle): the oracle
reproduces them (CPU), and the GPU assembly matches them (row-relative 1e-10, FP64)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import make_golden  # noqa: E402


def _fixtures():
    for name, g, dm, V, wake in make_golden.cases():
        d = np.load(os.path.join(HERE, name + ".npz"))
        yield name, g, dm, V, wake, d["A"], d["b"]


def test_oracle_reproduces_fixtures(oracle):
    for name, g, dm, V, wake, A0, b0 in _fixtures():
        A, b, _ = oracle.assemble(g, dm, oracle.source_strengths(g, V), V, wake=wake)
        assert np.abs(A - A0).max() <= 1e-13 * np.abs(A0).max(), name
        assert np.abs(b - b0).max() <= 1e-13 * np.abs(b0).max(), name


@pytest.mark.gpu
def test_gpu_matches_fixtures(vp):
    for name, g, dm, V, wake, A0, b0 in _fixtures():
        els = vp.build_elements(g)
        A, b, _ = vp.assemble(g, dm, els, vp.source_strengths(els, V), V, wake=wake)
        Ad = A.download()
        row = np.abs(A0).max(axis=1, keepdims=True)
        assert (np.abs(Ad - A0) / row).max() <= 1e-10, name
        assert np.abs(b - b0).max() <= 1e-10 * np.abs(b0).max(), name
