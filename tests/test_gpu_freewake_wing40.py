"""The free-wake workload against the oracle's fixture: the AR 8 NACA 0012 wing with 40 x 40 panels per side (6,556
triangles), alpha = 8 deg, |V∞| = 1, dt = 0.02 chord, particle core 0.05 chord, the reference's defaults otherwise
(tests/golden/make_freewake_golden.py, the oracle's FreeWakeSim). After 50 steps on the GPU:
  - FP64: CL by the pressure route and by Kutta-Joukowski within 1e-9 at every step, the same rows and particle counts,
    and the node rows and particle positions (the trajectories) within 1e-9 chord, strengths within 1e-9 of their
    scale;
  - mixed (FP32 kernels, FP64 sums): CL within 1e-6 at every step, positions within 1e-5 chord."""
import os
import sys

import numpy as np
import pytest

from vortexpanel_gpu import api
from vortexpanel_gpu import freewake as fw

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import make_freewake_golden as G  # noqa: E402


@pytest.fixture(scope="module")
def golden():
    with np.load(os.path.join(HERE, G.NAME + ".npz")) as d:
        return {k: d[k] for k in d.files}


@pytest.mark.parametrize("precision,tol_cl,tol_x", [("fp64", 1e-9, 1e-9), ("mixed", 1e-6, 1e-5)])
def test_fifty_steps_match_oracle(golden, precision, tol_cl, tol_x):
    w, V, eL, kw = G.case()
    S = w.span * w.chord
    sim = fw.FreeWakeSim(w.g, w.dm, V, fw.FreeWakeOptions(**kw), assembly=api.AssemblyOptions(precision=precision),
                         capacity=8192)
    assert sim.keep_rows == int(golden["keep_rows"])
    hist = sim.run(G.STEPS)
    cl_p = np.array([r["F_pressure"] @ eL / S for r in hist])
    cl_kj = np.array([r["F_kj"] @ eL / S for r in hist])
    assert np.array_equal([r["rows"] for r in hist], golden["rows"])
    assert np.array_equal([r["particles"] for r in hist], golden["particles_count"])
    assert np.abs(cl_p - golden["cl_pressure"]).max() < tol_cl, np.abs(cl_p - golden["cl_pressure"]).max()
    assert np.abs(cl_kj - golden["cl_kj"]).max() < tol_cl, np.abs(cl_kj - golden["cl_kj"]).max()
    st = sim.state
    P, P0 = st.particles, golden["particles"]
    assert P.shape == P0.shape
    assert np.abs(np.array(st.x) - golden["node_rows"]).max() < tol_x
    assert np.abs(P[:, :3] - P0[:, :3]).max() < tol_x
    assert np.abs(P[:, 3:] - P0[:, 3:]).max() < tol_x * np.abs(P0[:, 3:]).max()
