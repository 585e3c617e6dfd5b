"""Generates the free-wake fixture of tests/golden/ with the oracle's FreeWakeSim (oracle/freewake_oracle.py: the
reference's bookkeeping with the oracle's kernels and LAPACK): the wing of the free-wake workload, AR 8 NACA 0012 with
40 x 40 full-cosine panels per side (6,556 triangles), alpha = 8 deg, |V∞| = 1, dt = 0.02 chord, particle core 0.05
chord (a fixed radius), the other FreeWakeOptions at their defaults (max_rows :auto, no merging, te_len 0.3 |V∞| dt),
the reference's default AssemblyOptions; 50 steps. Stored: per step CL by the pressure route and by Kutta-Joukowski
(reference area span x chord, lift along (-sin a, 0, cos a)), the free rows and the particles; after the last step
the node rows and the particles (x, alpha, delta). About five minutes on 8 cores.

    python tests/golden/make_freewake_golden.py
"""
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "vortexpanel.jl_gb300"), os.path.join(ROOT, "oracle")]

import freewake_oracle as OF  # noqa: E402
from vortexpanel_gpu import meshes  # noqa: E402

NAME = "freewake_wing40_alpha8"
STEPS = 50
ALPHA = math.radians(8.0)


def case():
    """the wing, freestream, options and lift direction of the fixture"""
    w = meshes.wing(40, 40, aspect=8.0)
    V = np.array([math.cos(ALPHA), 0.0, math.sin(ALPHA)])
    eL = np.array([-math.sin(ALPHA), 0.0, math.cos(ALPHA)])
    return w, V, eL, dict(dt=0.02, core=0.05)


def main():
    w, V, eL, kw = case()
    S = w.span * w.chord
    t0 = time.time()
    sim = OF.FreeWakeSim(w.g, w.dm, V, OF.FreeWakeOptions(**kw))
    cl_p, cl_kj, rows, npart = [], [], [], []
    for k in range(STEPS):
        r = sim.step()
        cl_p.append(r["F_pressure"] @ eL / S)
        cl_kj.append(r["F_kj"] @ eL / S)
        rows.append(r["rows"])
        npart.append(r["particles"])
        print(f"step {k}: CL {cl_p[-1]:.6f} (KJ {cl_kj[-1]:.6f}), {r['rows']} rows, {r['particles']} particles, "
              f"{time.time() - t0:.0f} s", flush=True)
    st = sim.state
    np.savez_compressed(os.path.join(HERE, NAME + ".npz"), cl_pressure=np.array(cl_p), cl_kj=np.array(cl_kj),
                        rows=np.array(rows), particles_count=np.array(npart), node_rows=np.array(st.x),
                        particles=st.particles, keep_rows=np.array(sim.keep_rows))


if __name__ == "__main__":
    main()
