"""Generates the golden fixtures of tests/golden/ with the CPU oracle (oracle/): assembled A and b of the unit
icosphere at subdivision 1 (non-lifting, V∞ = (1, 0.3, -0.2)/|.|) and of a small lifting wing (6 x 3 panels per side,
AR 4) with its rigid wake, both with the reference's default AssemblyOptions. The reference itself (Julia) cannot run
here; the fixtures pin the GPU path and later oracle builds to these values.

    python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "vortexpanel.jl_gb300"), os.path.join(ROOT, "oracle")]

import oracle  # noqa: E402
from vortexpanel_gpu import meshes  # noqa: E402


def cases():
    V = np.array([1.0, 0.3, -0.2])
    V /= np.linalg.norm(V)
    g, dm = meshes.sphere_case(1)
    yield "icosphere1", g, dm, V, None
    w = meshes.wing(6, 3, aspect=4.0)
    a = math.radians(5.0)
    Vw = np.array([math.cos(a), 0.0, math.sin(a)])
    yield "wing6x3", w.g, w.dm, Vw, meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=1.0)


def main():
    oracle.build()
    for name, g, dm, V, wake in cases():
        sig = oracle.source_strengths(g, V)
        A, b, _ = oracle.assemble(g, dm, sig, V, wake=wake)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), A=A, b=b, V=V)
        print(name, A.shape)


if __name__ == "__main__":
    main()
