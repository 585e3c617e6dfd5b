"""The adjoint's order-independent sums (csrc/vp_fixed.cuh) on the host: a carry-save fixed-point accumulator (six
32-bit digits in 64-bit words) whose words are the same bit for bit whatever the order of the additions, sequential or
from concurrent threads with atomic adds on its words, and whose value is the exact sum of the addends rounded to
2^-130 each (compared with exact rationals and math.fsum). Compiled with g++ from tests/fixed_point_check.cpp."""
import math
import os
import struct
import subprocess
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "vortexpanel.jl_gb300", "csrc")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("fx") / "fixed_point_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", CSRC, os.path.join(HERE, "fixed_point_check.cpp"),
                    "-o", exe], check=True)
    return exe


def _run(exe, values):
    inp = f"{len(values)}\n" + "\n".join(repr(float(v)) for v in values) + "\n"
    out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    return [line.split() for line in out if line.strip()]


def _grid(v):
    """v on the accumulator's grid, in units of 2^-130, rounded half up in magnitude (exact integers)"""
    x = abs(Fraction(v)) * 2**130
    q = math.floor(x + Fraction(1, 2))
    return -q if v < 0 else q


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_order_independent_and_exact(harness, seed):
    rng = np.random.default_rng(seed)
    n = 4000
    mag = 10.0 ** rng.uniform(-30, 12, n)
    v = rng.choice([-1.0, 1.0], n) * rng.uniform(0.5, 1.0, n) * mag
    v[:50] = -v[50:100]  # exact cancellations
    runs = _run(harness, v)
    assert len(runs) == 7
    assert all(r[:7] == runs[0][:7] for r in runs), runs
    assert runs[0][6] == "0"
    got = float(runs[0][7])
    exact = sum(_grid(x) for x in v)
    ref = exact / 2**130
    assert abs(got - ref) <= 2 * abs(ref) * 2**-53 + 1e-300
    assert abs(got - math.fsum(v)) <= 1e-15 * abs(math.fsum(v)) + n * 2**-130


def test_words_and_flags(harness):
    # 1 + 2^-80 - 1: carries across words, then back to a value below one unit of the top word
    r = _run(harness, [1.0, 2.0**-80, -1.0])
    assert float(r[0][7]) == 2.0**-80 and all(x[:7] == r[0][:7] for x in r)
    # a negative total reads back negative; subnormals and values under half a unit vanish
    r = _run(harness, [-3.5, 1.25, 5e-324, 1e-45])
    assert float(r[0][7]) == -2.25
    # a non-finite addend or one beyond the range (|v| >= 2^61) sets the flag and reads back NaN
    for bad in (float("inf"), float("nan"), 2.0**61):
        r = _run(harness, [1.0, bad, 2.0])
        assert r[0][6] == "1" and math.isnan(float(r[0][7]))
    r = _run(harness, [2.0**61 * (1 - 2**-53), -1.0])
    assert float(r[0][7]) == 2.0**61 * (1 - 2**-53) - 1.0 and r[0][6] == "0"
    r = _run(harness, [-(2.0**61) * (1 - 2**-53), 1.0])
    assert float(r[0][7]) == -(2.0**61) * (1 - 2**-53) + 1.0 and r[0][6] == "0"
    # the digits: 0.5 is bit 129 of the 192-bit integer, digit 4 (bits 128-159) = 2; -0.5 negates the digit
    r = _run(harness, [0.5])
    assert r[0][:6] == ["0", "0", "0", "0", "2", "0"]
    assert struct.pack("<d", float(r[0][7])) == struct.pack("<d", 0.5)
    r = _run(harness, [-0.5, 0.25])
    assert r[0][:6] == ["0", "0", "0", "0", "-1", "0"] and float(r[0][7]) == -0.25
    # carries between digits resolve on reading: three addends of 2^32 - 1 units each take digit 0 past 32 bits
    r = _run(harness, [2.0**-98 - 2.0**-130] * 3)
    assert float(r[0][7]) == 3 * (2.0**-98 - 2.0**-130)
