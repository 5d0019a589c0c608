"""The FP32-pair arithmetic of the FP64-accurate step (csrc/df64.cuh), compiled
for the host by g++ without multiply-add contraction and checked against long
double on seeded inputs over 2^+-30: the bit-level split of a double into a pair
(h + l = q to 2^-48 of q; below float's normal range for l, 2^-48 of q plus 2^-149;
below 2^-126 zero; beyond float's range an infinity; NaN stays NaN), the sloppy
addition, the products, the quotient and the reciprocal square root.  Each bound
is in units of 2^-48 of the operation's scale (tests/df64_check.cpp).  No GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "fel-multi-phase-flow_gb300", "csrc")

# worst error over the samples, in units of 2^-48 of the scale
BOUNDS = {"split": 1.0, "split_small": 1.0, "add": 4.0, "mulf": 4.0, "mul": 16.0, "sqr": 16.0,
          "div": 32.0, "rsqrt": 32.0}


def test_pair_arithmetic_against_long_double(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "df64_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "df64_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {k: float(v) for k, v in (line.split() for line in out.split("\n") if line.strip())}
    assert got.pop("special") == 1.0, out
    for k, b in BOUNDS.items():
        assert got[k] <= b, (k, got)
