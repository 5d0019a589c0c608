"""The FP32-pair arithmetic (csrc/df64.cuh) and the FP32-pair WENO5 reverse core
(csrc/weno5_df.cuh), compiled for the host by g++ without multiply-add contraction
and checked against long double.  No GPU.

The pair operations on seeded inputs over 2^+-30 (tests/df64_check.cpp): the
bit-level split of a double into a pair (h + l = q to 2^-48 of q; below float's
normal range for l, 2^-48 of q plus 2^-149; below 2^-126 zero; beyond float's range
an infinity; NaN stays NaN), the sloppy addition, the products, the quotient and the
reciprocal square root, each bound in units of 2^-48 of the operation's scale.

The reverse core (tests/weno_rev_check.cpp) against the adjoint's FP64 walk
(cal_advu_weno5.f:44-255, weno5.h:2-70: R = num/den of the stencil's five
differences and dR/de) evaluated in long double, on stencils of six doubles in six
regimes (smooth waves over 1e-12 .. 1e10, small variations on a large mean,
constant and linear runs, jumps, noise, near-flat values): R within 1e-12 of the
largest difference and the gradient within 1e-10 of its largest entry (measured
1.3e-13 and 2.2e-11; the FP64 walk itself 3.6e-15 and 7.8e-13).  On the same
stencils the forward pair core of the FP64-accurate step (wdir_core, which takes
its differences between split values) within 1e-12 of the largest difference +
4e-13 of the largest value + 2^-94 (measured at most 0.2 of that)."""
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


def test_weno_reverse_core_against_long_double(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "weno_rev_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "weno_rev_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    rows = [line.split() for line in out.split("\n") if line.strip()]
    assert len(rows) == 6, out
    for name, r, g, r64, g64, fwd in rows:
        assert float(r) <= 1e-12, (name, out)
        assert float(g) <= 1e-10, (name, out)
        assert float(fwd) <= 1.0, (name, out)
