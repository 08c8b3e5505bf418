"""CPU: the correctly rounded division by the QR divisor (drot_math.cuh).

The kernels divide every prox value by the constant kappa with an
FMA-based residual correction instead of the IEEE division sequence.  This
test compiles the same header for the host and compares it with IEEE float
division on every significand of the binade [1, 2) plus 4M random dividends
over [2^-90, 2^30], for divisors that cover the QR range (kappa = 1 + rho *
r_weight, with rho = 2 and r_weight from 0 to 10, and awkward significands).
Scaling a by a power of two scales every step exactly, so one full binade
covers all normal dividends that keep the residuals normal.
"""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "native", "div_check.cpp")
INC = os.path.join(REPO, "regularized-drot_gb300", "csrc")

DIVISORS = ["1.002", "1.0000001", "1.9999999", "1.5", "3", "21", "7.77", "1.0199999",
            "1000.3", "1.3333334", "1.00002", "1.2", "11.000001"]


def test_division_matches_ieee(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "div_check")
    subprocess.check_call([cxx, "-O2", "-ffp-contract=off", "-I", INC, "-o", exe, SRC])
    out = subprocess.run([exe, *DIVISORS], capture_output=True, text=True)
    lines = out.stdout.strip().splitlines()
    assert len(lines) == len(DIVISORS)
    bad = {ln.split()[0]: int(ln.split()[1]) for ln in lines}
    assert out.returncode == 0 and all(v == 0 for v in bad.values()), bad


def test_gl_shrink_matches_double_formula(tmp_path):
    """The float-pair GL shrink factor against the reference's double formula
    (core/kernel_glr.hpp:125, 320) on 8M random (norm, lambda) pairs, half of
    them with lambda within 10% of the norm, where the factor nearly vanishes:
    at most a few 1-ulp differences (ties within 2^-44), none larger."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "shrink_check")
    subprocess.check_call([cxx, "-O2", "-ffp-contract=off", "-I", INC, "-o", exe,
                           os.path.join(REPO, "tests", "native", "shrink_check.cpp")])
    out = subprocess.run([exe], capture_output=True, text=True)
    n, exact, one, more = (int(v) for v in out.stdout.split())
    assert out.returncode == 0 and more == 0
    assert one <= n * 1e-5 and exact + one == n


def test_pair_sums_and_stop_threshold(tmp_path):
    """The float-pair reductions (mass, objective, squared residual) carry at
    least 2^-40 relative accuracy in the kernels' summation orders, and the
    squared-residual threshold reproduces sqrt(r2) < eps / <= eps exactly
    (drot_math.cuh: fp_add, fp_sqr, res2_threshold)."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "sum_check")
    subprocess.check_call([cxx, "-O2", "-ffp-contract=off", "-I", INC, "-o", exe,
                           os.path.join(REPO, "tests", "native", "sum_check.cpp")])
    out = subprocess.run([exe], capture_output=True, text=True)
    bad, worst = out.stdout.split()
    assert out.returncode == 0 and int(bad) == 0
    assert float(worst) < 2.0 ** -40
