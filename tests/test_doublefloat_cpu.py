"""Host checks of the double-float arithmetic behind the mixed-precision
element kernels (include/tad/Scalar.cuh: DoubleFloatValue for values,
DoubleFloat for gradients), compiled with g++ from the same header the device
kernels use.  Covers accuracy against long double, IEEE propagation of
infinities and NaNs, and the mixed scalar against Double<6> on the symmetric
Dirichlet triangle energy (tests/NewtonTest.cc:28-44)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "doublefloat_test.cpp")


def test_double_float_arithmetic(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "doublefloat_test"
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
