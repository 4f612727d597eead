"""Host check of the translation-deflated element projection
(include/tad/Projection.cuh) against the general k x k projection rule of
TinyAD (include/TinyAD/Utils/HessianProjection.hh:16-101), compiled with g++
from the header the device kernels use: invariant matrices take the deflated
form and agree with the general projection (FP64 to rounding, FP32 at FP32
accuracy, eps > 0 and eps < 0, an unused vertex), general matrices are
declined untouched.  d = 1..3, N = 2..5."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "projection_test.cpp")


def test_translation_deflated_projection(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "projection_test"
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
