"""Host check of the lane-split evaluation of the tetrahedron (9 reduced
derivatives; include/tad/Element.cuh SubsetElement and plane_line, the
symmetric Dirichlet functor of include/tad/Energies.cuh), compiled with g++
from the headers the device kernels use: the 12 index triples cover every
pair once, and their 3-derivative evaluations reproduce one dense
9-derivative evaluation (FP64 exactly; the FP32 lanes on staged positions at
FP32 accuracy)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "lane_split_test.cpp")


def test_lane_split_decomposition(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "lane_split_test"
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
