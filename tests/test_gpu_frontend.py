"""The C++ front end (include/tad/ScalarFunction.cuh): the reference's
NewtonTest / ScalarFunctionTest programs written with generic __device__
lambdas (tests/cpp/frontend_test.cu), built by build() and run on the GPU."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_cpp_frontend(tad):
    from tinyad_gb300 import build
    exe = build.FRONTEND_BIN
    if not os.path.exists(exe):
        build.build_frontend_test()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "frontend ok" in r.stdout
