"""CPU tests of the CUDA library's boundary: it builds for sm_103a, loads,
and exports every entry point include/tad.h declares (no compute calls)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "tad.h")).read()
    return sorted(set(re.findall(r"TAD_API\s+[\w\s\*]+?\b(tad_\w+)\s*\(", src)))


def test_header_symbols_listed():
    import tinyad_gb300
    syms = header_symbols()
    assert len(syms) >= 20
    assert sorted(tinyad_gb300.EXPORTS) == syms


def test_library_builds_and_exports():
    import ctypes
    from tinyad_gb300 import build
    lib = build.build()
    assert os.path.exists(lib)
    L = ctypes.CDLL(lib)
    for s in header_symbols():
        assert hasattr(L, s), s


def test_python_api_loads_without_gpu():
    import tinyad_gb300
    L = tinyad_gb300.load()
    assert L.tad_version().decode().startswith("tad-gb300")
    s = tinyad_gb300.default_settings()
    assert s.ls_max_iters == 64 and abs(s.ls_shrink - 0.8) < 1e-15 and abs(s.ls_armijo - 1e-4) < 1e-18


def test_problem_create_fails_loudly_without_gpu():
    """No CPU fallback: without a GPU, creating a problem is an error."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import tinyad_gb300
    with pytest.raises(RuntimeError):
        tinyad_gb300.ScalarFunction(2, 3)


def test_frontend_test_program_builds():
    """The C++ front end compiles as a user translation unit (no GPU needed)."""
    from tinyad_gb300 import build
    build.build()
    assert os.path.exists(build.FRONTEND_BIN)
