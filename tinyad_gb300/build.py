"""Build the CUDA library (libtad.so) in-tree for sm_103a.

One nvcc process per translation unit, in parallel, then one link.  Output:
tinyad_gb300/_build/libtad.so (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtad.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "--extended-lambda",
              "-Xcompiler", "-fPIC,-fvisibility=hidden,-fopenmp", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime() -> float:
    m = os.path.getmtime(FRONTEND_SRC) if os.path.exists(FRONTEND_SRC) else 0.0
    for d in (CSRC, os.path.join(ROOT, "include"), os.path.join(ROOT, "include", "tad")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".hh")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    flags = NVCC_FLAGS + (extra_flags or [])
    objs = []

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc()] + ARCH + flags + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_frontend_test()
    return LIB


FRONTEND_SRC = os.path.join(ROOT, "tests", "cpp", "frontend_test.cu")
FRONTEND_BIN = os.path.join(OUT, "frontend_test")


def build_frontend_test() -> str:
    """The C++ front-end test program (tests/cpp/frontend_test.cu), a user
    translation unit compiled against include/tad/ScalarFunction.cuh and
    linked with libtad.so."""
    cmd = [nvcc()] + ARCH + ["-std=c++17", "-O2", "--extended-lambda", "--expt-relaxed-constexpr",
                             "-I", os.path.join(ROOT, "include"), FRONTEND_SRC, "-o", FRONTEND_BIN,
                             "-L", OUT, "-ltad", "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"front-end test build failed:\n{r.stdout}\n{r.stderr}")
    return FRONTEND_BIN


if __name__ == "__main__":
    t = __import__("time").time()
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(f"{__import__('time').time() - t:.1f}s")
