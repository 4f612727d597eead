"""The element kernels' roofline numerator in bench.py (algorithmic flops per
element) is the op count of the library's own arithmetic: the counter in
oracle/ runs include/tad's scalar and projection code with counting types,
and must print the numbers bench.py reports against."""
import json
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_element_flops_match_the_counter():
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = subprocess.run(["sh", os.path.join(ROOT, "oracle", "flop_count.sh")], capture_output=True, text=True,
                         check=True, timeout=600)
    counts = json.loads(out.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench
    assert bench.ELEM_FLOPS[6] == counts["symdir_tri_k6"]["total"]
    assert bench.ELEM_FLOPS[12] == counts["symdir_tet_k12"]["total"]
    # the packed, reduced evaluation does less work than the reference's dense Double<k>
    for key in ("symdir_tri_k6", "symdir_tet_k12"):
        assert counts[key]["eval"] < counts[key]["reference_dense_eval"]
        assert counts[key]["total"] == counts[key]["eval"] + counts[key]["projection"]
