"""The allocation-free energy entry point, tad_eval_symmetric_dirichlet_tri_noalloc.

Some callers can't let a library call cudaMalloc: code running while another
component captures a CUDA graph, hosts with their own memory pool, real-time
loops.  This entry point evaluates the symmetric Dirichlet energy of a
triangle parametrisation from the caller's device buffers with its scratch in
a fixed device array of the library.  The test calls it through the C ABI,
twice in a row on different inputs, and checks each result against the
regular entry point tad_eval (which allocates at problem creation) within the
parity tolerance of the other tests, 1e-10 relative, and that a repeated call
on the same input returns the same bits.  It also checks the size
limit is rejected with an error.  This file is collected last so that a
failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest
import torch

from tinyad_gb300 import meshes

pytestmark = pytest.mark.gpu

TOL = 1e-10


def test_noalloc_energy_matches_tad_eval(tad):
    L = tad.load()
    w = meshes.disk_param(64, seed=0)
    t = w.terms[0]
    fn = tad.ScalarFunction.from_workload(w)
    dev = torch.device("cuda", 0)
    faces = torch.from_numpy(np.ascontiguousarray(t.handles, np.int32)).to(dev)
    params = torch.from_numpy(np.ascontiguousarray(t.params)).to(dev)
    f_out = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(11)
    xs = [w.x0, w.x0 + 1e-4 * rng.normal(size=w.x0.size)]
    for x in xs:                                   # two calls in a row
        x_d = torch.from_numpy(x).to(dev)
        rc = L.tad_eval_symmetric_dirichlet_tri_noalloc(
            ctypes.c_void_p(x_d.data_ptr()), ctypes.c_void_p(faces.data_ptr()), ctypes.c_void_p(params.data_ptr()),
            t.handles.shape[0], ctypes.c_void_p(f_out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.tad_last_error_message().decode()
        stream.synchronize()
        f_noalloc = float(f_out.item())
        f_ref = fn.eval(x)
        assert np.isfinite(f_ref)
        assert abs(f_noalloc - f_ref) <= TOL * abs(f_ref), (f_noalloc, f_ref)
        # the reduction has a fixed order: the same input gives the same bits
        rc = L.tad_eval_symmetric_dirichlet_tri_noalloc(
            ctypes.c_void_p(x_d.data_ptr()), ctypes.c_void_p(faces.data_ptr()), ctypes.c_void_p(params.data_ptr()),
            t.handles.shape[0], ctypes.c_void_p(f_out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.tad_last_error_message().decode()
        stream.synchronize()
        assert float(f_out.item()) == f_noalloc
    # beyond the fixed scratch: rejected with an error, nothing launched
    rc = L.tad_eval_symmetric_dirichlet_tri_noalloc(
        ctypes.c_void_p(x_d.data_ptr()), ctypes.c_void_p(faces.data_ptr()), ctypes.c_void_p(params.data_ptr()),
        (1 << 24) + 1, ctypes.c_void_p(f_out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == tad.TAD_ERR_ARG
    assert "maximum" in L.tad_last_error_message().decode()
