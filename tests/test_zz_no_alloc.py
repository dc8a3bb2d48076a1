"""The allocation-free pipeline entry point, mpkg_pipe_noalloc.

Some callers cannot allocate device memory themselves (a solver plug-in
inside an application whose memory pool owns the device, or a loop that
cannot take cudaMalloc's implicit synchronisation).  For them the library
keeps the pipeline's bookkeeping in a fixed file-scope device array and the
caller passes only the matrix and vv.  This test calls it through the C ABI
with device buffers the test allocates, twice in a row, and compares with
the plan-based pipeline entry point (same arithmetic, so bit for bit).
Collected last so that a stop-at-first-failure run has run everything
else; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import mpk_gb300 as M

pytestmark = pytest.mark.gpu


def _noalloc():
    f = M.lib().mpkg_pipe_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    return f


def test_noalloc_matches_plan_pipeline_twice(gpu):
    import torch
    a = M.Csr.laplacian(96, 64, 40, diag=6.0, off=-1.0)
    k = 6
    x = M.uniform(21, a.n)
    plan = M.Plan.pipe(a, k)
    want = np.zeros((k + 1) * a.n)
    want[:a.n] = x
    plan.exec_host(want)
    d_ptr = torch.from_numpy(a.ptr).cuda()
    d_col = torch.from_numpy(a.col).cuda()
    d_val = torch.from_numpy(a.val).cuda()
    f = _noalloc()
    for call in range(2):
        d_vv = torch.full(((k + 1) * a.n,), float("nan"), dtype=torch.float64, device="cuda")
        d_vv[:a.n] = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        rc = f(a.n, d_ptr.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), k, d_vv.data_ptr(), None)
        assert rc == 0, M.lib().mpkg_last_error().decode()
        got = d_vv.cpu().numpy()
        assert got.tobytes() == want.tobytes(), f"call {call}: {np.count_nonzero(got != want)} entries differ"


def test_noalloc_rejects_sizes_beyond_its_limit(gpu):
    import torch
    f = _noalloc()
    d = torch.zeros(4, dtype=torch.int32, device="cuda")
    v = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = f(4096 * 1024 + 1, d.data_ptr(), d.data_ptr(), v.data_ptr(), 2, v.data_ptr(), None)
    assert rc == M.ERANGE
    assert b"4096*1024" in M.lib().mpkg_last_error()
    rc = f(16, d.data_ptr(), d.data_ptr(), v.data_ptr(), 17, v.data_ptr(), None)
    assert rc == M.EINVAL
