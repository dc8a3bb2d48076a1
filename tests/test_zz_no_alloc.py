"""The allocation-free pipeline entry point, mpkg_pipe_noalloc.

Some callers cannot allocate device memory themselves (a solver plug-in
inside an application whose memory pool owns the device, or a loop that
cannot take cudaMalloc's implicit synchronisation).  For them the library
keeps the pipeline's bookkeeping in a fixed file-scope device array and the
caller passes only the matrix and vv.  This test calls it through the C ABI
with device buffers the test allocates, twice in a row, and compares with
the plan-based pipeline entry point and with the CPU oracle's FP64 FMA
chain (same arithmetic, so bit for bit).
Collected last so that a stop-at-first-failure run has run everything
else; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import mpk_gb300 as M
from oracle import oracle as O

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
    plan.close()
    assert want.tobytes() == O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA).tobytes()
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


def _run(f, a, k, x):
    import torch
    d_ptr = torch.from_numpy(a.ptr).cuda()
    d_col = torch.from_numpy(a.col).cuda()
    d_val = torch.from_numpy(a.val).cuda()
    d_vv = torch.full(((k + 1) * a.n,), float("nan"), dtype=torch.float64, device="cuda")
    d_vv[:a.n] = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    rc = f(a.n, d_ptr.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), k, d_vv.data_ptr(), None)
    return rc, d_vv


def test_noalloc_many_more_chunks_than_ctas_matches_oracle(gpu):
    """160^3 Laplacian: 16000 chunks of 256 rows, just under the limit, far
    more than the resident grid, so CTAs take many tickets each and wait on
    chunks that are not resident; bit for bit against the oracle, twice."""
    a = M.Csr.laplacian(160, 160, 160, diag=6.0, off=-1.0)
    k = 4
    x = M.uniform(5, a.n)
    want = O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA)
    f = _noalloc()
    for call in range(2):
        rc, d_vv = _run(f, a, k, x)
        assert rc == 0, M.lib().mpkg_last_error().decode()
        got = d_vv.cpu().numpy()
        assert got.tobytes() == want.tobytes(), f"call {call}: {np.count_nonzero(got != want)} entries differ"


def test_noalloc_rejects_malformed_csr_without_computing(gpu):
    """A column outside [0, n) or a decreasing ptr is found on the device
    before the pipeline runs: an error code, and vv beyond x untouched."""
    f = _noalloc()
    a = M.Csr.laplacian(8, 8, 8, diag=6.0, off=-1.0)
    k = 3
    x = M.uniform(1, a.n)
    for bad in (a.n, -1, 1 << 30):
        col = a.col.copy()
        col[37] = bad
        rc, d_vv = _run(f, M.Csr(a.ptr, col, a.val), k, x)
        assert rc == M.ERANGE, (bad, rc)
        assert b"column" in M.lib().mpkg_last_error()
        assert np.isnan(d_vv[a.n:].cpu().numpy()).all()
    ptr = a.ptr.copy()
    ptr[10], ptr[11] = ptr[11], ptr[10]
    rc, _ = _run(f, M.Csr(ptr, a.col, a.val), k, x)
    assert rc == M.EINVAL
    ptr = a.ptr.copy()
    ptr[0] = 1
    rc, _ = _run(f, M.Csr(ptr, a.col, a.val), k, x)
    assert rc == M.EINVAL
    # a well-formed call still runs after the refusals
    rc, d_vv = _run(f, a, k, x)
    assert rc == 0
    assert d_vv.cpu().numpy().tobytes() == O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA).tobytes()


def test_noalloc_rejects_bandwidth_beyond_the_resident_grid(gpu):
    """4M rows (15625 chunks), tridiagonal plus one entry coupling the first
    and the last row: the dependency reach spans every chunk, more than the
    resident grid can pipeline."""
    n = 4_000_000
    rows = np.arange(n)
    cols = np.stack([rows - 1, rows, rows + 1], axis=1)
    keep = (cols >= 0) & (cols < n)
    cnt = keep.sum(axis=1)
    cnt[0] += 1
    ptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    col = np.empty(ptr[-1], dtype=np.int32)
    col[0:2] = [0, 1]
    col[2] = n - 1
    col[3:] = cols[1:][keep[1:]]
    val = np.full(ptr[-1], 0.25)
    rc, _ = _run(_noalloc(), M.Csr(ptr, col, val), 4, M.uniform(2, n))
    assert rc == M.ERANGE
    assert b"bandwidth" in M.lib().mpkg_last_error()
