"""pdmpk buffers on the GPU: the reference prep's buf.bin / results.bin of
every rank, executed by one plan (a gather per batch for the
MPI_Ialltoallv, one launch per batch over all ranks' rows), bit for bit
against the oracle's emulation of the reference's MPI exec (both
arithmetic modes) and within the FP64 tolerance of the serial chain."""
import numpy as np
import pytest

import mpk_gb300 as M
import pdmpk_cases as PC
from oracle import oracle as O

pytestmark = pytest.mark.gpu

G = PC.load()
CASES = PC.cases(G)
TOL = 1e-13  # relative error of A^k x, FP64


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-np%d-nl%d-mm%d-wm%d" % c)
def test_pdmpk_buffers_bitwise(case, tmp_path, gpu):
    m, P, L, mm, wm = case
    a = M.Csr.read_mtx(PC.write_mtx(G, m, str(tmp_path)))
    bp, rp = PC.write_case(G, case, str(tmp_path))
    x = M.uniform(5, a.n)
    for arith, mode in ((M.ARITH_SEPARATE, O.MODE_SEPARATE), (M.ARITH_FMA, O.MODE_FMA)):
        plan = M.Plan.pdmpk(bp, rp, arith=arith)
        assert (plan.n, plan.nlevel) == (a.n, L)
        vv = np.full((L + 1) * a.n, 7.0)
        vv[:a.n] = x
        plan.exec_host(vv)
        want = O.pd_exec(bp, rp, x, mode)
        assert vv[L * a.n:].tobytes() == want.tobytes()
        assert np.all(vv[a.n:L * a.n] == 7.0)  # intermediate levels untouched
        chain = O.mpk(a.ptr, a.col, a.val, x, L, mode)[L * a.n:]
        assert np.linalg.norm(vv[L * a.n:] - chain) / np.linalg.norm(chain) < TOL


def test_pdmpk_product_prep_runs_on_gpu(tmp_path, gpu):
    """Buffers from the product's own prep (breadth-first partitions)
    execute to the chain's result."""
    a = M.Csr.laplacian(24, 24, 1, diag=4.0, off=-1.0)
    P, L = 6, 5
    bp = [str(tmp_path / f"r{r}.buf.bin") for r in range(P)]
    rp = [str(tmp_path / f"r{r}.results.bin") for r in range(P)]
    M.pdmpk_prep(a, P, L, bp, rp, mirror=0, weight=1, partitioner=M.PD_PART_BFS)
    x = M.uniform(9, a.n)
    plan = M.Plan.pdmpk(bp, rp, arith=M.ARITH_FMA)
    vv = np.zeros((L + 1) * a.n)
    vv[:a.n] = x
    plan.exec_host(vv)
    assert vv[L * a.n:].tobytes() == O.pd_exec(bp, rp, x, O.MODE_FMA).tobytes()
    chain = O.mpk(a.ptr, a.col, a.val, x, L, O.MODE_FMA)[L * a.n:]
    assert np.linalg.norm(vv[L * a.n:] - chain) / np.linalg.norm(chain) < TOL


def test_pdmpk_device_path(tmp_path, gpu):
    import torch
    case = CASES[-1]
    m, P, L, mm, wm = case
    a = M.Csr.read_mtx(PC.write_mtx(G, m, str(tmp_path)))
    bp, rp = PC.write_case(G, case, str(tmp_path))
    x = M.uniform(3, a.n)
    plan = M.Plan.pdmpk(bp, rp, arith=M.ARITH_SEPARATE)
    vv = torch.zeros((L + 1) * a.n, dtype=torch.float64, device="cuda")
    vv[:a.n] = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    plan.exec_device(vv.data_ptr())
    plan.sync()
    got = vv[L * a.n:].cpu().numpy()
    assert got.tobytes() == O.pd_exec(bp, rp, x, O.MODE_SEPARATE).tobytes()


@pytest.mark.parametrize("key", sorted(PC.ctest()))
def test_pdmpk_ctest_shapes_on_gpu(key, tmp_path, gpu):
    """Every CTest shape (tests/CMakeLists.txt:3-42) prepared by the product
    runs on one GPU bit for bit as the oracle's all-rank AsyncExec, and
    passes the reference's check (apps/check.cc:83: cos^2 against the
    chain within 1e-9)."""
    a, bp, rp = PC.ctest_prep(key, str(tmp_path))
    L = int(key.split("_")[2])
    x = M.uniform(17, a.n)
    plan = M.Plan.pdmpk(bp, rp, arith=M.ARITH_FMA)
    vv = np.zeros((L + 1) * a.n)
    vv[:a.n] = x
    plan.exec_host(vv)
    plan.close()
    got = vv[L * a.n:]
    assert got.tobytes() == O.pd_exec(bp, rp, x, O.MODE_FMA).tobytes()
    gold = O.mpk(a.ptr, a.col, a.val, x, L, O.MODE_FMA)[L * a.n:]
    cos2 = float(np.dot(got, gold)) ** 2 / (float(np.dot(got, got)) * float(np.dot(gold, gold)))
    assert abs(cos2 - 1.0) < 1e-9
