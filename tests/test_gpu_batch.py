"""Batched block-vector form on the GPU: many matrices x 16 right-hand
sides in one persistent (graph-replayed) launch, bit for bit against the
oracle's FP32 chain (single-precision FMA per entry in CSR order), and its
error against FP64."""
import numpy as np
import pytest

import mpk_gb300 as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_batch():
    return M.batch_workload(count=12, nmin=200, nmax=3000, seed=4)


def _inputs(mats, nrhs, seed):
    N = sum(m.n for m in mats)
    return M.uniform(seed, N * nrhs).astype(np.float32).reshape(N, nrhs)


def _oracle(mats, X, nlevel):
    outs, r0 = [], 0
    for m in mats:
        outs.append(O.spmm_f32(m.ptr, m.col, m.val.astype(np.float32), X[r0:r0 + m.n], nlevel))
        r0 += m.n
    return np.concatenate(outs, axis=1)


@pytest.mark.parametrize("nrhs", [4, 16, 32])
@pytest.mark.parametrize("tune", [False, True])
def test_batch_bitwise_vs_oracle(small_batch, nrhs, tune, gpu):
    mats, k = small_batch, 6
    X = _inputs(mats, nrhs, 7)
    plan = M.Plan.batch(mats, nrhs, k, tune=tune)
    vb = np.zeros((k + 1,) + X.shape, dtype=np.float32)
    vb[0] = X
    plan.exec_batch_host(vb)
    want = _oracle(mats, X, k)
    assert vb.tobytes() == want.tobytes()
    info = plan.batch_info()
    assert info["lanes_per_row"] * info["vector_width"] == nrhs
    assert info["nmat"] == len(mats) and info["rows"] == X.shape[0]


def test_batch_error_vs_fp64(small_batch, gpu):
    """FP32 values and vectors: per-power relative error against an FP64
    chain stays at single-precision level."""
    import scipy.sparse as sp
    mats, k, nrhs = small_batch, 6, 16
    X = _inputs(mats, nrhs, 9)
    plan = M.Plan.batch(mats, nrhs, k)
    vb = np.zeros((k + 1,) + X.shape, dtype=np.float32)
    vb[0] = X
    plan.exec_batch_host(vb)
    r0 = 0
    for m in mats:
        A = sp.csr_matrix((m.val, m.col, m.ptr), shape=(m.n, m.n))
        v = X[r0:r0 + m.n].astype(np.float64)
        for l in range(1, k + 1):
            v = A @ v
            got = vb[l, r0:r0 + m.n].astype(np.float64)
            assert np.linalg.norm(got - v) / np.linalg.norm(v) < 2e-5
        r0 += m.n


def test_batch_graph_replay_device(small_batch, gpu):
    import torch
    mats, k, nrhs = small_batch, 6, 16
    X = _inputs(mats, nrhs, 3)
    plan = M.Plan.batch(mats, nrhs, k)
    d = torch.zeros((k + 1,) + X.shape, dtype=torch.float32, device="cuda")
    d[0] = torch.from_numpy(X).cuda()
    torch.cuda.synchronize()
    for _ in range(4):  # first call captures the graph, later calls replay it
        plan.exec_batch_device(d.data_ptr())
        plan.sync()
    assert plan.batch_info()["graph"] == 1
    assert d.cpu().numpy().tobytes() == _oracle(mats, X, k).tobytes()


def test_batch_wait_times_out_and_recovers(small_batch, gpu):
    """The batched form's bounded waits give up on a flag that is never set
    (ETIMEOUT) and the same plan, its graph captured again, then runs bit
    for bit."""
    mats, k = small_batch, 6
    X = _inputs(mats, 16, 9)
    plan = M.Plan.batch(mats, 16, k, tune=False)
    plan.debug_stall(100)
    vb = np.zeros((k + 1,) + X.shape, dtype=np.float32)
    vb[0] = X
    with pytest.raises(M.MpkError) as e:
        plan.exec_batch_host(vb)
    assert e.value.code == M.ETIMEOUT
    plan.debug_stall(0)
    vb[1:] = 0
    plan.exec_batch_host(vb)
    assert vb.tobytes() == _oracle(mats, X, k).tobytes()
