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
@pytest.mark.parametrize("tune", [False, True, M.BATCH_STAGED, M.BATCH_STAGED2, M.BATCH_STAGED4])
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
    if not isinstance(tune, bool):
        assert info["staged"] == 1
        assert info["threads"] == {M.BATCH_STAGED: 1024, M.BATCH_STAGED2: 512, M.BATCH_STAGED4: 256}[tune]


@pytest.mark.parametrize("mode", [M.BATCH_STAGED, M.BATCH_STAGED2, M.BATCH_STAGED4])
@pytest.mark.parametrize("nrhs", [4, 32])
def test_batch_staged_partial_windows(mode, nrhs, gpu):
    """3-D stencils whose z-neighbours lie beyond the shared-memory window
    (at 32 right-hand sides the window holds 0.4-1.8 K rows, the
    z-stride is 1.6-2.5 K rows on each side; at 4 most spans fit): the
    entries outside it are read from global memory, the bits stay the
    oracle's.  Rows of 40-60 entries take the row loop's tail path."""
    mats = [M.Csr.laplacian(40, 40, 40, diag=6.0, off=-1.0), M.Csr.diffusion(50, 50, 24, sigma=0.5, seed=3),
            M.Csr.banded(5000, 64, 5, 30, seed=5), M.Csr.laplacian(7, 3, 1, diag=4.0, off=-1.0),
            M.Csr.banded(3000, 64, 40, 60, seed=6)]
    k = 5
    X = _inputs(mats, nrhs, 11)
    plan = M.Plan.batch(mats, nrhs, k, tune=mode)
    info = plan.batch_info()
    assert info["staged"] == 1 and info["window_bytes"] > 0
    vb = np.zeros((k + 1,) + X.shape, dtype=np.float32)
    vb[0] = X
    plan.exec_batch_host(vb)
    assert vb.tobytes() == _oracle(mats, X, k).tobytes()


@pytest.mark.parametrize("nrhs", [64, 128])
def test_batch_staged_wide_rows(small_batch, nrhs, gpu):
    """16 and 32 lanes per row (float4 each) in the window kernel: the
    window holds 110-450 rows of 256-512 bytes, the bits stay the
    oracle's."""
    mats, k = small_batch[:6], 3
    X = _inputs(mats, nrhs, 13)
    for mode in (M.BATCH_STAGED2, M.BATCH_STAGED4):
        plan = M.Plan.batch(mats, nrhs, k, tune=mode)
        info = plan.batch_info()
        assert info["staged"] == 1 and info["lanes_per_row"] == nrhs // 4
        vb = np.zeros((k + 1,) + X.shape, dtype=np.float32)
        vb[0] = X
        plan.exec_batch_host(vb)
        assert vb.tobytes() == _oracle(mats, X, k).tobytes()


def test_batch_staged_needs_four_rhs(small_batch, gpu):
    with pytest.raises(M.MpkError) as e:
        M.Plan.batch(small_batch, 2, 3, tune=M.BATCH_STAGED)
    assert e.value.code == M.EINVAL


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


@pytest.mark.parametrize("mode", [False, M.BATCH_STAGED, M.BATCH_STAGED4])
def test_batch_wait_times_out_and_recovers(small_batch, mode, gpu):
    """The batched form's bounded waits give up on a flag that is never set
    (ETIMEOUT) and the same plan, its graph captured again, then runs bit
    for bit."""
    mats, k = small_batch, 6
    X = _inputs(mats, 16, 9)
    plan = M.Plan.batch(mats, 16, k, tune=mode)
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
