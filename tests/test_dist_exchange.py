"""The pdmpk communication pattern among real CPU ranks: four gloo
processes, one per rank of a reference-prepared buffer set, each computing
its own batches and exchanging every batch's values with
all_to_all_single (the reference's MPI_Ialltoallv, pdmpk/buffers.cc:
163-191).  The gathered result must equal the single-process emulation
(the oracle) bit for bit: what the one-GPU plan replaces by a gather is
exactly this exchange.  Also checks bench.py's barrier / max-over-ranks
helpers with two ranks."""
import os
import socket
import sys
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _vec(data, f, dtype, width=1):
    o, c, size = f
    return np.frombuffer(data[o:o + c * size], dtype=dtype).reshape(-1, width) if width > 1 else \
        np.frombuffer(data[o:o + c * size], dtype=dtype)


def _rank_main(rank, P, port, bufs, res, x, out_path):
    sys.path.insert(0, HERE)
    import pdmpk_cases as PC
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=P)
    data = bufs[rank]
    f = PC.fields(data)
    mbuf_idx = int(np.frombuffer(data[8:12], dtype=np.int32)[0])
    pb = _vec(data, f["mbuf_pb"], np.uint64).astype(np.int64)
    orig = _vec(data, f["orig"], np.int32)
    sc, sd = _vec(data, f["sendcounts"], np.int32), _vec(data, f["sdispls"], np.int32)
    rc, rd = _vec(data, f["recvcounts"], np.int32), _vec(data, f["rdispls"], np.int32)
    sbi, sbpb = _vec(data, f["sbuf_idcs"], np.int32), _vec(data, f["sbuf_pb"], np.uint64).astype(np.int64)
    init, initpb = _vec(data, f["init"], np.int32, 2), _vec(data, f["init_pb"], np.uint64).astype(np.int64)
    mptr, mptrpb = _vec(data, f["mptr"], np.int32), _vec(data, f["mptr_pb"], np.uint64).astype(np.int64)
    mcol, mval = _vec(data, f["mcol"], np.int32), _vec(data, f["mval"], np.float64)
    mbuf = np.zeros(mbuf_idx)
    mbuf[:len(orig)] = x[orig]  # LoadInput with the original indices
    for b in range(len(pb)):  # every batch: exchange, then compute (AsyncExec order)
        cnt_s, cnt_r = sc[b * P:(b + 1) * P], rc[b * P:(b + 1) * P]
        send = mbuf[sbi[sbpb[b]:sbpb[b] + int(cnt_s.sum())]]
        recv = torch.zeros(int(cnt_r.sum()), dtype=torch.float64)
        dist.all_to_all_single(recv, torch.from_numpy(send.copy()), output_split_sizes=cnt_r.tolist(),
                               input_split_sizes=cnt_s.tolist())
        nrow = int(mptrpb[b + 1] - mptrpb[b])
        r0 = int(pb[b]) + nrow
        mbuf[r0:r0 + len(recv)] = recv.numpy()  # rdispls of a batch are contiguous from 0
        ii = int(initpb[b])
        for mi in range(nrow):
            tmp = 0.0
            if ii < initpb[b + 1] and pb[b] + mi == init[ii, 1]:
                tmp = mbuf[init[ii, 0]]
                ii += 1
            for mj in range(mptr[mptrpb[b] + mi], mptr[mptrpb[b] + mi + 1]):
                tmp = tmp + mval[mj] * mbuf[mcol[mj]]
            mbuf[pb[b] + mi] = tmp
    # results.bin: size_t count + original indices, then the (empty) values
    n_res = int(np.frombuffer(res[rank][0:8], dtype=np.uint64)[0])
    res_orig = np.frombuffer(res[rank][8:8 + 4 * n_res], dtype=np.int32)
    res_mbuf = _vec(data, f["res_mbuf"], np.int32)
    part = np.zeros(len(x))
    part[res_orig] = mbuf[res_mbuf]
    t = torch.from_numpy(part)
    dist.all_reduce(t)  # every row has exactly one owner
    if rank == 0:
        np.save(out_path, t.numpy())
    dist.destroy_process_group()


def test_pdmpk_exchange_among_gloo_ranks():
    sys.path.insert(0, HERE)
    import pdmpk_cases as PC
    import mpk_gb300 as M
    from oracle import oracle as O
    g = PC.load()
    case = ("m5p10", 4, 4, 2, 2)
    m, P, L, mm, wm = case
    bufs = [g[f"{m}__{P}_{L}_{mm}_{wm}__r{r}__buf"].tobytes() for r in range(P)]
    res = [g[f"{m}__{P}_{L}_{mm}_{wm}__r{r}__res"].tobytes() for r in range(P)]
    with tempfile.TemporaryDirectory() as d:
        bp, rp = PC.write_case(g, case, d)
        n = M.pdmpk_info(bp, rp)["n"]
        x = M.uniform(13, n)
        want = O.pd_exec(bp, rp, x, O.MODE_SEPARATE)
        out = os.path.join(d, "y.npy")
        mp.spawn(_rank_main, args=(P, _free_port(), bufs, res, x, out), nprocs=P, join=True)
        got = np.load(out)
    assert got.tobytes() == want.tobytes()


def _bench_helpers(rank, port, out_path):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    bench.barrier(2)
    v = bench.reduce_max(2, 1.0 + rank)
    if rank == 0:
        np.save(out_path, np.array([v]))
    dist.destroy_process_group()


def test_bench_max_over_ranks():
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "v.npy")
        mp.spawn(_bench_helpers, args=(_free_port(), out), nprocs=2, join=True)
        assert float(np.load(out)[0]) == 2.0
