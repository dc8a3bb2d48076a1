"""GPU parity: every executor against the reference's own results (golden
fixtures, bit for bit in the reference's non-contracted arithmetic) and
against the oracle (bit for bit in FMA arithmetic), plus the FP64 tolerance
of the task (1e-13 relative per power vector) and full-size checks on the
128^3 7-point workload."""
import hashlib
import os
import tempfile

import numpy as np
import pytest

import mpk_gb300 as M
from conftest import GOLDEN_CASES, golden_matrix, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-13  # relative error per power vector, FP64 paths


def _check_bits(g, key, vv):
    if key in g:
        bad = np.flatnonzero(vv.view(np.int64) != g[key].view(np.int64))
        assert bad.size == 0, f"{key}: {bad.size} words differ, first at {bad[:5]}"
    else:
        assert hashlib.sha256(vv.tobytes()).digest() == g[key + "_sha256"].tobytes(), key


def _run(plan, x, n, nlevel):
    vv = np.zeros((nlevel + 1) * n)
    vv[:n] = x
    plan.exec_host(vv)
    return vv


def _plans(name, g, a, arith):
    n, npart, nlevel, nphase = int(g["n"]), int(g["npart"]), int(g["nlevel"]), int(g["nphase"])
    out = {"tasks": M.Plan.from_tasks(a, npart, nlevel, nphase, g["off"], g["idx"], arith=arith),
           "spmv": M.Plan.spmv(a, nlevel, arith=arith),
           "pipe": M.Plan.pipe(a, nlevel, arith=arith),
           "wave": M.Plan.wave(a, nlevel, arith=arith)}
    if nphase == 0:
        out["tiles"] = M.Plan.pa1(a, g["parts"][0], npart, nlevel, exec=M.EXEC_TILES, arith=arith)
        out["pa1_tasks"] = M.Plan.pa1(a, g["parts"][0], npart, nlevel, exec=M.EXEC_TASKS, arith=arith)
    return out


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("valued", [False, True])
def test_executors_bitwise_vs_reference(name, valued, gpu):
    g = load_golden(name)
    a = golden_matrix(name)
    if not valued:
        a = a.pattern()
    n, nlevel = int(g["n"]), int(g["nlevel"])
    key = "vv_val" if valued else "vv_deg"
    for ex, plan in _plans(name, g, a, M.ARITH_SEPARATE).items():
        vv = _run(plan, g["x"], n, nlevel)
        _check_bits(g, key, vv)
        if not valued:
            _check_bits(g, "vv_spmv", vv)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_executors_bitwise_vs_oracle_fma(name, gpu):
    g = load_golden(name)
    a = golden_matrix(name)
    n, nlevel = int(g["n"]), int(g["nlevel"])
    want = O.mpk(a.ptr, a.col, a.val, g["x"], nlevel, O.MODE_FMA)
    for ex, plan in _plans(name, g, a, M.ARITH_FMA).items():
        vv = _run(plan, g["x"], n, nlevel)
        assert vv.tobytes() == want.tobytes(), ex


def test_config1_fp64_tolerance_vs_reference(gpu):
    """Config 1 (100^2 5-point, k=4, 4 parts): the default (FMA) GPU result
    is within 1e-13 per power vector of the reference's valued exec and of
    verify_val's gold chain (x = 1)."""
    g = load_golden("cfg1_4_4_0")
    a = golden_matrix("cfg1_4_4_0")
    n, nlevel = int(g["n"]), int(g["nlevel"])
    for ex, plan in _plans("cfg1_4_4_0", g, a, M.ARITH_FMA).items():
        for x, ref in ((g["x"], g["vv_val"]), (np.ones(n), g["gold_x1"])):
            vv = _run(plan, x, n, nlevel)
            for l in range(1, nlevel + 1):
                r = ref[l * n:(l + 1) * n]
                err = np.linalg.norm(vv[l * n:(l + 1) * n] - r) / np.linalg.norm(r)
                assert err <= TOL, (ex, l, err)


def test_all_ones_fixed_point_deg_operator(gpu):
    """The row-normalised operator maps 1 to 1 (mpk2/mpktest.c:43-51)."""
    a = M.Csr.laplacian(40, 30, 20).pattern()
    part = M.partition_rcb(a.coords, 64)
    for plan in (M.Plan.pa1(a, part, 64, 6), M.Plan.pipe(a, 6), M.Plan.spmv(a, 6), M.Plan.wave(a, 6),
                 M.Plan.wave(a, 6, arith=M.ARITH_DF64)):
        vv = _run(plan, np.ones(a.n), a.n, 6)
        assert np.max(np.abs(vv - 1.0)) < 1e-14


def test_device_pointer_path_matches_host_path(gpu):
    import torch
    a = M.Csr.laplacian(64, 64, 8)
    part = M.partition_rcb(a.coords, 32)
    x = M.uniform(11, a.n)
    for plan in (M.Plan.pa1(a, part, 32, 5), M.Plan.pipe(a, 5), M.Plan.spmv(a, 5), M.Plan.wave(a, 5),
                 M.Plan.wave(a, 5, arith=M.ARITH_DF64)):
        want = _run(plan, x, a.n, 5)
        d = torch.zeros(6 * a.n, dtype=torch.float64, device="cuda")
        d[:a.n] = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        for _ in range(3):  # repeated launches reuse the plan (pipeline epochs)
            plan.exec_device(d.data_ptr())
            plan.sync()
        assert d.cpu().numpy().tobytes() == want.tobytes()


@pytest.fixture(scope="module")
def config2():
    a = M.Csr.laplacian(128, 128, 128, diag=6.0, off=-1.0)
    part = M.partition_rcb(a.coords, 2048)
    x = M.uniform(1, a.n)
    want = O.mpk(a.ptr, a.col, a.val, x, 8, O.MODE_FMA)
    return a, part, x, want


@pytest.mark.parametrize("ex", ["tiles", "pipe", "spmv", "wave"])
def test_config2_full_size_bitwise_vs_oracle(config2, ex, gpu):
    """128^3 7-point, k=8, 2048 parts: bit-identical to the oracle chain."""
    a, part, x, want = config2
    plan = {"tiles": lambda: M.Plan.pa1(a, part, 2048, 8),
            "pipe": lambda: M.Plan.pipe(a, 8),
            "spmv": lambda: M.Plan.spmv(a, 8),
            "wave": lambda: M.Plan.wave(a, 8)}[ex]()
    vv = _run(plan, x, a.n, 8)
    bad = np.flatnonzero(vv.view(np.int64) != want.view(np.int64))
    assert bad.size == 0, f"{bad.size} differ, first {bad[:5]}"


def _rel_errors(vv, want, n, nlevel):
    out = []
    for l in range(1, nlevel + 1):
        r = want[l * n:(l + 1) * n]
        out.append(float(np.linalg.norm(vv[l * n:(l + 1) * n] - r) / np.linalg.norm(r)))
    return out


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("valued", [False, True])
def test_df64_executors_within_fp64_tolerance(name, valued, gpu):
    """Double-float arithmetic (FP32 pipes) with FP64 storage stays within
    the FP64 tolerance of the reference's results."""
    g = load_golden(name)
    a = golden_matrix(name)
    if not valued:
        a = a.pattern()
    n, npart, nlevel, nphase = int(g["n"]), int(g["npart"]), int(g["nlevel"]), int(g["nphase"])
    want = O.mpk(a.ptr, a.col, a.val, g["x"], nlevel, O.MODE_FMA)
    plans = {"pipe": M.Plan.pipe(a, nlevel, arith=M.ARITH_DF64), "wave": M.Plan.wave(a, nlevel, arith=M.ARITH_DF64)}
    if nphase == 0:
        plans["tiles"] = M.Plan.pa1(a, g["parts"][0], npart, nlevel, arith=M.ARITH_DF64)
    for ex, plan in plans.items():
        vv = _run(plan, g["x"], n, nlevel)
        assert vv[:n].tobytes() == g["x"].tobytes()
        errs = _rel_errors(vv, want, n, nlevel)
        assert max(errs) <= TOL, (ex, errs)


@pytest.mark.parametrize("ex", ["tiles", "pipe", "wave"])
def test_config2_df64_within_fp64_tolerance(config2, ex, gpu):
    a, part, x, want = config2
    plan = {"tiles": lambda: M.Plan.pa1(a, part, 2048, 8, arith=M.ARITH_DF64),
            "pipe": lambda: M.Plan.pipe(a, 8, arith=M.ARITH_DF64),
            "wave": lambda: M.Plan.wave(a, 8, arith=M.ARITH_DF64)}[ex]()
    vv = _run(plan, x, a.n, 8)
    errs = _rel_errors(vv, want, a.n, 8)
    assert max(errs) <= TOL, errs


@pytest.mark.parametrize("kind", ["pipe", "wave", "wave_df64"])
def test_pipeline_wait_times_out_and_recovers(kind, gpu):
    """A dependency flag that is never set: the bounded waits give up, the
    call reports ETIMEOUT, and the same plan then runs correctly."""
    a = M.Csr.laplacian(64, 64, 4)
    x = M.uniform(5, a.n)
    plan = {"pipe": lambda: M.Plan.pipe(a, 4), "wave": lambda: M.Plan.wave(a, 4),
            "wave_df64": lambda: M.Plan.wave(a, 4, arith=M.ARITH_DF64)}[kind]()
    plan.debug_stall(100)
    vv = np.zeros(5 * a.n)
    vv[:a.n] = x
    with pytest.raises(M.MpkError) as e:
        plan.exec_host(vv)
    assert e.value.code == M.ETIMEOUT
    plan.debug_stall(0)
    want = O.mpk(a.ptr, a.col, a.val, x, 4, O.MODE_FMA)
    got = _run(plan, x, a.n, 4)
    if kind == "wave_df64":
        assert max(_rel_errors(got, want, a.n, 4)) <= TOL
    else:
        assert got.tobytes() == want.tobytes()


def _bufs_dir(g, d):
    r = 0
    while f"bufs{r}" in g:
        g[f"bufs{r}"].tofile(os.path.join(d, f"rank{r}.bufs"))
        r += 1
    return r


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if c != "cfg1_4_4_0"])
def test_rank_buffers_on_gpu_bitwise(name, gpu):
    """The reference's MPI-2 rank buffers (written by its mpi2_mpkwrtbufs)
    executed by one GPU launch per phase: bit-identical to the reference's
    serial valued chain (the check of mpk2/run_script.sh:27), and to the
    oracle's emulation of the MPI exec in FMA arithmetic."""
    g = load_golden(name)
    n, nlevel = int(g["n"]), int(g["nlevel"])
    with tempfile.TemporaryDirectory() as d:
        P = _bufs_dir(g, d)
        plan = M.Plan.bufs(d, P, arith=M.ARITH_SEPARATE)
        vv = _run(plan, g["x"], n, nlevel)
        _check_bits(g, "vv_val", vv)
        plan = M.Plan.bufs(d, P, arith=M.ARITH_FMA)
        vv = _run(plan, g["x"], n, nlevel)
        want = O.bufs_exec([os.path.join(d, f"rank{r}.bufs") for r in range(P)], g["x"], nlevel, O.MODE_FMA)
        assert vv.tobytes() == want.tobytes()


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_fixed_point_wave_within_fp64_tolerance(name, gpu):
    """64-bit fixed-point rows (1/deg operator) stay within the FP64
    tolerance of the reference's exec_mpk_xd results."""
    g = load_golden(name)
    a = golden_matrix(name).pattern()
    n, nlevel = int(g["n"]), int(g["nlevel"])
    want = O.mpk(a.ptr, a.col, None, g["x"], nlevel, O.MODE_FMA)
    vv = _run(M.Plan.wave(a, nlevel, arith=M.ARITH_FIXED), g["x"], n, nlevel)
    assert vv[:n].tobytes() == g["x"].tobytes()
    errs = _rel_errors(vv, want, n, nlevel)
    assert max(errs) <= TOL, errs


def test_fixed_point_full_size_and_known_answers(config2, gpu):
    a, part, x, _ = config2
    g = a.pattern()
    want = O.mpk(g.ptr, g.col, None, x, 8, O.MODE_FMA)
    plan = M.Plan.wave(g, 8, arith=M.ARITH_FIXED)
    errs = _rel_errors(_run(plan, x, a.n, 8), want, a.n, 8)
    assert max(errs) <= TOL, errs
    ones = _run(plan, np.ones(a.n), a.n, 8)  # the 1/deg operator's fixed point, exactly
    assert np.all(ones == 1.0)
    big = _run(plan, 1e6 * x, a.n, 8)  # the scale follows max|x|
    assert max(_rel_errors(big, 1e6 * want, a.n, 8)) <= TOL
    with pytest.raises(M.MpkError):  # the valued operator has no fixed-point form
        M.Plan.wave(a, 8, arith=M.ARITH_FIXED)


def test_fixed_point_wait_times_out_and_recovers(gpu):
    a = M.Csr.laplacian(64, 64, 4).pattern()
    x = M.uniform(5, a.n)
    plan = M.Plan.wave(a, 4, arith=M.ARITH_FIXED)
    plan.debug_stall(100)
    vv = np.zeros(5 * a.n)
    vv[:a.n] = x
    with pytest.raises(M.MpkError) as e:
        plan.exec_host(vv)
    assert e.value.code == M.ETIMEOUT
    plan.debug_stall(0)
    want = O.mpk(a.ptr, a.col, None, x, 4, O.MODE_FMA)
    assert max(_rel_errors(_run(plan, x, a.n, 4), want, a.n, 4)) <= TOL


@pytest.mark.parametrize("valued", [False, True])
@pytest.mark.parametrize("arith", [M.ARITH_DF64, M.ARITH_FIXED, M.ARITH_FMA, M.ARITH_SEPARATE])
def test_host_mapped_execution_matches_device(arith, valued, gpu):
    """Page-locked host vv runs the wavefront through the host mapping (the
    ring forms keep their levels on the device; the FP64 forms write every
    level to the device copy and through the mapping); pageable vv goes
    through the copies; both give the device path's bits, twice in a row."""
    import torch
    if arith == M.ARITH_FIXED and valued:
        pytest.skip("fixed point runs the 1/deg operator only")
    a = M.Csr.laplacian(64, 64, 16)
    a = a if valued else a.pattern()
    k = 6
    x = M.uniform(21, a.n)
    plan = M.Plan.wave(a, k, arith=arith)
    d = torch.zeros((k + 1) * a.n, dtype=torch.float64, device="cuda")
    d[:a.n] = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    plan.exec_device(d.data_ptr())
    plan.sync()
    want = d.cpu().numpy()
    pinned = torch.zeros((k + 1) * a.n, dtype=torch.float64).pin_memory()
    pinned[:a.n] = torch.from_numpy(x)
    got_pinned = plan.exec_host(pinned.numpy()).copy()
    pinned[a.n:] = float("nan")
    again = plan.exec_host(pinned.numpy())
    got_pageable = _run(plan, x, a.n, k)
    plan.close()
    assert got_pinned.tobytes() == want.tobytes()
    assert again.tobytes() == want.tobytes()
    assert got_pageable.tobytes() == want.tobytes()
    assert np.array_equal(got_pinned[:a.n], x)  # x is read, not written


@pytest.mark.parametrize("arith,valued", [(M.ARITH_DF64, False), (M.ARITH_DF64, True), (M.ARITH_FIXED, False)])
def test_kspmv_same_arithmetic_as_wavefront(arith, valued, gpu):
    """The k-SpMV baseline in double-float and fixed point computes the
    wavefront's rows in the same arithmetic: the same bits, level for
    level, and within 1e-13 of the FP64 chain (so that the MPK/k-SpMV
    speed-up compares like with like)."""
    a = M.Csr.laplacian(48, 40, 36, diag=6.0, off=-1.0)
    a = a if valued else a.pattern()
    k = 8
    x = M.uniform(31, a.n)
    sp = M.Plan.spmv(a, k, arith=arith)
    wv = M.Plan.wave(a, k, arith=arith)
    got, want = _run(sp, x, a.n, k), _run(wv, x, a.n, k)
    info = sp.info()
    sp.close()
    wv.close()
    assert got.tobytes() == want.tobytes()
    ref = O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA)
    assert max(_rel_errors(got, ref, a.n, k)) <= TOL
    assert info["launches"] == k + (1 if arith == M.ARITH_DF64 else 2)
