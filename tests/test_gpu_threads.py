"""Thread safety per handle: plans used from several host threads at once
(each plan owns its stream; errors are recorded per thread) give the bits
of a single-threaded run.  The persistent executors are cooperative
launches, so concurrent calls also show that their grids never wait on
each other."""
import threading

import numpy as np
import pytest

import mpk_gb300 as M

pytestmark = pytest.mark.gpu


def _run(plan, x, n, k):
    vv = np.zeros((k + 1) * n)
    vv[:n] = x
    plan.exec_host(vv)
    return vv


@pytest.mark.parametrize("kinds", [("wave_df64", "wave_df64"), ("wave_fma", "pipe"), ("spmv", "tasks"),
                                   ("wave_df64", "spmv", "pipe", "wave_fixed")])
def test_concurrent_plans_match_serial(kinds, gpu):
    a0 = M.Csr.laplacian(48, 48, 32)
    a = a0.pattern()
    k = 6
    part = M.partition_rcb(a0.coords, 16)
    make = {"wave_df64": lambda: M.Plan.wave(a, k, arith=M.ARITH_DF64),
            "wave_fixed": lambda: M.Plan.wave(a, k, arith=M.ARITH_FIXED),
            "wave_fma": lambda: M.Plan.wave(a, k),
            "pipe": lambda: M.Plan.pipe(a, k),
            "spmv": lambda: M.Plan.spmv(a, k),
            "tasks": lambda: M.Plan.pa1(a, part, 16, k, exec=M.EXEC_TASKS)}
    plans = [make[kd]() for kd in kinds]
    xs = [M.uniform(40 + t, a.n) for t in range(len(kinds))]
    want = [_run(p, x, a.n, k) for p, x in zip(plans, xs)]
    errors = []

    def worker(t):
        try:
            for _ in range(25):
                got = _run(plans[t], xs[t], a.n, k)
                if got.tobytes() != want[t].tobytes():
                    errors.append(f"{kinds[t]}: bits differ")
                    return
        except Exception as e:  # recorded, the main thread asserts
            errors.append(f"{kinds[t]}: {e}")

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(len(kinds))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for p in plans:
        p.close()
    assert not errors, errors


def test_errors_are_per_thread(gpu):
    """Each thread sees its own last error."""
    msgs = {}

    def worker(t):
        try:
            M.Plan.wave(M.Csr(np.array([0, 1]), np.array([t + 5], dtype=np.int32)), 2)
        except M.MpkError as e:
            msgs[t] = (e.code, str(e))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert sorted(msgs) == [0, 1, 2, 3]
    assert all(code == M.ERANGE for code, _ in msgs.values())
