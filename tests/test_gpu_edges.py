"""Edge cases on the GPU, every executor against the oracle: empty rows
(the reference sums no terms and stores 0, mpk2/mpkexec.c:28-34), rows
longer than the staged, tiled and fixed-point limits (the limited forms
refuse them at plan time with MPKG_ERANGE), column offsets beyond the
int16 range, a one-sided structure, and one- and two-row matrices."""
import numpy as np
import pytest

import mpk_gb300 as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _from_rows(rows, coords):
    ptr = np.concatenate([[0], np.cumsum([len(c) for c in rows])]).astype(np.int32)
    return M.Csr(ptr, np.concatenate(rows).astype(np.int32), None, coords)


def _rows(a):
    return [set(a.col[a.ptr[i]:a.ptr[i + 1]].tolist()) for i in range(a.n)]


def _isolate(a, drop):
    """Vertices `drop` become isolated: their rows are emptied and they
    leave every other row (the structure stays symmetric)."""
    drop = set(drop)
    rows = [set() if i in drop else r - drop for i, r in enumerate(_rows(a))]
    return _from_rows([sorted(r) for r in rows], a.coords)


def _add_long_row(a, row, stride):
    """Vertex `row` joined to every stride-th vertex, both ways."""
    rows = _rows(a)
    for c in range(0, a.n, stride):
        rows[row].add(c)
        rows[c].add(row)
    return _from_rows([sorted(r) for r in rows], a.coords)


def _matrices():
    empty = _isolate(M.Csr.laplacian(24, 24), [0, 100, 333, 575])
    wide = _add_long_row(M.Csr.laplacian(40, 40, 40), 7, 150)  # 428 entries spanning 64000 columns
    both = _isolate(_add_long_row(M.Csr.laplacian(30, 30, 10), 4500, 20), [1, 2, 8999])
    # rows 0 and 5 emptied but still read by their neighbours: not symmetric
    lap = M.Csr.laplacian(24, 24)
    rows = _rows(lap)
    rows[0], rows[5] = set(), set()
    onesided = _from_rows([sorted(r) for r in rows], lap.coords)
    return {"empty_rows": empty, "long_far_row": wide, "empty_and_long": both, "one_sided": onesided}


MATS = None  # built on first use, after the session fixture has built the library


def _mat(name):
    global MATS
    if MATS is None:
        MATS = _matrices()
    return MATS[name]


def _run(plan, x, n, nlevel):
    vv = np.zeros((nlevel + 1) * n)
    vv[:n] = x
    plan.exec_host(vv)
    plan.close()
    return vv


def _relerr(got, want, n, nlevel):
    out = []
    for l in range(1, nlevel + 1):
        w = want[l * n:(l + 1) * n]
        out.append(float(np.linalg.norm(got[l * n:(l + 1) * n] - w) / max(np.linalg.norm(w), 1e-300)))
    return max(out)


def _part(a, npart):
    return M.partition_rcb(a.coords, npart)


@pytest.mark.parametrize("name", ["empty_rows", "long_far_row", "empty_and_long", "one_sided"])
@pytest.mark.parametrize("valued", [False, True])
def test_fma_executors_bitwise(name, valued, gpu):
    a = _mat(name)
    if valued:
        a = M.Csr(a.ptr, a.col, M.uniform(3, a.nnz), a.coords)
    k = 5
    x = M.uniform(11, a.n)
    want = O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA)
    part = _part(a, 8)
    plans = {"spmv": lambda: M.Plan.spmv(a, k), "wave": lambda: M.Plan.wave(a, k),
             "pipe": lambda: M.Plan.pipe(a, k)}
    if name != "one_sided":  # PA1 needs a symmetric structure (below)
        plans["tasks"] = lambda: M.Plan.pa1(a, part, 8, k, exec=M.EXEC_TASKS)
        if np.diff(a.ptr).max() <= 255:
            plans["tiles"] = lambda: M.Plan.pa1(a, part, 8, k, exec=M.EXEC_TILES)
        else:  # the tiles' sliced layout stores row lengths in a byte
            with pytest.raises(M.MpkError) as e:
                M.Plan.pa1(a, part, 8, k, exec=M.EXEC_TILES)
            assert e.value.code == M.ERANGE
    for ex, mk in plans.items():
        got = _run(mk(), x, a.n, k)
        bad = np.flatnonzero(got.view(np.int64) != want.view(np.int64))
        assert bad.size == 0, f"{ex}: {bad.size} words differ, first at {bad[:5]}"


@pytest.mark.parametrize("name", ["empty_rows", "long_far_row", "empty_and_long"])
def test_double_float_executors_within_tolerance(name, gpu):
    a = _mat(name).pattern()
    k = 5
    x = M.uniform(12, a.n)
    want = O.mpk(a.ptr, a.col, None, x, k, O.MODE_FMA)
    empty = np.flatnonzero(np.diff(a.ptr) == 0)
    part = _part(a, 8)
    plans = {"wave": lambda: M.Plan.wave(a, k, arith=M.ARITH_DF64),
             "pipe": lambda: M.Plan.pipe(a, k, arith=M.ARITH_DF64)}
    if np.diff(a.ptr).max() <= 255:
        plans["tiles"] = lambda: M.Plan.pa1(a, part, 8, k, exec=M.EXEC_TILES, arith=M.ARITH_DF64)
    for ex, mk in plans.items():
        got = _run(mk(), x, a.n, k)
        assert _relerr(got, want, a.n, k) <= TOL, ex
        for l in range(1, k + 1):  # an empty row is exactly +0
            assert np.all(got[l * a.n + empty].view(np.int64) == 0), ex


def test_fixed_point_limits(gpu):
    a = _mat("empty_rows").pattern()
    k = 6
    x = M.uniform(13, a.n)
    want = O.mpk(a.ptr, a.col, None, x, k, O.MODE_FMA)
    got = _run(M.Plan.wave(a, k, arith=M.ARITH_FIXED), x, a.n, k)
    assert _relerr(got, want, a.n, k) <= TOL
    empty = np.flatnonzero(np.diff(a.ptr) == 0)
    assert np.all(got[a.n:].reshape(k, a.n)[:, empty] == 0.0)
    with pytest.raises(M.MpkError) as e:  # a row of 427 entries is beyond the form's 255
        M.Plan.wave(_mat("long_far_row").pattern(), k, arith=M.ARITH_FIXED)
    assert e.value.code == M.ERANGE


def test_pa1_refuses_one_sided_structure(gpu):
    """PA1's distance-bounded tiles assume that j is a neighbour of i when i
    is a neighbour of j (graphs from METIS files are); a one-sided structure
    is refused at plan time instead of computing with missing inputs."""
    a = _mat("one_sided").pattern()
    with pytest.raises(M.MpkError) as e:
        M.Plan.pa1(a, _part(a, 8), 8, 4, exec=M.EXEC_TILES)
    assert e.value.code == M.ESTRUCT


@pytest.mark.parametrize("rows", [
    ([0, 1], [0]),           # one row, a self loop
    ([0, 1, 1], [1]),        # two rows, the second empty
    ([0, 2, 3], [0, 1, 1]),  # two rows
])
def test_tiny_matrices(rows, gpu):
    ptr, col = rows
    a = M.Csr(np.array(ptr), np.array(col, dtype=np.int32))
    k = 3
    x = np.array([0.75, -0.5][:a.n])
    want = O.mpk(a.ptr, a.col, None, x, k, O.MODE_FMA)
    for mk in (lambda: M.Plan.spmv(a, k), lambda: M.Plan.wave(a, k), lambda: M.Plan.pipe(a, k),
               lambda: M.Plan.wave(a, k, arith=M.ARITH_DF64), lambda: M.Plan.wave(a, k, arith=M.ARITH_FIXED)):
        got = _run(mk(), x, a.n, k)
        assert np.allclose(got, want, rtol=1e-15, atol=0), (got, want)


def test_matrix_without_entries_is_rejected(gpu):
    """A matrix with no entries at all is refused at plan time (EINVAL);
    the reference would return all-zero powers."""
    a = M.Csr(np.array([0, 0, 0]), np.zeros(0, dtype=np.int32))
    for mk in (lambda: M.Plan.spmv(a, 2), lambda: M.Plan.wave(a, 2), lambda: M.Plan.pipe(a, 2)):
        with pytest.raises(M.MpkError) as e:
            mk()
        assert e.value.code == M.EINVAL


def _random_csr(n, seed, unsorted, dups, far):
    """Random rows of 0..12 entries; columns near the row (or anywhere with
    `far`), optionally unsorted within rows and with repeated columns."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n):
        k = int(rng.integers(0, 13))
        if far:
            c = rng.integers(0, n, size=k)
        else:
            c = np.clip(i + rng.integers(-300, 301, size=k), 0, n - 1)
        if dups and k > 1:
            c[-1] = c[0]
        if not unsorted:
            c = np.sort(c)
        rows.append(c.astype(np.int32))
    ptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    return M.Csr(ptr, np.concatenate(rows).astype(np.int32), M.uniform(seed + 1, int(ptr[-1])))


@pytest.mark.parametrize("unsorted,dups,far", [(False, False, False), (True, False, False), (True, True, False),
                                               (False, False, True)])
def test_random_structures_bitwise(unsorted, dups, far, gpu):
    """Random sparse rows (empty rows included), columns in any order and
    repeated: the rows are summed in the stored order, as the reference
    does, so every executor matches the oracle bit for bit (valued and
    1/deg operators)."""
    a = _random_csr(20000, 31, unsorted, dups, far)
    k = 5
    x = M.uniform(32, a.n)
    for op in (a, a.pattern()):
        want = O.mpk(op.ptr, op.col, op.val, x, k, O.MODE_FMA)
        for ex, mk in (("spmv", lambda: M.Plan.spmv(op, k)), ("wave", lambda: M.Plan.wave(op, k)),
                       ("pipe", lambda: M.Plan.pipe(op, k))):
            try:
                plan = mk()
            except M.MpkError as e:  # the pipeline's chunk window cannot span columns anywhere
                assert ex == "pipe" and far and e.code == M.ERANGE, (ex, str(e))
                continue
            got = _run(plan, x, a.n, k)
            bad = np.flatnonzero(got.view(np.int64) != want.view(np.int64))
            assert bad.size == 0, f"{ex}: {bad.size} words differ"
        got = _run(M.Plan.wave(op, k, arith=M.ARITH_DF64), x, a.n, k)
        assert _relerr(got, want, a.n, k) <= TOL
