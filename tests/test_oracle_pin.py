"""Pins the CPU oracle (oracle/mpk_oracle.c) to the reference.

Every check compares the oracle with fixtures produced by the reference
mpk2 code itself (tests/golden/make_golden.py) or, where the reference was
compiled here (oracle/_ref), with the live reference library on random
inputs.  The reference fixtures were made by x86-64 builds that do not
contract a*b+c, so floating-point results are compared bit for bit against
the oracle's "separate" mode.
"""
import hashlib
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_matrix, load_golden
from oracle import oracle as O


def _graph_file(a, d):
    path = os.path.join(d, "g0")
    a.write_metis(path, ne=(a.nnz + a.n) // 2)
    return path


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_prep_matches_reference(name):
    g = load_golden(name)
    a = golden_matrix(name)
    n, npart, nlevel, nphase = int(g["n"]), int(g["npart"]), int(g["nlevel"]), int(g["nphase"])
    with tempfile.TemporaryDirectory() as d:
        ptr, col = O.read_graph(_graph_file(a, d))
        assert np.array_equal(ptr, a.ptr) and np.array_equal(col, a.col)
        parts = g["parts"]
        lev = None
        for ph in range(nphase):
            if ph == 0:
                lv = O.comp_level(ptr, col, parts[0], npart)
            else:
                lv = O.update_level(ptr, col, parts[ph], npart, g["levels"][ph - 1])
            assert np.array_equal(lv, g["levels"][ph]), f"levels phase {ph}"
            _, we = O.level_weights(ptr, col, lv)
            assert np.array_equal(we, g["weights"][ph]), f"weights phase {ph}"
            lev = lv
        sp = os.path.join(d, "s")
        O.write_skirt(sp, ptr, col, parts[0], npart, nlevel, lev)
        with open(sp, "rb") as f:
            assert f.read() == g["skirt"].tobytes(), "skirt file differs from the reference's"
        sl = O.read_skirt(sp, n, npart, nlevel)
        off, idx = O.prep_tasks(ptr, col, npart, nlevel, nphase, parts[: max(nphase, 1)],
                                g["levels"] if nphase else None, sl)
        assert np.array_equal(off, g["off"]) and np.array_equal(idx, g["idx"])


def _bits_equal(a, b):
    return a.tobytes() == b.tobytes()


def _vv_check(g, key, got):
    if key in g:
        assert _bits_equal(got, g[key]), key
    else:
        assert hashlib.sha256(got.tobytes()).digest() == g[key + "_sha256"].tobytes(), key


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_exec_matches_reference_bitwise(name):
    g = load_golden(name)
    a = golden_matrix(name)
    n, nlevel = int(g["n"]), int(g["nlevel"])
    vv = np.zeros((nlevel + 1) * n)
    vv[:n] = g["x"]
    O.exec_tasks(a.ptr, a.col, None, g["off"], g["idx"], vv, O.MODE_SEPARATE)
    _vv_check(g, "vv_deg", vv)
    vv[n:] = 0
    O.exec_tasks(a.ptr, a.col, a.val, g["off"], g["idx"], vv, O.MODE_SEPARATE)
    _vv_check(g, "vv_val", vv)
    vv[n:] = 0
    O.spmv_chain(a.ptr, a.col, None, nlevel, vv, O.MODE_SEPARATE)
    _vv_check(g, "vv_spmv", vv)
    if "gold_x1" in g:
        vv[:] = 0
        vv[:n] = 1.0
        O.spmv_chain(a.ptr, a.col, a.val, nlevel, vv, O.MODE_SEPARATE)
        assert _bits_equal(vv, g["gold_x1"])


def test_oracle_fma_mode_differs_only_by_rounding():
    g = load_golden("cfg1_4_4_0")
    a = golden_matrix("cfg1_4_4_0")
    n, nlevel = int(g["n"]), int(g["nlevel"])
    vv = O.mpk(a.ptr, a.col, a.val, g["x"], nlevel, O.MODE_FMA)
    ref = g["vv_val"]
    for l in range(1, nlevel + 1):
        r = ref[l * n:(l + 1) * n]
        e = np.linalg.norm(vv[l * n:(l + 1) * n] - r) / np.linalg.norm(r)
        assert e < 1e-14


@pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_vs_live_reference_random_graphs(seed):
    """Random sparse symmetric graphs and random partitions: the oracle's
    levels and skirts match the reference tools' files."""
    import subprocess
    import mpk_gb300 as M
    rng = np.random.default_rng(seed)
    n = int(rng.integers(40, 120))
    edges = set()
    for i in range(n):
        for _ in range(int(rng.integers(1, 4))):
            j = int(rng.integers(0, n))
            if i != j:
                edges.add((min(i, j), max(i, j)))
    for i in range(n - 1):  # connected
        edges.add((i, i + 1))
    rows = [[] for _ in range(n)]
    for i, j in sorted(edges):
        rows[i].append(j)
        rows[j].append(i)
    rows = [sorted(r) for r in rows]
    ptr = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    col = np.concatenate(rows).astype(np.int32)
    a = M.Csr(ptr, col)
    npart, nlevel = int(rng.integers(2, 6)), int(rng.integers(2, 6))
    part = rng.integers(0, npart, n).astype(np.int32)
    part[:npart] = np.arange(npart)
    with tempfile.TemporaryDirectory() as d:
        gp = os.path.join(d, "g0")
        a.write_metis(gp, ne=len(edges))
        np.savetxt(os.path.join(d, "p"), part, fmt="%d")
        subprocess.run([O.ref_tool("comp"), "level", gp, "x", os.path.join(d, "p"), os.path.join(d, "l0")],
                       check=True, stdout=subprocess.DEVNULL)
        lref = np.loadtxt(os.path.join(d, "l0"), dtype=np.int32)
        assert np.array_equal(O.comp_level(ptr, col, part, npart), lref)
        subprocess.run([O.ref_tool("skirt"), str(nlevel), gp, "x", os.path.join(d, "p"), os.path.join(d, "s")],
                       check=True, stdout=subprocess.DEVNULL)
        O.write_skirt(os.path.join(d, "s2"), ptr, col, part, npart, nlevel)
        assert open(os.path.join(d, "s"), "rb").read() == open(os.path.join(d, "s2"), "rb").read()


def _bufs_files(g, d):
    paths = []
    r = 0
    while f"bufs{r}" in g:
        p = os.path.join(d, f"rank{r}.bufs")
        g[f"bufs{r}"].tofile(p)
        paths.append(p)
        r += 1
    return paths


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if c != "cfg1_4_4_0"])
def test_oracle_mpi2_exec_equals_reference_gold_chain(name):
    """The reference's own MPI-2 test (mpk2/run_script.sh:21-27): the
    distributed valued exec over the rank buffers written by
    mpi2_mpkwrtbufs equals the serial chain bit for bit."""
    g = load_golden(name)
    with tempfile.TemporaryDirectory() as d:
        paths = _bufs_files(g, d)
        assert len(paths) == int(g["npart"])
        vv = O.bufs_exec(paths, g["x"], int(g["nlevel"]), O.MODE_SEPARATE)
    assert vv.tobytes() == g["vv_val"].tobytes()
