"""The reference's verification tools restated in the library, against
their known answers (fixtures made by tests/golden/make_golden.py from the
reference code):
* mpkg_lapjv against mpk2/lapjv.c:366 lapjv, permutation for permutation
  (ties included), and against brute force like lab/lapjv_test.cc:99-154;
* mpkg_work_count against mpk2/work_count.c's summary for the MPI-2 rank
  buffers of every golden case that carries them."""
import itertools
import json
import os
import shutil
import tempfile

import numpy as np
import pytest

import mpk_gb300 as M
from conftest import golden_matrix, load_golden

HERE = os.path.dirname(os.path.abspath(__file__))


def _lapjv_cases():
    f = np.load(os.path.join(HERE, "golden", "lapjv.npz"))
    off_s = off_p = 0
    for n in f["sizes"]:
        n = int(n)
        yield f["sums"][off_s:off_s + n * n].reshape(n, n), f["perms"][off_p:off_p + n]
        off_s += n * n
        off_p += n


def test_lapjv_matches_reference_permutations():
    count = 0
    for sums, want in _lapjv_cases():
        assert np.array_equal(M.lapjv(sums), want), sums
        count += 1
    assert count == 320


def test_lapjv_is_optimal_against_brute_force():
    rng = np.random.default_rng(5)
    for _ in range(300):
        s = rng.integers(0, 10000, (5, 5))
        p = M.lapjv(s)
        assert sorted(p.tolist()) == list(range(5))
        best = max(sum(s[q[j], j] for j in range(5)) for q in itertools.permutations(range(5)))
        assert sum(s[p[j], j] for j in range(5)) == best


def _prepared_dir(name, parent):
    """A golden case's MPI-2 directory with rank buffers written by the
    library's own prep (byte-identical to the reference's, see test_prep).
    The values file is found from the directory name up to its first '_'
    (the reference's convention), so the caller works from `parent` and
    passes the bare name."""
    g = load_golden(name)
    a = golden_matrix(name)
    npart, nphase = int(g["npart"]), int(g["nphase"])
    d = os.path.join(parent, name)
    os.makedirs(d)
    a.write_metis(os.path.join(d, "loop.g0"), ne=(a.nnz + a.n) // 2)
    a.write_values(os.path.join(parent, name.split("_")[0] + ".loop.val"))
    for ph in range(max(nphase, 1)):
        np.savetxt(os.path.join(d, f"g{ph}.part.{npart}"), g["parts"][ph], fmt="%d")
    for ph in range(nphase):
        np.savetxt(os.path.join(d, f"l{ph}"), g["levels"][ph], fmt="%d")
    g["skirt"].tofile(os.path.join(d, f"s{nphase}"))
    M.lib().mpkg_bufs_prepare.argtypes = [M.C.c_char_p]
    assert M.lib().mpkg_bufs_prepare(name.encode()) == 0, M.lib().mpkg_last_error().decode()
    return name


WORK = json.load(open(os.path.join(HERE, "golden", "work_count.json")))


@pytest.mark.parametrize("name", sorted(WORK))
def test_work_count_matches_reference(name, monkeypatch):
    parent = tempfile.mkdtemp()
    monkeypatch.chdir(parent)
    try:
        d = _prepared_dir(name, parent)
        assert M.work_count(d) == WORK[name]
    finally:
        shutil.rmtree(parent)


def test_work_count_errors(monkeypatch):
    name = sorted(WORK)[0]
    parent = tempfile.mkdtemp()
    monkeypatch.chdir(parent)
    try:
        d = _prepared_dir(name, parent)
        with pytest.raises(M.MpkError) as e:
            M.work_count("nonsense")
        assert e.value.code == M.EFORMAT  # not a ghead_npart_nlevel_nphase name
        os.remove(os.path.join(d, "rank1.bufs"))
        with pytest.raises(M.MpkError) as e:
            M.work_count(d)
        assert e.value.code == M.EIO
    finally:
        shutil.rmtree(parent)
