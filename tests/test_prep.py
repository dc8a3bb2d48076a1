"""Host prep of the product (levels, weights, skirts, task lists,
partitioners) against the reference's own outputs (golden fixtures) and the
oracle on random graphs."""
import os
import tempfile

import numpy as np
import pytest

import mpk_gb300 as M
from conftest import GOLDEN_CASES, golden_matrix, load_golden
from oracle import oracle as O


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_prep_bit_identical_to_reference(name):
    g = load_golden(name)
    a = golden_matrix(name)
    n, npart, nlevel, nphase = int(g["n"]), int(g["npart"]), int(g["nlevel"]), int(g["nphase"])
    parts = g["parts"]
    lev = None
    levels = []
    for ph in range(nphase):
        lev = M.levels(a, parts[ph], npart, None if ph == 0 else levels[-1])
        assert np.array_equal(lev, g["levels"][ph])
        _, we = M.level_weights(a, lev)
        assert np.array_equal(we, g["weights"][ph])
        levels.append(lev)
    with tempfile.TemporaryDirectory() as d:
        sp = os.path.join(d, "s")
        M.write_skirt(sp, a, parts[0], npart, nlevel, lev)
        assert open(sp, "rb").read() == g["skirt"].tobytes()
    off, idx = M.tasks(a, npart, nlevel, parts[: max(nphase, 1)], np.array(levels) if nphase else None)
    assert np.array_equal(off, g["off"]) and np.array_equal(idx, g["idx"])


def _random_graph(rng, n, extra):
    edges = set((i, i + 1) for i in range(n - 1))
    for _ in range(extra):
        i, j = rng.integers(0, n, 2)
        if i != j:
            edges.add((int(min(i, j)), int(max(i, j))))
    rows = [[i] for i in range(n)]  # with diagonal, as the loop graphs
    for i, j in edges:
        rows[i].append(j)
        rows[j].append(i)
    rows = [sorted(r) for r in rows]
    ptr = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    return M.Csr(ptr, np.concatenate(rows).astype(np.int32))


@pytest.mark.parametrize("seed", range(6))
def test_prep_matches_oracle_random(seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(50, 300))
    a = _random_graph(rng, n, int(rng.integers(n // 2, 2 * n)))
    npart, nlevel = int(rng.integers(2, 7)), int(rng.integers(2, 7))
    nphase = int(rng.integers(0, 3))
    parts = [M.partition_bfs(a, npart)]
    for _ in range(1, max(nphase, 1)):
        p = rng.integers(0, npart, n).astype(np.int32)
        p[:npart] = np.arange(npart)
        parts.append(p)
    levels = []
    for ph in range(nphase):
        if ph == 0:
            lo = O.comp_level(a.ptr, a.col, parts[0], npart)
        else:
            lo = O.update_level(a.ptr, a.col, parts[ph], npart, levels[-1])
        assert np.array_equal(M.levels(a, parts[ph], npart, None if ph == 0 else levels[-1]), lo)
        levels.append(lo)
    with tempfile.TemporaryDirectory() as d:
        s1, s2 = os.path.join(d, "s1"), os.path.join(d, "s2")
        M.write_skirt(s1, a, parts[0], npart, nlevel, levels[-1] if nphase else None)
        O.write_skirt(s2, a.ptr, a.col, parts[0], npart, nlevel, levels[-1] if nphase else None)
        assert open(s1).read() == open(s2).read()
        sl = O.read_skirt(s2, n, npart, nlevel)
    try:
        ro = O.prep_tasks(a.ptr, a.col, npart, nlevel, nphase, np.array(parts), np.array(levels) if nphase else None, sl)
    except ValueError:
        ro = None
    if ro is None:  # the reference's dependency check rejects this input: so must the product
        with pytest.raises(M.MpkError) as e:
            M.tasks(a, npart, nlevel, np.array(parts), np.array(levels) if nphase else None)
        assert e.value.code == M.ESTRUCT
    else:
        off, idx = M.tasks(a, npart, nlevel, np.array(parts), np.array(levels) if nphase else None)
        assert np.array_equal(off, ro[0]) and np.array_equal(idx, ro[1])


def test_partitioners_cover_and_balance():
    a = M.Csr.laplacian(32, 16, 8)
    p = M.partition_rcb(a.coords, 16)
    counts = np.bincount(p, minlength=16)
    assert counts.min() == counts.max() == a.n // 16
    q = M.partition_bfs(a, 10)
    counts = np.bincount(q, minlength=10)
    assert counts.sum() == a.n and counts.min() > 0 and counts.max() - counts.min() <= 1


def test_rcb_gives_boxes_for_config2_shape():
    a = M.Csr.laplacian(16, 16, 16)
    p = M.partition_rcb(a.coords, 16)
    for q in range(16):
        c = a.coords[p == q]
        ext = c.max(0) - c.min(0) + 1
        assert np.prod(ext) == len(c)  # every part is a box


@pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here")
@pytest.mark.parametrize("kind,size", [("m5p", 10), ("m7p", 9), ("m9p", 8), ("t5p", 7), ("cube", 5)])
def test_reference_stencils_match_gen2(kind, size):
    """The generator reproduces the reference gen2 tool's graph and values."""
    import subprocess
    a = M.Csr.stencil(kind, size)
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([O.ref_tool("gen2"), kind, str(size), os.path.join(d, "h")], check=True)
        ptr, col = O.read_graph(os.path.join(d, "h.loop.g0"))
        val = O.read_values(os.path.join(d, "h.loop.val"), int(ptr[-1]))
    assert np.array_equal(ptr, a.ptr) and np.array_equal(col, a.col) and np.array_equal(val, a.val)


def test_read_metis_errors():
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "g")
        open(p, "w").write("3 2 011\n1 2\n")
        with pytest.raises(M.MpkError) as e:
            M.Csr.read_metis(p)
        assert e.value.code == M.EFORMAT
        open(p, "w").write("3 2\n2\n1 3\n9\n")
        with pytest.raises(M.MpkError) as e:
            M.Csr.read_metis(p)
        assert e.value.code == M.ERANGE
        open(p, "w").write("3 1\n2 3\n1 3\n1 2\n")
        with pytest.raises(M.MpkError) as e:  # more than 2*ne columns
            M.Csr.read_metis(p)
        assert e.value.code == M.EFORMAT
        open(p, "w").write("3 2\n2\n1 3\n")
        with pytest.raises(M.MpkError) as e:  # missing row
            M.Csr.read_metis(p)
        assert e.value.code == M.EFORMAT
        with pytest.raises(M.MpkError) as e:
            M.Csr.read_metis(os.path.join(d, "missing"))
        assert e.value.code == M.EIO


def test_tasks_reject_bad_partition():
    a = M.Csr.laplacian(6, 6)
    with pytest.raises(M.MpkError) as e:
        M.tasks(a, 2, 2, np.full(a.n, 5, dtype=np.int32))
    assert e.value.code == M.ERANGE


def test_empty_part_pa1_tasks():
    """A part id with no vertices gets empty task lists, as in the reference."""
    a = M.Csr.laplacian(8, 8)
    part = M.partition_rcb(a.coords, 4)
    part[part == 3] = 2  # part 3 empty
    off, idx = M.tasks(a, 4, 3, part)
    assert off[4] - off[3] == 0
    with tempfile.TemporaryDirectory() as d:
        s = os.path.join(d, "s")
        O.write_skirt(s, a.ptr, a.col, part, 4, 3)
        sl = O.read_skirt(s, a.n, 4, 3)
    ro = O.prep_tasks(a.ptr, a.col, 4, 3, 0, part, None, sl)
    assert np.array_equal(off, ro[0]) and np.array_equal(idx, ro[1])


def _case_dir(name, g, a, parent):
    """The directory layout the reference's MPI-2 prep reads."""
    d = os.path.join(parent, name)
    os.makedirs(d)
    npart, nphase = int(g["npart"]), int(g["nphase"])
    a.write_metis(os.path.join(d, "loop.g0"), ne=(a.nnz + a.n) // 2)
    a.write_values(os.path.join(parent, name.split("_")[0] + ".loop.val"))
    for ph in range(max(nphase, 1)):
        np.savetxt(os.path.join(d, f"g{ph}.part.{npart}"), g["parts"][ph], fmt="%d")
    for ph in range(nphase):
        np.savetxt(os.path.join(d, f"l{ph}"), g["levels"][ph], fmt="%d")
    g["skirt"].tofile(os.path.join(d, f"s{nphase}"))
    return d


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if c != "cfg1_4_4_0"])
def test_mpi2_rank_buffers_byte_identical(name, monkeypatch):
    """mpkg_bufs_prepare writes the same rank<r>.bufs files as the
    reference's mpi2_mpkwrtbufs (fill_buffers + alloc_fill_mval), including
    the partition relabelling of phases > 0."""
    g = load_golden(name)
    a = golden_matrix(name)
    with tempfile.TemporaryDirectory() as parent:
        _case_dir(name, g, a, parent)
        monkeypatch.chdir(parent)
        M.lib().mpkg_bufs_prepare.argtypes = [M.C.c_char_p]
        rc = M.lib().mpkg_bufs_prepare(name.encode())
        assert rc == 0, M.lib().mpkg_last_error().decode()
        for r in range(int(g["npart"])):
            mine = np.fromfile(os.path.join(parent, name, f"rank{r}.bufs"), dtype=np.uint8)
            assert mine.tobytes() == g[f"bufs{r}"].tobytes(), f"rank {r}"
