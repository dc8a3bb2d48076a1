"""PA1 prep on the GPU.  Tile metadata (mpkg_tile_prep): the host build
against a plain Python restatement of its definition (CPU), and the GPU
build byte for byte against the host build (GPU); task lists
(mpkg_pa1_tasks): the GPU build against the host build.  A tile of part p holds the vertices
within nlevel arcs of p under the reference's skirt distance
(mpk2/lib.c:584-615: row i is one arc from every column it reads), sorted
by (distance, vertex); the rows within nlevel-1 arcs are computed at level
1 and get a sliced-ELL structure of local slots."""
from collections import deque

import numpy as np
import pytest

import mpk_gb300 as M
from conftest import GOLDEN_CASES, golden_matrix, load_golden


def _restated(a, part, npart, nlevel):
    n = a.n
    readers = [[] for _ in range(n)]  # readers[u]: rows that read column u
    for i in range(n):
        for j in a.col[a.ptr[i]:a.ptr[i + 1]]:
            readers[j].append(i)
    slot_off, shell, slot_vert, slice_off, ell_off, ell_col, ell_width = [0], [], [], [0], [0], [], []
    for p in range(npart):
        dist = {int(v): 0 for v in np.flatnonzero(part == p)}
        q = deque(sorted(dist))
        while q:
            u = q.popleft()
            if dist[u] >= nlevel:
                continue
            for i in readers[u]:
                if i not in dist:
                    dist[i] = dist[u] + 1
                    q.append(i)
        ball = sorted(dist, key=lambda v: (dist[v], v))
        shell.append([sum(1 for v in ball if dist[v] <= d) for d in range(nlevel + 1)])
        slot_vert += ball
        slot_off.append(len(slot_vert))
        loc = {v: s for s, v in enumerate(ball)}
        nrows = shell[-1][nlevel - 1]
        for r0 in range(0, nrows, 32):
            rows = ball[r0:min(nrows, r0 + 32)]
            w = max(a.ptr[v + 1] - a.ptr[v] for v in rows)
            block = np.full((w, 32), 0xFFFF, dtype=np.uint16)
            for r, v in enumerate(rows):
                for t, c in enumerate(a.col[a.ptr[v]:a.ptr[v + 1]]):
                    block[t, r] = loc[int(c)]
            ell_col.append(block.ravel())
            ell_width.append(w)
            ell_off.append(ell_off[-1] + 32 * w)
        slice_off.append(len(ell_width))
    return {"slot_off": np.array(slot_off), "shell": np.array(shell), "slot_vert": np.array(slot_vert),
            "slice_off": np.array(slice_off), "ell_off": np.array(ell_off),
            "ell_col": np.concatenate(ell_col) if ell_col else np.zeros(0, np.uint16),
            "ell_width": np.array(ell_width)}


ARRAYS = ("slot_off", "shell", "slot_vert", "slice_off", "ell_off", "ell_col", "ell_width")


def _same(got, want):
    for k in ARRAYS:
        assert np.array_equal(np.asarray(got[k]), np.asarray(want[k])), k


@pytest.mark.parametrize("nx,ny,nz,npart,nlevel", [(12, 12, 1, 6, 3), (8, 8, 6, 10, 4), (30, 1, 1, 3, 5)])
def test_host_tile_prep_matches_restatement(nx, ny, nz, npart, nlevel):
    a0 = M.Csr.laplacian(nx, ny, nz)
    a = a0.pattern()
    part = M.partition_rcb(a0.coords, npart)
    got = M.tile_prep(a, part, npart, nlevel, on_gpu=False)
    assert not got["built_on_gpu"]
    want = _restated(a, part, npart, nlevel)
    _same(got, want)
    assert got["max_slots"] == int(np.diff(want["slot_off"]).max())
    assert got["total_rows"] == int(sum(want["shell"][:, nlevel - l].sum() for l in range(1, nlevel + 1)))


def test_host_tile_prep_errors():
    a0 = M.Csr.laplacian(10, 10)
    a = a0.pattern()
    part = M.partition_rcb(a0.coords, 4)
    with pytest.raises(M.MpkError) as e:
        M.tile_prep(a, np.where(part == 3, 2, part), 4, 3, on_gpu=False)
    assert e.value.code == M.EINVAL  # empty part
    with pytest.raises(M.MpkError) as e:
        M.tile_prep(a, part, 3, 3, on_gpu=False)
    assert e.value.code == M.ERANGE  # part id out of range


def _cases():
    out = []
    for name in GOLDEN_CASES:
        g = load_golden(name)
        if int(g["nphase"]) == 0:
            out.append((name, golden_matrix(name).pattern(), g["parts"][0], int(g["npart"]), int(g["nlevel"])))
    a0 = M.Csr.laplacian(64, 64, 64)
    out.append(("cube64_512_8", a0.pattern(), M.partition_rcb(a0.coords, 512), 512, 8))
    a1 = M.Csr.laplacian(200, 200)
    out.append(("grid200_64_6", a1.pattern(), M.partition_rcb(a1.coords, 64), 64, 6))
    return out


@pytest.mark.gpu
def test_gpu_tile_prep_identical_to_host(gpu):
    for name, a, part, npart, nlevel in _cases():
        want = M.tile_prep(a, part, npart, nlevel, on_gpu=False)
        got = M.tile_prep(a, part, npart, nlevel, on_gpu=True)
        assert got["built_on_gpu"], name
        _same(got, want)
        assert (got["max_slots"], got["total_rows"]) == (want["max_slots"], want["total_rows"]), name


@pytest.mark.gpu
def test_gpu_tile_prep_falls_back_beyond_capacity(gpu):
    """Balls above 32768 vertices go to the host build, with equal results."""
    a0 = M.Csr.laplacian(64, 64, 16)
    a = a0.pattern()
    part = M.partition_rcb(a0.coords, 2)  # halves of 32768 vertices: balls beyond capacity
    got = M.tile_prep(a, part, 2, 3, on_gpu=True)
    assert not got["built_on_gpu"]
    _same(got, M.tile_prep(a, part, 2, 3, on_gpu=False))


def _from_rows(rows):
    ptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])])
    return M.Csr(ptr, np.concatenate([np.asarray(sorted(r), dtype=np.int32) for r in rows]))


@pytest.mark.gpu
def test_gpu_tile_prep_errors_as_host(gpu):
    """Every error comes from the host build, with its code and message."""
    a0 = M.Csr.laplacian(20, 20)
    part = M.partition_rcb(a0.coords, 4)
    rows = [set(a0.col[a0.ptr[i]:a0.ptr[i + 1]].tolist()) for i in range(a0.n)]
    wide = [set(r) for r in rows]
    for c in range(300):  # vertex 5 joined to 300 others, both ways: a row of 301 entries
        wide[5].add(c)
        wide[c].add(5)
    one = [set(r) for r in rows]
    one[9] = set()  # row 9 (beside another quadrant) reads nothing, but its neighbours read it
    cases = [(a0.pattern(), np.where(part == 3, 2, part), M.EINVAL),
             (_from_rows(wide), part, M.ERANGE),
             (_from_rows(one), part, M.ESTRUCT)]
    for b, pt, code in cases:
        with pytest.raises(M.MpkError) as e1:
            M.tile_prep(b, pt, 4, 3, on_gpu=False)
        with pytest.raises(M.MpkError) as e2:
            M.tile_prep(b, pt, 4, 3, on_gpu=True)
        assert e1.value.code == e2.value.code == code
        assert str(e1.value) == str(e2.value)


def test_host_pa1_tasks_equal_mpkg_tasks():
    a0 = M.Csr.laplacian(16, 16, 4)
    a = a0.pattern()
    part = M.partition_rcb(a0.coords, 12)
    off, idx, on = M.pa1_tasks(a, part, 12, 5, on_gpu=False)
    off2, idx2 = M.tasks(a, 12, 5, part, check=False)
    assert not on
    assert np.array_equal(off, off2) and np.array_equal(idx, idx2)


@pytest.mark.gpu
def test_gpu_pa1_tasks_identical_to_host(gpu):
    cases = _cases()
    a0 = M.Csr.laplacian(24, 24)
    part = M.partition_rcb(a0.coords, 6)
    cases.append(("empty_part", a0.pattern(), np.where(part == 5, 4, part), 6, 4))  # part 5 has no vertices
    cases.append(("one_level", a0.pattern(), part, 6, 1))
    for name, a, pt, npart, nlevel in cases:
        off, idx, on = M.pa1_tasks(a, pt, npart, nlevel, on_gpu=False)
        goff, gidx, gon = M.pa1_tasks(a, pt, npart, nlevel, on_gpu=True)
        assert gon and not on, name
        assert np.array_equal(goff, off) and np.array_equal(gidx, idx), name


@pytest.mark.gpu
def test_gpu_pa1_tasks_fall_back_beyond_capacity(gpu):
    a0 = M.Csr.laplacian(64, 64, 16)
    part = M.partition_rcb(a0.coords, 2)
    off, idx, on = M.pa1_tasks(a0.pattern(), part, 2, 3, on_gpu=True)
    assert not on
    off2, idx2, _ = M.pa1_tasks(a0.pattern(), part, 2, 3, on_gpu=False)
    assert np.array_equal(off, off2) and np.array_equal(idx, idx2)


# ---- DMPK phase levels and METIS weights on the GPU ------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if int(c.split("_")[3].rstrip("m")) > 0])
def test_gpu_phase_levels_and_weights_equal_reference(name, gpu):
    """comp_level / update_level and level2wcrs built on the GPU give the
    reference tools' levels and weight graphs on every multi-phase golden
    case (RCB, BFS and METIS partitions)."""
    g = load_golden(name)
    a = golden_matrix(name)
    npart = int(g["npart"])
    prev = None
    for ph in range(int(g["nphase"])):
        lev = M.levels(a, g["parts"][ph], npart, prev, on_gpu=True)
        assert np.array_equal(lev, g["levels"][ph]), f"phase {ph} levels"
        wv, we = M.level_weights(a, lev, on_gpu=True)
        wv_h, we_h = M.level_weights(a, lev)
        assert np.array_equal(we, g["weights"][ph]) and np.array_equal(wv, wv_h)
        prev = lev


@pytest.mark.gpu
def test_gpu_phase_levels_identical_to_host_large(gpu):
    """A 96^3 Laplacian in 512 parts, three phases with different
    partitions: the GPU levels and weights equal the host build's bytes."""
    a = M.Csr.laplacian(96, 96, 96).pattern()
    parts = [M.partition_rcb(a.coords, 512), M.partition_bfs(a, 512),
             M.partition_rcb(a.coords[:, ::-1].copy(), 512)]
    prev_g = prev_h = None
    for p in parts:
        lg = M.levels(a, p, 512, prev_g, on_gpu=True)
        lh = M.levels(a, p, 512, prev_h)
        assert np.array_equal(lg, lh)
        for x, y in zip(M.level_weights(a, lg, on_gpu=True), M.level_weights(a, lh)):
            assert np.array_equal(x, y)
        prev_g, prev_h = lg, lh
