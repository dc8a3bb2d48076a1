"""METIS partitions (the reference's partitioner, mpk2/driver.c:63-66 and
pdmpk/pdmpk_buffers.cc:183-202) through the product's prep, end to end.

The product links the METIS library bundled with the CUDA toolkit.  The
fixtures come from the reference's own tools: m9p24_8_4_2m runs the mpk2
driver's flow (partition, comp level, comp weight, partition the weighted
graph, ..., skirt, read_mpk + prep_mpk) with METIS at every phase, and
pdmpk_metis.json holds the reference pdmpk prep compiled against METIS on
the reference's CTest shapes (tests/golden/make_golden.py metis)."""
import hashlib
import json
import os
import tempfile

import numpy as np
import pytest

import mpk_gb300 as M
from conftest import GOLDEN, golden_matrix, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not M.have_metis(), reason="library built without METIS")


@pytest.mark.parametrize("kind,size,npart", [("m5p", 40, 8), ("m9p", 33, 6), ("cube", 12, 16)])
def test_partition_equals_gpmetis_call(kind, size, npart):
    """mpkg_partition_metis gives what gpmetis -ufactor=100 gives on the
    same graph (the oracle's METIS call on the pattern without diagonal)."""
    if not O.metis_available():
        pytest.skip("oracle METIS wrapper not built")
    a = M.Csr.stencil(kind, size)
    part, cut = M.partition_metis(a, npart, ufactor=100)
    assert np.array_equal(part, O.metis_kway(a.ptr, a.col, npart, 100))
    assert part.min() == 0 and part.max() == npart - 1 and cut > 0
    assert np.bincount(part).max() <= 1.10 * a.n / npart + 1  # ufactor 100: 10 % imbalance


def test_driver_flow_on_metis_parts_byte_identical():
    """The mpk2 driver's prep with METIS at every phase, run entirely by the
    product (partition, levels, weights, re-partition on the weighted
    graph, skirt, task lists): every intermediate equals the reference's."""
    name = "m9p24_8_4_2m"
    g = load_golden(name)
    a = golden_matrix(name)
    npart, nlevel, nphase = int(g["npart"]), int(g["nlevel"]), int(g["nphase"])
    parts, levels = [M.partition_metis(a, npart, ufactor=100)[0]], []
    for ph in range(nphase):
        if ph > 0:  # the weighted graph file carries vertex weight 1 (mpk2/lib.c:490)
            _, we = M.level_weights(a, levels[-1])
            ones = np.ones(a.n, dtype=np.int32)
            parts.append(M.partition_metis(a, npart, ufactor=100, vwgt=ones, adjwgt=we)[0])
        assert np.array_equal(parts[ph], g["parts"][ph]), f"phase {ph} partition"
        levels.append(M.levels(a, parts[ph], npart, levels[-1] if ph else None))
        assert np.array_equal(levels[-1], g["levels"][ph])
        assert np.array_equal(M.level_weights(a, levels[-1])[1], g["weights"][ph])
    with tempfile.TemporaryDirectory() as d:
        sp = os.path.join(d, "s")
        M.write_skirt(sp, a, parts[0], npart, nlevel, levels[-1])
        assert open(sp, "rb").read() == g["skirt"].tobytes()
    off, idx = M.tasks(a, npart, nlevel, np.array(parts), np.array(levels))
    assert np.array_equal(off, g["off"]) and np.array_equal(idx, g["idx"])


def _metis_ctest():
    with open(os.path.join(GOLDEN, "pdmpk_metis.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("key", sorted(_metis_ctest()))
def test_pdmpk_prep_with_metis_byte_identical(key, tmp_path):
    """pdmpk's prep partitioning with METIS (MPKG_PD_PART_METIS) writes the
    files of the reference prep compiled against METIS, byte for byte."""
    m, P, L = key.split("_")
    P, L = int(P), int(L)
    path = os.path.join(str(tmp_path), m + ".mtx")
    M.Csr.stencil(m[:3], int(m[3:])).write_mtx(path, pattern=True)
    a = M.Csr.read_mtx(path)
    bp = [os.path.join(str(tmp_path), f"r{r}.buf.bin") for r in range(P)]
    rp = [os.path.join(str(tmp_path), f"r{r}.results.bin") for r in range(P)]
    M.pdmpk_prep(a, P, L, bp, rp, mirror=5, weight=3, partitioner=M.PD_PART_METIS)
    got = [[hashlib.sha256(open(p, "rb").read()).hexdigest() for p in (b, r)] for b, r in zip(bp, rp)]
    assert got == _metis_ctest()[key]


def test_metis_fixture_differs_from_stand_in():
    """The METIS fixtures are not the block-shift stand-in's files."""
    with open(os.path.join(GOLDEN, "pdmpk_ctest.json")) as f:
        stand_in = json.load(f)
    metis = _metis_ctest()
    assert sum(metis[k] != stand_in[k] for k in metis) >= len(metis) // 2


def test_pa1_tasks_oracle_bounded_search_matches_reference():
    """The oracle's bounded-search PA1 task lists (used by the benchmark's
    CPU arms at sizes where the reference prep's dense skirt does not fit)
    equal the reference prep's lists on every PA1 golden case."""
    for name in ("m5p10_4_4_0", "cfg1_4_4_0", "cube6_8_3_0"):
        g = load_golden(name)
        a = golden_matrix(name)
        off, idx = O.pa1_tasks(a.ptr, a.col, g["parts"][0], int(g["npart"]), int(g["nlevel"]))
        assert np.array_equal(off, g["off"]) and np.array_equal(idx, g["idx"]), name
