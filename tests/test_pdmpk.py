"""pdmpk buffers on the host: the product's prep against the reference
prep's files (byte for byte), the oracle's execution of those files against
the FP64 chain, and validation of malformed buffers."""
import os

import numpy as np
import pytest

import mpk_gb300 as M
import pdmpk_cases as PC
from oracle import oracle as O

G = PC.load()
CASES = PC.cases(G)


def test_fixture_covers_every_mirror_and_weight_method():
    assert {c[3] for c in CASES} == set(range(6))
    assert {c[4] for c in CASES} == set(range(4))


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-np%d-nl%d-mm%d-wm%d" % c)
def test_prep_byte_identical(case, tmp_path):
    m, P, L, mm, wm = case
    a = M.Csr.read_mtx(PC.write_mtx(G, m, str(tmp_path)))
    bp = [str(tmp_path / f"r{r}.buf.bin") for r in range(P)]
    rp = [str(tmp_path / f"r{r}.results.bin") for r in range(P)]
    M.pdmpk_prep(a, P, L, bp, rp, mirror=mm, weight=wm)
    for r in range(P):
        key = f"{m}__{P}_{L}_{mm}_{wm}__r{r}"
        assert open(bp[r], "rb").read() == G[key + "__buf"].tobytes(), f"buf.bin of rank {r}"
        assert open(rp[r], "rb").read() == G[key + "__res"].tobytes(), f"results.bin of rank {r}"


@pytest.mark.parametrize("stuck", [str(s) for s in G["stuck"]])
def test_prep_reports_stuck_mirror_method(stuck, tmp_path):
    """Where the reference prep exits with "Couldn't finish", the product
    returns MPKG_ESTRUCT and writes nothing."""
    m, P, L, mm, wm = stuck.rsplit("_", 4)
    P, L, mm, wm = int(P), int(L), int(mm), int(wm)
    a = M.Csr.read_mtx(PC.write_mtx(G, m, str(tmp_path)))
    bp = [str(tmp_path / f"r{r}.buf.bin") for r in range(P)]
    rp = [str(tmp_path / f"r{r}.results.bin") for r in range(P)]
    with pytest.raises(M.MpkError) as e:
        M.pdmpk_prep(a, P, L, bp, rp, mirror=mm, weight=wm)
    assert e.value.code == M.ESTRUCT
    assert not os.path.exists(bp[0])


def _chain(a, x, L):
    return O.mpk(a.ptr, a.col, a.val, x, L, O.MODE_SEPARATE)[L * a.n:]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-np%d-nl%d-mm%d-wm%d" % c)
def test_oracle_exec_matches_chain(case, tmp_path):
    """The pdmpk check (apps/check.cc:25,83: cos^2 of the angle to the
    serial chain within 1e-9), tightened to 1e-13 relative error."""
    m, P, L, mm, wm = case
    a = M.Csr.read_mtx(PC.write_mtx(G, m, str(tmp_path)))
    bp, rp = PC.write_case(G, case, str(tmp_path))
    x = M.uniform(11, a.n)
    y = O.pd_exec(bp, rp, x, O.MODE_SEPARATE)
    want = _chain(a, x, L)
    cos2 = (y @ want) ** 2 / ((y @ y) * (want @ want))
    assert abs(1.0 - cos2) < 1e-9
    assert np.linalg.norm(y - want) / np.linalg.norm(want) < 1e-13


def test_info_reads_reference_files(tmp_path):
    case = CASES[0]
    m, P, L, mm, wm = case
    bp, rp = PC.write_case(G, case, str(tmp_path))
    info = M.pdmpk_info(bp, rp)
    a = M.Csr.read_mtx(PC.write_mtx(G, m, str(tmp_path)))
    assert info["n"] == a.n and info["nlevel"] == L and info["nbatch"] >= L
    assert info["rows"] >= a.n * L  # every (vertex, level) at least once


def test_malformed_buffers_are_rejected(tmp_path):
    case = CASES[0]
    bp, rp = PC.write_case(G, case, str(tmp_path))
    data = open(bp[1], "rb").read()
    with open(bp[1], "wb") as f:  # truncated file
        f.write(data[: len(data) // 2])
    with pytest.raises(M.MpkError) as e:
        M.pdmpk_info(bp, rp)
    assert e.value.code == M.EFORMAT
    with open(bp[1], "wb") as f:  # one mcol entry out of range
        arr = bytearray(data)
        o, c, _ = PC.fields(data)["mcol"]
        assert c > 0
        arr[o:o + 4] = (10 ** 8).to_bytes(4, "little", signed=True)
        f.write(bytes(arr))
    with pytest.raises(M.MpkError):
        M.pdmpk_info(bp, rp)
    with pytest.raises(M.MpkError) as e:  # missing rank file
        M.pdmpk_info(bp[:1] + [str(tmp_path / "nope")] + bp[2:], rp)
    assert e.value.code == M.EIO


CTEST = PC.ctest()


@pytest.mark.parametrize("key", sorted(CTEST))
def test_prep_ctest_shapes_byte_identical(key, tmp_path):
    """The reference's CTest shapes (tests/CMakeLists.txt:3-42: m5p/m9p
    meshes of size 10 and 100, 4 and 8 parts, 10 and 20 levels, mirror 5,
    weight 3, plus m5p4): the product's prep writes the reference prep's
    files, byte for byte (compared by sha256)."""
    import hashlib
    a, bp, rp = PC.ctest_prep(key, str(tmp_path))
    got = [[hashlib.sha256(open(p, "rb").read()).hexdigest() for p in (b, r)] for b, r in zip(bp, rp)]
    assert got == CTEST[key]
