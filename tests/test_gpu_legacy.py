"""The reference's mpk2 entry points as a relinked reference program calls
them (mpk2/mpktest.c:53-150, mpk2/mpkrun.c:49-74): read_mpk on a
ghead_npart_nlevel_nphase directory, prep_mpk, then exec_mpk{,_xs,_xd,_is,
_id}, vexec_mpk, exec_mpkt and spmv_exec_seq/par on the GPU.  The golden
fixtures were made by the reference's own read_mpk / prep_mpk /
exec_mpk_xd / vexec_mpk / spmv_exec_seq on the same directories
(tests/golden/make_golden.py); with MPK_GB300_ARITH=separate (the
reference's non-contracted build) every result equals them bit for bit,
and the default FMA arithmetic equals the oracle's FMA chain bit for bit."""
import hashlib
import os
import tempfile

import numpy as np
import pytest

import mpk_gb300 as M
from conftest import GOLDEN_CASES, golden_matrix, load_golden
from mpk2_dirs import EXEC_NAMES, legacy_lib as _lib, mpk_dir as _mpk_dir, read_crs_file as _read_crs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _same(g, key, vv):
    if key in g:
        assert vv.tobytes() == g[key].tobytes(), key
    else:
        assert hashlib.sha256(vv.tobytes()).digest() == g[key + "_sha256"].tobytes(), key


def _start(x, n, nlevel):
    vv = np.zeros((nlevel + 1) * n)
    vv[:n] = x
    return vv


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_legacy_entry_points_give_reference_bits(name, monkeypatch, gpu):
    monkeypatch.setenv("MPK_GB300_ARITH", "separate")
    g = load_golden(name)
    a = golden_matrix(name)
    n, nlevel = int(g["n"]), int(g["nlevel"])
    L = _lib()
    with tempfile.TemporaryDirectory() as parent:
        d = _mpk_dir(parent, name, g, a)
        mg = L.read_mpk(d.encode())
        assert mg, M.lib().mpkg_last_error().decode()
        vv = _start(g["x"], n, nlevel)
        L.prep_mpk(mg, vv.ctypes.data)
        for f in EXEC_NAMES:
            vv = _start(g["x"], n, nlevel)
            getattr(L, f)(mg, vv.ctypes.data, 4)
            _same(g, "vv_deg", vv)
        vv = _start(g["x"], n, nlevel)
        L.vexec_mpk(mg, vv.ctypes.data, a.val.ctypes.data)
        _same(g, "vv_val", vv)
        # exec_mpkt: the transposed layout vv[i * (k + 1) + l]
        vt = np.zeros((n, nlevel + 1))
        vt[:, 0] = g["x"]
        L.exec_mpkt(mg, vt.ctypes.data, 4)
        _same(g, "vv_deg", np.ascontiguousarray(vt.T).reshape(-1))
        g0 = _read_crs(L, os.path.join(d, "g0"))
        for par in (False, True):
            vv = _start(g["x"], n, nlevel)
            if par:
                L.spmv_exec_par(g0, vv.ctypes.data, nlevel, 4)
            else:
                L.spmv_exec_seq(g0, vv.ctypes.data, nlevel)
            _same(g, "vv_spmv", vv)
        L.del_crs(g0)
        L.del_mpk(mg)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_legacy_entry_points_fma_equal_oracle_chain(name, monkeypatch, gpu):
    """Default (FMA) arithmetic: every row of every level is one FMA chain
    in CSR order, whatever the schedule, so the task executor equals the
    oracle's serial chain bit for bit."""
    monkeypatch.delenv("MPK_GB300_ARITH", raising=False)
    g = load_golden(name)
    a = golden_matrix(name)
    n, nlevel = int(g["n"]), int(g["nlevel"])
    want = O.mpk(a.ptr, a.col, None, g["x"], nlevel, O.MODE_FMA)
    want_val = O.mpk(a.ptr, a.col, a.val, g["x"], nlevel, O.MODE_FMA)
    L = _lib()
    with tempfile.TemporaryDirectory() as parent:
        d = _mpk_dir(parent, name, g, a)
        mg = L.read_mpk(d.encode())
        assert mg
        vv = _start(g["x"], n, nlevel)
        L.prep_mpk(mg, vv.ctypes.data)
        vv = _start(g["x"], n, nlevel)
        L.exec_mpk_xd(mg, vv.ctypes.data, 4)
        assert vv.tobytes() == want.tobytes()
        vv = _start(g["x"], n, nlevel)
        L.vexec_mpk(mg, vv.ctypes.data, a.val.ctypes.data)
        assert vv.tobytes() == want_val.tobytes()
        L.del_mpk(mg)
