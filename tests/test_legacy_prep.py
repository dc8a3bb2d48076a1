"""The reference's mpk2 prep entry points through the library's legacy
names, as a relinked reference program calls them (mpk2/mpktest.c:53-90):
read_mpk on a ghead_npart_nlevel_nphase directory and prep_mpk give the
task lists the reference's own read_mpk + prep_mpk gave on the same files
(golden fixtures), and read_mpk reports bad directories through the last
error instead of exiting.  No GPU needed."""
import ctypes as C
import tempfile

import numpy as np
import pytest

import mpk_gb300 as M
from conftest import GOLDEN_CASES, golden_matrix, load_golden
from mpk2_dirs import legacy_lib, mpk_dir
from oracle import oracle as O


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_read_prep_give_reference_task_lists(name):
    g = load_golden(name)
    a = golden_matrix(name)
    L = legacy_lib()
    with tempfile.TemporaryDirectory() as parent:
        mg = L.read_mpk(mpk_dir(parent, name, g, a).encode())
        assert mg, M.lib().mpkg_last_error().decode()
        vv = np.zeros((int(g["nlevel"]) + 1) * int(g["n"]))
        L.prep_mpk(mg, vv.ctypes.data)
        off, idx = O.ref_tasks(C.cast(mg, C.POINTER(O.RefMpk)))
        assert np.array_equal(off, g["off"]) and np.array_equal(idx, g["idx"])
        L.del_mpk(mg)


def test_read_mpk_errors():
    """NULL and the last error where the reference prints and exits
    (mpk2/mpkread.c)."""
    L = legacy_lib()
    with tempfile.TemporaryDirectory() as parent:
        assert not L.read_mpk((parent + "/nounderscores").encode())
        assert "ghead_npart_nlevel_nphase" in M.lib().mpkg_last_error().decode()
        assert not L.read_mpk((parent + "/g_4_4_0").encode())  # no g0 inside
        assert "g0" in M.lib().mpkg_last_error().decode()
