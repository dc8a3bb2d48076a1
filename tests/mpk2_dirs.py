"""Helpers for the tests of the reference's mpk2 entry points: the
directory layout the reference's read_mpk reads, and ctypes signatures of
the legacy names the library exports (include/mpk2_compat.h)."""
import ctypes as C
import os

import numpy as np

import mpk_gb300 as M

EXEC_NAMES = ("exec_mpk", "exec_mpk_xs", "exec_mpk_xd", "exec_mpk_is", "exec_mpk_id")


def legacy_lib():
    L = M.lib()
    L.read_mpk.restype = C.c_void_p
    L.read_mpk.argtypes = [C.c_char_p]
    L.prep_mpk.restype = None
    L.prep_mpk.argtypes = [C.c_void_p, C.c_void_p]
    for f in EXEC_NAMES + ("exec_mpkt",):
        getattr(L, f).restype = None
        getattr(L, f).argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.vexec_mpk.restype = None
    L.vexec_mpk.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.read_crs.restype = C.c_void_p
    L.read_crs.argtypes = [C.c_void_p]
    for f in ("spmv_exec_seq",):
        getattr(L, f).restype = None
        getattr(L, f).argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.spmv_exec_par.restype = None
    L.spmv_exec_par.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    L.del_mpk.restype = None
    L.del_mpk.argtypes = [C.c_void_p]
    L.del_crs.restype = None
    L.del_crs.argtypes = [C.c_void_p]
    return L


def mpk_dir(parent, name, g, a):
    """The directory the reference's read_mpk reads (mpk2/mpkread.c): g0,
    gN.part.P, lN and the skirt file sNPHASE."""
    d = os.path.join(parent, name)
    os.makedirs(d)
    a.write_metis(os.path.join(d, "g0"), ne=(a.nnz + a.n) // 2)
    npart, nphase = int(g["npart"]), int(g["nphase"])
    for ph in range(max(nphase, 1)):
        np.savetxt(os.path.join(d, f"g{ph}.part.{npart}"), g["parts"][ph], fmt="%d")
    for ph in range(nphase):
        np.savetxt(os.path.join(d, f"l{ph}"), g["levels"][ph], fmt="%d")
    g["skirt"].tofile(os.path.join(d, f"s{nphase}"))
    return d


def read_crs_file(L, path):
    """read_crs on an opened METIS file; like the reference's
    (mpk2/lib.c:69-129) it closes the file itself."""
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    f = libc.fopen(path.encode(), b"r")
    assert f
    g0 = L.read_crs(f)
    assert g0
    return g0
