"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries, both built by oracle/Makefile:
  * ``_build/liboracle.so`` -- the C restatement in mpk_oracle.c;
  * ``_ref/libmpk2ref.so`` (+ tool binaries) -- the reference mpk2 C code
    compiled from its own sources, present only where those sources were.
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module.  The product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORACLE = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
LIBREF = os.path.join(REF_DIR, "libmpk2ref.so")

MODE_SEPARATE, MODE_FMA = 0, 1


def build(quiet=True):
    """make liboracle (always) and the reference (when its sources exist)."""
    out = subprocess.run(["make", "-s", "-C", HERE, "stage", "liboracle", "libmetis", "ref"],
                         stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout)
    if not quiet:
        print(out.stdout)


_o = None


def lib():
    global _o
    if _o is None:
        if not os.path.exists(LIBORACLE):
            build()
        _o = C.CDLL(LIBORACLE)
        P, I, L = C.c_void_p, C.c_int, C.c_long
        _o.orc_graph_count.restype = L
        _o.orc_graph_count.argtypes = [C.c_char_p, C.POINTER(I), C.POINTER(L)]
        _o.orc_graph_read.argtypes = [C.c_char_p, I, L, P, P]
        _o.orc_read_values.argtypes = [C.c_char_p, L, P]
        _o.orc_minplus.restype = L
        _o.orc_minplus.argtypes = [I, P, P, P, P, I, P, I]
        _o.orc_comp_level.argtypes = [I, P, P, P, I, P]
        _o.orc_update_level.argtypes = [I, P, P, P, I, P, P]
        _o.orc_level2weights.argtypes = [I, P, P, P, P, P]
        _o.orc_skirt_dist.argtypes = [I, P, P, P, I, P]
        _o.orc_write_skirt.argtypes = [C.c_char_p, I, P, P, P, I, P, I]
        _o.orc_read_skirt.argtypes = [C.c_char_p, I, I, I, P]
        _o.orc_prep_tasks.restype = L
        _o.orc_prep_tasks.argtypes = [I, P, P, I, I, I, P, P, P, P, P, L]
        _o.orc_exec_tasks.argtypes = [I, P, P, P, L, P, P, P, I]
        _o.orc_exec_tasks_t.argtypes = [I, I, P, P, L, P, P, P, I]
        _o.orc_spmv_chain.argtypes = [I, P, P, P, I, P, I]
        _o.orc_spmv_chain_par.argtypes = [I, P, P, P, I, P, I, I]
        _o.orc_exec_tasks_par.argtypes = [I, P, P, P, I, I, P, P, P, I, I]
    return _o


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def read_graph(path):
    o = lib()
    n, ne = C.c_int(), C.c_long()
    cnt = o.orc_graph_count(path.encode(), C.byref(n), C.byref(ne))
    if cnt < 0:
        raise ValueError(f"oracle: bad graph {path} ({cnt})")
    ptr = np.zeros(n.value + 1, dtype=np.int32)
    col = np.zeros(max(cnt, 1), dtype=np.int32)
    rc = o.orc_graph_read(path.encode(), n.value, cnt, _p(ptr), _p(col))
    if rc:
        raise ValueError(f"oracle: bad graph {path} ({rc})")
    return ptr, col[:cnt]


def read_values(path, nnz):
    val = np.zeros(nnz, dtype=np.float64)
    if lib().orc_read_values(path.encode(), nnz, _p(val)):
        raise ValueError("oracle: bad values file")
    return val


def comp_level(ptr, col, part, npart):
    n = len(ptr) - 1
    out = np.zeros(n, dtype=np.int32)
    lib().orc_comp_level(n, _p(ptr), _p(col), _p(np.ascontiguousarray(part, dtype=np.int32)), npart, _p(out))
    return out


def update_level(ptr, col, part, npart, level_org):
    n = len(ptr) - 1
    out = np.zeros(n, dtype=np.int32)
    lib().orc_update_level(n, _p(ptr), _p(col), _p(np.ascontiguousarray(part, dtype=np.int32)), npart,
                           _p(np.ascontiguousarray(level_org, dtype=np.int32)), _p(out))
    return out


def level_weights(ptr, col, level):
    n = len(ptr) - 1
    wv = np.zeros(n, dtype=np.int32)
    we = np.zeros(int(ptr[-1]), dtype=np.int32)
    lib().orc_level2weights(n, _p(ptr), _p(col), _p(np.ascontiguousarray(level, dtype=np.int32)), _p(wv), _p(we))
    return wv, we


def skirt_dist(ptr, col, part, p):
    n = len(ptr) - 1
    out = np.zeros(n, dtype=np.int32)
    lib().orc_skirt_dist(n, _p(ptr), _p(col), _p(np.ascontiguousarray(part, dtype=np.int32)), p, _p(out))
    return out


def write_skirt(path, ptr, col, part, npart, level, lev=None):
    n = len(ptr) - 1
    lv = None if lev is None else np.ascontiguousarray(lev, dtype=np.int32)
    rc = lib().orc_write_skirt(path.encode(), n, _p(ptr), _p(col), _p(np.ascontiguousarray(part, dtype=np.int32)),
                               npart, _p(lv), level)
    if rc:
        raise ValueError("oracle: write_skirt failed")


def read_skirt(path, n, npart, level):
    sl = np.zeros(npart * n, dtype=np.int32)
    rc = lib().orc_read_skirt(path.encode(), n, npart, level, _p(sl))
    if rc:
        raise ValueError(f"oracle: read_skirt failed ({rc})")
    return sl.reshape(npart, n)


def prep_tasks(ptr, col, npart, nlevel, nphase, parts, levels, sl):
    """-> (off, idx) or raises on the reference's structure errors."""
    n = len(ptr) - 1
    parts = np.ascontiguousarray(parts, dtype=np.int32)
    levels = None if levels is None else np.ascontiguousarray(levels, dtype=np.int32)
    sl = np.ascontiguousarray(sl, dtype=np.int32)
    off = np.zeros((nphase + 1) * npart + 1, dtype=np.int64)
    cap = n * nlevel + int(np.sum(np.where(sl >= 0, nlevel - sl + 1, 0)))
    idx = np.zeros(max(cap, 1), dtype=np.int64)
    cnt = lib().orc_prep_tasks(n, _p(ptr), _p(col), npart, nlevel, nphase, _p(parts), _p(levels), _p(sl),
                               _p(off), _p(idx), cap)
    if cnt < 0:
        raise ValueError(f"oracle: prep_tasks failed ({cnt})")
    return off, idx[:cnt]


def exec_tasks(ptr, col, val, off, idx, vv, mode=MODE_FMA):
    n = len(ptr) - 1
    lib().orc_exec_tasks(n, _p(ptr), _p(col), _p(val), len(off) - 1, _p(off), _p(idx), _p(vv), mode)
    return vv


def exec_tasks_par(ptr, col, val, nphase, npart, off, idx, vv, mode=MODE_FMA, nth=1):
    n = len(ptr) - 1
    lib().orc_exec_tasks_par(n, _p(ptr), _p(col), _p(val), nphase, npart, _p(off), _p(idx), _p(vv), mode, nth)
    return vv


def spmv_chain(ptr, col, val, nlevel, vv, mode=MODE_FMA):
    n = len(ptr) - 1
    lib().orc_spmv_chain(n, _p(ptr), _p(col), _p(val), nlevel, _p(vv), mode)
    return vv


def spmv_chain_par(ptr, col, val, nlevel, vv, mode=MODE_FMA, nth=1):
    n = len(ptr) - 1
    lib().orc_spmv_chain_par(n, _p(ptr), _p(col), _p(val), nlevel, _p(vv), mode, nth)
    return vv


def mpk(ptr, col, val, x, nlevel, mode=MODE_FMA):
    """[x, Ax, ..., A^k x] level-major (the serial chain)."""
    n = len(ptr) - 1
    vv = np.zeros((nlevel + 1) * n, dtype=np.float64)
    vv[:n] = x
    return spmv_chain(np.ascontiguousarray(ptr, dtype=np.int32), np.ascontiguousarray(col, dtype=np.int32),
                      None if val is None else np.ascontiguousarray(val, dtype=np.float64), nlevel, vv, mode)


def pa1_tasks(ptr, col, part, npart, nlevel):
    """PA1 task lists (orc_pa1_tasks: comp_skirt + prep_mpk's skirt loop
    with a bounded search): (off[npart+1], idx) in the reference layout."""
    o = lib()
    o.orc_pa1_tasks.restype = C.c_long
    o.orc_pa1_tasks.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                C.c_void_p, C.c_long]
    p = np.ascontiguousarray(ptr, dtype=np.int32)
    c = np.ascontiguousarray(col, dtype=np.int32)
    pt = np.ascontiguousarray(part, dtype=np.int32)
    off = np.zeros(npart + 1, dtype=np.int64)
    cnt = o.orc_pa1_tasks(len(p) - 1, _p(p), _p(c), _p(pt), npart, nlevel, _p(off), None, 0)
    if cnt < 0:
        raise ValueError(f"oracle: orc_pa1_tasks failed ({cnt})")
    idx = np.zeros(cnt, dtype=np.int64)
    cnt2 = o.orc_pa1_tasks(len(p) - 1, _p(p), _p(c), _p(pt), npart, nlevel, _p(off), _p(idx), cnt)
    if cnt2 != cnt:
        raise ValueError("oracle: orc_pa1_tasks count changed")
    return off, idx


def laplacian(nx, ny, nz, diag, offd):
    """The 3-D 7-point Laplacian of the workloads (orc_gen_laplacian)."""
    o = lib()
    o.orc_gen_laplacian.restype = C.c_long
    o.orc_gen_laplacian.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
    n = nx * ny * nz
    ptr = np.zeros(n + 1, dtype=np.int32)
    cap = 7 * n
    col = np.zeros(cap, dtype=np.int32)
    val = np.zeros(cap)
    e = o.orc_gen_laplacian(nx, ny, nz, diag, offd, _p(ptr), _p(col), _p(val))
    return ptr, col[:e].copy(), val[:e].copy()


def uniform(seed, n):
    """uniform[-1,1] doubles from the workloads' splitmix64 stream."""
    o = lib()
    o.orc_uniform.argtypes = [C.c_ulonglong, C.c_long, C.c_void_p]
    out = np.zeros(n)
    o.orc_uniform(seed, n, _p(out))
    return out


LIBMETIS = os.path.join(HERE, "_build", "libmetis_oracle.so")


def metis_available():
    return os.path.exists(LIBMETIS)


def metis_kway(ptr, col, npart, ufactor=0, vwgt=None, adjwgt=None):
    """k-way partition by the METIS library bundled with CUDA (the
    reference's partitioner), as `gpmetis -ufactor=<ufactor>` computes it:
    the graph without its diagonal, optional vertex and edge weights."""
    m = C.CDLL(LIBMETIS)
    m.orc_metis_kway.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                 C.c_void_p, C.c_void_p]
    p = np.ascontiguousarray(ptr, dtype=np.int32)
    c = np.ascontiguousarray(col, dtype=np.int32)
    vw = None if vwgt is None else np.ascontiguousarray(vwgt, dtype=np.int32)
    ew = None if adjwgt is None else np.ascontiguousarray(adjwgt, dtype=np.int32)
    part = np.zeros(len(p) - 1, dtype=np.int32)
    cut = C.c_long()
    if m.orc_metis_kway(len(p) - 1, _p(p), _p(c), None if vw is None else _p(vw), None if ew is None else _p(ew),
                        npart, ufactor, _p(part), C.byref(cut)) != 0:
        raise RuntimeError("METIS_PartGraphKway failed")
    return part


# ---------------------------------------------------------------- reference
def ref_available():
    return os.path.exists(LIBREF)


def ref_tool(name):
    return os.path.join(REF_DIR, name)


class RefTask(C.Structure):
    _fields_ = [("n", C.c_int), ("idx", C.POINTER(C.c_long)), ("th", C.c_int), ("t0", C.c_double),
                ("t1", C.c_double)]


class RefMpk(C.Structure):
    _fields_ = [("n", C.c_int), ("npart", C.c_int), ("nlevel", C.c_int), ("nphase", C.c_int),
                ("g0", C.c_void_p), ("plist", C.c_void_p), ("llist", C.c_void_p), ("sg", C.c_void_p),
                ("tlist", C.POINTER(RefTask)), ("idxsrc", C.POINTER(C.c_long)), ("idxallocsize", C.c_long)]


_r = None


def ref():
    """The reference mpk2 library compiled from its own sources."""
    global _r
    if _r is None:
        if not ref_available():
            raise FileNotFoundError("reference library not built (needs the reference sources)")
        _r = C.CDLL(LIBREF)
        _r.read_mpk.restype = C.POINTER(RefMpk)
        _r.read_mpk.argtypes = [C.c_char_p]
        _r.prep_mpk.argtypes = [C.POINTER(RefMpk), C.c_void_p]
        for f in ("exec_mpk", "exec_mpk_xs", "exec_mpk_xd", "exec_mpk_is", "exec_mpk_id", "exec_mpkt"):
            getattr(_r, f).argtypes = [C.POINTER(RefMpk), C.c_void_p, C.c_int]
        _r.vexec_mpk.argtypes = [C.POINTER(RefMpk), C.c_void_p, C.c_void_p]
        _r.spmv_exec_seq.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        _r.spmv_exec_par.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    return _r


def ref_tasks(mg):
    """Task lists of a reference mpk_t as (off, idx)."""
    m = mg.contents
    nl = (m.nphase + 1) * m.npart
    off = np.zeros(nl + 1, dtype=np.int64)
    parts = []
    for t in range(nl):
        tk = m.tlist[t]
        off[t + 1] = off[t] + tk.n
        if tk.n > 0:
            parts.append(np.ctypeslib.as_array(tk.idx, shape=(tk.n,)).copy())
    idx = np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)
    return off, idx


class RefCrs(C.Structure):
    _fields_ = [("n", C.c_int), ("ptr", C.POINTER(C.c_int)), ("col", C.POINTER(C.c_int))]


class RefTaskLists:
    """An in-memory reference mpk_t for PA1 task lists (no files, no dense
    skirt): enough for the reference exec_mpk* functions, which read only
    n, npart, nlevel, nphase, g0 and tlist (mpk2/mpkexec.c:10-130)."""

    def __init__(self, ptr, col, npart, nlevel, nphase, off, idx):
        self.ptr = np.ascontiguousarray(ptr, dtype=np.int32)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.idx = np.ascontiguousarray(idx, dtype=np.int64)
        self.crs = RefCrs(len(self.ptr) - 1, self.ptr.ctypes.data_as(C.POINTER(C.c_int)),
                          self.col.ctypes.data_as(C.POINTER(C.c_int)))
        nl = (nphase + 1) * npart
        self.tasks = (RefTask * nl)()
        base = self.idx.ctypes.data
        for t in range(nl):
            self.tasks[t].n = int(off[t + 1] - off[t])
            self.tasks[t].idx = C.cast(base + 8 * int(off[t]), C.POINTER(C.c_long))
        self.mpk = RefMpk(len(self.ptr) - 1, npart, nlevel, nphase, C.addressof(self.crs), None, None, None,
                          self.tasks, None, 0)

    def exec_xd(self, vv, nth):
        ref().exec_mpk_xd(C.byref(self.mpk), vv.ctypes.data_as(C.c_void_p), nth)


# ---------------------------------------------------------------- MPI-2 buffers
def bufs_exec(paths, x, nlevel, mode=MODE_FMA):
    """All ranks of the MPI-2 valued exec, emulated in one process
    (orc_bufs_exec): paths = rank0.bufs ... rank{P-1}.bufs."""
    o = lib()
    o.orc_bufs_read.restype = C.c_void_p
    o.orc_bufs_read.argtypes = [C.c_char_p]
    o.orc_bufs_exec.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    handles = []
    for p in paths:
        h = o.orc_bufs_read(p.encode())
        if not h:
            raise ValueError(f"oracle: cannot read {p}")
        handles.append(h)
    arr = (C.c_void_p * len(handles))(*handles)
    n = len(x)
    vv = np.zeros((nlevel + 1) * n)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    if o.orc_bufs_exec(len(handles), arr, _p(xx), _p(vv), mode) != 0:
        raise ValueError("oracle: buffers without values")
    return vv


# ---------------------------------------------------------------- pdmpk buffers
def pd_exec(buf_paths, res_paths, x, mode=MODE_FMA):
    """All ranks of pdmpk's exec emulated in one process (orc_pd_exec):
    returns A^k x."""
    o = lib()
    o.orc_pd_read.restype = C.c_void_p
    o.orc_pd_read.argtypes = [C.c_char_p, C.c_char_p]
    o.orc_pd_exec.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    hs = []
    for bp, rp in zip(buf_paths, res_paths):
        h = o.orc_pd_read(bp.encode(), rp.encode())
        if not h:
            raise ValueError(f"oracle: cannot read {bp}")
        hs.append(h)
    arr = (C.c_void_p * len(hs))(*hs)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(len(xx))
    if o.orc_pd_exec(len(hs), arr, _p(xx), _p(out), mode) != 0:
        raise ValueError("oracle: inconsistent pdmpk buffers")
    return out


def spmm_f32(ptr, col, val, X, nlevel):
    """Batched FP32 block-vector chain, fmaf per entry in CSR order
    (orc_spmm_f32); X: (n, nrhs) float32.  Returns (nlevel+1, n, nrhs)."""
    o = lib()
    o.orc_spmm_f32.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    n, nrhs = X.shape
    p = np.ascontiguousarray(ptr, dtype=np.int32)
    c = np.ascontiguousarray(col, dtype=np.int32)
    v = np.ascontiguousarray(val, dtype=np.float32)
    vb = np.zeros((nlevel + 1, n, nrhs), dtype=np.float32)
    vb[0] = X
    o.orc_spmm_f32(n, _p(p), _p(c), _p(v), nrhs, nlevel, _p(vb))
    return vb
