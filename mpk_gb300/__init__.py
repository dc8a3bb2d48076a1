"""mpk_gb300 -- GB300 matrix powers kernel (MPK).

Python host interface over the C ABI of ``libmpk_gb300.so`` (declared in
``include/mpk_gb300.h`` and ``include/mpk2_compat.h``).  The library is the
product: this module only marshals numpy arrays and torch device pointers.
It raises when the library is missing; there is no CPU fallback.

Level-major layout as in the reference: ``vv[l*n + i]`` holds (A^l x)_i,
``vv[0:n]`` is x (mpk2/mpktest.c:66-75).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmpk_gb300.so")

OK, EINVAL, EIO, EFORMAT, ESTRUCT, ECUDA, ETIMEOUT, ENOMEM, ERANGE = 0, -1, -2, -3, -4, -5, -6, -7, -8
ARITH_FMA, ARITH_SEPARATE, ARITH_DF64, ARITH_FIXED = 0, 1, 2, 3
BATCH_DEFAULT, BATCH_TUNE, BATCH_STAGED, BATCH_STAGED2, BATCH_STAGED4 = 0, 1, 2, 3, 4
EXEC_TASKS, EXEC_TILES, EXEC_PIPE, EXEC_SPMV, EXEC_BUFS, EXEC_MIXED, EXEC_PDMPK, EXEC_WAVE, EXEC_BATCH = \
    0, 1, 2, 3, 4, 5, 6, 7, 8
PD_PART_BLOCKSHIFT, PD_PART_BFS, PD_PART_METIS = 0, 1, 2
VALUE_F32, VALUE_BF16 = 0, 1

_ERRNAMES = {EINVAL: "EINVAL", EIO: "EIO", EFORMAT: "EFORMAT", ESTRUCT: "ESTRUCT", ECUDA: "ECUDA",
             ETIMEOUT: "ETIMEOUT", ENOMEM: "ENOMEM", ERANGE: "ERANGE"}


class MpkError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib():
    """The loaded C library (built in-tree by ``mpk_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


class TilesT(C.Structure):
    _fields_ = [("npart", C.c_int), ("nlevel", C.c_int), ("max_slots", C.c_int), ("built_on_gpu", C.c_int),
                ("total_rows", C.c_long), ("nslots", C.c_long), ("nslices", C.c_long), ("nell", C.c_long),
                ("slot_off", C.c_void_p), ("shell", C.c_void_p), ("slot_vert", C.c_void_p),
                ("slice_off", C.c_void_p), ("ell_off", C.c_void_p), ("ell_col", C.c_void_p),
                ("ell_width", C.c_void_p)]


class BatchInfo(C.Structure):
    _fields_ = [("nmat", C.c_int), ("nrhs", C.c_int), ("nlevel", C.c_int), ("rows", C.c_long), ("nnz", C.c_long),
                ("lanes_per_row", C.c_int), ("vector_width", C.c_int), ("group_bytes", C.c_long),
                ("ngroup", C.c_int), ("grid", C.c_int), ("graph", C.c_int), ("candidates", C.c_int),
                ("tune_ms", C.c_double), ("device_bytes", C.c_long), ("staged", C.c_int), ("threads", C.c_int),
                ("window_bytes", C.c_long)]


class CgInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("mpk_steps", C.c_int), ("converged", C.c_int), ("breakdowns", C.c_int),
                ("relres", C.c_double), ("basis_cond", C.c_double), ("ms", C.c_double),
                ("loop_ms", C.c_double), ("loop_launches", C.c_int)]


class PlanInfo(C.Structure):
    _fields_ = [("n", C.c_int), ("nlevel", C.c_int), ("nphase", C.c_int), ("npart", C.c_int),
                ("exec", C.c_int), ("arith", C.c_int), ("valued", C.c_int),
                ("nnz", C.c_long), ("rows_computed", C.c_long), ("device_bytes", C.c_long),
                ("launches", C.c_int), ("tiles_in_smem", C.c_int), ("max_tile_slots", C.c_int),
                ("pipe_chunk", C.c_int), ("pipe_reach", C.c_int), ("pipe_grid", C.c_int),
                ("tile_regs", C.c_int), ("tune_candidates", C.c_int), ("tune_ms", C.c_double)]


def _declare(L):
    P, I, Lg, D, V = C.c_void_p, C.c_int, C.c_long, C.c_double, C.c_void_p
    pp = C.POINTER(C.c_void_p)
    sig = {
        "mpkg_plan_tasks": (I, [I, P, P, P, I, I, I, P, P, I, pp]),
        "mpkg_plan_pa1": (I, [I, P, P, P, P, I, I, I, I, pp]),
        "mpkg_plan_pipe": (I, [I, P, P, P, I, I, I, pp]),
        "mpkg_plan_spmv": (I, [I, P, P, P, I, I, pp]),
        "mpkg_plan_wave": (I, [I, P, P, P, I, I, pp]),
        "mpkg_plan_wave_ctas": (I, [I, P, P, P, I, I, I, pp]),
        "mpkg_plan_batch": (I, [I, P, P, P, P, I, I, I, pp]),
        "mpkg_cg": (I, [I, P, P, P, P, P, D, I, C.POINTER(CgInfo)]),
        "mpkg_sstep_cg": (I, [I, P, P, P, P, P, I, P, D, D, I, C.POINTER(CgInfo)]),
        "mpkg_lanczos": (I, [I, P, P, P, I, C.c_uint64, P, P, P]),
        "mpkg_tridiag_eigs": (None, [I, P, P, P]),
        "mpkg_leja_order": (None, [I, P]),
        "mpkg_features": (I, [I, P, P, P, P, C.POINTER(D), C.POINTER(D)]),
        "mpkg_mlp_create": (I, [I, I, I, C.c_uint64, pp]),
        "mpkg_mlp_destroy": (None, [P]),
        "mpkg_mlp_nparams": (I, [P]),
        "mpkg_mlp_get_params": (I, [P, P]),
        "mpkg_mlp_set_params": (I, [P, P]),
        "mpkg_mlp_forward": (I, [P, I, P, P]),
        "mpkg_mlp_gradient": (I, [P, I, P, P, P, P]),
        "mpkg_mlp_train": (I, [P, I, P, P, I, I, C.c_float, C.c_uint64, P]),
        "mpkg_batch_info": (I, [P, C.POINTER(BatchInfo)]),
        "mpkg_exec_batch_device": (I, [P, P, P]),
        "mpkg_exec_batch_host": (I, [P, P]),
        "mpkg_plan_info": (I, [P, C.POINTER(PlanInfo)]),
        "mpkg_plan_bufs": (I, [C.c_char_p, I, I, pp]),
        "mpkg_plan_pdmpk": (I, [I, P, P, I, pp]),
        "mpkg_pdmpk_prep": (I, [I, P, P, P, I, I, I, I, I, P, P]),
        "mpkg_pdmpk_info": (I, [I, P, P, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(Lg)]),
        "mpkg_exec_host": (I, [P, P]),
        "mpkg_exec_device": (I, [P, P, P]),
        "mpkg_sync": (I, [P, P]),
        "mpkg_plan_destroy": (None, [P]),
        "mpkg_debug_pipe_stall": (I, [P, I]),
        "mpkg_spmv_chain_device": (I, [I, P, P, P, I, P, I, P]),
        "mpkg_read_metis": (I, [C.c_char_p, C.POINTER(I), C.POINTER(Lg), pp, pp]),
        "mpkg_read_mtx": (I, [C.c_char_p, C.POINTER(I), C.POINTER(Lg), pp, pp, pp]),
        "mpkg_read_values": (I, [C.c_char_p, Lg, pp]),
        "mpkg_free": (None, [P]),
        "mpkg_levels": (I, [I, P, P, P, I, P, P]),
        "mpkg_level_weights": (I, [I, P, P, P, P, P]),
        "mpkg_levels_gpu": (I, [I, P, P, P, I, P, P]),
        "mpkg_level_weights_gpu": (I, [I, P, P, P, P, P]),
        "mpkg_skirt_write": (I, [C.c_char_p, I, P, P, P, I, P, I]),
        "mpkg_tasks": (I, [I, P, P, I, I, I, P, P, I, P, pp, C.POINTER(Lg)]),
        "mpkg_tile_prep": (I, [I, P, P, P, I, I, I, C.POINTER(TilesT)]),
        "mpkg_tiles_free": (None, [C.POINTER(TilesT)]),
        "mpkg_pa1_tasks": (I, [I, P, P, P, I, I, I, P, pp, C.POINTER(Lg), C.POINTER(I)]),
        "mpkg_work_count": (I, [C.c_char_p, C.POINTER(Lg), C.POINTER(Lg), C.POINTER(Lg), C.POINTER(Lg),
                                C.POINTER(Lg)]),
        "mpkg_lapjv": (I, [P, I, P]),
        "mpkg_sstep_gram": (I, [I]),
        "mpkg_sstep_loop": (I, [I]),
        "mpkg_sstep_basis": (I, [I]),
        "mpkg_sstep_debug_stall": (I, [I]),
        "mpkg_partition_rcb": (I, [I, P, I, I, P]),
        "mpkg_partition_bfs": (I, [I, P, P, I, P]),
        "mpkg_have_metis": (I, []),
        "mpkg_partition_metis": (I, [I, P, P, P, P, I, I, P, P]),
        "mpkg_gen_stencil": (I, [C.c_char_p, I, C.POINTER(I), C.POINTER(Lg), pp, pp, pp]),
        "mpkg_gen_laplacian": (I, [I, I, I, D, D, C.POINTER(I), C.POINTER(Lg), pp, pp, pp, pp]),
        "mpkg_uniform": (None, [C.c_uint64, Lg, P]),
        "mpkg_gen_diffusion": (I, [I, I, I, D, D, D, D, D, C.c_uint64, C.POINTER(I), C.POINTER(Lg), pp, pp, pp]),
        "mpkg_gen_banded": (I, [Lg, I, I, I, C.c_uint64, C.POINTER(I), C.POINTER(Lg), pp, pp, pp]),
        "mpkg_plan_mixed": (I, [I, P, P, P, I, I, pp]),
        "mpkg_plan_mixed_tiles": (I, [I, P, P, P, P, I, I, I, pp]),
        "mpkg_plan_mixed_tiles_tuned": (I, [I, P, P, P, P, I, I, I, pp]),
        "mpkg_mixed_scale": (I, [P, C.POINTER(I), C.POINTER(Lg)]),
        "mpkg_exec_mixed_device": (I, [P, P, P]),
        "mpkg_bufs_prepare": (I, [C.c_char_p]),
        "mpkg_last_error": (C.c_char_p, []),
        "mpkg_version": (I, []),
        "mpkg_fp64_fma_rate": (I, [C.POINTER(D)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _check(rc):
    if rc != OK:
        raise MpkError(rc, lib().mpkg_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _take(p, count, dtype):
    """Copy a malloc'd C array into numpy and free it."""
    if count == 0:
        lib().mpkg_free(p)
        return np.zeros(0, dtype=dtype)
    ct = {np.int32: C.c_int, np.int64: C.c_long, np.float64: C.c_double}[dtype]
    arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(count,)).copy()
    lib().mpkg_free(p)
    return arr


# ---------------------------------------------------------------- matrices
class Csr:
    """CSR matrix with int32 indices; ``val is None`` is the 1/deg operator
    (mpk2/lib.h:10-14 crs0_t; pdmpk/csr.h:11-69 Csr)."""

    def __init__(self, ptr, col, val=None, coords=None):
        self.ptr = _i32(ptr)
        self.col = _i32(col)
        self.val = _f64(val)
        self.n = len(self.ptr) - 1
        self.nnz = int(self.ptr[-1])
        self.coords = coords

    def pattern(self):
        """Same graph, 1/deg operator (values dropped)."""
        return Csr(self.ptr, self.col, None, self.coords)

    @staticmethod
    def read_metis(path, values_path=None):
        L = lib()
        n, nnz = C.c_int(), C.c_long()
        pp, cp = C.c_void_p(), C.c_void_p()
        _check(L.mpkg_read_metis(path.encode(), C.byref(n), C.byref(nnz), C.byref(pp), C.byref(cp)))
        ptr = _take(pp, n.value + 1, np.int32)
        col = _take(cp, nnz.value, np.int32)
        val = None
        if values_path:
            vp = C.c_void_p()
            _check(L.mpkg_read_values(values_path.encode(), nnz.value, C.byref(vp)))
            val = _take(vp, nnz.value, np.float64)
        return Csr(ptr, col, val)

    @staticmethod
    def read_mtx(path):
        """Matrix Market file as pdmpk's Csr reads it (pattern => 1/deg)."""
        L = lib()
        n, nnz = C.c_int(), C.c_long()
        pp, cp, vp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(L.mpkg_read_mtx(os.fsencode(path), C.byref(n), C.byref(nnz), C.byref(pp), C.byref(cp),
                               C.byref(vp)))
        return Csr(_take(pp, n.value + 1, np.int32), _take(cp, nnz.value, np.int32),
                   _take(vp, nnz.value, np.float64))

    def write_mtx(self, path, pattern=False):
        """Matrix Market coordinate file, general, rows in CSR order
        (values printed with 17 significant digits)."""
        with open(path, "w") as f:
            f.write("%%%%MatrixMarket matrix coordinate %s general\n" % ("pattern" if pattern else "real"))
            f.write(f"{self.n} {self.n} {self.nnz}\n")
            rows = np.repeat(np.arange(self.n), np.diff(self.ptr)) + 1
            if pattern:
                for i, j in zip(rows, self.col + 1):
                    f.write(f"{i} {j}\n")
            else:
                for i, j, v in zip(rows, self.col + 1, self.val):
                    f.write("%d %d %.17g\n" % (i, j, v))

    @staticmethod
    def stencil(kind, size):
        """The reference gen2 stencils (mpk2/gen2.c:59-267)."""
        L = lib()
        n, nnz = C.c_int(), C.c_long()
        pp, cp, vp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(L.mpkg_gen_stencil(kind.encode(), size, C.byref(n), C.byref(nnz), C.byref(pp),
                                  C.byref(cp), C.byref(vp)))
        return Csr(_take(pp, n.value + 1, np.int32), _take(cp, nnz.value, np.int32),
                   _take(vp, nnz.value, np.float64))

    @staticmethod
    def laplacian(nx, ny, nz=1, diag=None, off=-1.0):
        """(2d+1)-point Laplacian on an nx*ny*nz grid, ascending columns."""
        if diag is None:
            diag = 4.0 if nz == 1 else 6.0
        L = lib()
        n, nnz = C.c_int(), C.c_long()
        pp, cp, vp, xp = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(L.mpkg_gen_laplacian(nx, ny, nz, diag, off, C.byref(n), C.byref(nnz), C.byref(pp),
                                    C.byref(cp), C.byref(vp), C.byref(xp)))
        coords = _take(xp, 3 * n.value, np.int32).reshape(-1, 3)
        return Csr(_take(pp, n.value + 1, np.int32), _take(cp, nnz.value, np.int32),
                   _take(vp, nnz.value, np.float64), coords)

    @staticmethod
    def diffusion(nx, ny, nz=1, sigma=1.0, wx=1.0, wy=1.0, wdiag=1.0, dominance=0.01, seed=0):
        """Variable-coefficient diffusion, log-normal(0, sigma) edge
        coefficients: 9-point on nx*ny (nz == 1) or 7-point on nx*ny*nz."""
        L = lib()
        n, nnz = C.c_int(), C.c_long()
        pp, cp, vp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(L.mpkg_gen_diffusion(nx, ny, nz, sigma, wx, wy, wdiag, dominance, seed, C.byref(n), C.byref(nnz),
                                    C.byref(pp), C.byref(cp), C.byref(vp)))
        return Csr(_take(pp, n.value + 1, np.int32), _take(cp, nnz.value, np.int32),
                   _take(vp, nnz.value, np.float64))

    @staticmethod
    def banded(n, bandwidth=64, nnz_min=5, nnz_max=30, seed=0):
        """Random banded, diagonally dominant operator (N(0,1) values)."""
        L = lib()
        nn, nnz = C.c_int(), C.c_long()
        pp, cp, vp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(L.mpkg_gen_banded(n, bandwidth, nnz_min, nnz_max, seed, C.byref(nn), C.byref(nnz), C.byref(pp),
                                 C.byref(cp), C.byref(vp)))
        return Csr(_take(pp, nn.value + 1, np.int32), _take(cp, nnz.value, np.int32),
                   _take(vp, nnz.value, np.float64))

    def write_metis(self, path, ne=None):
        with open(path, "w") as f:
            f.write(f"{self.n} {self.nnz // 2 if ne is None else ne}\n")
            for i in range(self.n):
                cols = self.col[self.ptr[i]:self.ptr[i + 1]] + 1
                f.write("".join(f"{c} " for c in cols) + "\n")

    def write_values(self, path):
        with open(path, "w") as f:
            f.write("".join(f"{v:.17g} " for v in self.val))


def _cstrs(paths):
    return C.cast((C.c_char_p * len(paths))(*[os.fsencode(x) for x in paths]), C.c_void_p)


def pdmpk_prep(a: Csr, npart, nlevel, buf_paths, results_paths, mirror=0, weight=0,
               partitioner=PD_PART_BLOCKSHIFT):
    """pdmpk prep of every rank (CommCompPatterns); writes buf_paths[r] and
    results_paths[r] in the reference's format."""
    if a.val is None:
        raise MpkError(EINVAL, "pdmpk prep needs matrix values")
    assert len(buf_paths) == npart and len(results_paths) == npart
    _check(lib().mpkg_pdmpk_prep(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), npart, nlevel, mirror, weight,
                                 partitioner, _cstrs(buf_paths), _cstrs(results_paths)))


def pdmpk_info(buf_paths, results_paths):
    """Loads and validates pdmpk buffers on the host: n, nlevel, batches,
    computed rows."""
    n, nl, nb, rows = C.c_int(), C.c_int(), C.c_int(), C.c_long()
    _check(lib().mpkg_pdmpk_info(len(buf_paths), _cstrs(buf_paths), _cstrs(results_paths), C.byref(n),
                                 C.byref(nl), C.byref(nb), C.byref(rows)))
    return dict(n=n.value, nlevel=nl.value, nbatch=nb.value, rows=rows.value)


def batch_workload(count=256, nmin=1000, nmax=200000, seed=0):
    """The batching workload: `count` matrices with n log-uniform in
    [nmin, nmax]; even indices random 2-D/3-D stencils (5-point or 9-point
    diffusion in 2-D, 7-point Laplacian or diffusion in 3-D), odd indices
    random banded (bandwidth 64, 5-30 entries per row, N(0,1) values,
    diagonally dominant).  Seeded per matrix."""
    rng = np.random.default_rng(seed)
    mats = []
    for m in range(count):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        s = int(rng.integers(1 << 62))
        if m % 2 == 1:
            mats.append(Csr.banded(n, 64, 5, 30, seed=s))
            continue
        kind = int(rng.integers(4))
        if kind < 2:  # 2-D
            nx = max(2, int(round(np.sqrt(n))))
            ny = max(2, n // nx)
            mats.append(Csr.laplacian(nx, ny, 1, diag=4.0, off=-1.0) if kind == 0
                        else Csr.diffusion(nx, ny, 1, sigma=0.5, seed=s))
        else:  # 3-D
            nx = max(2, int(round(n ** (1.0 / 3.0))))
            ny = nx
            nz = max(2, n // (nx * ny))
            mats.append(Csr.laplacian(nx, ny, nz, diag=6.0, off=-1.0) if kind == 2
                        else Csr.diffusion(nx, ny, nz, sigma=0.5, seed=s))
    return mats


def uniform(seed, n):
    """Uniform[-1, 1) doubles from the library's splitmix64 stream."""
    out = np.empty(n, dtype=np.float64)
    lib().mpkg_uniform(seed, n, _ptr(out))
    return out


# ---------------------------------------------------------------- host prep
def partition_rcb(coords, npart):
    coords = _i32(coords)
    n, dim = coords.shape
    part = np.empty(n, dtype=np.int32)
    _check(lib().mpkg_partition_rcb(n, _ptr(coords), dim, npart, _ptr(part)))
    return part


def fp64_fma_rate():
    """Peak FP64 FMA rate of the current GPU (FMAs per second)."""
    r = C.c_double()
    _check(lib().mpkg_fp64_fma_rate(C.byref(r)))
    return r.value


def have_metis():
    """True when the library links the CUDA toolkit's METIS."""
    return bool(lib().mpkg_have_metis())


def partition_metis(a: Csr, npart, ufactor=0, vwgt=None, adjwgt=None):
    """METIS k-way partition as `gpmetis -ufactor=<ufactor>` computes it
    (mpk2/driver.c:63-66): the graph without self loops, default options
    otherwise.  Returns (part, edgecut)."""
    part = np.empty(a.n, dtype=np.int32)
    vw, ew = _i32(vwgt), _i32(adjwgt)
    cut = C.c_long()
    _check(lib().mpkg_partition_metis(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(vw), _ptr(ew), npart, ufactor, _ptr(part),
                                      C.byref(cut)))
    return part, cut.value


def partition_bfs(a: Csr, npart):
    part = np.empty(a.n, dtype=np.int32)
    _check(lib().mpkg_partition_bfs(a.n, _ptr(a.ptr), _ptr(a.col), npart, _ptr(part)))
    return part


def levels(a: Csr, part, npart, level_org=None, on_gpu=False):
    """comp_level / update_level (mpk2/lib.c:330-412), on the host or the
    current GPU (same bytes)."""
    part = _i32(part)
    lo = _i32(level_org)
    out = np.empty(a.n, dtype=np.int32)
    fn = lib().mpkg_levels_gpu if on_gpu else lib().mpkg_levels
    _check(fn(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(part), npart, _ptr(lo), _ptr(out)))
    return out


def level_weights(a: Csr, level, on_gpu=False):
    """level2wcrs (mpk2/lib.c:504-537) -> (wv, we), on the host or the
    current GPU (same bytes)."""
    level = _i32(level)
    wv = np.empty(a.n, dtype=np.int32)
    we = np.empty(a.nnz, dtype=np.int32)
    fn = lib().mpkg_level_weights_gpu if on_gpu else lib().mpkg_level_weights
    _check(fn(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(level), _ptr(wv), _ptr(we)))
    return wv, we


def write_skirt(path, a: Csr, part, npart, nlevel, lev=None):
    """The `skirt` tool's output file (mpk2/skirt.c, mpk2/lib.c:584-654)."""
    part = _i32(part)
    lev = _i32(lev)
    _check(lib().mpkg_skirt_write(path.encode(), a.n, _ptr(a.ptr), _ptr(a.col), _ptr(part), npart,
                                  _ptr(lev), nlevel))


def tasks(a: Csr, npart, nlevel, parts, levels_=None, check=True):
    """prep_mpk task lists (mpk2/mpkprep.c:7-258) -> (off, idx)."""
    parts = np.atleast_2d(_i32(parts))
    nphase = 0 if levels_ is None else len(levels_)
    lv = None if levels_ is None else np.ascontiguousarray(np.atleast_2d(levels_), dtype=np.int32)
    off = np.empty((nphase + 1) * npart + 1, dtype=np.int64)
    ip, cnt = C.c_void_p(), C.c_long()
    _check(lib().mpkg_tasks(a.n, _ptr(a.ptr), _ptr(a.col), npart, nlevel, nphase, _ptr(parts),
                            _ptr(lv), 1 if check else 0, _ptr(off), C.byref(ip), C.byref(cnt)))
    return off, _take(ip, cnt.value, np.int64)


def tile_prep(a: Csr, part, npart, nlevel, on_gpu=True):
    """PA1 tile metadata (the balls of every part sorted by (distance,
    vertex) and the tiles' sliced-ELL local structure), built on the GPU
    (on_gpu) or on the host; a dict of numpy arrays plus 'built_on_gpu'."""
    part = _i32(part)
    t = TilesT()
    _check(lib().mpkg_tile_prep(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(part), npart, nlevel, 1 if on_gpu else 0,
                                C.byref(t)))
    try:
        def arr(ptr, count, dt):
            if count == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                         shape=(count,)).copy()
        out = {"slot_off": arr(t.slot_off, npart + 1, np.int64),
               "shell": arr(t.shell, npart * (nlevel + 1), np.int32).reshape(npart, nlevel + 1),
               "slot_vert": arr(t.slot_vert, t.nslots, np.int32),
               "slice_off": arr(t.slice_off, npart + 1, np.int64),
               "ell_off": arr(t.ell_off, t.nslices + 1, np.int64),
               "ell_col": arr(t.ell_col, t.nell, np.uint16),
               "ell_width": arr(t.ell_width, t.nslices, np.uint8),
               "max_slots": t.max_slots, "total_rows": t.total_rows, "built_on_gpu": bool(t.built_on_gpu)}
    finally:
        lib().mpkg_tiles_free(C.byref(t))
    return out


def pa1_tasks(a: Csr, part, npart, nlevel, on_gpu=True):
    """PA1 task lists (nphase = 0) built on the GPU or the host ->
    (off, idx, built_on_gpu)."""
    part = _i32(part)
    off = np.empty(npart + 1, dtype=np.int64)
    ip, cnt, on = C.c_void_p(), C.c_long(), C.c_int()
    _check(lib().mpkg_pa1_tasks(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(part), npart, nlevel, 1 if on_gpu else 0,
                                _ptr(off), C.byref(ip), C.byref(cnt), C.byref(on)))
    return off, _take(ip, cnt.value, np.int64), bool(on.value)


def work_count(dirname):
    """The reference work_count's counts for a prepared MPI-2 directory
    (mpk2/work_count.c): dict comm, ops, minops, nvert, redundant."""
    v = [C.c_long() for _ in range(5)]
    _check(lib().mpkg_work_count(dirname.encode(), *[C.byref(x) for x in v]))
    return dict(zip(("comm", "ops", "minops", "nvert", "redundant"), (x.value for x in v)))


def lapjv(sums):
    """The preps' label assignment (mpk2/lapjv.c:366): perm maximising
    sum_j sums[perm[j], j]."""
    s = np.ascontiguousarray(sums, dtype=np.int32)
    npart = s.shape[0]
    assert s.shape == (npart, npart)
    perm = np.empty(npart, dtype=np.int32)
    _check(lib().mpkg_lapjv(_ptr(s), npart, _ptr(perm)))
    return perm


# ---------------------------------------------------------------- plans
class Plan:
    """A device-resident MPK plan (matrix + schedule) executed many times."""

    def __init__(self, handle, a: Csr, nlevel):
        self._h = C.c_void_p(handle)
        self.n = a.n
        self.nlevel = nlevel

    @staticmethod
    def _make(fn, *args, a, nlevel):
        h = C.c_void_p()
        _check(fn(*args, C.byref(h)))
        return Plan(h.value, a, nlevel)

    @classmethod
    def pa1(cls, a: Csr, part, npart, nlevel, exec=EXEC_TILES, arith=ARITH_FMA):
        part = _i32(part)
        return cls._make(lib().mpkg_plan_pa1, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), _ptr(part),
                         npart, nlevel, exec, arith, a=a, nlevel=nlevel)

    @classmethod
    def from_tasks(cls, a: Csr, npart, nlevel, nphase, off, idx, arith=ARITH_FMA):
        off = np.ascontiguousarray(off, dtype=np.int64)
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        return cls._make(lib().mpkg_plan_tasks, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), npart, nlevel,
                         nphase, _ptr(off), _ptr(idx), arith, a=a, nlevel=nlevel)

    @classmethod
    def pipe(cls, a: Csr, nlevel, chunk=0, arith=ARITH_FMA):
        return cls._make(lib().mpkg_plan_pipe, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), nlevel, chunk,
                         arith, a=a, nlevel=nlevel)

    @classmethod
    def bufs(cls, directory, npart, arith=ARITH_FMA):
        """MPI-2 rank buffers (rank<r>.bufs in `directory`) on one GPU."""
        h = C.c_void_p()
        _check(lib().mpkg_plan_bufs(directory.encode(), npart, arith, C.byref(h)))
        p = Plan.__new__(Plan)
        p._h = h
        inf = p.info()
        p.n, p.nlevel = inf["n"], inf["nlevel"]
        return p

    @classmethod
    def pdmpk(cls, buf_paths, results_paths, arith=ARITH_FMA):
        """pdmpk buffers (one buf.bin / results.bin pair per rank) on one
        GPU; exec writes A^nlevel x to the last level of vv only."""
        bp, rp = _cstrs(buf_paths), _cstrs(results_paths)
        h = C.c_void_p()
        _check(lib().mpkg_plan_pdmpk(len(buf_paths), bp, rp, arith, C.byref(h)))
        p = Plan.__new__(Plan)
        p._h = h
        inf = p.info()
        p.n, p.nlevel = inf["n"], inf["nlevel"]
        return p

    @classmethod
    def mixed(cls, a: Csr, nlevel, value_type=VALUE_F32):
        """Mixed-precision form: FP32/BF16 values, FP32 basis scaled by 2^-e
        per level (A^l x = 2^(l e) v_l)."""
        return cls._make(lib().mpkg_plan_mixed, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), nlevel, value_type,
                         a=a, nlevel=nlevel)

    @classmethod
    def mixed_tiles(cls, a: Csr, part, npart, nlevel, value_type=VALUE_F32):
        """Mixed-precision form on PA1 tiles (temporal blocking: each part
        plus its nlevel-deep skirt computes every level on chip, its
        matrix rows read once per call); same bits as Plan.mixed."""
        part = _i32(part)
        return cls._make(lib().mpkg_plan_mixed_tiles, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), _ptr(part),
                         npart, nlevel, value_type, a=a, nlevel=nlevel)

    @classmethod
    def mixed_tiles_tuned(cls, a: Csr, coords, nlevel, value_type=VALUE_F32):
        """Plan.mixed_tiles with the part size chosen by timing RCB
        partitions of coords (n x dim) into parts of 384..1536 rows;
        info() gives the chosen npart."""
        coords = _i32(coords)
        return cls._make(lib().mpkg_plan_mixed_tiles_tuned, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val),
                         _ptr(coords), coords.shape[1], nlevel, value_type, a=a, nlevel=nlevel)

    def mixed_scale(self):
        """(e, number of values the storage type rounds)."""
        e, inexact = C.c_int(), C.c_long()
        _check(lib().mpkg_mixed_scale(self._h, C.byref(e), C.byref(inexact)))
        return e.value, inexact.value

    def exec_mixed_device(self, d_vv_ptr: int, stream: int = 0):
        _check(lib().mpkg_exec_mixed_device(self._h, C.c_void_p(d_vv_ptr), C.c_void_p(stream or None)))

    @classmethod
    def wave(cls, a: Csr, nlevel, arith=ARITH_FMA, ctas_per_sm=0):
        """Wavefront executor: one persistent launch, neighbour-only waits
        (ctas_per_sm > 0 caps the resident CTAs per SM)."""
        if ctas_per_sm:
            return cls._make(lib().mpkg_plan_wave_ctas, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), nlevel, arith,
                             ctas_per_sm, a=a, nlevel=nlevel)
        return cls._make(lib().mpkg_plan_wave, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), nlevel, arith,
                         a=a, nlevel=nlevel)

    @classmethod
    def batch(cls, mats, nrhs, nlevel, tune=True):
        """Batched block-vector form over a list of Csr (values cast to
        FP32): one persistent launch replayed as a CUDA graph.  tune: True
        (BATCH_TUNE, time every configuration), False (BATCH_DEFAULT), or
        BATCH_STAGED / BATCH_STAGED2 / BATCH_STAGED4 (the shared-memory
        window kernel at one, two or four CTAs per SM, untimed)."""
        keep = []
        n = np.array([m.n for m in mats], dtype=np.int32)
        arrs = []
        for m in mats:
            if m.val is None:
                raise MpkError(EINVAL, "the batched form needs matrix values")
            t = (_i32(m.ptr), _i32(m.col), np.ascontiguousarray(m.val, dtype=np.float32))
            keep.append(t)
        ptrs = (C.c_void_p * len(mats))(*[t[0].ctypes.data for t in keep])
        cols = (C.c_void_p * len(mats))(*[t[1].ctypes.data for t in keep])
        vals = (C.c_void_p * len(mats))(*[t[2].ctypes.data for t in keep])
        h = C.c_void_p()
        _check(lib().mpkg_plan_batch(len(mats), _ptr(n), C.cast(ptrs, C.c_void_p), C.cast(cols, C.c_void_p),
                                     C.cast(vals, C.c_void_p), nrhs, nlevel,
                                     int(tune) if not isinstance(tune, bool) else (1 if tune else 0), C.byref(h)))
        p = Plan.__new__(Plan)
        p._h = h
        p.n, p.nlevel, p.nrhs = int(n.sum()), nlevel, nrhs
        p.row0 = np.concatenate([[0], np.cumsum(n.astype(np.int64))])
        return p

    def batch_info(self) -> dict:
        inf = BatchInfo()
        _check(lib().mpkg_batch_info(self._h, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in BatchInfo._fields_}

    def exec_batch_host(self, vb: np.ndarray) -> np.ndarray:
        """vb: float32 (nlevel+1, N, nrhs) with level 0 filled; in place."""
        assert vb.dtype == np.float32 and vb.flags.c_contiguous and vb.size == (self.nlevel + 1) * self.n * self.nrhs
        _check(lib().mpkg_exec_batch_host(self._h, _ptr(vb)))
        return vb

    def exec_batch_device(self, d_vb_ptr: int, stream: int = 0):
        _check(lib().mpkg_exec_batch_device(self._h, C.c_void_p(d_vb_ptr), C.c_void_p(stream or None)))

    @classmethod
    def spmv(cls, a: Csr, nlevel, arith=ARITH_FMA):
        return cls._make(lib().mpkg_plan_spmv, a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), nlevel, arith,
                         a=a, nlevel=nlevel)

    def info(self) -> dict:
        inf = PlanInfo()
        _check(lib().mpkg_plan_info(self._h, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in PlanInfo._fields_}

    def exec_host(self, vv: np.ndarray) -> np.ndarray:
        """vv: float64 array of (nlevel+1)*n with x in vv[:n]; filled in place."""
        assert vv.dtype == np.float64 and vv.flags.c_contiguous and vv.size == (self.nlevel + 1) * self.n
        _check(lib().mpkg_exec_host(self._h, _ptr(vv)))
        return vv

    def exec_device(self, d_vv_ptr: int, stream: int = 0):
        """Asynchronous launch on device memory (e.g. a torch tensor's data_ptr())."""
        _check(lib().mpkg_exec_device(self._h, C.c_void_p(d_vv_ptr), C.c_void_p(stream or None)))

    def sync(self, stream: int = 0):
        _check(lib().mpkg_sync(self._h, C.c_void_p(stream or None)))

    def debug_stall(self, extra_levels):
        """Test hook: pipeline waits target `extra_levels` beyond the real
        level (0 restores normal behaviour)."""
        _check(lib().mpkg_debug_pipe_stall(self._h, extra_levels))

    def close(self):
        if self._h is not None and self._h.value:
            lib().mpkg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- s-step CG
NFEAT = 12


def _info_dict(inf):
    return {k: getattr(inf, k) for k, _ in CgInfo._fields_}


def cg(a: Csr, b, x0=None, tol=1e-8, max_iter=10000):
    """Standard FP64 CG on the GPU: (x, info)."""
    x = np.zeros(a.n) if x0 is None else np.array(x0, dtype=np.float64)
    b = _f64(b)
    inf = CgInfo()
    _check(lib().mpkg_cg(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), _ptr(b), _ptr(x), tol, max_iter,
                         C.byref(inf)))
    return x, _info_dict(inf)


GRAM_FP64, GRAM_DF64 = 0, 1
SSTEP_DEVICE_LOOP, SSTEP_HOST_LOOP = 0, 1
SSTEP_BASIS_MPK, SSTEP_BASIS_STEPS = 0, 1


def sstep_cg(a: Csr, b, s=8, shifts=None, scale=None, x0=None, tol=1e-8, max_outer=2000, gram=GRAM_FP64,
             loop=SSTEP_DEVICE_LOOP, basis=SSTEP_BASIS_STEPS):
    """s-step CG with an FP32 Newton basis (shifts None: monomial) scaled
    by `scale` per step (default: the Gershgorin upper bound / 2); the
    Gram matrix in FP64 (GRAM_FP64) or double-float (GRAM_DF64); the
    outer loop decided on the device (one graph launch per solve) or on
    the host (one launch and synchronisation per outer iteration)."""
    _check(lib().mpkg_sstep_gram(gram))
    _check(lib().mpkg_sstep_loop(loop))
    _check(lib().mpkg_sstep_basis(basis))
    x = np.zeros(a.n) if x0 is None else np.array(x0, dtype=np.float64)
    b = _f64(b)
    if scale is None:
        _, glo, ghi = features(a)
        scale = ghi / 2.0
    sh = None if shifts is None else _f64(np.asarray(shifts, dtype=np.float64))
    inf = CgInfo()
    _check(lib().mpkg_sstep_cg(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), _ptr(b), _ptr(x), s,
                               None if sh is None else _ptr(sh), float(scale), tol, max_outer, C.byref(inf)))
    return x, _info_dict(inf)


def lanczos(a: Csr, m, seed=0):
    """Ritz values (ascending) of m Lanczos steps, and the tridiagonal."""
    r, al, be = np.zeros(m), np.zeros(m), np.zeros(max(m - 1, 1))
    _check(lib().mpkg_lanczos(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), m, seed, _ptr(r), _ptr(al), _ptr(be)))
    return r, al, be


def tridiag_eigs(alpha, beta):
    al, be = _f64(alpha), _f64(beta if len(beta) else np.zeros(1))
    out = np.zeros(len(al))
    lib().mpkg_tridiag_eigs(len(al), _ptr(al), _ptr(be), _ptr(out))
    return out


def leja(points):
    x = np.array(points, dtype=np.float64)
    lib().mpkg_leja_order(len(x), _ptr(x))
    return x


def features(a: Csr):
    """(features[NFEAT] float32, Gershgorin lower, upper)."""
    f = np.zeros(NFEAT, dtype=np.float32)
    lo, hi = C.c_double(), C.c_double()
    _check(lib().mpkg_features(a.n, _ptr(a.ptr), _ptr(a.col), _ptr(a.val), _ptr(f), C.byref(lo), C.byref(hi)))
    return f, lo.value, hi.value


class Mlp:
    """nin -> width -> width -> nout MLP trained by the library's GPU kernels."""

    def __init__(self, nin=NFEAT, width=64, nout=8, seed=0):
        h = C.c_void_p()
        _check(lib().mpkg_mlp_create(nin, width, nout, seed, C.byref(h)))
        self._h, self.nin, self.width, self.nout = h, nin, width, nout

    @property
    def nparams(self):
        return lib().mpkg_mlp_nparams(self._h)

    def params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        _check(lib().mpkg_mlp_get_params(self._h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        _check(lib().mpkg_mlp_set_params(self._h, _ptr(p)))

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.nout), dtype=np.float32)
        _check(lib().mpkg_mlp_forward(self._h, X.shape[0], _ptr(X), _ptr(Y)))
        return Y

    def gradient(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = C.c_float()
        _check(lib().mpkg_mlp_gradient(self._h, X.shape[0], _ptr(X), _ptr(T), _ptr(g), C.byref(loss)))
        return g, loss.value

    def train(self, X, T, epochs=200, batch=64, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        curve = np.zeros(epochs, dtype=np.float32)
        _check(lib().mpkg_mlp_train(self._h, X.shape[0], _ptr(X), _ptr(T), epochs, batch, lr, seed, _ptr(curve)))
        return curve

    def close(self):
        if self._h:
            lib().mpkg_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
