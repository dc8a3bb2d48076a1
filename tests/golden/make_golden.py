"""Generates the golden fixtures in this directory from the REFERENCE code.

Run in a checkout that has the reference sources (vatai/mpk) available to
oracle/Makefile: the reference mpk2 library and tools are compiled from
their own sources into oracle/_ref/, then driven exactly as the reference
scripts drive them (mpk2/driver.c, mpk2/mpktest.c, mpk2/verify_val.c):

  comp level / comp weight  -> level files l<ph> and weight graphs g<ph+1>
  skirt                     -> skirt file s<nphase>
  read_mpk + prep_mpk       -> task lists
  exec_mpk / vexec_mpk      -> vv for a seeded x (1/deg and valued operator)
  verify_val                -> gold_result.bin (x = 1, valued operator)
  pdmpk prep (apps/prep.cc) -> per-rank buf.bin / results.bin (pdmpk.npz)
  lapjv, work_count         -> lapjv.npz, work_count.json (verification tools)
  pdmpk prep, CTest shapes  -> pdmpk_ctest.json (hashes of every rank's files)
  METIS partitions          -> m9p24_8_4_2m.npz (the mpk2 driver's flow with
                               METIS at every phase) and pdmpk_metis.json (the
                               CTest shapes with the reference prep compiled
                               against METIS)

Inputs (graphs, partitions, x) come from the product's generators and
partitioners, stored with the fixture: recursive coordinate bisection or
breadth-first bisection vectors, or METIS partitions.  METIS is the library
bundled with the CUDA toolkit; gpmetis itself is not installed, so the
driver's `gpmetis -ufactor=100 g<ph> P` calls (mpk2/driver.c:63-66) are
made through oracle/metis_part.c on the same graph files, and the reference
pdmpk prep is compiled a second time against METIS
(oracle/refshim_metis/metis.h).  The reference binaries here are x86-64 gcc -O2 builds, which do
not contract a*b+c, so every floating-point fixture is in the oracle's
"separate" arithmetic mode.

    python tests/golden/make_golden.py                # everything
    python tests/golden/make_golden.py verification   # lapjv + work_count only
    python tests/golden/make_golden.py ctest          # pdmpk CTest shapes only
    python tests/golden/make_golden.py metis          # the METIS fixtures only
"""
import ctypes as C
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import mpk_gb300 as M  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = [
    # name, grid (nx, ny, nz) or ("cube", size), npart, nlevel, nphase, partitioner, valued, seed
    dict(name="m5p10_4_4_0", grid=(10, 10, 1), npart=4, nlevel=4, nphase=0, part="rcb", seed=3),
    dict(name="cfg1_4_4_0", grid=(100, 100, 1), npart=4, nlevel=4, nphase=0, part="rcb", seed=0, gold=True),
    dict(name="m5p20_4_4_2", grid=(20, 20, 1), npart=4, nlevel=4, nphase=2, part="rcb+bfs", seed=5),
    dict(name="m5p16_4_6_3", grid=(16, 16, 1), npart=4, nlevel=6, nphase=3, part="bfs+rcb+bfs", seed=6),
    dict(name="cube6_8_3_0", grid=("cube", 6), npart=8, nlevel=3, nphase=0, part="bfs", seed=7),
]
# the driver's flow with METIS partitions at every phase (9-point mesh)
METIS_CASES = [
    dict(name="m9p24_8_4_2m", grid=("m9p", 24), npart=8, nlevel=4, nphase=2, part="metis", seed=9),
]


def read_weighted_graph(path):
    """A METIS graph file written by the reference's `comp weight`
    (header "n m 011": each line a vertex weight, then column/weight
    pairs): (ptr, col, vwgt, adjwgt), 0-based columns."""
    with open(path) as f:
        f.readline()
        ptr, col, vw, ew = [0], [], [], []
        for line in f:
            t = [int(v) for v in line.split()]
            vw.append(t[0])
            col += [c - 1 for c in t[1::2]]
            ew += t[2::2]
            ptr.append(len(col))
    return (np.array(ptr, dtype=np.int32), np.array(col, dtype=np.int32), np.array(vw, dtype=np.int32),
            np.array(ew, dtype=np.int32))


def loop_matrix(case):
    """The matrix with diagonal (the .loop.g0/.loop.val pair)."""
    if isinstance(case["grid"][0], str):
        return M.Csr.stencil(case["grid"][0], case["grid"][1])
    nx, ny, nz = case["grid"]
    return M.Csr.laplacian(nx, ny, nz, diag=4.0 if nz == 1 else 6.0, off=-1.0)


def partitions(case, a):
    kinds = case["part"].split("+")
    out = []
    for ph in range(max(case["nphase"], 1)):
        kind = kinds[min(ph, len(kinds) - 1)]
        if kind == "rcb":
            out.append(M.partition_rcb(a.coords, case["npart"]))
        else:
            out.append(M.partition_bfs(a, case["npart"]))
    return out


def run(cmd, **kw):
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, **kw)


def make(case, tmp):
    a = loop_matrix(case)
    n, npart, nlevel, nphase = a.n, case["npart"], case["nlevel"], case["nphase"]
    ghead = case["name"].split("_")[0]
    d = os.path.join(tmp, case["name"])
    os.makedirs(d)
    a.write_metis(os.path.join(d, "g0"), ne=(a.nnz + a.n) // 2)
    a.write_metis(os.path.join(d, "loop.g0"), ne=(a.nnz + a.n) // 2)
    a.write_values(os.path.join(tmp, ghead + ".loop.val"))
    metis = case["part"] == "metis"
    parts = [O.metis_kway(a.ptr, a.col, npart, 100)] if metis else partitions(case, a)
    for ph, p in enumerate(parts):
        np.savetxt(os.path.join(d, f"g{ph}.part.{npart}"), p, fmt="%d")
    comp, skirt = O.ref_tool("comp"), O.ref_tool("skirt")
    levels, weights = [], []
    for ph in range(nphase):
        if metis and ph > 0:  # gpmetis -ufactor=100 on the weighted graph of the phase
            gp, gc, vw, ew = read_weighted_graph(f"{d}/g{ph}")
            parts.append(O.metis_kway(gp, gc, npart, 100, vw, ew))
            np.savetxt(os.path.join(d, f"g{ph}.part.{npart}"), parts[-1], fmt="%d")
        args = [comp, "level", f"{d}/g0", "x", f"{d}/g{ph}.part.{npart}"]
        if ph > 0:
            args.append(f"{d}/l{ph - 1}")
        run(args + [f"{d}/l{ph}"])
        levels.append(np.loadtxt(f"{d}/l{ph}", dtype=np.int32).reshape(-1))
        wargs = [comp, "weight", f"{d}/g0", "x", f"{d}/g{ph}.part.{npart}"]
        if ph > 0:
            wargs.append(f"{d}/l{ph - 1}")
        run(wargs + [f"{d}/g{ph + 1}"])
        with open(f"{d}/g{ph + 1}") as f:
            f.readline()
            we = [int(t) for line in f for t in line.split()[1:][1::2]]
        weights.append(np.array(we, dtype=np.int32))
    sargs = [skirt, str(nlevel), f"{d}/g0", "x", f"{d}/g0.part.{npart}"]
    if nphase > 0:
        sargs.append(f"{d}/l{nphase - 1}")
    run(sargs + [f"{d}/s{nphase}"])
    with open(f"{d}/s{nphase}", "rb") as f:
        skirt_bytes = f.read()

    R = O.ref()
    x = M.uniform(case["seed"], n)
    mg = R.read_mpk(d.encode())
    vv = np.zeros((nlevel + 1) * n, dtype=np.float64)
    R.prep_mpk(mg, vv.ctypes.data_as(C.c_void_p))
    off, idx = O.ref_tasks(mg)
    vv[:] = 0.0
    vv[:n] = x
    R.exec_mpk_xd(mg, vv.ctypes.data_as(C.c_void_p), 2)
    vv_deg = vv.copy()
    vv[:] = 0.0
    vv[:n] = x
    R.vexec_mpk(mg, vv.ctypes.data_as(C.c_void_p), a.val.ctypes.data_as(C.c_void_p))
    vv_val = vv.copy()
    R.spmv_exec_seq.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    vv[:] = 0.0
    vv[:n] = x
    R.spmv_exec_seq(mg.contents.g0, vv.ctypes.data_as(C.c_void_p), nlevel)
    vv_spmv = vv.copy()
    out = dict(n=n, npart=npart, nlevel=nlevel, nphase=nphase, seed=case["seed"],
               parts=np.array(parts, dtype=np.int32), x=x,
               skirt=np.frombuffer(skirt_bytes, dtype=np.uint8),
               off=off, idx=idx, vv_deg=vv_deg, vv_val=vv_val, vv_spmv=vv_spmv)
    if n > 1000:  # keep the large fixture small: hashes for the 1/deg results
        for k in ("vv_deg", "vv_spmv"):
            out[k + "_sha256"] = np.frombuffer(hashlib.sha256(out.pop(k).tobytes()).digest(), dtype=np.uint8)
    if nphase:
        out["levels"] = np.array(levels, dtype=np.int32)
        out["weights"] = np.array(weights, dtype=np.int32)
    if n <= 1000:  # MPI-2 rank buffers from the reference prep (mpi2_mpkwrtbufs)
        for r in range(npart):
            run([O.ref_tool("mpi2_mpkwrtbufs"), case["name"]], cwd=tmp, env=dict(os.environ, MPK_RANK=str(r)))
            with open(os.path.join(d, f"rank{r}.bufs"), "rb") as f:
                out[f"bufs{r}"] = np.frombuffer(f.read(), dtype=np.uint8)
    if case.get("gold"):
        run([O.ref_tool("verify_val"), case["name"]], cwd=tmp)
        out["gold_x1"] = np.fromfile(os.path.join(d, "gold_result.bin"), dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
    return out


# pdmpk prep cases: (matrix, npart, nlevel, [(mirror, weight), ...]); the
# reference prep (apps/prep.cc) runs with the oracle's METIS stand-in
# (oracle/refshim/metis.h); STUCK lists combinations where it exits
# ("Couldn't finish").
PD_MATRICES = {
    "m5p10": lambda: M.Csr.laplacian(10, 10, 1, diag=4.0, off=-1.0),
    "m5p16": lambda: M.Csr.laplacian(16, 16, 1, diag=4.0, off=-1.0),
    "cube6": lambda: M.Csr.stencil("cube", 6),
    "m5p20p": lambda: M.Csr.laplacian(20, 20, 1, diag=4.0, off=-1.0),  # written as a pattern file
}
PD_CASES = [
    ("m5p10", 4, 4, [(0, 0), (1, 1), (2, 2), (3, 3), (4, 0), (5, 1)]),
    ("m5p16", 4, 6, [(0, 3), (1, 2), (4, 1), (5, 0)]),
    ("cube6", 8, 3, [(0, 1), (2, 3), (4, 2), (5, 0)]),
    ("m5p20p", 4, 5, [(0, 2), (2, 0), (4, 3), (5, 2)]),
]
PD_STUCK = [("cube6", 8, 3, 1, 0), ("m5p20p", 4, 5, 3, 1)]


def make_pdmpk(tmp):
    d = os.path.join(tmp, "pdmpk")
    os.makedirs(d)
    out = {}
    for m, P, L, combos in PD_CASES:
        mtx = os.path.join(d, m + ".mtx")
        PD_MATRICES[m]().write_mtx(mtx, pattern=m.endswith("p"))
        out[f"{m}__mtx"] = np.frombuffer(open(mtx, "rb").read(), dtype=np.uint8)
        for mm, wm in combos:
            run([O.ref_tool("pdmpk_prep"), "--matrix", m + ".mtx", "--npart", str(P), "--nlevel", str(L),
                 "--mirror", str(mm), "--weight", str(wm), "--keepfiles"], cwd=d)
            for r in range(P):
                stem = os.path.join(d, f"{m}.mtx-np{P}-nl{L}-mm{mm}-wm{wm}-r{r}-ref-oracle")
                key = f"{m}__{P}_{L}_{mm}_{wm}__r{r}"
                out[key + "__buf"] = np.frombuffer(open(stem + ".buf.bin", "rb").read(), dtype=np.uint8)
                out[key + "__res"] = np.frombuffer(open(stem + ".results.bin", "rb").read(), dtype=np.uint8)
    for m, P, L, mm, wm in PD_STUCK:
        mtx = os.path.join(d, m + ".mtx")
        r = subprocess.run([O.ref_tool("pdmpk_prep"), "--matrix", m + ".mtx", "--npart", str(P), "--nlevel",
                            str(L), "--mirror", str(mm), "--weight", str(wm)], cwd=d, capture_output=True)
        assert r.returncode != 0, "expected the reference prep to get stuck"
    out["stuck"] = np.array([f"{m}_{P}_{L}_{mm}_{wm}" for m, P, L, mm, wm in PD_STUCK])
    np.savez_compressed(os.path.join(HERE, "pdmpk.npz"), **out)
    return out


# The reference's CTest shapes (tests/CMakeLists.txt:3-42): gen2 meshes
# written as pattern Matrix Market files (1/deg values), mirror 5, weight 3.
PD_CTEST = [("m5p", 4, 4, 4)] + [(t, size, P, L) for t in ("m5p", "m9p") for size in (10, 100)
                                 for P in (4, 8) for L in (10, 20)]


def make_pdmpk_ctest(tmp):
    """sha256 of the reference prep's per-rank buf.bin / results.bin for
    every CTest shape (pdmpk_ctest.json)."""
    d = os.path.join(tmp, "ctest")
    os.makedirs(d)
    out = {}
    for t, size, P, L in PD_CTEST:
        m = f"{t}{size}"
        M.Csr.stencil(t, size).write_mtx(os.path.join(d, m + ".mtx"), pattern=True)
        run([O.ref_tool("pdmpk_prep"), "--matrix", m + ".mtx", "--npart", str(P), "--nlevel", str(L),
             "--mirror", "5", "--weight", "3", "--keepfiles"], cwd=d)
        ranks = []
        for r in range(P):
            stem = os.path.join(d, f"{m}.mtx-np{P}-nl{L}-mm5-wm3-r{r}-ref-oracle")
            ranks.append([hashlib.sha256(open(stem + ext, "rb").read()).hexdigest()
                          for ext in (".buf.bin", ".results.bin")])
        out[f"{m}_{P}_{L}"] = ranks
    with open(os.path.join(HERE, "pdmpk_ctest.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    return out


def make_pdmpk_metis(tmp):
    """sha256 of the reference prep's per-rank files for every CTest shape
    with the reference compiled against METIS (pdmpk_metis.json)."""
    d = os.path.join(tmp, "ctest_metis")
    os.makedirs(d)
    out = {}
    for t, size, P, L in PD_CTEST:
        m = f"{t}{size}"
        M.Csr.stencil(t, size).write_mtx(os.path.join(d, m + ".mtx"), pattern=True)
        run([O.ref_tool("pdmpk_prep_metis"), "--matrix", m + ".mtx", "--npart", str(P), "--nlevel", str(L),
             "--mirror", "5", "--weight", "3", "--keepfiles"], cwd=d)
        ranks = []
        for r in range(P):
            stem = os.path.join(d, f"{m}.mtx-np{P}-nl{L}-mm5-wm3-r{r}-ref-oracle")
            ranks.append([hashlib.sha256(open(stem + ext, "rb").read()).hexdigest()
                          for ext in (".buf.bin", ".results.bin")])
        out[f"{m}_{P}_{L}"] = ranks
    with open(os.path.join(HERE, "pdmpk_metis.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    return out


def make_metis(tmp):
    for case in METIS_CASES:
        out = make(case, tmp)
        print(case["name"], "n", out["n"], "tasks", len(out["idx"]))
    print(len(make_pdmpk_metis(tmp)), "pdmpk CTest shapes with METIS")


def make_verification(tmp):
    """Known answers of the reference's verification tools:
    * lapjv.npz: lapjv (mpk2/lapjv.c:366) permutations on seeded square
      matrices, half of them with many ties (entries in {0, 1, 2});
    * work_count.json: mpk2/work_count's summary (communication, ops,
      minops, nvert) and its redundancy lines for every golden case that
      carries rank buffers, run on a directory rebuilt from the fixture."""
    R = O.ref()
    R.lapjv.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    rng = np.random.default_rng(20191129)
    sizes, sums, perms = [], [], []
    for n in (2, 3, 4, 5, 6, 8, 12, 16):
        for t in range(40):
            s = np.ascontiguousarray(rng.integers(0, 3 if t % 2 else 10000, (n, n)), dtype=np.int32)
            p = np.zeros(n, dtype=np.int32)
            R.lapjv(s.ctypes.data, n, p.ctypes.data)
            sizes.append(n)
            sums.append(s.ravel())
            perms.append(p)
    np.savez_compressed(os.path.join(HERE, "lapjv.npz"), sizes=np.array(sizes, dtype=np.int32),
                        sums=np.concatenate(sums), perms=np.concatenate(perms))
    counts = {}
    for case in CASES:
        g = np.load(os.path.join(HERE, case["name"] + ".npz"))
        if "bufs0" not in g:
            continue
        a = loop_matrix(case)
        name, npart, nphase = case["name"], case["npart"], case["nphase"]
        d = os.path.join(tmp, name)
        os.makedirs(d)
        a.write_metis(os.path.join(d, "loop.g0"), ne=(a.nnz + a.n) // 2)
        for r in range(npart):
            g[f"bufs{r}"].tofile(os.path.join(d, f"rank{r}.bufs"))
        for ph in range(max(nphase, 1)):
            np.savetxt(os.path.join(d, f"g{ph}.part.{npart}"), g["parts"][ph], fmt="%d")
        for ph in range(nphase):
            np.savetxt(os.path.join(d, f"l{ph}"), g["levels"][ph], fmt="%d")
        g["skirt"].tofile(os.path.join(d, f"s{nphase}"))
        a.write_values(os.path.join(tmp, name.split("_")[0] + ".loop.val"))
        out = subprocess.run([O.ref_tool("work_count"), name], cwd=tmp, check=True, capture_output=True, text=True)
        with open(os.path.join(tmp, f"summary-{name}.log")) as f:
            f.readline()
            comm, ops, minops, nvert = (int(v) for v in f.readline().split())
        counts[name] = dict(comm=comm, ops=ops, minops=minops, nvert=nvert,
                            redundant=out.stdout.count("!!!Redundancy"))
    with open(os.path.join(HERE, "work_count.json"), "w") as f:
        json.dump(counts, f, indent=1)
        f.write("\n")
    return counts


def main():
    O.build()
    if not O.ref_available():
        sys.exit("reference sources not available: cannot regenerate golden fixtures")
    tmp = tempfile.mkdtemp()
    try:
        if sys.argv[1:] == ["verification"]:  # only the verification-tool answers
            print(make_verification(tmp))
            return
        if sys.argv[1:] == ["ctest"]:  # only the pdmpk CTest shapes
            print(len(make_pdmpk_ctest(tmp)), "pdmpk CTest shapes")
            return
        if sys.argv[1:] == ["metis"]:  # only the METIS fixtures
            make_metis(tmp)
            return
        for case in CASES:
            out = make(case, tmp)
            print(case["name"], "n", out["n"], "tasks", len(out["idx"]))
        out = make_pdmpk(tmp)
        print("pdmpk", len(out), "arrays")
        print(make_verification(tempfile.mkdtemp(dir=tmp)))
        print(len(make_pdmpk_ctest(tmp)), "pdmpk CTest shapes")
        make_metis(tmp)
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main()
