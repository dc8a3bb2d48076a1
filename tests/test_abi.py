"""The C-ABI library loads and exports every function include/*.h declares;
the mpk2-compatible structures keep the reference layout; bad inputs give
error codes (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import mpk_gb300 as M
from conftest import ROOT
from oracle import oracle as O

HEADERS = ["mpk_gb300.h", "mpk2_compat.h"]


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"typedef struct\s*\w*\s*\{.*?\}\s*\w+;", " ", text, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{)]*\)\s*;", text)
    return sorted(set(n for n in names if n not in ("if", "sizeof")))


@pytest.mark.parametrize("header", HEADERS)
def test_library_exports_every_declared_symbol(header):
    lib = C.CDLL(M.LIB_PATH)
    names = declared_functions(header)
    assert len(names) > 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_nm_lists_exports():
    out = subprocess.run(["nm", "-D", "--defined-only", M.LIB_PATH], stdout=subprocess.PIPE, text=True).stdout
    for n in declared_functions("mpk_gb300.h") + declared_functions("mpk2_compat.h"):
        assert re.search(r"\bT " + n + r"\b", out), n


def test_legacy_struct_layout():
    """Field offsets of mpk_t/task_t as compiled from include/mpk2_compat.h
    equal the reference's (mpk2/lib.h:78-99), checked with a C compiler."""
    src = r'''
    #include <stddef.h>
    #include <stdio.h>
    #include "mpk2_compat.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(mpk_t), offsetof(mpk_t, g0), offsetof(mpk_t, tlist),
             offsetof(mpk_t, idxallocsize), sizeof(task_t), offsetof(task_t, idx), offsetof(task_t, t1));
      return 0; }'''
    with tempfile.TemporaryDirectory() as d:
        open(os.path.join(d, "a.c"), "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", os.path.join(d, "a"),
                        os.path.join(d, "a.c")], check=True)
        got = subprocess.run([os.path.join(d, "a")], stdout=subprocess.PIPE, text=True).stdout.split()
    assert [int(v) for v in got] == [C.sizeof(O.RefMpk), O.RefMpk.g0.offset, O.RefMpk.tlist.offset,
                                     O.RefMpk.idxallocsize.offset, C.sizeof(O.RefTask), O.RefTask.idx.offset,
                                     O.RefTask.t1.offset]


def test_plan_argument_errors():
    a = M.Csr.laplacian(4, 4)
    bad = M.Csr(a.ptr.copy(), a.col.copy(), a.val)
    bad.col[3] = 99
    with pytest.raises(M.MpkError) as e:
        M.Plan.spmv(bad, 2)
    assert e.value.code in (M.ERANGE, M.ECUDA)
    with pytest.raises(M.MpkError) as e:
        M.Plan.pa1(a, np.zeros(a.n, dtype=np.int32), 1, 2, exec=M.EXEC_PIPE)
    assert e.value.code == M.EINVAL
    with pytest.raises(M.MpkError) as e:
        M.Plan.pa1(a, np.full(a.n, 7, dtype=np.int32), 2, 2)
    assert e.value.code == M.ERANGE


REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src")  # the reference sources staged by oracle/Makefile


@pytest.mark.skipif(not O.ref_available() or not os.path.exists(os.path.join(REF_SRC, "comp.c")),
                    reason="reference sources not present")
@pytest.mark.parametrize("tool", ["comp", "skirt"])
def test_reference_tools_relink_against_library(tool):
    """The reference's own comp.c / skirt.c mains, compiled against
    include/mpk2_compat.h and linked with libmpk_gb300.so instead of the
    reference lib.c, write byte-identical files."""
    a = M.Csr.laplacian(24, 24)
    part = M.partition_rcb(a.coords, 6)
    with tempfile.TemporaryDirectory() as d:
        shim = os.path.join(d, "lib.h")
        open(shim, "w").write('#include "mpk2_compat.h"\n')
        exe = os.path.join(d, tool)
        subprocess.run(["gcc", "-O2", "-w", "-I", d, "-I", os.path.join(ROOT, "include"),
                        os.path.join(REF_SRC, f"{tool}.c"), "-o", exe, M.LIB_PATH,
                        "-Wl,-rpath," + os.path.dirname(M.LIB_PATH)], check=True)
        g = os.path.join(d, "g0")
        a.write_metis(g, ne=(a.nnz + a.n) // 2)
        pf = os.path.join(d, "p")
        np.savetxt(pf, part, fmt="%d")
        if tool == "comp":
            runs = [["level", g, "x", pf], ["weight", g, "x", pf]]
        else:
            runs = [["5", g, "x", pf]]
        for r in runs:
            subprocess.run([exe] + r + [os.path.join(d, "mine")], check=True, stdout=subprocess.DEVNULL)
            subprocess.run([O.ref_tool(tool)] + r + [os.path.join(d, "ref")], check=True, stdout=subprocess.DEVNULL)
            assert open(os.path.join(d, "mine"), "rb").read() == open(os.path.join(d, "ref"), "rb").read()


@pytest.mark.skipif(not O.ref_available() or not os.path.exists(os.path.join(REF_SRC, "mpi2_mpkwrtbufs.c")),
                    reason="reference sources not present")
def test_reference_mpi2_prep_relinks_against_library(monkeypatch):
    """The reference's own mpi2_mpkwrtbufs.c main, compiled against
    include/mpk2_compat.h (plus the single-process mpi.h stand-in) and
    linked with libmpk_gb300.so, writes the same rank buffers as the
    reference build."""
    from conftest import golden_matrix, load_golden
    name = "m5p20_4_4_2"
    g = load_golden(name)
    a = golden_matrix(name)
    with tempfile.TemporaryDirectory() as d:
        for hdr in ("lib.h", "comm_data.h", "buffers.h"):
            open(os.path.join(d, hdr), "w").write('#include "mpk2_compat.h"\n')
        exe = os.path.join(d, "wrtbufs")
        subprocess.run(["gcc", "-O2", "-w", "-I", d, "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "oracle", "refshim"), os.path.join(REF_SRC, "mpi2_mpkwrtbufs.c"), "-o", exe,
                        M.LIB_PATH, "-Wl,-rpath," + os.path.dirname(M.LIB_PATH)], check=True)
        from test_prep import _case_dir
        _case_dir(name, g, a, d)
        monkeypatch.chdir(d)
        for r in range(int(g["npart"])):
            subprocess.run([exe, name], check=True, env=dict(os.environ, MPK_RANK=str(r)), stdout=subprocess.DEVNULL)
            mine = np.fromfile(os.path.join(d, name, f"rank{r}.bufs"), dtype=np.uint8)
            assert mine.tobytes() == g[f"bufs{r}"].tobytes(), f"rank {r}"


PD_PROG = r"""
// A pdmpk-style prep + reload written against include/pdmpk_gb300.h only
// (the shape of the reference's apps/prep.cc and Buffers::Load).
#include <cstdio>
#include <stdexcept>
#include <vector>
#include "pdmpk_gb300.h"
using namespace pdmpk_gb300;
int main(int argc, char **argv) {
  try {
    Csr bad(argv[2]);
    return 10;  // a bad banner must throw, as pdmpk/csr.cc does
  } catch (const std::logic_error &) {
  }
  const Csr csr(argv[1]);
  Args args;
  args.npart = 4;
  args.nlevel = 3;
  args.mirror_method = 2;
  args.weight_update_method = 1;
  std::vector<Buffers> bufs;
  if (CommCompPatterns(csr, args, &bufs) != 0) return 11;
  for (int r = 0; r < args.npart; r++) {
    const std::string b = Filename(argv[3], 4, 3, 2, 1, r, "gb300", "x", "buf.bin");
    const std::string s = Filename(argv[3], 4, 3, 2, 1, r, "gb300", "x", "results.bin");
    if (bufs[r].Dump(b, s) != 0) return 12;
    Buffers back(args.npart);
    if (back.Load(b, s) != 0) return 13;
    if (back.mcsr.mcol != bufs[r].mcsr.mcol || back.mbuf_idx != bufs[r].mbuf_idx ||
        back.phase_descriptors.size() != bufs[r].phase_descriptors.size() ||
        back.mpi_bufs.init_idcs != bufs[r].mpi_bufs.init_idcs)
      return 14;
    for (const PhaseDescriptor &pd : back.phase_descriptors)
      if (pd.bottom > pd.mid || pd.mid > pd.top || pd.top > args.nlevel) return 15;
  }
  std::printf("%d %d\n", csr.n, bufs[0].GetNumPhases());
  return 0;
}
"""


def test_pdmpk_cpp_interface(tmp_path):
    """include/pdmpk_gb300.h compiles as C++17 and links against the
    library; Csr throws on a bad banner; prep, Dump and Load round-trip;
    the files are the ones the product's C entry point writes."""
    src = tmp_path / "pd.cc"
    src.write_text(PD_PROG)
    exe = str(tmp_path / "pd")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe,
                    M.LIB_PATH, "-Wl,-rpath," + os.path.dirname(M.LIB_PATH)], check=True)
    a = M.Csr.laplacian(12, 12, 1, diag=4.0, off=-1.0)
    mtx = str(tmp_path / "m.mtx")
    a.write_mtx(mtx)
    bad = tmp_path / "bad.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n2 2\n")
    stem = str(tmp_path / "m.mtx")
    out = subprocess.run([exe, mtx, str(bad), stem], capture_output=True, text=True)
    assert out.returncode == 0, out.returncode
    n, nb = map(int, out.stdout.split())
    assert n == a.n and nb >= 3
    bp = [str(tmp_path / f"c{r}.buf.bin") for r in range(4)]
    rp = [str(tmp_path / f"c{r}.results.bin") for r in range(4)]
    M.pdmpk_prep(a, 4, 3, bp, rp, mirror=2, weight=1)
    for r in range(4):
        assert open(bp[r], "rb").read() == open(f"{stem}-np4-nl3-mm2-wm1-r{r}-gb300-x.buf.bin", "rb").read()
