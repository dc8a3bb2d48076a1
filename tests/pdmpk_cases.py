"""pdmpk golden cases (tests/golden/pdmpk.npz) unpacked into files."""
import os

import numpy as np

from conftest import GOLDEN


def load():
    return dict(np.load(os.path.join(GOLDEN, "pdmpk.npz")))


def cases(g):
    """(matrix, npart, nlevel, mirror, weight) of every stored prep."""
    out = set()
    for k in g:
        parts = k.split("__")
        if len(parts) == 4 and parts[3] in ("buf", "res"):
            P, L, mm, wm = map(int, parts[1].split("_"))
            out.add((parts[0], P, L, mm, wm))
    return sorted(out)


def write_mtx(g, m, d):
    path = os.path.join(d, m + ".mtx")
    with open(path, "wb") as f:
        f.write(g[f"{m}__mtx"].tobytes())
    return path


def write_case(g, case, d, tag="ref"):
    """The reference's per-rank files of one case; returns (buf, res) paths."""
    m, P, L, mm, wm = case
    bp, rp = [], []
    for r in range(P):
        key = f"{m}__{P}_{L}_{mm}_{wm}__r{r}"
        b = os.path.join(d, f"{tag}-{m}-{mm}-{wm}-r{r}.buf.bin")
        s = os.path.join(d, f"{tag}-{m}-{mm}-{wm}-r{r}.results.bin")
        with open(b, "wb") as f:
            f.write(g[key + "__buf"].tobytes())
        with open(s, "wb") as f:
            f.write(g[key + "__res"].tobytes())
        bp.append(b)
        rp.append(s)
    return bp, rp


# buf.bin layout (pdmpk/buffers.cc:194-206): two scalars, then vectors as
# size_t count + elements.
_FIELDS = [("mbuf_pb", 8), ("home", 4), ("orig", 4), ("pd", 6), ("res_mbuf", 4), ("sendcounts", 4),
           ("sdispls", 4), ("recvcounts", 4), ("rdispls", 4), ("sbuf_idcs", 4), ("sbuf_pb", 8), ("init", 8),
           ("init_pb", 8), ("mptr", 4), ("mptr_pb", 8), ("mcol", 4), ("mval", 8)]


def fields(data):
    """name -> (byte offset of the first element, count, element size)."""
    out, o = {}, 12
    for name, size in _FIELDS:
        c = int(np.frombuffer(data[o:o + 8], dtype=np.uint64)[0])
        out[name] = (o + 8, c, size)
        o += 8 + c * size
    assert o == len(data)
    return out


def ctest():
    """The reference's CTest shapes with the sha256 of every rank's
    (buf.bin, results.bin) from the reference prep: {"m9p100_8_20": [...]}."""
    import json
    with open(os.path.join(GOLDEN, "pdmpk_ctest.json")) as f:
        return json.load(f)


def ctest_prep(key, d):
    """The product's prep of one CTest shape (pattern MTX of the gen2 mesh,
    mirror 5, weight 3); returns (matrix, buf paths, results paths)."""
    import mpk_gb300 as M
    m, P, L = key.split("_")
    P, L = int(P), int(L)
    t, size = m[:3], int(m[3:])
    path = os.path.join(d, m + ".mtx")
    M.Csr.stencil(t, size).write_mtx(path, pattern=True)
    a = M.Csr.read_mtx(path)
    bp = [os.path.join(d, f"{key}-r{r}.buf.bin") for r in range(P)]
    rp = [os.path.join(d, f"{key}-r{r}.results.bin") for r in range(P)]
    M.pdmpk_prep(a, P, L, bp, rp, mirror=5, weight=3)
    return a, bp, rp
