"""Mixed-precision form (FP32/BF16 values, FP32 basis with exact
power-of-two level scaling): error per power against the FP64 oracle."""
import numpy as np
import pytest

import mpk_gb300 as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6  # relative error per power vector vs FP64 (FP32 storage)


def run_mixed(a, k, value_type, x):
    import torch
    plan = M.Plan.mixed(a, k, value_type)
    e, inexact = plan.mixed_scale()
    d = torch.zeros((k + 1) * a.n, dtype=torch.float32, device="cuda")
    d[:a.n] = torch.from_numpy(x.astype(np.float32)).cuda()
    torch.cuda.synchronize()
    plan.exec_mixed_device(d.data_ptr())
    plan.sync()
    v = d.cpu().numpy().astype(np.float64).reshape(k + 1, a.n)
    return v * (2.0 ** (e * np.arange(k + 1)))[:, None], e, inexact


def rel_errors(v, want, n, k):
    w = want.reshape(k + 1, n)
    return [float(np.linalg.norm(v[l] - w[l]) / np.linalg.norm(w[l])) for l in range(1, k + 1)]


def test_mixed_fp32_diffusion_9pt(gpu):
    a = M.Csr.diffusion(256, 256, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, seed=3)
    x = M.uniform(4, a.n)
    v, e, inexact = run_mixed(a, 8, M.VALUE_F32, x)
    want = O.mpk(a.ptr, a.col, a.val, x, 8, O.MODE_FMA)
    errs = rel_errors(v, want, a.n, 8)
    assert max(errs) <= MIXED_TOL, errs
    assert inexact > 0  # log-normal coefficients are not FP32 numbers


def test_mixed_bf16_lossless_on_stencil(gpu):
    """BF16 values are exact for stencil matrices (diagonal 6, off -1)."""
    a = M.Csr.laplacian(48, 40, 32, diag=6.0, off=-1.0)
    x = M.uniform(5, a.n)
    v, e, inexact = run_mixed(a, 8, M.VALUE_BF16, x)
    assert inexact == 0 and e == 4  # ||A||_inf = 12 -> 2^4
    want = O.mpk(a.ptr, a.col, a.val, x, 8, O.MODE_FMA)
    errs = rel_errors(v, want, a.n, 8)
    assert max(errs) <= MIXED_TOL, errs


def _conv_diff(nx, ny, c):
    """Upwind convection-diffusion on nx*ny: centre 4+c, west -1-c, east,
    south and north -1.  Strongly non-normal for large c (||A||_inf = 8+2c
    far above the spectral radius)."""
    yy, xx = np.divmod(np.arange(nx * ny), nx)
    ents = [((0, -1), -1.0), ((-1, 0), -1.0 - c), ((0, 0), 4.0 + c), ((1, 0), -1.0), ((0, 1), -1.0)]
    rows, cols, vals = [], [], []
    for (dx, dy), v in ents:
        ok = (xx + dx >= 0) & (xx + dx < nx) & (yy + dy >= 0) & (yy + dy < ny)
        i = np.nonzero(ok)[0]
        rows.append(i)
        cols.append(i + dx + nx * dy)
        vals.append(np.full(i.size, v))
    r, cc, vv = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    o = np.lexsort((cc, r))
    ptr = np.zeros(nx * ny + 1, dtype=np.int64)
    np.add.at(ptr, r[o] + 1, 1)
    return M.Csr(np.cumsum(ptr).astype(np.int32), cc[o].astype(np.int32), vv[o])


@pytest.mark.parametrize("c", [20.0, 100.0])
def test_mixed_nonnormal_31_levels_no_underflow(c, gpu):
    """The static 2^-e scaling (2^e >= ||A||_inf) on a strongly non-normal
    operator whose levels shrink by about ||A||_inf / rho per power: at
    the largest nlevel (31) no level entry that is nonzero in FP64 falls
    to an FP32 subnormal or zero, and every power stays within 1e-6 of
    FP64.  A basis could underflow only after about
    126 / log2(2^e / rho) powers."""
    a = _conv_diff(96, 80, c)
    k = 31
    x = M.uniform(9, a.n)
    v, e, _ = run_mixed(a, k, M.VALUE_F32, x)
    raw = v / (2.0 ** (e * np.arange(k + 1)))[:, None]
    want = O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA).reshape(k + 1, a.n)
    assert not np.any((np.abs(raw[1:]) < np.finfo(np.float32).tiny) & (want[1:] != 0))
    assert np.abs(raw[k]).max() < 0.1  # the basis shrinks, it does not grow
    assert max(rel_errors(v, want, a.n, k)) <= MIXED_TOL


def test_mixed_scaling_keeps_basis_bounded(gpu):
    a = M.Csr.laplacian(64, 64, 16, diag=6.0, off=-1.0)
    x = np.ones(a.n)
    v, e, _ = run_mixed(a, 12, M.VALUE_F32, x)
    raw = v / (2.0 ** (e * np.arange(13)))[:, None]
    assert np.all(np.abs(raw) <= 1.0 + 1e-6)


def test_mixed_runs_on_wavefront_schedule(gpu):
    """The mixed form runs on the wavefront schedule when its kernel fits
    the wavefront grid (plan info reports pipe_chunk 0)."""
    for a in (M.Csr.laplacian(64, 64, 16, diag=6.0, off=-1.0),
              M.Csr.diffusion(256, 256, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, dominance=0.01, seed=3)):
        for vt in (M.VALUE_F32, M.VALUE_BF16):
            plan = M.Plan.mixed(a, 6, vt)
            assert plan.info()["pipe_chunk"] == 0
            plan.close()


def test_mixed_wait_times_out_and_recovers(gpu):
    """The mixed wavefront's bounded waits give up on a flag that is never
    set (ETIMEOUT, context usable) and the same plan then runs correctly."""
    a = M.Csr.laplacian(48, 40, 32, diag=6.0, off=-1.0)
    x = M.uniform(5, a.n)
    plan = M.Plan.mixed(a, 6, M.VALUE_F32)
    assert plan.info()["pipe_chunk"] == 0  # the wavefront schedule
    plan.debug_stall(100)
    import torch
    d = torch.zeros(7 * a.n, dtype=torch.float32, device="cuda")
    d[:a.n] = torch.from_numpy(x.astype(np.float32)).cuda()
    torch.cuda.synchronize()
    plan.exec_mixed_device(d.data_ptr())
    with pytest.raises(M.MpkError) as e:
        plan.sync()
    assert e.value.code == M.ETIMEOUT
    plan.debug_stall(0)
    plan.close()
    v, e_, _ = run_mixed(a, 6, M.VALUE_F32, x)
    want = O.mpk(a.ptr, a.col, a.val, x, 6, O.MODE_FMA)
    assert max(rel_errors(v, want, a.n, 6)) <= MIXED_TOL


def test_mixed_values_beyond_l2_bitwise_vs_fp32_oracle(gpu):
    """2048^2 9-point diffusion: 151 MB of FP32 values, more than L2, so
    the plan loads them evict-first.  The
    levels equal the FP32 oracle's bit for bit (FP32 FMA in CSR order on
    the values scaled by the exact power of two) and stay within 1e-6 of
    FP64 per power."""
    a = M.Csr.diffusion(2048, 2048, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, dominance=0.01, seed=3)
    k = 8
    x = M.uniform(4, a.n)
    v, e, _ = run_mixed(a, k, M.VALUE_F32, x)
    got = (v / (2.0 ** (e * np.arange(k + 1)))[:, None]).astype(np.float32)
    sval = a.val.astype(np.float32) * np.float32(2.0 ** -e)
    want = O.spmm_f32(a.ptr, a.col, sval, x.astype(np.float32)[:, None], k)[:, :, 0]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    want64 = O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA)
    assert max(rel_errors(v, want64, a.n, k)) <= MIXED_TOL


def _mixed_bits(plan, x, k, n):
    import torch
    d = torch.full(((k + 1) * n,), float("nan"), dtype=torch.float32, device="cuda")
    d[:n] = torch.from_numpy(x.astype(np.float32)).cuda()
    torch.cuda.synchronize()
    plan.exec_mixed_device(d.data_ptr())
    plan.sync()
    return d.cpu().numpy()


@pytest.mark.parametrize("case", ["diffusion", "cube", "banded", "bigparts"])
@pytest.mark.parametrize("vt", [M.VALUE_F32, M.VALUE_BF16])
def test_mixed_tiles_bitwise_equal_wavefront(case, vt, gpu):
    """The PA1-tile schedule of the mixed form (temporal blocking) gives
    the wavefront schedule's bits: FP32 FMA in CSR order, exact 2^-e
    scaling.  Cases cover register-held rows (9- and 7-point stencils),
    rows wider than the register budget (random banded, up to 30 entries)
    and tiles with more rows than the threads hold (large parts).  PA1
    needs a symmetric pattern: the reference's skirt distance follows the
    columns a row reads (mpk2/lib.c:203-219), and only then does every
    column of a skirt row lie in the tile (mpk2/mpkprep.c:196-222 checks
    it)."""
    k = 6 if case != "bigparts" else 4
    if case == "diffusion":
        a = M.Csr.diffusion(192, 160, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, dominance=0.01, seed=3)
        part, npart = M.partition_rcb(_grid2(192, 160), 64), 64
    elif case == "cube":
        a = M.Csr.laplacian(40, 36, 32, diag=6.0, off=-1.0)
        part, npart = M.partition_rcb(a.coords, 48), 48
    elif case == "banded":  # symmetric pattern (PA1 needs one): B + B^T of a random banded B
        import scipy.sparse as sp
        bb = M.Csr.banded(3000, 64, 5, 30, seed=4)
        B = sp.csr_matrix((bb.val, bb.col, bb.ptr), shape=(bb.n, bb.n))
        S = (B + B.T).tocsr()
        S.sort_indices()
        a = M.Csr(S.indptr, S.indices, S.data)
        npart = 12
        part = (np.arange(a.n) * npart // a.n).astype(np.int32)
    else:
        a = M.Csr.laplacian(64, 64, 4, diag=6.0, off=-1.0)
        part, npart = M.partition_rcb(a.coords, 4), 4  # 4096-row parts: rows beyond the registers
    x = M.uniform(11, a.n)
    tiles = M.Plan.mixed_tiles(a, part, npart, k, vt)
    wave = M.Plan.mixed(a, k, vt)
    assert tiles.mixed_scale() == wave.mixed_scale()
    got, want = _mixed_bits(tiles, x, k, a.n), _mixed_bits(wave, x, k, a.n)
    tiles.close()
    wave.close()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        f"{np.count_nonzero(got.view(np.uint32) != want.view(np.uint32))} entries differ"


def _stencil2(nx, ny, offsets, seed):
    """2-D stencil on nx*ny with the given (dx, dy) offsets (a symmetric
    set), log-normal off-diagonal values, diagonally dominant rows."""
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    yy, xx = np.divmod(np.arange(nx * ny), nx)
    for dx, dy in offsets:
        ok = (xx + dx >= 0) & (xx + dx < nx) & (yy + dy >= 0) & (yy + dy < ny)
        i = np.nonzero(ok)[0]
        rows.append(i)
        cols.append(i + dx + nx * dy)
    r, c = np.concatenate(rows), np.concatenate(cols)
    o = np.lexsort((c, r))
    r, c = r[o], c[o]
    v = rng.lognormal(0.0, 1.0, r.size)
    off = r != c
    v[off] = -v[off]
    rs = np.bincount(r[off], weights=-v[off], minlength=nx * ny)
    v[~off] = rs[r[~off]] + 0.01
    ptr = np.zeros(nx * ny + 1, dtype=np.int64)
    np.add.at(ptr, r + 1, 1)
    return M.Csr(np.cumsum(ptr).astype(np.int32), c.astype(np.int32), v)


@pytest.mark.parametrize("case", ["lap5", "diff9", "wide11", "k1", "k2", "k12", "k20", "bigparts"])
@pytest.mark.parametrize("vt", [M.VALUE_F32, M.VALUE_BF16])
def test_mixed_register_tiles_bitwise_equal_wavefront(case, vt, gpu):
    """Tiles whose computed rows fit the register-resident kernel (at most
    2304 rows of at most 12 entries) run on it, several tiles per CTA,
    with the next tile's images streaming in while a tile computes; the
    bits equal the wavefront schedule's.  Row widths 5, 9 and 11 (padded
    to 12) select the kernel's three widths; k = 1 and 2 cover the x
    gather right after the first level, k = 12 and 20 small parts with
    deep skirts (20 levels of shells in the tile header).  Larger tiles keep the general tile kernel."""
    k = {"k1": 1, "k2": 2, "k12": 12, "k20": 20, "wide11": 5, "bigparts": 4}.get(case, 8)
    if case == "lap5":
        a = M.Csr.laplacian(300, 200, 1, diag=4.0, off=-1.0)
        part, npart = M.partition_rcb(_grid2(300, 200), 240), 240
    elif case == "wide11":
        offs = [(dx, dy) for dx in (-1, 0, 1) for dy in (-1, 0, 1)] + [(-2, 0), (2, 0)]
        a = _stencil2(200, 180, offs, seed=7)
        part, npart = M.partition_rcb(_grid2(200, 180), 300), 300
    elif case == "bigparts":
        a = M.Csr.laplacian(64, 64, 4, diag=6.0, off=-1.0)
        part, npart = M.partition_rcb(a.coords, 4), 4
    else:
        nx, ny, npart = {"diff9": (256, 200, 400), "k12": (128, 128, 256),
                         "k20": (96, 96, 1152)}.get(case, (128, 128, 100))
        a = M.Csr.diffusion(nx, ny, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, dominance=0.01, seed=5)
        part = M.partition_rcb(_grid2(nx, ny), npart)
    x = M.uniform(13, a.n)
    tiles = M.Plan.mixed_tiles(a, part, npart, k, vt)
    assert tiles.info()["tile_regs"] == (0 if case == "bigparts" else 1)
    wave = M.Plan.mixed(a, k, vt)
    got, want = _mixed_bits(tiles, x, k, a.n), _mixed_bits(wave, x, k, a.n)
    again = _mixed_bits(tiles, x, k, a.n)  # a second call on the same plan
    tiles.close()
    wave.close()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        f"{np.count_nonzero(got.view(np.uint32) != want.view(np.uint32))} entries differ"
    assert np.array_equal(again.view(np.uint32), want.view(np.uint32))


def test_mixed_tiles_tuned_part_size(gpu):
    """The part-size autotuner times RCB partitions into parts of 384 to
    1536 rows and keeps the fastest tile plan; whatever it picks gives
    the wavefront's bits."""
    a = M.Csr.diffusion(256, 200, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, dominance=0.01, seed=6)
    k = 8
    plan = M.Plan.mixed_tiles_tuned(a, _grid2(256, 200), k, M.VALUE_F32)
    inf = plan.info()
    assert inf["tune_candidates"] >= 3 and inf["tune_ms"] > 0
    assert inf["npart"] in {-(-a.n // rows) for rows in (384, 512, 768, 1024, 1536)}
    assert inf["tile_regs"] == 1
    x = M.uniform(17, a.n)
    got = _mixed_bits(plan, x, k, a.n)
    plan.close()
    wave = M.Plan.mixed(a, k, M.VALUE_F32)
    want = _mixed_bits(wave, x, k, a.n)
    wave.close()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("vt", [M.VALUE_F32, M.VALUE_BF16])
def test_mixed_register_tiles_empty_rows_vs_fp32_oracle(vt, gpu):
    """The register tile kernel on isolated vertices (empty rows: every
    entry is padding, the sum stays +0 as the FP32 chain's), bit for bit
    against the FP32 oracle on the stored values scaled by the exact 2^-e
    (FP32 values) and against the wavefront schedule (BF16 values).  A
    partition with an unused part id is refused, as by every PA1 plan."""
    k = 6
    base = M.Csr.laplacian(48, 40, 1, diag=4.0, off=-1.0)
    drop = {0, 77, 500, 1919}
    rows = [set() if i in drop else set(base.col[base.ptr[i]:base.ptr[i + 1]].tolist()) - drop
            for i in range(base.n)]
    ptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    col = np.concatenate([sorted(r) for r in rows]).astype(np.int32)
    val = np.where(col == np.repeat(np.arange(base.n), np.diff(ptr)), 4.0, -1.0)
    a = M.Csr(ptr, col, val)
    part, npart = M.partition_rcb(_grid2(48, 40), 20), 20
    with pytest.raises(M.MpkError) as e:
        M.Plan.mixed_tiles(a, (2 * part).astype(np.int32), 2 * npart, k, vt)
    assert e.value.code == M.EINVAL
    x = M.uniform(21, a.n)
    plan = M.Plan.mixed_tiles(a, part.astype(np.int32), npart, k, vt)
    assert plan.info()["tile_regs"] == 1
    e, _ = plan.mixed_scale()
    got = _mixed_bits(plan, x, k, a.n).reshape(k + 1, a.n)
    plan.close()
    if vt == M.VALUE_F32:
        sval = a.val.astype(np.float32) * np.float32(2.0 ** -e)
        want = O.spmm_f32(a.ptr, a.col, sval, x.astype(np.float32)[:, None], k)[:, :, 0]
    else:
        wave = M.Plan.mixed(a, k, vt)
        want = _mixed_bits(wave, x, k, a.n).reshape(k + 1, a.n)
        wave.close()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _grid2(nx, ny):
    i = np.arange(nx * ny)
    return np.stack([i % nx, i // nx, np.zeros_like(i)], axis=1).astype(np.int32)


def test_mixed_tiles_beyond_l2_bitwise_vs_fp32_oracle(gpu):
    """2048^2 9-point diffusion (151 MB of FP32 values, more than L2) on
    4096 PA1 tiles: the FP32 oracle's bits, and within 1e-6 of FP64 per
    power; BF16 values (log-normal coefficients, rounded) within the
    BF16 storage error of FP64."""
    a = M.Csr.diffusion(2048, 2048, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, dominance=0.01, seed=3)
    k = 8
    x = M.uniform(4, a.n)
    part = M.partition_rcb(_grid2(2048, 2048), 4096)
    plan = M.Plan.mixed_tiles(a, part, 4096, k, M.VALUE_F32)
    e, _ = plan.mixed_scale()
    got = _mixed_bits(plan, x, k, a.n).reshape(k + 1, a.n)
    plan.close()
    sval = a.val.astype(np.float32) * np.float32(2.0 ** -e)
    want = O.spmm_f32(a.ptr, a.col, sval, x.astype(np.float32)[:, None], k)[:, :, 0]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    want64 = O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA)
    v = got.astype(np.float64) * (2.0 ** (e * np.arange(k + 1)))[:, None]
    assert max(rel_errors(v, want64, a.n, k)) <= MIXED_TOL
    pb = M.Plan.mixed_tiles(a, part, 4096, k, M.VALUE_BF16)
    eb, inexact = pb.mixed_scale()
    gb = _mixed_bits(pb, x, k, a.n).reshape(k + 1, a.n)
    pb.close()
    assert inexact > 0  # log-normal coefficients are not BF16 numbers
    vb = gb.astype(np.float64) * (2.0 ** (eb * np.arange(k + 1)))[:, None]
    errs = rel_errors(vb, want64, a.n, k)
    assert max(errs) <= BF16_TOL, errs


BF16_TOL = 2e-2  # BF16 keeps 8 significand bits: about 2^-9 relative per value, k levels of it


def test_mixed_bf16_rounded_values_error_vs_fp64(gpu):
    """BF16 values on the log-normal diffusion matrix (values rounded):
    the error against the FP64 oracle per power stays within the BF16
    storage bound."""
    a = M.Csr.diffusion(512, 512, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, dominance=0.01, seed=3)
    k = 8
    x = M.uniform(4, a.n)
    v, e, inexact = run_mixed(a, k, M.VALUE_BF16, x)
    assert inexact > 0
    errs = rel_errors(v, O.mpk(a.ptr, a.col, a.val, x, k, O.MODE_FMA), a.n, k)
    assert max(errs) <= BF16_TOL, errs
