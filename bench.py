"""Benchmark: FP64 matrix powers kernel on one GB300 (or N replicas).

Workload (the GB300 configuration of the task): 3-D 7-point Laplacian on a
128^3 grid (n = 2,097,152, nnz = 14,581,760), CSR with int32 indices, the
reference's exec_mpk operator (row-normalised adjacency, A_ij = 1/deg(i)),
FP64 vectors, x ~ U[-1,1] (seed 1), k = 8 powers, 2048 METIS parts
(gpmetis -ufactor=100, through the METIS library bundled with the CUDA
toolkit; recursive coordinate bisection where the toolkit has none).  One
step = one MPK call computing [Ax, ..., A^8 x] into the level-major vv.

  value  : row-powers per second, k*n / (device time of one call), summed
           over ranks; device time from CUDA events around each call on the
           launching stream, L2 flushed (256 MiB write) before every call.
           Headline executor: the wavefront, FP64 FMA in CSR order -- the
           same bits as the reference's exec_mpk_xd built with FMA
           contraction (its result is checked bit for bit each run).
  e2e    : the same metric through mpkg_exec_host with pinned host buffers:
           x copied host->device and the k output vectors device->host
           inside the timed call.
  roofline: HBM bound; algorithmic bytes of one call
           B = 4*nnz + 4*(n+1) + 8*n*(k+1) (pattern once, x once, k outputs
           once) over the call's device time, against the measured copy
           bandwidth in MEASURED_PEAKS.json; plus the FP64 pipe bound (the
           call's nnz*k FMAs at the GPU's FP64 FMA rate, measured in this
           run), the one that binds plain FP64 on GB300.

--impl reference times the reference mpk2 exec_mpk_xd (compiled from its
own sources into oracle/_ref; the oracle's C restatement where absent) on
all host cores over the PA1 task lists of all 2048 parts (the lists
prep_mpk would build, from the oracle's bounded search; the reference prep
itself needs npart*n ints of skirt and npart*nlevel*n steps here).  That
process loads only the oracle's and the reference's libraries.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

K_LEVELS = 8
GRID = 128
NPART = 2048
SEED = 1
FLUSH_BYTES = 256 << 20


def box_partition(nx, ny, nz, npart):
    """Fallback partition without METIS: npart equal boxes (powers of two),
    splitting the longest side first (what recursive coordinate bisection
    gives on this grid)."""
    dims = [nx, ny, nz]
    cuts = [1, 1, 1]
    p = npart
    while p > 1:
        d = max(range(3), key=lambda t: (dims[t] / cuts[t], -t))
        cuts[d] *= 2
        p //= 2
    i = np.arange(nx * ny * nz)
    x, y, z = i % nx, (i // nx) % ny, i // (nx * ny)
    bx, by, bz = x // (nx // cuts[0]), y // (ny // cuts[1]), z // (nz // cuts[2])
    return ((bz * cuts[1] + by) * cuts[0] + bx).astype(np.int32)


def parts_kind():
    return "METIS k-way (gpmetis -ufactor=100)" if _metis() else "equal boxes (no METIS in this toolkit)"


_METIS = None


def _metis():
    global _METIS
    if _METIS is None:
        from oracle import oracle as O
        _METIS = O.metis_available()
    return _METIS


def workload():
    import mpk_gb300 as M
    a = M.Csr.laplacian(GRID, GRID, GRID, diag=6.0, off=-1.0)
    if _metis() and M.have_metis():
        part = M.partition_metis(a, NPART, ufactor=100)[0]
    else:
        part = box_partition(GRID, GRID, GRID, NPART)
    x = M.uniform(SEED, a.n)
    return a, part, x


def shared_config():
    """The workload, as both arms print it."""
    n = GRID ** 3
    return {"workload": "3-D 7-point Laplacian 128^3 (n=2,097,152, nnz=14,581,760), CSR int32, operator 1/deg "
                        "(the reference exec_mpk), FP64 vectors, x~U[-1,1] seed 1, k=8; PA1 over 2048 parts",
            "n": n, "nnz": 7 * n - 6 * GRID * GRID, "k": K_LEVELS, "parts": NPART, "partitioner": parts_kind(),
            "operator": "1/deg (mpk2/mpkexec.c:22-35)"}


def algorithmic_bytes(n, nnz, k, valued=False):
    """Matrix once (int32 columns, FP64 values when valued), row pointers,
    x once and k FP64 output levels written once."""
    return nnz * (12 if valued else 4) + 4 * (n + 1) + 8 * n * (k + 1)


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel):
    """DRAM bytes per launch of `kernel` on this workload from the committed
    ncu summary (profiles/ncu_traffic.json), or None."""
    p = os.path.join(HERE, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    e = d.get(kernel)
    return None if e is None else e.get("dram_bytes_per_launch")


class ClockSampler:
    """nvidia-smi clock/throttle samples (every 50 ms) from before the
    warm-up calls to the end of a tail of the same calls that follows the
    timed region (the timed steps alone last milliseconds)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.marks = {}

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def wait_first(self, timeout=5.0):
        """Until the first sample arrives (nvidia-smi takes a moment to start)."""
        t0 = time.perf_counter()
        while self.proc and not self.lines and time.perf_counter() - t0 < timeout:
            time.sleep(0.02)

    def mark(self, name):
        self.marks[name] = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def count(self):
        return len(self.lines)

    def summary(self):
        sm, mx, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lo = self.marks.get("warmup", 0)
        for line in self.lines[lo:]:
            f = [t.strip() for t in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        window = "warm-up calls, the timed steps and a tail of the same calls (about 1 s)"
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0, "window": window}
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None,
                "samples_in_timed_steps": self.marks.get("timed_end", 0) - self.marks.get("timed", 0),
                "window": window}


def dist_setup(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_device(plan, d_vv, steps, warmup, flush, stream):
    """Per-call CUDA-event times (ms) with an L2 flush before every call."""
    import torch
    for _ in range(warmup):
        flush.fill_(1.0)
        plan.exec_device(d_vv.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for e0, e1 in ev:
            flush.fill_(1.0)
            e0.record(stream)
            plan.exec_device(d_vv.data_ptr(), stream.cuda_stream)
            e1.record(stream)
    plan.sync(stream.cuda_stream)
    torch.cuda.synchronize()
    return [e0.elapsed_time(e1) for e0, e1 in ev]


class ReferenceRun:
    """The reference's exec_mpk_xd (oracle/_ref; else the oracle's
    restatement of the same loop) over the PA1 task lists of every part,
    all host threads.  Built from the oracle only: the matrix, x and the
    partition from its generators and METIS wrapper (or `part`), the task
    lists from its bounded search (orc_pa1_tasks, pinned to the reference
    prep's lists by tests/test_metis.py)."""

    def __init__(self, part=None):
        from oracle import oracle as O
        O.lib()
        ptr, col, _ = O.laplacian(GRID, GRID, GRID, 6.0, -1.0)
        n = len(ptr) - 1
        if part is None:
            part = O.metis_kway(ptr, col, NPART, 100) if _metis() else box_partition(GRID, GRID, GRID, NPART)
        t0 = time.perf_counter()
        off, idx = O.pa1_tasks(ptr, col, part, NPART, K_LEVELS)
        self.prep_s = time.perf_counter() - t0
        self.rows_eval = int(off[-1])
        self.n = n
        self.nth = os.cpu_count() or 1
        self.vv = np.zeros((K_LEVELS + 1) * n)
        self.vv[:n] = O.uniform(SEED, n)
        if O.ref_available():
            r = O.RefTaskLists(ptr, col, NPART, K_LEVELS, 0, off, idx)
            self.run = lambda: r.exec_xd(self.vv, self.nth)
            self.kind = "reference"
        else:
            self.run = lambda: O.exec_tasks_par(ptr, col, None, 0, NPART, off, idx, self.vv, O.MODE_FMA, self.nth)
            self.kind = "port"
        self._keep = (ptr, col, off, idx)

    def time(self, steps, warmup):
        for _ in range(warmup):
            self.run()
        ts = []
        for _ in range(steps):
            t0 = time.perf_counter()
            self.run()
            ts.append(time.perf_counter() - t0)
        return ts

    def sample(self):
        return (f"exec_mpk_xd over the PA1 task lists of all {NPART} parts ({self.rows_eval} row evaluations per "
                f"call, {self.rows_eval / (self.n * K_LEVELS):.2f}x the owned rows), {self.nth} OpenMP threads, "
                "1/deg operator, the whole call each step")


def time_mixed(plan, d_vv, steps, warmup, flush, stream):
    import torch
    for _ in range(warmup):
        flush.fill_(1.0)
        plan.exec_mixed_device(d_vv.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for e0, e1 in ev:
            flush.fill_(1.0)
            e0.record(stream)
            plan.exec_mixed_device(d_vv.data_ptr(), stream.cuda_stream)
            e1.record(stream)
    plan.sync(stream.cuda_stream)
    torch.cuda.synchronize()
    return [e0.elapsed_time(e1) for e0, e1 in ev]


def mixed_errors(v32, e, exact, n, k):
    v = v32.astype(np.float64).reshape(k + 1, n) * (2.0 ** (e * np.arange(k + 1)))[:, None]
    w = exact.reshape(k + 1, n)
    return [float(np.linalg.norm(v[l] - w[l]) / np.linalg.norm(w[l])) for l in range(1, k + 1)]


def bench_mixed(M, torch, a, x, k, exact, args, flush, stream):
    """The precision pattern: FP32 / BF16 values with an FP32 basis on this
    workload, and the 2048^2 9-point anisotropic diffusion (log-normal
    coefficients) in FP32 against the plain FP64 pipeline on the same
    matrix.  Errors are per power, relative, against FP64."""
    out = {}
    n = a.n
    for name, vt in (("f32", M.VALUE_F32), ("bf16", M.VALUE_BF16)):
        plan = M.Plan.mixed(a, k, vt)
        e, inexact = plan.mixed_scale()
        d = torch.zeros((k + 1) * n, dtype=torch.float32, device="cuda")
        d[:n] = torch.from_numpy(x.astype(np.float32)).cuda()
        t = statistics.mean(time_mixed(plan, d, min(args.steps, 100), args.warmup, flush, stream))
        errs = mixed_errors(d.cpu().numpy(), e, exact, n, k)
        out[f"cube128_{name}"] = {"ms_per_step": t, "value": k * n / (t * 1e-3) / 1e9, "rel_err_per_power": errs,
                                  "values_rounded": inexact,
                                  "bytes_per_call": a.nnz * (4 + (4 if vt == M.VALUE_F32 else 2)) + 4 * (n + 1) +
                                  4 * n * (k + 1)}
        plan.close()
    # config 3: 2048^2 9-point anisotropic diffusion, log-normal(0,1) edges
    b = M.Csr.diffusion(2048, 2048, sigma=1.0, wx=1.0, wy=0.1, wdiag=0.5, dominance=0.01, seed=3)
    xb = M.uniform(3, b.n)
    fp64 = {}
    for ex, mkp in (("spmv_fma", lambda: M.Plan.spmv(b, k)), ("wave_fma", lambda: M.Plan.wave(b, k)),
                    ("pipe_fma", lambda: M.Plan.pipe(b, k))):
        p64 = mkp()
        d64 = torch.zeros((k + 1) * b.n, dtype=torch.float64, device="cuda")
        d64[:b.n] = torch.from_numpy(xb).cuda()
        fp64[ex] = statistics.mean(time_device(p64, d64, min(args.steps, 50), args.warmup, flush, stream))
        ex64 = d64.cpu().numpy()  # all three are bit-identical (FP64 FMA in CSR order)
        p64.close()
        del d64
    best64 = min(fp64, key=fp64.get)
    t64 = fp64[best64]
    peak, _ = peaks()
    B32 = b.nnz * 8 + 4 * (b.n + 1) + 4 * b.n * (k + 1)
    res = {"n": b.n, "nnz": b.nnz, "fp64_ms": fp64, "fp64_best": best64, "algorithmic_bytes_f32": B32,
           "schedules": "wave: the wavefront (every level streams the matrix); tiles: PA1 tiles (RCB parts, part "
                        "size chosen by the plan's autotuner among 384..1536 rows) + 8-deep skirts, each tile's rows "
                        "held on chip for all levels"}
    i = np.arange(b.n)
    coords = np.stack([i % 2048, i // 2048, np.zeros_like(i)], axis=1).astype(np.int32)
    bits = {}
    for name, vt in (("f32", M.VALUE_F32), ("bf16", M.VALUE_BF16)):
        for sched in ("wave", "tiles"):
            p32 = M.Plan.mixed(b, k, vt) if sched == "wave" else M.Plan.mixed_tiles_tuned(b, coords, k, vt)
            e, inexact = p32.mixed_scale()
            d32 = torch.zeros((k + 1) * b.n, dtype=torch.float32, device="cuda")
            d32[:b.n] = torch.from_numpy(xb.astype(np.float32)).cuda()
            t32 = statistics.mean(time_mixed(p32, d32, min(args.steps, 100), args.warmup, flush, stream))
            got = d32.cpu().numpy()
            errs = mixed_errors(got, e, ex64, b.n, k)
            bits[(name, sched)] = got.view(np.uint32)
            info = p32.info()
            res[f"{name}_{sched}"] = {
                "ms_per_step": t32, "speedup_vs_best_fp64": t64 / t32, "rel_err_per_power": errs,
                "values_rounded": inexact, "value": k * b.n / (t32 * 1e-3) / 1e9,
                "rows_computed_per_output_row": info["rows_computed"] / (b.n * k),
                "achieved_gbs": B32 / (t32 * 1e-3) / 1e9, "frac_hbm": B32 / (t32 * 1e-3) / 1e9 / peak,
                "kernel": (("tiles_reg_kernel" if info["tile_regs"] else "tiles_mix_kernel") if sched == "tiles"
                           else "wave_mix_kernel")}
            if sched == "tiles":
                res[f"{name}_{sched}"].update(parts=info["npart"], part_sizes_timed=info["tune_candidates"],
                                              tune_ms=info["tune_ms"])
            p32.close()
            del d32
        res[f"{name}_tiles"]["bit_equal_wave"] = bool(np.array_equal(bits[(name, "wave")], bits[(name, "tiles")]))
    out["diffusion2048_9pt"] = res
    return out


def bench_batch(M, torch, args, flush, stream):
    """Batching workload: 256 matrices (n log-uniform in [1e3, 2e5], half
    random 2-D/3-D stencils, half random banded), 16 right-hand sides, FP32,
    k=6, one persistent graph-replayed launch, autotuned."""
    import scipy.sparse as sp
    k, nrhs = 6, 16
    mats = M.batch_workload(args.batch_mats, seed=0)
    N = sum(m.n for m in mats)
    nnz = sum(m.nnz for m in mats)
    t0 = time.perf_counter()
    mode = {"tune": True, "default": False, "staged": M.BATCH_STAGED, "staged2": M.BATCH_STAGED2,
            "staged4": M.BATCH_STAGED4}[args.batch_mode]
    plan = M.Plan.batch(mats, nrhs, k, tune=mode)
    plan_s = time.perf_counter() - t0
    X = M.uniform(1, N * nrhs).astype(np.float32)
    d = torch.zeros((k + 1) * N * nrhs, dtype=torch.float32, device="cuda")
    d[:N * nrhs] = torch.from_numpy(X).cuda()
    torch.cuda.synchronize()
    for _ in range(3):
        plan.exec_batch_device(d.data_ptr(), stream.cuda_stream)
    plan.sync(stream.cuda_stream)
    times = []
    for _ in range(max(3, min(args.steps, 20))):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.exec_batch_device(d.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        plan.sync(stream.cuda_stream)
        times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    vb = d.view(k + 1, N, nrhs)
    errs = [0.0] * k
    nm = len(mats)
    sample = sorted({j % nm for j in (0, 1, 2, 3, nm // 2, nm // 2 + 1, nm - 2, nm - 1)})
    row0 = np.concatenate([[0], np.cumsum([m.n for m in mats])])
    for j in sample:  # error of the FP32 form against FP64, per power
        m = mats[j]
        A = sp.csr_matrix((m.val, m.col, m.ptr), shape=(m.n, m.n))
        v = X.reshape(N, nrhs)[row0[j]:row0[j + 1]].astype(np.float64)
        for l in range(1, k + 1):
            v = A @ v
            got = vb[l, row0[j]:row0[j + 1]].double().cpu().numpy()
            errs[l - 1] = max(errs[l - 1], float(np.linalg.norm(got - v) / np.linalg.norm(v)))
    B = nnz * 8 + 4 * (N + 256) + 4 * N * nrhs * (1 + k)
    peak, _ = peaks()
    info = plan.batch_info()
    plan.close()
    return {"workload": f"{nm} matrices, n log-uniform [1e3, 2e5] (half random 2-D/3-D stencils, half random banded "
                        "bw 64, 5-30 nnz/row), 16 RHS FP32, k=6", "rows": N, "nnz": nnz, "ms_per_step": ms,
            "value": N * nrhs * k / (ms * 1e-3) / 1e9, "unit": "G row-RHS powers/s",
            "algorithmic_bytes": B, "achieved_gbs": B / (ms * 1e-3) / 1e9, "frac_hbm": B / (ms * 1e-3) / 1e9 / peak,
            "rel_err_per_power_vs_fp64": errs, "error_sample": f"{len(sample)} of the {nm} matrices, all 16 RHS",
            "plan_s": plan_s, "mode": args.batch_mode,
            "tuned": {kk: info[kk] for kk in ("lanes_per_row", "vector_width", "group_bytes", "ngroup", "grid",
                                              "threads", "staged", "window_bytes", "graph", "candidates",
                                              "tune_ms")},
            "gpu_launches_per_step": 1}


def bench_prep(M, a, part):
    """PA1 tile metadata of the headline workload (2048 RCB parts, k=8):
    the GPU build next to the host build (same bytes)."""
    g = a.pattern()
    out = {"workload": "128^3 7-point, 2048 RCB parts, k=8: balls within k arcs, sorted, sliced-ELL local slots"}
    M.tile_prep(g, part, NPART, K_LEVELS, on_gpu=True)  # warm-up (kernel load)
    t0 = time.perf_counter()
    dev = M.tile_prep(g, part, NPART, K_LEVELS, on_gpu=True)
    out["gpu_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    host = M.tile_prep(g, part, NPART, K_LEVELS, on_gpu=False)
    out["host_s"] = time.perf_counter() - t0
    out["built_on_gpu"] = dev["built_on_gpu"]
    out["identical"] = all(np.array_equal(dev[k], host[k]) for k in
                           ("slot_off", "shell", "slot_vert", "slice_off", "ell_off", "ell_col", "ell_width"))
    out["slots"] = int(len(host["slot_vert"]))
    out["local_columns"] = int(len(host["ell_col"]))
    return out


def bench_sstep(M):
    """s-step CG (s=8) on the 96^3 7-point variable-coefficient diffusion
    matrix (log-normal sigma=1), b ~ U[-1,1], tol 1e-8: monomial,
    Lanczos-shift and learned-shift bases next to standard FP64 CG."""
    from mpk_gb300 import shifts as S
    a = M.Csr.diffusion(96, 96, 96, sigma=1.0, dominance=0.01, seed=5)
    b = M.uniform(7, a.n)
    out = {"workload": "96^3 7-point diffusion, log-normal(sigma=1) coefficients, dominance 0.01, n=884736, "
                       "s=8, tol 1e-8 (true residual)"}
    _, out["cg_fp64"] = M.cg(a, b)
    _, out["monomial"] = M.sstep_cg(a, b, 8)
    t0 = time.perf_counter()
    sh = S.from_lanczos(a, 8)
    lan_ms = (time.perf_counter() - t0) * 1e3
    _, out["lanczos_shifts"] = M.sstep_cg(a, b, 8, shifts=sh)
    out["lanczos_shifts"]["shift_ms"] = lan_ms
    wpath = os.path.join(HERE, "mpk_gb300", "shift_mlp.npz")
    if os.path.exists(wpath):
        from mpk_gb300.train_shifts import load
        mlp, src = load(wpath), "mpk_gb300/shift_mlp.npz (trained on 2000 synthetic matrices)"
    else:
        X, T = S.training_set(400, seed=11)
        mlp, src = S.train(X, T, epochs=200)[0], "trained here on 400 synthetic matrices"
    t0 = time.perf_counter()
    sh = S.predict(mlp, a)
    pred_ms = (time.perf_counter() - t0) * 1e3
    _, out["learned_shifts"] = M.sstep_cg(a, b, 8, shifts=sh)
    out["learned_shifts"]["shift_ms"] = pred_ms
    out["learned_shifts"]["model"] = src
    # the same solve with the Gram matrix summed in double-float on the FP32 pipes
    _, out["learned_shifts_df64_gram"] = M.sstep_cg(a, b, 8, shifts=sh, gram=M.GRAM_DF64)
    # the same solve with the basis built by one matrix powers launch per
    # outer iteration (the default builds it with one launch per step)
    _, out["learned_shifts_mpk_basis"] = M.sstep_cg(a, b, 8, shifts=sh, basis=M.SSTEP_BASIS_MPK)
    out["basis"] = "one FP32 SpMV launch per Newton step, both blocks per launch (mpk_basis: one wavefront launch)"
    out["gram"] = "FP64 FMAs over the exact FP64 products of the FP32 basis (df64: double-float sums)"
    # the same solve with the outer loop driven from the host (one graph
    # launch and synchronisation per outer iteration)
    _, out["learned_shifts_host_loop"] = M.sstep_cg(a, b, 8, shifts=sh, loop=M.SSTEP_HOST_LOOP)
    out["loop"] = ("device-side: the whole solve is one graph launch (conditional WHILE node); "
                   "loop_ms = the iterations alone, ms = the whole call incl. matrix upload and setup")
    return out


def time_headline(plan, d_vv, steps, warmup, flush, stream, clk, world):
    """W warm-up calls, then exactly K timed calls (CUDA events on the
    launching stream around each call, an L2 flush before each), bracketed
    by a barrier and a device synchronisation; then untimed calls until
    about a second has passed, so that the clock sampler sees the load."""
    import torch
    clk.wait_first()
    t_start = time.perf_counter()
    clk.mark("warmup")
    for _ in range(warmup):
        flush.fill_(1.0)
        plan.exec_device(d_vv.data_ptr(), stream.cuda_stream)
    plan.sync(stream.cuda_stream)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clk.mark("timed")
    w0 = time.perf_counter()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for e0, e1 in ev:
            flush.fill_(1.0)
            e0.record(stream)
            plan.exec_device(d_vv.data_ptr(), stream.cuda_stream)
            e1.record(stream)
    plan.sync(stream.cuda_stream)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    clk.mark("timed_end")
    times = [e0.elapsed_time(e1) for e0, e1 in ev]
    tail = 0
    while time.perf_counter() - t_start < 1.2 or (clk.count() - clk.marks["warmup"] < 10 and tail < 20000):
        with torch.cuda.stream(stream):
            for _ in range(20):
                flush.fill_(1.0)
                plan.exec_device(d_vv.data_ptr(), stream.cuda_stream)
        plan.sync(stream.cuda_stream)
        tail += 20
        if time.perf_counter() - t_start > 10:
            break
    return times, wall, tail


def fp64_rate():
    import mpk_gb300 as M
    try:
        return M.fp64_fma_rate()
    except M.MpkError:
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--exec", default="wave", choices=["pipe", "wave", "tiles", "spmv", "tasks"])
    ap.add_argument("--arith", default="fma", choices=["fma", "separate", "df64", "fixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="time only the selected executor")
    ap.add_argument("--sections", default="variants,mixed,batched,sstep,prep",
                    help="comma list of the extra sections to run (variants, mixed, batched, sstep, prep; 'none')")
    ap.add_argument("--batch-mode", default="tune", choices=["tune", "default", "staged", "staged2", "staged4"],
                    help="batched section's kernel configuration: autotuned (the workload) or one fixed "
                         "configuration (for a profiler capture)")
    ap.add_argument("--batch-mats", type=int, default=256,
                    help="matrices of the batched section (256 = the workload; fewer for a profiler capture)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    sections = set() if args.no_variants else {t.strip() for t in args.sections.split(",")} - {"none", ""}
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    k = K_LEVELS

    if args.impl == "reference":
        # the reference arm: this process loads only oracle/ and the
        # reference's own code (no product library, no GPU)
        if rank != 0:
            return
        ref = ReferenceRun()
        ts = ref.time(args.steps, args.warmup)
        sec = statistics.mean(ts)
        value = k * ref.n / sec / 1e9
        line = {"impl": "reference", "metric": "MPK powers/sec (FP64, k*n output rows per second)",
                "value": value, "unit": "Grow-powers/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": sec * 1e3, "ms_min": min(ts) * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": shared_config(),
                "cpu_baseline": {"value": value, "unit": "Grow-powers/s", "cores": ref.nth, "kind": ref.kind,
                                 "sample": ref.sample(), "task_list_build_s": ref.prep_s},
                "e2e": {"value": value, "unit": "Grow-powers/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    dist_setup(args)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import mpk_gb300 as M
    torch.cuda.set_device(local)
    a, part, x = workload()
    n, nnz = a.n, a.nnz
    ARITHS = {"fma": M.ARITH_FMA, "separate": M.ARITH_SEPARATE, "df64": M.ARITH_DF64, "fixed": M.ARITH_FIXED}
    arith = ARITHS[args.arith]
    g = a.pattern()  # the 1/deg operator of the reference's exec_mpk

    def mk(ex, ar, mat=None):
        mat = g if mat is None else mat
        return {"pipe": lambda: M.Plan.pipe(mat, k, arith=ar),
                "wave": lambda: M.Plan.wave(mat, k, arith=ar),
                "tiles": lambda: M.Plan.pa1(mat, part, NPART, k, exec=M.EXEC_TILES, arith=ar),
                "tasks": lambda: M.Plan.pa1(mat, part, NPART, k, exec=M.EXEC_TASKS, arith=ar),
                "spmv": lambda: M.Plan.spmv(mat, k, arith=ar)}[ex]()
    plan = mk(args.exec, arith)
    info = plan.info()
    stream = torch.cuda.Stream()
    d_vv = torch.zeros((k + 1) * n, dtype=torch.float64, device="cuda")
    d_vv[:n] = torch.from_numpy(x).cuda()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    with ClockSampler(local) as clk:
        times, wall, tail = time_headline(plan, d_vv, args.steps, args.warmup, flush, stream, clk, world)
    ms = statistics.mean(times)
    ms_max = reduce_max(world, ms)
    value = world * k * n / (ms_max * 1e-3) / 1e9
    got = d_vv.cpu().numpy()

    # the FP64 chain (k chained SpMVs in FP64 FMA, CSR order: the bits of the
    # reference's exec_mpk_xd built with FMA contraction) and the
    # headline's error against it
    def relerr(v, ref):
        return max(float(np.linalg.norm(v[l * n:(l + 1) * n] - ref[l * n:(l + 1) * n]) /
                         np.linalg.norm(ref[l * n:(l + 1) * n])) for l in range(1, k + 1))

    rp = mk("spmv", M.ARITH_FMA)
    ref64 = np.zeros((k + 1) * n)
    ref64[:n] = x
    rp.exec_host(ref64)
    rp.close()
    headline_err = relerr(got, ref64)
    bit_equal = bool(got.tobytes() == ref64.tobytes())

    # the other executors and arithmetic forms on the same workload
    variants = {}
    if "variants" in sections:
        runs = [(ex, ar, None) for ex, ar in (("spmv", "fma"), ("wave", "fma"), ("spmv", "df64"), ("wave", "df64"),
                                              ("spmv", "fixed"), ("wave", "fixed"), ("pipe", "fma"), ("pipe", "df64"),
                                              ("tiles", "fma"), ("tiles", "df64"), ("tasks", "fma"))]
        runs += [("spmv", "fma", "valued"), ("wave", "fma", "valued"), ("wave", "df64", "valued")]
        ref_val = None
        for ex, ar, op in runs:
            if ex == args.exec and ar == args.arith and op is None:
                continue
            vp = mk(ex, ARITHS[ar], a if op else None)
            d2 = torch.zeros_like(d_vv)
            d2[:n] = d_vv[:n]
            t = statistics.mean(time_device(vp, d2, min(args.steps, 50), args.warmup, flush, stream))
            v2 = d2.cpu().numpy()
            if op and ref_val is None:
                ref_val = v2  # spmv fma valued runs first among the valued
            rv = ref_val if op else ref64
            variants[f"{ex}_{ar}" + ("_valued" if op else "")] = {
                "ms_per_step": t, "value": k * n / (t * 1e-3) / 1e9, "rel_err_max_vs_fp64": relerr(v2, rv),
                "bit_equal_fp64_fma_chain": bool(v2.tobytes() == rv.tobytes()),
                "algorithmic_bytes": algorithmic_bytes(n, nnz, k, valued=bool(op)),
                "rows_computed": vp.info()["rows_computed"]}
            vp.close()
            del d2

    # end to end through the host API, pinned host buffers
    hv = torch.zeros((k + 1) * n, dtype=torch.float64).pin_memory()
    hv[:n] = torch.from_numpy(x)
    hnp = hv.numpy()
    for _ in range(args.warmup):
        plan.exec_host(hnp)
    e2e_steps = max(3, min(args.steps, 50))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.exec_host(hnp)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = reduce_max(world, e2e_s)
    same = bool(np.array_equal(got, hnp))

    mixed = {}
    if "mixed" in sections:  # the mixed form runs the valued operator; its FP64 reference:
        vp = M.Plan.spmv(a, k, arith=M.ARITH_FMA)
        exact_val = np.zeros((k + 1) * n)
        exact_val[:n] = x
        vp.exec_host(exact_val)
        vp.close()
        mixed = bench_mixed(M, torch, a, x, k, exact_val, args, flush, stream)
    batched = bench_batch(M, torch, args, flush, stream) if "batched" in sections else {}
    sstep = bench_sstep(M) if "sstep" in sections else {}
    prep = bench_prep(M, a, part) if "prep" in sections else {}

    peak, peak_kind = peaks()
    B = algorithmic_bytes(n, nnz, k, valued=False)
    achieved = B / (ms * 1e-3) / 1e9
    kname = {"pipe": "flow_kernel", "wave": "wave_kernel", "tiles": "tiles_kernel", "tasks": "tasks_kernel",
             "spmv": "spmv_level_kernel"}[args.exec]
    if args.arith == "df64":
        kname = {"pipe": "flow_df_kernel", "wave": "wave_df_kernel", "tiles": "tiles_df_kernel"}.get(args.exec, kname)
    if args.arith == "fixed":
        kname = "wave_fix_kernel"
    traffic = profile_traffic(kname)
    rows = info["rows_computed"]
    fmas = nnz * k * (rows / (n * k))
    rate = fp64_rate()
    fp64 = None
    if args.arith in ("fma", "separate") and rate:
        fp64 = {"fma_per_call": fmas, "peak_fma_per_s": rate, "peak_source": "measured in this run "
                "(mpkg_fp64_fma_rate: independent FMA chains, best of five launches)",
                "bound_us": fmas / rate * 1e6, "achieved_fma_per_s": fmas / (ms * 1e-3),
                "frac": fmas / (ms * 1e-3) / rate}
    base_ms = variants.get("spmv_fma", {}).get("ms_per_step")
    # the MPK against k separate SpMV launches in the same arithmetic
    same_arith = {}
    for ar in ("fma", "df64", "fixed"):
        t_sp = variants.get(f"spmv_{ar}", {}).get("ms_per_step")
        t_mpk = ms if (args.exec == "wave" and args.arith == ar) else variants.get(f"wave_{ar}", {}).get("ms_per_step")
        if t_sp and t_mpk:
            same_arith[ar] = {"k_spmv_ms": t_sp, "mpk_wave_ms": t_mpk, "speedup": t_sp / t_mpk}
    cfg = dict(shared_config())
    line = {"metric": "MPK powers/sec (FP64, k*n output rows per second)", "value": value,
            "unit": "Grow-powers/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"df64": "df64", "fma": "f64", "separate": "f64", "fixed": "i64"}[args.arith], "data": "synthetic",
            "config": cfg, "executor": args.exec, "arith": args.arith,
            "l2": "flushed before every call (256 MiB write); per-call CUDA events",
            "parallelism": f"replicas{world}",
            "rel_err_max_vs_fp64": headline_err, "bit_equal_fp64_fma_chain": bit_equal, "tolerance": 1e-13,
            "e2e": {"value": world * k * n / e2e_s / 1e9, "unit": "Grow-powers/s",
                    "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n * k},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "algorithmic_bytes": B, "kernel": kname,
                         "traffic_note": "ncu dram bytes of one launch (profiles/ncu_traffic.json); output lines "
                                         "still dirty in L2 when the kernel ends are written back after it",
                         "fp64_pipe": fp64},
            "k_spmv_ms": base_ms, "speedup_vs_k_spmv": (base_ms / ms) if base_ms else None,
            "speedup_vs_k_spmv_same_arith": same_arith,
            "variants": variants, "mixed": mixed, "batched": batched, "sstep": sstep, "prep": prep,
            "gpu_launches": info["launches"] * args.steps,
            "clocks": clk.summary(), "wall_s_timed_region": wall, "tail_calls_for_clock_samples": tail,
            "host_device_agree": same,
            "plan": {kk: info[kk] for kk in ("rows_computed", "device_bytes", "pipe_reach", "pipe_grid",
                                            "tiles_in_smem", "max_tile_slots")}}
    if rank == 0 and not args.no_cpu_baseline:
        ref = ReferenceRun(part)
        ts = ref.time(5, 1)
        line["cpu_baseline"] = {"value": k * n / min(ts) / 1e9, "unit": "Grow-powers/s", "cores": ref.nth,
                                "kind": ref.kind, "sample": ref.sample() + ", best of 5 (as mpk2/mpktest.c:121-133)"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
