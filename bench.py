"""Benchmark: SpTRSV throughput (GB/s vs the HBM roofline) on one GB300,
plus time-to-1e-10 of IC0-PCG and of GMRES(30)+ILU0 (FP32 vs FP64
preconditioner).

Default workload (one "step" = one forward triangular solve):
  L = IC0 factor of the 3D 7-point Laplacian on a 64^3 grid + 1e-2 I
  (natural ordering, n = 262,144, nnz(L) = 1,036,288, 190 wavefront
  levels), 64 right-hand sides ~ N(0,1) in FP64, row-major n x 64.
The factor is computed on the GPU (the library's IC0).  Inputs are seeded
synthetic data of the named shape.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbsym|reference]

Under torchrun each rank solves its own replica (one system's rows do not
shard across GPUs: "replicas"); value is the sum over ranks of the per-rank
throughput measured over the max-over-ranks time.  With --shard rhs the
right-hand-side columns of one solve are split over the ranks instead,
each rank holding the factor (strong scaling, no collective on the data
path).

--impl reference times the reference's CPU executor for the same workload
on the host cores: the oracle's C restatement of sptrsv_csr_levelset
(one OpenMP parallel-for per level) and of sptrsv_csr with the columns
spread over threads; the faster is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sptrsv_gbs"
UNIT = "GB/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbsym", choices=["gbsym", "reference"])
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--rhs", type=int, default=64)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--extras-only", action="store_true")
    ap.add_argument("--supernodal-grid", type=int, default=0,
                    help="run only the supernodal-solve extra, on a G^3 grid's factor (profiling runs)")
    ap.add_argument("--workload", default="c2", choices=["c2", "c4"],
                    help="c2: one IC0 forward solve with --rhs right-hand sides (default); c4: the 512-system "
                         "batch, sharded over the ranks")
    ap.add_argument("--dtype", default="f64", choices=["f64", "f32"], help="c4 workload: factor and vectors")
    ap.add_argument("--shard", default="replicas", choices=["replicas", "rhs"],
                    help="c2 workload under torchrun: replicas (each rank solves all columns) or rhs "
                         "(the columns split over the ranks, each rank holding the whole factor)")
    ap.add_argument("--exec", default="auto",
                    choices=["auto", "levelset", "syncfree", "oneblock", "persistent", "cluster", "partitioned"],
                    help="force one executor instead of autotuning (profiling runs)")
    return ap.parse_args()


def algorithmic_bytes(nnz_l, n, k, vbytes=8, sbytes=8):
    """(V+4) nnz(L) + 4 (n+1) + 2 S k n: every stored value and index read
    once, the right-hand sides read once and the solution written once."""
    return (vbytes + 4) * nnz_l + 4 * (n + 1) + 2 * sbytes * k * n


_FP64_RATES = None


def fp64_rates():
    """(update, fma) FP64 throughput of this GPU in G op/s, measured once per
    process by the library's probe (gbsym_fp64_rates): a stream of exact
    updates (a rounded product and a rounded difference, both DFMAs) and a
    stream of general three-operand DFMAs.  Both run on the same FP64 pipe;
    the FMA stream reaches its peak (two DFMAs per SM per clock on GB300,
    about 626 G op/s), the update stream about 0.84 of it."""
    global _FP64_RATES
    if _FP64_RATES is None:
        import ctypes as C
        from sympiler_gb300._lib import check, lib
        u, f = C.c_double(), C.c_double()
        check(lib().gbsym_fp64_rates(C.byref(u), C.byref(f), None), "gbsym_fp64_rates")
        _FP64_RATES = (u.value, f.value)
    return _FP64_RATES


def fp64_peak():
    """The FP64 pipe's measured peak in G op/s: the faster of the probe's two
    DFMA streams (every FP64 operation of the exact paths is one DFMA)."""
    return max(fp64_rates())


def fp64_ops_exact(nnz_off, n, k):
    """FP64 operations of one exact solve: a multiply and a subtract per
    stored off-diagonal, three for the correctly rounded division."""
    return k * (2 * nnz_off + 3 * n)


def fp64_floor_s(nnz_off, n, k):
    """FP64-pipe time floor of one exact solve: its DFMAs (fp64_ops_exact)
    at the pipe's measured peak."""
    return fp64_ops_exact(nnz_off, n, k) / (fp64_peak() * 1e9)


def fp64_roofline(nnz_off, n, k, t):
    """FP64 roofline of one exact solve taking t seconds."""
    ops = fp64_ops_exact(nnz_off, n, k)
    floor = fp64_floor_s(nnz_off, n, k)
    u, f = fp64_rates()
    return {"bound": "fp64 pipe", "achieved": ops / t / 1e9, "peak": fp64_peak(),
            "unit": "G FP64 op/s", "frac": floor / t, "ops_per_solve": ops, "floor_ms": floor * 1e3,
            "rates_gops": {"update_stream": u, "fma_stream": f},
            "peak_source": "measured live (gbsym_fp64_rates): the faster of its two DFMA streams"}


def config(grid, k):
    return {"workload": "C2 IC0 factor of 3D 7-pt Laplacian %d^3 + 1e-2 I, forward SpTRSV, %d RHS FP64"
                        % (grid, k),
            "n": grid ** 3, "rhs": k, "ordering": "natural", "layout": "row-major n x k",
            "l2": "inputs 2*n*k*8 B; 256 MB L2 flush write between timed steps",
            "parallelism": "replicas"}


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference_c4(args):
    """The reference arm of the batched workload: every system's forward
    solve with the oracle's serial sptrsv_csr per right-hand side (the
    reference executor's arithmetic), systems spread over all host threads."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    from sympiler_gb300 import matgen as mg
    orc = oracle.orc()
    k, dt = 8, args.dtype
    systems = mg.batch_systems_upper(512, np.random.default_rng(44))
    Ls = []
    for n, p, i, x in systems:
        f, ok = orc.spic0_csr(n, p, i, x)
        Ls.append(mg.transpose(mg.CSR(n, p, i, f)))
    N = sum(L.n for L in Ls)
    nnz = sum(L.nnz for L in Ls)
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(45)
    Bs = [rng.standard_normal((k, L.n)) for L in Ls]
    if dt == "f32":
        Bs = [B.astype(np.float32) for B in Bs]
        L32 = [L.x.astype(np.float32) for L in Ls]
    pool = ThreadPoolExecutor(max_workers=cores)

    def one(q):
        L, X = Ls[q], Bs[q].copy()
        if dt == "f64":
            orc.sptrsv_csr_mrhs(L.n, *L.astuple(), X, k, 1)
        else:
            for c in range(k):
                orc.sptrsv_csr_f32(L.n, L.p, L.i, L32[q], X[c])
        return X

    order = sorted(range(len(Ls)), key=lambda q: -Ls[q].nnz)  # largest first
    for _ in range(max(1, min(args.warmup, 2))):
        list(pool.map(one, order))
    ts = []
    for _ in range(max(1, min(args.steps, 5))):
        t0 = time.perf_counter()
        list(pool.map(one, order))
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    vb = 8 if dt == "f64" else 4
    value = algorithmic_bytes(nnz, N, k, vb, vb) / t / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": dt, "data": "synthetic",
            "config": c4_config(dt, k, 512, 1),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "cpu": host_cpu(), "kind": "port",
                             "sample": "all 512 systems x %d RHS per step, serial solves spread over %d host "
                                       "threads; median of %d" % (k, cores, len(ts))},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference(args):
    world, rank, _ = dist_init()
    if rank != 0:
        return
    if args.workload == "c4":
        run_reference_c4(args)
        return
    import oracle
    from sympiler_gb300 import matgen as mg
    orc = oracle.orc()
    # the reference's own executors where they were compiled from its
    # sources (this needs the reference tree at build time), else the port
    ref = oracle.ref()
    A = mg.lap3d(args.grid, 1e-2)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    L = mg.transpose(mg.CSR(U.n, U.p, U.i, f))
    nl, lp, ls = orc.build_levelset_csr(L.n, L.p, L.i)
    k = args.rhs
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(0)
    sample_cols = max(1, min(k, 8))
    B = rng.standard_normal((sample_cols, L.n))
    Bk = rng.standard_normal((k, L.n))  # every column for the column-parallel form

    from concurrent.futures import ThreadPoolExecutor
    pool = ThreadPoolExecutor(max_workers=cores)

    def set_omp_threads(t):
        import ctypes
        try:
            ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(t))
        except OSError:
            pass

    def t_levelset(threads):
        X = B.copy()
        t0 = time.perf_counter()
        if ref is not None:  # one OpenMP level-set solve per column, as the reference runs it
            set_omp_threads(threads)
            for c in range(sample_cols):
                ref.sptrsv_csr_levelset(L.n, *L.astuple(), X[c], nl, lp, ls)
        else:
            orc.sptrsv_csr_levelset_mrhs(L.n, *L.astuple(), X, sample_cols, nl, lp, ls, threads)
        return (time.perf_counter() - t0) * k / sample_cols

    def t_colpar():
        # all k columns, serial solves spread over the host threads (the
        # threads share the memory system, as they would in use)
        X = Bk.copy()
        t0 = time.perf_counter()
        if ref is not None:  # serial sptrsv_csr per column, columns over host threads
            list(pool.map(lambda c: ref.sptrsv_csr(L.n, *L.astuple(), X[c]), range(k)))
        else:
            orc.sptrsv_csr_mrhs(L.n, *L.astuple(), X, k, cores)
        return time.perf_counter() - t0

    # the level-set executor at the best thread count of {1, 8, 16, 32, all}
    sweep = {}
    for t in sorted({c for c in (1, 8, 16, 32, cores) if c <= cores}):
        t_levelset(t)
        sweep[t] = statistics.median(t_levelset(t) for _ in range(3))
    best_t = min(sweep, key=sweep.get)
    for _ in range(max(1, min(args.warmup, 2))):
        t_levelset(best_t)
        t_colpar()
    ts_l, ts_c = [], []
    for _ in range(args.steps):
        ts_l.append(t_levelset(best_t))
        ts_c.append(t_colpar())
    set_omp_threads(cores)
    byt = algorithmic_bytes(L.nnz, L.n, k)
    tl, tc = statistics.median(ts_l), statistics.median(ts_c)
    best, kind = (tl, "sptrsv_csr_levelset, OpenMP per level, %d threads" % best_t) if tl <= tc else \
        (tc, "sptrsv_csr per column, columns over %s threads" % ("host" if ref is not None else "OpenMP"))
    value = byt / best / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": best * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config(args.grid, k),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "cpu": host_cpu(),
                             "kind": "reference" if ref is not None else "port",
                             "sample": "level set: %d of %d RHS columns per step (columns run one after "
                                       "another), scaled to %d; column-parallel: all %d columns; best of: "
                                       "levelset %.1f ms, column-parallel %.1f ms per %d-RHS solve; used: %s; "
                                       "levelset ms by threads: %s"
                                       % (sample_cols, k, k, k, tl * 1e3, tc * 1e3, k, kind,
                                          ", ".join("%d: %.1f" % (t, v * 1e3) for t, v in sorted(sweep.items())))},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def host_cpu():
    """The host CPU as /proc/cpuinfo names it: the model name where there is
    one (x86), else the architecture with the Arm implementer and part."""
    import platform
    fields = {}
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if ":" in line:
                    key, val = (t.strip() for t in line.split(":", 1))
                    fields.setdefault(key, val)
    except OSError:
        pass
    if "model name" in fields:
        return fields["model name"]
    parts = [platform.machine()]
    for key in ("CPU implementer", "CPU part"):
        if key in fields:
            parts.append("%s %s" % (key.lower(), fields[key]))
    return ", ".join(parts)


def cpu_baseline_sample(L, k, nl, lp, ls):
    """Bounded CPU sample of the same workload (oracle port, all host threads)."""
    import oracle
    orc = oracle.orc()
    cores = os.cpu_count() or 1
    cols = max(1, min(k, 4))
    B = np.random.default_rng(0).standard_normal((cols, L.n))
    X = B.copy()
    orc.sptrsv_csr_levelset_mrhs(L.n, *L.astuple(), X, cols, nl, lp, ls, cores)  # warm
    reps, t_tot = 0, 0.0
    while t_tot < 10.0 and reps < 400:
        X = B.copy()
        t0 = time.perf_counter()
        orc.sptrsv_csr_levelset_mrhs(L.n, *L.astuple(), X, cols, nl, lp, ls, cores)
        t_tot += time.perf_counter() - t0
        reps += 1
    t_solve = t_tot / reps * k / cols
    return {"value": algorithmic_bytes(L.nnz, L.n, k) / t_solve / 1e9, "unit": UNIT, "cores": cores,
            "kind": "port", "cpu": host_cpu(),
            "sample": "oracle sptrsv_csr_levelset (OpenMP per level, %d threads), %d RHS columns x %d "
                      "reps, scaled to %d RHS" % (cores, cols, reps, k)}


def _time(fn, reps, stream, flush=None):
    import torch
    ts = []
    for _ in range(reps):
        if flush is not None:
            flush.fill_(7)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b) / 1e3)
    return statistics.median(ts)


def bench_batch(dev, stream, flush, hop_us=None, k=8):
    """The 512 uneven SPD systems (80% shifted 2D Laplacians on 30..300
    grids, 20% random diagonally dominant, n 900..90,000), IC0 on the GPU,
    solved with 8 right-hand sides through the batch API (gbsym_batch_*) in
    one executor pass, FP64 and FP32.  Floors: HBM (algorithmic bytes at the
    measured copy bandwidth) and level latency (the pool's levels x hop_us,
    the per-level hop of the one-RHS FP32 sweep on the C2 factor)."""
    import torch
    from sympiler_gb300 import plans
    from sympiler_gb300._lib import EXEC_NAMES, LOWER_CSC
    t0 = time.perf_counter()
    idx, fac, N, nnz = c4_shard(0, 1, dev)
    res = {"systems": len(idx), "rows": N, "nnz_L": nnz, "setup_s": None, "api": "gbsym_batch_create_kind / "
           "gbsym_batch_autotune / gbsym_batch_solve"}
    rng = np.random.default_rng(45)
    peak, src = hbm_peak()
    for dt in ("f64", "f32"):
        bp = plans.BatchPlan(fac, dtype=dt, kind=LOWER_CSC)
        tdt = torch.float64 if dt == "f64" else torch.float32
        B = torch.from_numpy(rng.standard_normal((N, k))).to(dev).to(tdt)
        X = torch.empty_like(B)
        chosen = EXEC_NAMES.get(bp.autotune(k=k, dtype=dt))
        info = bp.info()

        def run():
            X.copy_(B)
            bp.solve(X)
        run()
        t = _time(run, 5, stream, flush) - _time(lambda: X.copy_(B), 5, stream, flush)
        bp.check()
        vb = 8 if dt == "f64" else 4
        byt = algorithmic_bytes(nnz, N, k, vb, vb)
        res[dt] = {"ms": t * 1e3, "batch_solves_per_s": 1.0 / t, "gbs": byt / t / 1e9,
                   "frac": byt / t / 1e9 / peak, "peak_gbs": peak, "peak_source": src,
                   "levels": info.levels, "executor": chosen, "tuning": bp.tuning(k),
                   "hbm_floor_ms": byt / peak / 1e6}
        if hop_us:
            res[dt]["floor_ms"] = max(byt / peak / 1e6, info.levels * hop_us / 1e3)
            res[dt]["floor_note"] = "max(HBM floor, levels x %.2f us one-RHS FP32 hop on the C2 factor)" % hop_us
        del bp, B, X
    res["setup_s"] = time.perf_counter() - t0
    return res


def bench_spmv(dev, stream, flush):
    """CSR SpMV y = A x (the Krylov drivers' system product) on the C3 and C2
    operators, FP64, L2 flushed before every timed call.  Bytes are
    B_spmv = (V + 4) nnz + 4 (n + 1) + 2 S n: every stored value and index
    read once, x read and y written once."""
    import torch
    from sympiler_gb300 import matgen as mg
    from sympiler_gb300.plans import CsrPlan
    peak = 6800.0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peak = json.load(fh).get("hbm_gbs") or peak
    except (OSError, ValueError):
        pass
    out = {}
    for name, A in (("c3_convdiff_96", mg.convdiff3d(96)), ("c2_lap3d_64", mg.lap3d(64, 1e-2))):
        P = CsrPlan(A.n, *A.astuple())
        x = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, A.n)).to(dev)
        y = torch.empty_like(x)
        P.spmv(x, y)
        t = _time(lambda: P.spmv(x, y), 10, stream, flush)
        byt = 12 * A.nnz + 4 * (A.n + 1) + 16 * A.n
        out[name] = {"n": A.n, "nnz": int(A.nnz), "us": t * 1e6, "gbs": byt / t / 1e9,
                     "hbm_frac": byt / t / 1e9 / peak,
                     "fp64_gops": 2 * A.nnz / t / 1e9, "fp64_frac": 2 * A.nnz / t / 1e9 / fp64_peak()}
        # spmv_csr_parallel on all host cores (CPU baseline leg only)
        try:
            import oracle
            cores = os.cpu_count() or 1
            xh, yh = x.cpu().numpy(), np.empty(A.n)
            o = oracle.orc()
            o.spmv_csr_parallel(A.n, *A.astuple(), xh, yh, cores)
            tc = []
            for _ in range(5):
                t0 = time.perf_counter()
                o.spmv_csr_parallel(A.n, *A.astuple(), xh, yh, cores)
                tc.append(time.perf_counter() - t0)
            out[name]["cpu_port"] = {"us": statistics.median(tc) * 1e6, "cores": cores, "cpu": host_cpu(),
                                     "speedup_gpu": statistics.median(tc) / t}
        except Exception as ex:  # the baseline must not hide the GPU numbers
            out[name]["cpu_port"] = {"error": str(ex)}
        del P
    return out


def bench_supernodal(dev, stream, flush, grid=64):
    """ParSy's supernodal solves (blockedLsolve / blockedLTsolve and their
    multi-RHS forms) on the supernodal Cholesky structure of the C2 operator
    (3D 7-point Laplacian 64^3) in geometric nested-dissection order:
    separators and leaf boxes of at most 64 nodes as supernodes, random
    diagonally dominant values.  FP64 ops count a multiply and an add per
    stored lower entry and three for each division; bytes are the used
    lower-block values, the row lists and x read and written once."""
    import torch
    from sympiler_gb300 import matgen as mg
    from sympiler_gb300 import sym_lib
    from sympiler_gb300.plans import SupernodalPlan
    S = mg.nd_supernodal(grid, grid, grid, leaf=64, rng=np.random.default_rng(1))
    w = np.diff(S.sup2col).astype(np.int64)
    nr = (S.Li_ptr[S.sup2col[1:]] - S.Li_ptr[S.sup2col[:-1]]).astype(np.int64)
    used_off = int(np.sum(w * (w - 1) // 2 + w * (nr - w)))
    t0 = time.perf_counter()
    P = SupernodalPlan(S)
    torch.cuda.synchronize()
    plan_s = time.perf_counter() - t0
    f_lev, t_lev = P.levels()
    out = {"workload": "supernodal Cholesky structure of the 3D 7-pt Laplacian %d^3, nested dissection" % grid,
           "n": S.n, "supernodes": S.nsup, "max_width": int(w.max()), "stored_values": int(len(S.Lx)),
           "used_offdiag": used_off, "levels": [f_lev, t_lev], "plan_s": plan_s,
           "gpu_launches_per_solve": 2}
    rng = np.random.default_rng(2)
    for k in (1, 64):
        X0 = torch.from_numpy(rng.standard_normal((k, S.n))).to(dev)
        X = X0.clone()
        ops = k * (2 * used_off + 3 * S.n)
        byt = 8 * (used_off + S.n) + 4 * int(nr.sum()) + 16 * S.n * k
        for tr in (False, True):
            def run():
                X.copy_(X0)
                P.solve(X if k > 1 else X[0], transposed=tr)
            run()
            P.check()
            t = _time(run, 5 if k == 1 else 3, stream, flush)
            P.check()
            key = "%s_k%d" % ("transposed" if tr else "forward", k)
            out[key] = {"ms": t * 1e3, "fp64_gops": ops / t / 1e9, "fp64_frac": ops / t / 1e9 / fp64_peak(),
                        "gbs": byt / t / 1e9}
    # end to end with host buffers, factor resident: H2D, solve, D2H
    hx = torch.from_numpy(rng.standard_normal(S.n)).pin_memory()
    dx = torch.empty(S.n, dtype=torch.float64, device=dev)
    hy = torch.empty(S.n, dtype=torch.float64).pin_memory()

    def e2e():
        dx.copy_(hx, non_blocking=True)
        P.solve(dx)
        hy.copy_(dx, non_blocking=True)
    e2e()
    out["forward_k1_e2e_ms"] = _time(e2e, 5, stream) * 1e3
    # the reference-facing drop-in: builds its plan, uploads the factor, solves
    xb = np.random.default_rng(3).standard_normal(S.n)
    x = xb.copy()
    t0 = time.perf_counter()
    assert sym_lib.parsy.blockedLsolve(S, x) == 1
    out["dropin_blockedLsolve_s"] = time.perf_counter() - t0
    # the reference's own serial blockedLsolve, compiled from its sources
    # (CPU baseline leg only)
    try:
        import oracle
        r = oracle.ref()
        kind = "reference" if r is not None else "port"
        xr = xb.copy()
        t0 = time.perf_counter()
        (r.blocked_lsolve if r is not None else oracle.orc().blocked_lsolve)(S, xr)
        cpu = time.perf_counter() - t0
        out["cpu_reference_blockedLsolve"] = {"s": cpu, "cores": 1, "kind": kind, "cpu": host_cpu(),
                                              "speedup_device": cpu / (out["forward_k1"]["ms"] / 1e3),
                                              "speedup_e2e": cpu / (out["forward_k1_e2e_ms"] / 1e3),
                                              "bit_exact": bool(np.array_equal(xr, x))}
    except Exception as ex:  # the baseline must not hide the GPU numbers
        out["cpu_reference_blockedLsolve"] = {"error": str(ex)}
    del P
    return out


def fp32_mrhs(L, dev, stream, flush, k=64):
    """FP32 storage and vectors, k right-hand sides, out of place, on a lower
    CSR factor: time, GB/s and fraction of HBM, with two floors: the HBM
    floor (algorithmic bytes at the measured copy bandwidth) and the
    level-latency floor (levels x the per-level hop of the plain one-RHS
    FP32 sync-free sweep on the same factor, measured here; the k-RHS sweep
    waits one level back as that one does, where the one-RHS look-through
    sweep, also reported, waits two)."""
    import torch
    from sympiler_gb300._lib import EXEC_NAMES, EXEC_SYNCFREE
    from sympiler_gb300.plans import TriPlan
    P = TriPlan(L.n, *L.astuple(), dtype="f32")
    ek = EXEC_NAMES.get(P.autotune(k=k, dtype="f32"))
    e1 = EXEC_NAMES.get(P.autotune(k=1, dtype="f32"))
    os.environ["GBSYM_SF_LOOKTHROUGH"] = "0"
    P1 = TriPlan(L.n, *L.astuple(), dtype="f32")
    os.environ.pop("GBSYM_SF_LOOKTHROUGH", None)
    P1.set_exec(EXEC_SYNCFREE)
    rng = np.random.default_rng(64)
    B = torch.from_numpy(rng.standard_normal((L.n, k)).astype(np.float32)).to(dev)
    X = torch.empty_like(B)
    b1 = B[:, 0].contiguous()
    x1 = torch.empty_like(b1)
    tk = _time(lambda: P.solve_into(B, X), 7, stream, flush)
    t1 = _time(lambda: P1.solve_into(b1, x1), 7, stream, flush)
    t1_lt = _time(lambda: P.solve_into(b1, x1), 7, stream, flush)  # the tuned one-RHS solve
    P.check()
    P1.check()
    levels = P.info().levels
    peak, src = hbm_peak()
    byt = algorithmic_bytes(L.nnz, L.n, k, 4, 4)
    return {"n": L.n, "nnz_L": int(L.nnz), "levels": levels, "rhs": k, "ms": tk * 1e3, "gbs": byt / tk / 1e9,
            "frac": byt / tk / 1e9 / peak, "peak_gbs": peak, "peak_source": src,
            "algorithmic_bytes": byt, "hbm_floor_ms": byt / peak / 1e6,
            "floor_ms": t1 * 1e3, "hop_us": t1 * 1e6 / levels,
            "one_rhs_tuned_ms": t1_lt * 1e3, "one_rhs_tuning": P.tuning(1),
            "floor_note": "level-latency floor = levels x the per-level hop of the plain one-RHS FP32 sync-free "
                          "sweep on the same factor, which waits one level back like the k-RHS sweep (%.1f us "
                          "measured; the tuned one-RHS solve, look-through included, %.1f us)"
                          % (t1 * 1e6, t1_lt * 1e6),
            "executors": {"k%d" % k: ek, "k1": e1}}


def fp64_mrhs(L, dev, stream, flush, k=64):
    """FP64, k right-hand sides, out of place, exact arithmetic, on a lower
    CSR factor: time, GB/s, HBM fraction and the FP64 roofline."""
    import torch
    from sympiler_gb300._lib import EXEC_NAMES
    from sympiler_gb300.plans import TriPlan
    P = TriPlan(L.n, *L.astuple())
    ek = EXEC_NAMES.get(P.autotune(k=k))
    B = torch.from_numpy(np.random.default_rng(65).standard_normal((L.n, k))).to(dev)
    X = torch.empty_like(B)
    t = _time(lambda: P.solve_into(B, X), 7, stream, flush)
    P.check()
    info = P.info()
    peak, src = hbm_peak()
    byt = algorithmic_bytes(L.nnz, L.n, k)
    ops = fp64_ops_exact(int(info.nnz_off), L.n, k)
    return {"n": L.n, "levels": info.levels, "rhs": k, "ms": t * 1e3, "gbs": byt / t / 1e9,
            "frac": byt / t / 1e9 / peak, "peak_source": src,
            "fp64_frac": fp64_floor_s(int(info.nnz_off), L.n, k) / t,
            "fp64_floor_ms": fp64_floor_s(int(info.nnz_off), L.n, k) * 1e3, "executor": ek}


def bench_c1(dev, stream, flush):
    """C1, the reference's CPU-runnable case: L = lower triangle of the 2D
    5-point Laplacian on a 100 x 100 grid (n = 10,000, 199 levels), one
    right-hand side, FP64; and SpMV with the full Laplacian.  The GPU solve
    is timed cold (L2 flushed) and warm (back to back); beside it the
    oracle's serial sptrsv_csr and spmv_csr on one host core (CPU leg
    only).  A problem this small is latency-bound on the GPU: 199 dependent
    levels cost more than a serial CPU solve that fits in L1/L2."""
    import torch
    from sympiler_gb300 import matgen as mg
    from sympiler_gb300._lib import EXEC_NAMES
    from sympiler_gb300.plans import CsrPlan, TriPlan
    A = mg.lap2d(100)
    L = mg.tril(A)
    P = TriPlan(L.n, *L.astuple())
    e1 = EXEC_NAMES.get(P.autotune(k=1))
    b = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, L.n)).to(dev)
    x = torch.empty_like(b)
    t_cold = _time(lambda: P.solve_into(b, x), 15, stream, flush)
    t_warm = _time(lambda: P.solve_into(b, x), 15, stream, None)
    P.check()
    Ap = CsrPlan(A.n, *A.astuple())
    y = torch.empty_like(b)
    t_spmv = _time(lambda: Ap.spmv(b, y), 15, stream, flush)
    trsv_b = algorithmic_bytes(L.nnz, L.n, 1)
    spmv_b = 12 * A.nnz + 4 * (A.n + 1) + 16 * A.n
    out = {"n": L.n, "levels": P.info().levels, "executor": e1,
           "sptrsv_us_cold": t_cold * 1e6, "sptrsv_us_warm": t_warm * 1e6,
           "sptrsv_solves_per_s": 1.0 / t_warm, "sptrsv_gbs_cold": trsv_b / t_cold / 1e9,
           "spmv_us_cold": t_spmv * 1e6, "spmv_gbs_cold": spmv_b / t_spmv / 1e9}
    try:
        import oracle
        o = oracle.orc()
        bh = b.cpu().numpy()
        ts = []
        for _ in range(21):
            xh = bh.copy()
            t0 = time.perf_counter()
            o.sptrsv_csr(L.n, *L.astuple(), xh)
            ts.append(time.perf_counter() - t0)
        yh = np.zeros(A.n)
        tsp = []
        for _ in range(21):
            t0 = time.perf_counter()
            o.spmv_csr(A.n, *A.astuple(), bh, yh)
            tsp.append(time.perf_counter() - t0)
        out["cpu_port"] = {"sptrsv_us": statistics.median(ts) * 1e6, "spmv_us": statistics.median(tsp) * 1e6,
                           "cores": 1, "cpu": host_cpu(),
                           "bit_identical": bool(np.array_equal(xh, x.cpu().numpy()))}
    except Exception as ex:  # the baseline must not hide the GPU numbers
        out["cpu_port"] = {"error": str(ex)}
    return out


def bench_adjoint(dev, stream, flush, g=1024, k=32):
    """Forward X = L^{-1} B and the reverse pass (L^T solve + value gradient)
    on the IC0 factor of the 1024^2 anisotropic variable-coefficient Poisson
    operator, 32 right-hand sides, FP64."""
    import torch
    from sympiler_gb300 import matgen as mg
    from sympiler_gb300 import plans
    from sympiler_gb300._lib import LOWER_CSC, UPPER_DIAG_FIRST
    rng = np.random.default_rng(55)
    A = mg.aniso_poisson2d(g, 0.01, 1.0, rng)
    U = mg.triu(A)
    dp, di = torch.from_numpy(U.p).to(dev), torch.from_numpy(U.i).to(dev)
    dv = torch.from_numpy(U.x.copy()).to(dev)
    plans.ic0_device(U.n, dv, dp, di)
    Lf = plans.TriPlan(U.n, dp, di, dv, kind=LOWER_CSC)
    Lt = plans.TriPlan(U.n, dp, di, dv, kind=UPPER_DIAG_FIRST)
    Lcsr = mg.transpose(mg.CSR(U.n, U.p, U.i, dv.cpu().numpy()))
    lp, li = torch.from_numpy(Lcsr.p).to(dev), torch.from_numpy(Lcsr.i).to(dev)
    ef = Lf.autotune(k=k)
    et = Lt.autotune(k=k)
    B = torch.from_numpy(rng.standard_normal((U.n, k))).to(dev)
    W = torch.from_numpy(rng.standard_normal((U.n, k))).to(dev)
    X = torch.empty_like(B)
    G = torch.empty_like(W)
    grad = torch.empty(Lcsr.nnz, dtype=torch.float64, device=dev)

    def fwd():
        X.copy_(B)
        Lf.solve(X)

    def bwd():
        G.copy_(W)
        plans.tri_adjoint(Lt, U.n, lp, li, X, G, grad)
    fwd()
    bwd()
    tf = _time(fwd, 5, stream, flush)
    tb = _time(bwd, 5, stream, flush)
    info = Lf.info()
    byt = algorithmic_bytes(Lcsr.nnz, U.n, k)
    fp32 = fp32_mrhs(Lcsr, dev, stream, flush, 64)
    fp64 = fp64_mrhs(Lcsr, dev, stream, flush, 64)
    return {"fp32_64rhs": fp32, "fp64_64rhs": fp64, "n": U.n, "nnz_L": Lcsr.nnz, "levels": info.levels, "rhs": k,
            "forward_ms": tf * 1e3, "forward_gbs": byt / tf / 1e9, "backward_ms": tb * 1e3,
            "executors": {"forward": ef, "transposed": et}}


def c4_shard(rank, world, dev):
    """This rank's share of the 512-system batch (LPT on rows + entries), its
    IC0 factors computed on the GPU in one pass over the shard's
    block-diagonal pool, returned as per-system lower CSCs (the upper CSRs
    IC0 works in): (indices, [(n, p, i, x)], rows, stored entries)."""
    import torch
    from sympiler_gb300 import matgen as mg
    from sympiler_gb300 import plans
    from sympiler_gb300.shard import shard_systems
    systems = mg.batch_systems_upper(512, np.random.default_rng(44))
    idx, mine = shard_systems(systems, rank, world)
    N, up, ui, ux, off = mg.block_diagonal(mine)
    dv = torch.from_numpy(ux).to(dev)
    plans.ic0_device(N, dv, torch.from_numpy(up).to(dev), torch.from_numpy(ui).to(dev))
    vals = dv.cpu().numpy()
    fac, e0 = [], 0
    for (n, p, i, x) in mine:
        e1 = e0 + int(p[n])
        fac.append((n, p, i, vals[e0:e1]))
        e0 = e1
    return idx, fac, N, int(up[-1])


def c4_config(dt, k, nsys, world):
    return {"workload": "C4 batch: 512 uneven SPD systems (80%% shifted 2D Laplacians 30..300 per side, 20%% "
                        "random diagonally dominant, n 900..90,000), IC0 factors, forward SpTRSV, %d RHS %s, "
                        "one batched sync-free launch per rank" % (k, dt.upper()),
            "systems": 512, "systems_rank0": nsys, "rhs": k, "layout": "row-major (sum n_s) x k",
            "l2": "inputs (about 1 GB in FP64) larger than L2; 256 MB L2 flush write between timed steps",
            "parallelism": "systems sharded over %d rank(s) by LPT on rows + entries; no collective on the "
                           "data path" % world}


def run_c4(args):
    """The batched workload as the timed step: each rank builds gbsym_batch
    over its shard of the 512 systems and solves it with 8 right-hand sides;
    value = algorithmic bytes of all ranks / the slowest rank's time."""
    import torch
    from sympiler_gb300 import plans
    from sympiler_gb300._lib import EXEC_NAMES, LOWER_CSC
    world, rank, local = dist_init()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    k, dt = 8, args.dtype
    idx, fac, N, nnz = c4_shard(rank, world, dev)
    if args.exec != "auto":  # one executor, no tuning (profiling runs)
        os.environ["GBSYM_TRI_EXEC"] = args.exec
    bp = plans.BatchPlan(fac, dtype=dt, kind=LOWER_CSC)
    chosen = EXEC_NAMES.get(bp.autotune(k=k, dtype=dt)) if args.exec == "auto" else args.exec
    info = bp.info()
    vb = 8 if dt == "f64" else 4
    byt = algorithmic_bytes(nnz, N, k, vb, vb)
    tdt = torch.float64 if dt == "f64" else torch.float32
    B = torch.from_numpy(np.random.default_rng(45 + rank).standard_normal((N, k))).to(dev).to(tdt)
    X = torch.empty_like(B)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def step(timed):
        X.copy_(B)
        flush.fill_(rank + 1)
        if not timed:
            bp.solve(X)
            return None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bp.solve(X)
        e1.record(stream)
        return e0, e1

    for _ in range(max(3, args.warmup)):
        step(False)
    bp.check()
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = plans.kernel_launches()
    evs = [step(True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    launches = plans.kernel_launches() - launches0
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    bp.check()
    t_step = sum(a.elapsed_time(b) for a, b in evs) / len(evs) / 1e3
    tot = torch.tensor([t_step, float(byt)], dtype=torch.float64, device=dev)
    if world > 1:
        tmax = tot[:1].clone()
        torch.distributed.all_reduce(tmax, op=torch.distributed.ReduceOp.MAX)
        bsum = tot[1:].clone()
        torch.distributed.all_reduce(bsum)
        t_step, byt_all = float(tmax.item()), float(bsum.item())
    else:
        byt_all = float(byt)
    # residual spot check on this rank's first system (scipy, FP64)
    import scipy.sparse as sp
    n0, p0, i0, x0 = fac[0]
    Lt0 = sp.csr_matrix((x0, i0, p0), shape=(n0, n0))
    xs = X[:n0, 0].double().cpu().numpy()
    resid = float(np.abs(Lt0.T @ xs - B[:n0, 0].double().cpu().numpy()).max())
    # end to end through the C ABI on pinned host buffers
    # (gbsym_batch_solve_host).  With 8 right-hand sides a row's values are
    # 32 or 64 bytes, below the 256 bytes from which the library solves a
    # page-locked buffer in place over the CPU-GPU link, so it stages
    # H2D + solve + D2H (in place measured 7.9 / 15.9 ms against 6.4 /
    # 13.1 ms staged).
    from sympiler_gb300.plans import host_solve_in_place
    Hb = torch.empty((N, k), dtype=tdt).pin_memory()
    Hb.copy_(B.cpu())
    Hx = torch.empty_like(Hb).pin_memory()

    def e2e_median(direct):
        if direct:
            os.environ.pop("GBSYM_HOST_DIRECT", None)
        else:
            os.environ["GBSYM_HOST_DIRECT"] = "0"
        for _ in range(2):
            Hx.copy_(Hb)
            bp.solve_host(Hx)
        ts = []
        for _ in range(max(3, args.steps // 2)):
            Hx.copy_(Hb)
            flush.fill_(rank + 1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            bp.solve_host(Hx)
            ts.append(time.perf_counter() - t0)
        os.environ.pop("GBSYM_HOST_DIRECT", None)
        return statistics.median(ts)

    e2e_staged = e2e_median(False)
    e2e_t = e2e_median(True)
    in_place = host_solve_in_place(Hx.data_ptr()) and k * vb >= 256
    e2e_exact = bool(torch.equal(Hx, X.cpu()))
    if world > 1:
        tt = torch.tensor([e2e_t, e2e_staged], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        e2e_t, e2e_staged = float(tt[0].item()), float(tt[1].item())
    peak, peak_src = hbm_peak()
    if rank == 0:
        line = {"metric": METRIC, "value": byt_all / t_step / 1e9, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
                "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": dt,
                "data": "synthetic", "config": dict(c4_config(dt, k, len(idx), world), rows_rank0=N,
                                                    levels_rank0=info.levels, executor=chosen,
                                                    tuning=bp.tuning(k)),
                "roofline": {"bound": "hbm", "achieved": byt / t_step / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": byt / t_step / 1e9 / peak, "peak_source": peak_src,
                             "traffic": load_traffic("c4_batch_%s_8rhs" % dt),
                             "algorithmic_bytes_per_solve": byt},
                "e2e": {"value": byt_all / e2e_t / 1e9, "unit": UNIT, "h2d_bytes_per_step": N * k * vb,
                        "d2h_bytes_per_step": N * k * vb, "ms_per_step": e2e_t * 1e3,
                        "api": "BatchPlan.solve_host (gbsym_batch_solve_host, pinned host x, row-major, "
                               "wall clock per call)",
                        "path": ("in place over the CPU-GPU link (sync-free sweep reads b and writes x in "
                                 "the host buffer)") if in_place else "staged: H2D + solve + D2H",
                        "bit_identical_to_device_solve": e2e_exact,
                        "staged_ms_per_step": e2e_staged * 1e3,
                        "staged_value": byt_all / e2e_staged / 1e9},
                "gpu_launches": int(launches), "clocks": clocks,
                "check": {"max_abs_residual_system0_col0": resid}}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            v = json.load(fh).get("hbm_gbs")
            if v:
                return float(v), "measured"
    except (OSError, ValueError):
        pass
    return 6800.0, "fallback"


def load_traffic(workload_key):
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as fh:
            return json.load(fh).get(workload_key)
    except (OSError, ValueError):
        return None


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "c4":
        run_c4(args)
        return
    import torch
    world, rank, local = dist_init()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.supernodal_grid:
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        out = bench_supernodal(dev, torch.cuda.current_stream(), flush, grid=args.supernodal_grid)
        if rank == 0:
            print(json.dumps({"extras": {"supernodal_nd": out}}), flush=True)
        return

    from sympiler_gb300 import matgen as mg
    from sympiler_gb300 import plans
    from sympiler_gb300._lib import UPPER_DIAG_FIRST
    from sympiler_gb300.plans import CsrPlan, TriPlan

    k_all = args.rhs
    shard_rhs = args.shard == "rhs" and world > 1
    if shard_rhs:
        from sympiler_gb300.shard import column_range
        c0, c1 = column_range(k_all, rank, world)
    else:
        c0, c1 = 0, k_all
    k = c1 - c0  # this rank's right-hand sides
    g = args.grid
    A = mg.lap3d(g, 1e-2)
    U = mg.triu(A)
    # IC0 on the GPU (the library's level-scheduled spic0_csr)
    vals = torch.from_numpy(U.x.copy()).to(dev)
    plans.ic0_device(U.n, vals, torch.from_numpy(U.p).to(dev), torch.from_numpy(U.i).to(dev))
    torch.cuda.synchronize()
    Lt = mg.CSR(U.n, U.p, U.i, vals.cpu().numpy())
    L = mg.transpose(Lt)
    plan = TriPlan(L.n, *L.astuple())
    from sympiler_gb300._lib import EXEC_NAMES
    if args.exec == "auto":
        tuned = {"k1": EXEC_NAMES.get(plan.autotune(k=1)), "k%d" % k: EXEC_NAMES.get(plan.autotune(k=k))}
    else:
        forced = {v: c for c, v in EXEC_NAMES.items()}[args.exec]
        plan.set_exec(forced)
        tuned = {"k1": args.exec, "k%d" % k: args.exec, "forced": True}
    info = plan.info()
    n = L.n
    byt = algorithmic_bytes(L.nnz, n, k)

    if shard_rhs:  # one problem, its columns split: every rank draws the same B
        B = torch.from_numpy(np.random.default_rng(1234).standard_normal((n, k_all))[:, c0:c1].copy()).to(dev)
    else:
        B = torch.from_numpy(np.random.default_rng(1234 + rank).standard_normal((n, k))).to(dev)
    X = torch.empty_like(B)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    result = {}

    if not args.extras_only:
        # one step: X = L^-1 B out of place (gbsym_tri_solve_into), B
        # resident and unchanged; the sync-free sweep publishes each result
        # straight into X
        def step(timed):
            flush.fill_(rank + 1)
            if timed:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                plan.solve_into(B, X)
                e1.record(stream)
                return e0, e1
            plan.solve_into(B, X)
            return None

        for _ in range(max(3, args.warmup)):
            step(False)
        torch.cuda.synchronize()
        sampler = ClockSampler(local)
        sampler.start()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        launches0 = plans.kernel_launches()
        w0 = time.perf_counter()
        evs = [step(True) for _ in range(args.steps)]
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        launches = plans.kernel_launches() - launches0
        if world > 1:
            torch.distributed.barrier()
        clocks = sampler.stop()
        times = [a.elapsed_time(b) / 1e3 for a, b in evs]
        t_step = sum(times) / len(times)
        if world > 1:
            tt = torch.tensor([t_step], device=dev)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t_step = float(tt.item())
        value_rank = byt / t_step / 1e9
        value = value_rank * world
        if shard_rhs:  # every rank's bytes (its factor copy and its columns) over the slowest rank's time
            bt = torch.tensor([float(byt)], dtype=torch.float64, device=dev)
            torch.distributed.all_reduce(bt)
            value = float(bt.item()) / t_step / 1e9

        # end to end through the C ABI on pinned host buffers.  On a coherent
        # CPU-GPU system the library solves such a buffer in place over the
        # link (each right-hand side read once, each result written once,
        # overlapped with the sweep); elsewhere it stages H2D + solve + D2H.
        # The staged path is timed too (GBSYM_HOST_DIRECT=0) for comparison.
        from sympiler_gb300.plans import host_solve_in_place
        Hb = torch.empty((n, k), dtype=torch.float64).pin_memory()
        Hb.copy_(B.cpu())
        Hx = torch.empty_like(Hb).pin_memory()

        def e2e_median(direct):
            if direct:
                os.environ.pop("GBSYM_HOST_DIRECT", None)
            else:
                os.environ["GBSYM_HOST_DIRECT"] = "0"
            for _ in range(2):
                Hx.copy_(Hb)
                plan.solve_host_ptr(Hx.data_ptr(), k)
            ts = []
            for _ in range(max(3, args.steps // 2)):
                Hx.copy_(Hb)
                flush.fill_(rank + 1)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                plan.solve_host_ptr(Hx.data_ptr(), k)
                ts.append(time.perf_counter() - t0)
            os.environ.pop("GBSYM_HOST_DIRECT", None)
            return statistics.median(ts)

        e2e_staged = e2e_median(False)
        e2e_step = e2e_median(True)
        in_place = host_solve_in_place(Hx.data_ptr())
        # the in-place result must equal the device-resident one bit for bit
        e2e_exact = bool(torch.equal(Hx, X.cpu()))

        # parity spot check of the timed result (first column) against a
        # plain FP64 dense-free check: residual of L x = b on one column
        x0 = X[:, 0].cpu().numpy()
        r = L.scipy() @ x0 - B[:, 0].cpu().numpy()
        resid = float(np.abs(r).max())

        peaks = {}
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
                peaks = json.load(fh)
        except (OSError, ValueError):
            pass
        peak = peaks.get("hbm_gbs")
        peak_src = "measured" if peak else "fallback"
        peak = peak or 6800.0
        traffic = load_traffic("c2_ic0_fwd_%drhs" % k)
        result.update({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "strong" if shard_rhs else "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": dict(config(g, k_all), levels=info.levels, nnz_L=int(L.nnz), executor=tuned,
                           parallelism=("%d RHS columns split over %d ranks (this rank: %d..%d), each rank "
                                        "holding the factor; no collective on the data path"
                                        % (k_all, world, c0, c1) if shard_rhs else "replicas"),
                           arithmetic="exact (reference operation order, bit-identical)",
                           api="gbsym_tri_solve_into: X = L^-1 B out of place, B unchanged",
                           wall_s_timed_region=wall),
            "roofline": {"bound": "hbm", "achieved": byt / t_step / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": byt / t_step / 1e9 / peak, "peak_source": peak_src,
                         "traffic": traffic,
                         "algorithmic_bytes_per_solve": byt,
                         "note": ("one solve = one graph of per-level kernels"
                                  if tuned["k%d" % k] == "levelset" else
                                  "one solve = the sentinel fill of X + one %s kernel launch" % tuned["k%d" % k])
                                 + "; duration from CUDA events on the launch stream"},
            "roofline_fp64": fp64_roofline(int(info.nnz_off), n, k, t_step),
            "e2e": {"value": byt / e2e_step / 1e9, "unit": UNIT, "h2d_bytes_per_step": n * k * 8,
                    "d2h_bytes_per_step": n * k * 8, "ms_per_step": e2e_step * 1e3,
                    "api": "gbsym_tri_solve_host (pinned host x, row-major, wall clock per call)",
                    "path": ("in place over the CPU-GPU link (sync-free sweep reads b and writes x "
                             "in the host buffer)") if in_place else "staged: H2D + solve + D2H",
                    "bit_identical_to_device_solve": e2e_exact,
                    "staged_ms_per_step": e2e_staged * 1e3,
                    "staged_value": byt / e2e_staged / 1e9},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "check": {"max_abs_residual_col0": resid},
        })

    if rank == 0 and not args.no_extras:
        extras = {}
        # 1-RHS forward solve on the same factor
        x1 = B[:, 0].contiguous()
        x1w = torch.empty_like(x1)
        for _ in range(3):
            x1w.copy_(x1)
            plan.solve(x1w)
        ts = []
        for _ in range(10):
            x1w.copy_(x1)
            flush.fill_(3)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.solve(x1w)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        t1 = statistics.median(ts)
        b1 = algorithmic_bytes(L.nnz, n, 1)
        extras["sptrsv_1rhs"] = {"us": t1 * 1e6, "gbs": b1 / t1 / 1e9, "levels": info.levels,
                                 "us_per_level": t1 * 1e6 / info.levels}

        # every executor on the same factor, 1 and k right-hand sides
        def time_exec(mode, xbuf, src, reps=5):
            plan.set_exec(mode)
            for _ in range(2):
                xbuf.copy_(src)
                plan.solve(xbuf)
            tt = []
            for _ in range(reps):
                xbuf.copy_(src)
                flush.fill_(5)
                a0 = torch.cuda.Event(enable_timing=True)
                a1 = torch.cuda.Event(enable_timing=True)
                a0.record(stream)
                plan.solve(xbuf)
                a1.record(stream)
                torch.cuda.synchronize()
                tt.append(a0.elapsed_time(a1) * 1e3)
            plan.check()
            return statistics.median(tt)
        ex = {}
        for arith_name, arith in (("exact", 0), ("fused", 1)):
            plan.set_arith(arith)
            for name, mode in (("levelset_graph_pdl", 1), ("syncfree", 2), ("persistent", 4), ("oneblock", 3),
                               ("cluster", 5), ("partitioned", 6)):
                key = "%s_%s" % (name, arith_name)
                ex[key] = {"us_1rhs": time_exec(mode, x1w, x1)}
                if mode not in (3, 6):  # one right-hand side only
                    ex[key]["us_%drhs" % k] = time_exec(mode, X, B)
        plan.set_arith(0)
        plan.set_exec(0)
        ex["autotuned"] = {"k1": EXEC_NAMES.get(plan.autotune(k=1)),
                           "k%d" % k: EXEC_NAMES.get(plan.autotune(k=k))}
        extras["executors"] = ex
        # the reference-facing drop-in per call (host arrays: upload, level
        # set, packing, solve, download), with the plan cache off and on,
        # beside a plan build alone and the host LBC inspector
        from sympiler_gb300 import sym_lib
        xb = B[:, 0].cpu().numpy()

        def dropin_once():
            xh = xb.copy()
            sym_lib.sptrsv_csr(L.n, L.p, L.i, L.x, xh)

        def wall_median(fn, reps=5):
            fn()
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                fn()
                ts.append(time.perf_counter() - t0)
            return statistics.median(ts)
        t_drop = wall_median(dropin_once)
        sym_lib.dropin_cache(2)
        t_drop_cached = wall_median(dropin_once)
        sym_lib.dropin_cache(0)

        def build_plan():
            TriPlan(L.n, *L.astuple())
            torch.cuda.synchronize()
        t_build = wall_median(build_plan, 3)
        t_lbc = wall_median(lambda: sym_lib.get_coarse_levelSet_DAG_CSC_tree(L.n, L.p, L.i, 0, 16, -1, 4000), 3)
        Cl = mg.tril(mg.convdiff3d(96))
        t_lbc_c3 = wall_median(lambda: sym_lib.get_coarse_levelSet_DAG_CSC_tree(Cl.n, Cl.p, Cl.i, 0, 16, -1, 4000),
                               3)

        def build_plan_c3():
            TriPlan(Cl.n, *Cl.astuple())
            torch.cuda.synchronize()
        t_build_c3 = wall_median(build_plan_c3, 3)
        extras["dropin_sptrsv_csr_c2"] = {
            "per_call_ms": t_drop * 1e3, "per_call_cached_ms": t_drop_cached * 1e3,
            "note": "sym_lib.sptrsv_csr on host arrays, one right-hand side; cached: gbsym_dropin_cache(2), "
                    "the plan built by the first call reused"}
        extras["inspectors"] = {
            "c2": {"plan_build_ms": t_build * 1e3, "lbc_host_ms": t_lbc * 1e3, "n": L.n},
            "c3_lower": {"plan_build_ms": t_build_c3 * 1e3, "lbc_host_ms": t_lbc_c3 * 1e3, "n": Cl.n},
            "note": "plan build = upload + GPU validation + GPU level set + packing (gbsym_tri_create from host "
                    "arrays); LBC = the host DAG LBC inspector (get_coarse_levelSet_DAG_CSC_tree's role, 16 "
                    "parts per coarse level, min level distance -1, division rate 4000)"}
        del Cl
        # the same factor in FP32 with 64 right-hand sides
        extras["sptrsv_64rhs_fp32_c2"] = fp32_mrhs(L, dev, stream, flush, 64)
        # in place (gbsym_tri_solve) beside the out-of-place headline step
        def in_place():
            X.copy_(B)
            plan.solve(X)
        t_ip = _time(in_place, 7, stream, flush)
        t_cp = _time(lambda: X.copy_(B), 7, stream, flush)
        extras["sptrsv_%drhs_in_place" % k] = {"ms_incl_copy": t_ip * 1e3, "copy_ms": t_cp * 1e3,
                                               "ms": (t_ip - t_cp) * 1e3}
        # IC0-PCG to 1e-10 on C2 (FP64 throughout)
        Pt = TriPlan(n, *Lt.astuple(), kind=UPPER_DIAG_FIRST)
        Pt.autotune(k=1)
        Ac = CsrPlan(n, *A.astuple())
        xs = np.random.default_rng(7).standard_normal(n)
        bb = torch.from_numpy(A.scipy() @ xs).to(dev)
        xx = torch.zeros(n, dtype=torch.float64, device=dev)
        plans.pcg(Ac, plan, Pt, bb, xx, tol=1e-10, maxit=2000)
        xx.zero_()
        res = plans.pcg(Ac, plan, Pt, bb, xx, tol=1e-10, maxit=2000)
        extras["pcg_c2"] = {"seconds": res.seconds, "iterations": res.iterations, "relres": res.relres,
                            "err_vs_xstar": float(np.linalg.norm(xx.cpu().numpy() - xs) / np.linalg.norm(xs))}
        # the same PCG on one host core: the restated driver over the
        # reference's serial kernels (CPU baseline leg only)
        try:
            import oracle
            t0 = time.perf_counter()
            _, it_c, rel_c = oracle.orc().pcg_ic0(n, A.astuple(), L.astuple(), Lt.astuple(), bb.cpu().numpy(),
                                                  1e-10, 2000)
            tc = time.perf_counter() - t0
            extras["pcg_c2"]["cpu_port"] = {"seconds": tc, "iterations": it_c, "relres": rel_c, "cores": 1,
                                            "cpu": host_cpu(), "speedup_gpu": tc / res.seconds}
        except Exception as ex:  # the baseline must not hide the GPU numbers
            extras["pcg_c2"]["cpu_port"] = {"error": str(ex)}
        # GMRES(30) + right ILU0 on the 96^3 convection-diffusion operator
        from sympiler_gb300._lib import ILU_UNIT_LOWER, ILU_UPPER
        C = mg.convdiff3d(96)
        d = mg.diag_ptr(C)
        dC = [torch.from_numpy(a).to(dev) for a in (C.p, C.i, C.x, d)]
        lu = torch.empty(C.nnz, dtype=torch.float64, device=dev)
        plans.ilu0_device(C.n, *dC, lu)
        Cp = CsrPlan(C.n, dC[0], dC[1], dC[2])
        bc = torch.from_numpy(np.random.default_rng(9).uniform(-1, 1, C.n)).to(dev)
        out = {}
        for prec in ("f32", "f64"):
            Lu = TriPlan(C.n, dC[0], dC[1], lu, kind=ILU_UNIT_LOWER, diags=dC[3], dtype=prec)
            Up = TriPlan(C.n, dC[0], dC[1], lu, kind=ILU_UPPER, diags=dC[3], dtype=prec)
            tuned_prec = [EXEC_NAMES.get(P.autotune(k=1, dtype=prec)) for P in (Lu, Up)]
            xg = torch.zeros(C.n, dtype=torch.float64, device=dev)
            plans.gmres(Cp, Lu, Up, bc, xg, mr=30, maxit=100, tol=1e-10)
            runs = []
            for _ in range(2):
                xg.zero_()
                runs.append(plans.gmres(Cp, Lu, Up, bc, xg, mr=30, maxit=100, tol=1e-10))
            best = min(runs, key=lambda r: r.seconds)
            # per-iteration split: one preconditioner apply (the two
            # triangular sweeps, in the plan's precision), one system SpMV,
            # and the rest (Gram-Schmidt passes, the device Givens step,
            # precision conversions, launch gaps)
            tdt = torch.float32 if prec == "f32" else torch.float64
            zsrc = bc.to(tdt)
            zz = torch.empty_like(zsrc)

            def apply_once():
                Lu.solve_into(zsrc, zz)
                Up.solve(zz)
            t_apply = _time(apply_once, 7, stream, flush)
            t_spmv = _time(lambda: Cp.spmv(bc, xg), 7, stream, flush)
            it_ms = best.seconds / max(1, best.iterations) * 1e3
            split = {"iteration_ms": it_ms, "precond_apply_ms": t_apply * 1e3, "spmv_ms": t_spmv * 1e3,
                     "rest_ms": it_ms - t_apply * 1e3 - t_spmv * 1e3}
            out[prec] = {"per_iteration": split,
                         "seconds": best.seconds, "iterations": best.iterations, "restarts": best.restarts,
                         "relres": best.relres, "status": best.status, "executors": tuned_prec}
        out["speedup_fp32_precond"] = out["f64"]["seconds"] / out["f32"]["seconds"]
        # the same GMRES on one host core: the restated driver over the
        # reference's serial kernels and lus_cr (CPU baseline leg only)
        try:
            import oracle
            t0 = time.perf_counter()
            _, it_c, rel_c = oracle.orc().gmres_ilu0(C.n, C.astuple(), lu.cpu().numpy(), d, bc.cpu().numpy(), 30, 100,
                                                     1e-10)
            tc = time.perf_counter() - t0
            out["cpu_port"] = {"seconds": tc, "iterations": it_c, "relres": rel_c, "cores": 1, "cpu": host_cpu(),
                               "speedup_gpu_f32": tc / out["f32"]["seconds"]}
            # one ILU0 apply (lus_cr) on one core, beside the GPU's
            luh = lu.cpu().numpy()
            rh = bc.cpu().numpy()
            t0 = time.perf_counter()
            oracle.orc().lus_cr(C.n, C.p, C.i, luh, d, rh)
            out["cpu_port"]["lus_cr_ms"] = (time.perf_counter() - t0) * 1e3
        except Exception as ex:  # the baseline must not hide the GPU numbers
            out["cpu_port"] = {"error": str(ex)}
        extras["gmres_c3"] = out
        del Cp, dC, lu
        extras["batch_c4"] = bench_batch(dev, stream, flush, extras["sptrsv_64rhs_fp32_c2"]["hop_us"])
        extras["adjoint_c5"] = bench_adjoint(dev, stream, flush)
        extras["sptrsv_64rhs_fp32_c5"] = extras["adjoint_c5"].pop("fp32_64rhs")
        extras["sptrsv_64rhs_fp64_c5"] = extras["adjoint_c5"].pop("fp64_64rhs")
        extras["c1_lap2d_100"] = bench_c1(dev, stream, flush)
        extras["spmv"] = bench_spmv(dev, stream, flush)
        extras["supernodal_c2_nd"] = bench_supernodal(dev, stream, flush)
        result["extras"] = extras
    if rank == 0:
        if not args.extras_only:
            try:
                import oracle  # noqa: F401  (CPU baseline leg only)
                o = oracle.orc()
                nl, lp, ls = o.build_levelset_csr(L.n, L.p, L.i)
                result["cpu_baseline"] = cpu_baseline_sample(L, k, nl, lp, ls)
            except Exception as ex:  # the baseline must not hide the GPU number
                result["cpu_baseline"] = {"value": None, "unit": UNIT, "error": str(ex)}
        print(json.dumps(result), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
