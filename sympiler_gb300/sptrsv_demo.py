"""The reference's SpTRSV demo on the GPU path.

    python -m sympiler_gb300.sptrsv_demo [matrix.mtx [p2 [p3]]] [--header] [--parts N]

mirrors demo/sptrsv_demo.cpp:32-132.  It reads a MatrixMarket file (or, with
no file, makes a seeded random 16 x 16 lower triangle of density about 0.2, as
the demo's random mode does), takes its lower triangle L (CSR and CSC), and
runs the demo's three variants through this library's drop-ins:

* serial         -- ``sptrsv_csr``,
* level set CSC  -- ``build_levelSet_CSC`` then ``sptrsv_csc_levelset``,
* LBC CSR        -- ``get_coarse_levelSet_DAG_CSC_tree(lp=parts, cp=p2,
  ic=p3)`` then ``sptrsv_csr_lbc``,

each timed end to end (host arrays in, solution out: upload, plan build and
solve), median of 5 as the demo's evaluator takes.  The inspectors run
outside the timed region, as in the demo.  It also times the solve alone
on a resident plan, with the autotuned executor.  Every variant's solution
must equal the serial one bit for bit, or the exit status is 1.

The CSV row has the demo's columns -- Matrix Name, Metis Enabled (always
"No": no reordering here), Number of Threads (the LBC part count), p2, p3,
Serial Non-fused, Parallel Levelset CSC, Parallel LBC CSR (seconds) -- and
one more, GPU Plan Solve.
"""
from __future__ import annotations

import argparse
import os
import statistics
import sys
import time

import numpy as np

from . import matgen as mg
from . import sym_lib
from .mtx import lower_triangle

HEADER = ("Matrix Name,Metis Enabled,Number of Threads,p2,p3,Serial Non-fused,Parallel Levelset CSC,"
          "Parallel LBC CSR,GPU Plan Solve,")


def _random_lower(n=16, density=0.2, seed=0):
    rng = np.random.default_rng(seed)
    mask = np.tril(rng.random((n, n)) < density, -1)
    r, c = np.nonzero(mask)
    vals = -rng.random(len(r))
    rr = np.concatenate([r, np.arange(n)])
    cc = np.concatenate([c, np.arange(n)])
    vv = np.concatenate([vals, 2.0 + np.abs(vals).sum() / max(n, 1) + rng.random(n)])
    import scipy.sparse as sp
    L = mg.from_scipy(sp.csr_matrix((vv, (rr, cc)), shape=(n, n)))
    Lc = mg.from_scipy(sp.csr_matrix((vv, (cc, rr)), shape=(n, n)))
    return L, Lc


def _median_time(fn, reps=5):
    ts = []
    out = None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts), out


def run(path=None, p2=-1, p3=4000, parts=None, header=False, out=sys.stdout) -> int:
    if path:
        L, Lc = lower_triangle(path)
        name = os.path.basename(path)
    else:
        L, Lc = _random_lower()
        name = "Random_%d" % L.n
    n = L.n
    parts = parts or (os.cpu_count() or 1)
    b = np.random.default_rng(1).uniform(-1.0, 1.0, n)

    def serial():
        x = b.copy()
        sym_lib.sptrsv_csr(n, L.p, L.i, L.x, x)
        return x

    t_ser, x_ser = _median_time(serial)

    nl, lp, ls = sym_lib.build_levelSet_CSC(n, Lc.p, Lc.i)

    def levelset():
        x = b.copy()
        sym_lib.sptrsv_csc_levelset(n, Lc.p, Lc.i, Lc.x, x, nl, lp, ls)
        return x

    t_lvl, x_lvl = _median_time(levelset)

    cl, clp, pn, cpp, nodes = sym_lib.get_coarse_levelSet_DAG_CSC_tree(n, L.p, L.i, 0, parts, p2, p3)

    def lbc():
        x = b.copy()
        sym_lib.sptrsv_csr_lbc(n, L.p, L.i, L.x, x, cl, clp, cpp, nodes)
        return x

    t_lbc, x_lbc = _median_time(lbc)

    t_plan = float("nan")
    try:
        import torch
        from .plans import TriPlan
        plan = TriPlan(n, *L.astuple())
        plan.autotune(k=1)
        xd = torch.from_numpy(b).cuda()
        w = torch.empty_like(xd)
        ts = []
        for _ in range(6):
            w.copy_(xd)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            plan.solve(w)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        plan.check()
        t_plan = statistics.median(ts[1:])
        same_plan = np.array_equal(w.cpu().numpy(), x_ser)
    except ImportError:
        same_plan = True
    ok = np.array_equal(x_lvl, x_ser) and np.array_equal(x_lbc, x_ser) and same_plan
    if header:
        print(HEADER, file=out)
    print("%s,No,%d,%d,%d,%.9g,%.9g,%.9g,%.9g," % (name, parts, p2, p3, t_ser, t_lvl, t_lbc, t_plan), file=out)
    if not ok:
        print("error: a variant's solution differs from the serial one", file=sys.stderr)
        return 1
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("matrix", nargs="?", help="MatrixMarket file (omit for the random 16 x 16 case)")
    ap.add_argument("p2", nargs="?", type=int, default=-1, help="LBC minimum level distance (demo default -1)")
    ap.add_argument("p3", nargs="?", type=int, default=4000, help="LBC division rate (demo default 4000)")
    ap.add_argument("--parts", type=int, default=None, help="LBC parts per coarse level (default: host cores)")
    ap.add_argument("--header", action="store_true", help="print the CSV header first")
    a = ap.parse_args(argv)
    return run(a.matrix, a.p2, a.p3, a.parts, a.header)


if __name__ == "__main__":
    sys.exit(main())
