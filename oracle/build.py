"""Build recipe for the oracle (test infrastructure only).

Two shared libraries:

* ``oracle/_build/liboracle.so`` -- the project's C restatement
  (``oracle/oracle.c``).  Built everywhere, including the GPU host, since it
  is the oracle of the parity tests and the CPU baseline of the benchmark.
* ``oracle/_ref/libsymref.so`` -- the reference's own C++ executors,
  compiled in place from the sympiler/sympiler source tree (never copied)
  together with ``oracle/ref_capi.cpp`` and the project-written
  ``oracle/ref_shim/aggregation/def.h``.  Built only where that source tree
  exists; it is used to pin the restatement.

Flags: ``-O3 -fopenmp -std=c++11 -ffp-contract=off``.  The reference's own
``-march=x86-64 -mavx2`` is dropped (the GPU host is aarch64), and
``-ffp-contract=off`` keeps "a - b*c" as a rounded multiply and a rounded
subtract on every architecture, matching the reference's x86-64 build.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "liboracle.so")
REF_SO = os.path.join(REF_DIR, "libsymref.so")

DEFAULT_REFERENCE_ROOT = "/root/reference"

# Reference translation units on the triangular-solve path.
REF_SOURCES = [
    "sparse_blas/sptrsv.cpp",
    "sparse_blas/spmv.cpp",
    "sparse_blas/spilu0.cpp",
    "sparse_blas/spic0.cpp",
    "sparse_blas/sptrsv_lt.cpp",
    "sparse_blas/dense_blas/BLAS.cpp",
    "sparse_blas/parsy/triangularSolve/Triangular_CSC.cpp",
    "sparse_blas/parsy/common/TreeUtils.cpp",
    "sparse_blas/parsy/common/Norm.cpp",
    "sparse_blas/parsy/symbolic/InspectionLevel_06.cpp",
    "sparse_blas/parsy/symbolic/PostOrderSpliting.cpp",
    "sparse_blas/parsy/matrixVector/spmv_CSC.cpp",
    "sparse_blas/parsy/gmres/mgmres.cpp",
    "sparse_blas/parsy/triangularSolve/Triangular_BCSC.cpp",
    "sparse_blas/parsy/triangularSolve/BLAS.cpp",
]

# The supernodal solves are built with the reference's own dense kernels
# (SYM_BLAS); the external-BLAS calls of their other forms are routed to an
# aborting stub declared by ref_shim/missing_blas.h.
EXTRA_FLAGS = {
    "sparse_blas/parsy/triangularSolve/Triangular_BCSC.cpp": [
        "-DSYM_BLAS", "-DSYM_DTRSM=ref_blas_missing", "-DSYM_DGEMM=ref_blas_missing",
        "-DSYM_DGEMV=ref_blas_missing", "-DSET_BLAS_THREAD(t)=((void)(t))",
        "-include", os.path.join(HERE, "ref_shim", "missing_blas.h")],
}

FLAGS = ["-O3", "-fopenmp", "-fPIC", "-ffp-contract=off"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement into ``oracle/_build/liboracle.so``."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if force or _stale(ORACLE_SO, [src, hdr, __file__]):
        _run(["gcc", "-std=c11", *FLAGS, "-shared", src, "-o", ORACLE_SO, "-lm"])
    return ORACLE_SO


def build_reference(reference_root: str | None = None, force: bool = False):
    """Compile the reference's executors into ``oracle/_ref/libsymref.so``.

    Returns the library path, or None when the reference tree is absent.
    """
    root = reference_root or os.environ.get("GBSYM_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT)
    if not os.path.isdir(os.path.join(root, "sparse_blas")):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    capi = os.path.join(HERE, "ref_capi.cpp")
    shim = os.path.join(HERE, "ref_shim", "aggregation", "def.h")
    blas_shim = os.path.join(HERE, "ref_shim", "missing_blas.h")
    srcs = [os.path.join(root, s) for s in REF_SOURCES]
    if not (force or _stale(REF_SO, srcs + [capi, shim, blas_shim, __file__])):
        return REF_SO
    inc = ["-I" + os.path.join(HERE, "ref_shim"), "-I" + os.path.join(root, "include"),
           "-I" + os.path.join(root, "include", "sympiler"),
           "-I" + os.path.join(root, "include", "sympiler", "parsy")]
    objs = []
    jobs = []
    for s, rel in list(zip(srcs, REF_SOURCES)) + [(capi, None)]:
        o = os.path.join(REF_DIR, (rel or "ref_capi.cpp").replace("/", "_").replace(".cpp", ".o"))
        objs.append(o)
        jobs.append(["g++", "-std=c++11", "-DENABLE_OPENMP", *FLAGS, *EXTRA_FLAGS.get(rel, []), *inc,
                     "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        list(ex.map(_run, jobs))
    _run(["g++", "-shared", "-fopenmp", *objs, "-o", REF_SO, "-Wl,--no-undefined", "-lm"])
    for o in objs:
        os.remove(o)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
