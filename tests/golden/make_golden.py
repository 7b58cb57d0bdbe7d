"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a checkout where the sympiler/sympiler source tree is available
(default /root/reference, or GBSYM_REFERENCE_ROOT):

    python tests/golden/make_golden.py

It (1) extracts the hand-written known-answer vectors of the reference's
Catch2 tests (Catch_tests/spmv_tests.cpp, Catch_tests/sptrsv_tests.cpp),
reading the test sources as text, and (2) compiles the reference's own
executors (oracle/build.py -> oracle/_ref/libsymref.so) and records their
outputs on seeded synthetic inputs.  The fixtures are small .npz files; the
GPU tests read them where the reference tree is absent.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import build as obuild  # noqa: E402
from sympiler_gb300 import matgen as mg  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("GBSYM_REFERENCE_ROOT", obuild.DEFAULT_REFERENCE_ROOT)


def _c_array(text, decl):
    """Numbers of the C initialiser `decl = {...};` in text."""
    m = re.search(re.escape(decl) + r"\s*=\s*\{([^}]*)\}", text)
    if not m:
        raise RuntimeError("array %s not found" % decl)
    return [float(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]


def catch_vectors():
    spmv = open(os.path.join(REF_ROOT, "Catch_tests", "spmv_tests.cpp")).read()
    trsv = open(os.path.join(REF_ROOT, "Catch_tests", "sptrsv_tests.cpp")).read()
    s1 = spmv[spmv.index('SECTION("Small SPMV1")'):spmv.index('SECTION("Small SPMV2")')]
    s2 = spmv[spmv.index('SECTION("Small SPMV2")'):spmv.index('SECTION("SpMV CSR, parallel')]
    t1 = trsv[trsv.index('SECTION("Small SPTRSV1")'):trsv.index('SECTION("Sptrsv CSR, parallel')]
    np.savez(os.path.join(OUT, "catch_spmv_4x4.npz"),
             Ap=np.array(_c_array(s1, "int Ap[5]"), dtype=np.int32),
             Ai=np.array(_c_array(s1, "int Ai[6]"), dtype=np.int32),
             Ax=np.array(_c_array(s1, "double Ax[6]"), dtype=np.float64),
             x=np.array(_c_array(s1, "double x[4]"), dtype=np.float64),
             z=np.array(_c_array(s1, "double z[4]"), dtype=np.float64))
    np.savez(os.path.join(OUT, "catch_spmv_10x10.npz"),
             Ap=np.array(_c_array(s2, "int Ap[11]"), dtype=np.int32),
             Ai=np.array(_c_array(s2, "int Ai[44]"), dtype=np.int32),
             Ax=np.ones(44), x=np.array(_c_array(s2, "double x[10]"), dtype=np.float64),
             z=np.array(_c_array(s2, "double z[10]"), dtype=np.float64))
    np.savez(os.path.join(OUT, "catch_sptrsv_10x10.npz"),
             Lp=np.array(_c_array(t1, "int Lp[11]"), dtype=np.int32),
             Li=np.array(_c_array(t1, "int Li[26]"), dtype=np.int32),
             Lx=np.ones(26), b=np.array(_c_array(t1, "double b0[10]"), dtype=np.float64),
             x=np.ones(10))


def etree_upper(n, Up, Ui):
    """Elimination tree of A from its upper CSR (= lower CSC): Liu's
    algorithm with path compression."""
    parent = np.full(n, -1, dtype=np.int32)
    anc = np.full(n, -1, dtype=np.int64)
    # column j of the upper triangle lists rows i < j: use the transpose
    T = mg.transpose(mg.CSR(n, Up, Ui, np.ones(len(Ui))))
    for j in range(n):
        for e in range(T.p[j], T.p[j + 1]):
            i = int(T.i[e])
            while i != -1 and i < j:
                nxt = anc[i]
                anc[i] = j
                if nxt == -1:
                    parent[i] = j
                i = nxt
    return parent


def main():
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("reference tree not found at %s" % REF_ROOT)
    orc = oracle.orc()
    catch_vectors()
    rng = np.random.default_rng(20240611)

    # C1: 2D 5-point Laplacian 100x100 -- forward solve, level set, SpMV
    A = mg.lap2d(100)
    L = mg.tril(A)
    b = rng.uniform(-1, 1, A.n)
    v = rng.uniform(-1, 1, A.n)
    x = b.copy()
    ref.sptrsv_csr(L.n, *L.astuple(), x)
    nl, lp, ls = orc.build_levelset_csr(L.n, L.p, L.i)
    xl = b.copy()
    ref.sptrsv_csr_levelset(L.n, *L.astuple(), xl, nl, lp, ls)
    y = np.zeros(A.n)
    ref.spmv_csr(A.n, *A.astuple(), v, y)
    z0 = rng.uniform(-1, 1, A.n)
    z = z0.copy()
    ref.spmv_csr_axpby(A.n, *A.astuple(), v, b, z, 0.75, -1.25)
    np.savez_compressed(os.path.join(OUT, "c1_lap2d_100.npz"), Ap=A.p, Ai=A.i, Ax=A.x, Lp=L.p, Li=L.i,
                        Lx=L.x, b=b, x=x, x_levelset=xl, level_ptr=lp, level_set=ls, v=v, y=y, z0=z0,
                        z=z, a=0.75, bb=-1.25)

    # random lower triangles at the (n, density) list of the reference's
    # serial-vs-parallel test (Catch_tests/sptrsv_tests.cpp:47-51)
    rl = {}
    for n, dens in [(10, 0.2), (100, 0.03), (500, 0.004), (1000, 0.0005), (10000, 0.0001)]:
        T = mg.random_lower(n, dens, rng)
        bb = np.ones(n)
        xs = bb.copy()
        ref.sptrsv_csr(n, *T.astuple(), xs)
        rl["n%d_p" % n], rl["n%d_i" % n], rl["n%d_x" % n], rl["n%d_sol" % n] = T.p, T.i, T.x, xs
    np.savez_compressed(os.path.join(OUT, "random_lower.npz"), **rl)

    # IC0 of a 3D 7-point Laplacian 10^3 + 1e-2 I; L^T solve; CSC solve; LBC
    A3 = mg.lap3d(10, 1e-2)
    U = mg.triu(A3)
    f = ref.spic0_csr(U.n, U.p, U.i, U.x)
    bb = rng.standard_normal(U.n)
    xt = bb.copy()
    ref.ltsolve(U.n, U.p, U.i, f, xt)
    xc = bb.copy()
    ref.sptrsv_csc(U.n, U.p, U.i, f, xc)
    Lcsr = mg.transpose(mg.CSR(U.n, U.p, U.i, f))
    parent = etree_upper(U.n, U.p, U.i)
    cost = np.diff(Lcsr.p).astype(np.float64)
    nlev, clp, cpp, cpart = ref.coarse_levelset6(U.n, parent, cost, 4, -1, 4000)
    xlbc = bb.copy()
    ref.sptrsv_csr_lbc(U.n, *Lcsr.astuple(), xlbc, nlev, clp, cpp, cpart)
    tl, tlp, tls = ref.tree_levelset(U.n, parent)
    np.savez_compressed(os.path.join(OUT, "ic0_lap3d_10.npz"), Up=U.p, Ui=U.i, Ux=U.x, factor=f, b=bb,
                        x_ltsolve=xt, x_csc=xc, etree=parent, lbc_level_no=nlev, lbc_level_ptr=clp,
                        lbc_par_ptr=cpp, lbc_partition=cpart, x_lbc=xlbc, tree_levels=tl,
                        tree_level_ptr=tlp, tree_level_set=tls)

    # IC0 of a random SPD matrix whose elimination tree is bushy, with the
    # reference's tree level set and tree LBC schedule (many partitions)
    R = mg.random_spd(2000, 4, rng)
    UR = mg.triu(R)
    fr = ref.spic0_csr(UR.n, UR.p, UR.i, UR.x)
    LR = mg.transpose(mg.CSR(UR.n, UR.p, UR.i, fr))
    par = etree_upper(UR.n, UR.p, UR.i)
    costr = np.diff(LR.p).astype(np.float64)
    rn, rlp, rpp, rpart = ref.coarse_levelset6(UR.n, par, costr, 4, -1, 100)
    br = rng.standard_normal(UR.n)
    xs_r = br.copy()
    ref.sptrsv_csr(UR.n, *LR.astuple(), xs_r)
    xl_r = br.copy()
    ref.sptrsv_csr_lbc(UR.n, *LR.astuple(), xl_r, rn, rlp, rpp, rpart)
    xr_r = np.zeros(UR.n)
    ref.sptrsv_csr_lbc_redundant(UR.n, *LR.astuple(), xr_r, br, rn, rlp, rpp, rpart)
    tln, tlp2, tls2 = ref.tree_levelset(UR.n, par)
    np.savez_compressed(os.path.join(OUT, "ic0_random_spd_2000.npz"), Up=UR.p, Ui=UR.i, Ux=UR.x,
                        factor=fr, b=br, x_serial=xs_r, x_lbc=xl_r, x_lbc_redundant=xr_r, etree=par,
                        lbc_level_no=rn, lbc_level_ptr=rlp, lbc_par_ptr=rpp, lbc_partition=rpart,
                        tree_levels=tln, tree_level_ptr=tlp2, tree_level_set=tls2)

    # ILU0 of a 3D convection-diffusion 8^3; ILU apply (lus_cr)
    Cd = mg.convdiff3d(8)
    d = mg.diag_ptr(Cd)
    lu = ref.spilu0_csr(Cd.n, Cd.p, Cd.i, Cd.x, d)
    r = rng.uniform(-1, 1, Cd.n)
    zz = ref.lus_cr(Cd.n, Cd.p, Cd.i, lu, d, r)
    xi = r.copy()
    ref.sptrsv_csr_ilu(Cd.n, Cd.p, Cd.i, lu, d, xi)
    np.savez_compressed(os.path.join(OUT, "ilu0_convdiff_8.npz"), Ap=Cd.p, Ai=Cd.i, Ax=Cd.x, diag=d,
                        lu=lu, r=r, z=zz, x_ilu=xi)
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
