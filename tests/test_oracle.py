"""The oracle (C restatement of the reference) against the reference's own
known answers: the Catch2 hand vectors, fixtures recorded from the compiled
reference, and -- where the reference tree is present -- the compiled
reference itself on fresh inputs."""
import numpy as np
import pytest

from conftest import golden
from sympiler_gb300 import matgen as mg


def test_catch_spmv_known_answers(orc):
    for name in ("catch_spmv_4x4", "catch_spmv_10x10"):
        d = golden(name)
        n = len(d["Ap"]) - 1
        y = np.zeros(n)
        orc.spmv_csr(n, d["Ap"], d["Ai"], d["Ax"], d["x"], y)
        assert np.array_equal(y, d["z"])


def test_catch_sptrsv_known_answer(orc):
    d = golden("catch_sptrsv_10x10")
    n = 10
    x = d["b"].copy()
    orc.sptrsv_csc(n, d["Lp"], d["Li"], d["Lx"], x)
    assert np.array_equal(x, d["x"])
    L = mg.transpose(mg.CSR(n, d["Lp"], d["Li"], d["Lx"]))
    x = d["b"].copy()
    orc.sptrsv_csr(n, *L.astuple(), x)
    assert np.array_equal(x, d["x"])


def test_c1_fixture_bit_exact(orc):
    d = golden("c1_lap2d_100")
    n = len(d["Lp"]) - 1
    x = d["b"].copy()
    orc.sptrsv_csr(n, d["Lp"], d["Li"], d["Lx"], x)
    assert np.array_equal(x, d["x"])
    nl, lp, ls = orc.build_levelset_csr(n, d["Lp"], d["Li"])
    assert nl == 199
    assert np.array_equal(lp, d["level_ptr"]) and np.array_equal(ls, d["level_set"])
    x = d["b"].copy()
    orc.sptrsv_csr_levelset(n, d["Lp"], d["Li"], d["Lx"], x, nl, lp, ls, 1)
    assert np.array_equal(x, d["x_levelset"])
    y = np.zeros(n)
    orc.spmv_csr(n, d["Ap"], d["Ai"], d["Ax"], d["v"], y)
    assert np.array_equal(y, d["y"])
    z = d["z0"].copy()
    orc.spmv_csr_axpby(n, d["Ap"], d["Ai"], d["Ax"], d["v"], d["b"], z, float(d["a"]), float(d["bb"]))
    assert np.array_equal(z, d["z"])


def test_random_lower_fixture(orc):
    d = golden("random_lower")
    for n in (10, 100, 500, 1000, 10000):
        x = np.ones(n)
        orc.sptrsv_csr(n, d["n%d_p" % n], d["n%d_i" % n], d["n%d_x" % n], x)
        assert np.array_equal(x, d["n%d_sol" % n])


def test_ic0_fixture(orc):
    d = golden("ic0_lap3d_10")
    n = len(d["Up"]) - 1
    f, ok = orc.spic0_csr(n, d["Up"], d["Ui"], d["Ux"])
    assert ok and np.array_equal(f, d["factor"])
    x = d["b"].copy()
    orc.ltsolve(n, d["Up"], d["Ui"], d["factor"], x)
    assert np.array_equal(x, d["x_ltsolve"])
    x = d["b"].copy()
    orc.sptrsv_csc(n, d["Up"], d["Ui"], d["factor"], x)
    assert np.array_equal(x, d["x_csc"])
    nl, lp, ls = orc.tree_levelset(n, d["etree"])
    assert nl == int(d["tree_levels"])
    assert np.array_equal(lp, d["tree_level_ptr"]) and np.array_equal(ls, d["tree_level_set"])


def test_lbc_fixture(orc):
    d = golden("ic0_random_spd_2000")
    n = len(d["Up"]) - 1
    f, ok = orc.spic0_csr(n, d["Up"], d["Ui"], d["Ux"])
    assert ok and np.array_equal(f, d["factor"])
    L = mg.transpose(mg.CSR(n, d["Up"], d["Ui"], d["factor"]))
    x = d["b"].copy()
    orc.sptrsv_csr(n, *L.astuple(), x)
    assert np.array_equal(x, d["x_serial"])
    x = d["b"].copy()
    orc.sptrsv_csr_lbc(n, *L.astuple(), x, int(d["lbc_level_no"]), d["lbc_level_ptr"], d["lbc_par_ptr"],
                       d["lbc_partition"])
    assert np.array_equal(x, d["x_lbc"])
    x = np.zeros(n)
    orc.sptrsv_csr_lbc_redundant(n, *L.astuple(), x, d["b"], int(d["lbc_level_no"]), d["lbc_level_ptr"],
                                 d["lbc_par_ptr"], d["lbc_partition"])
    assert np.array_equal(x, d["x_lbc_redundant"])
    nl, lp, ls = orc.tree_levelset(n, d["etree"])
    assert nl == int(d["tree_levels"])
    assert np.array_equal(lp, d["tree_level_ptr"]) and np.array_equal(ls, d["tree_level_set"])


def test_ilu0_fixture(orc):
    d = golden("ilu0_convdiff_8")
    n = len(d["Ap"]) - 1
    lu, ok = orc.spilu0_csr(n, d["Ap"], d["Ai"], d["Ax"], d["diag"])
    assert ok and np.array_equal(lu, d["lu"])
    assert np.array_equal(orc.lus_cr(n, d["Ap"], d["Ai"], lu, d["diag"], d["r"]), d["z"])
    x = d["r"].copy()
    orc.sptrsv_csr_ilu(n, d["Ap"], d["Ai"], lu, d["diag"], x)
    assert np.array_equal(x, d["x_ilu"])


@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_vs_compiled_reference(orc, ref, seed):
    rng = np.random.default_rng(seed)
    A = mg.convdiff3d(9)
    L = mg.tril(A)
    b = rng.uniform(-1, 1, A.n)
    x1, x2 = b.copy(), b.copy()
    orc.sptrsv_csr(A.n, *L.astuple(), x1)
    ref.sptrsv_csr(A.n, *L.astuple(), x2)
    assert np.array_equal(x1, x2)
    d = mg.diag_ptr(A)
    l1, _ = orc.spilu0_csr(A.n, A.p, A.i, A.x, d)
    l2 = ref.spilu0_csr(A.n, A.p, A.i, A.x, d)
    assert np.array_equal(l1, l2)
    assert np.array_equal(orc.lus_cr(A.n, A.p, A.i, l1, d, b), ref.lus_cr(A.n, A.p, A.i, l1, d, b))
    y1, y2 = np.zeros(A.n), np.zeros(A.n)
    orc.spmv_csr(A.n, *A.astuple(), b, y1)
    ref.spmv_csr(A.n, *A.astuple(), b, y2)
    assert np.array_equal(y1, y2)


def test_levelset_restatement_properties(orc):
    """Every dependency sits in an earlier level; rows ascend inside a level."""
    rng = np.random.default_rng(5)
    T = mg.random_lower(3000, 0.002, rng)
    nl, lp, ls = orc.build_levelset_csr(T.n, T.p, T.i)
    lev = np.empty(T.n, dtype=np.int64)
    for l in range(nl):
        seg = ls[lp[l]:lp[l + 1]]
        assert np.all(np.diff(seg) > 0)
        lev[seg] = l
    rows = np.repeat(np.arange(T.n), np.diff(T.p))
    off = T.i != rows
    assert np.all(lev[T.i[off]] < lev[rows[off]])
    # CSC variant gives the same schedule
    C = mg.transpose(T)
    nl2, lp2, ls2 = orc.build_levelset_csc(C.n, C.p, C.i)
    assert nl2 == nl and np.array_equal(lp, lp2) and np.array_equal(ls, ls2)


def test_pcg_and_gmres_oracles_converge(orc):
    A = mg.lap3d(8, 1e-2)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    Lt = mg.CSR(U.n, U.p, U.i, f)
    Lf = mg.transpose(Lt)
    rng = np.random.default_rng(3)
    xs = rng.standard_normal(A.n)
    b = A.scipy() @ xs
    x, it, rel = orc.pcg_ic0(A.n, A.astuple(), Lf.astuple(), Lt.astuple(), b, 1e-10, 500)
    assert rel <= 1e-10 and np.allclose(x, xs, atol=1e-7)
    C = mg.convdiff3d(8)
    d = mg.diag_ptr(C)
    lu, _ = orc.spilu0_csr(C.n, C.p, C.i, C.x, d)
    bc = rng.uniform(-1, 1, C.n)
    x, it, rel = orc.gmres_ilu0(C.n, C.astuple(), lu, d, bc, 30, 100, 1e-10)
    assert rel < 1e-9


def test_reference_lbc_factorisations_vs_serial_oracle(orc, ref):
    """The compiled reference's LBC factorisations against the serial oracle:
    spilu0_csr_lbc's rows do not depend on the schedule, so it equals
    spilu0_csr bit for bit; spic0_csr_lbc subtracts under `omp atomic`, so
    its order of updates (and its rounding) can differ run to run: within
    1e-12 of the serial factor."""
    from sympiler_gb300 import sym_lib
    A = mg.convdiff3d(10)
    d = mg.diag_ptr(A)
    Lpat = mg.tril(A)
    nl, lp, pn, pp, nodes = sym_lib.get_coarse_levelSet_DAG_CSC_tree(A.n, Lpat.p, Lpat.i, 0, 4, -1, 100)
    serial, ok = orc.spilu0_csr(A.n, A.p, A.i, A.x, d)
    assert ok
    assert np.array_equal(ref.spilu0_csr_lbc(A.n, A.p, A.i, A.x, d, nl, lp, pp, nodes), serial)
    S = mg.lap3d(10, 1e-2)
    U = mg.triu(S)
    L = mg.transpose(U)
    nl, lp, pn, pp, nodes = sym_lib.get_coarse_levelSet_DAG_CSC_tree(U.n, L.p, L.i, 0, 4, -1, 100)
    serial, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    assert ok
    lbc = ref.spic0_csr_lbc(U.n, U.p, U.i, U.x, nl, lp, pp, nodes)
    assert np.allclose(lbc, serial, rtol=1e-12, atol=0)
