"""GPU triangular solves through the C ABI against the reference's known
answers and the oracle.  FP64 rows are accumulated in the reference's order
without contraction, so the comparisons are bit-exact."""
import numpy as np
import pytest

from conftest import golden
from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def test_catch_known_answer(gpu):
    from sympiler_gb300 import sym_lib
    d = golden("catch_sptrsv_10x10")
    x = d["b"].copy()
    sym_lib.sptrsv_csc(10, d["Lp"], d["Li"], d["Lx"], x)
    assert np.array_equal(x, d["x"])
    L = mg.transpose(mg.CSR(10, d["Lp"], d["Li"], d["Lx"]))
    x = d["b"].copy()
    sym_lib.sptrsv_csr(10, *L.astuple(), x)
    assert np.array_equal(x, d["x"])
    x = d["b"].copy()
    assert sym_lib.parsy.lsolve(10, d["Lp"], d["Li"], d["Lx"], x) == 1
    assert np.array_equal(x, d["x"])


def test_c1_serial_and_levelset(gpu):
    from sympiler_gb300 import sym_lib
    d = golden("c1_lap2d_100")
    n = len(d["Lp"]) - 1
    x = d["b"].copy()
    sym_lib.sptrsv_csr(n, d["Lp"], d["Li"], d["Lx"], x)
    assert np.array_equal(x, d["x"])
    x = d["b"].copy()
    sym_lib.sptrsv_csr_levelset(n, d["Lp"], d["Li"], d["Lx"], x, len(d["level_ptr"]) - 1,
                                d["level_ptr"], d["level_set"])
    assert np.array_equal(x, d["x_levelset"])


def test_gpu_schedule_builder_bit_exact(gpu, orc):
    from sympiler_gb300 import sym_lib
    d = golden("c1_lap2d_100")
    n = len(d["Lp"]) - 1
    nl, lp, ls = sym_lib.build_levelset_csr(n, d["Lp"], d["Li"])
    assert nl == 199 and np.array_equal(lp, d["level_ptr"]) and np.array_equal(ls, d["level_set"])
    C = mg.transpose(mg.CSR(n, d["Lp"], d["Li"], d["Lx"]))
    nl2, lp2, ls2 = sym_lib.build_levelSet_CSC(n, C.p, C.i)
    assert nl2 == nl and np.array_equal(lp2, lp) and np.array_equal(ls2, ls)
    rng = np.random.default_rng(11)
    for n, dens in [(10, 0.2), (500, 0.004), (20000, 0.0003)]:
        T = mg.random_lower(n, dens, rng)
        a = orc.build_levelset_csr(n, T.p, T.i)
        b = sym_lib.build_levelset_csr(n, T.p, T.i)
        assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
        U = mg.transpose(T)
        a = orc.build_levelset_upper_csr(n, U.p, U.i)
        b = sym_lib.build_levelset_upper_csr(n, U.p, U.i)
        assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_tree_levelset_fixture_via_builder(gpu):
    """The reference's parsy::getLevelSet on an etree equals the DAG level set
    of the tree's child->parent edges."""
    from sympiler_gb300 import sym_lib
    d = golden("ic0_random_spd_2000")
    par = d["etree"]
    n = len(par)
    # row p lists its children: CSR with entries (parent, child)
    rows = par[par >= 0]
    cols = np.nonzero(par >= 0)[0]
    import scipy.sparse as sp
    T = mg.from_scipy(sp.coo_matrix((np.ones(len(rows)), (rows, cols)), shape=(n, n)))
    nl, lp, ls = sym_lib.build_levelset_csr(n, T.p, T.i)
    assert nl == int(d["tree_levels"])
    assert np.array_equal(lp, d["tree_level_ptr"]) and np.array_equal(ls, d["tree_level_set"])


def test_random_lower_differential(gpu):
    from sympiler_gb300 import sym_lib
    d = golden("random_lower")
    for n in (10, 100, 500, 1000, 10000):
        x = np.ones(n)
        sym_lib.sptrsv_csr(n, d["n%d_p" % n], d["n%d_i" % n], d["n%d_x" % n], x)
        assert np.array_equal(x, d["n%d_sol" % n]), n


def test_ic0_fixture_solves(gpu):
    from sympiler_gb300 import sym_lib
    d = golden("ic0_lap3d_10")
    n = len(d["Up"]) - 1
    x = d["b"].copy()
    assert sym_lib.ltsolve(n, d["Up"], d["Ui"], d["factor"], x) == 1
    assert np.array_equal(x, d["x_ltsolve"])
    x = d["b"].copy()
    assert sym_lib.parsy.ltsolve(n, d["Up"], d["Ui"], d["factor"], x) == 1
    assert np.array_equal(x, d["x_ltsolve"])
    x = d["b"].copy()
    sym_lib.sptrsv_csc(n, d["Up"], d["Ui"], d["factor"], x)
    assert np.array_equal(x, d["x_csc"])


def test_lbc_schedule_from_reference(gpu, orc):
    from sympiler_gb300 import sym_lib
    d = golden("ic0_random_spd_2000")
    n = len(d["Up"]) - 1
    L = mg.transpose(mg.CSR(n, d["Up"], d["Ui"], d["factor"]))
    sched = (int(d["lbc_level_no"]), d["lbc_level_ptr"], d["lbc_par_ptr"], d["lbc_partition"])
    x = d["b"].copy()
    sym_lib.sptrsv_csr_lbc(n, *L.astuple(), x, *sched)
    assert np.array_equal(x, d["x_lbc"])
    x = np.zeros(n)
    sym_lib.sptrsv_csr_lbc_redundant(n, *L.astuple(), x, d["b"], *sched)
    assert np.array_equal(x, d["x_lbc_redundant"])
    # CSC LBC and parsy::lsolveParH2 on the CSC of the same factor
    x = d["b"].copy()
    sym_lib.sptrsv_csc_lbc(n, d["Up"], d["Ui"], d["factor"], x, *sched)
    assert np.array_equal(x, d["x_serial"])
    x = d["b"].copy()
    assert sym_lib.parsy.lsolveParH2(n, d["Up"], d["Ui"], d["factor"], x, sched[0], sched[1], None,
                                     len(sched[2]) - 1, sched[2], sched[3]) == 1
    assert np.array_equal(x, d["x_serial"])
    # CSC level set
    nl, lp, ls = orc.build_levelset_csc(n, d["Up"], d["Ui"])
    x = d["b"].copy()
    sym_lib.sptrsv_csc_levelset(n, d["Up"], d["Ui"], d["factor"], x, nl, lp, ls)
    assert np.array_equal(x, d["x_serial"])
    x = d["b"].copy()
    assert sym_lib.parsy.lsolvePar(n, d["Up"], d["Ui"], d["factor"], x, nl, lp, ls) == 1
    assert np.array_equal(x, d["x_serial"])


def test_dag_lbc_schedule_drives_gpu_drop_ins(gpu, orc):
    """The library's own DAG LBC inspector feeding its LBC drop-ins, as the
    reference demo chains get_coarse_levelSet_DAG_CSC_tree into
    sptrsv_csr_lbc: results equal the serial oracle's bits."""
    from sympiler_gb300 import sym_lib
    d = golden("ic0_random_spd_2000")
    n = len(d["Up"]) - 1
    L = mg.transpose(mg.CSR(n, d["Up"], d["Ui"], d["factor"]))
    for parts in (2, 6, 64):
        nl, lp, pn, pp, nodes = sym_lib.get_coarse_levelSet_DAG_CSC_tree(n, L.p, L.i, 0, parts, -1, 100)
        x = d["b"].copy()
        sym_lib.sptrsv_csr_lbc(n, *L.astuple(), x, nl, lp, pp, nodes)
        assert np.array_equal(x, d["x_serial"])
        x = d["b"].copy()
        sym_lib.sptrsv_csc_lbc(n, d["Up"], d["Ui"], d["factor"], x, nl, lp, pp, nodes)
        assert np.array_equal(x, d["x_serial"])


def test_ilu_solves(gpu, orc):
    from sympiler_gb300 import sym_lib
    d = golden("ilu0_convdiff_8")
    n = len(d["Ap"]) - 1
    x = d["r"].copy()
    sym_lib.sptrsv_csr_ilu(n, d["Ap"], d["Ai"], d["lu"], d["diag"], x)
    assert np.array_equal(x, d["x_ilu"])
    z = np.zeros(n)
    sym_lib.parsy.lus_cr(n, int(d["Ap"][n]), d["Ap"], d["Ai"], d["lu"], d["diag"], d["r"], z)
    assert np.array_equal(z, d["z"])
    # ilu_lbc divides by the diagonal: compare with the oracle on a band LBC
    nl, lp, ls = orc.build_levelset_csr(n, *mg.tril(mg.CSR(n, d["Ap"], d["Ai"], d["lu"])).astuple()[:2])
    level_ptr = np.arange(nl + 1, dtype=np.int32)  # one partition per level
    x1, x2 = d["r"].copy(), d["r"].copy()
    orc.sptrsv_csr_ilu_lbc(n, d["Ap"], d["Ai"], d["lu"], d["diag"], x1, nl, level_ptr, lp, ls)
    sym_lib.sptrsv_csr_ilu_lbc(n, d["Ap"], d["Ai"], d["lu"], d["diag"], x2, nl, level_ptr, lp, ls)
    assert np.array_equal(x1, x2)


def test_bad_schedule_and_bad_matrix_are_rejected(gpu):
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import ERR_BAD_MATRIX, ERR_BAD_SCHEDULE, GbsymError
    d = golden("c1_lap2d_100")
    n = len(d["Lp"]) - 1
    lp, ls = d["level_ptr"].copy(), d["level_set"].copy()
    # swap two rows across levels 0 and 1: a dependency now sits in a later level
    ls[0], ls[lp[1]] = ls[lp[1]], ls[0]
    x = d["b"].copy()
    with pytest.raises(GbsymError) as e:
        sym_lib.sptrsv_csr_levelset(n, d["Lp"], d["Li"], d["Lx"], x, len(lp) - 1, lp, ls)
    assert e.value.status == ERR_BAD_SCHEDULE
    assert np.array_equal(x, d["b"])  # untouched on error
    # duplicate row in the level set
    ls2 = d["level_set"].copy()
    ls2[5] = ls2[6]
    with pytest.raises(GbsymError) as e:
        sym_lib.sptrsv_csr_levelset(n, d["Lp"], d["Li"], d["Lx"], x, len(lp) - 1, lp, ls2)
    assert e.value.status == ERR_BAD_SCHEDULE
    # LBC with two dependent rows in different partitions of one coarse level
    lvl = np.array([0, 2], dtype=np.int32)
    part_ptr = np.array([0, n // 2, n], dtype=np.int32)
    with pytest.raises(GbsymError) as e:
        sym_lib.sptrsv_csr_lbc(n, d["Lp"], d["Li"], d["Lx"], x, 1, lvl, part_ptr,
                               np.arange(n, dtype=np.int32))
    assert e.value.status == ERR_BAD_SCHEDULE
    # an entry above the diagonal in a lower CSR
    Li = d["Li"].copy()
    Li[0 + 1] = 5  # row 1's first off-diagonal now points forward
    with pytest.raises(GbsymError) as e:
        sym_lib.sptrsv_csr(n, d["Lp"], Li, d["Lx"], x)
    assert e.value.status == ERR_BAD_MATRIX


def test_empty_system(gpu):
    from sympiler_gb300 import sym_lib
    x = np.zeros(0)
    sym_lib.sptrsv_csr(0, np.zeros(1, dtype=np.int32), np.zeros(0, dtype=np.int32), np.zeros(0), x)
    nl, lp, ls = sym_lib.build_levelset_csr(0, np.zeros(1, dtype=np.int32), np.zeros(0, dtype=np.int32))
    assert nl == 0 and list(lp) == [0] and len(ls) == 0


def test_dropin_plan_cache(gpu, orc):
    """With the drop-in plan cache on, a second sptrsv_csr / sptrsv_csc call
    on the same arrays reuses the plan (fewer kernel launches: no level-set
    build, no packing) and stays bit-exact; a new caller version drops the
    plans, so values changed in place are picked up."""
    from sympiler_gb300 import sym_lib
    from sympiler_gb300.plans import kernel_launches
    L = mg.tril(mg.lap2d(80))
    Lt = mg.transpose(L)  # CSC of L
    rng = np.random.default_rng(31)
    sym_lib.dropin_cache(4)
    try:
        counts = []
        for call in range(3):
            b = rng.uniform(-1, 1, L.n)
            want = b.copy()
            orc.sptrsv_csr(L.n, *L.astuple(), want)
            x = b.copy()
            k0 = kernel_launches()
            sym_lib.sptrsv_csr(L.n, L.p, L.i, L.x, x)
            counts.append(kernel_launches() - k0)
            assert np.array_equal(x, want), call
            xc = b.copy()
            sym_lib.sptrsv_csc(L.n, Lt.p, Lt.i, Lt.x, xc)
            assert np.array_equal(xc, want), call
        assert counts[1] < counts[0] and counts[2] == counts[1], counts
        # values changed in place, announced by a new version
        L.x[L.p[1:] - 1] *= 2.0
        sym_lib.dropin_cache_version(1)
        b = rng.uniform(-1, 1, L.n)
        want = b.copy()
        orc.sptrsv_csr(L.n, *L.astuple(), want)
        x = b.copy()
        k0 = kernel_launches()
        sym_lib.sptrsv_csr(L.n, L.p, L.i, L.x, x)
        assert kernel_launches() - k0 > counts[1]  # rebuilt
        assert np.array_equal(x, want)
    finally:
        sym_lib.dropin_cache(0)
        sym_lib.dropin_cache_version(0)
