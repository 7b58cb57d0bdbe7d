"""LBC schedule inspectors (host code of libgbsym.so, no GPU needed): the
tree level set and tree LBC against the reference's own outputs, and the
DAG LBC's schedules executed by the oracle's LBC solve."""
import numpy as np
import pytest

from sympiler_gb300 import matgen as mg
from sympiler_gb300 import sym_lib
from sympiler_gb300._lib import GbsymError

from conftest import golden


def _cost_rows_of_L(U):
    """Entries per row of L = entries per column of the upper CSR U."""
    return np.bincount(U["Ui"], minlength=len(U["etree"])).astype(np.float64)


@pytest.mark.parametrize("name", ["ic0_random_spd_2000", "ic0_lap3d_10"])
def test_tree_levelset_matches_reference_fixture(name):
    g = golden(name)
    par = g["etree"].astype(np.int32)
    n = len(par)
    lp = np.zeros(n + 1, np.int32)
    ls = np.zeros(n, np.int32)
    nl = sym_lib.parsy.getLevelSet(n, par, lp, ls)
    assert nl == int(g["tree_levels"])
    assert np.array_equal(lp[: nl + 1], g["tree_level_ptr"][: nl + 1])
    assert np.array_equal(ls, g["tree_level_set"])


@pytest.mark.parametrize("name,params", [("ic0_random_spd_2000", (4, -1, 100)),
                                         ("ic0_lap3d_10", (4, -1, 4000))])
def test_coarse_levelset_matches_reference_fixture(name, params):
    g = golden(name)
    par = g["etree"].astype(np.int32)
    n = len(par)
    nl, lp, pn, pp, nodes = sym_lib.parsy.getCoarseLevelSet_6(n, par, None, *params, _cost_rows_of_L(g))
    assert nl == int(g["lbc_level_no"])
    assert np.array_equal(lp, g["lbc_level_ptr"][: nl + 1])
    assert np.array_equal(pp, g["lbc_par_ptr"][: pn + 1])
    assert np.array_equal(nodes, g["lbc_partition"][:n])


def _random_lower(rng, trial):
    kind = trial % 4
    if kind == 0:
        A = mg.random_spd(int(rng.integers(2, 1500)), int(rng.integers(1, 8)), rng)
    elif kind == 1:
        A = mg.lap2d(int(rng.integers(2, 40)))
    elif kind == 2:
        A = mg.lap3d(int(rng.integers(2, 10)))
    else:
        A = mg.random_spd(int(rng.integers(2, 300)), 1, rng)
    return mg.tril(A)


def test_tree_lbc_matches_compiled_reference_on_random_trees(ref):
    """Random elimination trees, costs and parameters against the
    reference's getCoarseLevelSet_6 compiled from its sources.  Costs are
    whole numbers: the reference asserts that its integer running total of
    the level costs equals the exact sum."""
    rng = np.random.default_rng(5)
    for trial in range(120):
        L = _random_lower(rng, trial)
        n = L.n
        par = sym_lib.etree_lower_csr(n, L.p, L.i)
        cost = np.diff(L.p).astype(np.float64) if trial % 3 else rng.integers(1, 10, n).astype(np.float64)
        ip = int(rng.choice([1, 2, 4, 6, 8, 16, 64]))
        mld = int(rng.choice([-1, 0, 1, 2, 3]))
        dr = int(rng.choice([2, 3, 4, 100, 4000]))
        want = ref.coarse_levelset6(n, par, cost, ip, mld, dr)
        got = sym_lib.parsy.getCoarseLevelSet_6(n, par, None, ip, mld, dr, cost)
        assert want[0] == got[0], (trial, n, ip, mld, dr)
        assert np.array_equal(want[1], got[1])
        assert np.array_equal(want[2], got[3])
        assert np.array_equal(want[3], got[4])


def _check_lbc_schedule(L, nl, lp, pn, pp, nodes):
    """Every row exactly once; each row's dependencies finish in an earlier
    coarse level or earlier in its own partition."""
    n = L.n
    assert lp[0] == 0 and lp[nl] == pn and pp[0] == 0 and pp[pn] == n
    assert np.array_equal(np.sort(nodes), np.arange(n))
    where = np.empty(n, np.int64)   # (coarse level, partition, position)
    coarse = np.empty(n, np.int64)
    for c in range(nl):
        for part in range(lp[c], lp[c + 1]):
            for q in range(pp[part], pp[part + 1]):
                where[nodes[q]] = part * (n + 1) + q
                coarse[nodes[q]] = c
    part_of = where // (n + 1)
    for i in range(n):
        for j in L.i[L.p[i]:L.p[i + 1]]:
            if j == i:
                continue
            assert coarse[j] < coarse[i] or (part_of[j] == part_of[i] and where[j] < where[i]), (i, j)


def test_dag_lbc_schedules_are_valid_and_solve_bit_exact(orc):
    rng = np.random.default_rng(11)
    for trial in range(24):
        L = _random_lower(rng, trial)
        vals = -rng.random(len(L.i))
        vals[L.p[1:] - 1] = 4.0 + rng.random(L.n)  # the diagonal, last in each row
        L = mg.CSR(L.n, L.p, L.i, vals)
        ip = int(rng.choice([2, 4, 8]))
        nl, lp, pn, pp, nodes = sym_lib.get_coarse_levelSet_DAG_CSC_tree(L.n, L.p, L.i, 0, ip, -1, 4000)
        _check_lbc_schedule(L, nl, lp, pn, pp, nodes)
        b = rng.standard_normal(L.n)
        serial = b.copy()
        orc.sptrsv_csr(L.n, L.p, L.i, L.x, serial)
        lbc = b.copy()
        orc.sptrsv_csr_lbc(L.n, L.p, L.i, L.x, lbc, nl, lp, pp, nodes)
        assert np.array_equal(serial, lbc)


def test_default_cost_is_entries_per_row():
    L = mg.tril(mg.random_spd(500, 4, np.random.default_rng(2)))
    a = sym_lib.get_coarse_levelSet_DAG_CSC_tree(L.n, L.p, L.i, 0, 4, -1, 100)
    b = sym_lib.get_coarse_levelSet_DAG_CSC_tree(L.n, L.p, L.i, 0, 4, -1, 100,
                                                 cost=np.diff(L.p).astype(np.float64))
    for u, v in zip(a, b):
        assert np.array_equal(np.asarray(u), np.asarray(v))


def test_inspectors_reject_bad_input():
    with pytest.raises(GbsymError):
        sym_lib.parsy.getLevelSet(3, np.array([2, 0, -1], np.int32), np.zeros(4, np.int32), np.zeros(3, np.int32))
    with pytest.raises(GbsymError):  # an upper entry in a lower CSR
        sym_lib.get_coarse_levelSet_DAG_CSC_tree(2, np.array([0, 2, 3], np.int32), np.array([0, 1, 1], np.int32),
                                                 0, 4, -1, 4000)
    with pytest.raises(GbsymError):  # no parts
        sym_lib.parsy.getCoarseLevelSet_6(2, np.array([1, -1], np.int32), None, 0, -1, 4000, np.ones(2))
    assert sym_lib.get_coarse_levelSet_DAG_CSC_tree(0, np.zeros(1, np.int32), np.zeros(0, np.int32),
                                                    0, 4, -1, 4000)[0] == 0


def test_inspectors_are_linear_on_path_shaped_trees():
    """A naturally ordered grid's elimination tree is a single path, so the
    level set has as many levels as nodes.  The reference's per-level window
    sweep is quadratic there; the inspectors must stay linear: a 300,000-node
    path and the DAG LBC of the 48^3 grid's factor each take well under a
    second, with the level set one node per level."""
    import time
    n = 300_000
    parent = np.arange(1, n + 1, dtype=np.int32)
    parent[-1] = -1
    lp, ls = np.zeros(n + 1, np.int32), np.zeros(n, np.int32)
    t0 = time.perf_counter()
    nl = sym_lib.parsy.getLevelSet(n, parent, lp, ls)
    cost = np.ones(n)
    lvl = sym_lib.parsy.getCoarseLevelSet_6(n, parent, None, 64, -1, 4000, cost)
    assert time.perf_counter() - t0 < 2.0
    assert nl == n and np.array_equal(ls, np.arange(n)) and np.array_equal(lp, np.arange(n + 1))
    assert lvl[2] >= 1 and np.array_equal(np.sort(lvl[4]), np.arange(n))
    L = mg.tril(mg.lap3d(48, 1e-2))
    t0 = time.perf_counter()
    sym_lib.get_coarse_levelSet_DAG_CSC_tree(L.n, L.p, L.i, 0, 64, -1, 4000)
    assert time.perf_counter() - t0 < 2.0
