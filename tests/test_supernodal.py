"""Supernodal (blocked CSC) solves: the C restatement against the reference
compiled from its sources, and the GPU entry points against the
restatement, bit for bit."""
import numpy as np
import pytest

from sympiler_gb300 import matgen as mg


def _structures(seed, count):
    rng = np.random.default_rng(seed)
    for t in range(count):
        yield mg.random_supernodal(int(rng.integers(1, 120)), int(rng.integers(1, 72)),
                                   int(rng.integers(0, 80)), rng, tree=bool(t % 3))


def _sn_levels(S, transposed=False):
    """Level set over supernodes (forward dependency DAG, or its reverse)."""
    lev = np.zeros(S.nsup, int)
    order = range(S.nsup - 1, -1, -1) if transposed else range(S.nsup)
    for s in order:
        c0, c1 = int(S.sup2col[s]), int(S.sup2col[s + 1])
        r0, r1 = int(S.Li_ptr[c0]), int(S.Li_ptr[c1])
        for row in S.Li[r0 + (c1 - c0):r1]:
            t = int(S.col2sup[row])
            if transposed:
                lev[s] = max(lev[s], lev[t] + 1)
            else:
                lev[t] = max(lev[t], lev[s] + 1)
    nl = int(lev.max()) + 1
    if transposed:
        lev = nl - 1 - lev  # the reference's LT loop walks levels from the last
    ls = np.argsort(lev, kind="stable").astype(np.int32)
    lp = np.zeros(nl + 1, np.int32)
    np.add.at(lp, lev + 1, 1)
    return nl, np.cumsum(lp).astype(np.int32), ls


def test_restatement_matches_compiled_reference(orc, ref):
    for t, S in enumerate(_structures(7, 40)):
        b = np.random.default_rng(t).standard_normal(S.n)
        x1 = b.copy()
        orc.blocked_lsolve(S, x1)
        x2 = b.copy()
        assert ref.blocked_lsolve(S, x2) == 1
        assert np.array_equal(x1, x2), t


def test_reference_leveled_forms_agree_up_to_their_atomic_order(orc, ref):
    S = mg.random_supernodal(200, 24, 40, np.random.default_rng(9))
    nl, lp, ls = _sn_levels(S)
    b = np.random.default_rng(4).standard_normal(S.n)
    x1 = b.copy()
    orc.blocked_lsolve(S, x1)
    x2 = b.copy()
    ref.leveled_blocked_lsolve(S, x2, nl, lp, ls)
    x3 = b.copy()
    parts = np.arange(S.nsup + 1, dtype=np.int32)
    ref.h2_leveled_blocked_lsolve(S, x3, nl, lp, ls, S.nsup, parts, ls)
    for x in (x2, x3):
        assert np.abs(x - x1).max() <= 1e-12 * np.abs(x1).max()


def test_restatement_against_dense_solves(orc):
    for t, S in enumerate(_structures(11, 12)):
        D = S.dense()
        b = np.random.default_rng(t).standard_normal(S.n)
        x = b.copy()
        orc.blocked_lsolve(S, x)
        assert np.allclose(x, np.linalg.solve(D, b), rtol=1e-12, atol=1e-12)
        x = b.copy()
        orc.blocked_ltsolve(S, x)
        assert np.allclose(x, np.linalg.solve(D.T, b), rtol=1e-12, atol=1e-12)


def test_nested_dissection_factors_match_reference_and_dense(orc, ref):
    for t, (dims, leaf) in enumerate([((12, 10, 9), 16), ((20, 1, 1), 4), ((9, 9, 1), 8), ((7, 6, 5), 27)]):
        S = mg.nd_supernodal(*dims, leaf=leaf, rng=np.random.default_rng(t))
        D = S.dense()
        b = np.random.default_rng(50 + t).standard_normal(S.n)
        x1 = b.copy()
        orc.blocked_lsolve(S, x1)
        x2 = b.copy()
        assert ref.blocked_lsolve(S, x2) == 1
        assert np.array_equal(x1, x2), dims
        assert np.abs(D @ x1 - b).max() <= 1e-13
        x3 = b.copy()
        orc.blocked_ltsolve(S, x3)
        assert np.abs(D.T @ x3 - b).max() <= 1e-13


# ---- GPU --------------------------------------------------------------------

@pytest.mark.gpu
def test_gpu_nested_dissection_factor_repeated_solves(gpu, orc):
    """A 24^3 grid's factor (separators up to 576 columns, off-block rows
    split across lanes): forward and transposed, one and many right-hand
    sides, several solves on one plan -- the task counters carry over
    between solves."""
    import torch
    from sympiler_gb300.plans import SupernodalPlan
    S = mg.nd_supernodal(24, 24, 24, leaf=64, rng=np.random.default_rng(3))
    assert np.diff(S.sup2col).max() == 576
    P = SupernodalPlan(S)
    rng = np.random.default_rng(4)
    for rep, (k, transposed) in enumerate([(1, False), (1, True), (8, False), (1, False), (13, True),
                                           (13, False), (1, True), (8, True)]):
        X = rng.standard_normal((k, S.n))
        W = X.copy()
        (orc.blocked_ltsolve if transposed else orc.blocked_lsolve)(S, W if k > 1 else W[0])
        Xd = torch.from_numpy(X.copy()).cuda()
        P.solve(Xd if k > 1 else Xd[0], transposed=transposed)
        P.check()
        assert np.array_equal(Xd.cpu().numpy(), W), (rep, k, transposed)


@pytest.mark.gpu
def test_gpu_nested_dissection_2d_wide_separator(gpu, orc):
    from sympiler_gb300 import sym_lib
    S = mg.nd_supernodal(150, 130, 1, leaf=16, rng=np.random.default_rng(6))
    assert np.diff(S.sup2col).max() == 130
    b = np.random.default_rng(7).standard_normal(S.n)
    for fn, ofn in ((sym_lib.parsy.blockedLsolve, orc.blocked_lsolve),
                    (sym_lib.parsy.blockedLTsolve, orc.blocked_ltsolve)):
        want = b.copy()
        ofn(S, want)
        x = b.copy()
        assert fn(S, x) == 1
        assert np.array_equal(x, want)


@pytest.mark.gpu
def test_gpu_blocked_solves_bit_exact(gpu, orc):
    from sympiler_gb300 import sym_lib
    for t, S in enumerate(_structures(21, 30)):
        rng = np.random.default_rng(100 + t)
        b = rng.standard_normal(S.n)
        want = b.copy()
        orc.blocked_lsolve(S, want)
        x = b.copy()
        assert sym_lib.parsy.blockedLsolve(S, x) == 1
        assert np.array_equal(x, want), t
        want_t = b.copy()
        orc.blocked_ltsolve(S, want_t)
        x = b.copy()
        assert sym_lib.parsy.blockedLTsolve(S, x) == 1
        assert np.array_equal(x, want_t), t
        k = 3
        X = rng.standard_normal((k, S.n))  # column-major n x k
        W = X.copy()
        orc.blocked_lsolve(S, W)
        Y = X.copy()
        assert sym_lib.parsy.blockedLsolve_mrhs(S, Y, k) == 1
        assert np.array_equal(Y, W)
        W = X.copy()
        orc.blocked_ltsolve(S, W)
        Y = X.copy()
        assert sym_lib.parsy.blockedLTsolve_mrhs(S, Y, k) == 1
        assert np.array_equal(Y, W)


@pytest.mark.gpu
def test_gpu_scheduled_forms_validate_and_match(gpu, orc):
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import ERR_BAD_SCHEDULE as GBSYM_ERR_BAD_SCHEDULE, lib
    S = mg.random_supernodal(150, 40, 60, np.random.default_rng(3))
    b = np.random.default_rng(5).standard_normal(S.n)
    want = b.copy()
    orc.blocked_lsolve(S, want)
    nl, lp, ls = _sn_levels(S)
    x = b.copy()
    assert sym_lib.parsy.leveledBlockedLsolve(S, x, nl, lp, ls) == 1
    assert np.array_equal(x, want)
    # LBC: every supernode level a coarse level of one-supernode parts; and
    # one coarse level holding one serial part
    pp = np.arange(S.nsup + 1, dtype=np.int32)
    for sched in ((nl, lp, S.nsup, pp, ls),
                  (1, np.array([0, 1], np.int32), 1, np.array([0, S.nsup], np.int32),
                   np.arange(S.nsup, dtype=np.int32))):
        x = b.copy()
        assert sym_lib.parsy.H2LeveledBlockedLsolve(S, x, *sched) == 1
        assert np.array_equal(x, want)
    want_t = b.copy()
    orc.blocked_ltsolve(S, want_t)
    tl, tlp, tls = _sn_levels(S, transposed=True)
    x = b.copy()
    assert sym_lib.parsy.H2LeveledBlockedLsolve(S, x, tl, tlp, S.nsup, pp, tls, transposed=True) == 1
    assert np.array_equal(x, want_t)
    X = np.random.default_rng(6).standard_normal((5, S.n))
    W = X.copy()
    orc.blocked_lsolve(S, W)
    Y = X.copy()
    assert sym_lib.parsy.H2LeveledBlockedLsolve_mrhs(S, Y, 5, nl, lp, S.nsup, pp, ls) == 1
    assert np.array_equal(Y, W)
    # a schedule that puts a supernode before one it depends on is rejected
    bad = ls[::-1].copy()
    x = b.copy()
    assert sym_lib.parsy.H2LeveledBlockedLsolve(S, x, 1, np.array([0, 1], np.int32), 1,
                                                np.array([0, S.nsup], np.int32), bad) == 0
    assert lib().gbsym_last_error() == GBSYM_ERR_BAD_SCHEDULE
    assert np.array_equal(x, b)  # untouched


@pytest.mark.gpu
def test_gpu_supernodal_plan_many_rhs_and_wide_supernodes(gpu, orc):
    import torch
    from sympiler_gb300.plans import SupernodalPlan
    S = mg.random_supernodal(60, 160, 120, np.random.default_rng(8))
    assert np.diff(S.sup2col).max() > 64
    P = SupernodalPlan(S)
    f, t = P.levels()
    assert f >= 1 and t >= 1
    for k in (1, 7, 70):
        X = np.random.default_rng(k).standard_normal((k, S.n))
        for transposed in (False, True):
            W = X.copy()
            (orc.blocked_ltsolve if transposed else orc.blocked_lsolve)(S, W if k > 1 else W[0])
            Xd = torch.from_numpy(X.copy()).cuda()
            P.solve(Xd if k > 1 else Xd[0], transposed=transposed)
            P.check()
            assert np.array_equal(Xd.cpu().numpy(), W), (k, transposed)


@pytest.mark.gpu
def test_gpu_supernodal_degenerate_shapes(gpu, orc):
    """A block-diagonal factor (no off-block rows: no products, no
    contributions), one dense supernode of 63 columns (two tiles), and zero
    right-hand sides; forward and transposed against the restatement."""
    import torch
    from sympiler_gb300.plans import SupernodalPlan
    cases = [mg.random_supernodal(40, 50, 0, np.random.default_rng(2)),
             mg.random_supernodal(1, 77, 0, np.random.default_rng(3))]
    assert np.diff(cases[1].sup2col)[0] == 63
    for S in cases:
        P = SupernodalPlan(S)
        for k in (1, 4):
            X = np.random.default_rng(k).standard_normal((k, S.n))
            for transposed in (False, True):
                W = X.copy()
                (orc.blocked_ltsolve if transposed else orc.blocked_lsolve)(S, W if k > 1 else W[0])
                Xd = torch.from_numpy(X.copy()).cuda()
                P.solve(Xd if k > 1 else Xd[0], transposed=transposed)
                P.check()
                assert np.array_equal(Xd.cpu().numpy(), W), (S.nsup, k, transposed)
        Xd = torch.zeros((0, S.n), dtype=torch.float64, device="cuda")
        P.solve(Xd)  # no right-hand sides: nothing to do
        P.check()
    E = mg.Supernodal(0, 0, np.zeros(1, np.uint64), np.zeros(0, np.int32), np.zeros(0), np.zeros(1, np.uint64),
                      np.zeros(0, np.int32), np.zeros(1, np.int32))
    P = SupernodalPlan(E)
    assert P.levels() == (0, 0)
    P.solve(torch.zeros(0, dtype=torch.float64, device="cuda"))
    P.check()


@pytest.mark.gpu
def test_gpu_solve_phases(gpu, orc):
    """parsy's LL^T solve phases (L then L^T, serial, multi-RHS and
    LBC-scheduled) and the LDL^T phase with a diagonal D, against the
    restatement run in the same order."""
    from sympiler_gb300 import sym_lib
    S = mg.nd_supernodal(14, 12, 10, leaf=27, rng=np.random.default_rng(12))
    rng = np.random.default_rng(13)
    b = rng.standard_normal(S.n)
    want = b.copy()
    orc.blocked_lsolve(S, want)
    orc.blocked_ltsolve(S, want)
    x = b.copy()
    sym_lib.parsy.solve_phase_ll_blocked(S, x)
    assert np.array_equal(x, want)
    nl, lp, ls = _sn_levels(S)
    pp = np.arange(S.nsup + 1, dtype=np.int32)
    x = b.copy()
    sym_lib.parsy.solve_phase_ll_blocked_parallel(S, x, nl, lp, S.nsup, pp, ls)
    assert np.array_equal(x, want)
    X = rng.standard_normal((3, S.n))
    W = X.copy()
    orc.blocked_lsolve(S, W)
    orc.blocked_ltsolve(S, W)
    Y = X.copy()
    sym_lib.parsy.solve_phase_ll_blocked_nrhs(S, Y, 3)
    assert np.array_equal(Y, W)
    Y = X.copy()
    sym_lib.parsy.solve_phase_ll_blocked_parallel_nrhs(S, Y, 3, nl, lp, S.nsup, pp, ls)
    assert np.array_equal(Y, W)
    d = rng.uniform(0.5, 2.0, S.n)
    want = b.copy()
    orc.blocked_lsolve(S, want)
    want = want / d
    orc.blocked_ltsolve(S, want)
    x = b.copy()
    sym_lib.parsy.solve_phase_ldl(S, d, x)
    assert np.array_equal(x, want)


@pytest.mark.gpu
def test_gpu_simplicial_solve_phases(gpu, orc):
    """parsy's simplicial solve phases on the CSC of an IC0 factor (the
    upper CSR of the factored triangle): lsolve, (x /= d), ltsolve, each
    the oracle's bits."""
    from sympiler_gb300 import sym_lib
    A = mg.lap2d(40)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    assert ok
    Lp, Li, Lx = U.p, U.i, f  # CSC of L, diagonal first in each column
    b = np.random.default_rng(14).standard_normal(U.n)
    d = np.random.default_rng(15).uniform(0.5, 2.0, U.n)
    for dv in (None, d):
        want = b.copy()
        orc.sptrsv_csc(U.n, Lp, Li, Lx, want)
        if dv is not None:
            want = want / dv
        orc.ltsolve(U.n, Lp, Li, Lx, want)
        x = b.copy()
        if dv is None:
            sym_lib.parsy.solve_phase_simplicial_ll(U.n, Lp, Li, Lx, x)
        else:
            sym_lib.parsy.solve_phase_simplicial_ldl(U.n, Lp, Li, Lx, dv, x)
        assert np.array_equal(x, want)


@pytest.mark.gpu
def test_gpu_supernodal_rejects_malformed_storage(gpu):
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import ERR_BAD_MATRIX as GBSYM_ERR_BAD_MATRIX, lib
    S = mg.random_supernodal(10, 6, 8, np.random.default_rng(1))
    Li = S.Li.copy()
    Li[0] = Li[0] + 1  # the first supernode's first row is not its first column
    bad = mg.Supernodal(S.n, S.nsup, S.Lp, Li, S.Lx, S.Li_ptr, S.col2sup, S.sup2col)
    x = np.ones(S.n)
    assert sym_lib.parsy.blockedLsolve(bad, x) == 0
    assert lib().gbsym_last_error() == GBSYM_ERR_BAD_MATRIX
