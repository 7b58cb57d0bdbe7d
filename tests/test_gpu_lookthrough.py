"""The look-through sweeps (spare lanes recompute each row's dependencies,
and with two levels theirs, so that rows wait two or three levels back;
for several right-hand sides every lane does so for its columns) against the plain
sync-free sweep and the oracle, bit for bit, for every row form it serves:
lower CSR with the diagonal last, unit lower and upper ILU factors, the
transposed (upper) solve, FP64 and FP32, exact and fused arithmetic.  Plans
whose rows do not fit a three-entry slab fall back to the plain sweep."""
import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def _plan(monkeypatch, lookthrough, *args, **kw):
    from sympiler_gb300._lib import EXEC_SYNCFREE
    from sympiler_gb300.plans import TriPlan
    monkeypatch.setenv("GBSYM_SF_LOOKTHROUGH", str(int(lookthrough)))
    P = TriPlan(*args, **kw)
    monkeypatch.delenv("GBSYM_SF_LOOKTHROUGH")
    P.set_exec(EXEC_SYNCFREE)
    return P


def _solve(P, b, dtype=torch.float64):
    x = torch.from_numpy(b.copy()).to(dtype).cuda()
    P.solve(x)
    P.check()
    return x.cpu().numpy()


@pytest.mark.parametrize("levels", [1, 2])
@pytest.mark.parametrize("grid", [(60, 50), (24, 20, 16)])
def test_lower_fp64_fp32_exact_and_fused(gpu, orc, monkeypatch, grid, levels):
    from sympiler_gb300._lib import ARITH_FUSED
    A = mg.lap2d(*grid) if len(grid) == 2 else mg.lap3d(grid[0], 1e-2)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    assert ok
    L = mg.transpose(mg.CSR(U.n, U.p, U.i, f))
    b = np.random.default_rng(5).standard_normal(L.n)
    ref = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), ref)
    on = _plan(monkeypatch, levels, L.n, *L.astuple())
    off = _plan(monkeypatch, 0, L.n, *L.astuple())
    assert on.tuning(1)["lookthrough"] == levels and off.tuning(1)["lookthrough"] == 0
    assert np.array_equal(_solve(on, b), ref)
    assert np.array_equal(_solve(off, b), ref)
    # FP32 storage and vectors: look-through equals the plain sweep and the FP32 oracle
    on32 = _plan(monkeypatch, levels, L.n, *L.astuple(), dtype="f32")
    off32 = _plan(monkeypatch, 0, L.n, *L.astuple(), dtype="f32")
    r32 = b.astype(np.float32)
    orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), r32)
    got = _solve(on32, b, torch.float32)
    assert np.array_equal(got, _solve(off32, b, torch.float32))
    assert np.array_equal(got, r32)
    # fused arithmetic: the two sweeps agree bit for bit
    on.set_arith(ARITH_FUSED)
    off.set_arith(ARITH_FUSED)
    assert np.array_equal(_solve(on, b), _solve(off, b))


@pytest.mark.parametrize("levels", [1, 2])
def test_ilu_factors_and_transposed(gpu, orc, monkeypatch, levels):
    from sympiler_gb300._lib import ILU_UNIT_LOWER, ILU_UPPER, UPPER_DIAG_FIRST
    C = mg.convdiff3d(20)
    d = mg.diag_ptr(C)
    lu, ok = orc.spilu0_csr(C.n, C.p, C.i, C.x, d)
    assert ok
    r = np.random.default_rng(6).uniform(-1, 1, C.n)
    ref = orc.lus_cr(C.n, C.p, C.i, lu, d, r)  # unit-lower then upper with division
    outs = []
    for lt in (levels, 0):
        Lu = _plan(monkeypatch, lt, C.n, C.p, C.i, lu, kind=ILU_UNIT_LOWER, diags=d)
        Up = _plan(monkeypatch, lt, C.n, C.p, C.i, lu, kind=ILU_UPPER, diags=d)
        x = torch.from_numpy(r.copy()).cuda()
        Lu.solve(x)
        Up.solve(x)
        Up.check()
        outs.append(x.cpu().numpy())
    assert np.array_equal(outs[0], ref) and np.array_equal(outs[1], ref)
    # the transposed solve of an IC0 factor (ltsolve's row form)
    A = mg.lap3d(18, 1e-2)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    Lt = mg.CSR(U.n, U.p, U.i, f)  # CSC of L = CSR of L^T, diagonal first
    b = np.random.default_rng(7).standard_normal(U.n)
    ref = b.copy()
    orc.ltsolve(U.n, *Lt.astuple(), ref)
    for lt in (levels, 0):
        P = _plan(monkeypatch, lt, U.n, *Lt.astuple(), kind=UPPER_DIAG_FIRST)
        assert np.array_equal(_solve(P, b), ref)


def test_wide_rows_fall_back_to_the_plain_sweep(gpu, orc, monkeypatch):
    L = mg.random_lower(3000, 0.004, np.random.default_rng(8))
    b = np.random.default_rng(9).uniform(-1, 1, L.n)
    ref = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), ref)
    P = _plan(monkeypatch, 1, L.n, *L.astuple())
    assert P.tuning(1)["lookthrough"] == 0  # rows of up to 22 entries
    assert np.array_equal(_solve(P, b), ref)


@pytest.mark.parametrize("k", [3, 8, 40])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_several_rhs_lookthrough(gpu, orc, monkeypatch, k, dtype):
    """The look-through sweep for several right-hand sides (every lane
    recomputes the row's dependencies for its own columns), in place and
    through the out-of-place entry, against the plain sweep and the oracle."""
    from sympiler_gb300._lib import LOWER_CSC
    from sympiler_gb300.plans import TriPlan
    for A in (mg.lap2d(40, 30), mg.lap3d(14, 1e-2)):
        U = mg.triu(A)
        f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
        assert ok
        tdt = torch.float64 if dtype == "f64" else torch.float32
        B = np.random.default_rng(k).standard_normal((U.n, k))
        plans = []
        for lt in ("1", "0"):
            monkeypatch.setenv("GBSYM_SF_LT_MRHS", lt)
            P = TriPlan(U.n, U.p, U.i, f, kind=LOWER_CSC, dtype=dtype)
            monkeypatch.delenv("GBSYM_SF_LT_MRHS")
            from sympiler_gb300._lib import EXEC_SYNCFREE
            P.set_exec(EXEC_SYNCFREE)
            plans.append(P)
        assert plans[0].tuning(k)["lookthrough"] == 1 and plans[1].tuning(k)["lookthrough"] == 0
        outs = []
        for P in plans:
            X = torch.from_numpy(B.copy()).to(tdt).cuda()
            P.solve(X)
            P.check()
            Y = torch.empty_like(X)
            P.solve_into(torch.from_numpy(B.copy()).to(tdt).cuda(), Y)
            P.check()
            assert torch.equal(X, Y)
            outs.append(X.cpu().numpy())
        assert np.array_equal(outs[0], outs[1])
        if dtype == "f64":
            for c in (0, k - 1):
                col = B[:, c].copy()
                orc.sptrsv_csc(U.n, U.p, U.i, f, col)
                assert np.array_equal(outs[0][:, c], col)


def _random_narrow_lower(n, rng, width):
    """A random lower triangle whose rows hold 0..3 off-diagonals at random
    earlier columns (some near, some far), diagonal last: irregular DAGs
    whose dependencies sit one or many levels back."""
    import scipy.sparse as sp
    rows, cols, vals = [], [], []
    for i in range(1, n):
        m = int(rng.integers(0, 4))
        if m == 0:
            continue
        near = rng.integers(max(0, i - width), i, size=m)
        far = rng.integers(0, i, size=m)
        pick = np.where(rng.uniform(size=m) < 0.7, near, far)
        for c in np.unique(pick):
            rows.append(i)
            cols.append(int(c))
            vals.append(float(rng.uniform(-1, 1)))
    d = 2.0 + rng.uniform(0, 1, n)
    r = np.concatenate([np.asarray(rows, dtype=np.int64), np.arange(n)])
    c = np.concatenate([np.asarray(cols, dtype=np.int64), np.arange(n)])
    m = sp.coo_matrix((np.concatenate([vals, d]), (r, c)), shape=(n, n))
    return mg.from_scipy(m)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_irregular_dags_all_forms(gpu, orc, monkeypatch, seed):
    """Random narrow lower triangles: the one-level and two-level one-RHS
    sweeps and the several-RHS sweep equal the oracle bit for bit."""
    from sympiler_gb300._lib import EXEC_SYNCFREE
    from sympiler_gb300.plans import TriPlan
    rng = np.random.default_rng(seed)
    L = _random_narrow_lower(int(rng.integers(3000, 12000)), rng, int(rng.integers(2, 200)))
    b = rng.standard_normal(L.n)
    ref = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), ref)
    for levels in (1, 2):
        P = _plan(monkeypatch, levels, L.n, *L.astuple())
        assert P.tuning(1)["lookthrough"] == levels
        assert np.array_equal(_solve(P, b), ref), levels
    k = 5
    B = rng.standard_normal((L.n, k))
    monkeypatch.setenv("GBSYM_SF_LT_MRHS", "1")
    P = TriPlan(L.n, *L.astuple())
    monkeypatch.delenv("GBSYM_SF_LT_MRHS")
    P.set_exec(EXEC_SYNCFREE)
    assert P.tuning(k)["lookthrough"] == 1
    X = torch.from_numpy(B.copy()).cuda()
    P.solve(X)
    P.check()
    got = X.cpu().numpy()
    for c in range(k):
        col = B[:, c].copy()
        orc.sptrsv_csr(L.n, *L.astuple(), col)
        assert np.array_equal(got[:, c], col), c


@pytest.mark.parametrize("n", [1, 2, 31, 33, 129])
def test_tiny_and_ragged_systems(gpu, orc, monkeypatch, n):
    """Systems smaller than a warp unit or one row past it, through the
    one-level and two-level one-RHS sweeps and the several-RHS sweep."""
    from sympiler_gb300._lib import EXEC_SYNCFREE
    from sympiler_gb300.plans import TriPlan
    rng = np.random.default_rng(n)
    L = _random_narrow_lower(n, rng, 3)
    b = rng.standard_normal(n)
    ref = b.copy()
    orc.sptrsv_csr(n, *L.astuple(), ref)
    for levels in (1, 2):
        P = _plan(monkeypatch, levels, n, *L.astuple())
        assert np.array_equal(_solve(P, b), ref), levels
    B = rng.standard_normal((n, 3))
    monkeypatch.setenv("GBSYM_SF_LT_MRHS", "1")
    P = TriPlan(n, *L.astuple())
    monkeypatch.delenv("GBSYM_SF_LT_MRHS")
    P.set_exec(EXEC_SYNCFREE)
    X = torch.from_numpy(B.copy()).cuda()
    P.solve(X)
    P.check()
    got = X.cpu().numpy()
    for c in range(3):
        col = B[:, c].copy()
        orc.sptrsv_csr(n, *L.astuple(), col)
        assert np.array_equal(got[:, c], col), c
