"""GPU SpMV and incomplete factorisations against the reference's known
answers and the oracle (bit-exact: same operation order, no contraction)."""
import numpy as np
import pytest
import torch

from conftest import golden
from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def test_spmv_catch_known_answers(gpu):
    from sympiler_gb300 import sym_lib
    for name in ("catch_spmv_4x4", "catch_spmv_10x10"):
        d = golden(name)
        n = len(d["Ap"]) - 1
        y = np.zeros(n)
        sym_lib.spmv_csr(n, d["Ap"], d["Ai"], d["Ax"], d["x"], y)
        assert np.array_equal(y, d["z"])
        y = np.zeros(n)
        sym_lib.spmv_csr_parallel(n, d["Ap"], d["Ai"], d["Ax"], d["x"], y)
        assert np.array_equal(y, d["z"])


def test_spmv_c1_fixture(gpu):
    from sympiler_gb300 import sym_lib
    d = golden("c1_lap2d_100")
    n = len(d["Ap"]) - 1
    y = np.zeros(n)
    sym_lib.spmv_csr(n, d["Ap"], d["Ai"], d["Ax"], d["v"], y)
    assert np.array_equal(y, d["y"])
    z = d["z0"].copy()
    sym_lib.spmv_csr(n, d["Ap"], d["Ai"], d["Ax"], d["v"], d["b"], z, float(d["a"]), float(d["bb"]))
    assert np.array_equal(z, d["z"])


@pytest.mark.parametrize("gen", ["lap3d64", "convdiff48", "random"])
def test_spmv_plan_large_fp64_fp32(gpu, orc, gen):
    from sympiler_gb300.plans import CsrPlan
    rng = np.random.default_rng(2)
    if gen == "lap3d64":
        A = mg.lap3d(64, 1e-2)
    elif gen == "convdiff48":
        A = mg.convdiff3d(48)
    else:
        A = mg.random_spd(50000, 40, rng)  # rows up to ~80 entries
    v = rng.uniform(-1, 1, A.n)
    ref = np.zeros(A.n)
    orc.spmv_csr(A.n, *A.astuple(), v, ref)
    P = CsrPlan(A.n, *A.astuple())
    y = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    P.spmv(torch.from_numpy(v).cuda(), y)
    torch.cuda.synchronize()
    assert np.array_equal(y.cpu().numpy(), ref)
    P32 = CsrPlan(A.n, *A.astuple(), dtype="f32")
    v32 = v.astype(np.float32)
    ref32 = np.zeros(A.n, dtype=np.float32)
    orc.spmv_csr_f32(A.n, A.p, A.i, A.x.astype(np.float32), v32, ref32)
    y32 = torch.zeros(A.n, dtype=torch.float32, device="cuda")
    P32.spmv(torch.from_numpy(v32).cuda(), y32)
    torch.cuda.synchronize()
    assert np.array_equal(y32.cpu().numpy(), ref32)


def test_ilu0_and_ic0_fixtures(gpu):
    from sympiler_gb300 import sym_lib
    d = golden("ilu0_convdiff_8")
    n = len(d["Ap"]) - 1
    l = np.zeros_like(d["Ax"])
    sym_lib.spilu0_csr(n, int(d["Ap"][n]), d["Ap"], d["Ai"], d["Ax"], d["diag"], l)
    assert np.array_equal(l, d["lu"])
    for name in ("ic0_lap3d_10", "ic0_random_spd_2000"):
        g = golden(name)
        n = len(g["Up"]) - 1
        v = g["Ux"].copy()
        sym_lib.spic0_csr(n, v, g["Up"], g["Ui"])
        assert np.array_equal(v, g["factor"]), name


def test_factors_at_workload_size(gpu, orc):
    from sympiler_gb300.plans import ic0_device, ilu0_device
    A = mg.lap3d(64, 1e-2)
    U = mg.triu(A)
    ref, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    v = torch.from_numpy(U.x.copy()).cuda()
    ic0_device(U.n, v, torch.from_numpy(U.p).cuda(), torch.from_numpy(U.i).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(v.cpu().numpy(), ref)
    C = mg.convdiff3d(40)
    d = mg.diag_ptr(C)
    refl, ok = orc.spilu0_csr(C.n, C.p, C.i, C.x, d)
    out = torch.zeros(C.nnz, dtype=torch.float64, device="cuda")
    ilu0_device(C.n, *(torch.from_numpy(a).cuda() for a in (C.p, C.i, C.x, d)), out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), refl)


def test_ic0_pivot_error(gpu):
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import ERR_PIVOT, GbsymError
    A = mg.lap2d(8)
    A = mg.from_scipy(A.scipy() - 8.0 * __import__("scipy").sparse.eye(A.n))  # indefinite
    U = mg.triu(A)
    v = U.x.copy()
    with pytest.raises(GbsymError) as e:
        sym_lib.spic0_csr(U.n, v, U.p, U.i)
    assert e.value.status == ERR_PIVOT


def _lbc_of_lower(n, p, i, parts):
    """The library's DAG LBC inspector on a lower CSR pattern (diagonal last),
    as the reference demo calls get_coarse_levelSet_DAG_CSC_tree."""
    from sympiler_gb300 import sym_lib
    nl, lp, pn, pp, nodes = sym_lib.get_coarse_levelSet_DAG_CSC_tree(n, p, i, 0, parts, -1, 100)
    return nl, lp, pp, nodes


@pytest.mark.parametrize("parts", [2, 8])
def test_spilu0_csr_lbc_drop_in(gpu, orc, parts):
    """spilu0_csr_lbc under a valid LBC schedule of the rows' dependencies
    equals the serial oracle bit for bit (ILU0's row arithmetic does not
    depend on the schedule); a schedule that runs a row before one it reads
    is refused and leaves l untouched."""
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import ERR_BAD_SCHEDULE, GbsymError
    for A in (mg.convdiff3d(12), mg.convdiff3d(7)):
        d = mg.diag_ptr(A)
        ref, ok = orc.spilu0_csr(A.n, A.p, A.i, A.x, d)
        assert ok
        Lpat = mg.tril(A)  # dependencies of row i: its entries left of the diagonal
        nl, lp, pp, nodes = _lbc_of_lower(A.n, Lpat.p, Lpat.i, parts)
        l = np.zeros_like(A.x)
        sym_lib.spilu0_csr_lbc(A.n, A.nnz, A.p, A.i, A.x, d, l, nl, lp, pp, nodes)
        assert np.array_equal(l, ref)
    bad = np.arange(A.n, dtype=np.int32)[::-1].copy()  # last row first: violates every dependency
    l = np.full_like(A.x, 7.0)
    with pytest.raises(GbsymError) as e:
        sym_lib.spilu0_csr_lbc(A.n, A.nnz, A.p, A.i, A.x, d, l, 1, np.array([0, 1], np.int32),
                               np.array([0, A.n], np.int32), bad)
    assert e.value.status == ERR_BAD_SCHEDULE
    assert np.all(l == 7.0)


@pytest.mark.parametrize("parts", [2, 8])
def test_spic0_csr_lbc_drop_in(gpu, orc, parts):
    """spic0_csr_lbc under a valid LBC schedule over the columns of L equals
    the serial spic0_csr (oracle and fixtures) bit for bit; an invalid
    schedule is refused and leaves val untouched."""
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import ERR_BAD_SCHEDULE, GbsymError
    for name in ("ic0_lap3d_10", "ic0_random_spd_2000"):
        g = golden(name)
        n = len(g["Up"]) - 1
        L = mg.transpose(mg.CSR(n, g["Up"], g["Ui"], g["Ux"]))  # CSR of L: the solve DAG of the columns
        nl, lp, pp, nodes = _lbc_of_lower(n, L.p, L.i, parts)
        v = g["Ux"].copy()
        sym_lib.spic0_csr_lbc(n, v, g["Up"], g["Ui"], nl, lp, pp, nodes)
        assert np.array_equal(v, g["factor"]), name
    A = mg.lap3d(16, 1e-2)
    U = mg.triu(A)
    ref, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    L = mg.transpose(U)
    nl, lp, pp, nodes = _lbc_of_lower(U.n, L.p, L.i, parts)
    v = U.x.copy()
    sym_lib.spic0_csr_lbc(U.n, v, U.p, U.i, nl, lp, pp, nodes)
    assert np.array_equal(v, ref)
    bad = np.arange(U.n, dtype=np.int32)[::-1].copy()
    v = U.x.copy()
    with pytest.raises(GbsymError) as e:
        sym_lib.spic0_csr_lbc(U.n, v, U.p, U.i, 1, np.array([0, 1], np.int32), np.array([0, U.n], np.int32), bad)
    assert e.value.status == ERR_BAD_SCHEDULE
    assert np.array_equal(v, U.x)


def _mixed_rows(n, rng):
    """Rows of 0..12 entries; a few rows of 40..90 entries and a few runs of
    32 rows of 14 entries each (so neighbouring threads' loops run very
    different lengths); empty rows; rows whose only product is -0."""
    import scipy.sparse as sp
    lens = rng.integers(0, 13, n)
    wide = rng.choice(n, size=max(1, n // 500), replace=False)
    lens[wide] = rng.integers(40, 91, wide.size)
    for w in rng.choice(max(1, n // 32), size=max(1, n // 3000), replace=False):
        lens[32 * w:32 * w + 32] = 14
    lens[rng.choice(n, size=max(1, n // 50), replace=False)] = 0
    lens = np.minimum(lens, n)
    rows = np.repeat(np.arange(n), lens)
    cols = np.concatenate([np.sort(rng.choice(n, size=l, replace=False)) for l in lens])
    vals = rng.uniform(-1, 1, rows.size)
    negz = rng.choice(n, size=max(1, n // 100), replace=False)
    m = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    m = sp.lil_matrix(m)
    for r in negz:
        m.rows[r] = [0]
        m.data[r] = [-1.0]
    return mg.from_scipy(sp.csr_matrix(m))


@pytest.mark.parametrize("n", [1, 31, 33, 5000, 70001])
def test_spmv_mixed_rows_signed_zeros_and_axpby(gpu, orc, n):
    """Ragged row lengths, empty rows, -0 products (0 + -0 = +0), sizes
    around one warp, and the accumulate form z = a (z + A x) + b y, bit for
    bit against the oracle in FP64 and FP32."""
    from sympiler_gb300.plans import CsrPlan
    rng = np.random.default_rng(n)
    A = _mixed_rows(n, rng)
    v = rng.uniform(-1, 1, n)
    v[0] = 0.0  # column 0 carries the -1 entries: their product is -0
    ref = np.zeros(n)
    orc.spmv_csr(A.n, *A.astuple(), v, ref)
    P = CsrPlan(A.n, *A.astuple())
    y = torch.full((n,), 5.0, dtype=torch.float64, device="cuda")
    P.spmv(torch.from_numpy(v).cuda(), y)
    got = y.cpu().numpy()
    assert np.array_equal(got, ref) and np.array_equal(np.signbit(got), np.signbit(ref))
    yv, z0 = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    zref = z0.copy()
    orc.spmv_csr_axpby(A.n, *A.astuple(), v, yv, zref, 0.75, -1.25)
    z = torch.from_numpy(z0.copy()).cuda()
    P.spmv_axpby(torch.from_numpy(v).cuda(), torch.from_numpy(yv).cuda(), z, 0.75, -1.25)
    assert np.array_equal(z.cpu().numpy(), zref)
    P32 = CsrPlan(A.n, *A.astuple(), dtype="f32")
    v32 = v.astype(np.float32)
    ref32 = np.zeros(n, dtype=np.float32)
    orc.spmv_csr_f32(A.n, A.p, A.i, A.x.astype(np.float32), v32, ref32)
    y32 = torch.zeros(n, dtype=torch.float32, device="cuda")
    P32.spmv(torch.from_numpy(v32).cuda(), y32)
    assert np.array_equal(y32.cpu().numpy(), ref32)
