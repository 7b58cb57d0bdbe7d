"""Device-resident plans at the workload sizes: multi-RHS, FP32, executors,
layouts, end-to-end host solves -- against the oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2_factor(orc):
    """IC0 factor of the 3D 7-point Laplacian 64^3 + 1e-2 I."""
    A = mg.lap3d(64, 1e-2)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    assert ok
    Lt = mg.CSR(U.n, U.p, U.i, f)  # CSC of L = upper CSR of L^T
    L = mg.transpose(Lt)
    return A, L, Lt


def _oracle_mrhs(orc, L, B_rowmajor):
    n, k = B_rowmajor.shape
    X = np.ascontiguousarray(B_rowmajor.T.copy())  # column-major n x k
    orc.sptrsv_csr_mrhs(n, *L.astuple(), X, k, 8)
    return X.T


@pytest.mark.parametrize("k", [1, 3, 8, 64])
def test_c2_forward_multi_rhs_bit_exact(gpu, orc, c2_factor, k):
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    rng = np.random.default_rng(k)
    B = rng.standard_normal((L.n, k))
    ref = _oracle_mrhs(orc, L, B)
    plan = TriPlan(L.n, *L.astuple())
    assert plan.info().levels == 190
    x = torch.from_numpy(B.copy()).cuda()
    plan.solve(x if k > 1 else x.view(-1))
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), ref)


@pytest.mark.parametrize("exec_mode", [1, 2, 3, 4, 5, 6])
def test_executors_agree(gpu, orc, c2_factor, exec_mode):
    from sympiler_gb300.plans import TriPlan
    _, L, Lt = c2_factor
    rng = np.random.default_rng(7)
    b = rng.standard_normal(L.n)
    ref = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), ref)
    plan = TriPlan(L.n, *L.astuple())
    plan.set_exec(exec_mode)
    x = torch.from_numpy(b.copy()).cuda()
    plan.solve(x)
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), ref)
    # the transposed (backward) solve on the CSC of L
    ref_t = b.copy()
    orc.ltsolve(L.n, *Lt.astuple(), ref_t)
    from sympiler_gb300._lib import UPPER_DIAG_FIRST
    pt = TriPlan(L.n, *Lt.astuple(), kind=UPPER_DIAG_FIRST)
    pt.set_exec(exec_mode)
    x = torch.from_numpy(b.copy()).cuda()
    pt.solve(x)
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), ref_t)


@pytest.mark.parametrize("exec_mode", [1, 2, 4, 5])
@pytest.mark.parametrize("k", [2, 3, 16, 64])
def test_multi_rhs_executors(gpu, orc, c2_factor, exec_mode, k):
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    rng = np.random.default_rng(100 + k)
    B = rng.standard_normal((L.n, k))
    ref = _oracle_mrhs(orc, L, B)
    plan = TriPlan(L.n, *L.astuple())
    plan.set_exec(exec_mode)
    x = torch.from_numpy(B.copy()).cuda()
    for _ in range(2):  # second run replays the cached graph / resets the barrier
        x.copy_(torch.from_numpy(B))
        plan.solve(x)
    plan.check()
    assert np.array_equal(x.cpu().numpy(), ref)


@pytest.mark.parametrize("exec_mode", [1, 2, 4, 5, 6])
@pytest.mark.parametrize("k", [1, 8])
def test_fused_arithmetic_within_tolerance(gpu, orc, c2_factor, exec_mode, k):
    """FUSED mode (one FMA per entry) stays within 1e-12 relative of the
    reference's FP64 result."""
    from sympiler_gb300._lib import ARITH_FUSED
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    rng = np.random.default_rng(200 + k)
    B = rng.standard_normal((L.n, k))
    ref = _oracle_mrhs(orc, L, B)
    plan = TriPlan(L.n, *L.astuple())
    plan.set_exec(exec_mode)
    plan.set_arith(ARITH_FUSED)
    x = torch.from_numpy(B.copy()).cuda()
    plan.solve(x if k > 1 else x.view(-1))
    plan.check()
    got = x.cpu().numpy()
    rel = np.abs(got - ref).max() / np.abs(ref).max()
    assert rel < 1e-12, rel


@pytest.mark.parametrize("rows", [64, 1000, 25600])
def test_partitioned_executor_partition_sizes(gpu, orc, c2_factor, monkeypatch, rows):
    """Contiguous partitions of 64 rows (many partitions per block), 1000
    rows and 25,600 rows (levels wider than a block inside a partition),
    forward and backward, FP64 and FP32 storage: the oracle's bits."""
    from sympiler_gb300._lib import EXEC_PARTITIONED, UPPER_DIAG_FIRST
    from sympiler_gb300.plans import TriPlan
    monkeypatch.setenv("GBSYM_PART_ROWS", str(rows))
    _, L, Lt = c2_factor
    b = np.random.default_rng(rows).standard_normal(L.n)
    for kind, M, solve in ((None, L, orc.sptrsv_csr), (UPPER_DIAG_FIRST, Lt, orc.ltsolve)):
        ref = b.copy()
        solve(L.n, *M.astuple(), ref)
        plan = TriPlan(L.n, *M.astuple()) if kind is None else TriPlan(L.n, *M.astuple(), kind=kind)
        plan.set_exec(EXEC_PARTITIONED)
        x = torch.from_numpy(b.copy()).cuda()
        for _ in range(2):
            x.copy_(torch.from_numpy(b))
            plan.solve(x)
        plan.check()
        assert np.array_equal(x.cpu().numpy(), ref)
    ref32 = b.astype(np.float32)
    orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), ref32)
    p32 = TriPlan(L.n, *L.astuple(), dtype="f32")
    p32.set_exec(EXEC_PARTITIONED)
    x32 = torch.from_numpy(b.astype(np.float32)).cuda()
    p32.solve(x32)
    p32.check()
    assert np.array_equal(x32.cpu().numpy(), ref32)


def _long_rows_lower(n=3000, seed=21):
    """Lower triangle whose rows hold 0 to ~60 off-diagonals, plus a few rows
    with hundreds: every executor's overflow path (entries past the 8-slot
    slab) runs.  Off-diagonals are scaled by the row length so the solution
    stays bounded."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    m = sp.random(n, n, density=0.02, format="coo", random_state=rng)
    low = m.row > m.col
    r, c = list(m.row[low]), list(m.col[low])
    for i in (n - 7, n - 5, n - 2):  # near-dense rows
        cols = np.arange(0, i, 7)
        r += [i] * len(cols)
        c += list(cols)
    r, c = np.array(r), np.array(c)
    M = sp.coo_matrix((np.ones(len(r)), (r, c)), shape=(n, n)).tocsr()
    M.data[:] = 1.0  # duplicates summed above
    lens = np.diff(M.indptr)
    M.data = rng.uniform(-1.0, 1.0, M.nnz) / (1.0 + np.repeat(lens, lens))
    D = sp.diags(1.0 + rng.uniform(0.0, 1.0, n))
    return mg.from_scipy(M + D)


@pytest.mark.parametrize("exec_mode", [1, 2, 3, 4, 5, 6])
def test_long_rows_every_executor(gpu, orc, exec_mode):
    from sympiler_gb300.plans import TriPlan
    L = _long_rows_lower()
    assert np.diff(L.p).max() > 100
    plan = TriPlan(L.n, *L.astuple())
    plan.set_exec(exec_mode)
    p32 = TriPlan(L.n, *L.astuple(), dtype="f32")
    p32.set_exec(exec_mode)
    rng = np.random.default_rng(exec_mode)
    for k in (1, 5, 64):
        B = rng.standard_normal((L.n, k))
        ref = _oracle_mrhs(orc, L, B)
        x = torch.from_numpy(B.copy()).cuda()
        plan.solve(x if k > 1 else x.view(-1))
        plan.check()
        assert np.array_equal(x.cpu().numpy(), ref), k
    b32 = rng.standard_normal(L.n).astype(np.float32)
    ref32 = b32.copy()
    orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), ref32)
    x32 = torch.from_numpy(b32.copy()).cuda()
    p32.solve(x32)
    p32.check()
    assert np.array_equal(x32.cpu().numpy(), ref32)


def _banded_lower(n, w, seed):
    """Lower triangle with w sub-diagonals: every row past the first w holds
    exactly w off-diagonals, so the plan's slab is w entries wide."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    offs = list(range(0, -w - 1, -1))
    diags = [1.0 + rng.uniform(0.0, 1.0, n)] + [rng.uniform(-1.0, 1.0, n - d) / (w + 1) for d in range(1, w + 1)]
    return mg.from_scipy(sp.diags(diags, offs, shape=(n, n), format="csr"))


def _banded_with_long_rows(n, w, seed):
    """_banded_lower plus three rows holding ~n/7 off-diagonals each: the
    slab stays w wide and those rows run the overflow path."""
    import scipy.sparse as sp
    B = _banded_lower(n, w, seed).scipy().tolil()
    rng = np.random.default_rng(seed + 1)
    for i in (n // 2, n - 3, n - 1):
        for j in range(0, i - w, 7):
            B[i, j] = rng.uniform(-1.0, 1.0) / n
    return mg.from_scipy(B.tocsr())


@pytest.mark.parametrize("w", [1, 2, 3, 4, 5, 8])
def test_syncfree_every_slab_width(gpu, orc, w):
    """The sync-free sweep is compiled once per slab width (2, 3, 4 and the
    full 8); each width's kernels match the oracle bit for bit in FP64 at 1,
    8 and 64 right-hand sides, with and without rows past the slab (the
    overflow path), and in FP32 at one."""
    from sympiler_gb300._lib import EXEC_SYNCFREE
    from sympiler_gb300.plans import TriPlan
    rng = np.random.default_rng(100 + w)
    for L in (_banded_lower(4099, w, seed=w), _banded_with_long_rows(4099, w, seed=w)):
        plan = TriPlan(L.n, *L.astuple())
        plan.set_exec(EXEC_SYNCFREE)
        for k in (1, 8, 64):
            B = rng.standard_normal((L.n, k))
            ref = _oracle_mrhs(orc, L, B)
            x = torch.from_numpy(B.copy()).cuda()
            plan.solve(x if k > 1 else x.view(-1))
            plan.check()
            assert np.array_equal(x.cpu().numpy(), ref), (w, k)
    L = _banded_lower(4099, w, seed=w)
    p32 = TriPlan(L.n, *L.astuple(), dtype="f32")
    p32.set_exec(EXEC_SYNCFREE)
    b32 = rng.standard_normal(L.n).astype(np.float32)
    ref32 = b32.copy()
    orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), ref32)
    x32 = torch.from_numpy(b32.copy()).cuda()
    p32.solve(x32)
    p32.check()
    assert np.array_equal(x32.cpu().numpy(), ref32), w


@pytest.mark.parametrize("alt", ["0", "1"])
@pytest.mark.parametrize("w", [3, 5])
def test_syncfree_lane_layouts_fp32_fp64(gpu, orc, monkeypatch, w, alt):
    """Both lane layouts of the multi-RHS sync-free sweep (FP64: one or two
    values per lane; FP32: four, or two when k is odd, or two), with and
    without rows past the
    slab: FP64 bit-exact against the oracle, FP32 against the FP32 oracle
    column by column."""
    from sympiler_gb300._lib import EXEC_SYNCFREE
    from sympiler_gb300.plans import TriPlan
    monkeypatch.setenv("GBSYM_SF_ALT_LANES", alt)
    rng = np.random.default_rng(300 + w)
    for L in (_banded_lower(3001, w, seed=w), _banded_with_long_rows(3001, w, seed=w)):
        for dt in ("f64", "f32"):
            plan = TriPlan(L.n, *L.astuple(), dtype=dt)
            plan.set_exec(EXEC_SYNCFREE)
            for k in (3, 8, 64):
                B = rng.standard_normal((L.n, k))
                if dt == "f64":
                    ref = _oracle_mrhs(orc, L, B)
                else:
                    B = B.astype(np.float32)
                    ref = np.empty_like(B)
                    for c in range(k):
                        r = np.ascontiguousarray(B[:, c])
                        orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), r)
                        ref[:, c] = r
                x = torch.from_numpy(B.copy()).cuda()
                plan.solve(x)
                plan.check()
                assert np.array_equal(x.cpu().numpy(), ref), (w, dt, k, alt)


@pytest.mark.parametrize("exec_mode", [1, 2, 4, 5])
def test_out_of_place_solve_every_executor(gpu, orc, c2_factor, exec_mode):
    """gbsym_tri_solve_into: x = L^-1 b with b unchanged, bit-identical to the
    in-place solve and the oracle at 1, 8 and 64 right-hand sides in FP64,
    and against the FP32 oracle in FP32."""
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    rng = np.random.default_rng(21)
    plan = TriPlan(L.n, *L.astuple())
    plan.set_exec(exec_mode)
    for k in (1, 8, 64):
        B = rng.standard_normal((L.n, k))
        ref = _oracle_mrhs(orc, L, B)
        b = torch.from_numpy(B.copy()).cuda()
        x = torch.full_like(b, 7.0)
        plan.solve_into(b if k > 1 else b.view(-1), x if k > 1 else x.view(-1))
        plan.check()
        assert np.array_equal(x.cpu().numpy(), ref), k
        assert np.array_equal(b.cpu().numpy(), B), k
    p32 = TriPlan(L.n, *L.astuple(), dtype="f32")
    p32.set_exec(exec_mode)
    B = rng.standard_normal((L.n, 4)).astype(np.float32)
    b = torch.from_numpy(B.copy()).cuda()
    x = torch.empty_like(b)
    p32.solve_into(b, x)
    p32.check()
    got = x.cpu().numpy()
    for c in range(4):
        r = np.ascontiguousarray(B[:, c])
        orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), r)
        assert np.array_equal(got[:, c], r), c


def test_autotune_picks_a_working_executor(gpu, orc, c2_factor):
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    plan = TriPlan(L.n, *L.astuple())
    chosen = plan.autotune(k=1)
    assert chosen in (1, 2, 3, 4, 5, 6)
    tun = plan.tuning(1)
    assert tun["exec"] == chosen and tun["lookthrough"] in (0, 1)
    assert tun["blocks_per_sm"] in (0, 1, 2, 3)
    b = np.random.default_rng(8).standard_normal(L.n)
    ref = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), ref)
    x = torch.from_numpy(b.copy()).cuda()
    plan.solve(x)
    plan.check()
    assert np.array_equal(x.cpu().numpy(), ref)


def test_fp32_storage_bit_exact_vs_fp32_oracle(gpu, orc, c2_factor):
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    rng = np.random.default_rng(3)
    b = rng.standard_normal(L.n).astype(np.float32)
    ref = b.copy()
    orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), ref)
    plan = TriPlan(L.n, *L.astuple(), dtype="f32")
    x = torch.from_numpy(b.copy()).cuda()
    plan.solve(x)
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), ref)
    B = rng.standard_normal((L.n, 16)).astype(np.float32)
    xb = torch.from_numpy(B.copy()).cuda()
    plan.solve(xb)
    torch.cuda.synchronize()
    got = xb.cpu().numpy()
    for c in (0, 7, 15):
        r = np.ascontiguousarray(B[:, c])
        orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), r)
        assert np.array_equal(got[:, c], r)


def test_column_major_and_host_solve(gpu, orc, c2_factor):
    from sympiler_gb300._lib import COL_MAJOR
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    rng = np.random.default_rng(9)
    k = 5
    Bc = rng.standard_normal((k, L.n))  # column-major n x k == k rows of n
    ref = Bc.copy()
    orc.sptrsv_csr_mrhs(L.n, *L.astuple(), ref, k, 8)
    plan = TriPlan(L.n, *L.astuple())
    x = torch.from_numpy(Bc.copy()).cuda()
    plan.solve(x, layout=COL_MAJOR)
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), ref)
    h = Bc.copy()
    plan.solve_host(h, layout=COL_MAJOR)
    assert np.array_equal(h, ref)


@pytest.mark.parametrize("k", [1, 8, 64])
@pytest.mark.parametrize("pinned", [True, False])
def test_host_solve_in_place_and_staged(gpu, orc, c2_factor, k, pinned):
    """Row-major host buffers: page-locked memory is solved in place over the
    CPU-GPU link where the system is coherent, pageable memory is staged;
    both must give the oracle's bits, twice in a row on one plan."""
    from sympiler_gb300._lib import ROW_MAJOR
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    rng = np.random.default_rng(100 + k)
    B = rng.standard_normal((L.n, k))
    ref = _oracle_mrhs(orc, L, B)
    plan = TriPlan(L.n, *L.astuple())
    for _ in range(2):
        if pinned:
            h = torch.from_numpy(B.copy()).pin_memory()
            plan.solve_host_ptr(h.data_ptr(), k, layout=ROW_MAJOR)
            got = h.numpy()
        else:
            got = B.copy()
            plan.solve_host(got, layout=ROW_MAJOR)
        assert np.array_equal(got.reshape(L.n, k), ref)


def test_plan_from_device_arrays_and_schedule(gpu, orc):
    from sympiler_gb300.plans import TriPlan
    A = mg.lap2d(100)
    L = mg.tril(A)
    nl, lp, ls = orc.build_levelset_csr(L.n, L.p, L.i)
    dev = [torch.from_numpy(a.copy()).cuda() for a in L.astuple()]
    plan = TriPlan(L.n, *dev, level_ptr=torch.from_numpy(lp).cuda(), level_set=torch.from_numpy(ls).cuda())
    got = plan.schedule()
    assert got[0] == nl and np.array_equal(got[1], lp) and np.array_equal(got[2], ls)
    b = np.random.default_rng(1).uniform(-1, 1, L.n)
    ref = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), ref)
    x = torch.from_numpy(b.copy()).cuda()
    plan.solve(x)
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), ref)


def test_batch_uneven_systems(gpu, orc):
    from sympiler_gb300.plans import BatchPlan
    rng = np.random.default_rng(4)
    systems, Ls = [], []
    for q in range(24):
        if q % 5 == 4:
            A = mg.random_spd(int(rng.integers(300, 3000)), 8, rng)
        else:
            A = mg.lap2d(int(rng.integers(30, 80)), int(rng.integers(30, 80)))
            A = mg.from_scipy(A.scipy() + float(rng.uniform(1e-3, 1)) * __import__("scipy").sparse.eye(A.n))
        U = mg.triu(A)
        f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
        assert ok
        L = mg.transpose(mg.CSR(U.n, U.p, U.i, f))
        Ls.append(L)
        systems.append((L.n, *L.astuple()))
    bp = BatchPlan(systems)
    k = 8
    N = int(bp.offsets[-1])
    B = rng.standard_normal((N, k))
    x = torch.from_numpy(B.copy()).cuda()
    bp.solve(x)
    torch.cuda.synchronize()
    got = x.cpu().numpy()
    for q, L in enumerate(Ls):
        a, z = bp.offsets[q], bp.offsets[q + 1]
        ref = _oracle_mrhs(orc, L, B[a:z])
        assert np.array_equal(got[a:z], ref), q
    # the batch solve captured in a CUDA graph and replayed on new inputs
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        bp.solve(x)
    for replay in range(2):
        B2 = rng.standard_normal((N, k))
        x.copy_(torch.from_numpy(B2))
        g.replay()
        torch.cuda.synchronize()
        got = x.cpu().numpy()
        for q in (0, len(Ls) // 2, len(Ls) - 1):
            a, z = bp.offsets[q], bp.offsets[q + 1]
            assert np.array_equal(got[a:z], _oracle_mrhs(orc, Ls[q], B2[a:z])), (replay, q)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("k", [8, 64])
def test_batch_host_buffers(gpu, orc, dtype, k):
    """gbsym_batch_solve_host: page-locked host buffers (in place over the
    CPU-GPU link where the system allows it and rows hold 256 bytes or
    more, else staged) and pageable ones (staged) give the device solve's
    bits; FP64 against the oracle as well."""
    from sympiler_gb300._lib import lib
    from sympiler_gb300.plans import BatchPlan
    rng = np.random.default_rng(41)
    systems, Ls = [], []
    for q in range(6):
        if q % 3 == 2:
            A = mg.random_spd(int(rng.integers(200, 1500)), 8, rng)
        else:
            A = mg.lap2d(int(rng.integers(20, 50)), int(rng.integers(20, 50)))
            A = mg.from_scipy(A.scipy() + 0.5 * __import__("scipy").sparse.eye(A.n))
        U = mg.triu(A)
        f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
        assert ok
        L = mg.transpose(mg.CSR(U.n, U.p, U.i, f))
        Ls.append(L)
        systems.append((L.n, *L.astuple()))
    bp = BatchPlan(systems, dtype=dtype)
    tdt = torch.float64 if dtype == "f64" else torch.float32
    N = int(bp.offsets[-1])
    B = torch.from_numpy(rng.standard_normal((N, k))).to(tdt)
    xd = B.clone().cuda()
    bp.solve(xd)
    torch.cuda.synchronize()
    want = xd.cpu()
    pinned = B.clone().pin_memory()
    bp.solve_host(pinned)
    assert torch.equal(pinned, want)
    pageable = B.clone()
    bp.solve_host(pageable)
    assert torch.equal(pageable, want)
    assert lib().gbsym_host_solve_in_place(C.c_void_p(pageable.data_ptr())) == 0
    if dtype == "f64":
        got = pinned.numpy()
        for q, L in enumerate(Ls):
            a, z = bp.offsets[q], bp.offsets[q + 1]
            assert np.array_equal(got[a:z], _oracle_mrhs(orc, L, B.numpy()[a:z])), q


def test_lower_csc_plan_matches_column_push_oracle(gpu, orc):
    """A plan built from the CSC of L (transposed on the GPU) reproduces the
    reference's column-push sptrsv_csc bit for bit."""
    from sympiler_gb300._lib import LOWER_CSC
    from sympiler_gb300.plans import TriPlan
    U = mg.triu(mg.random_spd(3000, 8, np.random.default_rng(12)))
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    b = np.random.default_rng(13).standard_normal(U.n)
    ref = b.copy()
    orc.sptrsv_csc(U.n, U.p, U.i, f, ref)
    dev = [torch.from_numpy(a.copy()).cuda() for a in (U.p, U.i, f)]
    P = TriPlan(U.n, *dev, kind=LOWER_CSC)
    x = torch.from_numpy(b.copy()).cuda()
    P.solve(x)
    P.check()
    assert np.array_equal(x.cpu().numpy(), ref)


@pytest.mark.parametrize("k", [1, 64])
def test_syncfree_solve_captured_in_cuda_graph(gpu, orc, c2_factor, k):
    """A plan's sync-free solve (sentinel fill + cooperative sweep) captured
    into a CUDA graph and replayed on new right-hand sides: every replay
    bit-exact.  The first, uncaptured solve allocates the plan's scratch and
    warp units; replays allocate nothing."""
    from sympiler_gb300._lib import EXEC_SYNCFREE
    from sympiler_gb300.plans import TriPlan
    _, L, _ = c2_factor
    plan = TriPlan(L.n, *L.astuple())
    plan.set_exec(EXEC_SYNCFREE)
    X = torch.zeros((L.n, k), dtype=torch.float64, device="cuda")
    Xv = X if k > 1 else X.view(-1)
    plan.solve(Xv)  # warm: scratch and unit lists
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        plan.solve(Xv)
    rng = np.random.default_rng(60 + k)
    for replay in range(3):
        B = rng.standard_normal((L.n, k))
        X.copy_(torch.from_numpy(B))
        g.replay()
        torch.cuda.synchronize()
        plan.check()
        assert np.array_equal(X.cpu().numpy(), _oracle_mrhs(orc, L, B)), replay
