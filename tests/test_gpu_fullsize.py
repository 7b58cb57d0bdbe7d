"""Parity at the full workload sizes, through the C ABI, against the oracle.

* 96^3 upwind convection-diffusion (n = 884,736): the GPU ILU0 factor, one
  FP64 and one FP32 ILU0 apply (lus_cr), and GMRES(30) with the FP64 and
  the FP32 preconditioner.
* 512 uneven SPD systems through the batch API (gbsym_batch_*), FP64 and
  FP32, 8 right-hand sides: every system against its own oracle solve.
* 1024^2 anisotropic Poisson IC0 factor (n = 1,048,576), 32 right-hand
  sides: the forward solve, and the adjoint against central finite
  differences on 100 random entries (the 64^2 instance is checked against a
  dense FP64 gradient in test_adjoint_dense_64).

Bars: bit-identical (np.array_equal) for every solve and factor; the Krylov
drivers by iteration count and residual; the adjoint by the relative
tolerance 1e-6 against finite differences at h = 1e-6.
"""
import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


# ---------------------------------------------------------------------------
# 96^3 convection-diffusion: ILU0 factor, applies, GMRES

@pytest.fixture(scope="module")
def c3(orc):
    C = mg.convdiff3d(96)
    d = mg.diag_ptr(C)
    lu, ok = orc.spilu0_csr(C.n, C.p, C.i, C.x, d)
    assert ok
    return C, d, lu


def test_c3_ilu0_factor_bit_exact(gpu, c3):
    from sympiler_gb300.plans import ilu0_device
    C, d, lu = c3
    assert C.n == 884736 and C.nnz == 6137856
    out = torch.zeros(C.nnz, dtype=torch.float64, device="cuda")
    ilu0_device(C.n, *(torch.from_numpy(a).cuda() for a in (C.p, C.i, C.x, d)), out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), lu)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_c3_ilu0_apply_bit_exact(gpu, orc, c3, prec):
    """M^-1 r as lus_cr computes it (mgmres.cpp:598-689): unit-lower forward
    solve then the upper solve with a division, on the two plans GMRES
    uses, in FP64 and in FP32 (factor and vectors)."""
    from sympiler_gb300._lib import ILU_UNIT_LOWER, ILU_UPPER
    from sympiler_gb300.plans import TriPlan
    C, d, lu = c3
    r = np.random.default_rng(9).uniform(-1, 1, C.n)
    Lu = TriPlan(C.n, C.p, C.i, lu, kind=ILU_UNIT_LOWER, diags=d, dtype=prec)
    Up = TriPlan(C.n, C.p, C.i, lu, kind=ILU_UPPER, diags=d, dtype=prec)
    assert Lu.info().levels == 286 and Up.info().levels == 286
    if prec == "f64":
        want = orc.lus_cr(C.n, C.p, C.i, lu, d, r)
        z = torch.from_numpy(r.copy()).cuda()
    else:
        want = orc.lus_cr_f32(C.n, C.p, C.i, lu.astype(np.float32), d, r.astype(np.float32))
        z = torch.from_numpy(r.astype(np.float32)).cuda()
    Lu.solve(z)
    Up.solve(z)
    Up.check()
    assert np.array_equal(z.cpu().numpy(), want)


def test_c3_gmres_fp64_and_fp32_preconditioner(gpu, orc, c3):
    """GMRES(30), right ILU0, tolerance 1e-10.  FP64 preconditioner: the
    iteration count within 2 of the oracle's driver.  FP32 preconditioner:
    converges to the same FP64 tolerance; both solutions agree with the
    oracle's to the accuracy the tolerance gives (stated bound 1e-7)."""
    from sympiler_gb300._lib import ILU_UNIT_LOWER, ILU_UPPER
    from sympiler_gb300.plans import CsrPlan, TriPlan, gmres
    C, d, lu = c3
    b = np.random.default_rng(9).uniform(-1, 1, C.n)
    xo, ito, relo = orc.gmres_ilu0(C.n, C.astuple(), lu, d, b, 30, 100, 1e-10)
    assert relo <= 1e-10
    A = CsrPlan(C.n, *C.astuple())
    bt = torch.from_numpy(b).cuda()
    iters = {}
    for prec in ("f64", "f32"):
        Lu = TriPlan(C.n, C.p, C.i, lu, kind=ILU_UNIT_LOWER, diags=d, dtype=prec)
        Up = TriPlan(C.n, C.p, C.i, lu, kind=ILU_UPPER, diags=d, dtype=prec)
        x = torch.zeros(C.n, dtype=torch.float64, device="cuda")
        res = gmres(A, Lu, Up, bt, x, mr=30, maxit=100, tol=1e-10)
        assert res.status == 0, prec
        assert res.relres <= 2e-10, (prec, res.relres)  # the true FP64 residual
        xg = x.cpu().numpy()
        err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
        assert err <= 1e-7, (prec, err)
        iters[prec] = res.iterations
    assert abs(iters["f64"] - ito) <= 2, (iters, ito)


# ---------------------------------------------------------------------------
# 512 uneven systems through the batch API

def _oracle_mrhs(orc, L, B_rowmajor, threads=8):
    n, k = B_rowmajor.shape
    X = np.ascontiguousarray(B_rowmajor.T.copy())  # column-major n x k
    orc.sptrsv_csr_mrhs(n, *L.astuple(), X, k, threads)
    return X.T


@pytest.fixture(scope="module")
def c4_systems(orc):
    """The batched workload's 512 systems (80% shifted 2D Laplacians on
    30..300 grids, 20% random diagonally dominant with n 900..90,000), IC0
    factors by the oracle, as lower CSRs (diagonal last)."""
    Ls = []
    for n, p, i, x in mg.batch_systems_upper(512, np.random.default_rng(44)):
        f, ok = orc.spic0_csr(n, p, i, x)
        assert ok
        Ls.append(mg.transpose(mg.CSR(n, p, i, f)))
    return Ls


def test_c4_batch_512_systems_fp64(gpu, orc, c4_systems):
    from sympiler_gb300.plans import BatchPlan
    Ls = c4_systems
    bp = BatchPlan([(L.n, *L.astuple()) for L in Ls])
    k = 8
    N = int(bp.offsets[-1])
    assert N == sum(L.n for L in Ls) == 15728058
    bp.autotune(k=k, dtype="f64")
    B = np.random.default_rng(45).standard_normal((N, k))
    x = torch.from_numpy(B.copy()).cuda()
    bp.solve(x)
    bp.check()
    got = x.cpu().numpy()
    for q, L in enumerate(Ls):
        a, z = bp.offsets[q], bp.offsets[q + 1]
        assert np.array_equal(got[a:z], _oracle_mrhs(orc, L, B[a:z])), q


def test_c4_batch_512_systems_fp32(gpu, orc, c4_systems):
    """FP32 factor and vectors; each system and right-hand side against the
    FP32 oracle solve (values rounded to FP32 once, as the plan stores them)."""
    from sympiler_gb300.plans import BatchPlan
    Ls = c4_systems
    bp = BatchPlan([(L.n, *L.astuple()) for L in Ls], dtype="f32")
    k = 8
    N = int(bp.offsets[-1])
    bp.autotune(k=k, dtype="f32")
    B = np.random.default_rng(46).standard_normal((N, k)).astype(np.float32)
    x = torch.from_numpy(B.copy()).cuda()
    bp.solve(x)
    bp.check()
    got = x.cpu().numpy()
    for q, L in enumerate(Ls):
        a, z = bp.offsets[q], bp.offsets[q + 1]
        v32 = L.x.astype(np.float32)
        for c in range(k):
            r = np.ascontiguousarray(B[a:z, c])
            orc.sptrsv_csr_f32(L.n, L.p, L.i, v32, r)
            assert np.array_equal(got[a:z, c], r), (q, c)


# ---------------------------------------------------------------------------
# 1024^2 anisotropic Poisson IC0: forward solve and adjoint

@pytest.fixture(scope="module")
def c5(orc):
    rng = np.random.default_rng(55)
    A = mg.aniso_poisson2d(1024, 0.01, 1.0, rng)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    assert ok
    Lt = mg.CSR(U.n, U.p, U.i, f)  # CSC of L
    L = mg.transpose(Lt)
    k = 32
    B = rng.standard_normal((L.n, k))
    W = rng.standard_normal((L.n, k))
    return L, Lt, B, W


def test_c5_forward_32rhs_bit_exact(gpu, orc, c5):
    from sympiler_gb300.plans import TriPlan
    L, _, B, _ = c5
    assert L.n == 1048576 and L.nnz == 3143680
    P = TriPlan(L.n, *L.astuple())
    assert P.info().levels == 2047
    P.autotune(k=B.shape[1])
    X = torch.from_numpy(B.copy()).cuda()
    P.solve(X)
    P.check()
    assert np.array_equal(X.cpu().numpy(), _oracle_mrhs(orc, L, B))


def _gpu_adjoint(L, Lt, B, W):
    """Forward X = L^-1 B and the reverse pass through the C ABI: returns
    (X, grad_B = L^-T W, grad on L's stored values)."""
    from sympiler_gb300._lib import UPPER_DIAG_FIRST
    from sympiler_gb300.plans import TriPlan, tri_adjoint
    P = TriPlan(L.n, *L.astuple())
    PT = TriPlan(L.n, *Lt.astuple(), kind=UPPER_DIAG_FIRST)
    X = torch.from_numpy(B.copy()).cuda()
    P.solve(X)
    g = torch.from_numpy(W.copy()).cuda()
    grad = torch.zeros(L.nnz, dtype=torch.float64, device="cuda")
    tri_adjoint(PT, L.n, torch.from_numpy(L.p).cuda(), torch.from_numpy(L.i).cuda(), X, g, grad)
    PT.check()
    return X.cpu().numpy(), g.cpu().numpy(), grad.cpu().numpy()


def test_c5_adjoint_finite_differences_100_entries(gpu, orc, c5):
    """loss = sum(W * X), X = L^-1 B.  The GPU value gradient on 100 random
    stored entries of L against central differences (h = 1e-6) of the loss
    computed by the oracle's forward solve; relative error <= 1e-6 on every
    entry.  The difference quotient sums W * (X(+h) - X(-h)), so unaffected
    rows cancel exactly instead of through two large sums."""
    import os
    L, Lt, B, W = c5
    k = B.shape[1]
    X, GB, grad = _gpu_adjoint(L, Lt, B, W)
    assert np.array_equal(X, _oracle_mrhs(orc, L, B))
    threads = os.cpu_count() or 1
    Bc = np.ascontiguousarray(B.T)
    Wc = np.ascontiguousarray(W.T)
    h = 1e-6
    for e in np.random.default_rng(7).choice(L.nnz, 100, replace=False):
        vp, vm = L.x.copy(), L.x.copy()
        vp[e] += h
        vm[e] -= h
        Xp, Xm = Bc.copy(), Bc.copy()
        orc.sptrsv_csr_mrhs(L.n, L.p, L.i, vp, Xp, k, threads)
        orc.sptrsv_csr_mrhs(L.n, L.p, L.i, vm, Xm, k, threads)
        fd = float(np.sum(Wc * (Xp - Xm))) / (2 * h)
        assert abs(fd - grad[e]) <= 1e-6 * abs(grad[e]), (int(e), fd, grad[e])


def test_adjoint_dense_64(gpu, orc):
    """The 64 x 64-grid instance of the same operator (n = 4096), 32
    right-hand sides: grad_B and the value gradient against a dense FP64
    reference (np.linalg.solve on the dense factor)."""
    rng = np.random.default_rng(64)
    A = mg.aniso_poisson2d(64, 0.01, 1.0, rng)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    assert ok
    Lt = mg.CSR(U.n, U.p, U.i, f)
    L = mg.transpose(Lt)
    k = 32
    B = rng.standard_normal((L.n, k))
    W = rng.standard_normal((L.n, k))
    X, GB, grad = _gpu_adjoint(L, Lt, B, W)
    Ld = L.scipy().toarray()
    GBd = np.linalg.solve(Ld.T, W)
    rows = np.repeat(np.arange(L.n), np.diff(L.p))
    Gd = -np.einsum("ir,ir->i", GBd[rows], X[L.i])
    assert np.max(np.abs(GB - GBd)) <= 1e-9 * np.max(np.abs(GBd))
    assert np.max(np.abs(grad - Gd)) <= 1e-9 * np.max(np.abs(Gd))
