"""PCG / GMRES drivers and the adjoint triangular solve."""
import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def _ic0_plans(orc, A):
    from sympiler_gb300._lib import UPPER_DIAG_FIRST
    from sympiler_gb300.plans import TriPlan
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    Lt = mg.CSR(U.n, U.p, U.i, f)
    L = mg.transpose(Lt)
    return L, Lt, TriPlan(L.n, *L.astuple()), TriPlan(L.n, *Lt.astuple(), kind=UPPER_DIAG_FIRST)


def test_pcg_matches_oracle(gpu, orc):
    from sympiler_gb300.plans import CsrPlan, pcg
    A = mg.lap3d(32, 1e-2)
    L, Lt, PL, PLt = _ic0_plans(orc, A)
    rng = np.random.default_rng(1)
    xs = rng.standard_normal(A.n)
    b = A.scipy() @ xs
    xo, ito, relo = orc.pcg_ic0(A.n, A.astuple(), L.astuple(), Lt.astuple(), b, 1e-10, 1000)
    bt = torch.from_numpy(b).cuda()
    x = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    res = pcg(CsrPlan(A.n, *A.astuple()), PL, PLt, bt, x, tol=1e-10, maxit=1000)
    assert res.status == 0 and res.relres <= 1e-10
    assert abs(res.iterations - ito) <= 2
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) < 1e-8
    assert np.linalg.norm(xg - xs) / np.linalg.norm(xs) < 1e-7


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_gmres_ilu0_right(gpu, orc, prec):
    from sympiler_gb300._lib import ILU_UNIT_LOWER, ILU_UPPER
    from sympiler_gb300.plans import CsrPlan, TriPlan, gmres
    A = mg.convdiff3d(32)
    d = mg.diag_ptr(A)
    lu, ok = orc.spilu0_csr(A.n, A.p, A.i, A.x, d)
    rng = np.random.default_rng(2)
    b = rng.uniform(-1, 1, A.n)
    xo, ito, relo = orc.gmres_ilu0(A.n, A.astuple(), lu, d, b, 30, 200, 1e-10)
    Lu = TriPlan(A.n, A.p, A.i, lu, kind=ILU_UNIT_LOWER, diags=d, dtype=prec)
    Up = TriPlan(A.n, A.p, A.i, lu, kind=ILU_UPPER, diags=d, dtype=prec)
    x = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    res = gmres(CsrPlan(A.n, *A.astuple()), Lu, Up, torch.from_numpy(b).cuda(), x, mr=30, maxit=200, tol=1e-10)
    assert res.status == 0
    assert res.relres < 2e-10  # true FP64 residual
    if prec == "f64":
        assert abs(res.iterations - ito) <= 2
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) < 1e-8


def _dense_grad(L, X, W):
    """dense FP64 reference: loss = sum W * (L^{-1} B); grad_B = L^{-T} W;
    grad_L = -grad_B X^T restricted to L's pattern."""
    Ld = L.scipy().toarray()
    GB = np.linalg.solve(Ld.T, W)
    G = -GB @ X.T
    rows = np.repeat(np.arange(L.n), np.diff(L.p))
    return GB, G[rows, L.i]


@pytest.mark.parametrize("k", [6, 8, 32])
def test_adjoint_dense_and_finite_differences(gpu, orc, k):
    """The reverse pass against a dense FP64 reference and central finite
    differences; k = 8 and 32 take the four-lanes-per-row value gradient,
    k = 6 the one-thread-per-row one."""
    from sympiler_gb300._lib import UPPER_DIAG_FIRST
    from sympiler_gb300.plans import TriPlan, tri_adjoint
    rng = np.random.default_rng(5)
    A = mg.aniso_poisson2d(24, 0.01, 1.0, rng)
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    Lt = mg.CSR(U.n, U.p, U.i, f)
    L = mg.transpose(Lt)
    B = rng.standard_normal((L.n, k))
    W = rng.standard_normal((L.n, k))
    P = TriPlan(L.n, *L.astuple())
    PT = TriPlan(L.n, *Lt.astuple(), kind=UPPER_DIAG_FIRST)
    X = torch.from_numpy(B.copy()).cuda()
    P.solve(X)
    g = torch.from_numpy(W.copy()).cuda()
    grad = torch.zeros(L.nnz, dtype=torch.float64, device="cuda")
    tri_adjoint(PT, L.n, torch.from_numpy(L.p).cuda(), torch.from_numpy(L.i).cuda(), X, g, grad)
    torch.cuda.synchronize()
    GB, Gd = _dense_grad(L, X.cpu().numpy(), W)
    assert np.allclose(g.cpu().numpy(), GB, rtol=1e-10, atol=1e-12)
    gr = grad.cpu().numpy()
    assert np.max(np.abs(gr - Gd)) <= 1e-9 * np.max(np.abs(Gd))

    def loss(vals):
        Lc = mg.CSR(L.n, L.p, L.i, vals)
        Xc = B.copy().T.copy()
        orc.sptrsv_csr_mrhs(L.n, *Lc.astuple(), Xc, k, 1)
        return float(np.sum(W * Xc.T))

    h = 1e-6
    for e in rng.choice(L.nnz, 25, replace=False):
        vp, vm = L.x.copy(), L.x.copy()
        vp[e] += h
        vm[e] -= h
        fd = (loss(vp) - loss(vm)) / (2 * h)
        assert abs(fd - gr[e]) <= 1e-6 * max(1.0, abs(gr[e])), (e, fd, gr[e])
