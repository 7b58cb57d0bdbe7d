"""The adjoint through torch.autograd (the wrapper in tests/tri_autograd.py):
forward gbsym_tri_solve_into, backward gbsym_tri_adjoint.  Checked with
torch.autograd.gradcheck on a small factor, and on the 64 x 64 anisotropic
Poisson IC0 factor with 32 right-hand sides against central finite
differences (h = 1e-6, oracle forward solves) on stored values of L and on
entries of B, relative error <= 1e-6."""
import os

import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def _ic0_lower(orc, A):
    U = mg.triu(A)
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    assert ok
    return mg.transpose(mg.CSR(U.n, U.p, U.i, f))


def test_gradcheck_small(gpu, orc):
    from tri_autograd import LowerPattern, tri_solve
    L = _ic0_lower(orc, mg.lap2d(6))
    pat = LowerPattern(L.n, L.p, L.i)
    rng = np.random.default_rng(8)
    vals = torch.from_numpy(L.x.copy()).cuda().requires_grad_(True)
    B = torch.from_numpy(rng.standard_normal((L.n, 3))).cuda().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda v, b: tri_solve(v, b, pat), (vals, B), eps=1e-6, atol=1e-8,
                                    rtol=1e-6)


def test_autograd_finite_differences_64(gpu, orc):
    from tri_autograd import LowerPattern, tri_solve
    rng = np.random.default_rng(64)
    L = _ic0_lower(orc, mg.aniso_poisson2d(64, 0.01, 1.0, rng))
    k = 32
    Bn = rng.standard_normal((L.n, k))
    Wn = rng.standard_normal((L.n, k))
    pat = LowerPattern(L.n, L.p, L.i)
    vals = torch.from_numpy(L.x.copy()).cuda().requires_grad_(True)
    B = torch.from_numpy(Bn.copy()).cuda().requires_grad_(True)
    X = tri_solve(vals, B, pat)
    loss = (torch.from_numpy(Wn).cuda() * X).sum()
    loss.backward()
    gv = vals.grad.cpu().numpy()
    gb = B.grad.cpu().numpy()
    threads = os.cpu_count() or 1
    Wc = np.ascontiguousarray(Wn.T)

    def solve(values, Bcols):
        Xc = Bcols.copy()
        orc.sptrsv_csr_mrhs(L.n, L.p, L.i, values, Xc, k, threads)
        return Xc

    h = 1e-6
    Bc = np.ascontiguousarray(Bn.T)
    for e in rng.choice(L.nnz, 20, replace=False):
        vp, vm = L.x.copy(), L.x.copy()
        vp[e] += h
        vm[e] -= h
        fd = float(np.sum(Wc * (solve(vp, Bc) - solve(vm, Bc)))) / (2 * h)
        assert abs(fd - gv[e]) <= 1e-6 * abs(gv[e]), ("value", int(e), fd, gv[e])
    for flat in rng.choice(L.n * k, 20, replace=False):
        i, r = divmod(int(flat), k)
        Bp, Bm = Bc.copy(), Bc.copy()
        Bp[r, i] += h
        Bm[r, i] -= h
        fd = float(np.sum(Wc * (solve(L.x, Bp) - solve(L.x, Bm)))) / (2 * h)
        assert abs(fd - gb[i, r]) <= 1e-6 * abs(gb[i, r]), ("rhs", i, r, fd, gb[i, r])
