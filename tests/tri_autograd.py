"""torch.autograd wrapper of the triangular solve, for the tests only.

X = L^{-1} B with L lower triangular in CSR (diagonal last), its pattern
fixed and its stored values a tensor.  The forward pass is the library's
solve (gbsym_tri_solve_into on a plan built from the values); the backward
pass is the library's adjoint (gbsym_tri_adjoint): grad_B = L^{-T} grad_X
by the transposed solve on the CSC of L, and the gradient on L's stored
values -grad_B[i] . X[j] for every stored entry (i, j).  X is kept from the
forward pass, so nothing is recomputed and memory stays O(nnz + n k).
"""
from __future__ import annotations

import numpy as np
import torch

from sympiler_gb300._lib import UPPER_DIAG_FIRST
from sympiler_gb300.plans import TriPlan, tri_adjoint


class LowerPattern:
    """The fixed pattern of L on the device, with the entry permutation
    that lists L's values in CSC order (the CSR of L^T)."""

    def __init__(self, n, Lp, Li, device="cuda"):
        self.n = int(n)
        Lp = np.ascontiguousarray(Lp, dtype=np.int32)
        Li = np.ascontiguousarray(Li, dtype=np.int32)
        rows = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(Lp))
        order = np.lexsort((rows, Li))  # by column, then row: CSC order
        cnt = np.bincount(Li, minlength=self.n)
        Tp = np.zeros(self.n + 1, dtype=np.int32)
        np.cumsum(cnt, out=Tp[1:])
        self.Lp = torch.from_numpy(Lp).to(device)
        self.Li = torch.from_numpy(Li).to(device)
        self.Tp = torch.from_numpy(Tp).to(device)
        self.Ti = torch.from_numpy(rows[order].astype(np.int32)).to(device)
        self.to_csc = torch.from_numpy(order.astype(np.int64)).to(device)


class TriSolve(torch.autograd.Function):
    """X = L^{-1} B; differentiable in L's stored values and in B."""

    @staticmethod
    def forward(ctx, values, B, pat):
        plan = TriPlan(pat.n, pat.Lp, pat.Li, values.detach().contiguous())
        X = torch.empty_like(B)
        plan.solve_into(B.detach().contiguous(), X)
        plan.check()
        ctx.pat = pat
        ctx.save_for_backward(values, X)
        return X

    @staticmethod
    def backward(ctx, grad_X):
        values, X = ctx.saved_tensors
        pat = ctx.pat
        vt = values.detach()[pat.to_csc].contiguous()
        PT = TriPlan(pat.n, pat.Tp, pat.Ti, vt, kind=UPPER_DIAG_FIRST)
        g = grad_X.detach().contiguous().clone()
        grad = torch.zeros_like(values)
        tri_adjoint(PT, pat.n, pat.Lp, pat.Li, X.contiguous(), g, grad)
        PT.check()
        return grad, g, None


def tri_solve(values, B, pat):
    return TriSolve.apply(values, B, pat)
