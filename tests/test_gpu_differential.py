"""The reference's randomised differential tests, on the GPU.

Catch_tests/sptrsv_tests.cpp:46-80 compares sptrsv_csr_levelset with the
serial sptrsv_csr, and Catch_tests/spmv_tests.cpp:76-106 compares
spmv_csr_parallel with spmv_csr, on random sparse matrices at
(n, density) in {(10, .2), (100, .03), (500, .004), (1000, 5e-4),
(10000, 1e-4)}.  Here the same sizes and densities (seeded synthetic
matrices: the reference's generator lives in its unvendored aggregation
dependency) run through the drop-ins and through every plan executor, each
compared bit for bit with the oracle's serial result."""
import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu

CASES = [(10, 0.2), (100, 0.03), (500, 0.004), (1000, 5e-4), (10000, 1e-4)]


@pytest.mark.parametrize("n,density", CASES)
def test_levelset_equals_serial(gpu, orc, n, density):
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import (EXEC_CLUSTER, EXEC_LEVELSET, EXEC_ONEBLOCK, EXEC_PARTITIONED,
                                     EXEC_PERSISTENT, EXEC_SYNCFREE)
    from sympiler_gb300.plans import TriPlan
    rng = np.random.default_rng(n)
    L = mg.random_lower(n, density, rng)
    b = rng.uniform(-1, 1, n)
    ref = b.copy()
    orc.sptrsv_csr(n, *L.astuple(), ref)
    # the drop-ins: serial form and level-set form with the GPU-built schedule
    x = b.copy()
    sym_lib.sptrsv_csr(n, *L.astuple(), x)
    assert np.array_equal(x, ref)
    nl, lp, ls = sym_lib.build_levelset_csr(n, L.p, L.i)
    x = b.copy()
    sym_lib.sptrsv_csr_levelset(n, *L.astuple(), x, nl, lp, ls)
    assert np.array_equal(x, ref)
    # every executor of a resident plan, one and three right-hand sides
    P = TriPlan(n, *L.astuple())
    B3 = rng.uniform(-1, 1, (n, 3))
    ref3 = np.empty_like(B3)
    for c in range(3):
        col = B3[:, c].copy()
        orc.sptrsv_csr(n, *L.astuple(), col)
        ref3[:, c] = col
    for e in (EXEC_LEVELSET, EXEC_SYNCFREE, EXEC_ONEBLOCK, EXEC_PERSISTENT, EXEC_CLUSTER, EXEC_PARTITIONED):
        P.set_exec(e)
        xd = torch.from_numpy(b.copy()).cuda()
        P.solve(xd)
        P.check()
        assert np.array_equal(xd.cpu().numpy(), ref), e
        Xd = torch.from_numpy(B3.copy()).cuda()
        P.solve(Xd)
        P.check()
        assert np.array_equal(Xd.cpu().numpy(), ref3), e


@pytest.mark.parametrize("n,density", CASES)
def test_spmv_parallel_equals_serial(gpu, orc, n, density):
    from sympiler_gb300 import sym_lib
    import scipy.sparse as sp
    rng = np.random.default_rng(100 + n)
    m = sp.random(n, n, density=density, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.uniform(-1.0, 1.0, s))
    A = mg.from_scipy(m + sp.eye(n, format="csr"))
    xv = rng.uniform(-1, 1, n)
    ref = np.zeros(n)
    orc.spmv_csr(n, *A.astuple(), xv, ref)
    y = np.zeros(n)
    sym_lib.spmv_csr(n, *A.astuple(), xv, y)
    assert np.array_equal(y, ref)
    y = np.zeros(n)
    sym_lib.spmv_csr_parallel(n, *A.astuple(), xv, y)
    assert np.array_equal(y, ref)
