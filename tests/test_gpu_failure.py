"""Failure detection without a GPU fault: bounded device waits report
GBSYM_ERR_TIMEOUT and the context stays usable; malformed inputs are
refused on the host side before anything runs."""
import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(gpu, orc):
    from sympiler_gb300._lib import ERR_TIMEOUT, lib
    from sympiler_gb300.plans import TriPlan
    st = lib().gbsym_selftest_bounded_wait(50_000_000, None)  # 50 ms
    assert st == ERR_TIMEOUT
    # the device still runs work correctly afterwards
    A = mg.lap2d(40)
    L = mg.tril(A)
    b = np.random.default_rng(0).uniform(-1, 1, A.n)
    ref = b.copy()
    orc.sptrsv_csr(A.n, *L.astuple(), ref)
    x = torch.from_numpy(b.copy()).cuda()
    P = TriPlan(A.n, *L.astuple())
    P.solve(x)
    P.check()
    assert np.array_equal(x.cpu().numpy(), ref)


def test_supernodal_waits_time_out_and_plan_recovers(gpu, orc):
    """The supernodal task graph's bounded waits: a solve whose counter
    targets cannot be reached gives up after the limit (about 50 ms here),
    reports GBSYM_ERR_TIMEOUT, and the same plan then solves bit-exactly."""
    from sympiler_gb300._lib import ERR_TIMEOUT, lib
    from sympiler_gb300.plans import SupernodalPlan
    S = mg.nd_supernodal(12, 10, 9, leaf=16, rng=np.random.default_rng(3))
    P = SupernodalPlan(S)
    assert lib().gbsym_sn_selftest_timeout(P._h, 100_000_000, None) == ERR_TIMEOUT
    b = np.random.default_rng(4).standard_normal(S.n)
    for transposed in (False, True, False):
        want = b.copy()
        (orc.blocked_ltsolve if transposed else orc.blocked_lsolve)(S, want)
        x = torch.from_numpy(b.copy()).cuda()
        P.solve(x, transposed=transposed)
        P.check()
        assert np.array_equal(x.cpu().numpy(), want)


def test_zero_pivot_reported_not_trapped(gpu):
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import ERR_PIVOT, GbsymError
    A = mg.convdiff3d(5)
    d = mg.diag_ptr(A)
    Ax = A.x.copy()
    Ax[d[7]] = 0.0  # a zero pivot appears in row 7
    A2 = mg.CSR(A.n, A.p, A.i, Ax)
    l = np.zeros_like(Ax)
    # the elimination itself may or may not hit the zero, depending on the
    # updates; make it certain by zeroing row 0's diagonal
    Ax[d[0]] = 0.0
    with pytest.raises(GbsymError) as e:
        sym_lib.spilu0_csr(A2.n, A2.nnz, A2.p, A2.i, Ax, d, l)
    assert e.value.status == ERR_PIVOT
