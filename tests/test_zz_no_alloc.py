"""The forward solve that allocates nothing (gbsym_sptrsv_csr_noalloc).

It serves callers that cannot allocate device memory -- an application
whose own pool allocator owns the device memory, or a loop that cannot take
cudaMalloc's device-wide synchronisation -- so its scratch is a static
array inside the library.  Checked through the C ABI against the oracle's
sptrsv_csr and against the library's existing forward solve
(gbsym_sptrsv_csr), bit for bit, on two calls in a row.  Collected last so
a run that stops at the first failure has run every other test; it also
passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _lower(orc, case):
    if case == "lap2d_100":
        return mg.tril(mg.lap2d(100))
    U = mg.triu(mg.lap3d(32, 1e-2))
    f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
    assert ok
    return mg.transpose(mg.CSR(U.n, U.p, U.i, f))


@pytest.mark.parametrize("case", ["lap2d_100", "ic0_lap3d_32"])
def test_noalloc_matches_oracle_and_existing_entry_point_twice(gpu, orc, case):
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import OK, lib
    L = _lower(orc, case)
    rng = np.random.default_rng(17)
    dLp, dLi, dLx = (torch.from_numpy(a.copy()).cuda() for a in L.astuple())
    for call in range(2):
        b = rng.uniform(-1, 1, L.n)
        want = b.copy()
        orc.sptrsv_csr(L.n, *L.astuple(), want)  # the oracle
        existing = b.copy()
        sym_lib.sptrsv_csr(L.n, *L.astuple(), existing)  # the existing entry point
        x = torch.from_numpy(b.copy()).cuda()
        st = lib().gbsym_sptrsv_csr_noalloc(L.n, _ptr(dLp), _ptr(dLi), _ptr(dLx), _ptr(x), None)
        assert st == OK, (call, st)
        got = x.cpu().numpy()
        assert np.array_equal(got, want), call
        assert np.array_equal(got, existing), call


def test_noalloc_reports_a_malformed_row_and_recovers(gpu, orc):
    """A column index at or above its row (still inside the arrays) is not a
    dependency of a lower triangle: the call returns GBSYM_ERR_BAD_MATRIX
    (the kernel checks the column before loading), and the next call on a
    valid matrix solves exactly."""
    from sympiler_gb300._lib import ERR_BAD_MATRIX, OK, lib
    L = mg.tril(mg.lap2d(40))
    bad_i = L.i.copy()
    row = 500
    bad_i[L.p[row]] = row + 3  # the row's first off-diagonal now points ahead
    b = np.random.default_rng(3).uniform(-1, 1, L.n)
    dLp, dLx = torch.from_numpy(L.p.copy()).cuda(), torch.from_numpy(L.x.copy()).cuda()
    x = torch.from_numpy(b.copy()).cuda()
    st = lib().gbsym_sptrsv_csr_noalloc(L.n, _ptr(dLp), _ptr(torch.from_numpy(bad_i).cuda()), _ptr(dLx),
                                        _ptr(x), None)
    assert st == ERR_BAD_MATRIX
    want = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), want)
    x = torch.from_numpy(b.copy()).cuda()
    st = lib().gbsym_sptrsv_csr_noalloc(L.n, _ptr(dLp), _ptr(torch.from_numpy(L.i.copy()).cuda()), _ptr(dLx),
                                        _ptr(x), None)
    assert st == OK
    assert np.array_equal(x.cpu().numpy(), want)


def test_noalloc_rejects_sizes_beyond_its_array(gpu):
    from sympiler_gb300._lib import ERR_SIZE, lib
    n = (1 << 19) + 1
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    di = torch.zeros(4, dtype=torch.int32, device="cuda")
    st = lib().gbsym_sptrsv_csr_noalloc(n, _ptr(di), _ptr(di), _ptr(dummy), _ptr(dummy), None)
    assert st == ERR_SIZE
    assert torch.count_nonzero(dummy).item() == 0
