"""The forward solve that allocates nothing (gbsym_sptrsv_csr_noalloc).

It serves callers that cannot allocate device memory -- an application
whose own pool allocator owns the device memory, or a loop that cannot take
cudaMalloc's device-wide synchronisation -- so its scratch is a static
array inside the library.  Checked through the C ABI against the existing
forward solve (gbsym_sptrsv_csr), on two calls in a row.  Collected last so
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


@pytest.mark.parametrize("case", ["lap2d_100", "ic0_lap3d_32"])
def test_noalloc_matches_existing_entry_point_twice(gpu, orc, case):
    from sympiler_gb300 import sym_lib
    from sympiler_gb300._lib import OK, lib
    if case == "lap2d_100":
        L = mg.tril(mg.lap2d(100))
    else:
        U = mg.triu(mg.lap3d(32, 1e-2))
        f, ok = orc.spic0_csr(U.n, U.p, U.i, U.x)
        L = mg.transpose(mg.CSR(U.n, U.p, U.i, f))
    rng = np.random.default_rng(17)
    dLp, dLi, dLx = (torch.from_numpy(a.copy()).cuda() for a in L.astuple())
    for call in range(2):
        b = rng.uniform(-1, 1, L.n)
        want = b.copy()
        sym_lib.sptrsv_csr(L.n, *L.astuple(), want)  # the existing entry point
        x = torch.from_numpy(b.copy()).cuda()
        st = lib().gbsym_sptrsv_csr_noalloc(L.n, _ptr(dLp), _ptr(dLi), _ptr(dLx), _ptr(x), None)
        assert st == OK, (call, st)
        assert np.array_equal(x.cpu().numpy(), want), call


def test_noalloc_rejects_sizes_beyond_its_array(gpu):
    from sympiler_gb300._lib import ERR_SIZE, lib
    n = (1 << 19) + 1
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    di = torch.zeros(4, dtype=torch.int32, device="cuda")
    st = lib().gbsym_sptrsv_csr_noalloc(n, _ptr(di), _ptr(di), _ptr(dummy), _ptr(dummy), None)
    assert st == ERR_SIZE
    assert torch.count_nonzero(dummy).item() == 0
