"""The one-block executor (one launch, one block) bit for bit against the
oracle, in all three of its forms:

- barrier-free with values published in shared memory (rows of up to four
  entries, solution and right-hand side fit in shared memory): the small
  cases here;
- level by level with three levels of row data in flight (rows of up to
  four entries, larger systems): the 30^3 and 200^2 cases;
- level by level with one level in flight (wider rows): the random case.

It also covers every slab width each form compiles, one to five levels in
both level-by-level and barrier-free forms, levels wider than the block, x
in shared memory and in global memory, and FP32 and fused arithmetic
against the sync-free sweep."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def _banded_lower(n, offsets, rng):
    """Lower triangle with off-diagonals at the given distances and the
    diagonal last in each row."""
    rows, cols = [], []
    for d in offsets:
        r = np.arange(d, n)
        rows.append(r)
        cols.append(r - d)
    rows.append(np.arange(n))
    cols.append(np.arange(n))
    r, c = np.concatenate(rows), np.concatenate(cols)
    v = np.where(r == c, 4.0 + rng.uniform(0, 1, r.size), rng.uniform(-1, 1, r.size))
    return mg.from_scipy(sp.coo_matrix((v, (r, c)), shape=(n, n)))


def _chain(n, depth, rng):
    """n rows in `depth` levels: row i depends on row i - n/depth."""
    step = max(1, n // depth)
    return _banded_lower(n, [step], rng)


def _cases():
    rng = np.random.default_rng(3)
    yield "lap2d_100_k2", mg.tril(mg.lap2d(100))
    yield "lap3d_20_k3", mg.tril(mg.lap3d(20, 1e-2))
    yield "band_k4", _banded_lower(3000, [1, 2, 40, 41], rng)
    yield "random_wide", mg.random_lower(3000, 0.004, np.random.default_rng(8))
    # one to five levels, small (barrier-free form) and, in FP64, too large
    # for shared memory (the pipelined form's partial rounds)
    for n in (600, 20000):
        for depth in (1, 2, 3, 4, 5):
            yield "chain_%d_%d_levels" % (n, depth), (mg.from_scipy(sp.eye(n, format="csr") * 2.0) if depth == 1
                                                      else _chain(n, depth, rng))
    yield "lap3d_30_wide_levels", mg.tril(mg.lap3d(30, 1e-2))
    yield "lap2d_200_x_global", mg.tril(mg.lap2d(200))


@pytest.mark.parametrize("name,L", list(_cases()), ids=[c[0] for c in _cases()])
def test_oneblock_exact(gpu, orc, name, L):
    from sympiler_gb300._lib import ARITH_FUSED, EXEC_ONEBLOCK, EXEC_SYNCFREE
    from sympiler_gb300.plans import TriPlan
    b = np.random.default_rng(L.n).uniform(-1, 1, L.n)
    ref = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), ref)
    P = TriPlan(L.n, *L.astuple())
    P.set_exec(EXEC_ONEBLOCK)
    x = torch.from_numpy(b.copy()).cuda()
    P.solve(x)
    P.check()
    assert np.array_equal(x.cpu().numpy(), ref)
    y = torch.empty_like(x)
    P.solve_into(torch.from_numpy(b).cuda(), y)
    P.check()
    assert np.array_equal(y.cpu().numpy(), ref)
    # FP32 against the FP32 oracle
    P32 = TriPlan(L.n, *L.astuple(), dtype="f32")
    P32.set_exec(EXEC_ONEBLOCK)
    x32 = torch.from_numpy(b.astype(np.float32)).cuda()
    P32.solve(x32)
    P32.check()
    r32 = b.astype(np.float32)
    orc.sptrsv_csr_f32(L.n, L.p, L.i, L.x.astype(np.float32), r32)
    assert np.array_equal(x32.cpu().numpy(), r32)
    # fused arithmetic: the same bits as the sync-free sweep's
    P.set_arith(ARITH_FUSED)
    Q = TriPlan(L.n, *L.astuple())
    Q.set_exec(EXEC_SYNCFREE)
    Q.set_arith(ARITH_FUSED)
    xf, xq = torch.from_numpy(b.copy()).cuda(), torch.from_numpy(b.copy()).cuda()
    P.solve(xf)
    Q.solve(xq)
    P.check()
    Q.check()
    assert torch.equal(xf, xq)
