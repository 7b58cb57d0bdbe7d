"""The correctly rounded division at the edges of its fast path.

The executors divide with Markstein's method (a reciprocal, a remainder
FMA and a correction FMA) when both operands are well inside the normal
range, and fall back to IEEE division otherwise: a dividend of biased
exponent outside [63, 2043], a divisor outside [3, 2043], exponents more
than 1000 apart, zeros, subnormals.  These tests put dividends and
divisors on every side of those guards -- exponents 0 (subnormal) to 2046,
the boundaries 62/63, 2/3, 2043/2044 and exponent differences of
999..1002, signed zeros -- through every level-packed executor and the
supernodal task graph, bit for bit against the oracle (IEEE division on
the CPU).
"""
import numpy as np
import pytest
import torch

from sympiler_gb300 import matgen as mg

pytestmark = pytest.mark.gpu


def _with_exponent(e, rng):
    """A random double with biased exponent e (0: a nonzero subnormal) and a
    random sign."""
    mant = int(rng.integers(1, 1 << 52))
    bits = (int(e) << 52) | mant
    if rng.uniform() < 0.5:
        bits |= 1 << 63
    return np.array([bits], dtype=np.uint64).view(np.float64)[0]


def _pairs(m, rng):
    """m (dividend, divisor) pairs around the guard boundaries, plus random
    exponents over the whole range and signed-zero dividends."""
    edges_a = [0, 1, 2, 60, 61, 62, 63, 64, 65, 1023, 2041, 2042, 2043, 2044, 2045, 2046]
    edges_b = [0, 1, 2, 3, 4, 5, 1023, 2041, 2042, 2043, 2044, 2045, 2046]
    out = []
    for ea in edges_a:
        for eb in edges_b:
            out.append((ea, eb))
    for d in (998, 999, 1000, 1001, 1002):
        for base in (1, 3, 40, 500, 1000):
            if base + d <= 2046:
                out.append((base + d, base))
                out.append((base, base + d))
    pairs = []
    while len(pairs) < m:
        for ea, eb in out:
            pairs.append((_with_exponent(ea, rng), _with_exponent(eb, rng)))
        for _ in range(len(out)):
            pairs.append((_with_exponent(int(rng.integers(0, 2047)), rng),
                          _with_exponent(int(rng.integers(0, 2047)), rng)))
        pairs.append((0.0, _with_exponent(int(rng.integers(0, 2047)), rng)))
        pairs.append((-0.0, _with_exponent(int(rng.integers(0, 2047)), rng)))
    a = np.array([p[0] for p in pairs[:m]])
    b = np.array([p[1] for p in pairs[:m]])
    return a, b


def _edge_triangle(levels, bench_rows, edge_rows, rng):
    """Lower CSR (diagonal last) in groups per level: benign rows B_l (each
    depends on B_{l-1} with coefficient 0.5, diagonal 2) and edge rows E_l,
    each depending on a B_{l-1} row through a stored zero, so that its
    accumulator reaches the division exactly as its right-hand side gives
    it; E_l rows have the edge divisors.  No row reads an E row, so an
    overflowed quotient stays where it is."""
    a, d = _pairs(levels * edge_rows, rng)
    p, ci, cv = [0], [], []
    b = []
    prev_b = None
    q = 0
    for lvl in range(levels):
        base = len(p) - 1
        cur_b = list(range(base, base + bench_rows))
        for r, row in enumerate(cur_b):
            if prev_b is not None:
                ci.append(prev_b[r])
                cv.append(0.5)
            ci.append(row)
            cv.append(2.0)
            p.append(len(ci))
            b.append(1.0 + r * 1e-3)
        for r in range(edge_rows):
            row = len(p) - 1
            if prev_b is not None:
                ci.append(prev_b[r % bench_rows])
                cv.append(0.0)
            ci.append(row)
            cv.append(d[q])
            p.append(len(ci))
            b.append(a[q])
            q += 1
        prev_b = cur_b
    n = len(p) - 1
    L = mg.CSR(n, np.array(p, dtype=np.int32), np.array(ci, dtype=np.int32), np.array(cv))
    return L, np.array(b)


@pytest.mark.parametrize("exec_mode", [1, 2, 3, 4, 5, 6])
def test_division_edges_every_executor(gpu, orc, exec_mode):
    from sympiler_gb300.plans import TriPlan
    rng = np.random.default_rng(2024)
    L, b = _edge_triangle(6, 128, 4096, rng)
    with np.errstate(all="ignore"):
        assert np.isfinite(b).all() and (L.x != 0).sum() == L.n + 5 * 128
    want = b.copy()
    orc.sptrsv_csr(L.n, *L.astuple(), want)
    assert not np.isnan(want).any()
    P = TriPlan(L.n, *L.astuple())
    assert P.info().levels == 6
    P.set_exec(exec_mode)
    x = torch.from_numpy(b.copy()).cuda()
    P.solve(x)
    P.check()
    got = x.cpu().numpy()
    bad = np.flatnonzero(got.view(np.uint64) != want.view(np.uint64))
    assert bad.size == 0, [(int(i), b[i], got[i], want[i]) for i in bad[:5]]


@pytest.mark.parametrize("exec_mode", [1, 2, 4, 5])
def test_division_edges_multi_rhs(gpu, orc, exec_mode):
    """Four right-hand sides: each row's divisor meets four dividends."""
    from sympiler_gb300.plans import TriPlan
    rng = np.random.default_rng(77)
    L, b0 = _edge_triangle(5, 64, 2048, rng)
    k = 4
    B = np.empty((L.n, k))
    B[:, 0] = b0
    for c in range(1, k):
        a, _ = _pairs(L.n, rng)
        B[:, c] = np.where(L.x[L.p[1:] - 1] == 2.0, b0, a)  # benign rows keep benign values
    want = np.ascontiguousarray(B.T.copy())
    orc.sptrsv_csr_mrhs(L.n, *L.astuple(), want, k, 1)
    want = want.T
    P = TriPlan(L.n, *L.astuple())
    P.set_exec(exec_mode)
    X = torch.from_numpy(B.copy()).cuda()
    P.solve(X)
    P.check()
    assert np.array_equal(X.cpu().numpy().view(np.uint64), want.view(np.uint64))


def test_division_edges_supernodal(gpu, orc):
    """The supernodal tiles' division (its own exponent window and IEEE
    fallback), forward and transposed: edge divisors on every diagonal,
    edge dividends as the right-hand side, every off-diagonal value a
    stored zero so each accumulator reaches its division unchanged.  Pairs
    whose quotient would overflow are left out, since a later product
    would turn an infinity into a NaN."""
    from sympiler_gb300.plans import SupernodalPlan
    rng = np.random.default_rng(5)
    S = mg.random_supernodal(300, max_width=40, max_off=30, rng=rng)
    a, d = _pairs(4 * S.n, rng)
    with np.errstate(all="ignore"):
        keep = np.isfinite(a / d)
    a, d = a[keep][: S.n], d[keep][: S.n]
    assert len(a) == S.n
    Lx = np.where(np.isnan(S.Lx), np.nan, 0.0)
    for s in range(S.nsup):
        c0, c1 = int(S.sup2col[s]), int(S.sup2col[s + 1])
        nr = int(S.Li_ptr[c1] - S.Li_ptr[c0])
        for j in range(c1 - c0):
            Lx[int(S.Lp[c0]) + j * nr + j] = d[c0 + j]
    S.Lx = Lx
    P = SupernodalPlan(S)
    for transposed in (False, True):
        want = a.copy()
        (orc.blocked_ltsolve if transposed else orc.blocked_lsolve)(S, want)
        assert not np.isnan(want).any()
        x = torch.from_numpy(a.copy()).cuda()
        P.solve(x, transposed=transposed)
        P.check()
        assert np.array_equal(x.cpu().numpy().view(np.uint64), want.view(np.uint64)), transposed
