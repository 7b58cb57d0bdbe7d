"""Seeded synthetic matrices for the SpTRSV / Krylov workloads.

The reference benchmarks its executors on SuiteSparse matrices and on random
lower-triangular patterns; neither travels here, so these generators build
the named stencil operators directly, in natural (lexicographic, x fastest)
ordering, as CSR with ascending column indices:

* ``lap2d(nx, ny)``            -- 5-point Laplacian, diagonal 4, off-diagonals -1.
* ``lap3d(g, shift)``          -- 7-point Laplacian on g^3, diagonal 6+shift.
* ``convdiff3d(g, vel, peclet)`` -- 7-point diffusion plus first-order upwind
  convection, scaled by h^2/nu: off-diagonal -1 (downwind side) and
  -1 - c_d (upwind side), diagonal 6 + sum_d |c_d|, with
  c_d = 2 * peclet * vhat_d (cell Peclet number |v| h / (2 nu)).
* ``aniso_poisson2d(g, eps, sigma, rng)`` -- cell-centred finite volumes for
  -d/dx(a du/dx) - eps d/dy(a du/dy), log-normal cell coefficients
  a = exp(sigma N(0,1)), harmonic face means, Dirichlet walls.
* ``random_spd(n, nnz_per_row, rng)`` -- symmetric pattern with N(0,1)
  off-diagonals, made strictly diagonally dominant.
* ``random_lower(n, density, rng)`` -- random lower triangle with a
  dominant diagonal (the reference's random_square_sparse + make_half test
  inputs are not available; this stands in for their shape).

All return ``CSR`` tuples (n, indptr int32, indices int32, data float64).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp


@dataclass
class CSR:
    n: int
    p: np.ndarray  # int32[n+1]
    i: np.ndarray  # int32[nnz]
    x: np.ndarray  # float64[nnz]

    @property
    def nnz(self) -> int:
        return int(self.p[self.n])

    def astuple(self):
        return self.p, self.i, self.x

    def scipy(self):
        return sp.csr_matrix((self.x, self.i, self.p), shape=(self.n, self.n))


def from_scipy(m) -> CSR:
    m = sp.csr_matrix(m)
    m.sum_duplicates()
    m.sort_indices()
    return CSR(m.shape[0], np.ascontiguousarray(m.indptr, dtype=np.int32),
               np.ascontiguousarray(m.indices, dtype=np.int32),
               np.ascontiguousarray(m.data, dtype=np.float64))


def _stencil(shape, center, offs):
    """Assemble a constant-coefficient stencil on a lexicographic grid.

    ``offs`` is a list of (axis, step, value) with step = +-1.
    """
    dims = list(shape)
    n = int(np.prod(dims))
    idx = np.arange(n, dtype=np.int64)
    coords = []
    rem = idx.copy()
    for d in dims:
        coords.append(rem % d)
        rem //= d
    rows = [idx]
    cols = [idx]
    vals = [np.full(n, center, dtype=np.float64)]
    stride = 1
    strides = []
    for d in dims:
        strides.append(stride)
        stride *= d
    for axis, step, value in offs:
        c = coords[axis]
        ok = (c + step >= 0) & (c + step < dims[axis])
        r = idx[ok]
        rows.append(r)
        cols.append(r + step * strides[axis])
        vals.append(np.full(r.size, value, dtype=np.float64))
    m = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    return from_scipy(m)


def lap2d(nx: int, ny: int | None = None) -> CSR:
    ny = nx if ny is None else ny
    return _stencil((nx, ny), 4.0, [(0, -1, -1.0), (0, 1, -1.0), (1, -1, -1.0), (1, 1, -1.0)])


def lap3d(g: int, shift: float = 0.0) -> CSR:
    offs = [(a, s, -1.0) for a in range(3) for s in (-1, 1)]
    return _stencil((g, g, g), 6.0 + shift, offs)


def convdiff3d(g: int, vel=(1.0, 0.5, 0.25), peclet: float = 0.5) -> CSR:
    v = np.asarray(vel, dtype=np.float64)
    vhat = v / np.linalg.norm(v)
    c = 2.0 * peclet * vhat
    offs = []
    for a in range(3):
        up = -1 if c[a] >= 0 else 1          # upwind neighbour
        offs.append((a, up, -1.0 - abs(c[a])))
        offs.append((a, -up, -1.0))
    return _stencil((g, g, g), 6.0 + float(np.abs(c).sum()), offs)


def aniso_poisson2d(g: int, eps: float = 0.01, sigma: float = 1.0,
                    rng: np.random.Generator | None = None) -> CSR:
    rng = np.random.default_rng(0) if rng is None else rng
    a = np.exp(sigma * rng.standard_normal((g, g)))  # a[y, x]
    n = g * g
    idx = np.arange(n).reshape(g, g)
    rows, cols, vals = [], [], []
    diag = np.zeros((g, g))

    def face(a1, a2):
        return 2.0 / (1.0 / a1 + 1.0 / a2)

    # x faces
    fx = face(a[:, :-1], a[:, 1:])
    rows += [idx[:, :-1].ravel(), idx[:, 1:].ravel()]
    cols += [idx[:, 1:].ravel(), idx[:, :-1].ravel()]
    vals += [-fx.ravel(), -fx.ravel()]
    diag[:, :-1] += fx
    diag[:, 1:] += fx
    diag[:, 0] += 2 * a[:, 0]
    diag[:, -1] += 2 * a[:, -1]
    # y faces (scaled by eps)
    fy = eps * face(a[:-1, :], a[1:, :])
    rows += [idx[:-1, :].ravel(), idx[1:, :].ravel()]
    cols += [idx[1:, :].ravel(), idx[:-1, :].ravel()]
    vals += [-fy.ravel(), -fy.ravel()]
    diag[:-1, :] += fy
    diag[1:, :] += fy
    diag[0, :] += 2 * eps * a[0, :]
    diag[-1, :] += 2 * eps * a[-1, :]
    rows.append(idx.ravel())
    cols.append(idx.ravel())
    vals.append(diag.ravel())
    m = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    return from_scipy(m)


def random_spd(n: int, nnz_per_row: int = 8, rng: np.random.Generator | None = None) -> CSR:
    rng = np.random.default_rng(0) if rng is None else rng
    k = max(1, (nnz_per_row - 1) // 2)
    r = np.repeat(np.arange(n), k)
    c = rng.integers(0, n, size=r.size)
    keep = r != c
    r, c = r[keep], c[keep]
    v = rng.standard_normal(r.size)
    m = sp.coo_matrix((np.concatenate([v, v]), (np.concatenate([r, c]), np.concatenate([c, r]))),
                      shape=(n, n)).tocsr()
    m.sum_duplicates()
    rowsum = np.asarray(abs(m).sum(axis=1)).ravel()
    m = m + sp.diags(rowsum + 1.0)
    return from_scipy(m)


def random_lower(n: int, density: float, rng: np.random.Generator | None = None,
                 unit_scale: bool = False) -> CSR:
    """Random lower-triangular CSR, diagonal last in every row."""
    rng = np.random.default_rng(0) if rng is None else rng
    m = sp.random(n, n, density=density, format="coo", random_state=rng,
                  data_rvs=lambda s: rng.uniform(-1.0, 1.0, s))
    low = m.row > m.col
    r, c, v = m.row[low], m.col[low], m.data[low]
    if unit_scale:
        v = np.ones_like(v)
    d = np.full(n, 2.0 if not unit_scale else 1.0) + (0 if unit_scale else rng.uniform(0, 1, n))
    mm = sp.coo_matrix((np.concatenate([v, d]), (np.concatenate([r, np.arange(n)]),
                                                  np.concatenate([c, np.arange(n)]))), shape=(n, n))
    return from_scipy(mm)


# ---- triangle extraction / transposition ---------------------------------

def tril(a: CSR, k: int = 0) -> CSR:
    return from_scipy(sp.tril(a.scipy(), k=k))


def triu(a: CSR, k: int = 0) -> CSR:
    return from_scipy(sp.triu(a.scipy(), k=k))


def transpose(a: CSR) -> CSR:
    """CSR of A^T (equivalently: the CSC arrays of A)."""
    return from_scipy(a.scipy().T.tocsr())


def diag_ptr(a: CSR) -> np.ndarray:
    """Index of the diagonal entry of each row (the ILU0 ``A_diag``/``ua``)."""
    out = np.empty(a.n, dtype=np.int32)
    for_rows = np.repeat(np.arange(a.n), np.diff(a.p))
    hit = np.nonzero(a.i == for_rows)[0]
    out[for_rows[hit]] = hit
    return out


def levels_wavefront(a: CSR) -> int:
    """Number of wavefront levels of tril(a) (for sizing only)."""
    L = tril(a)
    lev = np.zeros(a.n, dtype=np.int64)
    p, i = L.p, L.i
    for r in range(a.n):
        m = -1
        for j in range(p[r], p[r + 1] - 1):
            m = max(m, lev[i[j]])
        lev[r] = m + 1
    return int(lev.max() + 1) if a.n else 0


# ---- batched workload ----------------------------------------------------

def _lap2d_upper_shifted(nx: int, ny: int, shift: float):
    """Upper CSR (diagonal first) of the 5-point Laplacian + shift*I."""
    n = nx * ny
    idx = np.arange(n)
    x = idx % nx
    y = idx // nx
    right = x < nx - 1
    up = y < ny - 1
    cnt = 1 + right.astype(np.int64) + up.astype(np.int64)
    p = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(cnt, out=p[1:])
    nnz = int(p[-1])
    ci = np.empty(nnz, dtype=np.int32)
    cv = np.empty(nnz, dtype=np.float64)
    ci[p[:-1]] = idx
    cv[p[:-1]] = 4.0 + shift
    pos = p[:-1] + 1
    ci[pos[right]] = idx[right] + 1
    cv[pos[right]] = -1.0
    pos2 = pos + right
    ci[pos2[up]] = idx[up] + nx
    cv[pos2[up]] = -1.0
    return n, p.astype(np.int32), ci, cv


def batch_systems_upper(nsys: int = 512, rng: np.random.Generator | None = None,
                        lap_frac: float = 0.8, grid=(30, 300), rand_n=(900, 90000)):
    """The batched-solve workload: nsys independent SPD systems, as upper CSRs
    (diagonal first; the CSC of their lower triangles).  A fraction lap_frac
    are 2D 5-point Laplacians on nx, ny ~ U{grid} with a diagonal shift
    ~ U[1e-3, 1]; the rest are random symmetric matrices with about 8
    entries per row and N(0,1) off-diagonals, made strictly diagonally
    dominant, with n ~ U{rand_n}.  Returns a list of (n, p, i, x)."""
    rng = np.random.default_rng(0) if rng is None else rng
    out = []
    for q in range(nsys):
        if rng.uniform() < lap_frac:
            nx, ny = (int(v) for v in rng.integers(grid[0], grid[1] + 1, size=2))
            out.append(_lap2d_upper_shifted(nx, ny, float(rng.uniform(1e-3, 1.0))))
        else:
            n = int(rng.integers(rand_n[0], rand_n[1] + 1))
            U = triu(random_spd(n, 8, rng))
            out.append((U.n, U.p, U.i, U.x))
    return out


def block_diagonal(systems):
    """Concatenate square CSRs into one block-diagonal CSR; returns
    (N, p, i, x, row_offsets)."""
    ns = [s[0] for s in systems]
    off = np.zeros(len(systems) + 1, dtype=np.int64)
    np.cumsum(ns, out=off[1:])
    nnzs = [int(s[1][-1]) for s in systems]
    eoff = np.zeros(len(systems) + 1, dtype=np.int64)
    np.cumsum(nnzs, out=eoff[1:])
    N, E = int(off[-1]), int(eoff[-1])
    if N >= 2 ** 31 or E >= 2 ** 31:
        raise ValueError("batch too large for int32 indices")
    p = np.empty(N + 1, dtype=np.int32)
    ci = np.empty(E, dtype=np.int32)
    cx = np.empty(E, dtype=np.float64)
    for q, (n, sp_, si, sx) in enumerate(systems):
        p[off[q]:off[q + 1]] = sp_[:-1] + eoff[q]
        ci[eoff[q]:eoff[q + 1]] = si + off[q]
        cx[eoff[q]:eoff[q + 1]] = sx
    p[N] = E
    return N, p, ci, cx, off


# ---- supernodal (blocked CSC) factors ------------------------------------

@dataclass
class Supernodal:
    """A lower triangle in the blocked CSC layout of the reference's
    supernodal solves (parsy::blockedLsolve and relatives): supernode s owns
    columns sup2col[s] .. sup2col[s+1]-1 and the rows Li[Li_ptr[c0] ..
    Li_ptr[c1]) (its own columns first); its values are a column-major
    block of nSupR rows starting at Lx[Lp[c0]]."""
    n: int
    nsup: int
    Lp: np.ndarray       # uint64[n+1]  (size_t)
    Li: np.ndarray       # int32
    Lx: np.ndarray       # float64
    Li_ptr: np.ndarray   # uint64[n+1]  (size_t)
    col2sup: np.ndarray  # int32[n]
    sup2col: np.ndarray  # int32[nsup+1]

    def dense(self) -> np.ndarray:
        """The lower triangle as a dense array (unused storage ignored)."""
        L = np.zeros((self.n, self.n))
        for s in range(self.nsup):
            c0, c1 = int(self.sup2col[s]), int(self.sup2col[s + 1])
            r0, r1 = int(self.Li_ptr[c0]), int(self.Li_ptr[c1])
            rows = self.Li[r0:r1]
            nr = r1 - r0
            blk = self.Lx[int(self.Lp[c0]):int(self.Lp[c0]) + nr * (c1 - c0)].reshape(c1 - c0, nr)
            for j in range(c1 - c0):
                for k in range(j, nr):
                    L[rows[k], c0 + j] = blk[j, k]
        return L


def random_supernodal(nsup: int, max_width: int = 16, max_off: int = 40,
                      rng: np.random.Generator | None = None, tree: bool = True) -> Supernodal:
    """Seeded random supernodal lower triangle.  With ``tree`` the off-block
    rows of a supernode lie in the columns of its ancestors in a random
    supernode tree (the structure a Cholesky factor has); otherwise in any
    later columns.  Diagonal blocks dominate so solutions stay bounded; the
    unused upper halves of the diagonal blocks hold NaN, so a solve that
    read them would show it."""
    rng = np.random.default_rng(0) if rng is None else rng
    widths = rng.integers(1, max_width + 1, nsup)
    sup2col = np.concatenate([[0], np.cumsum(widths)]).astype(np.int32)
    n = int(sup2col[-1])
    parent = np.full(nsup, -1)
    for s in range(nsup - 1):
        parent[s] = int(rng.integers(s + 1, min(nsup, s + 1 + max(1, nsup // 8)) + 1)) if tree else -1
        if parent[s] >= nsup:
            parent[s] = -1
    Lp = np.zeros(n + 1, dtype=np.uint64)
    Li_ptr = np.zeros(n + 1, dtype=np.uint64)
    col2sup = np.zeros(n, dtype=np.int32)
    Li_parts, Lx_parts = [], []
    rbase = vbase = 0
    for s in range(nsup):
        c0, c1 = int(sup2col[s]), int(sup2col[s + 1])
        w = c1 - c0
        if tree:
            cand, a = [], parent[s]
            while a >= 0:
                cand.extend(range(int(sup2col[a]), int(sup2col[a + 1])))
                a = parent[a]
            cand = np.asarray(cand, dtype=np.int64)
        else:
            cand = np.arange(c1, n)
        m = min(len(cand), int(rng.integers(0, max_off + 1)))
        off = np.sort(rng.choice(cand, m, replace=False)) if m else np.zeros(0, dtype=np.int64)
        rows = np.concatenate([np.arange(c0, c1), off]).astype(np.int32)
        nr = len(rows)
        blk = rng.uniform(-1.0, 1.0, (w, nr)) / (2.0 * (w + m + 1))
        for j in range(w):
            blk[j, :j] = np.nan
            blk[j, j] = 1.0 + rng.uniform(0.0, 1.0)
        col2sup[c0:c1] = s
        Li_ptr[c0:c1] = rbase
        for j in range(w):
            Lp[c0 + j] = vbase + j * nr
        Li_parts.append(rows)
        Lx_parts.append(blk.reshape(-1))
        rbase += nr
        vbase += nr * w
    Li_ptr[n] = rbase
    Lp[n] = vbase
    return Supernodal(n, nsup, Lp, np.concatenate(Li_parts), np.concatenate(Lx_parts), Li_ptr,
                      col2sup, sup2col)


def nd_supernodal(nx: int, ny: int, nz: int = 1, leaf: int = 64,
                  rng: np.random.Generator | None = None) -> Supernodal:
    """Seeded supernodal lower triangle with the structure of the Cholesky
    factor of the 7-point (5-point when nz = 1) Laplacian on an nx x ny x nz
    grid in geometric nested-dissection order.

    Boxes are bisected across their longest side until they hold at most
    ``leaf`` nodes; each separator plane and each leaf box is one supernode,
    numbered after both halves (post-order).  A supernode's off-block rows
    are the grid neighbours of its box outside the box -- nodes of ancestor
    separators -- which is exactly the union of its columns' structures in
    the filled graph, so blocks are dense as a supernodal Cholesky stores
    them.  Values are random: off-diagonals of row r uniform in
    (-1, 1) / (entries of row r), diagonals in [2, 3), so solutions stay
    bounded; the unused upper halves of the diagonal blocks hold NaN."""
    rng = np.random.default_rng(0) if rng is None else rng
    dims = (nx, ny, nz)
    sups = []  # (own box, enclosing box), post-order

    def rec(box):
        size = [b - a for a, b in box]
        if size[0] * size[1] * size[2] <= leaf:
            sups.append((box, box))
            return
        d = int(np.argmax(size))
        m = (box[d][0] + box[d][1]) // 2
        lo, hi, sep = list(box), list(box), list(box)
        lo[d], hi[d], sep[d] = (box[d][0], m), (m + 1, box[d][1]), (m, m + 1)
        for half in (lo, hi):
            if half[d][1] > half[d][0]:
                rec(tuple(half))
        sups.append((tuple(sep), box))

    rec(((0, nx), (0, ny), (0, nz)))
    n = nx * ny * nz
    new = np.empty(n, dtype=np.int64)  # grid node (x + nx*(y + ny*z)) -> column

    def nodes(box):
        (x0, x1), (y0, y1), (z0, z1) = box
        z, y, x = np.meshgrid(np.arange(z0, z1), np.arange(y0, y1), np.arange(x0, x1), indexing="ij")
        return (x + nx * (y + ny * z)).reshape(-1)

    sup2col = np.zeros(len(sups) + 1, dtype=np.int32)
    c = 0
    for s, (own, _) in enumerate(sups):
        g = nodes(own)
        new[g] = np.arange(c, c + len(g))
        c += len(g)
        sup2col[s + 1] = c
    rows_of = []
    for own, box in sups:
        faces = []
        for d in range(3):
            for side, at in ((0, box[d][0] - 1), (1, box[d][1])):
                if 0 <= at < dims[d]:
                    f = list(box)
                    f[d] = (at, at + 1)
                    faces.append(new[nodes(tuple(f))])
        c0 = int(new[nodes(own)].min())
        w = int(np.prod([b - a for a, b in own]))
        off = np.sort(np.concatenate(faces)) if faces else np.zeros(0, dtype=np.int64)
        rows_of.append(np.concatenate([np.arange(c0, c0 + w), off]).astype(np.int32))
    nsup = len(sups)
    # entries per row, for the off-diagonal scale
    cnt = np.zeros(n, dtype=np.float64)
    for s in range(nsup):
        w = int(sup2col[s + 1] - sup2col[s])
        r = rows_of[s]
        cnt[r[w:]] += w
        cnt[r[:w]] += np.arange(w)
    cnt = np.maximum(cnt, 1.0)
    Lp = np.zeros(n + 1, dtype=np.uint64)
    Li_ptr = np.zeros(n + 1, dtype=np.uint64)
    col2sup = np.zeros(n, dtype=np.int32)
    Lx_parts = []
    rbase = vbase = 0
    for s in range(nsup):
        c0, c1 = int(sup2col[s]), int(sup2col[s + 1])
        w = c1 - c0
        r = rows_of[s]
        nr = len(r)
        blk = rng.uniform(-1.0, 1.0, (w, nr)) / cnt[r][None, :]
        jc, kr = np.tril_indices(w, -1)
        blk[jc, kr] = np.nan  # column j's rows k < j: the unused upper half
        blk[np.arange(w), np.arange(w)] = 2.0 + rng.uniform(0.0, 1.0, w)
        col2sup[c0:c1] = s
        Li_ptr[c0:c1] = rbase
        Lp[c0:c1] = vbase + np.arange(w, dtype=np.uint64) * np.uint64(nr)
        Lx_parts.append(blk.reshape(-1))
        rbase += nr
        vbase += nr * w
    Li_ptr[n] = rbase
    Lp[n] = vbase
    return Supernodal(n, nsup, Lp, np.concatenate(rows_of), np.concatenate(Lx_parts), Li_ptr,
                      col2sup, sup2col)
