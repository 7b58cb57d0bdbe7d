"""MatrixMarket input for the solve path.

The reference reads ``.mtx`` files in its demos (``read_mtx`` of the
aggregation dependency; its own reader is ``parsy::readMatrix``,
sparse_blas/parsy/common/Util.cpp:74-200, which accepts ``coordinate``
``real``/``integer`` files and builds the CSC).  This reader accepts the same
files plus ``pattern`` (values 1), in any entry order, and returns CSC/CSR
arrays in the int32/float64 layout every entry point of this library takes.
"""
from __future__ import annotations

import numpy as np

from .matgen import CSR


class MtxError(ValueError):
    pass


def read_mtx(path: str):
    """Read a coordinate MatrixMarket file.

    Returns ``(nrows, ncols, rows, cols, vals, symmetry)`` with zero-based
    int64 coordinates as stored (symmetric files keep their stored triangle)
    and ``symmetry`` one of ``general``, ``symmetric``, ``skew-symmetric``.
    """
    with open(path, "r") as fh:
        header = fh.readline().strip().lower().split()
        if len(header) != 5 or header[0] != "%%matrixmarket":
            raise MtxError("%s: not a MatrixMarket header" % path)
        _, obj, fmt, arith, sym = header
        if obj != "matrix" or fmt != "coordinate":
            raise MtxError("%s: only coordinate matrices are supported" % path)
        if arith not in ("real", "integer", "pattern"):
            raise MtxError("%s: %s entries are not supported" % (path, arith))
        if sym not in ("general", "symmetric", "skew-symmetric"):
            raise MtxError("%s: %s storage is not supported" % (path, sym))
        line = fh.readline()
        while line and (line.startswith("%") or not line.strip()):
            line = fh.readline()
        dims = line.split()
        if len(dims) != 3:
            raise MtxError("%s: missing size line" % path)
        nr, nc, nnz = (int(v) for v in dims)
        body = np.loadtxt(fh, ndmin=2) if nnz else np.zeros((0, 3))
    if body.shape[0] != nnz:
        raise MtxError("%s: %d entries declared, %d read" % (path, nnz, body.shape[0]))
    rows = body[:, 0].astype(np.int64) - 1
    cols = body[:, 1].astype(np.int64) - 1
    vals = np.ones(nnz) if arith == "pattern" else body[:, 2].astype(np.float64)
    if nnz and (rows.min() < 0 or cols.min() < 0 or rows.max() >= nr or cols.max() >= nc):
        raise MtxError("%s: entry outside the declared size" % path)
    return nr, nc, rows, cols, vals, sym


def _csr_from_coo(n, r, c, v) -> CSR:
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    if len(r) > 1 and np.any((r[1:] == r[:-1]) & (c[1:] == c[:-1])):
        raise MtxError("duplicate entries")
    p = np.zeros(n + 1, dtype=np.int32)
    np.add.at(p, r + 1, 1)
    return CSR(n, np.cumsum(p, dtype=np.int64).astype(np.int32), c.astype(np.int32), v.astype(np.float64))


def lower_triangle(path: str):
    """The lower triangle (with the diagonal) of a square matrix file, as the
    reference demo takes it (``make_half`` of the read matrix): for a
    symmetric file whichever triangle is stored, mirrored into the lower one;
    for a general file the entries on and below the diagonal.  Returns
    ``(L_csr, L_csc)`` -- the CSR of L (diagonal last in each row) and the
    CSC of L (diagonal first in each column) -- as :class:`matgen.CSR`
    tuples (the CSC is the CSR of L^T).  Every row needs its diagonal."""
    nr, nc, r, c, v, sym = read_mtx(path)
    if nr != nc:
        raise MtxError("%s: a triangular solve needs a square matrix" % path)
    if sym == "skew-symmetric":
        raise MtxError("%s: a skew-symmetric matrix has no diagonal to solve with" % path)
    if sym == "symmetric":
        up = r < c
        r, c = np.where(up, c, r), np.where(up, r, c)  # stored triangle mirrored into the lower
    else:
        keep = r >= c
        r, c, v = r[keep], c[keep], v[keep]
    L = _csr_from_coo(nr, r, c, v)
    last = L.p[1:] - 1
    ok = (np.diff(L.p) > 0) & (L.i[np.maximum(last, 0)] == np.arange(nr))
    if not np.all(ok):
        raise MtxError("%s: row %d has no diagonal entry" % (path, int(np.argmin(ok))))
    Lc = _csr_from_coo(nr, c, r, v)  # CSC of L = CSR of L^T
    return L, Lc


def write_mtx(path: str, L: CSR, symmetric: bool = False, comment: str = "") -> None:
    """Write a CSR as a coordinate real file (for fixtures and round trips)."""
    rows = np.repeat(np.arange(L.n), np.diff(L.p))
    with open(path, "w") as fh:
        fh.write("%%%%MatrixMarket matrix coordinate real %s\n" % ("symmetric" if symmetric else "general"))
        if comment:
            fh.write("%% %s\n" % comment)
        fh.write("%d %d %d\n" % (L.n, L.n, len(L.i)))
        for a, b, x in zip(rows, L.i, L.x):
            fh.write("%d %d %.17g\n" % (a + 1, b + 1, x))
