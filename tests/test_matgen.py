"""Synthetic operators have the sizes of the named workloads."""
import numpy as np

from sympiler_gb300 import matgen as mg


def test_c1_sizes():
    A = mg.lap2d(100)
    L = mg.tril(A)
    assert A.n == 10000 and A.nnz == 49600 and L.nnz == 29800
    assert np.all(L.i[L.p[1:] - 1] == np.arange(A.n))  # diagonal last


def test_c2_sizes():
    A = mg.lap3d(64, 1e-2)
    assert A.n == 262144 and A.nnz == 1810432
    U = mg.triu(A)
    assert U.nnz == 1036288
    assert np.all(U.i[U.p[:-1]] == np.arange(A.n))  # diagonal first


def test_c3_sizes_and_nonsymmetry():
    A = mg.convdiff3d(96)
    assert A.n == 884736 and A.nnz == 6137856
    S = mg.convdiff3d(6).scipy()
    assert abs(S - S.T).max() > 0.1
    d = S.diagonal()
    off = np.asarray(abs(S).sum(axis=1)).ravel() - np.abs(d)
    assert np.all(d >= off - 1e-12)  # weakly diagonally dominant


def test_c5_sizes():
    A = mg.aniso_poisson2d(32, 0.01, 1.0, np.random.default_rng(0))
    assert A.n == 1024 and A.nnz == 5 * 1024 - 4 * 32
    S = A.scipy()
    assert abs(S - S.T).max() < 1e-15


def test_level_counts_small():
    assert mg.levels_wavefront(mg.lap2d(20)) == 39
    assert mg.levels_wavefront(mg.lap3d(6)) == 16
