"""The reference's ``sym_lib`` entry points, running on the GPU.

Same names, argument order and in-place semantics as
``include/sympiler/sparse_blas_lib.h`` (and ``parsy`` for the CSC solves and
``lus_cr``), over numpy arrays in host memory: int32 index arrays, float64
values; ``x`` is overwritten with the solution.  Each call goes through the
C ABI of ``libgbsym.so``; a non-OK status raises :class:`GbsymError` (the C
drop-ins themselves never abort and record the status instead).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import GbsymError, lib

_I32 = np.int32
_F64 = np.float64


def _arr(a, dtype, name, writable=False):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        if writable:
            raise TypeError("%s must be a C-contiguous %s numpy array (updated in place)"
                            % (name, np.dtype(dtype).name))
        a = np.ascontiguousarray(a, dtype=dtype)
    return a


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _raise_last(where):
    st = lib().gbsym_last_error()
    if st != 0:
        raise GbsymError(st, where)


# ---- SpTRSV, CSR ----------------------------------------------------------

def sptrsv_csr(n, Lp, Li, Lx, x):
    """sparse_blas/sptrsv.cpp:17-25 -- forward solve, diagonal last in a row."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csr(n, _p(Lp), _p(Li), _p(Lx), _p(x))
    _raise_last("sptrsv_csr")


def sptrsv_csr_ilu(n, Lp, Li, Lx, diags, x):
    """sparse_blas/sptrsv.cpp:28-37 -- unit-lower part of an ILU0 factor."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    diags = _arr(diags, _I32, "diags")
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csr_ilu(n, _p(Lp), _p(Li), _p(Lx), _p(diags), _p(x))
    _raise_last("sptrsv_csr_ilu")


def sptrsv_csr_ilu_lbc(n, Lp, Li, Lx, diags, x, level_no, level_ptr, par_ptr, partition):
    """sparse_blas/sptrsv.cpp:109-127 (divides by the diagonal)."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    diags = _arr(diags, _I32, "diags")
    lp, pp, pa = (_arr(a, _I32, nm) for a, nm in ((level_ptr, "level_ptr"), (par_ptr, "par_ptr"),
                                                   (partition, "partition")))
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csr_ilu_lbc(n, _p(Lp), _p(Li), _p(Lx), _p(diags), _p(x), level_no, _p(lp),
                                   _p(pp), _p(pa))
    _raise_last("sptrsv_csr_ilu_lbc")


def sptrsv_csr_levelset(n, Lp, Li, Lx, x, levels, levelPtr, levelSet):
    """sparse_blas/sptrsv.cpp:40-55."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    lp, ls = _arr(levelPtr, _I32, "levelPtr"), _arr(levelSet, _I32, "levelSet")
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csr_levelset(n, _p(Lp), _p(Li), _p(Lx), _p(x), levels, _p(lp), _p(ls))
    _raise_last("sptrsv_csr_levelset")


def sptrsv_csr_lbc(n, Lp, Li, Lx, x, level_no, level_ptr, par_ptr, partition):
    """sparse_blas/sptrsv.cpp:57-76."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    lp, pp, pa = (_arr(a, _I32, nm) for a, nm in ((level_ptr, "level_ptr"), (par_ptr, "par_ptr"),
                                                   (partition, "partition")))
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csr_lbc(n, _p(Lp), _p(Li), _p(Lx), _p(x), level_no, _p(lp), _p(pp), _p(pa))
    _raise_last("sptrsv_csr_lbc")


def sptrsv_csr_lbc_redundant(n, Lp, Li, Lx, x, b, level_no, level_ptr, par_ptr, partition, tmp=None):
    """sparse_blas/sptrsv.cpp:78-107; ``tmp`` (per-thread scratch) is unused."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    b = _arr(b, _F64, "b")
    lp, pp, pa = (_arr(a, _I32, nm) for a, nm in ((level_ptr, "level_ptr"), (par_ptr, "par_ptr"),
                                                   (partition, "partition")))
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csr_lbc_redundant(n, _p(Lp), _p(Li), _p(Lx), _p(x), _p(b), level_no, _p(lp),
                                         _p(pp), _p(pa), None)
    _raise_last("sptrsv_csr_lbc_redundant")


# ---- SpTRSV, CSC ----------------------------------------------------------

def sptrsv_csc(n, Lp, Li, Lx, x):
    """sparse_blas/sptrsv.cpp:129-137 -- column push, diagonal first."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csc(n, _p(Lp), _p(Li), _p(Lx), _p(x))
    _raise_last("sptrsv_csc")


def sptrsv_csc_levelset(n, Lp, Li, Lx, x, levels, levelptr, levelset):
    """sparse_blas/sptrsv.cpp:139-156."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    lp, ls = _arr(levelptr, _I32, "levelptr"), _arr(levelset, _I32, "levelset")
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csc_levelset(n, _p(Lp), _p(Li), _p(Lx), _p(x), levels, _p(lp), _p(ls))
    _raise_last("sptrsv_csc_levelset")


def sptrsv_csc_lbc(n, Lp, Li, Lx, x, level_no, level_ptr, par_ptr, partition):
    """sparse_blas/sptrsv.cpp:158-174."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    lp, pp, pa = (_arr(a, _I32, nm) for a, nm in ((level_ptr, "level_ptr"), (par_ptr, "par_ptr"),
                                                   (partition, "partition")))
    x = _arr(x, _F64, "x", True)
    lib().gbsym_sptrsv_csc_lbc(n, _p(Lp), _p(Li), _p(Lx), _p(x), level_no, _p(lp), _p(pp), _p(pa))
    _raise_last("sptrsv_csc_lbc")


def ltsolve(n, Lp, Li, Lx, x):
    """sparse_blas/sptrsv_lt.cpp:11-20 -- L^T x = b on the CSC of L; returns 1/0."""
    Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
    x = _arr(x, _F64, "x", True)
    return lib().gbsym_ltsolve(n, _p(Lp), _p(Li), _p(Lx), _p(x))


class parsy:  # noqa: N801 -- mirrors the reference's nested namespace
    """sym_lib::parsy entry points (Triangular_CSC.h, mgmres.hpp)."""

    @staticmethod
    def lsolve(n, Lp, Li, Lx, x):
        Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
        x = _arr(x, _F64, "x", True)
        return lib().gbsym_parsy_lsolve(n, _p(Lp), _p(Li), _p(Lx), _p(x))

    @staticmethod
    def ltsolve(n, Lp, Li, Lx, x):
        Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
        x = _arr(x, _F64, "x", True)
        return lib().gbsym_parsy_ltsolve(n, _p(Lp), _p(Li), _p(Lx), _p(x))

    @staticmethod
    def lsolvePar(n, Lp, Li, Lx, x, levels, levelPtr, levelSet, chunk=1):  # noqa: N802
        Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
        lp, ls = _arr(levelPtr, _I32, "levelPtr"), _arr(levelSet, _I32, "levelSet")
        x = _arr(x, _F64, "x", True)
        return lib().gbsym_parsy_lsolvePar(n, _p(Lp), _p(Li), _p(Lx), _p(x), levels, _p(lp), _p(ls), chunk)

    @staticmethod
    def lsolveParH2(n, Lp, Li, Lx, x, levels, levelPtr, levelSet, parts, parPtr, partition,  # noqa: N802
                    chunk=1):
        Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
        lp = _arr(levelPtr, _I32, "levelPtr")
        ls = None if levelSet is None else _arr(levelSet, _I32, "levelSet")
        pp, pa = _arr(parPtr, _I32, "parPtr"), _arr(partition, _I32, "partition")
        x = _arr(x, _F64, "x", True)
        return lib().gbsym_parsy_lsolveParH2(n, _p(Lp), _p(Li), _p(Lx), _p(x), levels, _p(lp), _p(ls),
                                             parts, _p(pp), _p(pa), chunk)

    @staticmethod
    def getLevelSet(n, inTree, levelPtr, levelSet):  # noqa: N802,N803
        """sparse_blas/parsy/common/TreeUtils.cpp:89-140 -- level set of a
        forest into caller arrays levelPtr (n+1) and levelSet (n); returns
        the level count."""
        t = _arr(inTree, _I32, "inTree")
        lp, ls = _arr(levelPtr, _I32, "levelPtr", True), _arr(levelSet, _I32, "levelSet", True)
        nl = lib().gbsym_tree_levelset(int(n), _p(t), _p(lp), _p(ls))
        if nl < 0:
            raise GbsymError(-nl, "getLevelSet")
        return nl

    @staticmethod
    def getCoarseLevelSet_6(n, eTree, blk2col, innerParts, minLevelDist, divRate,  # noqa: N802,N803
                            nodeCost):
        """sparse_blas/parsy/symbolic/InspectionLevel_06.cpp:17-400 -- tree
        LBC.  blk2col is accepted and unused, as in the reference.  Returns
        (finaLevelNo, finaLevelPtr, partNo, finalPartPtr, finalNodePtr)."""
        return _lbc_call(lib().gbsym_coarse_levelset_tree, n,
                         (_arr(eTree, _I32, "eTree"), _arr(nodeCost, _F64, "nodeCost")),
                         innerParts, minLevelDist, divRate, "getCoarseLevelSet_6")

    # ---- supernodal (blocked CSC) solves: S is a matgen.Supernodal, x a
    # float64 array of n (or n_rhs rows of n: column-major n x n_rhs) ----
    @staticmethod
    def _sn(S):
        return (int(S.n), _p(_arr(S.Lp, np.uint64, "Lp")), _p(_arr(S.Li, _I32, "Li")),
                _p(_arr(S.Lx, _F64, "Lx")), 0, _p(_arr(S.Li_ptr, np.uint64, "Li_ptr")),
                _p(_arr(S.col2sup, _I32, "col2sup")), _p(_arr(S.sup2col, _I32, "sup2col")), int(S.nsup))

    @staticmethod
    def blockedLsolve(S, x):  # noqa: N802
        """Triangular_BCSC.cpp:23-58 -- supernodal forward solve in place."""
        x = _arr(x, _F64, "x", True)
        return lib().gbsym_parsy_blockedLsolve(*parsy._sn(S), _p(x))

    @staticmethod
    def blockedLTsolve(S, x):  # noqa: N802
        """Triangular_BCSC.cpp:124-184 -- supernodal transposed solve in place."""
        x = _arr(x, _F64, "x", True)
        return lib().gbsym_parsy_blockedLTsolve(*parsy._sn(S), _p(x))

    @staticmethod
    def blockedLsolve_mrhs(S, X, n_rhs, max_col=-1):  # noqa: N802
        X = _arr(X, _F64, "X", True)
        return lib().gbsym_parsy_blockedLsolve_mrhs(*parsy._sn(S), _p(X), int(n_rhs), int(max_col))

    @staticmethod
    def blockedLTsolve_mrhs(S, X, m_rhs, max_col=-1):  # noqa: N802
        X = _arr(X, _F64, "X", True)
        return lib().gbsym_parsy_blockedLTsolve_mrhs(*parsy._sn(S), _p(X), int(m_rhs), int(max_col))

    @staticmethod
    def leveledBlockedLsolve(S, x, levels, levelPtr, levelSet, chunk=1):  # noqa: N802,N803
        x = _arr(x, _F64, "x", True)
        lp, ls = _arr(levelPtr, _I32, "levelPtr"), _arr(levelSet, _I32, "levelSet")
        return lib().gbsym_parsy_leveledBlockedLsolve(*parsy._sn(S), _p(x), int(levels), _p(lp), _p(ls),
                                                      int(chunk))

    @staticmethod
    def H2LeveledBlockedLsolve(S, x, levels, levelPtr, parts, parPtr, partition, chunk=1,  # noqa: N802,N803
                               transposed=False):
        x = _arr(x, _F64, "x", True)
        lp, pp, pa = (_arr(levelPtr, _I32, "levelPtr"), _arr(parPtr, _I32, "parPtr"),
                      _arr(partition, _I32, "partition"))
        fn = lib().gbsym_parsy_H2LeveledBlockedLTsolve if transposed else lib().gbsym_parsy_H2LeveledBlockedLsolve
        return fn(*parsy._sn(S), _p(x), int(levels), _p(lp), None, int(parts), _p(pp), _p(pa), int(chunk))

    @staticmethod
    def H2LeveledBlockedLsolve_mrhs(S, X, n_rhs, levels, levelPtr, parts, parPtr, partition,  # noqa: N802,N803
                                    chunk=1, max_col=-1, transposed=False):
        X = _arr(X, _F64, "X", True)
        lp, pp, pa = (_arr(levelPtr, _I32, "levelPtr"), _arr(parPtr, _I32, "parPtr"),
                      _arr(partition, _I32, "partition"))
        fn = (lib().gbsym_parsy_H2LeveledBlockedLTsolve_mrhs if transposed
              else lib().gbsym_parsy_H2LeveledBlockedLsolve_mrhs)
        return fn(*parsy._sn(S), _p(X), int(n_rhs), int(levels), _p(lp), None, int(parts), _p(pp), _p(pa),
                  int(chunk), int(max_col))

    @staticmethod
    def solve_phase_simplicial_ll(n, Lp, Li, Lx, x):  # noqa: N803
        """solve_phase.cpp:23-28 -- lsolve then ltsolve on the CSC of L."""
        Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
        x = _arr(x, _F64, "x", True)
        lib().gbsym_parsy_solve_phase_simplicial_ll(int(n), _p(Lp), _p(Li), _p(Lx), _p(x))
        _raise_last("solve_phase_simplicial_ll")

    @staticmethod
    def solve_phase_simplicial_ldl(n, Lp, Li, Lx, d_val, x):  # noqa: N803
        """solve_phase.cpp:30-37 -- lsolve, x /= d, ltsolve."""
        Lp, Li, Lx = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"), _arr(Lx, _F64, "Lx")
        d, x = _arr(d_val, _F64, "d_val"), _arr(x, _F64, "x", True)
        lib().gbsym_parsy_solve_phase_simplicial_ldl(int(n), _p(Lp), _p(Li), _p(Lx), _p(d), _p(x))
        _raise_last("solve_phase_simplicial_ldl")

    # solve phases: (n, x, ..., col2sup, sup2col, Lp, Li, Lx, Li_ptr, nsup, nnz)
    @staticmethod
    def _phase(S):
        return (_p(_arr(S.col2sup, _I32, "col2sup")), _p(_arr(S.sup2col, _I32, "sup2col")),
                _p(_arr(S.Lp, np.uint64, "Lp")), _p(_arr(S.Li, _I32, "Li")), _p(_arr(S.Lx, _F64, "Lx")),
                _p(_arr(S.Li_ptr, np.uint64, "Li_ptr")), int(S.nsup), 0)

    @staticmethod
    def solve_phase_ll_blocked(S, x):
        """solve_phase.cpp:39-46 -- L then L^T, in place (raises on error)."""
        x = _arr(x, _F64, "x", True)
        lib().gbsym_parsy_solve_phase_ll_blocked(int(S.n), _p(x), *parsy._phase(S))
        _raise_last("solve_phase_ll_blocked")

    @staticmethod
    def solve_phase_ll_blocked_nrhs(S, X, n_rhs, max_col=-1):
        X = _arr(X, _F64, "X", True)
        a = parsy._phase(S)
        lib().gbsym_parsy_solve_phase_ll_blocked_nrhs(int(S.n), _p(X), int(n_rhs), *a, int(max_col))
        _raise_last("solve_phase_ll_blocked_nrhs")

    @staticmethod
    def solve_phase_ll_blocked_parallel(S, x, levels, levelPtr, parts, parPtr, partition, chunk=1):  # noqa: N803
        x = _arr(x, _F64, "x", True)
        lp, pp, pa = (_arr(levelPtr, _I32, "levelPtr"), _arr(parPtr, _I32, "parPtr"),
                      _arr(partition, _I32, "partition"))
        lib().gbsym_parsy_solve_phase_ll_blocked_parallel(int(S.n), _p(x), *parsy._phase(S), int(levels), _p(lp),
                                                          None, int(parts), _p(pp), _p(pa), int(chunk))
        _raise_last("solve_phase_ll_blocked_parallel")

    @staticmethod
    def solve_phase_ll_blocked_parallel_nrhs(S, X, n_rhs, levels, levelPtr, parts, parPtr, partition,  # noqa: N803
                                             chunk=1, max_col=-1):
        X = _arr(X, _F64, "X", True)
        lp, pp, pa = (_arr(levelPtr, _I32, "levelPtr"), _arr(parPtr, _I32, "parPtr"),
                      _arr(partition, _I32, "partition"))
        lib().gbsym_parsy_solve_phase_ll_blocked_parallel_nrhs(int(S.n), _p(X), int(n_rhs), *parsy._phase(S),
                                                               int(levels), _p(lp), None, int(parts), _p(pp),
                                                               _p(pa), int(chunk), int(max_col))
        _raise_last("solve_phase_ll_blocked_parallel_nrhs")

    @staticmethod
    def solve_phase_ldl(S, d_val, x):
        """solve_phase.cpp:96-112 -- L, x /= d, L^T, in place."""
        x = _arr(x, _F64, "x", True)
        d = _arr(d_val, _F64, "d_val")
        lib().gbsym_parsy_solve_phase_ldl(int(S.n), _p(d), _p(x), *parsy._phase(S))
        _raise_last("solve_phase_ldl")

    @staticmethod
    def lus_cr(n, nz_num, ia, ja, l, ua, r, z):
        """sparse_blas/parsy/gmres/mgmres.cpp:598-689 -- z = (LU)^{-1} r."""
        ia, ja, ua = _arr(ia, _I32, "ia"), _arr(ja, _I32, "ja"), _arr(ua, _I32, "ua")
        l, r = _arr(l, _F64, "l"), _arr(r, _F64, "r")
        z = _arr(z, _F64, "z", True)
        lib().gbsym_parsy_lus_cr(n, nz_num, _p(ia), _p(ja), _p(l), _p(ua), _p(r), _p(z))
        _raise_last("lus_cr")


# ---- SpMV -----------------------------------------------------------------

def spmv_csr(n, Ap, Ai, Ax, x, y, z=None, a=None, b=None):
    """sparse_blas/spmv.cpp:12-21 (y = A x), or with (z, a, b) the overload at
    spmv.cpp:23-34: z += A x (z is not cleared), then z = a z + b y."""
    Ap, Ai, Ax = _arr(Ap, _I32, "Ap"), _arr(Ai, _I32, "Ai"), _arr(Ax, _F64, "Ax")
    x = _arr(x, _F64, "x")
    if z is None:
        y = _arr(y, _F64, "y", True)
        lib().gbsym_spmv_csr(n, _p(Ap), _p(Ai), _p(Ax), _p(x), _p(y))
    else:
        y = _arr(y, _F64, "y")
        z = _arr(z, _F64, "z", True)
        lib().gbsym_spmv_csr_axpby(n, _p(Ap), _p(Ai), _p(Ax), _p(x), _p(y), _p(z), float(a), float(b))
    _raise_last("spmv_csr")


def spmv_csr_parallel(n, Ap, Ai, Ax, x, y):
    """sparse_blas/spmv.cpp:37-57."""
    Ap, Ai, Ax = _arr(Ap, _I32, "Ap"), _arr(Ai, _I32, "Ai"), _arr(Ax, _F64, "Ax")
    x = _arr(x, _F64, "x")
    y = _arr(y, _F64, "y", True)
    lib().gbsym_spmv_csr_parallel(n, _p(Ap), _p(Ai), _p(Ax), _p(x), _p(y))
    _raise_last("spmv_csr_parallel")


# ---- factor producers -----------------------------------------------------

def spilu0_csr(n, nnz, Ap, Ai, Ax, A_diag, l):
    """sparse_blas/spilu0.cpp:11-51 -- l receives the packed ILU0 factor."""
    Ap, Ai, Ax = _arr(Ap, _I32, "Ap"), _arr(Ai, _I32, "Ai"), _arr(Ax, _F64, "Ax")
    A_diag = _arr(A_diag, _I32, "A_diag")
    l = _arr(l, _F64, "l", True)
    lib().gbsym_spilu0_csr(n, nnz, _p(Ap), _p(Ai), _p(Ax), _p(A_diag), _p(l))
    _raise_last("spilu0_csr")


def spic0_csr(n, val, rowPtr, rowIdx):  # noqa: N803
    """sparse_blas/spic0.cpp:106-128 -- IC0 in place on the upper CSR of A."""
    val = _arr(val, _F64, "val", True)
    rowPtr, rowIdx = _arr(rowPtr, _I32, "rowPtr"), _arr(rowIdx, _I32, "rowIdx")
    lib().gbsym_spic0_csr(n, _p(val), _p(rowPtr), _p(rowIdx))
    _raise_last("spic0_csr")


def spilu0_csr_lbc(n, nnz, Ap, Ai, Ax, A_diag, l, level_no, level_ptr, par_ptr, partition, tempvecs=None):
    """sparse_blas/spilu0.cpp:54-106 -- the schedule is validated, then l
    receives the packed ILU0 factor (equal to spilu0_csr's); ``tempvecs``
    (per-thread scratch) is unused."""
    Ap, Ai, Ax = _arr(Ap, _I32, "Ap"), _arr(Ai, _I32, "Ai"), _arr(Ax, _F64, "Ax")
    A_diag = _arr(A_diag, _I32, "A_diag")
    lp, pp, pa = (_arr(a, _I32, nm) for a, nm in ((level_ptr, "level_ptr"), (par_ptr, "par_ptr"),
                                                   (partition, "partition")))
    l = _arr(l, _F64, "l", True)
    lib().gbsym_spilu0_csr_lbc(n, nnz, _p(Ap), _p(Ai), _p(Ax), _p(A_diag), _p(l), level_no, _p(lp), _p(pp),
                               _p(pa), None)
    _raise_last("spilu0_csr_lbc")


def spic0_csr_lbc(n, val, rowPtr, colIdx, level_no, level_ptr, par_ptr, partition):  # noqa: N803
    """sparse_blas/spic0.cpp:130-160 -- IC0 in place on the upper CSR of A
    under a validated LBC schedule over the columns of L; the result equals
    spic0_csr's bit for bit."""
    val = _arr(val, _F64, "val", True)
    rowPtr, colIdx = _arr(rowPtr, _I32, "rowPtr"), _arr(colIdx, _I32, "colIdx")
    lp, pp, pa = (_arr(a, _I32, nm) for a, nm in ((level_ptr, "level_ptr"), (par_ptr, "par_ptr"),
                                                   (partition, "partition")))
    lib().gbsym_spic0_csr_lbc(n, _p(val), _p(rowPtr), _p(colIdx), level_no, _p(lp), _p(pp), _p(pa))
    _raise_last("spic0_csr_lbc")


# ---- schedule builders ----------------------------------------------------

def _levels(fn, n, p, i, where):
    p, i = _arr(p, _I32, "ptr"), _arr(i, _I32, "idx")
    lp = C.POINTER(C.c_int)()
    ls = C.POINTER(C.c_int)()
    nl = fn(n, _p(p), _p(i), C.byref(lp), C.byref(ls))
    if nl < 0:
        raise GbsymError(-nl, where)
    try:
        level_ptr = np.ctypeslib.as_array(lp, shape=(nl + 1,)).copy()
        level_set = np.ctypeslib.as_array(ls, shape=(max(n, 1),))[:n].copy()
    finally:
        lib().gbsym_free(C.cast(lp, C.c_void_p))
        lib().gbsym_free(C.cast(ls, C.c_void_p))
    return nl, level_ptr, level_set


def build_levelSet_CSC(n, Lp, Li):  # noqa: N802
    """Level set of the lower CSC L (call sites: Catch_tests/sptrsv_tests.cpp:59,
    demo/sptrsv_demo_utils.h:42-45).  Returns (level_no, level_ptr, level_set)."""
    return _levels(lib().gbsym_build_levelset_csc, n, Lp, Li, "build_levelSet_CSC")


def build_levelset_csr(n, Lp, Li):
    return _levels(lib().gbsym_build_levelset_csr, n, Lp, Li, "build_levelset_csr")


def build_levelset_upper_csr(n, Up, Ui):
    return _levels(lib().gbsym_build_levelset_upper_csr, n, Up, Ui, "build_levelset_upper_csr")


# ---- LBC inspectors ---------------------------------------------------------

def _lbc_call(fn, n, arrays, inner_parts, min_level_dist, div_rate, where):
    nl, pn = C.c_int(0), C.c_int(0)
    lp, pp, nd = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    st = fn(int(n), *[_p(a) for a in arrays], int(inner_parts), int(min_level_dist), int(div_rate),
            C.byref(nl), C.byref(lp), C.byref(pn), C.byref(pp), C.byref(nd))
    if st != 0:
        raise GbsymError(st, where)
    if n == 0:
        z = np.zeros(1, dtype=_I32)
        return 0, z, 0, z.copy(), np.zeros(0, dtype=_I32)
    try:
        level_ptr = np.ctypeslib.as_array(lp, shape=(nl.value + 1,)).copy()
        part_ptr = np.ctypeslib.as_array(pp, shape=(pn.value + 1,)).copy()
        node_ptr = np.ctypeslib.as_array(nd, shape=(n,)).copy()
    finally:
        for q in (lp, pp, nd):
            lib().gbsym_free(C.cast(q, C.c_void_p))
    return nl.value, level_ptr, pn.value, part_ptr, node_ptr


def get_coarse_levelSet_DAG_CSC_tree(n, Lp, Li, stype, lp, cp, ic, cost=None):  # noqa: N802
    """LBC of the solve DAG of the lower CSR (Lp, Li), as the reference demo
    calls it (demo/sptrsv_demo_utils.h:78-90): lp = parts per coarse level,
    cp = minimum level distance, ic = division rate; cost defaults to the
    entries per row.  stype is accepted and unused.  Returns (level_no,
    level_ptr, part_no, part_ptr, node_ptr)."""
    arrays = (_arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li"),
              None if cost is None else _arr(cost, _F64, "cost"))
    return _lbc_call(lib().gbsym_build_lbc, n, arrays, lp, cp, ic, "get_coarse_levelSet_DAG_CSC_tree")


def etree_lower_csr(n, Lp, Li):
    """Elimination tree (parent array, -1 at roots) of the symmetric matrix
    whose lower triangle has the pattern of the CSR (Lp, Li)."""
    Lp, Li = _arr(Lp, _I32, "Lp"), _arr(Li, _I32, "Li")
    parent = np.zeros(max(int(n), 1), dtype=_I32)
    st = lib().gbsym_etree_lower_csr(int(n), _p(Lp), _p(Li), _p(parent))
    if st != 0:
        raise GbsymError(st, "etree_lower_csr")
    return parent[: int(n)]


# ---- drop-in plan cache (no counterpart in the reference) ---------------------

def dropin_cache(capacity):
    """Let the drop-ins keep up to ``capacity`` plans, keyed by the arrays
    they were given (0, the default, turns the cache off): see
    gbsym_dropin_cache in include/gbsym.h.  Changing a cached matrix's arrays
    in place requires a new :func:`dropin_cache_version`."""
    st = lib().gbsym_dropin_cache(int(capacity))
    if st != 0:
        raise GbsymError(st, "dropin_cache")


def dropin_cache_version(version):
    """Declare that matrices passed before may have changed: plans cached
    under another version are dropped."""
    lib().gbsym_dropin_cache_version(int(version))
