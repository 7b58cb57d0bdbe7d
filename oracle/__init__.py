"""Oracle for the GB300 SpTRSV executor -- TEST INFRASTRUCTURE ONLY.

``oracle.orc`` wraps the project's C restatement of the reference
(``oracle/oracle.c``); ``oracle.ref`` wraps the reference's own compiled C++
(``oracle/_ref/libsymref.so``) when it has been built.  Only the tests, the
smoke check and the benchmark's CPU-baseline leg may import this package;
the product (``sympiler_gb300``) never does.

All wrappers take numpy arrays (int32 indices, float64/float32 values) and,
like the reference, update ``x`` in place.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_i = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_z = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")  # size_t arrays
_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_int, _dbl, _vp = C.c_int, C.c_double, C.c_void_p


def _load(path):
    return C.CDLL(path, mode=C.RTLD_LOCAL)


def _bind(lib, name, restype, argtypes):
    fn = getattr(lib, name)
    fn.restype = restype
    fn.argtypes = argtypes
    return fn


class _Orc:
    """The C restatement."""

    def __init__(self, path):
        L = self.lib = _load(path)
        b = lambda n, r, a: _bind(L, n, r, a)  # noqa: E731
        self.sptrsv_csr = b("orc_sptrsv_csr", None, [_int, _i, _i, _d, _d])
        self.sptrsv_csr_ilu = b("orc_sptrsv_csr_ilu", None, [_int, _i, _i, _d, _i, _d])
        self._levelset = b("orc_sptrsv_csr_levelset", None, [_int, _i, _i, _d, _d, _int, _i, _i, _int])
        self.sptrsv_csr_lbc = b("orc_sptrsv_csr_lbc", None, [_int, _i, _i, _d, _d, _int, _i, _i, _i])
        self.sptrsv_csr_lbc_redundant = b("orc_sptrsv_csr_lbc_redundant", None,
                                          [_int, _i, _i, _d, _d, _d, _int, _i, _i, _i])
        self.sptrsv_csr_ilu_lbc = b("orc_sptrsv_csr_ilu_lbc", None,
                                    [_int, _i, _i, _d, _i, _d, _int, _i, _i, _i])
        self.sptrsv_csc = b("orc_sptrsv_csc", None, [_int, _i, _i, _d, _d])
        self.sptrsv_csc_levelset = b("orc_sptrsv_csc_levelset", None, [_int, _i, _i, _d, _d, _int, _i, _i])
        self.ltsolve = b("orc_ltsolve", _int, [_int, _i, _i, _d, _d])
        self._mrhs = b("orc_sptrsv_csr_mrhs", None, [_int, _i, _i, _d, _d, _int, _int])
        self._levelset_mrhs = b("orc_sptrsv_csr_levelset_mrhs", None,
                                [_int, _i, _i, _d, _d, _int, _int, _i, _i, _int])
        self.spmv_csr = b("orc_spmv_csr", None, [_int, _i, _i, _d, _d, _d])
        self.spmv_csr_axpby = b("orc_spmv_csr_axpby", None, [_int, _i, _i, _d, _d, _d, _d, _dbl, _dbl])
        self._spmv_par = b("orc_spmv_csr_parallel", None, [_int, _i, _i, _d, _d, _d, _int])
        self._spilu0 = b("orc_spilu0_csr", _int, [_int, _int, _i, _i, _d, _i, _d])
        self._spic0 = b("orc_spic0_csr", _int, [_int, _d, _i, _i])
        self._lus_cr = b("orc_lus_cr", None, [_int, _int, _i, _i, _d, _i, _d, _d])
        self._lus_cr_f32 = b("orc_lus_cr_f32", None, [_int, _i, _i, _f, _i, _f, _f])
        self.sptrsv_csr_f32 = b("orc_sptrsv_csr_f32", None, [_int, _i, _i, _f, _f])
        self.ltsolve_f32 = b("orc_ltsolve_f32", None, [_int, _i, _i, _f, _f])
        self.spmv_csr_f32 = b("orc_spmv_csr_f32", None, [_int, _i, _i, _f, _f, _f])
        self._lvl_csr = b("orc_build_levelset_csr", _int, [_int, _i, _i, _i, _i])
        self._lvl_csc = b("orc_build_levelset_csc", _int, [_int, _i, _i, _i, _i])
        self._lvl_up = b("orc_build_levelset_upper_csr", _int, [_int, _i, _i, _i, _i])
        self._lvl_tree = b("orc_tree_levelset", _int, [_int, _i, _i, _i])
        self._pcg = b("orc_pcg_ic0", _int, [_int, _i, _i, _d, _i, _i, _d, _i, _i, _d, _d, _d,
                                             _dbl, _int, C.POINTER(_dbl)])
        self._gmres = b("orc_gmres_ilu0", _int, [_int, _i, _i, _d, _d, _i, _d, _d, _int, _int,
                                                  _dbl, C.POINTER(_dbl)])
        self._blk_l = b("orc_blocked_lsolve", None, [_int, _z, _i, _d, _z, _i, _int, _d, _int])
        self._blk_lt = b("orc_blocked_ltsolve", None, [_int, _z, _i, _d, _z, _i, _int, _d, _int])

    def blocked_lsolve(self, S, X):
        """Supernodal forward solve; X is (nrhs, n) C-contiguous = column-major n x nrhs."""
        nrhs = 1 if X.ndim == 1 else X.shape[0]
        self._blk_l(S.n, S.Lp, S.Li, S.Lx, S.Li_ptr, S.sup2col, S.nsup, X, nrhs)

    def blocked_ltsolve(self, S, X):
        nrhs = 1 if X.ndim == 1 else X.shape[0]
        self._blk_lt(S.n, S.Lp, S.Li, S.Lx, S.Li_ptr, S.sup2col, S.nsup, X, nrhs)

    # ---- convenience wrappers returning numpy arrays ----------------------
    def sptrsv_csr_levelset(self, n, Lp, Li, Lx, x, levels, lp, ls, nthreads=1):
        self._levelset(n, Lp, Li, Lx, x, levels, lp, ls, nthreads)

    def sptrsv_csr_mrhs(self, n, Lp, Li, Lx, X_colmajor, k, nthreads=1):
        self._mrhs(n, Lp, Li, Lx, X_colmajor, k, nthreads)

    def sptrsv_csr_levelset_mrhs(self, n, Lp, Li, Lx, X_colmajor, k, levels, lp, ls, nthreads=1):
        self._levelset_mrhs(n, Lp, Li, Lx, X_colmajor, k, levels, lp, ls, nthreads)

    def spmv_csr_parallel(self, n, Ap, Ai, Ax, x, y, nthreads=1):
        self._spmv_par(n, Ap, Ai, Ax, x, y, nthreads)

    def spilu0_csr(self, n, Ap, Ai, Ax, A_diag):
        l = np.empty_like(Ax)
        ok = self._spilu0(n, int(Ap[n]), Ap, Ai, Ax, A_diag, l)
        return l, bool(ok)

    def spic0_csr(self, n, Up, Ui, Ux):
        """IC0 of the upper CSR of A; returns the factor values (new array)."""
        v = np.array(Ux, dtype=np.float64, copy=True)
        ok = self._spic0(n, v, Up, Ui)
        return v, bool(ok)

    def lus_cr(self, n, ia, ja, l, ua, r):
        z = np.empty(n, dtype=np.float64)
        self._lus_cr(n, int(ia[n]), ia, ja, l, ua, np.ascontiguousarray(r, dtype=np.float64), z)
        return z

    def lus_cr_f32(self, n, ia, ja, l32, ua, r32):
        z = np.empty(n, dtype=np.float32)
        self._lus_cr_f32(n, ia, ja, l32, ua, np.ascontiguousarray(r32, dtype=np.float32), z)
        return z

    def _sets(self, fn, n, p, i):
        lp = np.zeros(n + 1, dtype=np.int32)
        ls = np.zeros(max(n, 1), dtype=np.int32)
        nl = fn(n, p, i, lp, ls)
        return nl, lp[: nl + 1].copy(), ls[:n].copy()

    def build_levelset_csr(self, n, Lp, Li):
        return self._sets(self._lvl_csr, n, Lp, Li)

    def build_levelset_csc(self, n, Lp, Li):
        return self._sets(self._lvl_csc, n, Lp, Li)

    def build_levelset_upper_csr(self, n, Up, Ui):
        return self._sets(self._lvl_up, n, Up, Ui)

    def tree_levelset(self, n, tree):
        lp = np.zeros(n + 1, dtype=np.int32)
        ls = np.zeros(max(n, 1), dtype=np.int32)
        nl = self._lvl_tree(n, np.ascontiguousarray(tree, dtype=np.int32), lp, ls)
        return nl, lp[: nl + 1].copy(), ls[:n].copy()

    def pcg_ic0(self, n, A, L, Lt, b, tol=1e-10, maxit=10000, x0=None):
        x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
        rel = C.c_double(0)
        it = self._pcg(n, *A, *L, *Lt, np.ascontiguousarray(b), x, tol, maxit, C.byref(rel))
        return x, it, rel.value

    def gmres_ilu0(self, n, A, lu, ua, b, mr=30, itr_max=1000, tol=1e-10, x0=None):
        x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
        rel = C.c_double(0)
        it = self._gmres(n, *A, lu, ua, np.ascontiguousarray(b), x, mr, itr_max, tol, C.byref(rel))
        return x, it, rel.value


class _Ref:
    """The reference's own compiled executors (built from its source tree)."""

    def __init__(self, path):
        L = self.lib = _load(path)
        b = lambda n, r, a: _bind(L, n, r, a)  # noqa: E731
        self.sptrsv_csr = b("ref_sptrsv_csr", None, [_int, _i, _i, _d, _d])
        self.sptrsv_csr_ilu = b("ref_sptrsv_csr_ilu", None, [_int, _i, _i, _d, _i, _d])
        self.sptrsv_csr_levelset = b("ref_sptrsv_csr_levelset", None, [_int, _i, _i, _d, _d, _int, _i, _i])
        self.sptrsv_csr_lbc = b("ref_sptrsv_csr_lbc", None, [_int, _i, _i, _d, _d, _int, _i, _i, _i])
        self._lbc_red = b("ref_sptrsv_csr_lbc_redundant", None,
                          [_int, _i, _i, _d, _d, _d, _int, _i, _i, _i, _d])
        self.sptrsv_csr_ilu_lbc = b("ref_sptrsv_csr_ilu_lbc", None,
                                    [_int, _i, _i, _d, _i, _d, _int, _i, _i, _i])
        self.sptrsv_csc = b("ref_sptrsv_csc", None, [_int, _i, _i, _d, _d])
        self.sptrsv_csc_levelset = b("ref_sptrsv_csc_levelset", None, [_int, _i, _i, _d, _d, _int, _i, _i])
        self.sptrsv_csc_lbc = b("ref_sptrsv_csc_lbc", None, [_int, _i, _i, _d, _d, _int, _i, _i, _i])
        self.ltsolve = b("ref_ltsolve", _int, [_int, _i, _i, _d, _d])
        self.parsy_lsolve = b("ref_parsy_lsolve", _int, [_int, _i, _i, _d, _d])
        self.parsy_ltsolve = b("ref_parsy_ltsolve", _int, [_int, _i, _i, _d, _d])
        self.parsy_lsolvePar = b("ref_parsy_lsolvePar", _int, [_int, _i, _i, _d, _d, _int, _i, _i, _int])
        self.parsy_lsolveParH2 = b("ref_parsy_lsolveParH2", _int,
                                   [_int, _i, _i, _d, _d, _int, _i, _i, _int, _i, _i, _int])
        self.spmv_csr = b("ref_spmv_csr", None, [_int, _i, _i, _d, _d, _d])
        self.spmv_csr_axpby = b("ref_spmv_csr_axpby", None, [_int, _i, _i, _d, _d, _d, _d, _dbl, _dbl])
        self.spmv_csr_parallel = b("ref_spmv_csr_parallel", None, [_int, _i, _i, _d, _d, _d])
        self._spilu0 = b("ref_spilu0_csr", None, [_int, _int, _i, _i, _d, _i, _d])
        self._spic0 = b("ref_spic0_csr", None, [_int, _d, _i, _i])
        self._spilu0_lbc = b("ref_spilu0_csr_lbc", None, [_int, _int, _i, _i, _d, _i, _d, _int, _i, _i, _i])
        self._spic0_lbc = b("ref_spic0_csr_lbc", None, [_int, _d, _i, _i, _int, _i, _i, _i])
        self._lus_cr = b("ref_lus_cr", None, [_int, _int, _i, _i, _d, _i, _d, _d])
        self._tree_lvl = b("ref_tree_levelset", _int, [_int, _i, _i, _i])
        self._coarse6 = b("ref_coarse_levelset6", _int,
                          [_int, _i, _int, _int, _int, _d, _i, _i, _i, C.POINTER(_int)])
        self._blk_l = b("ref_blocked_lsolve", _int, [_int, _z, _i, _d, _z, _i, _i, _int, _d])
        self._blk_l_lvl = b("ref_leveled_blocked_lsolve", _int,
                            [_int, _z, _i, _d, _z, _i, _i, _int, _d, _int, _i, _i])
        self._blk_l_h2 = b("ref_h2_leveled_blocked_lsolve", _int,
                           [_int, _z, _i, _d, _z, _i, _i, _int, _d, _int, _i, _i, _int, _i, _i])

    def blocked_lsolve(self, S, x):
        return self._blk_l(S.n, S.Lp, S.Li, S.Lx, S.Li_ptr, S.col2sup, S.sup2col, S.nsup, x)

    def leveled_blocked_lsolve(self, S, x, levels, lp, ls):
        return self._blk_l_lvl(S.n, S.Lp, S.Li, S.Lx, S.Li_ptr, S.col2sup, S.sup2col, S.nsup, x,
                               levels, lp, ls)

    def h2_leveled_blocked_lsolve(self, S, x, levels, lp, ls, parts, pp, part):
        return self._blk_l_h2(S.n, S.Lp, S.Li, S.Lx, S.Li_ptr, S.col2sup, S.sup2col, S.nsup, x,
                              levels, lp, ls, parts, pp, part)

    def sptrsv_csr_lbc_redundant(self, n, Lp, Li, Lx, x, b, level_no, lp, pp, part, nthreads=64):
        tmp = np.zeros(n * nthreads, dtype=np.float64)
        self._lbc_red(n, Lp, Li, Lx, x, b, level_no, lp, pp, part, tmp)

    def spilu0_csr(self, n, Ap, Ai, Ax, A_diag):
        l = np.empty_like(Ax)
        self._spilu0(n, int(Ap[n]), Ap, Ai, Ax, A_diag, l)
        return l

    def spic0_csr(self, n, Up, Ui, Ux):
        # the reference reads Li one entry past a row; pad so the read of the
        # last row's successor stays inside the buffer
        Ui_pad = np.concatenate([Ui, np.array([n], dtype=np.int32)])
        v = np.array(Ux, dtype=np.float64, copy=True)
        self._spic0(n, v, Up, Ui_pad)
        return v

    def spilu0_csr_lbc(self, n, Ap, Ai, Ax, A_diag, level_no, lp, pp, part):
        l = np.empty_like(Ax)
        self._spilu0_lbc(n, int(Ap[n]), Ap, Ai, Ax, A_diag, l, level_no, lp, pp, part)
        return l

    def spic0_csr_lbc(self, n, Up, Ui, Ux, level_no, lp, pp, part):
        # padded like spic0_csr: the reference reads one index past a row
        Ui_pad = np.concatenate([Ui, np.array([n], dtype=np.int32)])
        v = np.array(Ux, dtype=np.float64, copy=True)
        self._spic0_lbc(n, v, Up, Ui_pad, level_no, lp, pp, part)
        return v

    def lus_cr(self, n, ia, ja, l, ua, r):
        z = np.empty(n, dtype=np.float64)
        self._lus_cr(n, int(ia[n]), ia, ja, np.ascontiguousarray(l), ua,
                     np.array(r, dtype=np.float64, copy=True), z)
        return z

    def tree_levelset(self, n, tree):
        lp = np.zeros(n + 1, dtype=np.int32)
        ls = np.zeros(max(n, 1), dtype=np.int32)
        nl = self._tree_lvl(n, np.ascontiguousarray(tree, dtype=np.int32), lp, ls)
        return nl, lp[: nl + 1].copy(), ls[:n].copy()

    def coarse_levelset6(self, n, etree, cost, inner_parts=4, min_level_dist=-1, div_rate=4000):
        lp = np.zeros(n + 1, dtype=np.int32)
        pp = np.zeros(n + 1, dtype=np.int32)
        part = np.zeros(max(n, 1), dtype=np.int32)
        pn = C.c_int(0)
        nl = self._coarse6(n, np.ascontiguousarray(etree, dtype=np.int32), inner_parts,
                           min_level_dist, div_rate, np.ascontiguousarray(cost, dtype=np.float64),
                           lp, pp, part, C.byref(pn))
        return nl, lp[: nl + 1].copy(), pp[: pn.value + 1].copy(), part[:n].copy()


_orc = None
_ref = None


def orc() -> _Orc:
    """The C restatement (built on first use)."""
    global _orc
    if _orc is None:
        _orc = _Orc(_build.build_oracle())
    return _orc


def ref():
    """The reference's compiled executors, or None where its tree is absent."""
    global _ref
    if _ref is None:
        path = _build.REF_SO if os.path.exists(_build.REF_SO) else _build.build_reference()
        if path is None or not os.path.exists(path):
            return None
        try:
            _ref = _Ref(path)
        except OSError:
            return None
    return _ref
