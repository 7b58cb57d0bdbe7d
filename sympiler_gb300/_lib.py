"""ctypes binding of ``libgbsym.so`` (declared in ``include/gbsym.h``).

Loading fails loudly when the library has not been built: there is no
fallback implementation behind this package.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbsym.so")

_int, _dbl, _vp, _ull, _ll, _sz = C.c_int, C.c_double, C.c_void_p, C.c_ulonglong, C.c_longlong, C.c_size_t
_pi = C.POINTER(C.c_int)
_pd = C.POINTER(C.c_double)
_ppi = C.POINTER(C.POINTER(C.c_int))


class TriInfo(C.Structure):
    _fields_ = [("n", _int), ("levels", _int), ("nnz_off", _ll), ("dtype", _int), ("exec", _int),
                ("max_level_rows", _int), ("bytes_matrix", _ll)]


class KrylovResult(C.Structure):
    _fields_ = [("iterations", _int), ("restarts", _int), ("relres", _dbl), ("seconds", _dbl),
                ("status", _int)]


# name -> (restype, argtypes); every entry point of include/gbsym.h
SIGNATURES = {
    "gbsym_last_error": (_int, []),
    "gbsym_status_string": (C.c_char_p, [_int]),
    "gbsym_free": (None, [_vp]),
    "gbsym_kernel_launches": (_ull, []),
    "gbsym_dropin_cache": (_int, [_int]),
    "gbsym_dropin_cache_version": (None, [_ull]),
    # drop-ins
    "gbsym_sptrsv_csr": (None, [_int, _vp, _vp, _vp, _vp]),
    "gbsym_sptrsv_csr_ilu": (None, [_int, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_sptrsv_csr_ilu_lbc": (None, [_int, _vp, _vp, _vp, _vp, _vp, _int, _vp, _vp, _vp]),
    "gbsym_sptrsv_csr_levelset": (None, [_int, _vp, _vp, _vp, _vp, _int, _vp, _vp]),
    "gbsym_sptrsv_csr_lbc": (None, [_int, _vp, _vp, _vp, _vp, _int, _vp, _vp, _vp]),
    "gbsym_sptrsv_csr_lbc_redundant": (None, [_int, _vp, _vp, _vp, _vp, _vp, _int, _vp, _vp, _vp, _vp]),
    "gbsym_sptrsv_csc": (None, [_int, _vp, _vp, _vp, _vp]),
    "gbsym_sptrsv_csc_levelset": (None, [_int, _vp, _vp, _vp, _vp, _int, _vp, _vp]),
    "gbsym_sptrsv_csc_lbc": (None, [_int, _vp, _vp, _vp, _vp, _int, _vp, _vp, _vp]),
    "gbsym_ltsolve": (_int, [_int, _vp, _vp, _vp, _vp]),
    "gbsym_parsy_lsolve": (_int, [_int, _vp, _vp, _vp, _vp]),
    "gbsym_parsy_ltsolve": (_int, [_int, _vp, _vp, _vp, _vp]),
    "gbsym_parsy_lsolvePar": (_int, [_int, _vp, _vp, _vp, _vp, _int, _vp, _vp, _int]),
    "gbsym_parsy_lsolveParH2": (_int, [_int, _vp, _vp, _vp, _vp, _int, _vp, _vp, _int, _vp, _vp, _int]),
    "gbsym_spmv_csr": (None, [_int, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_spmv_csr_axpby": (None, [_int, _vp, _vp, _vp, _vp, _vp, _vp, _dbl, _dbl]),
    "gbsym_spmv_csr_parallel": (None, [_int, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_spilu0_csr": (None, [_int, _int, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_spic0_csr": (None, [_int, _vp, _vp, _vp]),
    "gbsym_spilu0_csr_lbc": (None, [_int, _int, _vp, _vp, _vp, _vp, _vp, _int, _vp, _vp, _vp, _vp]),
    "gbsym_spic0_csr_lbc": (None, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp]),
    "gbsym_parsy_lus_cr": (None, [_int, _int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_build_levelset_csc": (_int, [_int, _vp, _vp, _ppi, _ppi]),
    "gbsym_build_levelset_csr": (_int, [_int, _vp, _vp, _ppi, _ppi]),
    "gbsym_build_levelset_upper_csr": (_int, [_int, _vp, _vp, _ppi, _ppi]),
    # plans
    "gbsym_tri_create": (_int, [C.POINTER(_vp), _int, _vp, _vp, _vp, _vp, _int, _int, _int, _vp, _vp,
                                _int, _vp]),
    "gbsym_tri_destroy": (_int, [_vp]),
    "gbsym_tri_get_info": (_int, [_vp, C.POINTER(TriInfo)]),
    "gbsym_tri_set_exec": (_int, [_vp, _int]),
    "gbsym_tri_check": (_int, [_vp, _vp]),
    "gbsym_selftest_bounded_wait": (_int, [_ll, _vp]),
    "gbsym_fp64_rates": (_int, [_vp, _vp, _vp]),
    "gbsym_batch_solve_host": (_int, [_vp, _vp, _int, _int]),
    "gbsym_tri_set_arith": (_int, [_vp, _int]),
    "gbsym_tri_autotune": (_int, [_vp, _int, _int, _vp, _pi]),
    "gbsym_tri_get_schedule": (_int, [_vp, _vp, _vp]),
    "gbsym_tri_solve": (_int, [_vp, _vp, _int, _int, _int, _vp]),
    "gbsym_tri_solve_b": (_int, [_vp, _vp, _vp, _vp]),
    "gbsym_tri_solve_into": (_int, [_vp, _vp, _vp, _int, _int, _vp]),
    "gbsym_tri_solve_host": (_int, [_vp, _vp, _int, _int]),
    "gbsym_host_solve_in_place": (_int, [_vp]),
    "gbsym_tree_levelset": (_int, [_int, _vp, _vp, _vp]),
    "gbsym_coarse_levelset_tree": (_int, [_int, _vp, _vp, _int, _int, _int, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_build_lbc": (_int, [_int, _vp, _vp, _vp, _int, _int, _int, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_etree_lower_csr": (_int, [_int, _vp, _vp, _vp]),
    "gbsym_parsy_blockedLsolve": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp]),
    "gbsym_parsy_blockedLTsolve": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp]),
    "gbsym_parsy_blockedLsolve_mrhs": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp, _int, _int]),
    "gbsym_parsy_blockedLTsolve_mrhs": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp, _int, _int]),
    "gbsym_parsy_leveledBlockedLsolve": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp, _int, _vp, _vp, _int]),
    "gbsym_parsy_H2LeveledBlockedLsolve": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp, _int, _vp, _vp, _int, _vp, _vp, _int]),
    "gbsym_parsy_H2LeveledBlockedLTsolve": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp, _int, _vp, _vp, _int, _vp, _vp, _int]),
    "gbsym_parsy_H2LeveledBlockedLsolve_mrhs": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp, _int, _int, _vp, _vp, _int, _vp, _vp, _int, _int]),
    "gbsym_parsy_H2LeveledBlockedLTsolve_mrhs": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp, _int, _int, _vp, _vp, _int, _vp, _vp, _int, _int]),
    "gbsym_parsy_solve_phase_simplicial_ll": (None, [_int, _vp, _vp, _vp, _vp]),
    "gbsym_parsy_solve_phase_simplicial_ldl": (None, [_int, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_parsy_solve_phase_ll_blocked": (None, [_sz, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _int]),
    "gbsym_parsy_solve_phase_ll_blocked_nrhs": (None, [_sz, _vp, _int, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _int, _int]),
    "gbsym_parsy_solve_phase_ll_blocked_parallel": (None, [_sz, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _int, _int, _vp, _vp, _int, _vp, _vp, _int]),
    "gbsym_parsy_solve_phase_ll_blocked_parallel_nrhs": (None, [_sz, _vp, _int, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _int, _int, _vp, _vp, _int, _vp, _vp, _int, _int]),
    "gbsym_parsy_solve_phase_ldl": (None, [_sz, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _int]),
    "gbsym_sn_create": (_int, [_vp, _int, _vp, _vp, _vp, _vp, _vp, _int, _vp]),
    "gbsym_sn_destroy": (_int, [_vp]),
    "gbsym_sn_levels": (_int, [_vp, _vp, _vp]),
    "gbsym_sn_solve": (_int, [_vp, _vp, _int, _int, _vp]),
    "gbsym_sn_check": (_int, [_vp, _vp]),
    "gbsym_alloc": (_vp, [_sz]),
    "gbsym_sn_selftest_timeout": (_int, [_vp, _ll, _vp]),
    "gbsym_csr_create": (_int, [C.POINTER(_vp), _int, _int, _vp, _vp, _vp, _int, _int, _vp]),
    "gbsym_csr_destroy": (_int, [_vp]),
    "gbsym_csr_spmv": (_int, [_vp, _vp, _vp, _int, _vp]),
    "gbsym_csr_spmv_axpby": (_int, [_vp, _vp, _vp, _vp, _dbl, _dbl, _vp]),
    "gbsym_ilu0_device": (_int, [_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbsym_ic0_device": (_int, [_int, _vp, _vp, _vp, _vp]),
    "gbsym_pcg": (_int, [_vp, _vp, _vp, _vp, _vp, _dbl, _int, C.POINTER(KrylovResult), _vp]),
    "gbsym_gmres": (_int, [_vp, _vp, _vp, _vp, _vp, _int, _int, _dbl, C.POINTER(KrylovResult), _vp]),
    "gbsym_tri_adjoint": (_int, [_vp, _int, _vp, _vp, _vp, _vp, _int, _vp, _vp]),
    "gbsym_batch_create": (_int, [C.POINTER(_vp), _int, _vp, _vp, _vp, _vp, _int, _vp]),
    "gbsym_batch_destroy": (_int, [_vp]),
    "gbsym_batch_solve": (_int, [_vp, _vp, _int, _int, _vp]),
    "gbsym_batch_row_offsets": (_int, [_vp, _vp]),
    "gbsym_batch_create_kind": (_int, [C.POINTER(_vp), _int, _vp, _vp, _vp, _vp, _int, _int, _vp]),
    "gbsym_batch_autotune": (_int, [_vp, _int, _int, _vp, _pi]),
    "gbsym_batch_check": (_int, [_vp, _vp]),
    "gbsym_batch_get_info": (_int, [_vp, C.POINTER(TriInfo)]),
    "gbsym_batch_get_tuning": (_int, [_vp, _int, _pi]),
    "gbsym_tri_get_tuning": (_int, [_vp, _int, _pi]),
    "gbsym_sptrsv_csr_noalloc": (_int, [_int, _vp, _vp, _vp, _vp, _vp]),
}

_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libgbsym.so is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python sympiler_gb300/build.py`")
        L = C.CDLL(LIB_PATH, mode=C.RTLD_GLOBAL)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class GbsymError(RuntimeError):
    def __init__(self, status: int, where: str = ""):
        self.status = status
        msg = lib().gbsym_status_string(status).decode()
        super().__init__("%s: gbsym status %d (%s)" % (where, status, msg))


# status codes (include/gbsym.h)
OK, ERR_NULL_ARG, ERR_BAD_SCHEDULE, ERR_PIVOT, ERR_TIMEOUT, ERR_CUDA, ERR_BAD_MATRIX, ERR_SIZE, \
    ERR_NOT_CONVERGED, ERR_UNSUPPORTED = range(10)
LOWER_DIAG_LAST, UPPER_DIAG_FIRST, ILU_UNIT_LOWER, ILU_UPPER, ILU_LOWER_DIV, LOWER_CSC = range(6)
F64, F32 = 0, 1
COL_MAJOR, ROW_MAJOR = 0, 1
EXEC_AUTO, EXEC_LEVELSET, EXEC_SYNCFREE, EXEC_ONEBLOCK, EXEC_PERSISTENT, EXEC_CLUSTER, EXEC_PARTITIONED = range(7)
EXEC_NAMES = {EXEC_LEVELSET: "levelset", EXEC_SYNCFREE: "syncfree", EXEC_ONEBLOCK: "oneblock",
              EXEC_PERSISTENT: "persistent", EXEC_CLUSTER: "cluster", EXEC_PARTITIONED: "partitioned"}
ARITH_EXACT, ARITH_FUSED = 0, 1


def check(status: int, where: str = ""):
    if status != OK:
        raise GbsymError(status, where)
