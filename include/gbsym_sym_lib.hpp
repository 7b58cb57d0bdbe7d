// gbsym_sym_lib.hpp -- drop-in for the triangular-solve path of the
// reference's C++ API (include/sympiler/sparse_blas_lib.h, namespace
// sym_lib; include/sympiler/parsy/triangularSolve/Triangular_CSC.h and
// include/sympiler/parsy/gmres/mgmres.hpp, namespace sym_lib::parsy).
//
// A caller that included those headers includes this one instead and links
// libgbsym.so in place of the reference's sparse_blas objects: the
// signatures, argument meanings and in-place behaviour are the reference's,
// the work runs on the GPU.  The void functions never abort; their status
// is available from gbsym_last_error().
//
// build_levelSet_CSC stands in for the reference's (unvendored) aggregation
// dependency at its call sites (Catch_tests/sptrsv_tests.cpp:59,
// demo/sptrsv_demo_utils.h:42-45): it returns arrays allocated with new[],
// which those callers release with delete[].
#ifndef GBSYM_SYM_LIB_HPP
#define GBSYM_SYM_LIB_HPP

#include <cstddef>
#include <cstring>

#include "gbsym.h"

namespace sym_lib {

// ---- SpMV (sparse_blas_lib.h:19-37) ----------------------------------------
inline void spmv_csr(int n, const int *Ap, const int *Ai, const double *Ax, const double *x,
                     double *y) {
  gbsym_spmv_csr(n, Ap, Ai, Ax, x, y);
}
inline void spmv_csr(int n, const int *Ap, const int *Ai, const double *Ax, const double *x,
                     const double *y, double *z, double a, double b) {
  gbsym_spmv_csr_axpby(n, Ap, Ai, Ax, x, y, z, a, b);
}
inline void spmv_csr_parallel(int n, const int *Ap, const int *Ai, const double *Ax,
                              const double *x, double *y) {
  gbsym_spmv_csr_parallel(n, Ap, Ai, Ax, x, y);
}

// ---- SpTRSV, CSR (sparse_blas_lib.h:126-161) ---------------------------------
inline void sptrsv_csr(int n, int *Lp, int *Li, double *Lx, double *x) {
  gbsym_sptrsv_csr(n, Lp, Li, Lx, x);
}
inline void sptrsv_csr_ilu(int n, const int *Lp, const int *Li, const double *Lx,
                           const int *diags, double *x) {
  gbsym_sptrsv_csr_ilu(n, Lp, Li, Lx, diags, x);
}
inline void sptrsv_csr_ilu_lbc(int n, const int *Lp, const int *Li, const double *Lx,
                               const int *diags, double *x, const int level_no,
                               const int *level_ptr, const int *par_ptr, const int *partition) {
  gbsym_sptrsv_csr_ilu_lbc(n, Lp, Li, Lx, diags, x, level_no, level_ptr, par_ptr, partition);
}
inline void sptrsv_csr_levelset(int n, const int *Lp, const int *Li, const double *Lx, double *x,
                                int levels, const int *levelPtr, const int *levelSet) {
  gbsym_sptrsv_csr_levelset(n, Lp, Li, Lx, x, levels, levelPtr, levelSet);
}
inline void sptrsv_csr_lbc(int n, int *Lp, int *Li, double *Lx, double *x, int level_no,
                           int *level_ptr, int *par_ptr, int *partition) {
  gbsym_sptrsv_csr_lbc(n, Lp, Li, Lx, x, level_no, level_ptr, par_ptr, partition);
}
inline void sptrsv_csr_lbc_redundant(int n, int *Lp, int *Li, double *Lx, double *x, double *b,
                                     int level_no, int *level_ptr, int *par_ptr, int *partition,
                                     double *tmp) {
  gbsym_sptrsv_csr_lbc_redundant(n, Lp, Li, Lx, x, b, level_no, level_ptr, par_ptr, partition, tmp);
}

// ---- SpTRSV, CSC (sparse_blas_lib.h:170-178, 330) ------------------------------
inline void sptrsv_csc(int n, int *Lp, int *Li, double *Lx, double *x) {
  gbsym_sptrsv_csc(n, Lp, Li, Lx, x);
}
inline void sptrsv_csc_levelset(int n, int *Lp, int *Li, double *Lx, double *x, int levels,
                                const int *levelptr, const int *levelset) {
  gbsym_sptrsv_csc_levelset(n, Lp, Li, Lx, x, levels, levelptr, levelset);
}
inline void sptrsv_csc_lbc(int n, int *Lp, int *Li, double *Lx, double *x, int level_no,
                           int *level_ptr, int *par_ptr, int *partition) {
  gbsym_sptrsv_csc_lbc(n, Lp, Li, Lx, x, level_no, level_ptr, par_ptr, partition);
}
inline int ltsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  return gbsym_ltsolve(n, Lp, Li, Lx, x);
}

// ---- factor producers (sparse_blas_lib.h:242-245, 276-282) ------------------------
inline void spic0_csr(int n, double *val, int *rowPtr, int *rowIdx) {
  gbsym_spic0_csr(n, val, rowPtr, rowIdx);
}
inline void spilu0_csr(int n, int nnz, const int *Ap, const int *Ai, const double *Ax,
                       const int *A_diag, double *l) {
  gbsym_spilu0_csr(n, nnz, Ap, Ai, Ax, A_diag, l);
}
inline void spic0_csr_lbc(int n, double *val, int *rowPtr, int *colIdx, int level_no,
                          int *level_ptr, int *par_ptr, int *partition) {
  gbsym_spic0_csr_lbc(n, val, rowPtr, colIdx, level_no, level_ptr, par_ptr, partition);
}
inline void spilu0_csr_lbc(int n, int nnz, const int *Ap, const int *Ai, const double *Ax,
                           const int *A_diag, double *l, int level_no, const int *level_ptr,
                           const int *par_ptr, const int *partition, int *tempvecs) {
  gbsym_spilu0_csr_lbc(n, nnz, Ap, Ai, Ax, A_diag, l, level_no, level_ptr, par_ptr, partition,
                       tempvecs);
}

// ---- schedule builder at the reference's build_levelSet_CSC call sites ------------
inline int build_levelSet_CSC(size_t n, const int *Lp, const int *Li, int *&levelPtr,
                              int *&levelSet) {
  int *lp = nullptr, *ls = nullptr;
  const int nl = gbsym_build_levelset_csc((int)n, Lp, Li, &lp, &ls);
  levelPtr = nullptr;
  levelSet = nullptr;
  if (nl < 0) return nl;
  levelPtr = new int[nl + 1];
  levelSet = new int[n > 0 ? n : 1];
  std::memcpy(levelPtr, lp, sizeof(int) * (size_t)(nl + 1));
  if (n) std::memcpy(levelSet, ls, sizeof(int) * n);
  gbsym_free(lp);
  gbsym_free(ls);
  return nl;
}

namespace detail {
// Copy an LBC result from gbsym_free'd buffers into new[] arrays sized as
// the reference sizes them (level and part pointers n+1, nodes n).
inline void lbc_to_new(size_t n, int st, int nl, int *lp, int np, int *pp, int *nd, int &level_no,
                       int *&level_ptr, int &part_no, int *&part_ptr, int *&node_ptr) {
  level_ptr = new int[n + 1]();
  part_ptr = new int[n + 1]();
  node_ptr = new int[n > 0 ? n : 1]();
  level_no = 0;
  part_no = 0;
  if (st == GBSYM_OK && n > 0) {
    level_no = nl;
    part_no = np;
    std::memcpy(level_ptr, lp, sizeof(int) * (size_t)(nl + 1));
    std::memcpy(part_ptr, pp, sizeof(int) * (size_t)(np + 1));
    std::memcpy(node_ptr, nd, sizeof(int) * n);
  }
  gbsym_free(lp);
  gbsym_free(pp);
  gbsym_free(nd);
}
}  // namespace detail

// LBC of the solve DAG of a lower CSR, at the reference demo's call site
// (demo/sptrsv_demo_utils.h:78-90; the function belongs to the unvendored
// aggregation dependency).  lp = parts per coarse level, cp = minimum level
// distance, ic = division rate; stype is unused.  Outputs are new[] arrays.
inline int get_coarse_levelSet_DAG_CSC_tree(size_t n, const int *Lp, const int *Li, int /*stype*/,
                                            int &final_level_no, int *&fina_level_ptr, int &part_no,
                                            int *&final_part_ptr, int *&final_node_ptr, int lp, int cp,
                                            int ic, double *cost) {
  int nl = 0, np = 0, *a = nullptr, *b = nullptr, *c = nullptr;
  const int st = gbsym_build_lbc((int)n, Lp, Li, cost, lp, cp, ic, &nl, &a, &np, &b, &c);
  detail::lbc_to_new(n, st, nl, a, np, b, c, final_level_no, fina_level_ptr, part_no, final_part_ptr,
                     final_node_ptr);
  return st == GBSYM_OK ? final_level_no : -st;
}

namespace parsy {
// TreeUtils.h getLevelSet (TreeUtils.cpp:89-140): caller-allocated arrays.
inline int getLevelSet(size_t n, const int *inTree, int *levelPtr, int *levelSet) {
  return gbsym_tree_levelset((int)n, inTree, levelPtr, levelSet);
}
// InspectionLevel_06.h:13 (InspectionLevel_06.cpp:17-400); blk2col and
// parLevelSet are unused, as in the reference.
inline int getCoarseLevelSet_6(size_t n, const int *eTree, const int * /*blk2col*/, int &finaLevelNo,
                               int *&finaLevelPtr, int *& /*parLevelSet*/, int &partNo, int *&finalPartPtr,
                               int *&finalNodePtr, int innerParts, int minLevelDist, int divRate,
                               double *nodeCost) {
  int nl = 0, np = 0, *a = nullptr, *b = nullptr, *c = nullptr;
  const int st = gbsym_coarse_levelset_tree((int)n, eTree, nodeCost, innerParts, minLevelDist, divRate, &nl,
                                            &a, &np, &b, &c);
  detail::lbc_to_new(n, st, nl, a, np, b, c, finaLevelNo, finaLevelPtr, partNo, finalPartPtr, finalNodePtr);
  return finaLevelNo;
}
// Triangular_CSC.h:14-36
inline int lsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  return gbsym_parsy_lsolve(n, Lp, Li, Lx, x);
}
inline int ltsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  return gbsym_parsy_ltsolve(n, Lp, Li, Lx, x);
}
inline int lsolvePar(int n, int *Lp, int *Li, double *Lx, double *x, int levels, int *levelPtr,
                     int *levelSet, int chunk) {
  return gbsym_parsy_lsolvePar(n, Lp, Li, Lx, x, levels, levelPtr, levelSet, chunk);
}
inline int lsolveParH2(int n, int *Lp, int *Li, double *Lx, double *x, int levels, int *levelPtr,
                       int *levelSet, int parts, int *parPtr, int *partition, int chunk) {
  return gbsym_parsy_lsolveParH2(n, Lp, Li, Lx, x, levels, levelPtr, levelSet, parts, parPtr,
                                 partition, chunk);
}
// Triangular_BCSC.h: supernodal (blocked CSC) solves
inline int blockedLsolve(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr, int *col2sup,
                         int *sup2col, int supNo, double *x) {
  return gbsym_parsy_blockedLsolve(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x);
}
inline int blockedLsolve_mrhs(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr, int *col2sup,
                              int *sup2col, int supNo, double *x, int n_rhs, int max_col = -1) {
  return gbsym_parsy_blockedLsolve_mrhs(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x, n_rhs, max_col);
}
inline int blockedLTsolve(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr, int *col2sup,
                          int *sup2col, int supNo, double *x) {
  return gbsym_parsy_blockedLTsolve(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x);
}
inline int blockedLTsolve_mrhs(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr, int *col2sup,
                               int *sup2col, int supNo, double *x, int m_rhs, int max_col = -1) {
  return gbsym_parsy_blockedLTsolve_mrhs(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x, m_rhs, max_col);
}
inline int leveledBlockedLsolve(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr, int *col2sup,
                                int *sup2col, int supNo, double *x, int levels, int *levelPtr, int *levelSet,
                                int chunk) {
  return gbsym_parsy_leveledBlockedLsolve(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x, levels,
                                          levelPtr, levelSet, chunk);
}
inline int H2LeveledBlockedLsolve(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr, int *col2sup,
                                  int *sup2col, int supNo, double *x, int levels, int *levelPtr, int *levelSet,
                                  int parts, int *parPtr, int *partition, int chunk) {
  return gbsym_parsy_H2LeveledBlockedLsolve(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x, levels,
                                            levelPtr, levelSet, parts, parPtr, partition, chunk);
}
inline int H2LeveledBlockedLTsolve(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr, int *col2sup,
                                   int *sup2col, int supNo, double *x, int levels, int *levelPtr, int *levelSet,
                                   int parts, int *parPtr, int *partition, int chunk) {
  return gbsym_parsy_H2LeveledBlockedLTsolve(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x, levels,
                                             levelPtr, levelSet, parts, parPtr, partition, chunk);
}
inline int H2LeveledBlockedLsolve_mrhs(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr,
                                       int *col2sup, int *sup2col, int supNo, double *x, int n_rhs, int levels,
                                       int *levelPtr, int *levelSet, int parts, int *parPtr, int *partition,
                                       int chunk, int max_col = -1) {
  return gbsym_parsy_H2LeveledBlockedLsolve_mrhs(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x, n_rhs,
                                                 levels, levelPtr, levelSet, parts, parPtr, partition, chunk,
                                                 max_col);
}
inline int H2LeveledBlockedLTsolve_mrhs(int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr,
                                        int *col2sup, int *sup2col, int supNo, double *x, int m_rhs, int levels,
                                        int *levelPtr, int *levelSet, int parts, int *parPtr, int *partition,
                                        int chunk, int max_col = -1) {
  return gbsym_parsy_H2LeveledBlockedLTsolve_mrhs(n, Lp, Li, Lx, NNZ, Li_ptr, col2sup, sup2col, supNo, x, m_rhs,
                                                  levels, levelPtr, levelSet, parts, parPtr, partition, chunk,
                                                  max_col);
}
// linear_solver/solve_phase.h:21-29
inline void solve_phase_simplicial_ll(int n, int *Lp, int *Li, double *Lx, double *x) {
  gbsym_parsy_solve_phase_simplicial_ll(n, Lp, Li, Lx, x);
}
inline void solve_phase_simplicial_ldl(int n, int *Lp, int *Li, double *Lx, double *d_val, double *x) {
  gbsym_parsy_solve_phase_simplicial_ldl(n, Lp, Li, Lx, d_val, x);
}
// linear_solver/solve_phase.h:35-62
inline void solve_phase_ll_blocked(size_t n, double *x, int *col2sup, int *sup2col, size_t *newCol, int *newRow,
                                   double *newVal, size_t *rowP, size_t nBlocks, int nnz) {
  gbsym_parsy_solve_phase_ll_blocked(n, x, col2sup, sup2col, newCol, newRow, newVal, rowP, nBlocks, nnz);
}
inline void solve_phase_ll_blocked_nrhs(size_t n, double *x, int n_rhs, int *col2sup, int *sup2col, size_t *newCol,
                                        int *newRow, double *newVal, size_t *rowP, size_t nBlocks, int nnz,
                                        int max_col) {
  gbsym_parsy_solve_phase_ll_blocked_nrhs(n, x, n_rhs, col2sup, sup2col, newCol, newRow, newVal, rowP, nBlocks, nnz,
                                          max_col);
}
inline void solve_phase_ll_blocked_parallel(size_t n, double *x, int *col2sup, int *sup2col, size_t *newCol,
                                            int *newRow, double *newVal, size_t *rowP, size_t nBlocks, int nnz,
                                            int levels, int *levelPtr, int *levelSet, int parts, int *parPtr,
                                            int *partition, int chunk) {
  gbsym_parsy_solve_phase_ll_blocked_parallel(n, x, col2sup, sup2col, newCol, newRow, newVal, rowP, nBlocks, nnz,
                                              levels, levelPtr, levelSet, parts, parPtr, partition, chunk);
}
inline void solve_phase_ll_blocked_parallel_nrhs(size_t n, double *x, int n_rhs, int *col2sup, int *sup2col,
                                                 size_t *newCol, int *newRow, double *newVal, size_t *rowP,
                                                 size_t nBlocks, int nnz, int levels, int *levelPtr, int *levelSet,
                                                 int parts, int *parPtr, int *partition, int chunk, int max_col) {
  gbsym_parsy_solve_phase_ll_blocked_parallel_nrhs(n, x, n_rhs, col2sup, sup2col, newCol, newRow, newVal, rowP,
                                                   nBlocks, nnz, levels, levelPtr, levelSet, parts, parPtr,
                                                   partition, chunk, max_col);
}
inline void solve_phase_ldl(size_t n, double *d_val, double *x, int *col2sup, int *sup2col, size_t *newCol,
                            int *newRow, double *newVal, size_t *rowP, size_t nBlocks, int nnz) {
  gbsym_parsy_solve_phase_ldl(n, d_val, x, col2sup, sup2col, newCol, newRow, newVal, rowP, nBlocks, nnz);
}
// mgmres.hpp:41
inline void lus_cr(int n, int nz_num, int ia[], int ja[], double l[], int ua[], double r[],
                   double z[]) {
  gbsym_parsy_lus_cr(n, nz_num, ia, ja, l, ua, r, z);
}
}  // namespace parsy

}  // namespace sym_lib

#endif
