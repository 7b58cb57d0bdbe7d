/*
 * ref_capi.cpp -- extern "C" entry points over the reference's own compiled
 * C++ (sympiler/sympiler, namespace sym_lib), so that Python tests can call
 * the unmodified reference executors through ctypes.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled together with the reference's source
 * files, in place, into the oracle's reference library by oracle/build.py.
 * The reference sources are not copied; this file only forwards calls.
 *
 * The supernodal solve phase (solve_phase_*.cpp) and the DFS reach need
 * BLAS/METIS and are not on the triangular-solve path; mgmres.cpp references
 * them from its LDL^T-preconditioned drivers, which are never called here.
 * They are defined below as stubs that abort, so the library links with no
 * undefined symbols.
 */
#include <omp.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sympiler/sparse_blas_lib.h"
#include "sympiler/parsy/gmres/mgmres.hpp"
#include "sympiler/parsy/triangularSolve/Triangular_CSC.h"
#include "sympiler/parsy/common/TreeUtils.h"
#include "sympiler/parsy/symbolic/InspectionLevel_06.h"
#include "sympiler/parsy/triangularSolve/Triangular_BCSC.h"

namespace sym_lib {
namespace parsy {
[[noreturn]] static void not_built(const char *what) {
  std::fprintf(stderr, "oracle reference library: %s is not built\n", what);
  std::abort();
}
int solve_phase_ldl(size_t, double *, double *, int *, int *, size_t *, int *,
                    double *, size_t *, size_t, int) {
  not_built("solve_phase_ldl");
}
int solve_phase_ldl_blocked(size_t, double *, double *, int *, int *, size_t *,
                            int *, double *, size_t *, size_t, int) {
  not_built("solve_phase_ldl_blocked");
}
int solve_phase_ldl_blocked_parallel(size_t, double *, double *, int *, int *,
                                     size_t *, int *, double *, size_t *,
                                     size_t, int, int, int *, int *, int,
                                     int *, int *, int) {
  not_built("solve_phase_ldl_blocked_parallel");
}
int solve_phase_ldl_blocked_parallel_permuted_update(
    size_t, double *, double *, int *, int *, size_t *, int *, double *,
    size_t *, size_t, int, int, int *, int *, int, int *, int *, int, int,
    int *, int *, bool *, int *, double *) {
  not_built("solve_phase_ldl_blocked_parallel_permuted_update");
}
int reach(int, int *, int *, int *, int *, int, int *, const int *) {
  not_built("reach");
}
}  // namespace parsy
}  // namespace sym_lib

using namespace sym_lib;

extern "C" {
void ref_sptrsv_csr(int n, int *Lp, int *Li, double *Lx, double *x) {
  sptrsv_csr(n, Lp, Li, Lx, x);
}
void ref_sptrsv_csr_ilu(int n, const int *Lp, const int *Li, const double *Lx,
                        const int *diags, double *x) {
  sptrsv_csr_ilu(n, Lp, Li, Lx, diags, x);
}
void ref_sptrsv_csr_levelset(int n, const int *Lp, const int *Li,
                             const double *Lx, double *x, int levels,
                             const int *levelPtr, const int *levelSet) {
  sptrsv_csr_levelset(n, Lp, Li, Lx, x, levels, levelPtr, levelSet);
}
void ref_sptrsv_csr_lbc(int n, int *Lp, int *Li, double *Lx, double *x,
                        int level_no, int *level_ptr, int *par_ptr,
                        int *partition) {
  sptrsv_csr_lbc(n, Lp, Li, Lx, x, level_no, level_ptr, par_ptr, partition);
}
void ref_sptrsv_csr_lbc_redundant(int n, int *Lp, int *Li, double *Lx,
                                  double *x, double *b, int level_no,
                                  int *level_ptr, int *par_ptr,
                                  int *partition, double *tmp) {
  sptrsv_csr_lbc_redundant(n, Lp, Li, Lx, x, b, level_no, level_ptr, par_ptr,
                           partition, tmp);
}
void ref_sptrsv_csr_ilu_lbc(int n, const int *Lp, const int *Li,
                            const double *Lx, const int *diags, double *x,
                            int level_no, const int *level_ptr,
                            const int *par_ptr, const int *partition) {
  sptrsv_csr_ilu_lbc(n, Lp, Li, Lx, diags, x, level_no, level_ptr, par_ptr,
                     partition);
}
void ref_sptrsv_csc(int n, int *Lp, int *Li, double *Lx, double *x) {
  sptrsv_csc(n, Lp, Li, Lx, x);
}
void ref_sptrsv_csc_levelset(int n, int *Lp, int *Li, double *Lx, double *x,
                             int levels, const int *levelptr,
                             const int *levelset) {
  sptrsv_csc_levelset(n, Lp, Li, Lx, x, levels, levelptr, levelset);
}
void ref_sptrsv_csc_lbc(int n, int *Lp, int *Li, double *Lx, double *x,
                        int level_no, int *level_ptr, int *par_ptr,
                        int *partition) {
  sptrsv_csc_lbc(n, Lp, Li, Lx, x, level_no, level_ptr, par_ptr, partition);
}
int ref_ltsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  return ltsolve(n, Lp, Li, Lx, x);
}
int ref_parsy_lsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  return parsy::lsolve(n, Lp, Li, Lx, x);
}
int ref_parsy_ltsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  return parsy::ltsolve(n, Lp, Li, Lx, x);
}
int ref_parsy_lsolvePar(int n, int *Lp, int *Li, double *Lx, double *x,
                        int levels, int *levelPtr, int *levelSet, int chunk) {
  return parsy::lsolvePar(n, Lp, Li, Lx, x, levels, levelPtr, levelSet, chunk);
}
int ref_parsy_lsolveParH2(int n, int *Lp, int *Li, double *Lx, double *x,
                          int levels, int *levelPtr, int *levelSet, int parts,
                          int *parPtr, int *partition, int chunk) {
  return parsy::lsolveParH2(n, Lp, Li, Lx, x, levels, levelPtr, levelSet,
                            parts, parPtr, partition, chunk);
}
void ref_spmv_csr(int n, const int *Ap, const int *Ai, const double *Ax,
                  const double *x, double *y) {
  spmv_csr(n, Ap, Ai, Ax, x, y);
}
void ref_spmv_csr_axpby(int n, const int *Ap, const int *Ai, const double *Ax,
                        const double *x, const double *y, double *z, double a,
                        double b) {
  spmv_csr(n, Ap, Ai, Ax, x, y, z, a, b);
}
void ref_spmv_csr_parallel(int n, const int *Ap, const int *Ai,
                           const double *Ax, const double *x, double *y) {
  spmv_csr_parallel(n, Ap, Ai, Ax, x, y);
}
void ref_spilu0_csr(int n, int nnz, const int *Ap, const int *Ai,
                    const double *Ax, const int *A_diag, double *l) {
  spilu0_csr(n, nnz, Ap, Ai, Ax, A_diag, l);
}
void ref_spic0_csr(int n, double *val, int *rowPtr, int *rowIdx) {
  spic0_csr(n, val, rowPtr, rowIdx);
}
// The reference's per-thread scratch: n ints per OpenMP thread (its thread
// number picks the slice), all -1, as its header asks.
void ref_spilu0_csr_lbc(int n, int nnz, const int *Ap, const int *Ai,
                        const double *Ax, const int *A_diag, double *l,
                        int level_no, const int *level_ptr, const int *par_ptr,
                        const int *partition) {
  std::vector<int> tmp((size_t)n * (omp_get_max_threads() + 1), -1);
  spilu0_csr_lbc(n, nnz, Ap, Ai, Ax, A_diag, l, level_no, level_ptr, par_ptr,
                 partition, tmp.data());
}
void ref_spic0_csr_lbc(int n, double *val, int *rowPtr, int *colIdx,
                       int level_no, int *level_ptr, int *par_ptr,
                       int *partition) {
  spic0_csr_lbc(n, val, rowPtr, colIdx, level_no, level_ptr, par_ptr, partition);
}
void ref_lus_cr(int n, int nz_num, int *ia, int *ja, double *l, int *ua,
                double *r, double *z) {
  parsy::lus_cr(n, nz_num, ia, ja, l, ua, r, z);
}
int ref_tree_levelset(int n, const int *tree, int *levelPtr, int *levelSet) {
  return parsy::getLevelSet((size_t)n, tree, levelPtr, levelSet);
}
/* parsy::getCoarseLevelSet_6 with the output arrays it allocates copied into
 * caller buffers of n+1 slots each, then released. */
int ref_coarse_levelset6(int n, const int *eTree, int innerParts,
                         int minLevelDist, int divRate, double *nodeCost,
                         int *level_ptr, int *part_ptr, int *node_ptr,
                         int *part_no_out) {
  int finaLevelNo = 0, partNo = 0;
  int *finaLevelPtr = nullptr, *parLevelSet = nullptr, *finalPartPtr = nullptr,
      *finalNodePtr = nullptr;
  int *blk2col = new int[n + 1];
  for (int i = 0; i <= n; i++) blk2col[i] = i;
  parsy::getCoarseLevelSet_6((size_t)n, eTree, blk2col, finaLevelNo,
                             finaLevelPtr, parLevelSet, partNo, finalPartPtr,
                             finalNodePtr, innerParts, minLevelDist, divRate,
                             nodeCost);
  for (int i = 0; i <= finaLevelNo; i++) level_ptr[i] = finaLevelPtr[i];
  for (int i = 0; i <= partNo; i++) part_ptr[i] = finalPartPtr[i];
  for (int i = 0; i < n; i++) node_ptr[i] = finalNodePtr[i];
  *part_no_out = partNo;
  delete[] blk2col;
  delete[] finaLevelPtr;
  delete[] finalPartPtr;
  delete[] finalNodePtr;
  delete[] parLevelSet;
  return finaLevelNo;
}

/* Supernodal (blocked CSC) forward solves, built with the reference's own
 * dense kernels (SYM_BLAS).  Their multi-right-hand-side forms call an
 * external BLAS, which is not built here: those calls land in
 * ref_blas_missing and abort. */
int ref_blocked_lsolve(int n, size_t *Lp, int *Li, double *Lx, size_t *Li_ptr,
                       int *col2sup, int *sup2col, int supNo, double *x) {
  return parsy::blockedLsolve(n, Lp, Li, Lx, 0, Li_ptr, col2sup, sup2col, supNo, x);
}
int ref_leveled_blocked_lsolve(int n, size_t *Lp, int *Li, double *Lx,
                               size_t *Li_ptr, int *col2sup, int *sup2col,
                               int supNo, double *x, int levels, int *levelPtr,
                               int *levelSet) {
  return parsy::leveledBlockedLsolve(n, Lp, Li, Lx, 0, Li_ptr, col2sup, sup2col,
                                     supNo, x, levels, levelPtr, levelSet, 1);
}
int ref_h2_leveled_blocked_lsolve(int n, size_t *Lp, int *Li, double *Lx,
                                  size_t *Li_ptr, int *col2sup, int *sup2col,
                                  int supNo, double *x, int levels,
                                  int *levelPtr, int *levelSet, int parts,
                                  int *parPtr, int *partition) {
  return parsy::H2LeveledBlockedLsolve(n, Lp, Li, Lx, 0, Li_ptr, col2sup, sup2col,
                                       supNo, x, levels, levelPtr, levelSet,
                                       parts, parPtr, partition, 1);
}
void ref_blas_missing(...) {
  std::fprintf(stderr, "reference build: external BLAS routine called (not built)\n");
  std::abort();
}
}
