/*
 * gbsym.h -- C ABI of the GB300 sparse triangular-solve executor.
 *
 * Two layers:
 *
 *  1. Drop-ins.  One `gbsym_*` function per reference function on the
 *     triangular-solve path of sympiler/sympiler, with the reference's
 *     argument list, argument meaning and in-place behaviour.  All arrays are
 *     caller-owned HOST memory; the call uploads, runs on the current CUDA
 *     device, downloads and returns when the result is in the caller's
 *     buffer.  `void` drop-ins record their status for gbsym_last_error();
 *     they never abort.  The reference function each one replaces is cited
 *     beside it (paths inside the sympiler source tree).
 *
 *  2. Plans.  Device-resident operators (level-packed triangles, CSR
 *     matrices) built once and applied many times on a caller stream, with
 *     device pointers; the Krylov drivers, the adjoint and the batched
 *     executor sit on top of them.  A `void *stream` argument is a
 *     cudaStream_t; NULL means the CUDA default (legacy) stream.
 *
 * Conventions shared with the reference:
 *   - int32 CSR/CSC arrays; lower-triangular CSR has the diagonal LAST in
 *     each row, lower-triangular CSC has it FIRST in each column;
 *   - the right-hand side is passed in x and overwritten by the solution;
 *   - multi-RHS arrays are column-major n x k (x[i + j*n]), as in
 *     SolverSettings::solve_only (sparse_blas/parsy/cholesky_solver.cpp:
 *     805-813); plans also accept row-major n x k (x[i*k + j]), which is the
 *     layout the executor computes in.
 *
 * Floating point: every row of every solve and product is accumulated in
 * the reference's storage order with separately rounded multiply and
 * subtract (no fused multiply-add) and a correctly rounded division, so
 * FP64 results are bit-identical to the reference compiled without
 * floating-point contraction, whatever the row lengths.  The opt-in fused
 * arithmetic of gbsym_tri_set_arith is the one exception.
 */
#ifndef GBSYM_H
#define GBSYM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ------------------------------------------------------------ */
enum gbsym_status {
  GBSYM_OK = 0,
  GBSYM_ERR_NULL_ARG = 1,      /* a required pointer is NULL               */
  GBSYM_ERR_BAD_SCHEDULE = 2,  /* level/partition arrays violate the DAG   */
  GBSYM_ERR_PIVOT = 3,         /* zero/non-positive pivot in a factor      */
  GBSYM_ERR_TIMEOUT = 4,       /* a bounded device wait gave up            */
  GBSYM_ERR_CUDA = 5,          /* a CUDA runtime call failed               */
  GBSYM_ERR_BAD_MATRIX = 6,    /* malformed CSR/CSC (bounds, diagonal)     */
  GBSYM_ERR_SIZE = 7,          /* size argument out of range               */
  GBSYM_ERR_NOT_CONVERGED = 8, /* Krylov driver hit its iteration limit    */
  GBSYM_ERR_UNSUPPORTED = 9    /* option combination not implemented       */
};

/* Status of the most recent drop-in call on this host thread. */
int gbsym_last_error(void);
const char *gbsym_status_string(int status);
/* Host buffers returned by the schedule builders; release with gbsym_free.
 * gbsym_alloc gives a buffer of the same kind (NULL for 0 bytes or when
 * memory is exhausted), for callers that hand buffers back to the library's
 * owner conventions. */
void *gbsym_alloc(size_t bytes);
void gbsym_free(void *p);
/* Number of kernels this library has launched in this process so far. */
unsigned long long gbsym_kernel_launches(void);

/* Drop-in plan cache.  No counterpart in the reference: its executors keep
 * nothing between calls, while a drop-in here uploads the matrix, checks it
 * and builds a plan on every call.  capacity > 0 lets the drop-ins keep up
 * to that many plans (least recently used evicted), keyed by the device,
 * the matrix kind, n, the entry count, the array pointers (values,
 * indices, diagonal pointers, schedule arrays) and the caller's version;
 * a later call with the same key reuses the plan and uploads only x.  The
 * cache checks nothing else: whenever the caller changes a cached matrix's
 * arrays in place it must pass a new version to
 * gbsym_dropin_cache_version, which drops every cached plan.  capacity 0
 * (the default) turns the cache off and frees the plans not in use.
 * Returns GBSYM_ERR_SIZE for a negative capacity. */
int gbsym_dropin_cache(int capacity);
void gbsym_dropin_cache_version(unsigned long long version);

/* ---- drop-ins: SpTRSV, CSR row-pull ------------------------------------- */
/* sparse_blas/sptrsv.cpp:17-25 ; include/sympiler/sparse_blas_lib.h:126-127 */
void gbsym_sptrsv_csr(int n, int *Lp, int *Li, double *Lx, double *x);
/* sparse_blas/sptrsv.cpp:28-37 ; sparse_blas_lib.h:137 (unit lower, no divide) */
void gbsym_sptrsv_csr_ilu(int n, const int *Lp, const int *Li, const double *Lx,
                          const int *diags, double *x);
/* sparse_blas/sptrsv.cpp:109-127 ; sparse_blas_lib.h:139-141 (divides by Lx[diags[i]]) */
void gbsym_sptrsv_csr_ilu_lbc(int n, const int *Lp, const int *Li,
                              const double *Lx, const int *diags, double *x,
                              const int level_no, const int *level_ptr,
                              const int *par_ptr, const int *partition);
/* sparse_blas/sptrsv.cpp:40-55 ; sparse_blas_lib.h:146-148 */
void gbsym_sptrsv_csr_levelset(int n, const int *Lp, const int *Li,
                               const double *Lx, double *x, int levels,
                               const int *levelPtr, const int *levelSet);
/* sparse_blas/sptrsv.cpp:57-76 ; sparse_blas_lib.h:151-153 */
void gbsym_sptrsv_csr_lbc(int n, int *Lp, int *Li, double *Lx, double *x,
                          int level_no, int *level_ptr, int *par_ptr,
                          int *partition);
/* sparse_blas/sptrsv.cpp:78-107 ; sparse_blas_lib.h:157-161.  tmp is the
 * reference's per-thread scratch; it is not read and not written here. */
void gbsym_sptrsv_csr_lbc_redundant(int n, int *Lp, int *Li, double *Lx,
                                    double *x, double *b, int level_no,
                                    int *level_ptr, int *par_ptr,
                                    int *partition, double *tmp);

/* ---- drop-ins: SpTRSV, CSC ---------------------------------------------- */
/* sparse_blas/sptrsv.cpp:129-137 ; sparse_blas_lib.h:170 */
void gbsym_sptrsv_csc(int n, int *Lp, int *Li, double *Lx, double *x);
/* sparse_blas/sptrsv.cpp:139-156 ; sparse_blas_lib.h:174-175 */
void gbsym_sptrsv_csc_levelset(int n, int *Lp, int *Li, double *Lx, double *x,
                               int levels, const int *levelptr,
                               const int *levelset);
/* sparse_blas/sptrsv.cpp:158-174 ; sparse_blas_lib.h:177-178 */
void gbsym_sptrsv_csc_lbc(int n, int *Lp, int *Li, double *Lx, double *x,
                          int level_no, int *level_ptr, int *par_ptr,
                          int *partition);
/* sparse_blas/sptrsv_lt.cpp:11-20 ; sparse_blas_lib.h:330.  L^T x = b on the
 * CSC of L.  Returns 0 on NULL input, 1 on success (as the reference). */
int gbsym_ltsolve(int n, int *Lp, int *Li, double *Lx, double *x);
/* sparse_blas/parsy/triangularSolve/Triangular_CSC.cpp:18-28, 30-40, 57-76,
 * 78-101 ; include/sympiler/parsy/triangularSolve/Triangular_CSC.h */
int gbsym_parsy_lsolve(int n, int *Lp, int *Li, double *Lx, double *x);
int gbsym_parsy_ltsolve(int n, int *Lp, int *Li, double *Lx, double *x);
int gbsym_parsy_lsolvePar(int n, int *Lp, int *Li, double *Lx, double *x,
                          int levels, int *levelPtr, int *levelSet, int chunk);
int gbsym_parsy_lsolveParH2(int n, int *Lp, int *Li, double *Lx, double *x,
                            int levels, int *levelPtr, int *levelSet,
                            int parts, int *parPtr, int *partition, int chunk);

/* ---- drop-ins: SpMV ------------------------------------------------------ */
/* sparse_blas/spmv.cpp:12-21 ; sparse_blas_lib.h:19-20 */
void gbsym_spmv_csr(int n, const int *Ap, const int *Ai, const double *Ax,
                    const double *x, double *y);
/* sparse_blas/spmv.cpp:23-34 ; sparse_blas_lib.h:32-33.  z += A x (z is NOT
 * cleared), then z = a z + b y. */
void gbsym_spmv_csr_axpby(int n, const int *Ap, const int *Ai, const double *Ax,
                          const double *x, const double *y, double *z,
                          double a, double b);
/* sparse_blas/spmv.cpp:37-57 ; sparse_blas_lib.h:36-37 */
void gbsym_spmv_csr_parallel(int n, const int *Ap, const int *Ai,
                             const double *Ax, const double *x, double *y);

/* ---- drop-ins: factor producers and the ILU apply ----------------------- */
/* sparse_blas/spilu0.cpp:11-51 ; sparse_blas_lib.h:276-277 */
void gbsym_spilu0_csr(int n, int nnz, const int *Ap, const int *Ai,
                      const double *Ax, const int *A_diag, double *l);
/* sparse_blas/spic0.cpp:106-128 ; sparse_blas_lib.h:242 (upper CSR of A, in place) */
void gbsym_spic0_csr(int n, double *val, int *rowPtr, int *rowIdx);
/* sparse_blas/spilu0.cpp:54-106 ; sparse_blas_lib.h:279-282.  The LBC
 * schedule (level_ptr into par_ptr into partition) is validated against
 * the dependencies of the rows (entries left of each diagonal); an invalid
 * one records GBSYM_ERR_BAD_SCHEDULE and leaves l untouched.  ILU0's row
 * sequence does not depend on the schedule, so l equals gbsym_spilu0_csr's
 * bit for bit.  tempvecs (the reference's per-thread scratch) is not used. */
void gbsym_spilu0_csr_lbc(int n, int nnz, const int *Ap, const int *Ai,
                          const double *Ax, const int *A_diag, double *l,
                          int level_no, const int *level_ptr,
                          const int *par_ptr, const int *partition,
                          int *tempvecs);
/* sparse_blas/spic0.cpp:130-160 ; sparse_blas_lib.h:243-245.  The schedule
 * is over the columns of L (rows of the upper CSR) and is validated against
 * the solve DAG of L.  The reference subtracts under `omp atomic`, so its
 * result depends on thread timing; this one applies every update in
 * gbsym_spic0_csr's (serial) order and equals it bit for bit. */
void gbsym_spic0_csr_lbc(int n, double *val, int *rowPtr, int *colIdx,
                         int level_no, int *level_ptr, int *par_ptr,
                         int *partition);
/* sparse_blas/parsy/gmres/mgmres.cpp:598-689 ; include/sympiler/parsy/gmres/mgmres.hpp:41 */
void gbsym_parsy_lus_cr(int n, int nz_num, int *ia, int *ja, double *l,
                        int *ua, double *r, double *z);

/* ---- drop-ins: schedule builders ---------------------------------------- */
/* Replaces build_levelSet_CSC of the reference's `aggregation` dependency
 * (call sites Catch_tests/sptrsv_tests.cpp:59, demo/sptrsv_demo_utils.h:
 * 42-45).  Computed on the GPU.  level(i) = 0 without off-diagonals, else
 * 1 + max level of its dependencies; rows ascending inside each level.
 * *level_ptr (level_no+1 ints) and *level_set (n ints) are allocated here;
 * release them with gbsym_free.  Returns level_no, or -status on error. */
int gbsym_build_levelset_csc(int n, const int *Lp, const int *Li,
                             int **level_ptr, int **level_set);
/* The same DAG read from the CSR of L (diagonal last). */
int gbsym_build_levelset_csr(int n, const int *Lp, const int *Li,
                             int **level_ptr, int **level_set);
/* Level set of the backward solve on an upper CSR (diagonal first). */
int gbsym_build_levelset_upper_csr(int n, const int *Up, const int *Ui,
                                   int **level_ptr, int **level_set);

/* LBC schedule inspectors (host code; no GPU needed).  Their outputs feed
 * gbsym_sptrsv_csr_lbc / _ilu_lbc / _lbc_redundant / _csc_lbc and
 * gbsym_parsy_lsolveParH2: level_ptr[level_no+1] indexes part_ptr,
 * part_ptr[part_no+1] indexes node_ptr[n].
 *
 * Replaces parsy::getLevelSet (sparse_blas/parsy/common/TreeUtils.cpp:89-140):
 * level set of a forest (parent[v] > v, or -1 for a root), leaves first,
 * ascending index within a level.  level_ptr (n+1 ints) and level_set (n
 * ints) are caller-allocated, as in the reference.  Returns level_no, or
 * -status. */
int gbsym_tree_levelset(int n, const int *parent, int *level_ptr, int *level_set);
/* Replaces parsy::getCoarseLevelSet_6
 * (sparse_blas/parsy/symbolic/InspectionLevel_06.cpp:17-400): tree LBC of a
 * forest with per-node costs; inner_parts, min_level_dist and div_rate mean
 * what innerParts, minLevelDist and divRate mean there.  *level_ptr,
 * *part_ptr (n+1 ints each) and *node_ptr (n ints) are allocated here;
 * release them with gbsym_free. */
int gbsym_coarse_levelset_tree(int n, const int *parent, const double *node_cost,
                               int inner_parts, int min_level_dist, int div_rate,
                               int *level_no, int **level_ptr, int *part_no,
                               int **part_ptr, int **node_ptr);
/* Replaces get_coarse_levelSet_DAG_CSC_tree at its call site
 * (demo/sptrsv_demo_utils.h:78-90; the function lives in the unvendored
 * aggregation dependency): LBC of the solve DAG of L, given as the CSR of a
 * lower triangle.  The tree LBC runs on the elimination tree of L's
 * symmetric pattern, which orders every dependency of the solve.  cost may
 * be NULL for the demo's cost, the entries per row.  Outputs as
 * gbsym_coarse_levelset_tree. */
int gbsym_build_lbc(int n, const int *Lp, const int *Li, const double *cost,
                    int inner_parts, int min_level_dist, int div_rate,
                    int *level_no, int **level_ptr, int *part_no,
                    int **part_ptr, int **node_ptr);
/* Elimination tree of the symmetric matrix whose lower triangle has the
 * pattern of the CSR (Lp, Li): parent[n], -1 at roots. */
int gbsym_etree_lower_csr(int n, const int *Lp, const int *Li, int *parent);

/* ---- supernodal (blocked CSC) solves ----------------------------------- */
/* Storage of the reference's ParSy blocked solves: supernode s owns columns
 * sup2col[s] .. sup2col[s+1]-1 (sup2col has supNo+1 entries, 0 .. n); its
 * rows are Li[Li_ptr[c0] .. Li_ptr[c1]), its own columns first, then the
 * rows below it ascending; its values are a column-major block of
 * Li_ptr[c1] - Li_ptr[c0] rows at Lx + Lp[c0] (only the lower triangle of
 * the diagonal block is read).  Lp and Li_ptr have n+1 size_t entries.  NNZ
 * and col2sup are accepted and unused (the reference's blocked solves do not
 * read them either).  x is host memory, column-major n x rhs, solved in
 * place; the functions return 1 on success and 0 otherwise (the status is
 * in gbsym_last_error()), as the reference's return 1/0.
 *
 * Forward: the reference's order, bit for bit (its dense kernels'
 * groupings).  Replaces parsy::blockedLsolve
 * (sparse_blas/parsy/triangularSolve/Triangular_BCSC.cpp:23-58). */
int gbsym_parsy_blockedLsolve(int n, size_t *Lp, int *Li, double *Lx, int NNZ,
                              size_t *Li_ptr, int *col2sup, int *sup2col,
                              int supNo, double *x);
/* Replaces parsy::blockedLsolve_mrhs (Triangular_BCSC.cpp:62-121): each of
 * the n_rhs columns as blockedLsolve solves it; max_col is unused. */
int gbsym_parsy_blockedLsolve_mrhs(int n, size_t *Lp, int *Li, double *Lx,
                                   int NNZ, size_t *Li_ptr, int *col2sup,
                                   int *sup2col, int supNo, double *x,
                                   int n_rhs, int max_col);
/* Replaces parsy::leveledBlockedLsolve (Triangular_BCSC.cpp:401-449): the
 * level set over supernodes is validated; the result equals blockedLsolve's
 * (the reference's atomic updates make its own order vary). */
int gbsym_parsy_leveledBlockedLsolve(int n, size_t *Lp, int *Li, double *Lx,
                                     int NNZ, size_t *Li_ptr, int *col2sup,
                                     int *sup2col, int supNo, double *x,
                                     int levels, int *levelPtr, int *levelSet,
                                     int chunk);
/* Replaces parsy::H2LeveledBlockedLsolve (Triangular_BCSC.cpp:512-581) and
 * its _mrhs form: the LBC schedule over supernodes (levelPtr -> parPtr ->
 * partition) is validated; results as blockedLsolve's. */
int gbsym_parsy_H2LeveledBlockedLsolve(int n, size_t *Lp, int *Li, double *Lx,
                                       int NNZ, size_t *Li_ptr, int *col2sup,
                                       int *sup2col, int supNo, double *x,
                                       int levels, int *levelPtr,
                                       int *levelSet, int parts, int *parPtr,
                                       int *partition, int chunk);
int gbsym_parsy_H2LeveledBlockedLsolve_mrhs(
    int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr,
    int *col2sup, int *sup2col, int supNo, double *x, int n_rhs, int levels,
    int *levelPtr, int *levelSet, int parts, int *parPtr, int *partition,
    int chunk, int max_col);
/* Transposed solve L^T x = b.  Replaces parsy::blockedLTsolve
 * (Triangular_BCSC.cpp:124-184), its _mrhs form and
 * H2LeveledBlockedLTsolve(_mrhs).  The reference computes this with an
 * external BLAS (dgemv/dtrsm, summation order the library's) or, in its
 * SYM_BLAS build, with the forward kernels (marked FIXME there); here each
 * supernode column subtracts its off-block rows' products in storage order,
 * then the diagonal block's transpose is solved backward. */
int gbsym_parsy_blockedLTsolve(int n, size_t *Lp, int *Li, double *Lx, int NNZ,
                               size_t *Li_ptr, int *col2sup, int *sup2col,
                               int supNo, double *x);
int gbsym_parsy_blockedLTsolve_mrhs(int n, size_t *Lp, int *Li, double *Lx,
                                    int NNZ, size_t *Li_ptr, int *col2sup,
                                    int *sup2col, int supNo, double *x,
                                    int m_rhs, int max_col);
int gbsym_parsy_H2LeveledBlockedLTsolve(int n, size_t *Lp, int *Li, double *Lx,
                                        int NNZ, size_t *Li_ptr, int *col2sup,
                                        int *sup2col, int supNo, double *x,
                                        int levels, int *levelPtr,
                                        int *levelSet, int parts, int *parPtr,
                                        int *partition, int chunk);
int gbsym_parsy_H2LeveledBlockedLTsolve_mrhs(
    int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr,
    int *col2sup, int *sup2col, int supNo, double *x, int m_rhs, int levels,
    int *levelPtr, int *levelSet, int parts, int *parPtr, int *partition,
    int chunk, int max_col);

/* The simplicial (CSC) solve phases: parsy::lsolve, then for LDL^T
 * x[i] /= d_val[i], then parsy::ltsolve, on the GPU; x in place; void (the
 * status is in gbsym_last_error()).  Replace parsy::solve_phase_simplicial_ll
 * and _ldl (sparse_blas/parsy/linear_solver/solve_phase.cpp:23-37). */
void gbsym_parsy_solve_phase_simplicial_ll(int n, int *Lp, int *Li, double *Lx,
                                           double *x);
void gbsym_parsy_solve_phase_simplicial_ldl(int n, int *Lp, int *Li,
                                            double *Lx, double *d_val,
                                            double *x);

/* The supernodal LL^T solve phases: the forward solve, then the transposed
 * one, on one resident plan; x (n x n_rhs, column-major) in place.  void,
 * as in the reference: the status is in gbsym_last_error().  The
 * scheduled forms validate the LBC schedule for both directions (the
 * transposed solve walks it backward).  Replace parsy::
 * solve_phase_ll_blocked, _nrhs, _parallel and _parallel_nrhs
 * (sparse_blas/parsy/linear_solver/solve_phase.cpp:39-94). */
void gbsym_parsy_solve_phase_ll_blocked(size_t n, double *x, int *col2sup,
                                        int *sup2col, size_t *newCol,
                                        int *newRow, double *newVal,
                                        size_t *rowP, size_t nBlocks, int nnz);
void gbsym_parsy_solve_phase_ll_blocked_nrhs(size_t n, double *x, int n_rhs,
                                             int *col2sup, int *sup2col,
                                             size_t *newCol, int *newRow,
                                             double *newVal, size_t *rowP,
                                             size_t nBlocks, int nnz,
                                             int max_col);
void gbsym_parsy_solve_phase_ll_blocked_parallel(
    size_t n, double *x, int *col2sup, int *sup2col, size_t *newCol,
    int *newRow, double *newVal, size_t *rowP, size_t nBlocks, int nnz,
    int levels, int *levelPtr, int *levelSet, int parts, int *parPtr,
    int *partition, int chunk);
void gbsym_parsy_solve_phase_ll_blocked_parallel_nrhs(
    size_t n, double *x, int n_rhs, int *col2sup, int *sup2col,
    size_t *newCol, int *newRow, double *newVal, size_t *rowP,
    size_t nBlocks, int nnz, int levels, int *levelPtr, int *levelSet,
    int parts, int *parPtr, int *partition, int chunk, int max_col);
/* The LDL^T solve phase with a diagonal D: forward solve, x[i] /= d[i]
 * (IEEE division, as parsy::scale_vec_vec), transposed solve.  Replaces
 * parsy::solve_phase_ldl (solve_phase.cpp:96-112). */
void gbsym_parsy_solve_phase_ldl(size_t n, double *d_val, double *x,
                                 int *col2sup, int *sup2col, size_t *newCol,
                                 int *newRow, double *newVal, size_t *rowP,
                                 size_t nBlocks, int nnz);

/* Supernodal plan: the factor resident on the GPU with its solve task
 * lists (host arrays in).  gbsym_sn_solve works on device memory, x
 * column-major n x k, forward (transposed = 0) or L^T (transposed = 1);
 * stream-ordered, one solve at a time per plan.  gbsym_sn_check
 * synchronises the stream and returns (and clears) the plan's sticky
 * device error: GBSYM_ERR_TIMEOUT if a bounded wait of an earlier solve
 * gave up. */
typedef struct gbsym_sn_s *gbsym_sn;
int gbsym_sn_create(gbsym_sn *out, int n, const size_t *Lp, const int *Li,
                    const double *Lx, const size_t *Li_ptr, const int *sup2col,
                    int supNo, void *stream);
int gbsym_sn_destroy(gbsym_sn t);
int gbsym_sn_levels(gbsym_sn t, int *forward_levels, int *transposed_levels);
int gbsym_sn_solve(gbsym_sn t, double *x, int k, int transposed, void *stream);
int gbsym_sn_check(gbsym_sn t, void *stream);
/* Bounded-wait self-test: one forward solve on scratch data whose counter
 * targets are one epoch ahead, so its waits on contributions cannot
 * complete and give up after limit_cycles SM cycles.  Returns the error
 * word the launch left (GBSYM_ERR_TIMEOUT where some supernode receives
 * contributions), then clears the plan's counters; later solves are
 * unaffected.  No fault, no hang: every wait is bounded. */
int gbsym_sn_selftest_timeout(gbsym_sn t, long long limit_cycles, void *stream);

/* ======================================================================== */
/* Plans (device-resident).                                                 */
/* ======================================================================== */

/* How a stored row defines a triangular row of the solve. */
enum gbsym_tri_kind {
  GBSYM_LOWER_DIAG_LAST = 0,  /* CSR of L: off-diagonals then the diagonal  */
  GBSYM_UPPER_DIAG_FIRST = 1, /* CSC of L read as CSR of L^T (ltsolve), or
                                 the CSR of an upper triangle              */
  GBSYM_ILU_UNIT_LOWER = 2,   /* [p[i], diags[i]), no division            */
  GBSYM_ILU_UPPER = 3,        /* (diags[i], p[i+1]), divide by diagonal   */
  GBSYM_ILU_LOWER_DIV = 4,    /* [p[i], diags[i]), divide by l[diags[i]]  */
  GBSYM_LOWER_CSC = 5         /* CSC of L, diagonal first in each column
                                 (sptrsv_csc); transposed on the GPU      */
};
enum gbsym_dtype { GBSYM_F64 = 0, GBSYM_F32 = 1 };
enum gbsym_layout { GBSYM_COL_MAJOR = 0, GBSYM_ROW_MAJOR = 1 };
enum gbsym_exec {
  GBSYM_EXEC_AUTO = 0,      /* autotuner choice                            */
  GBSYM_EXEC_LEVELSET = 1,  /* one launch per level, captured in a graph   */
  GBSYM_EXEC_SYNCFREE = 2,  /* one persistent launch, per-row ready flags  */
  GBSYM_EXEC_ONEBLOCK = 3,  /* one thread block sweeps all levels          */
  GBSYM_EXEC_PERSISTENT = 4, /* one cooperative launch, grid barrier/level */
  GBSYM_EXEC_CLUSTER = 5,    /* thread-block clusters, hardware cluster
                                barrier per level; k > 1 splits columns
                                over clusters                             */
  GBSYM_EXEC_PARTITIONED = 6 /* contiguous row partitions, one block each:
                                dependencies inside a partition through
                                shared memory, across partitions sync-free
                                (k = 1; k > 1 runs SYNCFREE)              */
};

/* Arithmetic of the row updates.  EXACT: every x_i -= L_ij x_j is a
 * rounded product followed by a rounded difference and the division is
 * correctly rounded -- the reference's operation sequence, bit-identical
 * results.  FUSED: one fused multiply-add per entry (results within a few
 * ulps of the reference; fewer FP64 operations). */
enum gbsym_arith { GBSYM_ARITH_EXACT = 0, GBSYM_ARITH_FUSED = 1 };

typedef struct gbsym_tri_s *gbsym_tri;

typedef struct {
  int n;
  int levels;          /* wavefront depth                                  */
  long long nnz_off;   /* stored off-diagonal entries                      */
  int dtype;           /* GBSYM_F64 / GBSYM_F32 value storage              */
  int exec;            /* executor chosen for k = 1                        */
  int max_level_rows;  /* widest level                                     */
  long long bytes_matrix; /* device bytes of the packed triangle           */
} gbsym_tri_info;

/* Build a level-packed triangle from a stored matrix.
 * p/i/x/diags may be host (on_device = 0) or device (on_device = 1)
 * pointers; diags is needed for the GBSYM_ILU_* kinds only.  level_ptr /
 * level_set may be NULL (the schedule is built on the GPU) or a level
 * schedule to execute (validated first: GBSYM_ERR_BAD_SCHEDULE).
 * value_dtype chooses FP64 or FP32 storage of the packed values (x is
 * always FP64 on input; FP32 storage rounds it once). */
int gbsym_tri_create(gbsym_tri *out, int n, const int *p, const int *i,
                     const double *x, const int *diags, int kind,
                     int value_dtype, int on_device, const int *level_ptr,
                     const int *level_set, int levels, void *stream);
int gbsym_tri_destroy(gbsym_tri t);
int gbsym_tri_get_info(gbsym_tri t, gbsym_tri_info *info);
/* Force an executor (GBSYM_EXEC_*); AUTO restores the autotuned choice. */
int gbsym_tri_set_exec(gbsym_tri t, int exec);
/* Choose the row arithmetic (GBSYM_ARITH_*); EXACT is the default. */
int gbsym_tri_set_arith(gbsym_tri t, int arith);
/* Times every executor on this plan for k right-hand sides of the given
 * dtype (on scratch memory; the caller's data is not touched), keeps the
 * fastest for later solves with k (k == 1 or k > 1) and remembers it for
 * plans with the same level count, mean row length, k and dtype.  The
 * chosen GBSYM_EXEC_* is returned in *chosen when non-NULL.  Synchronises
 * the stream. */
int gbsym_tri_autotune(gbsym_tri t, int k, int dtype, void *stream, int *chosen);
/* The executor settings solves with k right-hand sides use (after
 * gbsym_tri_autotune, the tuned ones): tuning[0] the GBSYM_EXEC_*,
 * tuning[1] the sync-free sweep's blocks per SM (0: its default by k),
 * tuning[2] for k > 1 its lane layout in bit 0 (1: the alternative) and
 * in bit 1 whether it looks through one level, for k = 1 how many levels it
 * looks through (0, 1 or 2).  Looking through, each row recomputes its
 * dependencies' values (the spare lanes with one right-hand side -- and
 * with two levels their dependencies' too -- every lane for its own columns
 * with several), so rows wait two (three) levels back; plans whose rows
 * fit a three-entry slab.  No counterpart in the reference. */
int gbsym_tri_get_tuning(gbsym_tri t, int k, int *tuning);
/* Waits for `stream` and returns the first error a device-side check of
 * this plan recorded since the last call (e.g. GBSYM_ERR_TIMEOUT from a
 * bounded wait), clearing it; GBSYM_OK when none. */
int gbsym_tri_check(gbsym_tri t, void *stream);
/* Failure-detection self-test: runs the executors' bounded grid-barrier
 * wait with one participant that never arrives and a limit of limit_ns
 * (at most 10 s).  Returns GBSYM_ERR_TIMEOUT when the wait gave up and
 * reported it, which is the expected outcome; the context stays usable. */
int gbsym_selftest_bounded_wait(long long limit_ns, void *stream);
/* No counterpart in the reference: a measurement aid for roofline figures.
 * Measures this GPU's FP64 throughput, in G operations/s, for the two forms
 * the exact solves issue: the update acc = RN(acc - RN(v*x)) (a rounded
 * product and a rounded difference: *update_gops) and general fused
 * multiply-adds with three variable operands (the division's remainder and
 * correction steps: *fma_gops).  Two short kernels; synchronises `stream`. */
int gbsym_fp64_rates(double *update_gops, double *fma_gops, void *stream);
/* Copy the schedule into host buffers of levels+1 and n ints. */
int gbsym_tri_get_schedule(gbsym_tri t, int *level_ptr, int *level_set);

/* Solve in place on device memory: x holds k right-hand sides in the given
 * layout and dtype (FP64 or FP32 vectors, matching the plan's value
 * storage).  Stream-ordered. */
int gbsym_tri_solve(gbsym_tri t, void *x, int k, int layout, int dtype,
                    void *stream);
/* Out of place on device memory: x = L^-1 b for k row-major right-hand
 * sides (n x k, dtype matching the plan's value storage); b is left
 * unchanged and must not overlap x (b == x solves in place).  The results
 * are bit-identical to gbsym_tri_solve's.  With k >= 32 the sync-free
 * executor reads b and publishes each result straight into x, so it writes
 * the solution once instead of twice; a solution value whose bits are all
 * ones (a NaN carried from a NaN input) is then stored as the default NaN.
 * Otherwise b is copied into x and solved in place.  Stream-ordered. */
int gbsym_tri_solve_into(gbsym_tri t, const void *b, void *x, int k, int dtype,
                         void *stream);
/* The lbc_redundant row formula: x_i = ((0 - sum_j L_ij x_j) + b_i)/L_ii. */
int gbsym_tri_solve_b(gbsym_tri t, const double *b, double *x, void *stream);
/* End-to-end: x is HOST memory (pinned or pageable); the call returns when
 * the solution is in x.  Pageable memory, and any memory on a system whose
 * GPU does not share the CPU's page tables, is staged: copied in, solved,
 * copied back.  Page-locked memory on a coherent CPU-GPU system (Grace with
 * NVLink-C2C) is solved in place: the sync-free sweep reads each right-hand
 * side and writes each result directly in the caller's buffer, so the
 * transfers overlap the sweep instead of preceding and following it
 * (row-major layout, or k = 1).  Results are identical either way. */
int gbsym_tri_solve_host(gbsym_tri t, double *x, int k, int layout);
/* 1 if gbsym_tri_solve_host would solve the host buffer x in place (it is
 * page-locked and the current GPU shares the CPU's page tables), else 0. */
int gbsym_host_solve_in_place(const void *x);

/* ---- CSR matrix plan (SpMV) -------------------------------------------- */
typedef struct gbsym_csr_s *gbsym_csr;
int gbsym_csr_create(gbsym_csr *out, int n, int ncols, const int *p,
                     const int *i, const double *x, int value_dtype,
                     int on_device, void *stream);
int gbsym_csr_destroy(gbsym_csr a);
/* y = A x  (FP64 or FP32 vectors matching the stored dtype). */
int gbsym_csr_spmv(gbsym_csr a, const void *x, void *y, int dtype, void *stream);
/* z = alpha (z + A x) + beta y, the reference's accumulate form. */
int gbsym_csr_spmv_axpby(gbsym_csr a, const double *x, const double *y,
                         double *z, double alpha, double beta, void *stream);

/* ---- GPU factorisations on device plans --------------------------------- */
/* ILU0 of a CSR with sorted columns and a diagonal in every row: returns in
 * l_dev (device, nnz doubles) the packed factor of spilu0_csr.
 * All pointers are device pointers. */
int gbsym_ilu0_device(int n, const int *Ap, const int *Ai, const double *Ax,
                      const int *A_diag, double *l, void *stream);
/* IC0 (spic0_csr) in place on the device copy of the upper CSR of A. */
int gbsym_ic0_device(int n, double *val, const int *rowPtr, const int *rowIdx,
                     void *stream);

/* ---- Krylov drivers (device vectors) ------------------------------------ */
typedef struct {
  int iterations;       /* PCG iterations / GMRES inner steps              */
  int restarts;         /* GMRES outer cycles                              */
  double relres;        /* final ||b - A x|| / ||b|| computed in FP64       */
  double seconds;       /* wall time of the solve, device-synchronised     */
  int status;
} gbsym_krylov_result;

/* IC0-preconditioned CG.  L is the plan of the forward solve (lower CSR of
 * the factor), Lt the plan of the transposed solve (its CSC as an upper
 * CSR).  b, x are device FP64 vectors; x holds the initial guess. */
int gbsym_pcg(gbsym_csr A, gbsym_tri L, gbsym_tri Lt, const double *b,
              double *x, double tol, int maxit, gbsym_krylov_result *res,
              void *stream);
/* Right-preconditioned GMRES(mr) with ILU0: Lu = unit-lower plan, U = upper
 * plan of the same packed factor.  The preconditioner runs in the dtype
 * the two plans store (FP32 or FP64); SpMV, Arnoldi, Givens and the
 * residual are FP64, all on the device.  1 <= mr <= 1024
 * (GBSYM_ERR_UNSUPPORTED beyond). */
int gbsym_gmres(gbsym_csr A, gbsym_tri Lu, gbsym_tri U, const double *b,
                double *x, int mr, int maxit, double tol,
                gbsym_krylov_result *res, void *stream);

/* ---- adjoint of the triangular solve ------------------------------------ */
/* Given X = L^{-1} B (row-major n x k, device) and G = dloss/dX, computes
 * G_B = L^{-T} G in place in g (Lt = plan of L^T, i.e. the CSC of L as an
 * upper CSR) and the gradient on L's stored values,
 * grad[p] = -sum_r G_B[row(p), r] * X[col(p), r], for every stored entry p
 * of the CSR of L (the diagonal included: grad = -sum_r G_B[i,r] X[i,r]).
 * Lp/Li are the device CSR arrays of L (diagonal last). */
int gbsym_tri_adjoint(gbsym_tri Lt, int n, const int *Lp, const int *Li,
                      const double *X, double *g, int k, double *grad,
                      void *stream);

/* ---- batched uneven systems --------------------------------------------- */
typedef struct gbsym_batch_s *gbsym_batch;
/* nsys lower triangles (CSR, diagonal last) given as host arrays of host
 * pointers; all are packed into one device pool and solved by one
 * persistent launch over (system, level) work items. */
int gbsym_batch_create(gbsym_batch *out, int nsys, const int *n,
                       const int *const *Lp, const int *const *Li,
                       const double *const *Lx, int value_dtype, void *stream);
/* The same with the triangles' storage named: GBSYM_LOWER_DIAG_LAST (as
 * gbsym_batch_create) or GBSYM_LOWER_CSC (lower CSC, diagonal first: the
 * upper CSR an IC0 factor is computed in, as spic0_csr leaves it).  Every
 * column index must lie inside its own system (GBSYM_ERR_BAD_MATRIX
 * otherwise). */
int gbsym_batch_create_kind(gbsym_batch *out, int nsys, const int *n,
                            const int *const *Lp, const int *const *Li,
                            const double *const *Lx, int kind, int value_dtype,
                            void *stream);
int gbsym_batch_destroy(gbsym_batch b);
/* x: device, concatenation of the systems' row-major n_s x k blocks (FP64
 * or FP32).  offsets (host, nsys+1) receives the row offset of each system
 * when non-NULL. */
int gbsym_batch_solve(gbsym_batch b, void *x, int k, int dtype, void *stream);
/* As gbsym_batch_solve on HOST memory (row-major, the batch's dtype).  When
 * x is page-locked, the GPU shares the host's page tables (Grace +
 * NVLink-C2C) and a row's k values take at least 256 bytes, the sweep reads
 * each right-hand side and writes each result across the link once, in
 * place; otherwise the solve is staged through a device copy (bulk copies
 * serve short rows faster).  Synchronises. */
int gbsym_batch_solve_host(gbsym_batch b, void *x, int k, int dtype);
int gbsym_batch_row_offsets(gbsym_batch b, long long *offsets);
/* Executor choice for k right-hand sides, timed on the batch itself (as
 * gbsym_tri_autotune on the pooled triangle). */
int gbsym_batch_autotune(gbsym_batch b, int k, int dtype, void *stream, int *chosen);
/* Synchronises `stream`; returns a status a bounded device wait recorded. */
int gbsym_batch_check(gbsym_batch b, void *stream);
/* Size, levels and storage of the pooled triangle. */
int gbsym_batch_get_info(gbsym_batch b, gbsym_tri_info *info);
/* gbsym_tri_get_tuning of the batch's pool. */
int gbsym_batch_get_tuning(gbsym_batch b, int k, int *tuning);

/* ---- forward solve that allocates nothing ------------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- an application whose own pool allocator owns all device memory,
 * or a loop that cannot take the device-wide synchronisation of cudaMalloc/
 * cudaFree.  Solves L x = b in place (x holds b on entry), L lower CSR with
 * the diagonal last in each row, all pointers DEVICE pointers, with the
 * reference sptrsv_csr arithmetic (bit-identical results).  Its only scratch
 * is a static device array inside this library (4 MiB per GPU, held until
 * the process exits), so n is limited to 524,288 rows; larger n returns
 * GBSYM_ERR_SIZE without touching x.  The first call on a device does that
 * device's set-up (it looks up the array's address); calls that overlap on
 * the GPU share the array and race.  Returns when the solve is done: every
 * call synchronises `stream` and reads an error word back to the host, so
 * it cannot be captured into a CUDA graph.
 * Precondition: Lp[0..n] is non-decreasing and Lp[n] lies within Li and
 * Lx -- the kernel reads Li[Lp[i] .. Lp[i+1]) unchecked.  Column indices
 * are checked: one outside [0, i) in row i returns GBSYM_ERR_BAD_MATRIX.
 * After GBSYM_ERR_BAD_MATRIX or GBSYM_ERR_TIMEOUT, x is undefined. */
int gbsym_sptrsv_csr_noalloc(int n, const int *Lp, const int *Li, const double *Lx, double *x,
                             void *stream);

#ifdef __cplusplus
}
#endif
#endif
