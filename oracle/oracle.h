/*
 * oracle.h -- CPU restatement of the reference's sparse triangular-solve
 * executor path (sympiler/sympiler, namespace sym_lib).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is the oracle the GPU path is compared against: the
 * parity tests, the smoke check and the CPU-baseline leg of the benchmark are
 * its only users.
 *
 * Every function restates one reference function (file:line given beside it)
 * with the same floating-point operation order.  Built with
 * -ffp-contract=off so that "a - b*c" is a rounded product followed by a
 * rounded subtraction on every host architecture, which is what the reference
 * computes on x86-64 (no FMA in its default build).
 */
#ifndef GBSYM_ORACLE_H
#define GBSYM_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- SpTRSV, CSR row-pull (sparse_blas/sptrsv.cpp) ---------------------- */
void orc_sptrsv_csr(int n, const int *Lp, const int *Li, const double *Lx, double *x);
void orc_sptrsv_csr_ilu(int n, const int *Lp, const int *Li, const double *Lx,
                        const int *diags, double *x);
void orc_sptrsv_csr_levelset(int n, const int *Lp, const int *Li, const double *Lx,
                             double *x, int levels, const int *levelPtr,
                             const int *levelSet, int nthreads);
void orc_sptrsv_csr_lbc(int n, const int *Lp, const int *Li, const double *Lx,
                        double *x, int level_no, const int *level_ptr,
                        const int *par_ptr, const int *partition);
void orc_sptrsv_csr_lbc_redundant(int n, const int *Lp, const int *Li,
                                  const double *Lx, double *x, const double *b,
                                  int level_no, const int *level_ptr,
                                  const int *par_ptr, const int *partition);
void orc_sptrsv_csr_ilu_lbc(int n, const int *Lp, const int *Li, const double *Lx,
                            const int *diags, double *x, int level_no,
                            const int *level_ptr, const int *par_ptr,
                            const int *partition);
/* ---- SpTRSV, CSC column-push (sparse_blas/sptrsv.cpp, Triangular_CSC.cpp) */
void orc_sptrsv_csc(int n, const int *Lp, const int *Li, const double *Lx, double *x);
void orc_sptrsv_csc_levelset(int n, const int *Lp, const int *Li, const double *Lx,
                             double *x, int levels, const int *levelPtr,
                             const int *levelSet);
int orc_ltsolve(int n, const int *Lp, const int *Li, const double *Lx, double *x);

/* ---- multi-RHS helpers (column-major n x k, as the reference's solve_only) */
void orc_sptrsv_csr_mrhs(int n, const int *Lp, const int *Li, const double *Lx,
                         double *X, int k, int nthreads);
void orc_sptrsv_csr_levelset_mrhs(int n, const int *Lp, const int *Li,
                                  const double *Lx, double *X, int k, int levels,
                                  const int *levelPtr, const int *levelSet,
                                  int nthreads);

/* ---- SpMV (sparse_blas/spmv.cpp) --------------------------------------- */
void orc_spmv_csr(int n, const int *Ap, const int *Ai, const double *Ax,
                  const double *x, double *y);
void orc_spmv_csr_axpby(int n, const int *Ap, const int *Ai, const double *Ax,
                        const double *x, const double *y, double *z, double a,
                        double b);
void orc_spmv_csr_parallel(int n, const int *Ap, const int *Ai, const double *Ax,
                           const double *x, double *y, int nthreads);

/* ---- factorisations (sparse_blas/spilu0.cpp, spic0.cpp) ----------------- */
int orc_spilu0_csr(int n, int nnz, const int *Ap, const int *Ai, const double *Ax,
                   const int *A_diag, double *l);
int orc_spic0_csr(int n, double *Lx, const int *Lp, const int *Li);

/* ---- ILU apply (sparse_blas/parsy/gmres/mgmres.cpp:598-689) ------------- */
void orc_lus_cr(int n, int nz_num, const int *ia, const int *ja, const double *l,
                const int *ua, const double *r, double *z);
void orc_lus_cr_f32(int n, const int *ia, const int *ja, const float *l,
                    const int *ua, const float *r, float *z);

/* ---- FP32 executors (same operation order, single precision) ------------ */
void orc_sptrsv_csr_f32(int n, const int *Lp, const int *Li, const float *Lx, float *x);
void orc_ltsolve_f32(int n, const int *Lp, const int *Li, const float *Lx, float *x);
void orc_spmv_csr_f32(int n, const int *Ap, const int *Ai, const float *Ax,
                      const float *x, float *y);

/* ---- schedules ----------------------------------------------------------- */
/* DAG wavefront level set of a lower-triangular CSR (diagonal last).
 * Returns the number of levels; level_ptr has n+1 slots, level_set n. */
int orc_build_levelset_csr(int n, const int *Lp, const int *Li, int *level_ptr,
                           int *level_set);
/* Same DAG from the CSC of L (diagonal first). */
int orc_build_levelset_csc(int n, const int *Lp, const int *Li, int *level_ptr,
                           int *level_set);
/* Level set of the backward (upper) solve: row i depends on columns > i. */
int orc_build_levelset_upper_csr(int n, const int *Up, const int *Ui,
                                 int *level_ptr, int *level_set);
/* parsy::getLevelSet on an elimination tree (TreeUtils.cpp:89-140). */
int orc_tree_levelset(int n, const int *tree, int *level_ptr, int *level_set);

/* ---- Krylov drivers ------------------------------------------------------ */
/* IC0-preconditioned CG on CSR A; preconditioner = L (CSR lower) forward,
 * then L^T backward using the CSC of L (= CSR of L^T).  Returns iterations;
 * writes the final relative residual to *relres. */
int orc_pcg_ic0(int n, const int *Ap, const int *Ai, const double *Ax,
                const int *Lp, const int *Li, const double *Lx,
                const int *Ltp, const int *Lti, const double *Ltx,
                const double *b, double *x, double tol, int maxit,
                double *relres);
/* Right-ILU0-preconditioned restarted GMRES(mr) with modified Gram-Schmidt
 * and Givens rotations.  Returns inner iterations used. */
int orc_gmres_ilu0(int n, const int *Ap, const int *Ai, const double *Ax,
                   const double *lu, const int *ua, const double *b, double *x,
                   int mr, int itr_max, double tol_rel, double *relres);

/* ---- supernodal (blocked CSC) solves ----------------------------------- */
/* Supernode s owns columns sup2col[s] .. sup2col[s+1]-1; its rows are
 * Li[Li_ptr[c0] .. Li_ptr[c1]) (the diagonal block's rows first) and its
 * values a column-major block of nSupR rows at Lx + Lp[c0].  x is n x nrhs,
 * column-major (leading dimension n).
 *
 * Forward solve in the order of parsy::blockedLsolve
 * (sparse_blas/parsy/triangularSolve/Triangular_BCSC.cpp:23-58) with its
 * dense kernels dlsolve_blas_nonUnit and dmatvec_blas
 * (sparse_blas/parsy/triangularSolve/BLAS.cpp:12-121, 123-185), column by
 * column. */
void orc_blocked_lsolve(int n, const size_t *Lp, const int *Li, const double *Lx,
                        const size_t *Li_ptr, const int *sup2col, int supNo,
                        double *x, int nrhs);
/* Transposed (backward) solve L^T x = b on the same storage: supernodes in
 * decreasing order; per supernode column j, x_j minus the sum over the
 * off-block rows r (from the last) of L[r, j] x_r, grouped as dmatvec_blas
 * groups a row (runs of 8, 4, 1; run sums added to a running +0); then the diagonal block's transpose backward, column j from the
 * last: x_j /= L[j, j], then x_i -= L[j, i] x_j for i < j. */
void orc_blocked_ltsolve(int n, const size_t *Lp, const int *Li, const double *Lx,
                         const size_t *Li_ptr, const int *sup2col, int supNo,
                         double *x, int nrhs);

#ifdef __cplusplus
}
#endif
#endif
