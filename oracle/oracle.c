/*
 * oracle.c -- CPU restatement of the reference's sparse triangular-solve
 * executor path.  TEST INFRASTRUCTURE ONLY: the product library never links,
 * loads or calls this file.  See oracle.h for the contract.
 *
 * Each function names the reference function and lines it restates (paths
 * are relative to the sympiler/sympiler source tree).  The floating-point
 * operation order of every row is the reference's; compile with
 * -ffp-contract=off.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* One row of the CSR pull solve: x_i = (x_i - sum_j L_ij x_j) / L_ii, with  */
/* the subtraction done entry by entry in storage order                     */
/* (sparse_blas/sptrsv.cpp:20-23).                                          */
static inline void row_pull(int i, const int *Lp, const int *Li,
                            const double *Lx, double *x) {
  double xi = x[i];
  for (int j = Lp[i]; j < Lp[i + 1] - 1; j++) xi -= Lx[j] * x[Li[j]];
  x[i] = xi / Lx[Lp[i + 1] - 1];
}

/* sparse_blas/sptrsv.cpp:17-25 */
void orc_sptrsv_csr(int n, const int *Lp, const int *Li, const double *Lx,
                    double *x) {
  for (int i = 0; i < n; i++) row_pull(i, Lp, Li, Lx, x);
}

/* sparse_blas/sptrsv.cpp:28-37 -- unit lower part of an ILU0-packed CSR,
 * stops at the diagonal pointer, no division. */
void orc_sptrsv_csr_ilu(int n, const int *Lp, const int *Li, const double *Lx,
                        const int *diags, double *x) {
  for (int i = 0; i < n; i++) {
    double xi = x[i];
    for (int j = Lp[i]; j < diags[i]; j++) xi -= Lx[j] * x[Li[j]];
    x[i] = xi;
  }
}

/* sparse_blas/sptrsv.cpp:40-55 -- one parallel-for per level. */
void orc_sptrsv_csr_levelset(int n, const int *Lp, const int *Li,
                             const double *Lx, double *x, int levels,
                             const int *levelPtr, const int *levelSet,
                             int nthreads) {
  (void)n;
#ifdef _OPENMP
  if (nthreads > 1) {
#pragma omp parallel num_threads(nthreads)
    for (int l = 0; l < levels; l++) {
#pragma omp for schedule(static)
      for (int k = levelPtr[l]; k < levelPtr[l + 1]; ++k)
        row_pull(levelSet[k], Lp, Li, Lx, x);
    }
    return;
  }
#endif
  (void)nthreads;
  for (int l = 0; l < levels; l++)
    for (int k = levelPtr[l]; k < levelPtr[l + 1]; ++k)
      row_pull(levelSet[k], Lp, Li, Lx, x);
}

/* sparse_blas/sptrsv.cpp:57-76 -- coarse level, then partitions, then the
 * rows of a partition in their listed order. */
void orc_sptrsv_csr_lbc(int n, const int *Lp, const int *Li, const double *Lx,
                        double *x, int level_no, const int *level_ptr,
                        const int *par_ptr, const int *partition) {
  (void)n;
  for (int i1 = 0; i1 < level_no; ++i1)
    for (int j1 = level_ptr[i1]; j1 < level_ptr[i1 + 1]; ++j1)
      for (int k1 = par_ptr[j1]; k1 < par_ptr[j1 + 1]; ++k1)
        row_pull(partition[k1], Lp, Li, Lx, x);
}

/* sparse_blas/sptrsv.cpp:78-107 -- the sum starts from zero in a scratch
 * vector, b is added last, then the division: x_i = ((0 - sum) + b_i)/L_ii. */
void orc_sptrsv_csr_lbc_redundant(int n, const int *Lp, const int *Li,
                                  const double *Lx, double *x, const double *b,
                                  int level_no, const int *level_ptr,
                                  const int *par_ptr, const int *partition) {
  (void)n;
  for (int i1 = 0; i1 < level_no; ++i1)
    for (int j1 = level_ptr[i1]; j1 < level_ptr[i1 + 1]; ++j1)
      for (int k1 = par_ptr[j1]; k1 < par_ptr[j1 + 1]; ++k1) {
        int i = partition[k1];
        double t = 0.0;
        for (int j = Lp[i]; j < Lp[i + 1] - 1; j++) t -= Lx[j] * x[Li[j]];
        t = (t + b[i]) / Lx[Lp[i + 1] - 1];
        x[i] = t;
      }
}

/* sparse_blas/sptrsv.cpp:109-127 -- as sptrsv_csr_ilu but it DOES divide by
 * Lx[diags[i]] (the reference's LBC variant differs from the serial one). */
void orc_sptrsv_csr_ilu_lbc(int n, const int *Lp, const int *Li,
                            const double *Lx, const int *diags, double *x,
                            int level_no, const int *level_ptr,
                            const int *par_ptr, const int *partition) {
  (void)n;
  for (int i1 = 0; i1 < level_no; ++i1)
    for (int j1 = level_ptr[i1]; j1 < level_ptr[i1 + 1]; ++j1)
      for (int k1 = par_ptr[j1]; k1 < par_ptr[j1 + 1]; ++k1) {
        int i = partition[k1];
        int dia = diags[i];
        double xi = x[i];
        for (int j = Lp[i]; j < dia; j++) xi -= Lx[j] * x[Li[j]];
        x[i] = xi / Lx[dia];
      }
}

/* sparse_blas/sptrsv.cpp:129-137 (= parsy::lsolve Triangular_CSC.cpp:18-28)
 * column push, diagonal first in each column. */
void orc_sptrsv_csc(int n, const int *Lp, const int *Li, const double *Lx,
                    double *x) {
  for (int i = 0; i < n; i++) {
    x[i] /= Lx[Lp[i]];
    for (int j = Lp[i] + 1; j < Lp[i + 1]; j++) x[Li[j]] -= Lx[j] * x[i];
  }
}

/* sparse_blas/sptrsv.cpp:139-156, executed in level order by one thread (the
 * reference's atomics make its own order nondeterministic). */
void orc_sptrsv_csc_levelset(int n, const int *Lp, const int *Li,
                             const double *Lx, double *x, int levels,
                             const int *levelPtr, const int *levelSet) {
  (void)n;
  for (int l = 0; l < levels; l++)
    for (int p = levelPtr[l]; p < levelPtr[l + 1]; p++) {
      int node = levelSet[p];
      x[node] /= Lx[Lp[node]];
      for (int j = Lp[node] + 1; j < Lp[node + 1]; j++)
        x[Li[j]] -= Lx[j] * x[node];
    }
}

/* sparse_blas/sptrsv_lt.cpp:11-20 (= parsy::ltsolve Triangular_CSC.cpp:30-40)
 * L^T x = b with L in CSC, diagonal first. */
int orc_ltsolve(int n, const int *Lp, const int *Li, const double *Lx,
                double *x) {
  if (!Lp || !Li || !x) return 0;
  for (int j = n - 1; j >= 0; j--) {
    double xj = x[j];
    for (int p = Lp[j] + 1; p < Lp[j + 1]; p++) xj -= Lx[p] * x[Li[p]];
    x[j] = xj / Lx[Lp[j]];
  }
  return 1;
}

/* Column-major n x k right-hand sides, one reference solve per column (the
 * layout of SolverSettings::solve_only, cholesky_solver.cpp:805-813). */
void orc_sptrsv_csr_mrhs(int n, const int *Lp, const int *Li, const double *Lx,
                         double *X, int k, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int c = 0; c < k; c++) orc_sptrsv_csr(n, Lp, Li, Lx, X + (size_t)c * n);
  (void)nthreads;
}

void orc_sptrsv_csr_levelset_mrhs(int n, const int *Lp, const int *Li,
                                  const double *Lx, double *X, int k,
                                  int levels, const int *levelPtr,
                                  const int *levelSet, int nthreads) {
  for (int c = 0; c < k; c++)
    orc_sptrsv_csr_levelset(n, Lp, Li, Lx, X + (size_t)c * n, levels, levelPtr,
                            levelSet, nthreads);
}

/* ------------------------------------------------------------------------ */
/* sparse_blas/spmv.cpp:12-21 */
void orc_spmv_csr(int n, const int *Ap, const int *Ai, const double *Ax,
                  const double *x, double *y) {
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int j = Ap[i]; j < Ap[i + 1]; j++) s += Ax[j] * x[Ai[j]];
    y[i] = s;
  }
}

/* sparse_blas/spmv.cpp:23-34 -- z is NOT cleared: z_i += A_i x, then
 * z_i = a z_i + b y_i. */
void orc_spmv_csr_axpby(int n, const int *Ap, const int *Ai, const double *Ax,
                        const double *x, const double *y, double *z, double a,
                        double b) {
  for (int i = 0; i < n; i++) {
    double s = z[i];
    for (int j = Ap[i]; j < Ap[i + 1]; j++) s += Ax[j] * x[Ai[j]];
    z[i] = a * s + b * y[i];
  }
}

/* sparse_blas/spmv.cpp:37-57 */
void orc_spmv_csr_parallel(int n, const int *Ap, const int *Ai,
                           const double *Ax, const double *x, double *y,
                           int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int j = Ap[i]; j < Ap[i + 1]; j++) s += Ax[j] * x[Ai[j]];
    y[i] = s;
  }
  (void)nthreads;
}

/* ------------------------------------------------------------------------ */
/* sparse_blas/spilu0.cpp:11-51 -- IKJ ILU0 on sorted CSR with diagonal
 * pointers; l takes A's pattern (unit-L multipliers + U with diagonal).
 * Returns 0 when the reference's asserts would fire (missing or zero
 * diagonal), 1 otherwise. */
int orc_spilu0_csr(int n, int nnz, const int *Ap, const int *Ai,
                   const double *Ax, const int *A_diag, double *l) {
  int *iw = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int ok = 1;
  for (int j = 0; j < n; j++) iw[j] = -1;
  for (int k = 0; k < nnz; k++) l[k] = Ax[k];
  for (int i = 0; i < n; i++) {
    for (int k = Ap[i]; k < Ap[i + 1]; k++) iw[Ai[k]] = k;
    int j, jrow = 0;
    for (j = Ap[i]; j < Ap[i + 1]; ++j) {
      jrow = Ai[j];
      if (i <= jrow) break;
      double tl = l[j] / l[A_diag[jrow]];
      l[j] = tl;
      for (int jj = A_diag[jrow] + 1; jj < Ap[jrow + 1]; jj++) {
        int jw = iw[Ai[jj]];
        if (jw != -1) l[jw] = l[jw] - tl * l[jj];
      }
    }
    if (A_diag[i] != j || jrow != i || l[j] == 0.0) ok = 0;
    for (int k = Ap[i]; k < Ap[i + 1]; k++) iw[Ai[k]] = -1;
  }
  free(iw);
  return ok;
}

/* sparse_blas/spic0.cpp:106-128 -- right-looking IC0 on the upper CSR of A
 * (= lower CSC), in place.  Returns 0 on a non-positive pivot (the
 * reference asserts), 1 otherwise.  The inner scan reads Li[l+1] one entry
 * past the row, exactly as the reference does; for l+1 == Lp[i+1] that is
 * the next row's diagonal column i+1 <= Li[k], so the scan continues to
 * the row end. */
int orc_spic0_csr(int n, double *Lx, const int *Lp, const int *Li) {
  int ok = 1;
  for (int i = 0; i < n; i++) {
    if (!(Lx[Lp[i]] > 0)) ok = 0;
    Lx[Lp[i]] = sqrt(Lx[Lp[i]]);
    double d = Lx[Lp[i]];
    for (int m = Lp[i] + 1; m < Lp[i + 1]; m++) Lx[m] = Lx[m] / d;
    for (int m = Lp[i] + 1; m < Lp[i + 1]; m++) {
      for (int k = Lp[Li[m]]; k < Lp[Li[m] + 1]; k++) {
        for (int l = m; l < Lp[i + 1] && (l + 1 >= Lp[n] || Li[l + 1] <= Li[k]);
             l++) {
          if (Li[l] == Li[k]) Lx[k] -= Lx[m] * Lx[l];
        }
      }
    }
  }
  return ok;
}

/* ------------------------------------------------------------------------ */
/* sparse_blas/parsy/gmres/mgmres.cpp:598-689 -- unit-L forward over
 * [ia[i], ua[i]) for i >= 1, then U backward over (ua[i], ia[i+1]) with a
 * division by l[ua[i]]. */
void orc_lus_cr(int n, int nz_num, const int *ia, const int *ja,
                const double *l, const int *ua, const double *r, double *z) {
  (void)nz_num;
  double *w = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; i++) w[i] = r[i];
  for (int i = 1; i < n; i++)
    for (int j = ia[i]; j < ua[i]; j++) w[i] = w[i] - l[j] * w[ja[j]];
  for (int i = n - 1; 0 <= i; i--) {
    for (int j = ua[i] + 1; j < ia[i + 1]; j++) w[i] = w[i] - l[j] * w[ja[j]];
    w[i] = w[i] / l[ua[i]];
  }
  for (int i = 0; i < n; i++) z[i] = w[i];
  free(w);
}

void orc_lus_cr_f32(int n, const int *ia, const int *ja, const float *l,
                    const int *ua, const float *r, float *z) {
  float *w = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; i++) w[i] = r[i];
  for (int i = 1; i < n; i++)
    for (int j = ia[i]; j < ua[i]; j++) w[i] = w[i] - l[j] * w[ja[j]];
  for (int i = n - 1; 0 <= i; i--) {
    for (int j = ua[i] + 1; j < ia[i + 1]; j++) w[i] = w[i] - l[j] * w[ja[j]];
    w[i] = w[i] / l[ua[i]];
  }
  for (int i = 0; i < n; i++) z[i] = w[i];
  free(w);
}

void orc_sptrsv_csr_f32(int n, const int *Lp, const int *Li, const float *Lx,
                        float *x) {
  for (int i = 0; i < n; i++) {
    float xi = x[i];
    for (int j = Lp[i]; j < Lp[i + 1] - 1; j++) xi -= Lx[j] * x[Li[j]];
    x[i] = xi / Lx[Lp[i + 1] - 1];
  }
}

void orc_ltsolve_f32(int n, const int *Lp, const int *Li, const float *Lx,
                     float *x) {
  for (int j = n - 1; j >= 0; j--) {
    float xj = x[j];
    for (int p = Lp[j] + 1; p < Lp[j + 1]; p++) xj -= Lx[p] * x[Li[p]];
    x[j] = xj / Lx[Lp[j]];
  }
}

void orc_spmv_csr_f32(int n, const int *Ap, const int *Ai, const float *Ax,
                      const float *x, float *y) {
  for (int i = 0; i < n; i++) {
    float s = 0.0f;
    for (int j = Ap[i]; j < Ap[i + 1]; j++) s += Ax[j] * x[Ai[j]];
    y[i] = s;
  }
}

/* ------------------------------------------------------------------------ */
/* Level-set convention of the reference's (unvendored) build_levelSet_CSC
 * (call sites Catch_tests/sptrsv_tests.cpp:59, demo/sptrsv_demo_utils.h:
 * 42-45): level(i) = 0 when row i has no off-diagonal entry, else
 * 1 + max level(j) over its off-diagonal columns j; level_ptr is the
 * exclusive prefix sum of the level sizes; rows are listed in ascending
 * index inside each level (the scan order of parsy::getLevelSet,
 * TreeUtils.cpp:101-110). */
static int levels_to_sets(int n, const int *lev, int *level_ptr,
                          int *level_set) {
  int nl = 0;
  for (int i = 0; i < n; i++)
    if (lev[i] + 1 > nl) nl = lev[i] + 1;
  for (int l = 0; l <= nl; l++) level_ptr[l] = 0;
  for (int i = 0; i < n; i++) level_ptr[lev[i] + 1]++;
  for (int l = 0; l < nl; l++) level_ptr[l + 1] += level_ptr[l];
  int *fill = (int *)malloc(sizeof(int) * (size_t)(nl > 0 ? nl : 1));
  for (int l = 0; l < nl; l++) fill[l] = level_ptr[l];
  for (int i = 0; i < n; i++) level_set[fill[lev[i]]++] = i;
  free(fill);
  return nl;
}

int orc_build_levelset_csr(int n, const int *Lp, const int *Li, int *level_ptr,
                           int *level_set) {
  int *lev = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
  for (int i = 0; i < n; i++) {
    int m = -1;
    for (int j = Lp[i]; j < Lp[i + 1]; j++) {
      int c = Li[j];
      if (c < i && lev[c] > m) m = lev[c];
    }
    lev[i] = m + 1;
  }
  int nl = levels_to_sets(n, lev, level_ptr, level_set);
  free(lev);
  return nl;
}

int orc_build_levelset_csc(int n, const int *Lp, const int *Li, int *level_ptr,
                           int *level_set) {
  int *lev = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
  for (int j = 0; j < n; j++)
    for (int p = Lp[j]; p < Lp[j + 1]; p++) {
      int r = Li[p];
      if (r > j && lev[j] + 1 > lev[r]) lev[r] = lev[j] + 1;
    }
  int nl = levels_to_sets(n, lev, level_ptr, level_set);
  free(lev);
  return nl;
}

int orc_build_levelset_upper_csr(int n, const int *Up, const int *Ui,
                                 int *level_ptr, int *level_set) {
  int *lev = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
  for (int i = n - 1; i >= 0; i--) {
    int m = -1;
    for (int j = Up[i]; j < Up[i + 1]; j++) {
      int c = Ui[j];
      if (c > i && lev[c] > m) m = lev[c];
    }
    lev[i] = m + 1;
  }
  int nl = levels_to_sets(n, lev, level_ptr, level_set);
  free(lev);
  return nl;
}

/* parsy::getLevelSet, sparse_blas/parsy/common/TreeUtils.cpp:89-140: repeated
 * ascending scans that take every unvisited node with no remaining child.
 * A node's level is therefore its height above the leaves. */
int orc_tree_levelset(int n, const int *tree, int *level_ptr, int *level_set) {
  int *nchild = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
  char *visited = (char *)calloc((size_t)(n > 0 ? n : 1), 1);
  for (int k = 0; k < n; k++)
    if (tree[k] >= 0) nchild[tree[k]]++;
  int cur = 0, cnt = 0;
  level_ptr[0] = 0;
  while (cnt < n) {
    int start = cnt;
    for (int i = 0; i < n; i++)
      if (nchild[i] == 0 && !visited[i]) {
        visited[i] = 1;
        level_set[cnt++] = i;
      }
    cur++;
    level_ptr[cur] = cnt;
    if (cnt == start) break; /* cycle guard: not a forest */
    for (int l = start; l < cnt; l++) {
      int c = level_set[l];
      if (tree[c] >= 0) nchild[tree[c]]--;
    }
  }
  free(nchild);
  free(visited);
  return cur;
}

/* ------------------------------------------------------------------------ */
static double dot(int n, const double *a, const double *b) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* IC0 preconditioned CG.  No PCG exists in the reference; this follows
 * Saad, Iterative Methods for Sparse Linear Systems, 2nd ed., Algorithm 9.1,
 * with M^{-1} = L^{-T} L^{-1} applied as Cholesky::solve does
 * (sparse_blas/linear_solver/Cholesky.cpp:32-37): forward solve on L, then
 * the transposed solve (ltsolve) on the CSC of L. */
int orc_pcg_ic0(int n, const int *Ap, const int *Ai, const double *Ax,
                const int *Lp, const int *Li, const double *Lx,
                const int *Ltp, const int *Lti, const double *Ltx,
                const double *b, double *x, double tol, int maxit,
                double *relres) {
  size_t nb = sizeof(double) * (size_t)(n > 0 ? n : 1);
  double *r = (double *)malloc(nb), *z = (double *)malloc(nb);
  double *p = (double *)malloc(nb), *q = (double *)malloc(nb);
  orc_spmv_csr(n, Ap, Ai, Ax, x, q);
  for (int i = 0; i < n; i++) r[i] = b[i] - q[i];
  double bnorm = sqrt(dot(n, b, b));
  if (bnorm == 0.0) bnorm = 1.0;
  memcpy(z, r, nb);
  orc_sptrsv_csr(n, Lp, Li, Lx, z);
  orc_ltsolve(n, Ltp, Lti, Ltx, z);
  memcpy(p, z, nb);
  double rz = dot(n, r, z);
  double rel = sqrt(dot(n, r, r)) / bnorm;
  int it = 0;
  while (rel > tol && it < maxit) {
    orc_spmv_csr(n, Ap, Ai, Ax, p, q);
    double alpha = rz / dot(n, p, q);
    for (int i = 0; i < n; i++) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
    }
    it++;
    rel = sqrt(dot(n, r, r)) / bnorm;
    if (rel <= tol) break;
    memcpy(z, r, nb);
    orc_sptrsv_csr(n, Lp, Li, Lx, z);
    orc_ltsolve(n, Ltp, Lti, Ltx, z);
    double rz1 = dot(n, r, z);
    double beta = rz1 / rz;
    rz = rz1;
    for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
  }
  if (relres) *relres = rel;
  free(r); free(z); free(p); free(q);
  return it;
}

/* mgmres.cpp:186-251 */
static void mult_givens(double c, double s, int k, double *g) {
  double g1 = c * g[k] - s * g[k + 1];
  double g2 = s * g[k] + c * g[k + 1];
  g[k] = g1;
  g[k + 1] = g2;
}

/* Restarted GMRES(mr) following pmgmres_ldlt_cr (mgmres.cpp:839-987):
 * MGS Arnoldi (911-916), the re-orthogonalisation test with delta = 1e-3
 * (919-928), Givens rotations (937-954), the stop test on |g[k+1]| (964)
 * and back substitution (971-982).  Differences, chosen for the
 * nonsymmetric operator: the system SpMV is the general CSR product
 * (ax_cr, mgmres.cpp:20-113) and the ILU0 preconditioner (lus_cr) is
 * applied on the RIGHT, so the update is x += M^{-1} (V y). */
int orc_gmres_ilu0(int n, const int *Ap, const int *Ai, const double *Ax,
                   const double *lu, const int *ua, const double *b, double *x,
                   int mr, int itr_max, double tol_rel, double *relres) {
  const double delta = 1.0e-03;
  size_t nb = sizeof(double) * (size_t)(n > 0 ? n : 1);
  double *r = (double *)malloc(nb), *w = (double *)malloc(nb);
  double *v = (double *)malloc(nb * (size_t)(mr + 1));
  double *h = (double *)calloc((size_t)(mr + 1) * mr, sizeof(double));
  double *c = (double *)calloc((size_t)mr + 1, sizeof(double));
  double *s = (double *)calloc((size_t)mr + 1, sizeof(double));
  double *g = (double *)calloc((size_t)mr + 1, sizeof(double));
  double *y = (double *)calloc((size_t)mr + 1, sizeof(double));
#define H(i, j) h[(size_t)(i) * mr + (j)]
#define V(j) (v + (size_t)(j) * n)
  int itr_used = 0;
  double rho = 0.0, rho_tol = 0.0;
  double bnorm = sqrt(dot(n, b, b));
  for (int itr = 0; itr < itr_max; itr++) {
    orc_spmv_csr(n, Ap, Ai, Ax, x, r);
    for (int i = 0; i < n; i++) r[i] = b[i] - r[i];
    rho = sqrt(dot(n, r, r));
    if (itr == 0) rho_tol = rho * tol_rel;
    if (rho <= rho_tol || rho == 0.0) break;
    for (int i = 0; i < n; i++) V(0)[i] = r[i] / rho;
    g[0] = rho;
    for (int i = 1; i < mr + 1; i++) g[i] = 0.0;
    for (size_t i = 0; i < (size_t)(mr + 1) * mr; i++) h[i] = 0.0;
    int k, k_copy = 0;
    for (k = 0; k < mr; k++) {
      k_copy = k;
      orc_lus_cr(n, Ap[n], Ap, Ai, lu, ua, V(k), w);
      orc_spmv_csr(n, Ap, Ai, Ax, w, V(k + 1));
      double av = sqrt(dot(n, V(k + 1), V(k + 1)));
      for (int j = 0; j <= k; j++) {
        H(j, k) = dot(n, V(k + 1), V(j));
        for (int i = 0; i < n; i++) V(k + 1)[i] -= H(j, k) * V(j)[i];
      }
      H(k + 1, k) = sqrt(dot(n, V(k + 1), V(k + 1)));
      if ((av + delta * H(k + 1, k)) == av) {
        for (int j = 0; j < k + 1; j++) {
          double ht = dot(n, V(k + 1), V(j));
          H(j, k) += ht;
          for (int i = 0; i < n; i++) V(k + 1)[i] -= ht * V(j)[i];
        }
        H(k + 1, k) = sqrt(dot(n, V(k + 1), V(k + 1)));
      }
      if (H(k + 1, k) != 0.0)
        for (int i = 0; i < n; i++) V(k + 1)[i] /= H(k + 1, k);
      if (0 < k) {
        for (int i = 0; i < k + 2; i++) y[i] = H(i, k);
        for (int j = 0; j < k; j++) mult_givens(c[j], s[j], j, y);
        for (int i = 0; i < k + 2; i++) H(i, k) = y[i];
      }
      double mu = sqrt(H(k, k) * H(k, k) + H(k + 1, k) * H(k + 1, k));
      if (mu == 0.0) break;
      c[k] = H(k, k) / mu;
      s[k] = -H(k + 1, k) / mu;
      H(k, k) = c[k] * H(k, k) - s[k] * H(k + 1, k);
      H(k + 1, k) = 0.0;
      mult_givens(c[k], s[k], k, g);
      rho = fabs(g[k + 1]);
      itr_used++;
      if (rho <= rho_tol) break;
    }
    k = k_copy;
    y[k] = g[k] / H(k, k);
    for (int i = k - 1; 0 <= i; i--) {
      y[i] = g[i];
      for (int j = i + 1; j < k + 1; j++) y[i] -= H(i, j) * y[j];
      y[i] /= H(i, i);
    }
    for (int i = 0; i < n; i++) {
      double t = 0.0;
      for (int j = 0; j < k + 1; j++) t += V(j)[i] * y[j];
      r[i] = t;
    }
    orc_lus_cr(n, Ap[n], Ap, Ai, lu, ua, r, w);
    for (int i = 0; i < n; i++) x[i] += w[i];
    if (rho <= rho_tol) break;
  }
  orc_spmv_csr(n, Ap, Ai, Ax, x, r);
  for (int i = 0; i < n; i++) r[i] = b[i] - r[i];
  if (relres) *relres = sqrt(dot(n, r, r)) / (bnorm > 0 ? bnorm : 1.0);
#undef H
#undef V
  free(r); free(w); free(v); free(h); free(c); free(s); free(g); free(y);
  return itr_used;
}

/* ---- supernodal (blocked CSC) solves -------------------------------------- */

/* Dense lower solve of the w x w diagonal block M (column-major, leading
 * dimension ld) in place on rhs, with the reference's grouping: columns in
 * runs of 8 while at least 8 remain past the current one, then runs of 4,
 * then at most one run of 2 and one single column.  Inside a run each
 * unknown subtracts the run's earlier unknowns left to right and divides;
 * then every later row subtracts the run's products left to right
 * (sparse_blas/parsy/triangularSolve/BLAS.cpp:12-106). */
static void blk_diag_solve(int ld, int w, const double *M, double *rhs) {
  int fc = 0;
  for (;;) {
    int g;
    if (fc < w - 7) g = 8;
    else if (fc < w - 3) g = 4;
    else if (fc < w - 1) g = 2;
    else if (fc == w - 1) g = 1;
    else break;
    double xg[8];
    for (int a = 0; a < g; ++a) {
      double v = rhs[fc + a];
      for (int b = 0; b < a; ++b) v = v - xg[b] * M[(size_t)(fc + b) * ld + fc + a];
      xg[a] = v / M[(size_t)(fc + a) * ld + fc + a];
    }
    for (int a = 0; a < g; ++a) rhs[fc + a] = xg[a];
    for (int k = fc + g; k < w; ++k) {
      double v = rhs[k];
      for (int b = 0; b < g; ++b) v = v - xg[b] * M[(size_t)(fc + b) * ld + k];
      rhs[k] = v;
    }
    fc += g;
    if (g <= 2) {
      /* after a run of 2 only a single column can remain, and after the
         single column nothing */
      if (g == 2 && fc == w - 1) continue;
      break;
    }
  }
}

/* out[k] = the dot of off-block row w + k of the ld x ncol block M
 * (column-major) with vec, for the nrow = ld - w rows below a w-row
 * diagonal block, in the reference's grouping: column runs of 8 while 8
 * remain, then 4, then 1; each run's products summed left to right, then
 * added to the running value, which starts at +0.  Runs are outermost so
 * that every pass walks the rows contiguously, as dmatvec_blas does
 * (BLAS.cpp:123-185); each row's arithmetic is unchanged by that. */
static void blk_rows_dot(int ld, int ncol, const double *M, int nrow, const double *vec, double *out) {
  const int w = ld - nrow;
  for (int k = 0; k < nrow; ++k) out[k] = 0.0;
  int fc = 0;
  while (fc < ncol - 7) {
    const double *m0 = M + (size_t)fc * ld + w;
    for (int k = 0; k < nrow; ++k) {
      double s = vec[fc] * m0[k];
      for (int b = 1; b < 8; ++b) s = s + vec[fc + b] * m0[(size_t)b * ld + k];
      out[k] = out[k] + s;
    }
    fc += 8;
  }
  while (fc < ncol - 3) {
    const double *m0 = M + (size_t)fc * ld + w;
    for (int k = 0; k < nrow; ++k) {
      double s = vec[fc] * m0[k];
      for (int b = 1; b < 4; ++b) s = s + vec[fc + b] * m0[(size_t)b * ld + k];
      out[k] = out[k] + s;
    }
    fc += 4;
  }
  while (fc < ncol) {
    const double *m0 = M + (size_t)fc * ld + w;
    for (int k = 0; k < nrow; ++k) out[k] = out[k] + vec[fc] * m0[k];
    fc += 1;
  }
}

/* The off-block part of column q in the transposed solve: sum over the
 * nb off-block rows of col[r] * x[rows[r]], taken from the LAST row
 * backward and grouped as blk_rows_dot groups a row: runs of 8 while 8
 * remain, then 4, then 1; each run summed in that order, then added to a
 * running value that starts at +0.  This order is this library's own (its
 * GPU solve consumes the ancestors' unknowns as they appear, top down): the
 * reference's SYM_BLAS build has no transposed kernel of its own
 * (blockedLTsolve, Triangular_BCSC.cpp:124-177, applies the forward
 * kernels there and marks it FIXME). */
static double blk_col_dot(int nb, const double *col, const int *rows, const double *x) {
  double acc = 0.0;
  int fc = 0;
#define RP(e) (nb - 1 - (e))
  while (fc < nb - 7) {
    double s = x[rows[RP(fc)]] * col[RP(fc)];
    for (int b = 1; b < 8; ++b) s = s + x[rows[RP(fc + b)]] * col[RP(fc + b)];
    acc = acc + s;
    fc += 8;
  }
  while (fc < nb - 3) {
    double s = x[rows[RP(fc)]] * col[RP(fc)];
    for (int b = 1; b < 4; ++b) s = s + x[rows[RP(fc + b)]] * col[RP(fc + b)];
    acc = acc + s;
    fc += 4;
  }
  while (fc < nb) {
    acc = acc + x[rows[RP(fc)]] * col[RP(fc)];
    fc += 1;
  }
#undef RP
  return acc;
}

/* Triangular_BCSC.cpp:23-58: per supernode in increasing order, the dense
 * diagonal solve, then the off-block product subtracted from the rows it
 * reaches. */
void orc_blocked_lsolve(int n, const size_t *Lp, const int *Li, const double *Lx,
                        const size_t *Li_ptr, const int *sup2col, int supNo,
                        double *x, int nrhs) {
  int maxoff = 1;
  for (int s = 0; s < supNo; ++s) {
    const int w = sup2col[s + 1] - sup2col[s];
    const int nr = (int)(Li_ptr[sup2col[s + 1]] - Li_ptr[sup2col[s]]);
    if (nr - w > maxoff) maxoff = nr - w;
  }
  double *tmp = (double *)malloc(sizeof(double) * (size_t)maxoff);
  for (int j = 0; j < nrhs; ++j) {
    double *xj = x + (size_t)j * n;
    for (int s = 0; s < supNo; ++s) {
      const int c0 = sup2col[s], c1 = sup2col[s + 1], w = c1 - c0;
      const int nr = (int)(Li_ptr[c1] - Li_ptr[c0]);
      const double *M = Lx + Lp[c0];
      blk_diag_solve(nr, w, M, xj + c0);
      blk_rows_dot(nr, w, M, nr - w, xj + c0, tmp);
      for (int k = w; k < nr; ++k) {
        const int r = Li[Li_ptr[c0] + k];
        xj[r] = xj[r] - tmp[k - w];
      }
    }
  }
  free(tmp);
}

void orc_blocked_ltsolve(int n, const size_t *Lp, const int *Li, const double *Lx,
                         const size_t *Li_ptr, const int *sup2col, int supNo,
                         double *x, int nrhs) {
  for (int j = 0; j < nrhs; ++j) {
    double *xj = x + (size_t)j * n;
    for (int s = supNo - 1; s >= 0; --s) {
      const int c0 = sup2col[s], c1 = sup2col[s + 1], w = c1 - c0;
      const int nr = (int)(Li_ptr[c1] - Li_ptr[c0]);
      const double *M = Lx + Lp[c0];
      for (int q = 0; q < w; ++q)
        xj[c0 + q] = xj[c0 + q] - blk_col_dot(nr - w, M + (size_t)q * nr + w, Li + Li_ptr[c0] + w, xj);
      /* the diagonal block's transpose backward: unknown i subtracts
       * L[q, i] x_q for q from the last down to i + 1, then divides (the
       * solved x_q are final when i is reached; column i is contiguous) */
      for (int i = w - 1; i >= 0; --i) {
        const double *Mi = M + (size_t)i * nr;
        double v = xj[c0 + i];
        for (int q = w - 1; q > i; --q) v = v - Mi[q] * xj[c0 + q];
        xj[c0 + i] = v / Mi[i];
      }
    }
  }
}
