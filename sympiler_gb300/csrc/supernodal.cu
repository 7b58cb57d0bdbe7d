// supernodal.cu -- forward and transposed solves with a supernodal
// (blocked CSC) factor: the reference's ParSy blocked solves
// (sparse_blas/parsy/triangularSolve/Triangular_BCSC.cpp).
//
// Storage (the reference's): supernode s owns columns c0 = sup2col[s] ..
// c1 = sup2col[s+1]; its rows are Li[Li_ptr[c0] .. Li_ptr[c1]), its own
// columns first, and its values a column-major block of nr = Li_ptr[c1] -
// Li_ptr[c0] rows at Lx + Lp[c0].  x is column-major n x k.
//
// Forward solve.  The reference (blockedLsolve, :23-58) walks supernodes in
// order: a dense solve of the diagonal block (dlsolve_blas_nonUnit), then
// the off-block rows' products (dmatvec_blas) pushed into the rows they
// reach.  Every row therefore receives its subtractions in increasing
// source order.  Here a supernode pulls them instead: for each of its rows,
// the contributions of its sources in increasing order, each product
// formed in dmatvec_blas's grouping -- so the results are the reference's,
// bit for bit, while supernodes of one level run in parallel without
// atomics (the reference's leveled variants subtract under `omp atomic`,
// whose order varies).  The dense diagonal solve follows
// dlsolve_blas_nonUnit's grouping (runs of 8, 4, 2, 1 columns; left-to-right
// subtraction chains; IEEE division).  Both kernels' groupings are restated
// from parsy/triangularSolve/BLAS.cpp:12-185.
//
// Transposed solve.  The reference's SYM_BLAS build applies the forward
// kernels here (its own FIXME); its BLAS build calls dgemv/dtrsm, whose
// summation order is the library's.  This file solves L^T x = b in an order
// of its own: per supernode column j, x_j minus the off-block rows'
// products in storage order, then the diagonal block's transpose backward.
//
// Supernodes are scheduled by the levels of the supernode dependency DAG
// (one launch per level; a block per supernode).
#include <algorithm>
#include <memory>
#include <vector>

#include "common.cuh"

struct gbsym_sn_s {
  int n = 0, nsup = 0, nlev = 0, nblev = 0, max_w = 0;
  std::vector<int> h_lev_ptr, h_blev_ptr;
  gbsym::DBuf<int> c0, nr, rb;          // per supernode: first column, rows, row base
  gbsym::DBuf<long long> vb;            // per supernode: value base (Lp[c0])
  gbsym::DBuf<int> rows;                // Li
  gbsym::DBuf<double> vals;             // Lx
  gbsym::DBuf<int> pull_ptr, pull_src, pull_k;  // forward: per column, (source, row position)
  gbsym::DBuf<int> lev_set, blev_set;   // supernodes in forward / backward level order
};

namespace gbsym {
namespace {

constexpr int kSnBlock = 128;
constexpr int kSnSmem = 5120;  // values of shared memory per block (40 KB)

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// One off-block row's product with the source's solved values, in
// dmatvec_blas's grouping: runs of 8 columns while 8 remain past the
// current one, then runs of 4, then single columns; each run summed left to
// right, then added to the running value, which starts at +0.
__device__ double row_dot(const double *__restrict__ M, int ld, int ncol, int k, const double *__restrict__ v) {
  double acc = 0.0;
  int fc = 0;
  while (fc < ncol - 7) {
    double s = dm(v[fc], M[(size_t)fc * ld + k]);
#pragma unroll
    for (int b = 1; b < 8; ++b) s = da(s, dm(v[fc + b], M[(size_t)(fc + b) * ld + k]));
    acc = da(acc, s);
    fc += 8;
  }
  while (fc < ncol - 3) {
    double s = dm(v[fc], M[(size_t)fc * ld + k]);
#pragma unroll
    for (int b = 1; b < 4; ++b) s = da(s, dm(v[fc + b], M[(size_t)(fc + b) * ld + k]));
    acc = da(acc, s);
    fc += 4;
  }
  while (fc < ncol) {
    acc = da(acc, dm(v[fc], M[(size_t)fc * ld + k]));
    ++fc;
  }
  return acc;
}

// Forward: one block per supernode of the level.  Right-hand sides are done
// kc columns at a time so that the w x kc values fit in shared memory.
__global__ void __launch_bounds__(kSnBlock)
k_sn_forward(const int *__restrict__ lev_set, int base, const int *__restrict__ c0s, const int *__restrict__ nrs,
             const long long *__restrict__ vbs, const double *__restrict__ Lx, const int *__restrict__ pull_ptr,
             const int *__restrict__ pull_src, const int *__restrict__ pull_k, double *__restrict__ x, int n,
             int k) {
  __shared__ double rhs[kSnSmem];
  __shared__ double xg[8 * 64];
  const int t = lev_set[base + blockIdx.x];
  const int c0 = c0s[t], w = c0s[t + 1] - c0, ld = nrs[t];
  const double *M = Lx + vbs[t];
  const int kc = max(1, min(min(k, 64), kSnSmem / w));
  for (int j0 = 0; j0 < k; j0 += kc) {
    const int kk = min(kc, k - j0);
    // pull: each row's subtractions from its sources in increasing order
    for (int idx = threadIdx.x; idx < w * kk; idx += blockDim.x) {
      const int q = idx % w, jj = idx / w;
      const int r = c0 + q;
      double *xc = x + (size_t)(j0 + jj) * n;
      double acc = xc[r];
      for (int p = pull_ptr[r]; p < pull_ptr[r + 1]; ++p) {
        const int s = pull_src[p];
        const int sc0 = c0s[s];
        acc = ds(acc, row_dot(Lx + vbs[s], nrs[s], c0s[s + 1] - sc0, pull_k[p], xc + sc0));
      }
      rhs[jj * w + q] = acc;
    }
    __syncthreads();
    // the diagonal block, in runs of 8, 4, 2, 1 columns
    int fc = 0;
    while (fc < w) {
      const int g = fc < w - 7 ? 8 : fc < w - 3 ? 4 : fc < w - 1 ? 2 : 1;
      for (int jj = threadIdx.x; jj < kk; jj += blockDim.x) {
        double *rv = rhs + jj * w;
        for (int a = 0; a < g; ++a) {
          double v = rv[fc + a];
          for (int b = 0; b < a; ++b) v = ds(v, dm(xg[jj * 8 + b], M[(size_t)(fc + b) * ld + fc + a]));
          v = __ddiv_rn(v, M[(size_t)(fc + a) * ld + fc + a]);
          xg[jj * 8 + a] = v;
          rv[fc + a] = v;
        }
      }
      __syncthreads();
      const int rem = w - fc - g;
      for (int idx = threadIdx.x; idx < rem * kk; idx += blockDim.x) {
        const int q = fc + g + idx % rem, jj = idx / rem;
        double v = rhs[jj * w + q];
        for (int b = 0; b < g; ++b) v = ds(v, dm(xg[jj * 8 + b], M[(size_t)(fc + b) * ld + q]));
        rhs[jj * w + q] = v;
      }
      __syncthreads();
      fc += g;
    }
    for (int idx = threadIdx.x; idx < w * kk; idx += blockDim.x) {
      const int q = idx % w, jj = idx / w;
      x[(size_t)(j0 + jj) * n + c0 + q] = rhs[jj * w + q];
    }
    __syncthreads();
  }
}

// Transposed: per supernode column j, x_j minus the off-block rows'
// products in storage order; then the diagonal block's transpose backward.
__global__ void __launch_bounds__(kSnBlock)
k_sn_transposed(const int *__restrict__ lev_set, int base, const int *__restrict__ c0s, const int *__restrict__ nrs,
                const int *__restrict__ rbs, const long long *__restrict__ vbs, const int *__restrict__ rows,
                const double *__restrict__ Lx, double *__restrict__ x, int n, int k) {
  __shared__ double rhs[kSnSmem];
  const int t = lev_set[base + blockIdx.x];
  const int c0 = c0s[t], w = c0s[t + 1] - c0, ld = nrs[t];
  const int *rw = rows + rbs[t];
  const double *M = Lx + vbs[t];
  const int kc = max(1, min(k, kSnSmem / w));
  for (int j0 = 0; j0 < k; j0 += kc) {
    const int kk = min(kc, k - j0);
    for (int idx = threadIdx.x; idx < w * kk; idx += blockDim.x) {
      const int q = idx % w, jj = idx / w;
      const double *xc = x + (size_t)(j0 + jj) * n;
      double acc = xc[c0 + q];
      for (int r = w; r < ld; ++r) acc = ds(acc, dm(M[(size_t)q * ld + r], xc[rw[r]]));
      rhs[jj * w + q] = acc;
    }
    __syncthreads();
    for (int q = w - 1; q >= 0; --q) {
      for (int jj = threadIdx.x; jj < kk; jj += blockDim.x)
        rhs[jj * w + q] = __ddiv_rn(rhs[jj * w + q], M[(size_t)q * ld + q]);
      __syncthreads();
      for (int idx = threadIdx.x; idx < q * kk; idx += blockDim.x) {
        const int i = idx % q, jj = idx / q;
        rhs[jj * w + i] = ds(rhs[jj * w + i], dm(M[(size_t)i * ld + q], rhs[jj * w + q]));
      }
      __syncthreads();
    }
    for (int idx = threadIdx.x; idx < w * kk; idx += blockDim.x) {
      const int q = idx % w, jj = idx / w;
      x[(size_t)(j0 + jj) * n + c0 + q] = rhs[jj * w + q];
    }
    __syncthreads();
  }
}

// Levels of a DAG over supernodes given as successor lists in increasing
// node order (forward) or predecessor lists in decreasing order (backward).
void levels_from(const std::vector<int> &lev, int nsup, std::vector<int> &ptr, std::vector<int> &set) {
  int nl = 0;
  for (int v : lev) nl = std::max(nl, v + 1);
  ptr.assign(nl + 1, 0);
  for (int v : lev) ptr[v + 1]++;
  for (int l = 0; l < nl; ++l) ptr[l + 1] += ptr[l];
  set.assign(nsup, 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int s = 0; s < nsup; ++s) set[fill[lev[s]]++] = s;
}

gbsym_sn_s *sn_build(int n, const size_t *Lp, const int *Li, const double *Lx, const size_t *Li_ptr,
                     const int *sup2col, int nsup, cudaStream_t s) {
  GB_CHECK(n >= 0 && nsup >= 0, GBSYM_ERR_SIZE);
  GB_CHECK(n == 0 || (Lp && Li && Lx && Li_ptr && sup2col), GBSYM_ERR_NULL_ARG);
  GB_CHECK(nsup > 0 || n == 0, GBSYM_ERR_BAD_MATRIX);
  std::unique_ptr<gbsym_sn_s> t(new gbsym_sn_s());
  t->n = n;
  t->nsup = nsup;
  if (n == 0) return t.release();
  GB_CHECK(sup2col[0] == 0 && sup2col[nsup] == n, GBSYM_ERR_BAD_MATRIX);
  std::vector<int> c0(nsup + 1), nr(nsup), rb(nsup);
  std::vector<long long> vb(nsup);
  std::vector<int> col2sup(n);
  size_t nvals = 0;
  for (int q = 0; q < nsup; ++q) {
    const int a = sup2col[q], z = sup2col[q + 1];
    GB_CHECK(z > a, GBSYM_ERR_BAD_MATRIX);
    const size_t r0 = Li_ptr[a], r1 = Li_ptr[z];
    GB_CHECK(r1 >= r0 + (size_t)(z - a) && r1 - r0 < (size_t)1 << 30, GBSYM_ERR_BAD_MATRIX);
    c0[q] = a;
    nr[q] = (int)(r1 - r0);
    rb[q] = (int)r0;
    vb[q] = (long long)Lp[a];
    for (int j = 0; j < z - a; ++j) {
      GB_CHECK(Li[r0 + j] == a + j, GBSYM_ERR_BAD_MATRIX);  // the diagonal block's rows first
      col2sup[a + j] = q;
    }
    for (size_t k = r0 + (z - a); k < r1; ++k)  // off-block rows below the supernode, ascending
      GB_CHECK(Li[k] >= z && Li[k] < n && (k == r0 + (z - a) || Li[k] > Li[k - 1]), GBSYM_ERR_BAD_MATRIX);
    nvals = std::max(nvals, (size_t)Lp[a] + (r1 - r0) * (size_t)(z - a));
    t->max_w = std::max(t->max_w, z - a);
  }
  c0[nsup] = n;
  GB_CHECK(t->max_w <= kSnSmem, GBSYM_ERR_UNSUPPORTED);
  const size_t nrows = Li_ptr[n];
  // forward pull lists (sources ascending) and both level schedules
  std::vector<int> cnt(n + 1, 0), flev(nsup, 0), blev(nsup, 0);
  for (int q = 0; q < nsup; ++q) {
    const int w = c0[q + 1] - c0[q];
    for (int k = w; k < nr[q]; ++k) {
      const int r = Li[rb[q] + k];
      cnt[r + 1]++;
      flev[col2sup[r]] = std::max(flev[col2sup[r]], flev[q] + 1);
    }
  }
  for (int q = nsup - 1; q >= 0; --q) {
    const int w = c0[q + 1] - c0[q];
    for (int k = w; k < nr[q]; ++k) blev[q] = std::max(blev[q], blev[col2sup[Li[rb[q] + k]]] + 1);
  }
  for (int r = 0; r < n; ++r) cnt[r + 1] += cnt[r];
  std::vector<int> psrc(std::max(cnt[n], 1)), pk(std::max(cnt[n], 1));
  {
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int q = 0; q < nsup; ++q) {
      const int w = c0[q + 1] - c0[q];
      for (int k = w; k < nr[q]; ++k) {
        const int r = Li[rb[q] + k];
        psrc[fill[r]] = q;
        pk[fill[r]] = k;
        fill[r]++;
      }
    }
  }
  std::vector<int> lset, bset;
  levels_from(flev, nsup, t->h_lev_ptr, lset);
  levels_from(blev, nsup, t->h_blev_ptr, bset);
  t->nlev = (int)t->h_lev_ptr.size() - 1;
  t->nblev = (int)t->h_blev_ptr.size() - 1;
  upload(t->c0, c0.data(), c0.size(), false, s);
  upload(t->nr, nr.data(), nr.size(), false, s);
  upload(t->rb, rb.data(), rb.size(), false, s);
  upload(t->vb, vb.data(), vb.size(), false, s);
  upload(t->rows, Li, nrows, false, s);
  upload(t->vals, Lx, nvals, false, s);
  upload(t->pull_ptr, cnt.data(), cnt.size(), false, s);
  upload(t->pull_src, psrc.data(), psrc.size(), false, s);
  upload(t->pull_k, pk.data(), pk.size(), false, s);
  upload(t->lev_set, lset.data(), lset.size(), false, s);
  upload(t->blev_set, bset.data(), bset.size(), false, s);
  GB_CUDA(cudaStreamSynchronize(s));
  return t.release();
}

void sn_solve(gbsym_sn_s *t, double *x, int k, bool transposed, cudaStream_t s) {
  if (t->n == 0 || k == 0) return;
  if (!transposed) {
    for (int l = 0; l < t->nlev; ++l) {
      const int a = t->h_lev_ptr[l], z = t->h_lev_ptr[l + 1];
      k_sn_forward<<<z - a, kSnBlock, 0, s>>>(t->lev_set.p, a, t->c0.p, t->nr.p, t->vb.p, t->vals.p,
                                              t->pull_ptr.p, t->pull_src.p, t->pull_k.p, x, t->n, k);
      check_launch();
    }
  } else {
    // backward level 0 holds the supernodes whose rows below are all final
    // (none below them): they go first
    for (int l = 0; l < t->nblev; ++l) {
      const int a = t->h_blev_ptr[l], z = t->h_blev_ptr[l + 1];
      k_sn_transposed<<<z - a, kSnBlock, 0, s>>>(t->blev_set.p, a, t->c0.p, t->nr.p, t->rb.p, t->vb.p,
                                                 t->rows.p, t->vals.p, x, t->n, k);
      check_launch();
    }
  }
}

// Every supernode once; each dependency finished in an earlier coarse
// level, or earlier in the same partition (partition order is serial).
void sn_validate_lbc(const gbsym_sn_s *t, const size_t *Li_ptr, const int *Li, const int *sup2col, int levels,
                     const int *level_ptr, const int *par_ptr, const int *partition, bool transposed) {
  const int ns = t->nsup;
  GB_CHECK(levels >= 0 && level_ptr && par_ptr && partition, GBSYM_ERR_NULL_ARG);
  std::vector<int> lvl(ns, -1), pos(ns, -1), part(ns, -1);
  int seen = 0;
  for (int l = 0; l < levels; ++l)
    for (int p = level_ptr[l]; p < level_ptr[l + 1]; ++p)
      for (int q = par_ptr[p]; q < par_ptr[p + 1]; ++q) {
        const int v = partition[q];
        GB_CHECK(v >= 0 && v < ns && lvl[v] < 0, GBSYM_ERR_BAD_SCHEDULE);
        lvl[v] = transposed ? levels - 1 - l : l;
        pos[v] = transposed ? -q : q;
        part[v] = p;
        ++seen;
      }
  GB_CHECK(seen == ns, GBSYM_ERR_BAD_SCHEDULE);
  std::vector<int> col2sup(t->n);
  for (int q = 0; q < ns; ++q)
    for (int c = sup2col[q]; c < sup2col[q + 1]; ++c) col2sup[c] = q;
  for (int q = 0; q < ns; ++q) {
    const int a = sup2col[q], z = sup2col[q + 1];
    for (size_t k = Li_ptr[a] + (z - a); k < Li_ptr[z]; ++k) {
      const int dst = col2sup[Li[k]];  // q must finish before dst (forward); after it (transposed)
      const int before = transposed ? dst : q, after = transposed ? q : dst;
      GB_CHECK(lvl[before] < lvl[after] || (part[before] == part[after] && pos[before] < pos[after]),
               GBSYM_ERR_BAD_SCHEDULE);
    }
  }
}

void sn_dropin(int n, const size_t *Lp, const int *Li, const double *Lx, const size_t *Li_ptr, const int *sup2col,
               int supNo, double *x, int k, bool transposed, int levels, const int *level_ptr, const int *par_ptr,
               const int *partition) {
  GB_CHECK(k >= 0, GBSYM_ERR_SIZE);
  if (n == 0 || k == 0) return;
  GB_CHECK(x, GBSYM_ERR_NULL_ARG);
  cudaStream_t s = thread_stream();
  std::unique_ptr<gbsym_sn_s> t(sn_build(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, s));
  if (par_ptr) sn_validate_lbc(t.get(), Li_ptr, Li, sup2col, levels, level_ptr, par_ptr, partition, transposed);
  DBuf<double> dx;
  upload(dx, x, (size_t)n * k, false, s);
  sn_solve(t.get(), dx.p, k, transposed, s);
  GB_CUDA(cudaMemcpyAsync(x, dx.p, (size_t)n * k * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
}

// A plain level set over supernodes, validated as the one-part-per-node LBC
// schedule it is.
void sn_dropin_levels(int n, const size_t *Lp, const int *Li, const double *Lx, const size_t *Li_ptr,
                      const int *sup2col, int supNo, double *x, int k, bool transposed, int levels,
                      const int *level_ptr, const int *level_set) {
  GB_CHECK(n == 0 || (level_ptr && level_set), GBSYM_ERR_NULL_ARG);
  std::vector<int> pp(supNo + 1);
  for (int q = 0; q <= supNo; ++q) pp[q] = q;
  sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, k, transposed, levels, level_ptr, n ? pp.data() : nullptr,
            level_set);
}

int status_to_int() { return last_error() == GBSYM_OK ? 1 : 0; }

}  // namespace
}  // namespace gbsym

using namespace gbsym;

extern "C" {

int gbsym_sn_create(gbsym_sn *out, int n, const size_t *Lp, const int *Li, const double *Lx, const size_t *Li_ptr,
                    const int *sup2col, int supNo, void *stream) {
  if (!out) return GBSYM_ERR_NULL_ARG;
  *out = nullptr;
  return guarded([&] { *out = sn_build(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, (cudaStream_t)stream); });
}

int gbsym_sn_destroy(gbsym_sn t) {
  delete t;
  return GBSYM_OK;
}

int gbsym_sn_levels(gbsym_sn t, int *forward_levels, int *transposed_levels) {
  if (!t) return GBSYM_ERR_NULL_ARG;
  if (forward_levels) *forward_levels = t->nlev;
  if (transposed_levels) *transposed_levels = t->nblev;
  return GBSYM_OK;
}

int gbsym_sn_solve(gbsym_sn t, double *x, int k, int transposed, void *stream) {
  if (!t || (!x && t->n && k)) return GBSYM_ERR_NULL_ARG;
  if (k < 0) return GBSYM_ERR_SIZE;
  return guarded([&] { sn_solve(t, x, k, transposed != 0, (cudaStream_t)stream); });
}

#define GBSYM_SN_ARGS                                                                                      \
  int n, size_t *Lp, int *Li, double *Lx, int NNZ, size_t *Li_ptr, int *col2sup, int *sup2col, int supNo, \
      double *x

int gbsym_parsy_blockedLsolve(GBSYM_SN_ARGS) {
  (void)NNZ;
  (void)col2sup;
  set_last_error(guarded([&] { sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, 1, false, 0, nullptr, nullptr, nullptr); }));
  return status_to_int();
}

int gbsym_parsy_blockedLTsolve(GBSYM_SN_ARGS) {
  (void)NNZ;
  (void)col2sup;
  set_last_error(guarded([&] { sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, 1, true, 0, nullptr, nullptr, nullptr); }));
  return status_to_int();
}

int gbsym_parsy_blockedLsolve_mrhs(GBSYM_SN_ARGS, int n_rhs, int max_col) {
  (void)NNZ;
  (void)col2sup;
  (void)max_col;
  set_last_error(guarded([&] { sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, n_rhs, false, 0, nullptr, nullptr, nullptr); }));
  return status_to_int();
}

int gbsym_parsy_blockedLTsolve_mrhs(GBSYM_SN_ARGS, int m_rhs, int max_col) {
  (void)NNZ;
  (void)col2sup;
  (void)max_col;
  set_last_error(guarded([&] { sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, m_rhs, true, 0, nullptr, nullptr, nullptr); }));
  return status_to_int();
}

int gbsym_parsy_leveledBlockedLsolve(GBSYM_SN_ARGS, int levels, int *levelPtr, int *levelSet, int chunk) {
  (void)NNZ;
  (void)col2sup;
  (void)chunk;
  set_last_error(guarded([&] {
    sn_dropin_levels(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, 1, false, levels, levelPtr, levelSet);
  }));
  return status_to_int();
}

int gbsym_parsy_H2LeveledBlockedLsolve(GBSYM_SN_ARGS, int levels, int *levelPtr, int *levelSet, int parts,
                                       int *parPtr, int *partition, int chunk) {
  (void)NNZ;
  (void)col2sup;
  (void)levelSet;
  (void)parts;
  (void)chunk;
  set_last_error(guarded([&] {
    GB_CHECK(n == 0 || (levelPtr && parPtr && partition), GBSYM_ERR_NULL_ARG);
    sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, 1, false, levels, levelPtr, n ? parPtr : nullptr, partition);
  }));
  return status_to_int();
}

int gbsym_parsy_H2LeveledBlockedLTsolve(GBSYM_SN_ARGS, int levels, int *levelPtr, int *levelSet, int parts,
                                        int *parPtr, int *partition, int chunk) {
  (void)NNZ;
  (void)col2sup;
  (void)levelSet;
  (void)parts;
  (void)chunk;
  set_last_error(guarded([&] {
    GB_CHECK(n == 0 || (levelPtr && parPtr && partition), GBSYM_ERR_NULL_ARG);
    sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, 1, true, levels, levelPtr, n ? parPtr : nullptr, partition);
  }));
  return status_to_int();
}

int gbsym_parsy_H2LeveledBlockedLsolve_mrhs(GBSYM_SN_ARGS, int n_rhs, int levels, int *levelPtr, int *levelSet,
                                            int parts, int *parPtr, int *partition, int chunk, int max_col) {
  (void)NNZ;
  (void)col2sup;
  (void)levelSet;
  (void)parts;
  (void)chunk;
  (void)max_col;
  set_last_error(guarded([&] {
    GB_CHECK(n == 0 || (levelPtr && parPtr && partition), GBSYM_ERR_NULL_ARG);
    sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, n_rhs, false, levels, levelPtr, n ? parPtr : nullptr,
              partition);
  }));
  return status_to_int();
}

int gbsym_parsy_H2LeveledBlockedLTsolve_mrhs(GBSYM_SN_ARGS, int m_rhs, int levels, int *levelPtr, int *levelSet,
                                             int parts, int *parPtr, int *partition, int chunk, int max_col) {
  (void)NNZ;
  (void)col2sup;
  (void)levelSet;
  (void)parts;
  (void)chunk;
  (void)max_col;
  set_last_error(guarded([&] {
    GB_CHECK(n == 0 || (levelPtr && parPtr && partition), GBSYM_ERR_NULL_ARG);
    sn_dropin(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, x, m_rhs, true, levels, levelPtr, n ? parPtr : nullptr,
              partition);
  }));
  return status_to_int();
}

}  // extern "C"
