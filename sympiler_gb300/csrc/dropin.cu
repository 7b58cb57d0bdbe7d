// dropin.cu -- the reference-signature entry points (host memory in, host
// memory out) and the library runtime: per-thread streams, status, launch
// accounting.
//
// Each drop-in uploads the caller's arrays, builds a level-packed plan on
// the GPU (validating any schedule the caller passes), runs the GPU
// executor and copies the result back before returning, so a caller of the
// reference (sparse_blas_lib.h, Triangular_CSC.h, mgmres.hpp) sees the same
// in-place semantics.  Repeated solves with one matrix should use the plan
// API instead, which keeps the matrix resident.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "csr.cuh"
#include "tri.cuh"

namespace gbsym {

std::atomic<unsigned long long> g_launches{0};
static thread_local int t_last_error = GBSYM_OK;
void set_last_error(int code) { t_last_error = code; }
int last_error() { return t_last_error; }

cudaStream_t thread_stream() {
  struct PerThread {
    std::vector<cudaStream_t> streams;
  };
  static thread_local PerThread pt;
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if ((int)pt.streams.size() <= dev) pt.streams.resize(dev + 1, nullptr);
  if (!pt.streams[dev]) GB_CUDA(cudaStreamCreateWithFlags(&pt.streams[dev], cudaStreamNonBlocking));
  return pt.streams[dev];
}

// SM count of the current device, cached per device.  The entries are
// atomics: any host thread may fill one (they all store the same value).
int num_sms() {
  static std::atomic<int> cache[64];
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 64) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c) return c;
  }
  int v = 0;
  GB_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
  if (dev < 64) cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

// ---------------------------------------------------------------------------
// helpers
struct HostLevels {
  int levels;
  const int *ptr;
  const int *set;
};
struct HostLbc {
  int level_no;
  const int *level_ptr, *par_ptr, *partition;
};

// ---------------------------------------------------------------------------
// Opt-in plan cache of the drop-ins.  A reference caller that solves with
// one matrix in a loop (Cholesky::solve, the demo's repeated runs) would
// otherwise pay for the upload, the validation and the plan build on every
// call.  With the cache on, a drop-in whose arguments name the same arrays
// (the same pointers, n, entry count, kind and schedule arrays) on the same
// device under the same caller version reuses the plan it built the first
// time, after checking nothing: the caller declares, by changing the
// version, that any cached matrix's arrays changed in place.  Plans are
// evicted least recently used beyond the capacity.  A cached plan is used
// by one call at a time (its own lock); other matrices proceed in parallel.
struct CacheKey {
  int dev = 0, kind = 0, n = 0, nnz = 0, levels = 0;
  const void *ptr[8] = {};
  unsigned long long version = 0;
  bool operator==(const CacheKey &o) const {
    return dev == o.dev && kind == o.kind && n == o.n && nnz == o.nnz && levels == o.levels &&
           version == o.version && std::memcmp(ptr, o.ptr, sizeof(ptr)) == 0;
  }
};
struct CachedPlan {
  CacheKey key;
  std::unique_ptr<gbsym_tri_s> plan;
  std::mutex use;
  unsigned long long last = 0;
};
static std::mutex g_cache_mu;
static std::vector<std::shared_ptr<CachedPlan>> g_cache;
static int g_cache_cap = 0;
static unsigned long long g_cache_version = 0, g_cache_clock = 0;

static CacheKey cache_key(int n, int nnz, int kind, const void *p, const void *i, const void *v,
                          const void *diags, const HostLevels *lv, const HostLbc *lbc) {
  CacheKey k;
  GB_CUDA(cudaGetDevice(&k.dev));
  k.kind = kind;
  k.n = n;
  k.nnz = nnz;
  k.ptr[0] = p;
  k.ptr[1] = i;
  k.ptr[2] = v;
  k.ptr[3] = diags;
  if (lv) {
    k.levels = lv->levels;
    k.ptr[4] = lv->ptr;
    k.ptr[5] = lv->set;
  }
  if (lbc) {
    k.levels = -1 - lbc->level_no;
    k.ptr[4] = lbc->level_ptr;
    k.ptr[5] = lbc->par_ptr;
    k.ptr[6] = lbc->partition;
  }
  std::lock_guard<std::mutex> lk(g_cache_mu);
  k.version = g_cache_version;
  return k;
}

static std::shared_ptr<CachedPlan> cache_find(const CacheKey &k) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  if (g_cache_cap <= 0) return nullptr;
  for (auto &e : g_cache)
    if (e->key == k) {
      e->last = ++g_cache_clock;
      return e;
    }
  return nullptr;
}

static void cache_put(const CacheKey &k, std::unique_ptr<gbsym_tri_s> plan) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  if (g_cache_cap <= 0 || k.version != g_cache_version) return;
  auto e = std::make_shared<CachedPlan>();
  e->key = k;
  e->plan = std::move(plan);
  e->last = ++g_cache_clock;
  g_cache.push_back(std::move(e));
  while ((int)g_cache.size() > g_cache_cap) {
    auto lru = std::min_element(g_cache.begin(), g_cache.end(),
                                [](const std::shared_ptr<CachedPlan> &a, const std::shared_ptr<CachedPlan> &b) {
                                  return a->last < b->last;
                                });
    g_cache.erase(lru);  // a call still using it keeps it alive
  }
}

// Solve on a plan the cache holds: upload x (and b), solve, download.
static void cached_solve(CachedPlan &c, int n, double *x, const double *b, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(c.use);
  DBuf<double> dx, db;
  upload(dx, x, n, false, s);
  if (b) upload(db, b, n, false, s);
  tri_solve_rowmajor(c.plan.get(), dx.p, b ? db.p : nullptr, 1, GBSYM_F64, s);
  const int code = tri_read_error(c.plan.get(), s);
  if (code) throw Err{code};
  GB_CUDA(cudaMemcpyAsync(x, dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
}

// Solve one triangle stored as (p, i, v[, diags]) of the given kind, in
// place on host x (b non-null: the redundant row formula).
static void tri_dropin(int n, const int *p, const int *i, const double *v, const int *diags,
                       int kind, double *x, const double *b, const HostLevels *lv,
                       const HostLbc *lbc) {
  GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
  if (n == 0) return;
  GB_CHECK(p && i && v && x, GBSYM_ERR_NULL_ARG);
  cudaStream_t s = thread_stream();
  const int nnz = p[n];
  GB_CHECK(nnz >= 0, GBSYM_ERR_BAD_MATRIX);
  const CacheKey key = cache_key(n, nnz, kind, p, i, v, diags, lv, lbc);
  if (auto c = cache_find(key)) {
    cached_solve(*c, n, x, b, s);
    return;
  }
  DBuf<int> dp, di, dd, dls;
  DBuf<double> dv, dx, db;
  upload(dp, p, n + 1, false, s);
  upload(di, i, nnz, false, s);
  upload(dv, v, nnz, false, s);
  if (diags) upload(dd, diags, n, false, s);
  if (lv) upload(dls, lv->set, n, false, s);
  if (lbc) {
    validate_matrix(n, dp.p, di.p, dd.p, kind, s);
    validate_lbc(n, dp.p, di.p, dd.p, kind, lbc->level_no, lbc->level_ptr, lbc->par_ptr,
                 lbc->partition, s);
  }
  std::unique_ptr<gbsym_tri_s> t(tri_build(n, dp.p, di.p, dv.p, dd.p, kind, GBSYM_F64,
                                           lv ? lv->ptr : nullptr, lv ? dls.p : nullptr,
                                           lv ? lv->levels : 0, s));
  upload(dx, x, n, false, s);
  if (b) upload(db, b, n, false, s);
  tri_solve_rowmajor(t.get(), dx.p, b ? db.p : nullptr, 1, GBSYM_F64, s);
  const int code = tri_read_error(t.get(), s);
  if (code) throw Err{code};
  GB_CUDA(cudaMemcpyAsync(x, dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  cache_put(key, std::move(t));
}

// Lower-triangular CSC (diagonal first in each column) -> CSR pull form
// (diagonal last in each row) on the device.  The transposed rows list
// columns in ascending order, which is the order the column-push solve
// applies its updates to each row, so the pull solve reproduces it.
struct DevCsr {
  DBuf<int> p, i;
  DBuf<double> x;
};

__global__ void k_gather_vals(long long m, const double *__restrict__ src, const int *__restrict__ idx,
                              double *dst) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m;
       t += (long long)gridDim.x * blockDim.x)
    dst[t] = src[idx[t]];
}

static void csc_lower_to_csr(int n, const int *Lp, const int *Li, const double *Lx, DevCsr &out,
                             cudaStream_t s) {
  const int nnz = Lp[n];
  for (int j = 0; j < n; ++j) {
    GB_CHECK(Lp[j] <= Lp[j + 1], GBSYM_ERR_BAD_MATRIX);
    GB_CHECK(Lp[j] < Lp[j + 1] && Li[Lp[j]] == j, GBSYM_ERR_BAD_MATRIX);  // diagonal first
    for (int e = Lp[j] + 1; e < Lp[j + 1]; ++e)
      GB_CHECK(Li[e] > j && Li[e] < n, GBSYM_ERR_BAD_MATRIX);
  }
  DBuf<int> dp, di;
  DBuf<double> dx;
  upload(dp, Lp, n + 1, false, s);
  upload(di, Li, nnz, false, s);
  upload(dx, Lx, nnz, false, s);
  Transposed T;
  transpose_pattern(n, nnz, dp.p, di.p, T, s);
  out.p = std::move(T.rp);
  out.i = std::move(T.ci);
  out.x.alloc(nnz);
  if (nnz) {
    k_gather_vals<<<std::min(div_up(nnz, 256), num_sms() * 8), 256, 0, s>>>(nnz, dx.p, T.src.p,
                                                                             out.x.p);
    check_launch();
  }
  GB_CUDA(cudaStreamSynchronize(s));
}

static void csc_dropin(int n, const int *Lp, const int *Li, const double *Lx, double *x,
                       const HostLevels *lv, const HostLbc *lbc) {
  GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
  if (n == 0) return;
  GB_CHECK(Lp && Li && Lx && x, GBSYM_ERR_NULL_ARG);
  cudaStream_t s = thread_stream();
  const CacheKey key = cache_key(n, Lp[n], GBSYM_LOWER_CSC, Lp, Li, Lx, nullptr, lv, lbc);
  if (auto c = cache_find(key)) {
    cached_solve(*c, n, x, nullptr, s);
    return;
  }
  DevCsr L;
  csc_lower_to_csr(n, Lp, Li, Lx, L, s);
  DBuf<int> dls;
  if (lv) upload(dls, lv->set, n, false, s);
  if (lbc)
    validate_lbc(n, L.p.p, L.i.p, nullptr, GBSYM_LOWER_DIAG_LAST, lbc->level_no, lbc->level_ptr,
                 lbc->par_ptr, lbc->partition, s);
  std::unique_ptr<gbsym_tri_s> t(tri_build(n, L.p.p, L.i.p, L.x.p, nullptr, GBSYM_LOWER_DIAG_LAST,
                                           GBSYM_F64, lv ? lv->ptr : nullptr,
                                           lv ? dls.p : nullptr, lv ? lv->levels : 0, s));
  DBuf<double> dx;
  upload(dx, x, n, false, s);
  tri_solve_rowmajor(t.get(), dx.p, nullptr, 1, GBSYM_F64, s);
  const int code = tri_read_error(t.get(), s);
  if (code) throw Err{code};
  GB_CUDA(cudaMemcpyAsync(x, dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  cache_put(key, std::move(t));
}

__global__ void k_div_by_vec(double *__restrict__ x, const double *__restrict__ d, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    x[t] = __ddiv_rn(x[t], d[t]);
}

// parsy's simplicial solve phases (solve_phase.cpp:23-37): lsolve on the
// CSC of L (the column-push order, reproduced by the pull form), x /= d
// for LDL^T (IEEE division, as scale_vec_vec), then ltsolve on the same
// CSC read as an upper CSR with the diagonal first.
static void simplicial_phase(int n, const int *Lp, const int *Li, const double *Lx, const double *d, double *x) {
  GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
  if (n == 0) return;
  GB_CHECK(Lp && Li && Lx && x, GBSYM_ERR_NULL_ARG);
  cudaStream_t s = thread_stream();
  DevCsr L;
  csc_lower_to_csr(n, Lp, Li, Lx, L, s);
  const int nnz = Lp[n];
  DBuf<int> cp, ci;
  DBuf<double> cx, dx, dd;
  upload(cp, Lp, n + 1, false, s);
  upload(ci, Li, nnz, false, s);
  upload(cx, Lx, nnz, false, s);
  std::unique_ptr<gbsym_tri_s> lo(tri_build(n, L.p.p, L.i.p, L.x.p, nullptr, GBSYM_LOWER_DIAG_LAST, GBSYM_F64,
                                            nullptr, nullptr, 0, s));
  std::unique_ptr<gbsym_tri_s> up(tri_build(n, cp.p, ci.p, cx.p, nullptr, GBSYM_UPPER_DIAG_FIRST, GBSYM_F64,
                                            nullptr, nullptr, 0, s));
  upload(dx, x, n, false, s);
  tri_solve_rowmajor(lo.get(), dx.p, nullptr, 1, GBSYM_F64, s);
  if (d) {
    upload(dd, d, n, false, s);
    k_div_by_vec<<<std::max(1, std::min(div_up(n, 256), num_sms() * 8)), 256, 0, s>>>(dx.p, dd.p, n);
    check_launch();
  }
  tri_solve_rowmajor(up.get(), dx.p, nullptr, 1, GBSYM_F64, s);
  int code = tri_read_error(lo.get(), s);
  if (!code) code = tri_read_error(up.get(), s);
  if (code) throw Err{code};
  GB_CUDA(cudaMemcpyAsync(x, dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
}

static int max_col_plus_one(int n, const int *Ap, const int *Ai) {
  int m = n;
  for (int e = Ap[0]; e < Ap[n]; ++e) m = std::max(m, Ai[e] + 1);
  return m;
}

static void spmv_dropin(int n, const int *Ap, const int *Ai, const double *Ax, const double *x,
                        const double *y, double *z, double a, double b, bool accumulate) {
  GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
  if (n == 0) return;
  GB_CHECK(Ap && Ai && Ax && x && z && (!accumulate || y), GBSYM_ERR_NULL_ARG);
  cudaStream_t s = thread_stream();
  const int ncols = max_col_plus_one(n, Ap, Ai);
  std::unique_ptr<gbsym_csr_s> A(csr_build(n, ncols, Ap, Ai, Ax, GBSYM_F64, false, s));
  DBuf<double> dx, dy, dz;
  upload(dx, x, ncols, false, s);
  if (accumulate) {
    upload(dy, y, n, false, s);
    upload(dz, z, n, false, s);
    csr_spmv_axpby(A.get(), dx.p, dy.p, dz.p, a, b, s);
  } else {
    dz.alloc(n);
    csr_spmv(A.get(), dx.p, dz.p, GBSYM_F64, s);
  }
  GB_CUDA(cudaMemcpyAsync(z, dz.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
}

static void host_check_pattern(int n, const int *p, const int *i) {
  GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
  if (n == 0) return;
  GB_CHECK(p && i, GBSYM_ERR_NULL_ARG);
  for (int r = 0; r < n; ++r) {
    GB_CHECK(p[r] <= p[r + 1], GBSYM_ERR_BAD_MATRIX);
    for (int e = p[r]; e < p[r + 1]; ++e) GB_CHECK(i[e] >= 0 && i[e] < n, GBSYM_ERR_BAD_MATRIX);
  }
}

// Level set of a pattern on the GPU, returned in malloc'd host buffers.
static int levelset_dropin(int n, const int *p, const int *i, bool csc, bool upper,
                           int **level_ptr, int **level_set) {
  GB_CHECK(level_ptr && level_set, GBSYM_ERR_NULL_ARG);
  *level_ptr = nullptr;
  *level_set = nullptr;
  host_check_pattern(n, p, i);
  cudaStream_t s = thread_stream();
  int nlev = 0;
  DBuf<int> lp, ls;
  if (n > 0) {
    DBuf<int> dp, di;
    upload(dp, p, n + 1, false, s);
    upload(di, i, p[n], false, s);
    if (csc) {
      Transposed T;
      transpose_pattern(n, p[n], dp.p, di.p, T, s);
      nlev = build_levels_device(n, T.rp.p, T.ci.p, nullptr, upper ? kKindStrictUpper : kKindStrictLower,
                                 lp, ls, s);
    } else {
      nlev = build_levels_device(n, dp.p, di.p, nullptr, upper ? kKindStrictUpper : kKindStrictLower,
                                 lp, ls, s);
    }
  }
  int *hp = (int *)std::malloc(sizeof(int) * (size_t)(nlev + 1));
  int *hs = (int *)std::malloc(sizeof(int) * (size_t)std::max(n, 1));
  GB_CHECK(hp && hs, GBSYM_ERR_SIZE);
  hp[0] = 0;
  if (n > 0) {
    GB_CUDA(cudaMemcpyAsync(hp, lp.p, (nlev + 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaMemcpyAsync(hs, ls.p, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
  }
  *level_ptr = hp;
  *level_set = hs;
  return nlev;
}

}  // namespace gbsym

using namespace gbsym;

template <class F>
static void record(F &&f) {
  set_last_error(guarded(std::forward<F>(f)));
}

extern "C" {

int gbsym_last_error(void) { return last_error(); }

const char *gbsym_status_string(int status) {
  switch (status) {
    case GBSYM_OK: return "ok";
    case GBSYM_ERR_NULL_ARG: return "null argument";
    case GBSYM_ERR_BAD_SCHEDULE: return "schedule violates the dependency DAG";
    case GBSYM_ERR_PIVOT: return "zero or non-positive pivot";
    case GBSYM_ERR_TIMEOUT: return "bounded device wait timed out";
    case GBSYM_ERR_CUDA: return "CUDA runtime error";
    case GBSYM_ERR_BAD_MATRIX: return "malformed matrix";
    case GBSYM_ERR_SIZE: return "size out of range";
    case GBSYM_ERR_NOT_CONVERGED: return "iteration limit reached";
    case GBSYM_ERR_UNSUPPORTED: return "unsupported option";
    default: return "unknown status";
  }
}

void *gbsym_alloc(size_t bytes) { return bytes ? std::malloc(bytes) : nullptr; }
void gbsym_free(void *p) { std::free(p); }

unsigned long long gbsym_kernel_launches(void) { return g_launches.load(); }

int gbsym_dropin_cache(int capacity) {
  if (capacity < 0) return GBSYM_ERR_SIZE;
  std::vector<std::shared_ptr<CachedPlan>> dropped;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache_cap = capacity;
    while ((int)g_cache.size() > capacity) {
      dropped.push_back(std::move(g_cache.back()));
      g_cache.pop_back();
    }
  }
  return GBSYM_OK;  // plans not in use are freed here, as `dropped` goes
}

void gbsym_dropin_cache_version(unsigned long long version) {
  std::vector<std::shared_ptr<CachedPlan>> dropped;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  if (version == g_cache_version) return;
  g_cache_version = version;
  dropped.swap(g_cache);  // no entry can match any more
}

// ---- SpTRSV CSR -----------------------------------------------------------
void gbsym_sptrsv_csr(int n, int *Lp, int *Li, double *Lx, double *x) {
  record([&] { tri_dropin(n, Lp, Li, Lx, nullptr, GBSYM_LOWER_DIAG_LAST, x, nullptr, nullptr, nullptr); });
}

void gbsym_sptrsv_csr_ilu(int n, const int *Lp, const int *Li, const double *Lx, const int *diags,
                          double *x) {
  record([&] {
    GB_CHECK(n == 0 || diags, GBSYM_ERR_NULL_ARG);
    tri_dropin(n, Lp, Li, Lx, diags, GBSYM_ILU_UNIT_LOWER, x, nullptr, nullptr, nullptr);
  });
}

void gbsym_sptrsv_csr_ilu_lbc(int n, const int *Lp, const int *Li, const double *Lx,
                              const int *diags, double *x, const int level_no,
                              const int *level_ptr, const int *par_ptr, const int *partition) {
  record([&] {
    GB_CHECK(n == 0 || diags, GBSYM_ERR_NULL_ARG);
    HostLbc lbc{level_no, level_ptr, par_ptr, partition};
    tri_dropin(n, Lp, Li, Lx, diags, GBSYM_ILU_LOWER_DIV, x, nullptr, nullptr, n ? &lbc : nullptr);
  });
}

void gbsym_sptrsv_csr_levelset(int n, const int *Lp, const int *Li, const double *Lx, double *x,
                               int levels, const int *levelPtr, const int *levelSet) {
  record([&] {
    GB_CHECK(n == 0 || (levelPtr && levelSet), GBSYM_ERR_NULL_ARG);
    HostLevels lv{levels, levelPtr, levelSet};
    tri_dropin(n, Lp, Li, Lx, nullptr, GBSYM_LOWER_DIAG_LAST, x, nullptr, n ? &lv : nullptr, nullptr);
  });
}

void gbsym_sptrsv_csr_lbc(int n, int *Lp, int *Li, double *Lx, double *x, int level_no,
                          int *level_ptr, int *par_ptr, int *partition) {
  record([&] {
    HostLbc lbc{level_no, level_ptr, par_ptr, partition};
    tri_dropin(n, Lp, Li, Lx, nullptr, GBSYM_LOWER_DIAG_LAST, x, nullptr, nullptr, n ? &lbc : nullptr);
  });
}

void gbsym_sptrsv_csr_lbc_redundant(int n, int *Lp, int *Li, double *Lx, double *x, double *b,
                                    int level_no, int *level_ptr, int *par_ptr, int *partition,
                                    double *tmp) {
  (void)tmp;
  record([&] {
    GB_CHECK(n == 0 || b, GBSYM_ERR_NULL_ARG);
    HostLbc lbc{level_no, level_ptr, par_ptr, partition};
    tri_dropin(n, Lp, Li, Lx, nullptr, GBSYM_LOWER_DIAG_LAST, x, b, nullptr, n ? &lbc : nullptr);
  });
}

// ---- SpTRSV CSC -----------------------------------------------------------
void gbsym_sptrsv_csc(int n, int *Lp, int *Li, double *Lx, double *x) {
  record([&] { csc_dropin(n, Lp, Li, Lx, x, nullptr, nullptr); });
}

void gbsym_sptrsv_csc_levelset(int n, int *Lp, int *Li, double *Lx, double *x, int levels,
                               const int *levelptr, const int *levelset) {
  record([&] {
    GB_CHECK(n == 0 || (levelptr && levelset), GBSYM_ERR_NULL_ARG);
    HostLevels lv{levels, levelptr, levelset};
    csc_dropin(n, Lp, Li, Lx, x, n ? &lv : nullptr, nullptr);
  });
}

void gbsym_sptrsv_csc_lbc(int n, int *Lp, int *Li, double *Lx, double *x, int level_no,
                          int *level_ptr, int *par_ptr, int *partition) {
  record([&] {
    HostLbc lbc{level_no, level_ptr, par_ptr, partition};
    csc_dropin(n, Lp, Li, Lx, x, nullptr, n ? &lbc : nullptr);
  });
}

int gbsym_ltsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  if (!Lp || !Li || !x) {
    set_last_error(GBSYM_ERR_NULL_ARG);
    return 0;
  }
  record([&] { tri_dropin(n, Lp, Li, Lx, nullptr, GBSYM_UPPER_DIAG_FIRST, x, nullptr, nullptr, nullptr); });
  return last_error() == GBSYM_OK ? 1 : 0;
}

int gbsym_parsy_lsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  if (!Lp || !Li || !x) {
    set_last_error(GBSYM_ERR_NULL_ARG);
    return 0;
  }
  gbsym_sptrsv_csc(n, Lp, Li, Lx, x);
  return last_error() == GBSYM_OK ? 1 : 0;
}

int gbsym_parsy_ltsolve(int n, int *Lp, int *Li, double *Lx, double *x) {
  return gbsym_ltsolve(n, Lp, Li, Lx, x);
}

void gbsym_parsy_solve_phase_simplicial_ll(int n, int *Lp, int *Li, double *Lx, double *x) {
  record([&] { simplicial_phase(n, Lp, Li, Lx, nullptr, x); });
}

void gbsym_parsy_solve_phase_simplicial_ldl(int n, int *Lp, int *Li, double *Lx, double *d_val, double *x) {
  record([&] {
    GB_CHECK(n <= 0 || d_val, GBSYM_ERR_NULL_ARG);
    simplicial_phase(n, Lp, Li, Lx, d_val, x);
  });
}

int gbsym_parsy_lsolvePar(int n, int *Lp, int *Li, double *Lx, double *x, int levels,
                          int *levelPtr, int *levelSet, int chunk) {
  (void)chunk;
  if (!Lp || !Li || !x) {
    set_last_error(GBSYM_ERR_NULL_ARG);
    return 0;
  }
  gbsym_sptrsv_csc_levelset(n, Lp, Li, Lx, x, levels, levelPtr, levelSet);
  return last_error() == GBSYM_OK ? 1 : 0;
}

int gbsym_parsy_lsolveParH2(int n, int *Lp, int *Li, double *Lx, double *x, int levels,
                            int *levelPtr, int *levelSet, int parts, int *parPtr,
                            int *partition, int chunk) {
  (void)levelSet;
  (void)parts;
  (void)chunk;
  if (!Lp || !Li || !x) {
    set_last_error(GBSYM_ERR_NULL_ARG);
    return 0;
  }
  gbsym_sptrsv_csc_lbc(n, Lp, Li, Lx, x, levels, levelPtr, parPtr, partition);
  return last_error() == GBSYM_OK ? 1 : 0;
}

// ---- SpMV -----------------------------------------------------------------
void gbsym_spmv_csr(int n, const int *Ap, const int *Ai, const double *Ax, const double *x,
                    double *y) {
  record([&] { spmv_dropin(n, Ap, Ai, Ax, x, nullptr, y, 0, 0, false); });
}

void gbsym_spmv_csr_axpby(int n, const int *Ap, const int *Ai, const double *Ax, const double *x,
                          const double *y, double *z, double a, double b) {
  record([&] { spmv_dropin(n, Ap, Ai, Ax, x, y, z, a, b, true); });
}

void gbsym_spmv_csr_parallel(int n, const int *Ap, const int *Ai, const double *Ax,
                             const double *x, double *y) {
  gbsym_spmv_csr(n, Ap, Ai, Ax, x, y);
}

// ---- factor producers and the ILU apply -----------------------------------
// ILU0 of the CSR (Ap, Ai, Ax) with diagonal positions A_diag into l, on the
// GPU.  With an LBC schedule, the schedule is first checked against the
// rows' dependencies (the entries left of each diagonal); ILU0's arithmetic
// per row does not depend on the order rows run in, so the factor is the
// same either way.
static void ilu0_dropin(int n, int nnz, const int *Ap, const int *Ai, const double *Ax,
                        const int *A_diag, double *l, const HostLbc *lbc) {
  GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
  if (n == 0) return;
  GB_CHECK(Ap && Ai && Ax && A_diag && l, GBSYM_ERR_NULL_ARG);
  GB_CHECK(nnz == Ap[n], GBSYM_ERR_BAD_MATRIX);
  cudaStream_t s = thread_stream();
  DBuf<int> dp, di, dd;
  DBuf<double> dx, dl(nnz);
  upload(dp, Ap, n + 1, false, s);
  upload(di, Ai, nnz, false, s);
  upload(dx, Ax, nnz, false, s);
  upload(dd, A_diag, n, false, s);
  if (lbc) {
    validate_matrix(n, dp.p, di.p, dd.p, GBSYM_ILU_UNIT_LOWER, s);
    validate_lbc(n, dp.p, di.p, dd.p, GBSYM_ILU_UNIT_LOWER, lbc->level_no, lbc->level_ptr, lbc->par_ptr,
                 lbc->partition, s);
  }
  int st = guarded([&] { ilu0_device(n, dp.p, di.p, dx.p, dd.p, dl.p, s); });
  if (st == GBSYM_ERR_BAD_MATRIX) throw Err{st};
  GB_CUDA(cudaMemcpyAsync(l, dl.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (st) throw Err{st};
}

// IC0 in place on the upper CSR of A (diagonal first in each row), on the
// GPU.  With an LBC schedule over the columns of L, the schedule is first
// checked against the solve DAG of L: column c must come after every column
// i whose row of the upper CSR holds c.  The updates are applied in the
// serial order whatever the schedule.
static void ic0_dropin(int n, double *val, const int *rowPtr, const int *colIdx, const HostLbc *lbc) {
  GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
  if (n == 0) return;
  GB_CHECK(val && rowPtr && colIdx, GBSYM_ERR_NULL_ARG);
  const int nnz = rowPtr[n];
  GB_CHECK(nnz >= 0, GBSYM_ERR_BAD_MATRIX);
  if (lbc) {
    // structure first, on the host, before any kernel indexes with it
    GB_CHECK(rowPtr[0] == 0, GBSYM_ERR_BAD_MATRIX);
    for (int r = 0; r < n; ++r) {
      GB_CHECK(rowPtr[r] < rowPtr[r + 1] && colIdx[rowPtr[r]] == r, GBSYM_ERR_BAD_MATRIX);
      for (int e = rowPtr[r] + 1; e < rowPtr[r + 1]; ++e)
        GB_CHECK(colIdx[e] > r && colIdx[e] < n, GBSYM_ERR_BAD_MATRIX);
    }
  }
  cudaStream_t s = thread_stream();
  DBuf<int> dp, di;
  DBuf<double> dv;
  upload(dp, rowPtr, n + 1, false, s);
  upload(di, colIdx, nnz, false, s);
  upload(dv, val, nnz, false, s);
  if (lbc) {
    Transposed L;  // CSR of L: row c lists the columns i <= c, diagonal last
    transpose_pattern(n, nnz, dp.p, di.p, L, s);
    validate_lbc(n, L.rp.p, L.ci.p, nullptr, GBSYM_LOWER_DIAG_LAST, lbc->level_no, lbc->level_ptr,
                 lbc->par_ptr, lbc->partition, s);
  }
  int st = guarded([&] { ic0_device(n, dv.p, dp.p, di.p, s); });
  if (st == GBSYM_ERR_BAD_MATRIX) throw Err{st};
  GB_CUDA(cudaMemcpyAsync(val, dv.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (st) throw Err{st};
}

void gbsym_spilu0_csr(int n, int nnz, const int *Ap, const int *Ai, const double *Ax,
                      const int *A_diag, double *l) {
  record([&] { ilu0_dropin(n, nnz, Ap, Ai, Ax, A_diag, l, nullptr); });
}

void gbsym_spilu0_csr_lbc(int n, int nnz, const int *Ap, const int *Ai, const double *Ax,
                          const int *A_diag, double *l, int level_no, const int *level_ptr,
                          const int *par_ptr, const int *partition, int *tempvecs) {
  (void)tempvecs;
  record([&] {
    HostLbc lbc{level_no, level_ptr, par_ptr, partition};
    ilu0_dropin(n, nnz, Ap, Ai, Ax, A_diag, l, n ? &lbc : nullptr);
  });
}

void gbsym_spic0_csr(int n, double *val, int *rowPtr, int *rowIdx) {
  record([&] { ic0_dropin(n, val, rowPtr, rowIdx, nullptr); });
}

void gbsym_spic0_csr_lbc(int n, double *val, int *rowPtr, int *colIdx, int level_no, int *level_ptr,
                         int *par_ptr, int *partition) {
  record([&] {
    HostLbc lbc{level_no, level_ptr, par_ptr, partition};
    ic0_dropin(n, val, rowPtr, colIdx, n ? &lbc : nullptr);
  });
}

void gbsym_parsy_lus_cr(int n, int nz_num, int *ia, int *ja, double *l, int *ua, double *r,
                        double *z) {
  record([&] {
    GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
    if (n == 0) return;
    GB_CHECK(ia && ja && l && ua && r && z, GBSYM_ERR_NULL_ARG);
    GB_CHECK(nz_num == ia[n], GBSYM_ERR_BAD_MATRIX);
    cudaStream_t s = thread_stream();
    DBuf<int> dp, di, dd;
    DBuf<double> dl, dz;
    upload(dp, ia, n + 1, false, s);
    upload(di, ja, nz_num, false, s);
    upload(dl, l, nz_num, false, s);
    upload(dd, ua, n, false, s);
    std::unique_ptr<gbsym_tri_s> lo(tri_build(n, dp.p, di.p, dl.p, dd.p, GBSYM_ILU_UNIT_LOWER,
                                              GBSYM_F64, nullptr, nullptr, 0, s));
    std::unique_ptr<gbsym_tri_s> up(tri_build(n, dp.p, di.p, dl.p, dd.p, GBSYM_ILU_UPPER, GBSYM_F64,
                                              nullptr, nullptr, 0, s));
    upload(dz, r, n, false, s);
    tri_solve_rowmajor(lo.get(), dz.p, nullptr, 1, GBSYM_F64, s);
    tri_solve_rowmajor(up.get(), dz.p, nullptr, 1, GBSYM_F64, s);
    int code = tri_read_error(lo.get(), s);
    if (!code) code = tri_read_error(up.get(), s);
    if (code) throw Err{code};
    GB_CUDA(cudaMemcpyAsync(z, dz.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
  });
}

// ---- schedule builders ----------------------------------------------------
int gbsym_build_levelset_csc(int n, const int *Lp, const int *Li, int **level_ptr, int **level_set) {
  int nl = 0;
  const int st = guarded([&] { nl = levelset_dropin(n, Lp, Li, true, false, level_ptr, level_set); });
  set_last_error(st);
  return st ? -st : nl;
}

int gbsym_build_levelset_csr(int n, const int *Lp, const int *Li, int **level_ptr, int **level_set) {
  int nl = 0;
  const int st = guarded([&] { nl = levelset_dropin(n, Lp, Li, false, false, level_ptr, level_set); });
  set_last_error(st);
  return st ? -st : nl;
}

int gbsym_build_levelset_upper_csr(int n, const int *Up, const int *Ui, int **level_ptr,
                                   int **level_set) {
  int nl = 0;
  const int st = guarded([&] { nl = levelset_dropin(n, Up, Ui, false, true, level_ptr, level_set); });
  set_last_error(st);
  return st ? -st : nl;
}

}  // extern "C"
