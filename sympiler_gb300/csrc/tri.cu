// tri.cu -- level-packed sparse triangles on the GPU: schedule builder,
// schedule/matrix validation, packing and the triangular-solve executors.
//
// The reference executes a triangular solve row by row (sptrsv_csr,
// sparse_blas/sptrsv.cpp:17-25), level by level with one OpenMP fork/join
// per level (sptrsv_csr_levelset, sptrsv.cpp:40-55) or by coarse level and
// partition (sptrsv_csr_lbc, sptrsv.cpp:57-76).  Here the rows of the
// triangle are re-packed in level order at plan time so that the row block
// of a level is one contiguous range of (column, value) pairs, staged into
// shared memory with coalesced loads; each row is then accumulated by one
// thread in the reference's storage order.  Dependencies between levels are
// kernel boundaries (one launch per level, captured in a CUDA graph), or
// block barriers when one thread block sweeps all levels.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>

#include "tri.cuh"

namespace gbsym {

// ---------------------------------------------------------------------------
// row definitions per triangle kind
struct RowDef {
  int lo, hi, dpos;  // off-diagonals [lo, hi); diagonal position or -1
};

__device__ __forceinline__ RowDef row_def(int kind, const int *__restrict__ p,
                                          const int *__restrict__ diags, int i) {
  switch (kind) {
    case GBSYM_LOWER_DIAG_LAST: return {p[i], p[i + 1] - 1, p[i + 1] - 1};
    case GBSYM_UPPER_DIAG_FIRST: return {p[i] + 1, p[i + 1], p[i]};
    case GBSYM_ILU_UNIT_LOWER: return {p[i], diags[i], -1};
    case GBSYM_ILU_UPPER: return {diags[i] + 1, p[i + 1], diags[i]};
    case kKindStrictLower:
    case kKindStrictUpper: return {p[i], p[i + 1], -1};
    default: return {p[i], diags[i], diags[i]};  // GBSYM_ILU_LOWER_DIV
  }
}

__device__ __forceinline__ void record_error(int *err, int code, int where) {
  if (atomicCAS(err, 0, code) == 0) err[1] = where;
}

// ---------------------------------------------------------------------------
// matrix validation
__global__ void k_validate_matrix(int n, const int *__restrict__ p, const int *__restrict__ ci,
                                  const int *__restrict__ diags, int kind, int upper, int *err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int a = p[i], z = p[i + 1];
    if (z < a) { record_error(err, GBSYM_ERR_BAD_MATRIX, i); continue; }
    if (diags && (kind >= GBSYM_ILU_UNIT_LOWER) && (diags[i] < a || diags[i] >= z)) {
      record_error(err, GBSYM_ERR_BAD_MATRIX, i);
      continue;
    }
    if (z == a && kind != GBSYM_ILU_UNIT_LOWER) { record_error(err, GBSYM_ERR_BAD_MATRIX, i); continue; }
    const RowDef r = row_def(kind, p, diags, i);
    for (int e = r.lo; e < r.hi; ++e) {
      const int c = ci[e];
      const bool ok = upper ? (c > i && c < n) : (c >= 0 && c < i);
      if (!ok) { record_error(err, GBSYM_ERR_BAD_MATRIX, i); break; }
    }
  }
}

static void read_err(const DBuf<int> &err, cudaStream_t s, int *host2) {
  GB_CUDA(cudaMemcpyAsync(host2, err.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
}

void validate_matrix(int n, const int *d_p, const int *d_i, const int *d_diags, int kind,
                     cudaStream_t s) {
  if (n == 0) return;
  DBuf<int> err(2);
  GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
  k_validate_matrix<<<std::min(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(
      n, d_p, d_i, d_diags, kind, kind_is_upper(kind), err.p);
  check_launch();
  int h[2];
  read_err(err, s, h);
  if (h[0]) throw Err{h[0]};
}

// ---------------------------------------------------------------------------
// Schedule builder: level(i) = 0 without dependencies, else 1 + the maximum
// level of its dependencies (the rule of the reference's build_levelSet_CSC
// call sites).  Computed by one persistent launch: warps claim 32-row chunks
// in dependency order from a ticket counter, so every chunk a warp waits on
// has been claimed by a running warp.  A lane first waits (bounded) for its
// dependencies in earlier chunks, read from memory as their warps publish
// them; dependencies inside its own chunk are lower lanes of the same warp
// and are applied afterwards in one pass of 32 shuffles in lane order (lane
// s's level is final when the pass reaches it, all its in-chunk
// dependencies being below it).  A chain of consecutive rows -- the x lines
// of a grid in natural order -- then costs one shuffle per row instead of a
// memory round trip.
__global__ void k_levels_syncfree(int n, const int *__restrict__ p, const int *__restrict__ ci,
                                  const int *__restrict__ diags, int kind, int upper,
                                  int *level, int *ctl /* ticket, err, where, maxlev */) {
  const int lane = threadIdx.x & 31;
  const int nchunks = (n + 31) >> 5;
  int my_max = -1;
  for (;;) {
    int chunk = 0;
    if (lane == 0) chunk = atomicAdd(&ctl[0], 1);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk >= nchunks) break;
    const int base = chunk << 5;
    const int idx = base + lane;
    const bool active = idx < n;
    const int row = active ? (upper ? n - 1 - idx : idx) : 0;
    int lo = 0, hi = 0;
    if (active) {
      const RowDef r = row_def(kind, p, diags, row);
      lo = r.lo;
      hi = r.hi;
    }
    int lev = 0, j = lo;
    unsigned inmask = 0;  // dependencies inside this chunk, as lane bits
    bool done = !active;
    unsigned long long t0 = globaltimer_ns();
    long long iters = 0;
    while (__any_sync(0xffffffffu, !done)) {
      if (!done) {
        bool progressed = false;
        while (j < hi) {
          const int c = ci[j];
          if (kind >= kKindStrictLower && (upper ? c <= row : c >= row)) {
            ++j;  // builder kinds: only entries on the dependency side count
            continue;
          }
          const int cidx = upper ? n - 1 - c : c;
          if (cidx >= base) {  // a lower lane of this warp: applied by the shuffle pass
            inmask |= 1u << (cidx - base);
            ++j;
            progressed = true;
            continue;
          }
          const int lc = ld_relaxed(&level[c]);
          if (lc < 0) break;
          lev = max(lev, lc + 1);
          ++j;
          progressed = true;
        }
        if (j >= hi) {
          done = true;
        } else {
          if (progressed) t0 = globaltimer_ns();
          if (++iters > kWaitLimitIters || globaltimer_ns() - t0 > kWaitLimitNs) {
            if (atomicCAS(&ctl[1], 0, GBSYM_ERR_TIMEOUT) == 0) ctl[2] = row;
            done = true;
          }
        }
      }
      __syncwarp();
      int stop = lane == 0 ? ld_relaxed(&ctl[1]) : 0;  // another warp gave up
      if (__shfl_sync(0xffffffffu, stop, 0) != 0) break;
    }
    int stop = lane == 0 ? ld_relaxed(&ctl[1]) : 0;
    if (__shfl_sync(0xffffffffu, stop, 0) != 0) break;
    for (int s = 0; s < 32; ++s) {
      const int v = __shfl_sync(0xffffffffu, lev, s);
      if ((inmask >> s) & 1u) lev = max(lev, v + 1);
    }
    if (active) {
      st_relaxed(&level[row], lev);
      my_max = max(my_max, lev);
    }
  }
  for (int o = 16; o; o >>= 1) my_max = max(my_max, __shfl_xor_sync(0xffffffffu, my_max, o));
  if (lane == 0 && my_max >= 0) atomicMax(&ctl[3], my_max);
}

__global__ void k_iota(int n, int *v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

__global__ void k_level_bounds(int n, const unsigned *__restrict__ sorted_lev, int *level_ptr,
                               int nlev) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const unsigned l = sorted_lev[k];
    if (k == 0 || sorted_lev[k - 1] != l) level_ptr[l] = k;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) level_ptr[nlev] = n;
}

static int bits_for(int v) {
  int b = 1;
  while ((1 << b) <= v && b < 31) ++b;
  return b;
}

int build_levels_device(int n, const int *d_p, const int *d_i, const int *d_diags, int kind,
                        DBuf<int> &d_level_ptr, DBuf<int> &d_level_set, cudaStream_t s) {
  if (n == 0) {
    d_level_ptr.alloc(1);
    GB_CUDA(cudaMemsetAsync(d_level_ptr.p, 0, sizeof(int), s));
    d_level_set.alloc(0);
    return 0;
  }
  DBuf<int> level(n), ctl(4);
  GB_CUDA(cudaMemsetAsync(level.p, 0xff, n * sizeof(int), s));
  GB_CUDA(cudaMemsetAsync(ctl.p, 0, 4 * sizeof(int), s));
  GB_CUDA(cudaMemsetAsync(ctl.p + 3, 0xff, sizeof(int), s));
  const int warps = div_up(n, 32);
  const int blocks = std::max(1, std::min(div_up(warps, 8), num_sms() * 4));
  k_levels_syncfree<<<blocks, 256, 0, s>>>(n, d_p, d_i, d_diags, kind, kind_is_upper(kind),
                                           level.p, ctl.p);
  check_launch();
  int h[4];
  GB_CUDA(cudaMemcpyAsync(h, ctl.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (h[1]) throw Err{h[1]};
  const int nlev = h[3] + 1;
  // stable sort of row indices by level: ascending row order inside a level
  DBuf<int> vals_in(n);
  DBuf<unsigned> keys_out(n);
  d_level_set.alloc(n);
  k_iota<<<std::min(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(n, vals_in.p);
  check_launch();
  size_t tmp_bytes = 0;
  const int end_bit = bits_for(nlev);
  GB_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, (const unsigned *)level.p,
                                          keys_out.p, vals_in.p, d_level_set.p, n, 0, end_bit, s));
  DBuf<char> tmp(tmp_bytes);
  GB_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, (const unsigned *)level.p,
                                          keys_out.p, vals_in.p, d_level_set.p, n, 0, end_bit, s));
  count_launch(4);
  d_level_ptr.alloc(nlev + 1);
  k_level_bounds<<<std::min(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(n, keys_out.p,
                                                                        d_level_ptr.p, nlev);
  check_launch();
  GB_CUDA(cudaStreamSynchronize(s));
  return nlev;
}

// ---------------------------------------------------------------------------
// schedule validation
__device__ __forceinline__ int upper_bound_dev(const int *a, int len, int key) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// position k of a level set -> level of its row
__global__ void k_assign_levels(int n, const int *__restrict__ level_ptr, int levels,
                                const int *__restrict__ level_set, int *lev_of, int *err) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int r = level_set[k];
    if (r < 0 || r >= n) { record_error(err, GBSYM_ERR_BAD_SCHEDULE, k); continue; }
    const int l = upper_bound_dev(level_ptr, levels + 1, k) - 1;
    if (atomicExch(&lev_of[r], l) != -1) record_error(err, GBSYM_ERR_BAD_SCHEDULE, r);
  }
}

__global__ void k_check_levels(int n, const int *__restrict__ p, const int *__restrict__ ci,
                               const int *__restrict__ diags, int kind,
                               const int *__restrict__ lev_of, int *err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const RowDef r = row_def(kind, p, diags, i);
    const int li = lev_of[i];
    for (int e = r.lo; e < r.hi; ++e)
      if (lev_of[ci[e]] >= li) { record_error(err, GBSYM_ERR_BAD_SCHEDULE, i); break; }
  }
}

static void validate_levelset(int n, const int *d_p, const int *d_i, const int *d_diags, int kind,
                              int levels, const int *h_level_ptr, const int *d_level_set,
                              cudaStream_t s) {
  GB_CHECK(levels >= 0 && h_level_ptr, GBSYM_ERR_BAD_SCHEDULE);
  GB_CHECK(h_level_ptr[0] == 0 && h_level_ptr[levels] == n, GBSYM_ERR_BAD_SCHEDULE);
  for (int l = 0; l < levels; ++l)
    GB_CHECK(h_level_ptr[l] <= h_level_ptr[l + 1], GBSYM_ERR_BAD_SCHEDULE);
  if (n == 0) return;
  DBuf<int> lp(levels + 1), lev_of(n), err(2);
  GB_CUDA(cudaMemcpyAsync(lp.p, h_level_ptr, (levels + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemsetAsync(lev_of.p, 0xff, n * sizeof(int), s));
  GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
  const int g = std::min(div_up(n, 256), num_sms() * 8);
  k_assign_levels<<<g, 256, 0, s>>>(n, lp.p, levels, d_level_set, lev_of.p, err.p);
  check_launch();
  k_check_levels<<<g, 256, 0, s>>>(n, d_p, d_i, d_diags, kind, lev_of.p, err.p);
  check_launch();
  int h[2];
  read_err(err, s, h);
  if (h[0]) throw Err{h[0]};
}

__global__ void k_assign_lbc(int n, const int *__restrict__ level_ptr, int level_no,
                             const int *__restrict__ par_ptr, int nparts,
                             const int *__restrict__ partition, int *cl_of, int *pid_of,
                             int *pos_of, int *err) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int r = partition[k];
    if (r < 0 || r >= n) { record_error(err, GBSYM_ERR_BAD_SCHEDULE, k); continue; }
    const int pid = upper_bound_dev(par_ptr, nparts + 1, k) - 1;
    const int cl = upper_bound_dev(level_ptr, level_no + 1, pid) - 1;
    if (atomicExch(&pos_of[r], k) != -1) { record_error(err, GBSYM_ERR_BAD_SCHEDULE, r); continue; }
    cl_of[r] = cl;
    pid_of[r] = pid;
  }
}

__global__ void k_check_lbc(int n, const int *__restrict__ p, const int *__restrict__ ci,
                            const int *__restrict__ diags, int kind, const int *__restrict__ cl_of,
                            const int *__restrict__ pid_of, const int *__restrict__ pos_of,
                            int *err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const RowDef r = row_def(kind, p, diags, i);
    for (int e = r.lo; e < r.hi; ++e) {
      const int c = ci[e];
      const bool ok = cl_of[c] < cl_of[i] || (pid_of[c] == pid_of[i] && pos_of[c] < pos_of[i]);
      if (!ok) { record_error(err, GBSYM_ERR_BAD_SCHEDULE, i); break; }
    }
  }
}

void validate_lbc(int n, const int *d_p, const int *d_i, const int *d_diags, int kind,
                  int level_no, const int *h_level_ptr, const int *h_par_ptr,
                  const int *h_partition, cudaStream_t s) {
  GB_CHECK(level_no >= 0 && h_level_ptr && h_par_ptr && h_partition, GBSYM_ERR_NULL_ARG);
  GB_CHECK(h_level_ptr[0] == 0, GBSYM_ERR_BAD_SCHEDULE);
  for (int l = 0; l < level_no; ++l) GB_CHECK(h_level_ptr[l] <= h_level_ptr[l + 1], GBSYM_ERR_BAD_SCHEDULE);
  const int nparts = h_level_ptr[level_no];
  GB_CHECK(nparts >= 0 && h_par_ptr[0] == 0 && h_par_ptr[nparts] == n, GBSYM_ERR_BAD_SCHEDULE);
  for (int q = 0; q < nparts; ++q) GB_CHECK(h_par_ptr[q] <= h_par_ptr[q + 1], GBSYM_ERR_BAD_SCHEDULE);
  if (n == 0) return;
  DBuf<int> lp(level_no + 1), pp(nparts + 1), part(n), cl(n), pid(n), pos(n), err(2);
  GB_CUDA(cudaMemcpyAsync(lp.p, h_level_ptr, (level_no + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemcpyAsync(pp.p, h_par_ptr, (nparts + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemcpyAsync(part.p, h_partition, n * sizeof(int), cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemsetAsync(pos.p, 0xff, n * sizeof(int), s));
  GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
  const int g = std::min(div_up(n, 256), num_sms() * 8);
  k_assign_lbc<<<g, 256, 0, s>>>(n, lp.p, level_no, pp.p, nparts, part.p, cl.p, pid.p, pos.p, err.p);
  check_launch();
  int h[2];
  read_err(err, s, h);
  if (h[0]) throw Err{h[0]};
  k_check_lbc<<<g, 256, 0, s>>>(n, d_p, d_i, d_diags, kind, cl.p, pid.p, pos.p, err.p);
  check_launch();
  read_err(err, s, h);
  if (h[0]) throw Err{h[0]};
}

// ---------------------------------------------------------------------------
// packing
__global__ void k_pack_counts(int n, const int *__restrict__ perm, const int *__restrict__ p,
                              const int *__restrict__ diags, int kind, int *len, int *hist) {
  __shared__ int sh[kSlabMax + 2];
  if (threadIdx.x < kSlabMax + 2) sh[threadIdx.x] = 0;
  __syncthreads();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const RowDef r = row_def(kind, p, diags, perm[k]);
    const int c = r.hi - r.lo;
    len[k] = c;
    atomicAdd(&sh[min(c, kSlabMax + 1)], 1);
  }
  __syncthreads();
  if (threadIdx.x < kSlabMax + 2) atomicAdd(&hist[threadIdx.x], sh[threadIdx.x]);
}

__global__ void k_overflow_counts(int n, const int *__restrict__ len, int K, int *cnt) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= n; k += gridDim.x * blockDim.x)
    cnt[k] = k < n ? max(0, len[k] - K) : 0;
}

template <class V>
__global__ void k_pack_rows(int n, const int *__restrict__ perm, const int *__restrict__ p,
                            const int *__restrict__ ci_in, const double *__restrict__ x_in,
                            const int *__restrict__ diags, int kind, int K, int npad,
                            const int *__restrict__ ovp, int *sci, V *sv, int *oci, V *ov, V *dg) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int k = warp; k < n; k += nwarps) {
    const RowDef r = row_def(kind, p, diags, perm[k]);
    const int c = r.hi - r.lo;
    for (int t = lane; t < max(c, K); t += 32) {
      if (t < K) {  // slab slots past the row's length hold a harmless zero entry
        sci[(size_t)t * npad + k] = t < c ? ci_in[r.lo + t] : 0;
        sv[(size_t)t * npad + k] = t < c ? (V)x_in[r.lo + t] : (V)0;
      } else {
        oci[ovp[k] + t - K] = ci_in[r.lo + t];
        ov[ovp[k] + t - K] = (V)x_in[r.lo + t];
      }
    }
    if (lane == 0) dg[k] = r.dpos >= 0 ? (V)x_in[r.dpos] : (V)1;
  }
}

// Slab width: the K in [0, kSlabMax] with the fewest bytes (slab slots
// plus overflow entries plus overflow pointers), preferring a wider slab
// while it costs at most a quarter more -- entries in the slab are loaded
// before a level kernel waits on its predecessor, overflow entries after.
static int choose_slab_width(int n, const int *hist) {
  long long best_cost = -1;
  int bestK = 0;
  long long cost[kSlabMax + 1];
  for (int K = 0; K <= kSlabMax; ++K) {
    long long over = 0, rows_over = 0;
    for (int c = K + 1; c <= kSlabMax; ++c) {
      over += (long long)(c - K) * hist[c];
      rows_over += hist[c];
    }
    // rows longer than kSlabMax: their excess is counted at kSlabMax + 1
    over += (long long)(kSlabMax + 1 - K) * hist[kSlabMax + 1];
    rows_over += hist[kSlabMax + 1];
    cost[K] = (long long)K * n + over + (rows_over ? n : 0);
    if (best_cost < 0 || cost[K] < best_cost) {
      best_cost = cost[K];
      bestK = K;
    }
  }
  int K = bestK;
  for (int c = kSlabMax; c > bestK; --c)
    if (cost[c] * 4 <= best_cost * 5) {
      K = c;
      break;
    }
  return K;
}

__device__ __forceinline__ double rcp_rn(double v) { return __drcp_rn(v); }
__device__ __forceinline__ float rcp_rn(float v) { return __frcp_rn(v); }

template <class V>
__global__ void k_reciprocals(int n, const V *__restrict__ dg, V *rc) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    rc[k] = rcp_rn(dg[k]);
}

template <class V>
static void pack_values(gbsym_tri_s *t, const int *d_p, const int *d_i, const double *d_x,
                        const int *d_diags, DBuf<V> &sv, DBuf<V> &ov, DBuf<V> &dg, DBuf<V> &rc,
                        cudaStream_t s) {
  const int n = t->n;
  sv.alloc((size_t)t->K * t->npad);
  ov.alloc(t->nov);
  dg.alloc(n);
  rc.alloc(n);
  if (!n) return;
  const int gw = std::max(1, std::min(div_up(n, 8), num_sms() * 16));
  k_pack_rows<V><<<gw, 256, 0, s>>>(n, t->perm.p, d_p, d_i, d_x, d_diags, t->kind, t->K, t->npad,
                                    t->ovp.p, t->sci.p, sv.p, t->oci.p, ov.p, dg.p);
  check_launch();
  k_reciprocals<V><<<std::min(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(n, dg.p, rc.p);
  check_launch();
}

// Dependency columns in packed-row numbering, for the sync-free sweep's
// scratch copy of the solution, which it keeps in packed (level) order: a
// warp unit then publishes its rows into one contiguous run, and the
// dependencies of consecutive rows of a level, which are mostly
// consecutive rows of earlier levels, are read in runs too.  Slots past a
// row's length are never read; they are set to 0.
__global__ void k_inverse_perm(int n, const int *__restrict__ perm, int *__restrict__ inv) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) inv[perm[k]] = k;
}
__global__ void k_packed_slab_cols(int n, int K, int npad, const int *__restrict__ len,
                                   const int *__restrict__ sci, const int *__restrict__ inv, int *__restrict__ scp) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    for (int q = 0; q < K; ++q) {
      const size_t at = (size_t)q * npad + k;
      scp[at] = q < len[k] ? inv[sci[at]] : 0;
    }
}
__global__ void k_packed_ov_cols(long long m, const int *__restrict__ oci, const int *__restrict__ inv,
                                 int *__restrict__ ocp) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m;
       e += (long long)gridDim.x * blockDim.x)
    ocp[e] = inv[oci[e]];
}

static void build_packed_cols(gbsym_tri_s *t, cudaStream_t s) {
  const int n = t->n;
  t->scp.alloc((size_t)t->K * t->npad);
  t->ocp.alloc(t->nov);
  if (!n) return;
  DBuf<int> inv(n);
  const int g = std::max(1, std::min(div_up(n, 256), num_sms() * 8));
  k_inverse_perm<<<g, 256, 0, s>>>(n, t->perm.p, inv.p);
  check_launch();
  if (t->K) {
    k_packed_slab_cols<<<g, 256, 0, s>>>(n, t->K, t->npad, t->len.p, t->sci.p, inv.p, t->scp.p);
    check_launch();
  }
  if (t->nov) {
    k_packed_ov_cols<<<std::max(1, std::min(div_up(t->nov, 256), num_sms() * 8)), 256, 0, s>>>(
        t->nov, t->oci.p, inv.p, t->ocp.p);
    check_launch();
  }
  GB_CUDA(cudaStreamSynchronize(s));  // inv is freed on return
}

// ---------------------------------------------------------------------------
// plan construction
gbsym_tri_s *tri_build(int n, const int *d_p, const int *d_i, const double *d_x,
                       const int *d_diags, int kind, int vdtype, const int *h_level_ptr,
                       const int *d_level_set, int levels, cudaStream_t s) {
  GB_CHECK(n >= 0, GBSYM_ERR_SIZE);
  GB_CHECK(kind >= GBSYM_LOWER_DIAG_LAST && kind <= GBSYM_ILU_LOWER_DIV, GBSYM_ERR_UNSUPPORTED);
  GB_CHECK(vdtype == GBSYM_F64 || vdtype == GBSYM_F32, GBSYM_ERR_UNSUPPORTED);
  GB_CHECK(kind < GBSYM_ILU_UNIT_LOWER || d_diags, GBSYM_ERR_NULL_ARG);
  std::unique_ptr<gbsym_tri_s> t(new gbsym_tri_s());
  t->n = n;
  t->kind = kind;
  t->vdtype = vdtype;
  GB_CUDA(cudaStreamCreateWithFlags(&t->cap_stream, cudaStreamNonBlocking));
  t->err.alloc(2);
  GB_CUDA(cudaMemsetAsync(t->err.p, 0, 2 * sizeof(int), s));
  validate_matrix(n, d_p, d_i, d_diags, kind, s);
  // schedule
  DBuf<int> lset;
  if (d_level_set) {
    validate_levelset(n, d_p, d_i, d_diags, kind, levels, h_level_ptr, d_level_set, s);
    t->nlev = levels;
    t->h_lev_ptr.assign(h_level_ptr, h_level_ptr + levels + 1);
    t->lev_ptr.alloc(levels + 1);
    GB_CUDA(cudaMemcpyAsync(t->lev_ptr.p, h_level_ptr, (levels + 1) * sizeof(int),
                            cudaMemcpyHostToDevice, s));
    lset.alloc(n);
    if (n) GB_CUDA(cudaMemcpyAsync(lset.p, d_level_set, n * sizeof(int), cudaMemcpyDeviceToDevice, s));
  } else {
    t->nlev = build_levels_device(n, d_p, d_i, d_diags, kind, t->lev_ptr, lset, s);
    t->h_lev_ptr.resize(t->nlev + 1);
    GB_CUDA(cudaMemcpyAsync(t->h_lev_ptr.data(), t->lev_ptr.p, (t->nlev + 1) * sizeof(int),
                            cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
  }
  t->perm = std::move(lset);
  for (int l = 0; l < t->nlev; ++l)
    t->max_level_rows = std::max(t->max_level_rows, t->h_lev_ptr[l + 1] - t->h_lev_ptr[l]);
  // pack: lengths and the slab-width histogram, overflow pointers, values
  t->len.alloc(n);
  DBuf<int> hist(kSlabMax + 2);
  GB_CUDA(cudaMemsetAsync(hist.p, 0, (kSlabMax + 2) * sizeof(int), s));
  const int g = std::max(1, std::min(div_up(n + 1, 256), num_sms() * 8));
  if (n) {
    k_pack_counts<<<g, 256, 0, s>>>(n, t->perm.p, d_p, d_diags, kind, t->len.p, hist.p);
    check_launch();
  }
  int h_hist[kSlabMax + 2];
  GB_CUDA(cudaMemcpyAsync(h_hist, hist.p, sizeof(h_hist), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  t->K = choose_slab_width(n, h_hist);
  t->npad = std::max(n, 1);
  t->ovp.alloc(n + 1);
  k_overflow_counts<<<g, 256, 0, s>>>(n, t->len.p, t->K, t->ovp.p);
  check_launch();
  size_t tmp_bytes = 0;
  GB_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, t->ovp.p, t->ovp.p, n + 1, s));
  DBuf<char> tmp(tmp_bytes);
  GB_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tmp_bytes, t->ovp.p, t->ovp.p, n + 1, s));
  count_launch(2);
  int nov = 0;
  GB_CUDA(cudaMemcpyAsync(&nov, t->ovp.p + n, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  t->nov = nov;
  long long nnz_off = 0;
  for (int c = 0; c <= kSlabMax; ++c) nnz_off += (long long)c * h_hist[c];
  t->sci.alloc((size_t)t->K * t->npad);
  t->oci.alloc(nov);
  if (vdtype == GBSYM_F64)
    pack_values<double>(t.get(), d_p, d_i, d_x, d_diags, t->sv64, t->ov64, t->dg64, t->rc64, s);
  else
    pack_values<float>(t.get(), d_p, d_i, d_x, d_diags, t->sv32, t->ov32, t->dg32, t->rc32, s);
  // exact off-diagonal count (rows longer than the histogram's last bin)
  {
    std::vector<int> lens(n);
    if (n) GB_CUDA(cudaMemcpyAsync(lens.data(), t->len.p, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    nnz_off = 0;
    for (int v : lens) nnz_off += v;
  }
  t->nnz_off = nnz_off;
  build_packed_cols(t.get(), s);
  t->bar.alloc(1);
  GB_CUDA(cudaMemsetAsync(t->bar.p, 0, sizeof(unsigned), s));
  choose_exec(t.get());
  GB_CUDA(cudaStreamSynchronize(s));
  return t.release();
}

}  // namespace gbsym

gbsym_tri_s::~gbsym_tri_s() {
  for (auto &g : graphs)
    if (g.exec_graph) cudaGraphExecDestroy(g.exec_graph);
  if (cap_stream) cudaStreamDestroy(cap_stream);
}

namespace gbsym {

// ---------------------------------------------------------------------------
// CSC input: every column starts with its diagonal and lists rows below it
__global__ void k_check_csc_lower(int n, const int *__restrict__ p, const int *__restrict__ ri, int *err) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int a = p[j], z = p[j + 1];
    bool bad = z <= a || ri[a] != j;
    for (int e = a + 1; !bad && e < z; ++e) bad = ri[e] <= j || ri[e] >= n;
    if (bad) record_error(err, GBSYM_ERR_BAD_MATRIX, j);
  }
}

void check_csc_lower(int n, const int *p, const int *ri, cudaStream_t s) {
  if (!n) return;
  DBuf<int> err(2);
  GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
  k_check_csc_lower<<<std::min(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(n, p, ri, err.p);
  check_launch();
  int h[2];
  read_err(err, s, h);
  if (h[0]) throw Err{h[0]};
}

__global__ void k_gather_f64(long long m, const double *__restrict__ src, const int *__restrict__ idx,
                             double *dst) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m;
       t += (long long)gridDim.x * blockDim.x)
    dst[t] = src[idx[t]];
}

void gather_values(long long m, const double *src, const int *idx, double *dst, cudaStream_t s) {
  if (!m) return;
  k_gather_f64<<<(int)std::min<long long>(div_up(m, 256), num_sms() * 8), 256, 0, s>>>(m, src, idx, dst);
  check_launch();
}

template <class T>
void run_syncfree(gbsym_tri_s *t, T *x, int k, cudaStream_t s, const T *b);  // exec_syncfree.cu

}  // namespace gbsym

// ---------------------------------------------------------------------------
// C API: plans
using namespace gbsym;

__global__ void k_transpose(const double *__restrict__ in, double *__restrict__ out, int rows,
                            int cols) {
  // in: rows x cols row-major -> out: cols x rows row-major
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = bx + j, c = by + threadIdx.x;
    if (r < cols && c < rows) out[(size_t)r * rows + c] = tile[threadIdx.x][j];
  }
}

static void transpose_dev(const double *in, double *out, int rows, int cols, cudaStream_t s) {
  dim3 grid(div_up(cols, 32), div_up(rows, 32)), block(32, 8);
  k_transpose<<<grid, block, 0, s>>>(in, out, rows, cols);
  check_launch();
}

extern "C" int gbsym_tri_create(gbsym_tri *out, int n, const int *p, const int *i, const double *x,
                                const int *diags, int kind, int value_dtype, int on_device,
                                const int *level_ptr, const int *level_set, int levels,
                                void *stream) {
  gbsym::PhaseRange phase_("gbsym_tri_create");
  if (!out || (n > 0 && (!p || !i || !x))) return GBSYM_ERR_NULL_ARG;
  *out = nullptr;
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    DBuf<int> dp, di, dd, dls;
    DBuf<double> dx;
    const int *pp = p, *ii = i, *dg = diags, *ls = level_set;
    const double *xx = x;
    std::vector<int> hlp;
    int nnz = 0;
    if (!on_device) {
      nnz = n ? p[n] : 0;
      upload(dp, p, n + 1, false, s);
      upload(di, i, nnz, false, s);
      upload(dx, x, nnz, false, s);
      if (diags) upload(dd, diags, n, false, s);
      if (level_set) upload(dls, level_set, n, false, s);
      pp = dp.p; ii = di.p; xx = dx.p; dg = diags ? dd.p : nullptr; ls = level_set ? dls.p : nullptr;
      if (level_set) {
        GB_CHECK(level_ptr, GBSYM_ERR_NULL_ARG);
        hlp.assign(level_ptr, level_ptr + levels + 1);
      }
    } else if (level_set) {
      GB_CHECK(level_ptr && levels >= 0, GBSYM_ERR_NULL_ARG);
      hlp.resize(levels + 1);
      GB_CUDA(cudaMemcpyAsync(hlp.data(), level_ptr, (levels + 1) * sizeof(int),
                              cudaMemcpyDeviceToHost, s));
      GB_CUDA(cudaStreamSynchronize(s));
    }
    if (kind == GBSYM_LOWER_CSC) {
      // CSC of a lower triangle (diagonal first in each column): transpose
      // on the device into the CSR pull form (diagonal last in each row).
      // The transposed rows list columns ascending, the order in which the
      // column-push solve (sptrsv_csc) updates each row.
      int nz = 0;
      if (n) {
        GB_CUDA(cudaMemcpyAsync(&nz, pp + n, sizeof(int), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
      }
      check_csc_lower(n, pp, ii, s);
      Transposed T;
      transpose_pattern(n, nz, pp, ii, T, s);
      DBuf<double> tx(nz);
      gather_values(nz, xx, T.src.p, tx.p, s);
      *out = tri_build(n, T.rp.p, T.ci.p, tx.p, nullptr, GBSYM_LOWER_DIAG_LAST, value_dtype,
                       level_set ? hlp.data() : nullptr, ls, levels, s);
      return;
    }
    *out = tri_build(n, pp, ii, xx, dg, kind, value_dtype, level_set ? hlp.data() : nullptr, ls,
                     levels, s);
  });
}

extern "C" int gbsym_tri_destroy(gbsym_tri t) {
  delete t;
  return GBSYM_OK;
}

extern "C" int gbsym_tri_get_info(gbsym_tri t, gbsym_tri_info *info) {
  if (!t || !info) return GBSYM_ERR_NULL_ARG;
  info->n = t->n;
  info->levels = t->nlev;
  info->nnz_off = t->nnz_off;
  info->dtype = t->vdtype;
  info->exec = effective_exec(t, 1, false);
  info->max_level_rows = t->max_level_rows;
  const long long vs = t->vdtype == GBSYM_F64 ? 8 : 4;
  info->bytes_matrix = ((long long)t->K * t->npad + t->nov) * (vs + 4) + (long long)t->n * (2 * vs + 8) +
                       (t->nov ? (t->n + 1) * 4ll : 0) + (t->nlev + 1) * 4ll;
  return GBSYM_OK;
}

extern "C" int gbsym_tri_set_exec(gbsym_tri t, int exec) {
  if (!t) return GBSYM_ERR_NULL_ARG;
  if (exec < GBSYM_EXEC_AUTO || exec > GBSYM_EXEC_PARTITIONED) return GBSYM_ERR_UNSUPPORTED;
  t->exec_forced = exec;
  return GBSYM_OK;
}

extern "C" int gbsym_tri_check(gbsym_tri t, void *stream) {
  if (!t) return GBSYM_ERR_NULL_ARG;
  int code = GBSYM_OK;
  const int st = guarded([&] { code = tri_read_error(t, (cudaStream_t)stream); });
  return st ? st : code;
}

extern "C" int gbsym_tri_get_schedule(gbsym_tri t, int *level_ptr, int *level_set) {
  if (!t || !level_ptr || !level_set) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    std::copy(t->h_lev_ptr.begin(), t->h_lev_ptr.end(), level_ptr);
    if (t->n) GB_CUDA(cudaMemcpy(level_set, t->perm.p, t->n * sizeof(int), cudaMemcpyDeviceToHost));
  });
}

extern "C" int gbsym_tri_solve(gbsym_tri t, void *x, int k, int layout, int dtype, void *stream) {
  gbsym::PhaseRange phase_("gbsym_tri_solve");
  if (!t || (!x && t->n && k)) return GBSYM_ERR_NULL_ARG;
  if (k < 0) return GBSYM_ERR_SIZE;
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    if (k > 1 && layout == GBSYM_COL_MAJOR) {
      GB_CHECK(dtype == GBSYM_F64, GBSYM_ERR_UNSUPPORTED);
      const size_t bytes = (size_t)t->n * k * sizeof(double);
      t->scratch.reserve(bytes);
      double *rm = (double *)t->scratch.p;
      transpose_dev((const double *)x, rm, k, t->n, s);  // k x n -> n x k
      tri_solve_rowmajor(t, rm, nullptr, k, dtype, s);
      transpose_dev(rm, (double *)x, t->n, k, s);
    } else {
      tri_solve_rowmajor(t, x, nullptr, k, dtype, s);
    }
  });
}

extern "C" int gbsym_tri_solve_into(gbsym_tri t, const void *b, void *x, int k, int dtype, void *stream) {
  gbsym::PhaseRange phase_("gbsym_tri_solve_into");
  if (!t || (t->n && k > 0 && (!x || !b))) return GBSYM_ERR_NULL_ARG;
  if (k < 0) return GBSYM_ERR_SIZE;
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    if (b == x) tri_solve_rowmajor(t, x, nullptr, k, dtype, s);
    else tri_solve_into(t, b, x, k, dtype, s);
  });
}

extern "C" int gbsym_tri_solve_b(gbsym_tri t, const double *b, double *x, void *stream) {
  gbsym::PhaseRange phase_("gbsym_tri_solve_b");
  if (!t || (t->n && (!x || !b))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    tri_solve_rowmajor(t, x, b, 1, GBSYM_F64, s);
  });
}

// Device pointer through which kernels may read and write the page-locked
// host buffer p in place, or null when the buffer must be staged: p is not
// page-locked, or the GPU does not share the CPU's page tables (a PCIe
// system, where zero-copy access would run at link latency per access).
// GBSYM_HOST_DIRECT=0 forces staging.
static void *host_direct_pointer(void *p) {
  const char *e = std::getenv("GBSYM_HOST_DIRECT");
  if (e && e[0] == '0') return nullptr;
  int dev = 0, coherent = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&coherent, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
  if (!coherent) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return a.devicePointer;
}

namespace gbsym {
// Row-major host-buffer solve in the plan's precision: in place over the
// CPU-GPU link when the buffer is page-locked, the GPU shares the host's
// page tables and a row's values are at least 256 bytes (each right-hand
// side read once and each result written once by the sync-free sweep, rows
// exchanging values through its device scratch), else staged through a
// device copy.  Shorter rows make the sweep's link traffic one small
// request per row, which the link serves more slowly than a bulk copy (the
// 512-system batch with 8 right-hand sides: 7.9 ms in place against 6.4 ms
// staged in FP32, 15.9 against 13.1 ms in FP64).  Synchronises.
void tri_solve_host_rowmajor(gbsym_tri_s *t, void *x, int k, int dtype) {
  cudaStream_t s = thread_stream();
  if (t->n == 0 || k == 0) return;
  GB_CHECK(dtype == GBSYM_F64 || dtype == GBSYM_F32, GBSYM_ERR_UNSUPPORTED);
  GB_CHECK((dtype == GBSYM_F64) == (t->vdtype == GBSYM_F64), GBSYM_ERR_UNSUPPORTED);
  const size_t row_bytes = (size_t)k * (dtype == GBSYM_F64 ? sizeof(double) : sizeof(float));
  if (void *dp = row_bytes >= 256 ? host_direct_pointer(x) : nullptr) {
    if (dtype == GBSYM_F64) run_syncfree<double>(t, static_cast<double *>(dp), k, s, nullptr);
    else run_syncfree<float>(t, static_cast<float *>(dp), k, s, nullptr);
  } else {
    const size_t bytes = (size_t)t->n * k * (dtype == GBSYM_F64 ? sizeof(double) : sizeof(float));
    t->io.reserve(bytes);
    GB_CUDA(cudaMemcpyAsync(t->io.p, x, bytes, cudaMemcpyHostToDevice, s));
    tri_solve_rowmajor(t, t->io.p, nullptr, k, dtype, s);
    GB_CUDA(cudaMemcpyAsync(x, t->io.p, bytes, cudaMemcpyDeviceToHost, s));
  }
  const int code = tri_read_error(t, s);
  if (code) throw Err{code};
}
}  // namespace gbsym

extern "C" int gbsym_host_solve_in_place(const void *x) {
  int r = 0;
  if (!x) return 0;
  const int st = guarded([&] { r = host_direct_pointer(const_cast<void *>(x)) != nullptr; });
  return st ? 0 : r;
}

extern "C" int gbsym_tri_solve_host(gbsym_tri t, double *x, int k, int layout) {
  gbsym::PhaseRange phase_("gbsym_tri_solve_host");
  if (!t || (!x && t->n && k)) return GBSYM_ERR_NULL_ARG;
  if (k < 0) return GBSYM_ERR_SIZE;
  return guarded([&] {
    cudaStream_t s = thread_stream();
    if (t->n == 0 || k == 0) return;
    GB_CHECK(t->vdtype == GBSYM_F64, GBSYM_ERR_UNSUPPORTED);
    if (k == 1 || layout == GBSYM_ROW_MAJOR) {
      if (void *dp = host_direct_pointer(x)) {
        // in place over the CPU-GPU link: the sync-free sweep reads each
        // right-hand side once and writes each result once, and rows
        // exchange values through its device scratch, never through x
        run_syncfree<double>(t, static_cast<double *>(dp), k, s, nullptr);
        const int code = tri_read_error(t, s);
        if (code) throw Err{code};
        return;
      }
    }
    const size_t bytes = (size_t)t->n * k * sizeof(double);
    t->io.reserve(bytes);
    double *dx = (double *)t->io.p;
    if (bytes) GB_CUDA(cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, s));
    int st = gbsym_tri_solve(t, dx, k, layout, GBSYM_F64, s);
    if (st) throw Err{st};
    if (bytes) GB_CUDA(cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, s));
    const int code = tri_read_error(t, s);
    if (code) throw Err{code};
  });
}
