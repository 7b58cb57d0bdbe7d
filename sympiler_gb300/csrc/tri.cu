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
// has been claimed by a running warp; inside a chunk the lanes retry in
// rounds until all 32 rows are resolved.  Waits are bounded.
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
    const int idx = (chunk << 5) + lane;
    const bool active = idx < n;
    const int row = active ? (upper ? n - 1 - idx : idx) : 0;
    int lo = 0, hi = 0;
    if (active) {
      const RowDef r = row_def(kind, p, diags, row);
      lo = r.lo;
      hi = r.hi;
    }
    int lev = 0, j = lo;
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
          const int lc = ld_relaxed(&level[c]);
          if (lc < 0) break;
          lev = max(lev, lc + 1);
          ++j;
          progressed = true;
        }
        if (j >= hi) {
          st_relaxed(&level[row], lev);
          my_max = max(my_max, lev);
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
                              const int *__restrict__ diags, int kind, int *cnt, int *maxcnt) {
  int m = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= n; k += gridDim.x * blockDim.x) {
    if (k == n) { cnt[k] = 0; continue; }
    const RowDef r = row_def(kind, p, diags, perm[k]);
    cnt[k] = r.hi - r.lo;
    m = max(m, r.hi - r.lo);
  }
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxcnt, m);
}

template <class V>
__global__ void k_pack_rows(int n, const int *__restrict__ perm, const int *__restrict__ p,
                            const int *__restrict__ ci_in, const double *__restrict__ x_in,
                            const int *__restrict__ diags, int kind, const int *__restrict__ rp,
                            int *ci_out, V *val_out, V *dg_out) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int k = warp; k < n; k += nwarps) {
    const RowDef r = row_def(kind, p, diags, perm[k]);
    const int base = rp[k];
    for (int t = lane; t < r.hi - r.lo; t += 32) {
      ci_out[base + t] = ci_in[r.lo + t];
      val_out[base + t] = (V)x_in[r.lo + t];
    }
    if (lane == 0) dg_out[k] = r.dpos >= 0 ? (V)x_in[r.dpos] : (V)1;
  }
}

// ---------------------------------------------------------------------------
// executors
constexpr int kLvlBlock = 128;   // rows per block, one thread per row
constexpr int kLvlChunk = 1024;  // staged entries per pass

// One level, one right-hand side.  The level's packed row block
// [r0, r1) is staged chunk by chunk into shared memory with coalesced
// loads, then each thread accumulates its row in storage order.
template <class T, bool REDUNDANT>
__global__ void __launch_bounds__(kLvlBlock)
k_level_1rhs(TriView<T> A, T *__restrict__ x, const T *__restrict__ b, int r_begin, int r_end) {
  __shared__ int s_ci[kLvlChunk];
  __shared__ T s_v[kLvlChunk];
  const int r0 = r_begin + blockIdx.x * kLvlBlock;
  const int r1 = min(r0 + kLvlBlock, r_end);
  const int row = r0 + threadIdx.x;
  const bool active = row < r1;
  const int e0 = A.rp[r0], e1 = A.rp[r1];
  int lo = 0, hi = 0, orig = 0;
  T acc = T(0);
  if (active) {
    lo = A.rp[row];
    hi = A.rp[row + 1];
    orig = A.perm[row];
    if (!REDUNDANT) acc = x[orig];
  }
  for (int c0 = e0; c0 < e1; c0 += kLvlChunk) {
    const int c1 = min(c0 + kLvlChunk, e1);
    if (c0 != e0) __syncthreads();
    for (int e = c0 + threadIdx.x; e < c1; e += kLvlBlock) {
      s_ci[e - c0] = A.ci[e];
      s_v[e - c0] = A.val[e];
    }
    __syncthreads();
    if (active) {
      const int a = max(lo, c0), z = min(hi, c1);
      for (int e = a; e < z; ++e) acc = sub_rn(acc, mul_rn(s_v[e - c0], x[s_ci[e - c0]]));
    }
  }
  if (active) {
    if (REDUNDANT) acc = add_rn(acc, b[orig]);
    if (A.dg) acc = div_rn(acc, A.dg[row]);
    x[orig] = acc;
  }
}

// One level, k right-hand sides stored row-major (x[i*k + r]).  G lanes
// share a row; each lane owns VEC consecutive right-hand sides per step, so
// a dependency's k values are read as one coalesced segment.
template <class T, int VEC> struct VecT;
template <> struct VecT<double, 1> { using t = double; };
template <> struct VecT<double, 2> { using t = double2; };
template <> struct VecT<float, 1> { using t = float; };
template <> struct VecT<float, 2> { using t = float2; };
template <> struct VecT<float, 4> { using t = float4; };

template <class T, int VEC>
__device__ __forceinline__ void vload(const T *p, T (&v)[VEC]) {
  using V = typename VecT<T, VEC>::t;
  const V t = *reinterpret_cast<const V *>(p);
  const T *s = reinterpret_cast<const T *>(&t);
#pragma unroll
  for (int q = 0; q < VEC; ++q) v[q] = s[q];
}
template <class T, int VEC>
__device__ __forceinline__ void vstore(T *p, const T (&v)[VEC]) {
  using V = typename VecT<T, VEC>::t;
  V t;
  T *s = reinterpret_cast<T *>(&t);
#pragma unroll
  for (int q = 0; q < VEC; ++q) s[q] = v[q];
  *reinterpret_cast<V *>(p) = t;
}

template <class T, int G, int VEC>
__global__ void __launch_bounds__(256)
k_level_mrhs(TriView<T> A, T *__restrict__ x, int k, int r_begin, int r_end) {
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int lane = threadIdx.x % G;
  const int row = r_begin + gid;
  if (row >= r_end) return;
  const int lo = A.rp[row], hi = A.rp[row + 1];
  const size_t orig = (size_t)A.perm[row];
  const T d = A.dg ? A.dg[row] : T(1);
  for (int r = lane * VEC; r < k; r += G * VEC) {
    T acc[VEC];
    vload<T, VEC>(x + orig * k + r, acc);
    for (int e = lo; e < hi; ++e) {
      const T v = A.val[e];
      T xv[VEC];
      vload<T, VEC>(x + (size_t)A.ci[e] * k + r, xv);
#pragma unroll
      for (int q = 0; q < VEC; ++q) acc[q] = sub_rn(acc[q], mul_rn(v, xv[q]));
    }
    if (A.dg) {
#pragma unroll
      for (int q = 0; q < VEC; ++q) acc[q] = div_rn(acc[q], d);
    }
    vstore<T, VEC>(x + orig * k + r, acc);
  }
}

// Whole solve in one thread block: levels are separated by __syncthreads.
// x lives in shared memory when it fits (xs != x), otherwise in global
// memory (stores of this block are visible to its own threads after the
// barrier).  The next level's row data is loaded into registers before the
// barrier so only the gathers of x sit on the dependency chain.
constexpr int kOneBlock = 1024;
constexpr int kOnePf = 8;  // prefetched entries per row

template <class T>
__global__ void __launch_bounds__(kOneBlock)
k_oneblock_1rhs(TriView<T> A, T *__restrict__ xg, const int *__restrict__ lev_ptr, int nlev,
                int n, int x_in_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *xs = x_in_smem ? reinterpret_cast<T *>(smem_raw) : xg;
  if (x_in_smem) {
    for (int i = threadIdx.x; i < n; i += kOneBlock) xs[i] = xg[i];
    __syncthreads();
  }
  // prefetch state for the row this thread handles first in the level
  int lo = 0, hi = 0, orig = 0;
  int pci[kOnePf];
  T pv[kOnePf];
  T pd = T(1);
  auto prefetch = [&](int row) {
    lo = A.rp[row];
    hi = A.rp[row + 1];
    orig = A.perm[row];
    pd = A.dg ? A.dg[row] : T(1);
#pragma unroll
    for (int q = 0; q < kOnePf; ++q) {
      if (lo + q < hi) { pci[q] = A.ci[lo + q]; pv[q] = A.val[lo + q]; }
    }
  };
  int r0 = lev_ptr[0], r1 = nlev > 0 ? lev_ptr[1] : 0;
  if (threadIdx.x < r1 - r0) prefetch(r0 + threadIdx.x);
  for (int l = 0; l < nlev; ++l) {
    const int nr0 = r1;
    const int nr1 = (l + 1 < nlev) ? lev_ptr[l + 2] : nr0;
    // first row of this thread in level l (prefetched)
    int row = r0 + threadIdx.x;
    if (row < r1) {
      T acc = xs[orig];
#pragma unroll
      for (int q = 0; q < kOnePf; ++q)
        if (lo + q < hi) acc = sub_rn(acc, mul_rn(pv[q], xs[pci[q]]));
      for (int e = lo + kOnePf; e < hi; ++e) acc = sub_rn(acc, mul_rn(A.val[e], xs[A.ci[e]]));
      if (A.dg) acc = div_rn(acc, pd);
      xs[orig] = acc;
    }
    // remaining rows of a wide level
    for (row += kOneBlock; row < r1; row += kOneBlock) {
      const int a = A.rp[row], z = A.rp[row + 1], o = A.perm[row];
      T acc = xs[o];
      for (int e = a; e < z; ++e) acc = sub_rn(acc, mul_rn(A.val[e], xs[A.ci[e]]));
      if (A.dg) acc = div_rn(acc, A.dg[row]);
      xs[o] = acc;
    }
    if (threadIdx.x < nr1 - nr0) prefetch(nr0 + threadIdx.x);
    r0 = nr0;
    r1 = nr1;
    __syncthreads();
  }
  if (x_in_smem) {
    for (int i = threadIdx.x; i < n; i += kOneBlock) xg[i] = xs[i];
  }
}

template <class T>
static TriView<T> view_of(const gbsym_tri_s *t);
template <>
TriView<double> view_of<double>(const gbsym_tri_s *t) { return t->view64(); }
template <>
TriView<float> view_of<float>(const gbsym_tri_s *t) { return t->view32(); }

template <class T, int G>
static void launch_mrhs_g(const TriView<T> &A, T *x, int k, int a, int z, cudaStream_t s) {
  const int rows = z - a;
  const int rows_per_block = 256 / G;
  const int grid = div_up(rows, rows_per_block);
  const bool v4 = sizeof(T) == 4 && (k % 4 == 0) && ((uintptr_t)x % 16 == 0);
  const bool v2 = (k % 2 == 0) && ((uintptr_t)x % (2 * sizeof(T)) == 0);
  if (sizeof(T) == 4 && v4)
    k_level_mrhs<T, G, (sizeof(T) == 4 ? 4 : 2)><<<grid, 256, 0, s>>>(A, x, k, a, z);
  else if (v2)
    k_level_mrhs<T, G, 2><<<grid, 256, 0, s>>>(A, x, k, a, z);
  else
    k_level_mrhs<T, G, 1><<<grid, 256, 0, s>>>(A, x, k, a, z);
  check_launch();
}

template <class T>
static void launch_level(const TriView<T> &A, T *x, const T *b, int k, int a, int z,
                         cudaStream_t s) {
  if (z <= a) return;
  if (k == 1) {
    const int grid = div_up(z - a, kLvlBlock);
    if (b)
      k_level_1rhs<T, true><<<grid, kLvlBlock, 0, s>>>(A, x, b, a, z);
    else
      k_level_1rhs<T, false><<<grid, kLvlBlock, 0, s>>>(A, x, nullptr, a, z);
    check_launch();
    return;
  }
  // lanes per row: enough to cover k with 2-wide (FP64) / 4-wide (FP32) loads
  const int per = sizeof(T) == 8 ? 2 : 4;
  const int need = div_up(k, per);
  if (need <= 2) launch_mrhs_g<T, 2>(A, x, k, a, z, s);
  else if (need <= 4) launch_mrhs_g<T, 4>(A, x, k, a, z, s);
  else if (need <= 8) launch_mrhs_g<T, 8>(A, x, k, a, z, s);
  else if (need <= 16) launch_mrhs_g<T, 16>(A, x, k, a, z, s);
  else launch_mrhs_g<T, 32>(A, x, k, a, z, s);
}

template <class T>
static void issue_levels(gbsym_tri_s *t, T *x, const T *b, int k, cudaStream_t s) {
  const TriView<T> A = view_of<T>(t);
  for (int l = 0; l < t->nlev; ++l) launch_level<T>(A, x, b, k, t->h_lev_ptr[l], t->h_lev_ptr[l + 1], s);
}

static size_t oneblock_smem(const gbsym_tri_s *t, int dsize) {
  const size_t need = (size_t)t->n * dsize;
  return need <= 200 * 1024 ? need : 0;
}

template <class T>
static void issue_oneblock(gbsym_tri_s *t, T *x, cudaStream_t s) {
  const size_t sm = oneblock_smem(t, sizeof(T));
  if (sm > 48 * 1024)
    GB_CUDA(cudaFuncSetAttribute(k_oneblock_1rhs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm));
  k_oneblock_1rhs<T><<<1, kOneBlock, sm, s>>>(view_of<T>(t), x, t->lev_ptr.p, t->nlev, t->n,
                                              sm > 0 ? 1 : 0);
  check_launch();
}

static int effective_exec(const gbsym_tri_s *t, int k, bool redundant) {
  int e = t->exec_forced != GBSYM_EXEC_AUTO ? t->exec_forced : t->exec;
  if (e == GBSYM_EXEC_ONEBLOCK && (k != 1 || redundant)) e = GBSYM_EXEC_LEVELSET;
  if (e == GBSYM_EXEC_SYNCFREE) e = GBSYM_EXEC_LEVELSET;  // not built for this path yet
  return e;
}

// Level launches are captured once per (x, b, k, dtype) into a CUDA graph
// and replayed; the plan keeps the eight most recent.
template <class T>
static void run_levelset_graph(gbsym_tri_s *t, T *x, const T *b, int k, int dtype, cudaStream_t s) {
  GraphEntry *hit = nullptr;
  for (auto &g : t->graphs)
    if (g.x == x && g.b == b && g.k == k && g.dtype == dtype) hit = &g;
  if (!hit) {
    if (t->graphs.size() >= 8) {
      auto old = std::min_element(t->graphs.begin(), t->graphs.end(),
                                  [](const GraphEntry &a, const GraphEntry &c) { return a.stamp < c.stamp; });
      cudaGraphExecDestroy(old->exec_graph);
      t->graphs.erase(old);
    }
    GraphEntry g;
    g.x = x; g.b = b; g.k = k; g.dtype = dtype;
    cudaGraph_t graph;
    GB_CUDA(cudaStreamBeginCapture(t->cap_stream, cudaStreamCaptureModeThreadLocal));
    const unsigned long long before = g_launches.load();
    try {
      issue_levels<T>(t, x, b, k, t->cap_stream);
    } catch (...) {
      cudaStreamEndCapture(t->cap_stream, &graph);
      throw;
    }
    g.nodes = g_launches.load() - before;
    g_launches.fetch_sub(g.nodes);  // counted when replayed
    GB_CUDA(cudaStreamEndCapture(t->cap_stream, &graph));
    GB_CUDA(cudaGraphInstantiate(&g.exec_graph, graph, 0));
    cudaGraphDestroy(graph);
    t->graphs.push_back(g);
    hit = &t->graphs.back();
  }
  hit->stamp = ++t->graph_clock;
  GB_CUDA(cudaGraphLaunch(hit->exec_graph, s));
  count_launch(hit->nodes);
}

template <class T>
static void solve_typed(gbsym_tri_s *t, T *x, const T *b, int k, int dtype, cudaStream_t s) {
  if (t->n == 0 || k == 0) return;
  const int e = effective_exec(t, k, b != nullptr);
  if (e == GBSYM_EXEC_ONEBLOCK) {
    issue_oneblock<T>(t, x, s);
    return;
  }
  if (t->nlev <= 2) {
    issue_levels<T>(t, x, b, k, s);
    return;
  }
  run_levelset_graph<T>(t, x, b, k, dtype, s);
}

void tri_solve_rowmajor(gbsym_tri_s *t, void *x, const void *b, int k, int dtype, cudaStream_t s) {
  if (dtype == GBSYM_F64) {
    GB_CHECK(t->vdtype == GBSYM_F64, GBSYM_ERR_UNSUPPORTED);
    solve_typed<double>(t, (double *)x, (const double *)b, k, dtype, s);
  } else {
    GB_CHECK(t->vdtype == GBSYM_F32 && b == nullptr, GBSYM_ERR_UNSUPPORTED);
    solve_typed<float>(t, (float *)x, nullptr, k, dtype, s);
  }
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
  // pack
  t->rp.alloc(n + 1);
  DBuf<int> maxcnt(1);
  GB_CUDA(cudaMemsetAsync(maxcnt.p, 0, sizeof(int), s));
  const int g = std::max(1, std::min(div_up(n + 1, 256), num_sms() * 8));
  k_pack_counts<<<g, 256, 0, s>>>(n, t->perm.p, d_p, d_diags, kind, t->rp.p, maxcnt.p);
  check_launch();
  size_t tmp_bytes = 0;
  GB_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, t->rp.p, t->rp.p, n + 1, s));
  DBuf<char> tmp(tmp_bytes);
  GB_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tmp_bytes, t->rp.p, t->rp.p, n + 1, s));
  count_launch(2);
  int nnz_off = 0;
  GB_CUDA(cudaMemcpyAsync(&nnz_off, t->rp.p + n, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  t->nnz_off = nnz_off;
  t->ci.alloc(nnz_off);
  const int gw = std::max(1, std::min(div_up(n, 8), num_sms() * 16));
  if (vdtype == GBSYM_F64) {
    t->val64.alloc(nnz_off);
    t->dg64.alloc(n);
    if (n)
      k_pack_rows<double><<<gw, 256, 0, s>>>(n, t->perm.p, d_p, d_i, d_x, d_diags, kind, t->rp.p,
                                             t->ci.p, t->val64.p, t->dg64.p);
  } else {
    t->val32.alloc(nnz_off);
    t->dg32.alloc(n);
    if (n)
      k_pack_rows<float><<<gw, 256, 0, s>>>(n, t->perm.p, d_p, d_i, d_x, d_diags, kind, t->rp.p,
                                            t->ci.p, t->val32.p, t->dg32.p);
  }
  if (n) check_launch();
  // executor choice: one block when the whole solve is a short sweep
  const char *force = std::getenv("GBSYM_TRI_EXEC");
  t->exec = (t->max_level_rows <= 2048 && (double)n / std::max(1, t->nlev) <= 1024.0)
                ? GBSYM_EXEC_ONEBLOCK
                : GBSYM_EXEC_LEVELSET;
  if (force) {
    if (!std::strcmp(force, "levelset")) t->exec = GBSYM_EXEC_LEVELSET;
    else if (!std::strcmp(force, "oneblock")) t->exec = GBSYM_EXEC_ONEBLOCK;
  }
  GB_CUDA(cudaStreamSynchronize(s));
  return t.release();
}

}  // namespace gbsym

gbsym_tri_s::~gbsym_tri_s() {
  for (auto &g : graphs)
    if (g.exec_graph) cudaGraphExecDestroy(g.exec_graph);
  if (cap_stream) cudaStreamDestroy(cap_stream);
}

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
  info->bytes_matrix = t->nnz_off * (vs + 4) + (long long)t->n * (vs + 8) + 4 + (t->nlev + 1) * 4ll;
  return GBSYM_OK;
}

extern "C" int gbsym_tri_set_exec(gbsym_tri t, int exec) {
  if (!t) return GBSYM_ERR_NULL_ARG;
  if (exec < GBSYM_EXEC_AUTO || exec > GBSYM_EXEC_ONEBLOCK) return GBSYM_ERR_UNSUPPORTED;
  t->exec_forced = exec;
  return GBSYM_OK;
}

extern "C" int gbsym_tri_get_schedule(gbsym_tri t, int *level_ptr, int *level_set) {
  if (!t || !level_ptr || !level_set) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    std::copy(t->h_lev_ptr.begin(), t->h_lev_ptr.end(), level_ptr);
    if (t->n) GB_CUDA(cudaMemcpy(level_set, t->perm.p, t->n * sizeof(int), cudaMemcpyDeviceToHost));
  });
}

extern "C" int gbsym_tri_solve(gbsym_tri t, void *x, int k, int layout, int dtype, void *stream) {
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

extern "C" int gbsym_tri_solve_b(gbsym_tri t, const double *b, double *x, void *stream) {
  if (!t || (t->n && (!x || !b))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    tri_solve_rowmajor(t, x, b, 1, GBSYM_F64, s);
  });
}

extern "C" int gbsym_tri_solve_host(gbsym_tri t, double *x, int k, int layout) {
  if (!t || (!x && t->n && k)) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    cudaStream_t s = thread_stream();
    const size_t bytes = (size_t)t->n * k * sizeof(double);
    t->io.reserve(bytes);
    double *dx = (double *)t->io.p;
    if (bytes) GB_CUDA(cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, s));
    int st = gbsym_tri_solve(t, dx, k, layout, GBSYM_F64, s);
    if (st) throw Err{st};
    if (bytes) GB_CUDA(cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
  });
}
