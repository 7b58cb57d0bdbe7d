// exec_part.cu -- PARTITIONED executor: contiguous row partitions, one
// thread block each, sync-free between partitions (one right-hand side).
//
// The reference's LBC executors (sptrsv_csr_lbc, sparse_blas/sptrsv.cpp:
// 57-76) give each thread a partition of rows that it solves in serial
// order, with a barrier between coarse levels.  Here a partition is a
// contiguous range of R rows in topological order (ascending row index for
// a lower triangle, descending for an upper one) and belongs to one thread
// block, which walks the partition's rows level by level: the rows of one
// level in parallel, a block barrier between levels.  A dependency inside
// the partition is read from shared memory (written by this block one or
// more levels earlier); a dependency in an earlier partition is polled from
// the sync-free scratch y, where every solved value is published with a
// single relaxed store over an all-ones sentinel, as in the sync-free
// executor.  There is no barrier between partitions.
//
// On meshes in natural order most of a row's dependencies lie in the same
// contiguous range and cost a block barrier and a shared-memory read
// instead of a round trip through L2.  What remains on the critical path
// is the chain of cross-partition hops (on a 3D grid every row has one, its
// neighbour a plane below), so the gain over the sync-free sweep is modest
// there (measured 433 vs 457 us on the 64^3 IC0 factor); the autotuner
// tries it at several partition sizes.
//
// Progress: partition p waits only on partitions q < p (topological order),
// a block takes partitions blockIdx.x, blockIdx.x + gridDim.x, ... in
// increasing order, and the launch is cooperative (every block resident),
// so the smallest unfinished partition can always proceed.  Waits are
// bounded: a thread that sees no progress for about two seconds records
// GBSYM_ERR_TIMEOUT and the blocks leave at their next level boundary.
#include <algorithm>
#include <vector>

#include "exec_common.cuh"

namespace gbsym {
namespace {

constexpr int kPartBlock = 128;
constexpr long long kPartWaitCycles = 1ll << 32;  // about two seconds

__device__ __forceinline__ double part_ld(const double *p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ float part_ld(const float *p) {
  float v;
  asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void part_st(double *p, double v) {
  long long b = __double_as_longlong(v);
  if (b == -1ll) b = 0x7ff8000000000000ll;  // never publish the sentinel
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(b) : "memory");
}
__device__ __forceinline__ void part_st(float *p, float v) {
  int b = __float_as_int(v);
  if (b == -1) b = 0x7fc00000;
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(b) : "memory");
}
__device__ __forceinline__ bool part_unset(double v) { return __double_as_longlong(v) == -1ll; }
__device__ __forceinline__ bool part_unset(float v) { return __float_as_int(v) == -1; }

// Wait for one published value (bounded).  On timeout or on an error
// recorded elsewhere, *stop is set and a placeholder returned.
template <class T>
__device__ __forceinline__ T part_wait(const T *p, int *err, int *stop) {
  T v = part_ld(p);
  if (!part_unset(v)) return v;
  const long long t0 = clock64();
  for (int round = 1;; ++round) {
    __nanosleep(32);
    v = part_ld(p);
    if (!part_unset(v)) return v;
    if ((round & 63) == 0) {
      if (clock64() - t0 > kPartWaitCycles) atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
      if (ld_relaxed(err) != 0) {
        *stop = 1;
        return T(0);
      }
    }
  }
}

// One row: slab dependencies from shared memory when they lie in this
// partition, else from the published scratch (all loads issued before any
// wait); overflow entries in order; then publish.
template <class T, int AR>
__device__ __forceinline__ void part_row(const TriView<T> &A, const RowStatic<T> &rs, T acc, T *__restrict__ x,
                                         T *__restrict__ y, T *xs, int n, int upper, int lo, int R, int *err,
                                         int *stop) {
  T xv[kSlabMax];
  unsigned remote = 0;
#pragma unroll
  for (int s = 0; s < kSlabMax; ++s)
    if (s < A.K && s < rs.len) {
      const int pos = upper ? n - 1 - rs.c[s] : rs.c[s];
      if ((unsigned)(pos - lo) < (unsigned)R) xv[s] = xs[pos - lo];
      else remote |= 1u << s;
    }
#pragma unroll
  for (int s = 0; s < kSlabMax; ++s)
    if ((remote >> s) & 1u) xv[s] = part_ld(y + rs.c[s]);
#pragma unroll
  for (int s = 0; s < kSlabMax; ++s)
    if (((remote >> s) & 1u) && part_unset(xv[s])) xv[s] = part_wait(y + rs.c[s], err, stop);
#pragma unroll
  for (int s = 0; s < kSlabMax; ++s)
    if (s < A.K && s < rs.len) acc = msub<AR>(acc, rs.v[s], xv[s]);
  for (int t = A.K; t < rs.len; ++t) {
    const int e = rs.ovb + t - A.K;
    const int c = A.oci[e];
    const int pos = upper ? n - 1 - c : c;
    const T v = (unsigned)(pos - lo) < (unsigned)R ? xs[pos - lo] : part_wait(y + c, err, stop);
    acc = msub<AR>(acc, A.ov[e], v);
  }
  acc = row_finish(A, rs, acc);
  x[rs.orig] = acc;
  xs[(upper ? n - 1 - rs.orig : rs.orig) - lo] = acc;
  part_st(y + rs.orig, acc);
}

// A thread's first row of the next level is loaded (static row data and
// right-hand side) before the current level is solved, so those loads are
// in flight across the level's work and barrier.
template <class T, int AR>
__global__ void __launch_bounds__(kPartBlock)
k_part_sweep(TriView<T> A, T *__restrict__ x, T *__restrict__ y, int n, int upper, int R, int nparts,
             const int *__restrict__ part_group, const int *__restrict__ group_ptr,
             const int *__restrict__ rows, int *err) {
  extern __shared__ __align__(16) unsigned char part_smem[];
  T *xs = reinterpret_cast<T *>(part_smem);  // this partition's solved values, by position
  __shared__ int stop;
  if (threadIdx.x == 0) stop = 0;
  __syncthreads();
  for (int p = blockIdx.x; p < nparts; p += gridDim.x) {
    const int lo = p * R;  // topological positions [lo, lo + R)
    const int g0 = part_group[p], g1 = part_group[p + 1];
    RowStatic<T> cur;
    T bcur = T(0);
    bool have = false;
    {
      const int q = group_ptr[g0] + threadIdx.x;
      if (q < group_ptr[g0 + 1]) {
        load_row(A, rows[q], cur);
        bcur = x[cur.orig];
        have = true;
      }
    }
    for (int g = g0; g < g1; ++g) {
      const int qa = group_ptr[g], qz = group_ptr[g + 1];
      RowStatic<T> nxt;
      T bnxt = T(0);
      bool have_n = false;
      if (g + 1 < g1) {
        const int qn = qz + threadIdx.x;
        if (qn < group_ptr[g + 2]) {
          load_row(A, rows[qn], nxt);
          bnxt = x[nxt.orig];
          have_n = true;
        }
      }
      if (have) part_row<T, AR>(A, cur, bcur, x, y, xs, n, upper, lo, R, err, &stop);
      for (int q = qa + threadIdx.x + blockDim.x; q < qz; q += blockDim.x) {
        RowStatic<T> rs;
        load_row(A, rows[q], rs);
        part_row<T, AR>(A, rs, x[rs.orig], x, y, xs, n, upper, lo, R, err, &stop);
      }
      __syncthreads();  // this level's values are in xs for the next
      if (stop) return;
      cur = nxt;
      bcur = bnxt;
      have = have_n;
    }
  }
}

bool kind_is_upper(int kind) {
  return kind == GBSYM_UPPER_DIAG_FIRST || kind == GBSYM_ILU_UPPER || kind == kKindStrictUpper;
}

// Largest partition the shared memory holds, and the default partition
// size: one partition per SM (at least 64 rows).
int part_rows_max(int vbytes) { return (200 * 1024) / vbytes; }

int part_rows_default(const gbsym_tri_s *t, int vbytes) {
  const int r = std::max(64, div_up(t->n, num_sms()));
  return std::min(r, part_rows_max(vbytes));
}

// Partitions of R consecutive topological positions; within each, the
// plan's packed rows in packed order (level-major, ascending row), cut
// into groups at level changes.
void build_partitions(gbsym_tri_s *t, int R, cudaStream_t s) {
  auto &P = t->part;
  if (P.R == R) return;
  const int n = t->n;
  const bool upper = kind_is_upper(t->kind);
  std::vector<int> perm(n);
  GB_CUDA(cudaMemcpyAsync(perm.data(), t->perm.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  const int np = div_up(n, R);
  std::vector<int> start(np + 1, 0), rows(n), level(n);
  for (int l = 0; l < t->nlev; ++l)
    for (int k = t->h_lev_ptr[l]; k < t->h_lev_ptr[l + 1]; ++k) level[k] = l;
  auto part_of = [&](int k) { return (upper ? n - 1 - perm[k] : perm[k]) / R; };
  for (int k = 0; k < n; ++k) start[part_of(k) + 1]++;
  for (int p = 0; p < np; ++p) start[p + 1] += start[p];
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int k = 0; k < n; ++k) rows[fill[part_of(k)]++] = k;
  }
  std::vector<int> pg(np + 1, 0), gp;
  gp.reserve((size_t)np * 4 + 1);
  for (int p = 0; p < np; ++p) {
    pg[p] = (int)gp.size();
    for (int q = start[p]; q < start[p + 1]; ++q)
      if (q == start[p] || level[rows[q]] != level[rows[q - 1]]) gp.push_back(q);
  }
  pg[np] = (int)gp.size();
  gp.push_back(n);
  upload(P.part_group, pg.data(), pg.size(), false, s);
  upload(P.group_ptr, gp.data(), gp.size(), false, s);
  upload(P.rows, rows.data(), rows.size(), false, s);
  P.nparts = np;
  P.ngroups = (int)gp.size() - 1;
  P.R = R;
  GB_CUDA(cudaStreamSynchronize(s));
}

template <class T, int AR>
void part_launch(gbsym_tri_s *t, T *x, T *y, cudaStream_t s) {
  auto &P = t->part;
  const size_t smem = (size_t)P.R * sizeof(T);
  auto kern = k_part_sweep<T, AR>;
  GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPartBlock, smem));
  GB_CHECK(per_sm > 0, GBSYM_ERR_UNSUPPORTED);
  const int grid = std::max(1, std::min(P.nparts, per_sm * num_sms()));
  TriView<T> A = view_of<T>(t);
  int n = t->n, upper = kind_is_upper(t->kind) ? 1 : 0, R = P.R, np = P.nparts;
  const int *pg = P.part_group.p, *gp = P.group_ptr.p, *rows = P.rows.p;
  int *err = t->err.p;
  void *params[] = {&A, &x, &y, &n, &upper, &R, &np, (void *)&pg, (void *)&gp, (void *)&rows, &err};
  GB_CUDA(cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(kPartBlock), params, smem, s));
  check_launch();
}

}  // namespace

void fill_sentinel(void *y, size_t bytes, cudaStream_t s);  // exec_syncfree.cu

template <class T>
void run_part(gbsym_tri_s *t, T *x, cudaStream_t s) {
  const int R = t->part_rows_pref > 0 ? std::min(t->part_rows_pref, part_rows_max(sizeof(T)))
                                      : part_rows_default(t, sizeof(T));
  build_partitions(t, std::max(1, R), s);
  const size_t bytes = (size_t)t->n * sizeof(T);
  t->sfy.reserve(bytes);
  T *y = reinterpret_cast<T *>(t->sfy.p);
  fill_sentinel(y, bytes, s);
  if (t->arith == kArithFused) part_launch<T, kArithFused>(t, x, y, s);
  else part_launch<T, kArithExact>(t, x, y, s);
}

template void run_part<double>(gbsym_tri_s *, double *, cudaStream_t);
template void run_part<float>(gbsym_tri_s *, float *, cudaStream_t);

}  // namespace gbsym
