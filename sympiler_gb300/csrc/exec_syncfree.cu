// exec_syncfree.cu -- SYNCFREE executor: one persistent launch, no level
// barriers; every row waits only for its own dependencies.
//
// Rows are processed in packed (level) order, which is a topological order
// of the solve's dependency DAG.  The rows are cut into warp units (32 rows
// for one right-hand side, one row per warp for 64) and unit u goes to warp
// u mod W, each warp walking its units in increasing order.  A unit only
// waits on earlier units; the smallest unfinished unit therefore always has
// all its dependencies done, and since the launch is cooperative (every warp
// co-resident) the sweep cannot deadlock.
//
// Readiness is a per-row flag holding the epoch (solve count) in which the
// row was finished, so flags never need resetting.  A finished row's x
// values are stored, then the group leader fences (release) and writes the
// flag; a waiting row's leader reads its dependencies' flags with relaxed
// loads, all in flight together, and fences (acquire) once they all match
// before the group gathers x through L2.  Waits are bounded: a row that sees
// no progress for the wait limit records GBSYM_ERR_TIMEOUT and every warp
// leaves the sweep.
#include <algorithm>

#include "exec_common.cuh"

namespace gbsym {

constexpr int kSfBlock = 256;

__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

template <class T, int G, int VEC, int AR>
__global__ void __launch_bounds__(kSfBlock)
k_syncfree(TriView<T> A, T *__restrict__ x, int k, int n, int *__restrict__ flags, int epoch, int *err) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int RPW = 32 / G;  // rows per warp unit
  const int lane = threadIdx.x & 31;
  const int gl = lane % G;
  const int leader = lane - gl;
  const int sub = lane / G;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nunits = (n + RPW - 1) / RPW;
  for (int u = warp; u < nunits; u += nwarps) {
    const int row = u * RPW + sub;
    const bool active = row < n;
    RowStatic<T> rs;
    if (active) load_row(A, row, rs);
    bool done = !active;
    int j = 0;  // dependencies confirmed so far (leader lanes)
    unsigned long long t0 = globaltimer_ns();
    int rounds = 0;
    for (;;) {
      if (!__any_sync(FULL, !done)) break;
      int ready = 0;
      if (!done && gl == 0) {
        const int jprev = j;
        int f[kSlabMax];
#pragma unroll
        for (int q = 0; q < kSlabMax; ++q)
          if (q < A.K && q >= j && q < rs.len) f[q] = ld_relaxed(&flags[rs.c[q]]);
#pragma unroll
        for (int q = 0; q < kSlabMax; ++q)
          if (q < A.K && q == j && q < rs.len && f[q] == epoch) ++j;
        if (j >= A.K)
          while (j < rs.len && ld_relaxed(&flags[A.oci[rs.ovb + j - A.K]]) == epoch) ++j;
        ready = j >= rs.len;
        if (j != jprev) t0 = globaltimer_ns();
        if (ready) fence_acq_rel();  // acquire: the producers' stores are visible
      }
      ready = __shfl_sync(FULL, ready, leader);
      __syncwarp();
      if (ready && !done) {
        if (G == 1) {
          T acc = ldx(x + rs.orig);
          acc = row_accumulate<T, true, AR>(A, rs, x, acc);
          x[rs.orig] = row_finish(A, rs, acc);
        } else {
          row_mrhs<T, G, VEC, true, AR>(A, rs, x, k, gl);
        }
      }
      __syncwarp();
      if (ready && !done) {
        if (gl == 0) {
          __threadfence();  // release: this group's x stores before the flag
          st_relaxed(&flags[rs.orig], epoch);
        }
        done = true;
      }
      if ((++rounds & 31) == 0) {
        if (!done && gl == 0 && globaltimer_ns() - t0 > kWaitLimitNs) {
          atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
          done = true;
        }
        const int e = lane == 0 ? ld_relaxed(err) : 0;
        if (__shfl_sync(FULL, e, 0) != 0) return;
      }
    }
  }
}

template <class K, class... Args>
static void launch_coop(K kernel, cudaStream_t s, Args... args) {
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kSfBlock, 0));
  const int grid = std::max(1, per_sm) * num_sms();
  void *params[] = {(void *)&args...};
  GB_CUDA(cudaLaunchCooperativeKernel((const void *)kernel, dim3(grid), dim3(kSfBlock), params, 0, s));
  check_launch();
}

template <class T, int G, int AR>
static void sf_g(gbsym_tri_s *t, T *x, int k, int epoch, cudaStream_t s) {
  const TriView<T> A = view_of<T>(t);
  const bool v4 = sizeof(T) == 4 && (k % 4 == 0) && ((uintptr_t)x % 16 == 0);
  const bool v2 = (k % 2 == 0) && ((uintptr_t)x % (2 * sizeof(T)) == 0);
  if (v4)
    launch_coop(k_syncfree<T, G, (sizeof(T) == 4 ? 4 : 2), AR>, s, A, x, k, t->n, t->flags.p, epoch, t->err.p);
  else if (v2)
    launch_coop(k_syncfree<T, G, 2, AR>, s, A, x, k, t->n, t->flags.p, epoch, t->err.p);
  else
    launch_coop(k_syncfree<T, G, 1, AR>, s, A, x, k, t->n, t->flags.p, epoch, t->err.p);
}

template <class T, int AR>
static void sf_ar(gbsym_tri_s *t, T *x, int k, int epoch, cudaStream_t s) {
  if (k == 1) {
    launch_coop(k_syncfree<T, 1, 1, AR>, s, view_of<T>(t), x, 1, t->n, t->flags.p, epoch, t->err.p);
    return;
  }
  switch (lanes_for(k, sizeof(T))) {
    case 2: sf_g<T, 2, AR>(t, x, k, epoch, s); break;
    case 4: sf_g<T, 4, AR>(t, x, k, epoch, s); break;
    case 8: sf_g<T, 8, AR>(t, x, k, epoch, s); break;
    case 16: sf_g<T, 16, AR>(t, x, k, epoch, s); break;
    default: sf_g<T, 32, AR>(t, x, k, epoch, s); break;
  }
}

template <class T>
void run_syncfree(gbsym_tri_s *t, T *x, int k, cudaStream_t s) {
  if (t->flags.n < (size_t)t->n) {
    t->flags.alloc(t->n);
    GB_CUDA(cudaMemsetAsync(t->flags.p, 0, t->n * sizeof(int), s));
    t->epoch = 0;
  }
  if (++t->epoch >= (1 << 30)) {  // wrap: clear the flags once
    GB_CUDA(cudaMemsetAsync(t->flags.p, 0, t->n * sizeof(int), s));
    t->epoch = 1;
  }
  if (t->arith == kArithFused) sf_ar<T, kArithFused>(t, x, k, t->epoch, s);
  else sf_ar<T, kArithExact>(t, x, k, t->epoch, s);
}

template void run_syncfree<double>(gbsym_tri_s *, double *, int, cudaStream_t);
template void run_syncfree<float>(gbsym_tri_s *, float *, int, cudaStream_t);

}  // namespace gbsym
