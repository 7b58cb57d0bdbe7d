// exec_sweep.cu -- PERSISTENT and ONEBLOCK executors: one launch sweeps all
// wavefront levels.
//
// PERSISTENT: a cooperative launch (every block co-resident); levels are
// separated by a bounded grid barrier -- one release-add per block, acquire
// polling -- and each thread loads the static part of its next row before
// it enters the barrier.  ONEBLOCK: the sweep in a single block, for
// systems whose levels are a few hundred rows wide.  Plans whose rows fit
// a slab of up to four entries run barrier-free with every value published
// in shared memory when the solution and right-hand side fit there
// (k_oneblock_sf), else level by level with three levels of row data in
// flight (k_oneblock_pf); wider rows run level by level with __syncthreads
// as the barrier and x staged in shared memory when it fits.
#include <algorithm>

#include "exec_syncfree.cuh"

namespace gbsym {

// Grid barrier: every block adds 1 with release semantics after its
// stores, then polls with acquire until all blocks of generation `target`
// have arrived.  Returns false (and records GBSYM_ERR_TIMEOUT) when the
// wait runs out, after which every block leaves the sweep.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned target, int *err,
                                             unsigned long long limit_ns = kWaitLimitNs) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    red_release_add(bar, 1u);
    int ok = 1;
    long long it = 0;
    const unsigned long long t0 = globaltimer_ns();
    while ((int)(ld_acquire_u32(bar) - target) < 0) {
      ++it;
      if (it > kWaitLimitIters || ((it & 255) == 0 && globaltimer_ns() - t0 > limit_ns) ||
          ((it & 255) == 0 && ld_relaxed(err) != 0)) {
        atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
        ok = 0;
        break;
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

constexpr int kPersistBlock = 256;
constexpr int kOneBlock = 512;

template <class T, bool ONE_BLOCK, int AR>
__global__ void __launch_bounds__(ONE_BLOCK ? kOneBlock : kPersistBlock)
k_sweep_1rhs(TriView<T> A, T *__restrict__ xg, const int *__restrict__ lev_ptr, int nlev, int n,
             int xs_smem, unsigned *bar, int *err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *x = (ONE_BLOCK && xs_smem) ? reinterpret_cast<T *>(smem_raw) : xg;
  if (ONE_BLOCK && xs_smem) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = xg[i];
    __syncthreads();
  }
  constexpr bool CG = !ONE_BLOCK;
  const int nthr = gridDim.x * blockDim.x;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  RowStatic<T> rs;
  int r0 = lev_ptr[0], r1 = lev_ptr[1];
  if (r0 + gtid < r1) load_row(A, r0 + gtid, rs);
  for (int l = 0; l < nlev; ++l) {
    int row = r0 + gtid;
    if (row < r1) {
      T acc = ldv<T, CG>(x + rs.orig);
      acc = row_accumulate<T, CG, AR>(A, rs, x, acc);
      x[rs.orig] = row_finish(A, rs, acc);
    }
    for (row += nthr; row < r1; row += nthr) {
      RowStatic<T> r2;
      load_row(A, row, r2);
      T acc = ldv<T, CG>(x + r2.orig);
      acc = row_accumulate<T, CG, AR>(A, r2, x, acc);
      x[r2.orig] = row_finish(A, r2, acc);
    }
    if (l + 1 < nlev) {
      const int n0 = r1, n1 = lev_ptr[l + 2];
      if (n0 + gtid < n1) load_row(A, n0 + gtid, rs);
      if (ONE_BLOCK) {
        __syncthreads();
      } else if (!grid_barrier(bar, (unsigned)(l + 1) * gridDim.x, err)) {
        return;
      }
      r0 = n0;
      r1 = n1;
    }
  }
  if (ONE_BLOCK && xs_smem) {
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) xg[i] = x[i];
  }
}

template <class T, int G, int VEC, int AR>
__global__ void __launch_bounds__(kPersistBlock)
k_sweep_mrhs(TriView<T> A, T *__restrict__ x, int k, const int *__restrict__ lev_ptr, int nlev,
             unsigned *bar, int *err) {
  const int ngroups = gridDim.x * blockDim.x / G;
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int lane = threadIdx.x % G;
  RowStatic<T> rs;
  int r0 = lev_ptr[0], r1 = lev_ptr[1];
  if (r0 + gid < r1) load_row(A, r0 + gid, rs);
  for (int l = 0; l < nlev; ++l) {
    int row = r0 + gid;
    if (row < r1) row_mrhs<T, G, VEC, true, AR>(A, rs, x, k, lane);
    for (row += ngroups; row < r1; row += ngroups) {
      RowStatic<T> r2;
      load_row(A, row, r2);
      row_mrhs<T, G, VEC, true, AR>(A, r2, x, k, lane);
    }
    if (l + 1 < nlev) {
      const int n0 = r1, n1 = lev_ptr[l + 2];
      if (n0 + gid < n1) load_row(A, n0 + gid, rs);
      if (!grid_barrier(bar, (unsigned)(l + 1) * gridDim.x, err)) return;
      r0 = n0;
      r1 = n1;
    }
  }
}

static size_t oneblock_smem(const gbsym_tri_s *t, int dsize) {
  const size_t need = (size_t)t->n * dsize;
  return need <= 200 * 1024 ? need : 0;
}

// ONEBLOCK with a three-level pipeline of row data.  A level's arithmetic
// is one short dependent chain (a few FP64 operations on values in shared
// memory), shorter than an L2 round trip; loading the next level's rows
// while the barrier drains hides only the barrier, so every level would
// wait for a round trip.  Here each thread keeps the static data (row
// bounds, permutation, diagonal, slab entries) of its row in three levels
// in registers, in three rotating buffers: a buffer is refilled for level
// l + 3 as soon as level l is done with it, so every load has two whole
// levels to arrive.  Rows past the block's width in wide levels load their
// data directly.  Measured per level on 2D Laplacians (one RHS): 0.69 us
// against 1.1 us for the one-level prefetch.  Prefetching the rows into L1
// two levels ahead instead (prefetch instructions, no registers) measured
// between the two.
template <class T, int KS>
struct OneblockStage {
  int a, b;  // the level's row range
  RowStatic<T, KS> r;
};

template <class T, int AR, int KS>
__global__ void __launch_bounds__(kOneBlock)
k_oneblock_pf(TriView<T> A, T *__restrict__ xg, const int *__restrict__ lev_ptr, int nlev, int n, int xs_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *x = xs_smem ? reinterpret_cast<T *>(smem_raw) : xg;
  if (xs_smem) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = xg[i];
    __syncthreads();
  }
  const int tid = threadIdx.x;
  auto fetch = [&](int l, OneblockStage<T, KS> &st) {
    if (l < nlev) {
      st.a = lev_ptr[l];
      st.b = lev_ptr[l + 1];
      if (st.a + tid < st.b) load_row(A, st.a + tid, st.r);
    }
  };
  auto solve_row = [&](const RowStatic<T, KS> &r) {
    T acc = x[r.orig];
    T xv[KS];
#pragma unroll
    for (int q = 0; q < KS; ++q)
      if (q < A.K && q < r.len) xv[q] = x[r.c[q]];
#pragma unroll
    for (int q = 0; q < KS; ++q)
      if (q < A.K && q < r.len) acc = msub<AR>(acc, r.v[q], xv[q]);
    for (int t = A.K; t < r.len; ++t) {
      const int e = r.ovb + t - A.K;
      acc = msub<AR>(acc, A.ov[e], x[A.oci[e]]);
    }
    x[r.orig] = row_finish(A, r, acc);
  };
  auto level = [&](const OneblockStage<T, KS> &st) {
    if (st.a + tid < st.b) solve_row(st.r);
    for (int row = st.a + tid + kOneBlock; row < st.b; row += kOneBlock) {
      RowStatic<T, KS> r2;
      load_row(A, row, r2);
      solve_row(r2);
    }
  };
  OneblockStage<T, KS> s0, s1, s2;
  fetch(0, s0);
  fetch(1, s1);
  fetch(2, s2);
  for (int l = 0; l < nlev; l += 3) {
    level(s0);
    fetch(l + 3, s0);
    __syncthreads();
    if (l + 1 >= nlev) break;
    level(s1);
    fetch(l + 4, s1);
    __syncthreads();
    if (l + 2 >= nlev) break;
    level(s2);
    fetch(l + 5, s2);
    __syncthreads();
  }
  if (xs_smem) {
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) xg[i] = x[i];
  }
}

// ONEBLOCK, sync-free form, for plans whose rows fit a slab of at most
// four entries and whose right-hand side and solution fit in shared memory
// together: one block and no barriers.  The right-hand side is gathered
// into shared memory in packed row order; the block's warps take the
// plan's 32-row units in turn (unit u to warp u mod W, each warp in
// increasing order; units hold rows of one level, so the argument of the
// sync-free sweep rules out deadlock), and every value is published into a
// shared-memory copy of the solution that starts as an all-ones bit pattern
// (a NaN no arithmetic produces).  A waiting lane polls the values its row
// reads there, a few cycles away instead of an L2 round trip, and a warp
// loads its next units' row data while it works on the current one.
constexpr int kObsfThreads = 512;

template <class T>
__device__ __forceinline__ bool ob_empty(T v) {
  if constexpr (sizeof(T) == 8) return __double_as_longlong(v) == -1ll;
  else return __float_as_int(v) == -1;
}
template <class T>
__device__ __forceinline__ T ob_empty_value() {
  if constexpr (sizeof(T) == 8) return __longlong_as_double(-1ll);
  else return __int_as_float(-1);
}

template <class T, int AR, int KS>
__global__ void __launch_bounds__(kObsfThreads)
k_oneblock_sf(TriView<T> A, T *__restrict__ x, int n, const int *__restrict__ unit_row,
              const int *__restrict__ unit_cnt, int nunits, int *err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *ys = reinterpret_cast<T *>(smem_raw);  // published values, packed order
  T *bs = ys + n;                           // right-hand side, packed order
  int *ur = reinterpret_cast<int *>(bs + n), *uc = ur + nunits;
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    bs[i] = x[A.perm[i]];
    ys[i] = ob_empty_value<T>();
  }
  for (int i = threadIdx.x; i < nunits; i += blockDim.x) {
    ur[i] = unit_row[i];
    uc[i] = unit_cnt[i];
  }
  __syncthreads();
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  volatile T *yv = ys;
  auto fetch = [&](int u, RowStatic<T, KS> &r, int &row, bool &act) {
    act = false;
    if (u < nunits) {
      row = ur[u] + lane;
      act = lane < uc[u];
      if (act) load_row(A, row, r);
    }
  };
  // false when the wait ran out (or another warp's did)
  auto solve = [&](const RowStatic<T, KS> &r, int row, bool act) -> bool {
    const int ns = act ? min(r.len, A.K) : 0;
    const unsigned need = (1u << ns) - 1u;
    unsigned got = 0;
    T xv[KS];
    bool done = need == 0;
    const long long t0 = clock64();
    int rounds = 0;
    while (__any_sync(FULL, !done)) {
      if (!done) {
#pragma unroll
        for (int q = 0; q < KS; ++q)
          if (q < ns && !((got >> q) & 1u)) {
            const T v = yv[r.c[q]];
            if (!ob_empty(v)) {
              xv[q] = v;
              got |= 1u << q;
            }
          }
        done = got == need;
      }
      if ((++rounds & 255) == 0) {
        if (!done && clock64() - t0 > (1ll << 32)) {
          atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
          s_abort = 1;
        }
        if (__any_sync(FULL, *(volatile int *)&s_abort != 0)) return false;
      }
    }
    if (act) {
      T acc = bs[row];
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < ns) acc = msub<AR>(acc, r.v[q], xv[q]);
      const T out = row_finish(A, r, acc);
      x[r.orig] = out;
      yv[row] = ob_empty(out) ? (sizeof(T) == 8 ? T(__longlong_as_double(0x7ff8000000000000ll))
                                                : T(__int_as_float(0x7fc00000)))
                              : out;
    }
    return true;
  };
  RowStatic<T, KS> ra, rb;
  int rowa = 0, rowb = 0;
  bool acta, actb;
  fetch(warp, ra, rowa, acta);
  fetch(warp + nw, rb, rowb, actb);
  for (int u = warp; u < nunits; u += 2 * nw) {
    if (!solve(ra, rowa, acta)) return;
    fetch(u + 2 * nw, ra, rowa, acta);
    if (u + nw >= nunits) break;
    if (!solve(rb, rowb, actb)) return;
    fetch(u + 3 * nw, rb, rowb, actb);
  }
}

template <class T, int AR, int KS>
static void oneblock_sf(gbsym_tri_s *t, T *x, const Units &U, size_t sm, cudaStream_t s) {
  auto kern = k_oneblock_sf<T, AR, KS>;
  if (sm > 48 * 1024)
    GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  kern<<<1, kObsfThreads, sm, s>>>(view_packed_of<T>(t), x, t->n, U.row, U.cnt, U.n, t->err.p);
  check_launch();
}

template <class T, int AR, int KS>
static void oneblock_pf(gbsym_tri_s *t, T *x, size_t sm, cudaStream_t s) {
  auto kern = k_oneblock_pf<T, AR, KS>;
  if (sm > 48 * 1024)
    GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  kern<<<1, kOneBlock, sm, s>>>(view_of<T>(t), x, t->lev_ptr.p, t->nlev, t->n, sm > 0 ? 1 : 0);
  check_launch();
}

template <class T, int AR>
static void oneblock_ar(gbsym_tri_s *t, T *x, cudaStream_t s) {
  const size_t sm = oneblock_smem(t, sizeof(T));
  // rows of up to four entries with the solution and right-hand side in
  // shared memory: the barrier-free form (C1, 2D 100^2: 133 us warm and 139
  // cold, against 136 and 215 for the pipelined barrier form; 3D 20^3: 64
  // against 81 us)
  if (t->nov == 0 && t->K <= 4 && t->n > 0) {
    const Units U = sf_units(t, 32);
    const size_t need = 2 * (size_t)t->n * sizeof(T) + 2 * (size_t)U.n * sizeof(int);
    if (need <= 200 * 1024) {
      if (t->K <= 2) oneblock_sf<T, AR, 2>(t, x, U, need, s);
      else if (t->K == 3) oneblock_sf<T, AR, 3>(t, x, U, need, s);
      else oneblock_sf<T, AR, 4>(t, x, U, need, s);
      return;
    }
  }
  // slabs of up to four entries: the pipelined kernel (C1, 2D 100^2: 138
  // against 221 us; 3D 30^3: 190 against 239 us); wider slabs keep the
  // one-level prefetch, whose registers the pipeline's three buffers would
  // spill
  if (t->K <= 4) {
    if (t->K <= 2) oneblock_pf<T, AR, 2>(t, x, sm, s);
    else if (t->K == 3) oneblock_pf<T, AR, 3>(t, x, sm, s);
    else oneblock_pf<T, AR, 4>(t, x, sm, s);
    return;
  }
  auto kern = k_sweep_1rhs<T, true, AR>;
  if (sm > 48 * 1024)
    GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  kern<<<1, kOneBlock, sm, s>>>(view_of<T>(t), x, t->lev_ptr.p, t->nlev, t->n, sm > 0 ? 1 : 0, t->bar.p,
                                t->err.p);
  check_launch();
}

template <class T>
void run_oneblock(gbsym_tri_s *t, T *x, cudaStream_t s) {
  if (t->arith == kArithFused) oneblock_ar<T, kArithFused>(t, x, s);
  else oneblock_ar<T, kArithExact>(t, x, s);
}

// Grid of the persistent sweep: enough groups to cover the widest level,
// bounded by what is co-resident (the cooperative launch checks it).
template <class K>
static int persist_grid(gbsym_tri_s *t, K kernel, int lanes_per_row) {
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistBlock, 0));
  const int cap = std::max(1, per_sm) * num_sms();
  const long long want = div_up((long long)t->max_level_rows * lanes_per_row, kPersistBlock);
  int g = (int)std::min<long long>(cap, std::max<long long>(1, want));
  if (t->persist_blocks > 0) g = std::min(g, t->persist_blocks);
  return g;
}

template <class K, class... Args>
static void launch_coop(K kernel, int grid, cudaStream_t s, Args... args) {
  void *params[] = {(void *)&args...};
  GB_CUDA(cudaLaunchCooperativeKernel((const void *)kernel, dim3(grid), dim3(kPersistBlock), params, 0, s));
  check_launch();
}

template <class T, int G, int AR>
static void persist_mrhs_g(gbsym_tri_s *t, T *x, int k, cudaStream_t s) {
  const TriView<T> A = view_of<T>(t);
  const int *lp = t->lev_ptr.p;
  const bool v4 = sizeof(T) == 4 && (k % 4 == 0) && ((uintptr_t)x % 16 == 0);
  const bool v2 = (k % 2 == 0) && ((uintptr_t)x % (2 * sizeof(T)) == 0);
  if (v4) {
    auto kern = k_sweep_mrhs<T, G, (sizeof(T) == 4 ? 4 : 2), AR>;
    launch_coop(kern, persist_grid(t, kern, G), s, A, x, k, lp, t->nlev, t->bar.p, t->err.p);
  } else if (v2) {
    auto kern = k_sweep_mrhs<T, G, 2, AR>;
    launch_coop(kern, persist_grid(t, kern, G), s, A, x, k, lp, t->nlev, t->bar.p, t->err.p);
  } else {
    auto kern = k_sweep_mrhs<T, G, 1, AR>;
    launch_coop(kern, persist_grid(t, kern, G), s, A, x, k, lp, t->nlev, t->bar.p, t->err.p);
  }
}

template <class T, int AR>
static void persist_ar(gbsym_tri_s *t, T *x, int k, cudaStream_t s) {
  if (k == 1) {
    auto kern = k_sweep_1rhs<T, false, AR>;
    launch_coop(kern, persist_grid(t, kern, 1), s, view_of<T>(t), x, (const int *)t->lev_ptr.p, t->nlev,
                t->n, 0, t->bar.p, t->err.p);
    return;
  }
  switch (lanes_for(k, sizeof(T))) {
    case 2: persist_mrhs_g<T, 2, AR>(t, x, k, s); break;
    case 4: persist_mrhs_g<T, 4, AR>(t, x, k, s); break;
    case 8: persist_mrhs_g<T, 8, AR>(t, x, k, s); break;
    case 16: persist_mrhs_g<T, 16, AR>(t, x, k, s); break;
    default: persist_mrhs_g<T, 32, AR>(t, x, k, s); break;
  }
}

template <class T>
void run_persist(gbsym_tri_s *t, T *x, int k, cudaStream_t s) {
  GB_CUDA(cudaMemsetAsync(t->bar.p, 0, sizeof(unsigned), s));
  if (t->arith == kArithFused) persist_ar<T, kArithFused>(t, x, k, s);
  else persist_ar<T, kArithExact>(t, x, k, s);
}

// Self-test of the bounded wait: block 1 never arrives, so block 0's barrier
// wait can only end through its limit, recording GBSYM_ERR_TIMEOUT.
__global__ void k_selftest_barrier(unsigned *bar, int *err, unsigned long long limit_ns) {
  if (blockIdx.x == 1) return;
  grid_barrier(bar, 2u, err, limit_ns);
}

int selftest_timeout(unsigned long long limit_ns, cudaStream_t s) {
  DBuf<unsigned> bar(1);
  DBuf<int> err(2);
  GB_CUDA(cudaMemsetAsync(bar.p, 0, sizeof(unsigned), s));
  GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
  unsigned *bp = bar.p;
  int *ep = err.p;
  void *params[] = {(void *)&bp, (void *)&ep, (void *)&limit_ns};
  GB_CUDA(cudaLaunchCooperativeKernel((const void *)k_selftest_barrier, dim3(2), dim3(32), params, 0, s));
  check_launch();
  int h[2];
  GB_CUDA(cudaMemcpyAsync(h, err.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  return h[0];
}

template void run_oneblock<double>(gbsym_tri_s *, double *, cudaStream_t);
template void run_oneblock<float>(gbsym_tri_s *, float *, cudaStream_t);
template void run_persist<double>(gbsym_tri_s *, double *, int, cudaStream_t);
template void run_persist<float>(gbsym_tri_s *, float *, int, cudaStream_t);

}  // namespace gbsym

namespace gbsym {

// FP64 throughput probe: every thread runs two independent chains of
// MODE 0: the exact update acc = RN(acc - RN(v*x)) as the sweeps issue it,
// MODE 1: general fused multiply-adds with three variable operands (the
// form of the division's remainder and correction steps).
// Every iteration XORs the low mantissa bits of v with the iteration count
// (integer ops, another pipe), so that no stage of the compiler can hoist
// the product RN(v*x) out of the loop: an empty asm statement is not
// enough, as it leaves no instruction behind for the assembler to respect.
template <int MODE>
__global__ void __launch_bounds__(256) k_fp64_rate(int iters, double *out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double v[2], x[2], a[2];
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    v[c] = 1e-4 * (1 + ((t * 7 + c * 3) & 15));
    x[c] = 1.0 + 0.01 * ((t + c) & 31);
    a[c] = 10.0 + c + 0.001 * (t & 63);
  }
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      v[c] = __longlong_as_double(__double_as_longlong(v[c]) ^ (long long)(it & 1023));
      if (MODE == 0) a[c] = msub<kArithExact>(a[c], v[c], x[c]);
      else a[c] = __fma_rn(__fma_rn(a[c], v[c], x[c]), x[c], v[c]);
    }
  }
  out[t] = a[0] + a[1];
}

template <int MODE>
static double fp64_rate(double *out, cudaStream_t s) {
  const int grid = 4 * num_sms(), iters = 4096;
  struct Events {
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Events() {
      for (auto v : e)
        if (v) cudaEventDestroy(v);
    }
  } ev;
  GB_CUDA(cudaEventCreate(&ev.e[0]));
  GB_CUDA(cudaEventCreate(&ev.e[1]));
  k_fp64_rate<MODE><<<grid, 256, 0, s>>>(iters / 8, out);  // warm-up
  check_launch();
  GB_CUDA(cudaEventRecord(ev.e[0], s));
  k_fp64_rate<MODE><<<grid, 256, 0, s>>>(iters, out);
  check_launch();
  GB_CUDA(cudaEventRecord(ev.e[1], s));
  GB_CUDA(cudaEventSynchronize(ev.e[1]));
  float ms = 0.f;
  GB_CUDA(cudaEventElapsedTime(&ms, ev.e[0], ev.e[1]));
  return 2.0 * 2.0 * grid * 256.0 * iters / (ms * 1e-3) / 1e9;  // two ops per update, two chains
}

}  // namespace gbsym

extern "C" int gbsym_fp64_rates(double *update_gops, double *fma_gops, void *stream) {
  if (!update_gops || !fma_gops) return GBSYM_ERR_NULL_ARG;
  return gbsym::guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    gbsym::DBuf<double> out((size_t)4 * gbsym::num_sms() * 256);
    *update_gops = gbsym::fp64_rate<0>(out.p, s);
    *fma_gops = gbsym::fp64_rate<1>(out.p, s);
  });
}

extern "C" int gbsym_selftest_bounded_wait(long long limit_ns, void *stream) {
  if (limit_ns <= 0 || limit_ns > 10000000000ll) return GBSYM_ERR_SIZE;
  int code = GBSYM_OK;
  const int st = gbsym::guarded([&] { code = gbsym::selftest_timeout((unsigned long long)limit_ns, (cudaStream_t)stream); });
  return st ? st : code;
}
