// exec_sf_lt.cu -- the look-through sync-free sweeps: every row recomputes
// the values it depends on instead of waiting for them, so it waits on
// values at least two levels back (three for the two-level form) instead
// of one.  Three forms: one right-hand side over one level (the default
// where the plan allows it), one right-hand side over two levels, and
// several right-hand sides over one level (autotuner candidates).
//
// With one right-hand side a row takes four lanes of which one computes;
// here the other three each recompute one of the row's dependencies from
// that dependency's own row data and right-hand side.  Row i needs x_j for
// its dependencies j; lane q+1 rebuilds x_j = (b_j - sum L_jm x_m) / L_jj
// with the same operation sequence the owner of row j uses (storage order,
// separately rounded products and differences, the same division), so the
// value is bit-identical to the one j's owner publishes.  A row therefore
// waits only for its dependencies' dependencies, and each publish -> poll
// hop of the sweep (the L2 round trip that bounds one-right-hand-side
// solves) now advances the wavefront by two levels, at the cost of a second
// dependent FP64 chain per row and of loads the idle lanes would not make.
//
// Every row is still computed and published by its owner, so rows whose
// dependencies look through to it see its value as before.  The solve is
// in place: the right-hand sides are first gathered into a packed-order
// copy (other rows read b_j there, since x_j is overwritten when row j
// finishes), the published values go to the plan's packed scratch.  Used
// for plans whose rows all fit a slab of at most three entries (the three
// spare lanes cover every dependency) and no overflow entries.
//
// Deadlock freedom is the plain sweep's argument: a unit waits only on
// values of rows at least two levels earlier, which belong to earlier
// units, every warp walks its units in order and the launch is cooperative.
#include <algorithm>

#include "exec_syncfree_kernel.cuh"

namespace gbsym {

// b copied into packed order and the scratch set to the sentinel, in one pass
template <class T>
__global__ void k_lt_prep(int n, const int *__restrict__ perm, const T *__restrict__ x, T *__restrict__ bp,
                          T *__restrict__ y) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    bp[r] = x[perm[r]];
    if constexpr (sizeof(T) == 8) reinterpret_cast<unsigned long long *>(y)[r] = ~0ull;
    else reinterpret_cast<unsigned *>(y)[r] = ~0u;
  }
}

template <class T, int AR, int KS>
__global__ void __launch_bounds__(kSfBlock, 3)
k_syncfree_lt(TriView<T> A, T *x, T *y, const T *__restrict__ bp, const int *__restrict__ unit_row,
              const int *__restrict__ unit_cnt, int nunits, int nsm, int *err) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int gl = lane & 3;    // 0: the row itself; q + 1: its dependency q
  const int sub = lane >> 2;  // row of the unit (eight rows per warp unit)
  const int warp = deal_warp(nsm);
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int u = warp; u < nunits; u += nwarps) {
    const bool active = sub < unit_cnt[u];
    const int row = unit_row[u] + sub;
    const int rlen = active ? min(A.len[row], A.K) : 0;
    // lane 0 holds row `row`; lane q + 1 holds dependency q of it
    const bool work = active && (gl == 0 || gl - 1 < rlen);
    const int me = !work ? 0 : (gl == 0 ? row : A.sci[(size_t)(gl - 1) * A.npad + row]);
    RowStatic<T, KS> rs;
    if (work) load_row(A, me, rs);
    T acc = work ? bp[me] : T(0);
    // dependency lanes poll the values their row reads: two rounds of loads
    // in flight, as in the plain sweep's one-value lanes
    const bool dep = work && gl > 0;
    const int ns = dep ? min(rs.len, A.K) : 0;
    const unsigned need = (1u << ns) - 1u;
    unsigned got = 0;
    T xv[KS], va[KS], vb[KS];
    bool done = !dep || ns == 0;
    auto issue = [&](T (&buf)[KS]) {
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < ns && !((got >> q) & 1u)) {
          T v[1];
          ld_rlx<T, 1>(y + rs.c[q], v);
          buf[q] = v[0];
        }
    };
    auto absorb = [&](T (&buf)[KS]) {
      bool moved = false;
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < ns && !((got >> q) & 1u) && !is_sentinel(buf[q])) {
          xv[q] = buf[q];
          got |= 1u << q;
          moved = true;
        }
      if (got == need) done = true;
      return moved;
    };
    if (!done) issue(va);
    long long t0 = clock_now();
    int rounds = 0;
    bool odd = false;
    while (__any_sync(FULL, !done)) {
      bool moved = false;
      if (!done) {
        if (!odd) {
          issue(vb);
          moved = absorb(va);
        } else {
          issue(va);
          moved = absorb(vb);
        }
        if (moved) t0 = clock_now();
      }
      odd = !odd;
      if (!__any_sync(FULL, moved)) __nanosleep(32);
      if ((++rounds & 63) == 0) {
        if (!done && clock_now() - t0 > kWaitLimitCycles) {
          atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
          done = true;
        }
        const int e = lane == 0 ? ld_relaxed(err) : 0;
        if (__shfl_sync(FULL, e, 0) != 0) return;
      }
    }
    // dependency lanes: x_j exactly as row j's owner computes it
    T xj = T(0);
    if (dep) {
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < ns) acc = msub<AR>(acc, rs.v[q], xv[q]);
      xj = row_finish(A, rs, acc);
    }
    const int base = lane & ~3;
    T d[3];
    d[0] = __shfl_sync(FULL, xj, base + 1);
    d[1] = __shfl_sync(FULL, xj, base + 2);
    d[2] = __shfl_sync(FULL, xj, base + 3);
    if (work && gl == 0) {
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < rlen) acc = msub<AR>(acc, rs.v[q], d[q]);
      const T out = row_finish(A, rs, acc);
      x[rs.orig] = out;
      T o[1] = {not_sentinel(out)};
      st_rlx<T, 1>(y + row, o);
    }
  }
}

// ---- one right-hand side, two levels ----------------------------------------
// Sixteen lanes per row (two rows per warp unit): lane 0 the row, lanes
// 1..3 its dependencies j, lanes 4..12 the dependencies of those (lane
// 4 + 3q + m: dependency m of dependency q).  The outer lanes poll values
// three levels back and recompute their rows, the middle lanes rebuild the
// dependencies from those, lane 0 its row: each publish -> poll hop then
// advances the wavefront three levels, for three dependent row chains.
template <class T, int AR, int KS>
__global__ void __launch_bounds__(kSfBlock, 3)
k_syncfree_lt2(TriView<T> A, T *x, T *y, const T *__restrict__ bp, const int *__restrict__ unit_row,
               const int *__restrict__ unit_cnt, int nunits, int nsm, int *err) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int gl = lane & 15;
  const int sub = lane >> 4;
  const int base = lane & 16;
  const int warp = deal_warp(nsm);
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int q1 = gl >= 4 ? (gl - 4) / 3 : gl - 1;  // dependency of the row this lane follows
  const int m2 = gl >= 4 ? (gl - 4) % 3 : 0;       // outer lanes: dependency of that dependency
  for (int u = warp; u < nunits; u += nwarps) {
    const bool active = sub < unit_cnt[u];
    const int row = unit_row[u] + sub;
    const int rlen = active ? min(A.len[row], A.K) : 0;
    int me = row;
    bool work = active && gl <= 12;
    if (work && gl > 0) {
      if (q1 < rlen) {
        me = A.sci[(size_t)q1 * A.npad + row];
        if (gl >= 4) {
          const int l1 = min(A.len[me], A.K);
          if (m2 < l1) me = A.sci[(size_t)m2 * A.npad + me];
          else work = false;
        }
      } else {
        work = false;
      }
    }
    RowStatic<T, KS> rs;
    if (work) load_row(A, me, rs);
    T acc = work ? bp[me] : T(0);
    const bool outer = work && gl >= 4;
    const int ns = outer ? min(rs.len, A.K) : 0;
    const unsigned need = (1u << ns) - 1u;
    unsigned got = 0;
    T xv[KS], va[KS], vb[KS];
    bool done = !outer || ns == 0;
    auto issue = [&](T (&buf)[KS]) {
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < ns && !((got >> q) & 1u)) {
          T v[1];
          ld_rlx<T, 1>(y + rs.c[q], v);
          buf[q] = v[0];
        }
    };
    auto absorb = [&](T (&buf)[KS]) {
      bool moved = false;
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < ns && !((got >> q) & 1u) && !is_sentinel(buf[q])) {
          xv[q] = buf[q];
          got |= 1u << q;
          moved = true;
        }
      if (got == need) done = true;
      return moved;
    };
    if (!done) issue(va);
    long long t0 = clock_now();
    int rounds = 0;
    bool odd = false;
    while (__any_sync(FULL, !done)) {
      bool moved = false;
      if (!done) {
        if (!odd) {
          issue(vb);
          moved = absorb(va);
        } else {
          issue(va);
          moved = absorb(vb);
        }
        if (moved) t0 = clock_now();
      }
      odd = !odd;
      if (!__any_sync(FULL, moved)) __nanosleep(32);
      if ((++rounds & 63) == 0) {
        if (!done && clock_now() - t0 > kWaitLimitCycles) {
          atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
          done = true;
        }
        const int e = lane == 0 ? ld_relaxed(err) : 0;
        if (__shfl_sync(FULL, e, 0) != 0) return;
      }
    }
    // outer lanes: their rows from polled values
    T v2 = T(0);
    if (outer) {
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < ns) acc = msub<AR>(acc, rs.v[q], xv[q]);
      v2 = row_finish(A, rs, acc);
    }
    // middle lanes (1..3): their rows from the outer lanes' values
    const int src2 = (gl >= 1 && gl <= 3) ? base + 4 + 3 * (gl - 1) : lane;
    T d2[3];
    d2[0] = __shfl_sync(FULL, v2, src2);
    d2[1] = __shfl_sync(FULL, v2, gl >= 1 && gl <= 3 ? src2 + 1 : lane);
    d2[2] = __shfl_sync(FULL, v2, gl >= 1 && gl <= 3 ? src2 + 2 : lane);
    T v1 = T(0);
    if (work && gl >= 1 && gl <= 3) {
      const int l1 = min(rs.len, A.K);
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < l1) acc = msub<AR>(acc, rs.v[q], d2[q]);
      v1 = row_finish(A, rs, acc);
    }
    T d1[3];
    d1[0] = __shfl_sync(FULL, v1, base + 1);
    d1[1] = __shfl_sync(FULL, v1, base + 2);
    d1[2] = __shfl_sync(FULL, v1, base + 3);
    if (work && gl == 0) {
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (q < rlen) acc = msub<AR>(acc, rs.v[q], d1[q]);
      const T out = row_finish(A, rs, acc);
      x[rs.orig] = out;
      T o[1] = {not_sentinel(out)};
      st_rlx<T, 1>(y + row, o);
    }
  }
}

template <class T, int AR, int KS>
static void lt2_launch(gbsym_tri_s *t, T *x, T *y, const T *bp, cudaStream_t s) {
  const TriView<T> A = view_packed_of<T>(t);
  const Units U = sf_units(t, 2);
  launch_coop(t, 1, k_syncfree_lt2<T, AR, KS>, s, A, x, y, bp, U.row, U.cnt, U.n, t->sf_deal, t->err.p);
}

// ---- several right-hand sides ---------------------------------------------
// Right-hand sides copied into packed row order (row-major n x k) and the
// scratch set to the sentinel, in one pass: a warp per row, its lanes over
// the row's k values (no division per element).
template <class T>
__global__ void k_lt_prep_mrhs(int n, int k, const int *__restrict__ perm, const T *__restrict__ x,
                               T *__restrict__ bp, T *__restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += nw) {
    const size_t src = (size_t)perm[row] * k, dst = (size_t)row * k;
    for (int c = lane; c < k; c += 32) {
      bp[dst + c] = x[src + c];
      if constexpr (sizeof(T) == 8) reinterpret_cast<unsigned long long *>(y)[dst + c] = ~0ull;
      else reinterpret_cast<unsigned *>(y)[dst + c] = ~0u;
    }
  }
}

// G lanes per row, one value each, columns r = gl + s*G.  Every lane of a
// row recomputes, for its own columns, the values of the row's dependencies
// (from their rows, their right-hand sides and the values they depend on,
// exactly as their owners compute them), then its row: it waits only for
// values two levels back.  The arithmetic per value triples on stencil rows
// of two or three entries; the sweep pays it where the publish -> poll hop,
// not the arithmetic, bounds it (deep narrow wavefronts), and the autotuner
// decides per plan.
template <class T, int G, int AR, int KS>
__global__ void __launch_bounds__(kSfBlock, KS <= 2 ? 3 : 2)
k_syncfree_lt_mrhs(TriView<T> A, T *x, T *y, const T *__restrict__ bp, int k, const int *__restrict__ unit_row,
                   const int *__restrict__ unit_cnt, int nunits, int nsm, int *err) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int gl = lane % G;
  const int sub = lane / G;
  const int warp = deal_warp(nsm);
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nslices = (k + G - 1) / G;
  for (int u = warp; u < nunits; u += nwarps) {
    const bool active = sub < unit_cnt[u];
    const int row = unit_row[u] + sub;
    RowStatic<T, KS> rs;
    RowStatic<T, KS> ds[KS];
    if (active) load_row(A, row, rs);
    const int nq = active ? min(rs.len, A.K) : 0;
#pragma unroll
    for (int q = 0; q < KS; ++q)
      if (q < nq) load_row(A, rs.c[q], ds[q]);
    for (int sl = 0; sl < nslices; ++sl) {
      const int r = gl + sl * G;
      const bool live = active && r < k;
      T acc = live ? bp[(size_t)row * k + r] : T(0);
      T aq[KS], xv[KS][KS];
      unsigned got = 0, need = 0;
#pragma unroll
      for (int q = 0; q < KS; ++q)
        if (live && q < nq) {
          aq[q] = bp[(size_t)rs.c[q] * k + r];
#pragma unroll
          for (int m = 0; m < KS; ++m)
            if (m < min(ds[q].len, A.K)) need |= 1u << (q * KS + m);
        }
      bool done = !live || need == 0;
      long long t0 = clock_now();
      int rounds = 0;
      while (__any_sync(FULL, !done)) {
        bool moved = false;
        if (!done) {
#pragma unroll
          for (int q = 0; q < KS; ++q)
#pragma unroll
            for (int m = 0; m < KS; ++m)
              if (((need & ~got) >> (q * KS + m)) & 1u) {
                T v[1];
                ld_rlx<T, 1>(y + (size_t)ds[q].c[m] * k + r, v);
                xv[q][m] = v[0];  // a value already seen is never loaded again
              }
#pragma unroll
          for (int q = 0; q < KS; ++q)
#pragma unroll
            for (int m = 0; m < KS; ++m)
              if ((((need & ~got) >> (q * KS + m)) & 1u) && !is_sentinel(xv[q][m])) {
                got |= 1u << (q * KS + m);
                moved = true;
              }
          if (got == need) done = true;
          if (moved) t0 = clock_now();
        }
        if (!__any_sync(FULL, moved)) __nanosleep(32);
        if ((++rounds & 63) == 0) {
          if (!done && clock_now() - t0 > kWaitLimitCycles) {
            atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
            done = true;
          }
          const int e = lane == 0 ? ld_relaxed(err) : 0;
          if (__shfl_sync(FULL, e, 0) != 0) return;
        }
      }
      if (live) {
        T xq[KS];
#pragma unroll
        for (int q = 0; q < KS; ++q)
          if (q < nq) {
            T a = aq[q];
#pragma unroll
            for (int m = 0; m < KS; ++m)
              if (m < min(ds[q].len, A.K)) a = msub<AR>(a, ds[q].v[m], xv[q][m]);
            xq[q] = row_finish(A, ds[q], a);
          }
#pragma unroll
        for (int q = 0; q < KS; ++q)
          if (q < nq) acc = msub<AR>(acc, rs.v[q], xq[q]);
        const T out = row_finish(A, rs, acc);
        x[(size_t)rs.orig * k + r] = out;
        T o[1] = {not_sentinel(out)};
        st_rlx<T, 1>(y + (size_t)row * k + r, o);
      }
    }
  }
}

template <class T, int G, int AR, int KS>
static void lt_mrhs_launch(gbsym_tri_s *t, T *x, T *y, const T *bp, int k, cudaStream_t s) {
  const TriView<T> A = view_packed_of<T>(t);
  const Units U = sf_units(t, 32 / G);
  launch_coop(t, k, k_syncfree_lt_mrhs<T, G, AR, KS>, s, A, x, y, bp, k, U.row, U.cnt, U.n, t->sf_deal,
              t->err.p);
}

template <class T, int AR, int KS>
static void lt_mrhs_g(gbsym_tri_s *t, T *x, T *y, const T *bp, int k, cudaStream_t s) {
  if (k <= 2) lt_mrhs_launch<T, 2, AR, KS>(t, x, y, bp, k, s);
  else if (k <= 4) lt_mrhs_launch<T, 4, AR, KS>(t, x, y, bp, k, s);
  else if (k <= 8) lt_mrhs_launch<T, 8, AR, KS>(t, x, y, bp, k, s);
  else if (k <= 16) lt_mrhs_launch<T, 16, AR, KS>(t, x, y, bp, k, s);
  else lt_mrhs_launch<T, 32, AR, KS>(t, x, y, bp, k, s);
}

template <class T>
void run_syncfree_lt_mrhs(gbsym_tri_s *t, T *x, int k, cudaStream_t s) {
  GB_CHECK(t->K <= 3 && t->nov == 0 && k >= 1, GBSYM_ERR_UNSUPPORTED);
  const size_t bytes = (size_t)t->n * k * sizeof(T);
  t->sfy.reserve(bytes);
  t->sfb.reserve(bytes);
  T *y = reinterpret_cast<T *>(t->sfy.p);
  T *bp = reinterpret_cast<T *>(t->sfb.p);
  const int grid = std::max(1, std::min(div_up(t->n, 8), num_sms() * 8));  // eight warps (rows) per block
  k_lt_prep_mrhs<T><<<grid, 256, 0, s>>>(t->n, k, t->perm.p, x, bp, y);
  check_launch();
  const bool fused = t->arith == kArithFused;
  if (t->K <= 2) {
    if (fused) lt_mrhs_g<T, kArithFused, 2>(t, x, y, bp, k, s);
    else lt_mrhs_g<T, kArithExact, 2>(t, x, y, bp, k, s);
  } else {
    if (fused) lt_mrhs_g<T, kArithFused, 3>(t, x, y, bp, k, s);
    else lt_mrhs_g<T, kArithExact, 3>(t, x, y, bp, k, s);
  }
}

template void run_syncfree_lt_mrhs<double>(gbsym_tri_s *, double *, int, cudaStream_t);
template void run_syncfree_lt_mrhs<float>(gbsym_tri_s *, float *, int, cudaStream_t);

template <class T, int AR, int KS>
static void lt_launch(gbsym_tri_s *t, T *x, T *y, const T *bp, cudaStream_t s) {
  const TriView<T> A = view_packed_of<T>(t);
  const Units U = sf_units(t, 8);
  launch_coop(t, 1, k_syncfree_lt<T, AR, KS>, s, A, x, y, bp, U.row, U.cnt, U.n, t->sf_deal, t->err.p);
}

template <class T>
void run_syncfree_lt(gbsym_tri_s *t, T *x, cudaStream_t s) {
  GB_CHECK(t->K <= 3 && t->nov == 0, GBSYM_ERR_UNSUPPORTED);
  const size_t bytes = (size_t)t->n * sizeof(T);
  t->sfy.reserve(bytes);
  t->sfb.reserve(bytes);
  T *y = reinterpret_cast<T *>(t->sfy.p);
  T *bp = reinterpret_cast<T *>(t->sfb.p);
  const int grid = std::max(1, std::min(div_up(t->n, 256), num_sms() * 8));
  k_lt_prep<T><<<grid, 256, 0, s>>>(t->n, t->perm.p, x, bp, y);
  check_launch();
  const bool fused = t->arith == kArithFused;
  if (t->sf_lookthrough == 2) {
    if (t->K <= 2) {
      if (fused) lt2_launch<T, kArithFused, 2>(t, x, y, bp, s);
      else lt2_launch<T, kArithExact, 2>(t, x, y, bp, s);
    } else {
      if (fused) lt2_launch<T, kArithFused, 3>(t, x, y, bp, s);
      else lt2_launch<T, kArithExact, 3>(t, x, y, bp, s);
    }
    return;
  }
  if (t->K <= 2) {
    if (fused) lt_launch<T, kArithFused, 2>(t, x, y, bp, s);
    else lt_launch<T, kArithExact, 2>(t, x, y, bp, s);
  } else {
    if (fused) lt_launch<T, kArithFused, 3>(t, x, y, bp, s);
    else lt_launch<T, kArithExact, 3>(t, x, y, bp, s);
  }
}

template void run_syncfree_lt<double>(gbsym_tri_s *, double *, cudaStream_t);
template void run_syncfree_lt<float>(gbsym_tri_s *, float *, cudaStream_t);

}  // namespace gbsym
