// exec_syncfree_kernel.cuh -- SYNCFREE executor kernel: one persistent
// launch, no level barriers; every (row, right-hand-side slice) waits only
// for the values it reads.
//
// Rows are processed in packed (level) order, which is a topological order
// of the solve's dependency DAG.  The rows are cut into warp units (32 rows
// for one right-hand side, one row per warp for 64) and unit u goes to warp
// u mod W, each warp walking its units in increasing order.  A unit only
// waits on earlier units; the smallest unfinished unit therefore always has
// all its dependencies done, and since the launch is cooperative (every warp
// co-resident) the sweep cannot deadlock.
//
// Values are their own ready flags.  Before the sweep a scratch copy y of
// the solution is filled with an all-ones bit pattern (a NaN no arithmetic
// produces); a finished value is stored to x and, with a relaxed store, to
// y.  A waiting lane polls the y values it needs with relaxed loads -- the
// poll is the gather -- and proceeds once none of them is the sentinel.
// Each 4- or 8-byte value is written by one store and read by one load, so
// a value seen is a value finished: no fence is needed anywhere, which on
// this part removes over a microsecond from every step of the dependency
// chain.  Waits are bounded: a lane that sees no progress for the wait
// limit records GBSYM_ERR_TIMEOUT and every warp leaves the sweep.
//
// This header holds the kernel and its launch dispatch; each exec_sf_ks*.cu
// instantiates it for one slab width.
#pragma once

#include <algorithm>
#include <cstdint>

#include "exec_syncfree.cuh"

namespace gbsym {

__device__ __forceinline__ bool is_sentinel(double v) { return __double_as_longlong(v) == -1ll; }
__device__ __forceinline__ bool is_sentinel(float v) { return __float_as_int(v) == -1; }
__device__ __forceinline__ double not_sentinel(double v) {
  return is_sentinel(v) ? __longlong_as_double(0x7ff8000000000000ll) : v;
}
__device__ __forceinline__ float not_sentinel(float v) {
  return is_sentinel(v) ? __int_as_float(0x7fc00000) : v;
}

// relaxed (L2-coherent, never hoisted) loads and stores of 1/2/4 values
template <class T, int VEC>
__device__ __forceinline__ void ld_rlx(const T *p, T (&v)[VEC]);
template <>
__device__ __forceinline__ void ld_rlx<double, 1>(const double *p, double (&v)[1]) {
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v[0]) : "l"(p) : "memory");
}
template <>
__device__ __forceinline__ void ld_rlx<double, 2>(const double *p, double (&v)[2]) {
  asm volatile("ld.relaxed.gpu.global.v2.f64 {%0, %1}, [%2];" : "=d"(v[0]), "=d"(v[1]) : "l"(p) : "memory");
}
template <>
__device__ __forceinline__ void ld_rlx<float, 1>(const float *p, float (&v)[1]) {
  asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v[0]) : "l"(p) : "memory");
}
template <>
__device__ __forceinline__ void ld_rlx<float, 2>(const float *p, float (&v)[2]) {
  asm volatile("ld.relaxed.gpu.global.v2.f32 {%0, %1}, [%2];" : "=f"(v[0]), "=f"(v[1]) : "l"(p) : "memory");
}
template <>
__device__ __forceinline__ void ld_rlx<float, 4>(const float *p, float (&v)[4]) {
  asm volatile("ld.relaxed.gpu.global.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]) : "l"(p) : "memory");
}
template <class T, int VEC>
__device__ __forceinline__ void st_rlx(T *p, const T (&v)[VEC]);
template <>
__device__ __forceinline__ void st_rlx<double, 1>(double *p, const double (&v)[1]) {
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v[0]) : "memory");
}
template <>
__device__ __forceinline__ void st_rlx<double, 2>(double *p, const double (&v)[2]) {
  asm volatile("st.relaxed.gpu.global.v2.f64 [%0], {%1, %2};" ::"l"(p), "d"(v[0]), "d"(v[1]) : "memory");
}
template <>
__device__ __forceinline__ void st_rlx<float, 1>(float *p, const float (&v)[1]) {
  asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v[0]) : "memory");
}
template <>
__device__ __forceinline__ void st_rlx<float, 2>(float *p, const float (&v)[2]) {
  asm volatile("st.relaxed.gpu.global.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(v[0]), "f"(v[1]) : "memory");
}
template <>
__device__ __forceinline__ void st_rlx<float, 4>(float *p, const float (&v)[4]) {
  asm volatile("st.relaxed.gpu.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v[0]), "f"(v[1]),
               "f"(v[2]), "f"(v[3])
               : "memory");
}

template <class T, int VEC>
__device__ __forceinline__ bool all_ready(const T (&v)[VEC]) {
  bool ok = true;
#pragma unroll
  for (int u = 0; u < VEC; ++u) ok = ok && !is_sentinel(v[u]);
  return ok;
}

// Bounded waits count SM clock cycles (a register read, unlike the global
// timer); 2^32 cycles is about two seconds at this part's clocks.
__device__ __forceinline__ long long clock_now() { return clock64(); }

// Entries past the slab are polled and accumulated this many at a time:
// one L2 round trip per group instead of one per entry (rows longer than
// the slab otherwise wait a round trip per extra entry, twice).  Two for
// the kernels whose registers four would spill.
template <class T, int VEC>
constexpr int ov_batch() { return (sizeof(T) == 8 || VEC == 4) ? 2 : 4; }
constexpr long long kWaitLimitCycles = 1ll << 32;

// Position of this warp in the order units are dealt.  A cooperative grid
// of R blocks per SM over nsm SMs places blocks b and b + nsm on one SM (the
// usual round-robin placement); dealing unit u to
//   v = ((b / nsm) * warps_per_block + w) * nsm + b % nsm
// puts consecutive units on consecutive SMs and then on different warp
// slots of an SM, so a level's units spread evenly over SMs and their
// sub-partitions instead of filling a contiguous range of blocks (which
// gives some SMs twice the rows of others).  The map is a bijection of the
// warps, so any placement stays correct.  nsm = 0 keeps the plain order.
__device__ __forceinline__ int deal_warp(int nsm) {
  const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5, b = blockIdx.x;
  if (nsm <= 0 || gridDim.x % nsm != 0) return b * wpb + w;
  return ((b / nsm) * wpb + w) * nsm + b % nsm;
}

// G lanes per row; each lane owns the slices r = gl*VEC + s*G*VEC of its
// row and works on one slice at a time.  Warp units hold rows of a single
// level (units are cut per level), so no row of a unit waits on another.
// Per slice the warp first polls until every lane holds all the values its
// slice reads -- a loop with no floating-point work, so polling rounds cost
// the FP64 pipe nothing -- and then each lane computes and publishes its
// slice once, in storage order.
// A narrow slab (KS = 4) fits in 80 registers without spilling, which lets
// three blocks share an SM; the full slab fits two blocks (128 registers).
// OVB: entries past the slab are polled and accumulated OVB at a time; a
// plan without such entries runs the OVB = 0 kernel, which has no code
// (and holds no registers) for them.
template <class T, int G, int VEC, int AR, int KS, int OVB>
__global__ void __launch_bounds__(kSfBlock, KS <= 4 ? 3 : 2)
k_syncfree(TriView<T> A, T *x, T *y, const T *b, int k, const int *__restrict__ unit_row,
           const int *__restrict__ unit_cnt, int nunits, int nsm, int *err) {
  // in place (b null): right-hand sides from x, results to x and published
  // to y, the plan's scratch, in packed row order (A's dependency columns
  // are then packed row numbers); out of place: right-hand sides from b,
  // results published to y = x in the caller's row order
  const T *rhs = b ? b : x;
  const bool store_x = y != x;
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int gl = lane % G;
  const int sub = lane / G;
  const int warp = deal_warp(nsm);
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nslices = (k + G * VEC - 1) / (G * VEC);
  for (int u = warp; u < nunits; u += nwarps) {
    const bool active = sub < unit_cnt[u];
    const int row = unit_row[u] + sub;
    RowStatic<T, KS> rs;
    if (active) load_row(A, row, rs);
    const int ns = active ? min(rs.len, A.K) : 0;
    for (int sl = 0; sl < nslices; ++sl) {
      const int r = gl * VEC + sl * G * VEC;
      bool done = !(active && r < k);
      T xv[KS][VEC];
      unsigned got = 0;
      const unsigned need = (1u << ns) - 1u;
      int jo = A.K;          // next overflow dependency
      bool slab_done = false;  // the slab's updates are in acc
      T acc[VEC];
      if (!done) vload<T, VEC, false>(rhs + (size_t)rs.orig * k + r, acc);
      long long t0 = clock_now();
      int rounds = 0;
      // With one value per lane, polling keeps two rounds of slab loads in
      // flight: round i+1 is issued before round i's results are examined,
      // so a value published just after one poll left is seen about half an
      // L2 round trip later instead of a whole one (measured 18-23% off the
      // one-right-hand-side sweeps).  The two buffers alternate without
      // copies (a copy would wait for the loads).  Wider lanes keep a single
      // round: the second buffer's registers would halve their occupancy.
      constexpr bool kTwoRounds = VEC == 1;
      T va[KS][VEC], vb[KS][VEC];
      auto issue = [&](T (&buf)[KS][VEC]) {
#pragma unroll
        for (int q = 0; q < KS; ++q)
          if (q < ns && !((got >> q) & 1u)) ld_rlx<T, VEC>(y + (size_t)rs.c[q] * k + r, buf[q]);
      };
      auto absorb = [&](T (&buf)[KS][VEC]) {
        bool moved = false;
#pragma unroll
        for (int q = 0; q < KS; ++q)
          if (q < ns && !((got >> q) & 1u) && all_ready<T, VEC>(buf[q])) {
#pragma unroll
            for (int w = 0; w < VEC; ++w) xv[q][w] = buf[q][w];
            got |= 1u << q;
            moved = true;
          }
        // overflow dependencies, OVB per round, once the slab is complete:
        // the slab's updates are applied first (storage order), then each
        // overflow value is applied as soon as it and the ones before it
        // are ready -- no second round trip to load them again
        if constexpr (OVB > 0) {
          if (got == need && jo < rs.len) {
            if (!slab_done) {
#pragma unroll
              for (int q = 0; q < KS; ++q)
                if (q < ns) {
#pragma unroll
                  for (int w = 0; w < VEC; ++w) acc[w] = msub<AR>(acc[w], rs.v[q], xv[q][w]);
                }
              slab_done = true;
            }
            T v[OVB][VEC], a[OVB];
#pragma unroll
            for (int b = 0; b < OVB; ++b)
              if (jo + b < rs.len) {
                const int e = rs.ovb + jo + b - A.K;
                ld_rlx<T, VEC>(y + (size_t)A.oci[e] * k + r, v[b]);
                a[b] = A.ov[e];
              }
            bool run = true;
#pragma unroll
            for (int b = 0; b < OVB; ++b)
              if (run && jo < rs.len && all_ready<T, VEC>(v[b])) {
#pragma unroll
                for (int w = 0; w < VEC; ++w) acc[w] = msub<AR>(acc[w], a[b], v[b][w]);
                ++jo;
                moved = true;
              } else {
                run = false;
              }
          }
        }
        if (got == need && (OVB == 0 || jo >= rs.len)) done = true;
        return moved;
      };
      if (kTwoRounds && !done) issue(va);
      bool odd = false;
      while (__any_sync(FULL, !done)) {
        bool moved = false;
        if (!done) {
          if (!kTwoRounds) {
            issue(va);
            moved = absorb(va);
          } else if (!odd) {
            issue(vb);
            moved = absorb(va);
          } else {
            issue(va);
            moved = absorb(vb);
          }
          if (moved) t0 = clock_now();
        }
        odd = !odd;
        if (!__any_sync(FULL, moved)) __nanosleep(32);  // nothing moved: back off briefly
        if ((++rounds & 63) == 0) {
          if (!done && clock_now() - t0 > kWaitLimitCycles) {
            atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
            done = true;  // give up on this slice; the launch is abandoned
          }
          const int e = lane == 0 ? ld_relaxed(err) : 0;
          if (__shfl_sync(FULL, e, 0) != 0) return;
        }
      }
      if (active && r < k) {
        // the slab's updates, unless the overflow polling applied them
        if (!slab_done) {
#pragma unroll
          for (int q = 0; q < KS; ++q)
            if (q < ns) {
#pragma unroll
              for (int w = 0; w < VEC; ++w) acc[w] = msub<AR>(acc[w], rs.v[q], xv[q][w]);
            }
        }
        T out[VEC];
#pragma unroll
        for (int w = 0; w < VEC; ++w) {
          acc[w] = row_finish(A, rs, acc[w]);
          out[w] = not_sentinel(acc[w]);
        }
        if (store_x) vstore<T, VEC>(x + (size_t)rs.orig * k + r, acc);
        st_rlx<T, VEC>(y + (size_t)(store_x ? row : rs.orig) * k + r, out);
      }
    }
  }
}

template <class K, class... Args>
static void launch_coop(gbsym_tri_s *t, int k_of_launch, K kernel, cudaStream_t s, Args... args) {
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kSfBlock, 0));
  // fewer resident warps poll less, more hide the FP64 chain: one block per
  // SM measured best for one right-hand side, two for a few, three (where
  // the registers allow) for 32 and more (C2 factor: 262 us at one RHS;
  // 277 / 279 / 310 us at 8 RHS and 974 / 573 / 500 us at 64 RHS with
  // one / two / three blocks)
  int want = t->sf_blocks_per_sm;
  if (want <= 0) want = t->sf_bps_tuned[k_of_launch > 1 ? 1 : 0];
  if (want <= 0) want = k_of_launch == 1 ? 1 : (k_of_launch < 32 ? 2 : 3);
  const int grid = std::max(1, std::min(per_sm, want)) * num_sms();
  void *params[] = {(void *)&args...};
  GB_CUDA(cudaLaunchCooperativeKernel((const void *)kernel, dim3(grid), dim3(kSfBlock), params, 0, s));
  check_launch();
}

// KS: slab capacity compiled into the kernel's registers.  A kernel whose
// unrolled slab loops match the plan's slab width issues no guard
// instructions for slots a row cannot have, which the polling loop repeats
// every round (C2 64-RHS: 500 us at KS = 4 against 416 us at KS = 3).
template <class T, int G, int AR, int KS, bool OV>
static void sf_gk(gbsym_tri_s *t, T *x, T *y, const T *b, int k, cudaStream_t s) {
  const TriView<T> A = y != x ? view_packed_of<T>(t) : view_of<T>(t);
  const Units U = sf_units(t, 32 / G);
  // FP64 takes one value per lane: the polling then keeps two rounds of
  // loads in flight, which outweighs the narrower loads (measured 6-25%
  // faster for 8 to 64 right-hand sides on the C2 factor).  FP32 keeps
  // 2- or 4-wide lanes by default, which measured faster there for 8 and
  // 64; the autotuner may choose two values per lane (sf_alt_lanes), which
  // halves the rows of a warp unit at 8 right-hand sides.
  if constexpr (sizeof(T) == 4) {
    if (k > 1 && t->sf_alt_lanes == 1) {
      if (k % 2 == 0 && ((uintptr_t)x | (uintptr_t)(b ? b : x)) % 8 == 0)
        launch_coop(t, k, k_syncfree<T, G, 2, AR, KS, OV ? ov_batch<T, 2>() : 0>, s, A, x, y, b, k, U.row, U.cnt, U.n, t->sf_deal, t->err.p);
      else
        launch_coop(t, k, k_syncfree<T, G, 1, AR, KS, OV ? ov_batch<T, 1>() : 0>, s, A, x, y, b, k, U.row, U.cnt, U.n, t->sf_deal, t->err.p);
      return;
    }
    if (k % 4 == 0 && ((uintptr_t)x | (uintptr_t)(b ? b : x)) % 16 == 0) {
      launch_coop(t, k, k_syncfree<T, G, 4, AR, KS, OV ? ov_batch<T, 4>() : 0>, s, A, x, y, b, k, U.row, U.cnt, U.n, t->sf_deal, t->err.p);
      return;
    }
    if (k % 2 == 0 && ((uintptr_t)x | (uintptr_t)(b ? b : x)) % 8 == 0) {
      launch_coop(t, k, k_syncfree<T, G, 2, AR, KS, OV ? ov_batch<T, 2>() : 0>, s, A, x, y, b, k, U.row, U.cnt, U.n, t->sf_deal, t->err.p);
      return;
    }
  }
  launch_coop(t, k, k_syncfree<T, G, 1, AR, KS, OV ? ov_batch<T, 1>() : 0>, s, A, x, y, b, k, U.row, U.cnt, U.n, t->sf_deal, t->err.p);
}

template <class T, int AR, int KS, bool OV>
static void sf_ar(gbsym_tri_s *t, T *x, T *y, const T *b, int k, cudaStream_t s) {
  if (k == 1) {
    // one right-hand side: 8 rows per warp unit (4 lanes each, one active).
    // A unit waits for all its rows' dependencies before computing, so
    // fewer rows per unit shorten that wait; fewer than 8 costs more in
    // FP64 issue slots than it saves (measured on the C2 and C3 factors:
    // 8 rows 4-5% faster than 32, 1 row twice as slow)
    sf_gk<T, 4, AR, KS, OV>(t, x, y, b, k, s);
    return;
  }
  // FP64 lanes carry one value each, so by default a row takes the next
  // power of two at or above k lanes (at most 32): one slice per row up to
  // 32 right-hand sides (C2: 8 RHS 260 -> 246 us, 32 RHS 325 -> 308 us
  // against half as many lanes, each taking two slices).  Which is faster
  // depends on the matrix (the C4 batch prefers half at 8 RHS), so the
  // autotuner chooses (sf_alt_lanes).  FP32 lanes carry four values (two
  // when k is not a multiple of four) by default, two as the alternative.
  int g64 = 2;
  while (g64 < k && g64 < 32) g64 <<= 1;
  int g32alt = 2;
  while (g32alt * 2 < k && g32alt < 32) g32alt <<= 1;
  const bool alt = t->sf_alt_lanes == 1;
  const int lanes = sizeof(T) == 8 ? (alt ? lanes_for(k, sizeof(T)) : g64) : (alt ? g32alt : lanes_for(k, sizeof(T)));
  switch (lanes) {
    case 2: sf_gk<T, 2, AR, KS, OV>(t, x, y, b, k, s); break;
    case 4: sf_gk<T, 4, AR, KS, OV>(t, x, y, b, k, s); break;
    case 8: sf_gk<T, 8, AR, KS, OV>(t, x, y, b, k, s); break;
    case 16: sf_gk<T, 16, AR, KS, OV>(t, x, y, b, k, s); break;
    default: sf_gk<T, 32, AR, KS, OV>(t, x, y, b, k, s); break;
  }
}

template <class T, int KS, bool OV>
void sf_run_ks(gbsym_tri_s *t, T *x, T *y, const T *b, int k, cudaStream_t s) {
  if (t->arith == kArithFused) sf_ar<T, kArithFused, KS, OV>(t, x, y, b, k, s);
  else sf_ar<T, kArithExact, KS, OV>(t, x, y, b, k, s);
}

}  // namespace gbsym
