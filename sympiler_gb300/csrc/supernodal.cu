// supernodal.cu -- forward and transposed solves with a supernodal
// (blocked CSC) factor: the reference's ParSy blocked solves
// (sparse_blas/parsy/triangularSolve/Triangular_BCSC.cpp).
//
// Storage (the reference's): supernode s owns columns c0 = sup2col[s] ..
// c1 = sup2col[s+1]; its rows are Li[Li_ptr[c0] .. Li_ptr[c1]), its own
// columns first, and its values a column-major block of nr = Li_ptr[c1] -
// Li_ptr[c0] rows at Lx + Lp[c0].  x is column-major n x k.
//
// Forward order.  The reference (blockedLsolve, :23-58) walks supernodes in
// order: a dense solve of the diagonal block (dlsolve_blas_nonUnit), then
// the off-block rows' products (dmatvec_blas) subtracted from the rows they
// reach.  Row q of a supernode therefore sees: the products of its sources
// in increasing source order, then -- dlsolve_blas_nonUnit's runs of 8, 4,
// 2, 1 columns unrolled -- one rounded product and one rounded difference
// per earlier column of its own block, in column order, and finally an
// IEEE division.  Each off-block product is dmatvec_blas's grouping: column
// runs of 8 while 8 remain, then 4, then single columns, each run summed
// left to right, the run sums added to a running +0.  Both groupings are
// restated from parsy/triangularSolve/BLAS.cpp:12-185; results here are the
// reference's, bit for bit.
//
// Transposed order (this library's own: under SYM_BLAS the reference's
// blockedLTsolve, Triangular_BCSC.cpp:124-177, applies the forward kernels
// and is marked FIXME).  Supernodes in decreasing order; column q: x_q minus
// its off-block column's product with the solved rows, in the same run
// grouping but taken from the last off-block row backward; then one rounded
// product and difference per later column of the diagonal block, from the
// last; then the division.
//
// Execution.  FP64 on this part issues one warp instruction per 67.5 cycles
// per SM sub-partition, so a supernode of w columns is far too much work for
// one block: the top separator of a 3D grid alone holds w^2/2 products on a
// critical path of w dependent (multiply, subtract, divide) steps.  One
// persistent launch works through a task list in which every task is one
// warp's:
//   forward  D(s, i)  rows 32i..32i+31 of s's diagonal block: pull the
//                     sources' products (in source order), apply the columns
//                     of tiles 0..i-1, solve the tile;
//            P(s, o)  32/H off-block rows of s, H lanes per row splitting
//                     its column runs; the run sums are chained in order
//                     through shuffles.  Products go to a contribution
//                     buffer, one slot per (source, off-block row).
//   transposed O(s, a)  32/H columns' off-block products, x_q updated in
//                     place;  T(s, i)  tiles from the last, mirror of D.
// Every solved unknown is also stored, the moment it is divided, into a
// scratch copy of x filled with a sentinel before the launch.  Tiles below
// it and product tasks poll that copy and use each value as soon as it
// appears, so a supernode's tiles hand off column by column and its
// products finish right behind its solve.  Contributions and transposed
// updates are counted on per-supernode counters that the tiles wait on.
// Tiles and products form two queues, each listed by supernode level with
// a supernode's tasks together and taken in list order through its own
// atomic counter: warp 0 of every block takes tiles, the other warps
// products, so the dependent chains of the tiles never share an SM
// sub-partition's FP64 pipe with product work.  A task waits only on tasks
// earlier in the common order (all waits bounded); the lowest unfinished
// task is therefore always held by a running warp or next in its queue,
// and no wait can deadlock.  Counters grow across
// solves (a solve's targets are multiples of its epoch), so nothing but the
// scratch copy is reset between solves.
#include <algorithm>
#include <climits>
#include <memory>
#include <vector>

#include "common.cuh"
#include "exec_common.cuh"

namespace gbsym {
struct SnTask {
  int kind;  // low byte: kind; bits 8.. : target count (forward products)
  int sup, a, b;
};
// One task queue: tasks in supernode blocks (block b: tb[b] .. tb[b+1]),
// and the value its counter reached after the solves so far.
struct SnQueue {
  DBuf<SnTask> task;
  DBuf<int> tb;
  int ntask = 0;
  unsigned long long ctr = 0;
};
}  // namespace gbsym

struct gbsym_sn_s {
  int n = 0, nsup = 0, nlev = 0, nblev = 0;
  int grid = 0;              // blocks of the persistent launch
  int groups = 0;            // right-hand-side groups the counters are laid out for
  unsigned long long ef = 0, et = 0;  // solves since the counters were cleared
  long long ncontrib = 0;
  size_t contrib_k = 0;
  std::vector<int> h_lev_ptr, h_blev_ptr;
  gbsym::DBuf<int> c0, nr, hf, need_in, n_ot;
  gbsym::DBuf<long long> rb, vb, coff;
  gbsym::DBuf<int> rows;
  gbsym::DBuf<double> vals;
  gbsym::DBuf<int> pull_ptr, pull_idx;
  gbsym::SnQueue q[4];  // forward tiles, forward products, transposed tiles, transposed products
  gbsym::DBuf<int> gt_tg;
  gbsym::DBuf<unsigned long long> flags;  // 4 queue counters + 2 x nsup x groups
  gbsym::DBuf<double> contrib, yscr;
  gbsym::DBuf<int> err;
};

namespace gbsym {
void fill_sentinel(void *y, size_t bytes, cudaStream_t s);  // exec_syncfree.cu

namespace {

constexpr int kSnWarps = 4;
// Right-hand sides per task.  Each right-hand side is its own pipeline of
// tasks; measured on the 64^3 nested-dissection factor, one per task beat
// 2, 4 and 8 per task at 8 and at 64 right-hand sides (9.2 / 66 ms against
// 11.3 / 71, 16.2 / 84 and 25.3 / 96 ms forward): fewer registers keep more
// warps resident and the independent pipelines overlap.
constexpr int kSnRhs = 1;
constexpr unsigned kFull = 0xffffffffu;
constexpr long long kSnWaitCycles = 1ll << 32;  // about two seconds
enum { kD = 0, kP = 1, kO = 2, kT = 3 };

struct SnView {
  int n, k, groups, nblk;
  int ntask[2];  // per role: tiles, products
  const int *c0, *nr, *hsplit, *need_in, *n_ot;
  const long long *rb, *vb, *coff;
  const int *rows;
  const double *vals;
  const int *pull_ptr, *pull_idx;
  const SnTask *task[2];
  const int *tb[2];
  const int *gt_tg;
  unsigned long long *ctr[2], *in;
  double *x, *contrib, *y;
  long long ncontrib;
  unsigned long long epoch, base[2];
  long long wait_cycles;  // bounded waits give up after this many SM cycles
  int *err;
};

// Exact arithmetic as fused multiply-adds (bit-identical to the separate
// operations, signed zeros included): RN(a*b) = fma(a, b, -0) and
// RN(s + p) = fma(p, 1, s).  Inline PTX is never executed speculatively,
// so guarded lanes and right-hand sides cost no FP64 issue.
__device__ __forceinline__ double xmul(double a, double b) {
  double r;
  asm("fma.rn.f64 %0, %1, %2, 0d8000000000000000;" : "=d"(r) : "d"(a), "d"(b));
  return r;
}
__device__ __forceinline__ double xadd(double s, double p) {
  double r;
  asm("fma.rn.f64 %0, %1, 0d3FF0000000000000, %2;" : "=d"(r) : "d"(p), "d"(s));
  return r;
}
__device__ __forceinline__ double xsub(double s, double p) {
  double r;
  asm("fma.rn.f64 %0, %1, 0dBFF0000000000000, %2;" : "=d"(r) : "d"(p), "d"(s));
  return r;
}
// RN(s + RN(a*b))
__device__ __forceinline__ double xmadd(double s, double a, double b) { return xadd(s, xmul(a, b)); }

__device__ __forceinline__ unsigned long long ld_acq64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_rel64(unsigned long long *p) {
  asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(p) : "memory");
}

// The scratch copy of x that tiles of a supernode poll: all ones until
// the value is stored (a NaN that no division produces).
__device__ __forceinline__ bool unsolved(double v) { return __double_as_longlong(v) == -1ll; }
__device__ __forceinline__ double ld_rlx_f64(const double *p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_rlx_f64(double *p, double v) {
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void cp_async8(double *dst, const double *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// a / b correctly rounded, given y = RN(1/b): Markstein's three FMAs
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990).  The theorem needs every
// intermediate normal: b's exponent in [3, 2043], a's in [63, 2043] and
// within 1000 of b's.  The lane precomputes the window of a's exponent that
// its b allows ([lo, hi]; empty as 4096, 4096 when b itself is out of
// range), so the check is one unsigned compare beside the FMAs; outside it,
// IEEE division, in a call (a branch the compiler cannot turn into
// predicated FP64 work, which this part would issue on every lane).
__device__ __noinline__ double ieee_div(double a, double b) { return __ddiv_rn(a, b); }
struct DivWindow {
  int lo, hi;
  __device__ explicit DivWindow(double b) {
    const int eb = (int)((__double_as_longlong(b) >> 52) & 0x7ff);
    const bool valid = eb >= 3 && eb <= 2043;
    lo = valid ? max(63, eb - 1000) : 4096;
    hi = valid ? min(2043, eb + 1000) : 4096;
  }
};
__device__ __forceinline__ double quotient(double a, double b, double y, const DivWindow &W) {
  double q;
  asm("fma.rn.f64 %0, %1, %2, 0d8000000000000000;" : "=d"(q) : "d"(a), "d"(y));
  const double r = __fma_rn(-q, b, a);
  double res = __fma_rn(r, y, q);
  const int ea = (int)((__double_as_longlong(a) >> 52) & 0x7ff);
  if ((unsigned)(ea - W.lo) > (unsigned)(W.hi - W.lo)) res = ieee_div(a, b);
  return res;
}

// Every lane waits (with its own acquire) until *f >= want.  Gives up after
// about two seconds, recording GBSYM_ERR_TIMEOUT, or at once when another
// wait has; the task then runs on, so every counter still reaches its
// target and the launch ends.
__device__ bool sn_wait(const unsigned long long *f, unsigned long long want, int *err, long long limit) {
  if (__all_sync(kFull, ld_acq64(f) >= want)) return true;
  const long long t0 = __shfl_sync(kFull, clock64(), 0);
  for (;;) {
    __nanosleep(40);
    if (__all_sync(kFull, ld_acq64(f) >= want)) return true;
    if (__any_sync(kFull, ld_relaxed(err) != 0)) return false;
    if (__shfl_sync(kFull, clock64() - t0 > limit, 0)) {
      if ((threadIdx.x & 31) == 0) atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
      return false;
    }
  }
}

__device__ __forceinline__ bool lane_zero() { return (threadIdx.x & 31) == 0; }

// After the warp's stores: make them visible before the task is counted.
__device__ __forceinline__ void sn_fence() {
  __threadfence();
  __syncwarp();
}

// Column (or row) runs of dmatvec_blas: w / 8 runs of 8, then at most one
// of 4, then single ones.
struct Runs {
  int n8, n4, nruns;
  __device__ explicit Runs(int w) {
    n8 = w >> 3;
    const int rem = w & 7;
    n4 = rem >= 4;
    nruns = n8 + n4 + (rem - 4 * n4);
  }
  __device__ void at(int r, int &start, int &size) const {
    if (r < n8) {
      start = r << 3;
      size = 8;
    } else if (n4 && r == n8) {
      start = n8 << 3;
      size = 4;
    } else {
      start = (n8 << 3) + 4 * n4 + (r - n8 - n4);
      size = 1;
    }
  }
};

// The grouped product sum of one row (forward: entries E[c*estride] and
// values xb[c], c = 0, 1, ...) or one column (transposed: entries E[p] and
// values xb[idx[p]] for storage positions p = len-1, len-2, ...), for kr
// right-hand sides xstride apart.  Lane (rho, h) computes the run sums of
// runs h, h + H, ...; the running value, which starts at +0, adds them in
// run order, taken from the H lanes of its row by shuffles.
//
// Values are read from the sentinel scratch copy as they are published:
// forward, the supernode's own unknowns appear in increasing order while
// its diagonal tiles run; transposed, the ancestors' unknowns appear top
// down, which is why the transposed runs start from the last off-block row.
// A run waits (bounded) until all its values are there, so the products
// finish right behind the solve instead of after it.
template <int KR, bool TR>
__device__ __forceinline__ void grouped_sum(int len, int H, int rho, int h, bool act, const double *__restrict__ E,
                                            size_t estride, const int *__restrict__ idx, const double *xb,
                                            size_t xstride, int kr, double (&acc)[KR], int *err, long long limit,
                                            bool &failed) {
  const Runs R(len);
#pragma unroll
  for (int j = 0; j < KR; ++j) acc[j] = 0.0;
  long long t0 = 0;
  for (int base = 0; base < R.nruns; base += H) {
    // one lane polls the step's last value in publication order (forward:
    // its highest column; transposed: its lowest row, the ancestors being
    // solved top down) before the warp loads the rest
    {
      int cl, szl;
      R.at(min(base + H, R.nruns) - 1, cl, szl);
      const int el = cl + szl - 1;
      const size_t xl = TR ? (size_t)__ldg(idx + (len - 1 - el)) : (size_t)el;
      int ns = 64;
      for (int j = 0; j < kr && !failed; ++j) {
        const double *pl = xb + (size_t)j * xstride + xl;
        while (!__shfl_sync(kFull, lane_zero() ? !unsolved(ld_rlx_f64(pl)) : false, 0)) {
          if (t0 == 0) t0 = __shfl_sync(kFull, clock64(), 0);
          __nanosleep(ns);
          ns = min(2 * ns, 1024);
          if (__any_sync(kFull, ld_relaxed(err) != 0)) failed = true;
          if (__shfl_sync(kFull, clock64() - t0 > limit, 0)) {
            if (lane_zero()) atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
            failed = true;
          }
          if (failed) break;
        }
      }
    }
    const int r = base + h;
    const bool has = act && r < R.nruns;
    int cs = 0, sz = 0;
    if (has) R.at(r, cs, sz);
    double m[8];
    size_t xo[8];
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int e = cs + b;
      const int p = TR ? len - 1 - e : e;
      m[b] = b < sz ? __ldg(E + (size_t)p * estride) : 0.0;
      xo[b] = b < sz ? (TR ? (size_t)__ldg(idx + p) : (size_t)p) : 0;
    }
    double s[KR];
#pragma unroll
    for (int j = 0; j < KR; ++j) {
      s[j] = 0.0;
      if (j < kr) {
        double xv[8];
        for (;;) {
          bool ok = true;
#pragma unroll
          for (int b = 0; b < 8; ++b) {
            xv[b] = 0.0;
            if (b < sz) {
              xv[b] = ld_rlx_f64(xb + (size_t)j * xstride + xo[b]);
              ok = ok && !unsolved(xv[b]);
            }
          }
          if (__all_sync(kFull, ok) || failed) break;
          if (t0 == 0) t0 = __shfl_sync(kFull, clock64(), 0);
          __nanosleep(100);
          if (__any_sync(kFull, ld_relaxed(err) != 0)) failed = true;
          if (__shfl_sync(kFull, clock64() - t0 > limit, 0)) {
            if ((threadIdx.x & 31) == 0) atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
            failed = true;
          }
        }
        if (has) {
          double a = xmul(xv[0], m[0]);
#pragma unroll
          for (int b = 1; b < 8; ++b)
            if (b < sz) a = xmadd(a, xv[b], m[b]);
          s[j] = a;
        }
      }
    }
    const int top = min(H, R.nruns - base);
    for (int hh = 0; hh < top; ++hh) {
#pragma unroll
      for (int j = 0; j < KR; ++j)
        if (j < kr) {
          const double sv = __shfl_sync(kFull, s[j], rho * H + hh);
          if (act) acc[j] = xadd(acc[j], sv);
        }
    }
  }
}

// Stages the 32 x 32 entries a tile of supernode rows/columns 32i..
// applies from tile J (own: J == i, only the strictly triangular part) into
// S[cc][lane], the entry lane uses at step cc; entries a lane does not use
// are zero.  Forward: row 32i + lane, column 32J + cc, read with lanes on
// consecutive rows.  Transposed: column 32i + lane, row 32J + c with
// c = cnt - 1 - cc, read down each column (lane = row c) for coalescing and
// written transposed.
__device__ __forceinline__ void stage_tile(double (*S)[32], const double *__restrict__ M, int ld, int w, int i, int J,
                                           int cnt, bool fwd, bool own, int lane) {
  if (fwd) {
    const int q = (i << 5) + lane;
#pragma unroll 4
    for (int cc = 0; cc < 32; ++cc) {
      const bool use = q < w && cc < cnt && (!own || lane > cc);
      if (use) cp_async8(&S[cc][lane], M + (size_t)((J << 5) + cc) * ld + q);
      else S[cc][lane] = 0.0;
    }
  } else {
    const int c = lane;  // the row this lane reads: 32J + c
#pragma unroll 4
    for (int qq = 0; qq < 32; ++qq) {
      const int col = (i << 5) + qq;
      if (c < cnt) {
        const bool use = col < w && (!own || qq < c);
        if (use) cp_async8(&S[cnt - 1 - c][qq], M + (size_t)col * ld + (J << 5) + c);
        else S[cnt - 1 - c][qq] = 0.0;
      }
    }
    for (int cc = cnt; cc < 32; ++cc) S[cc][lane] = 0.0;
  }
  cp_async_commit();
}

template <int KR>
__global__ void __launch_bounds__(kSnWarps * 32) k_sn(SnView V) {
  __shared__ double sm_own[32][32], sm_app[32][32];  // the tile warp's staging
  const int lane = threadIdx.x & 31;
  // Warp 0 of a block takes diagonal tiles, the others products: a
  // block's warps sit on different SM sub-partitions, so a tile's
  // dependent chain never shares its FP64 pipe with product work.
  const int role = (threadIdx.x >> 5) == 0 ? 0 : 1;
  const int *__restrict__ tb = V.tb[role];
  const unsigned long long total = (unsigned long long)V.ntask[role] * V.groups;
  for (;;) {
    unsigned long long u = 0;
    if (lane == 0) u = atomicAdd(V.ctr[role], 1ull) - V.base[role];
    u = __shfl_sync(kFull, u, 0);
    if (u >= total) break;
    // supernode block b holds groups x (tb[b+1] - tb[b]) task slots; the
    // last block with tb[b] * groups <= u is not empty
    int lo = 0, hi = V.nblk;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if ((unsigned long long)tb[mid] * V.groups <= u) lo = mid;
      else hi = mid;
    }
    const int nb = tb[lo + 1] - tb[lo];
    const unsigned long long off = u - (unsigned long long)tb[lo] * V.groups;
    const int g = (int)(off / nb);
    const SnTask T = V.task[role][tb[lo] + (int)(off % nb)];
    const int kind = T.kind & 0xff, t = T.sup;
    const int j0 = g * KR, kr = min(KR, V.k - j0);
    const int c0 = V.c0[t], w = V.c0[t + 1] - c0, ld = V.nr[t];
    const int nt = (w + 31) >> 5;
    const double *__restrict__ M = V.vals + V.vb[t];
    double *const xg = V.x + (size_t)j0 * V.n;
    const size_t fi = (size_t)t * V.groups + g;

    if (kind == kD || kind == kT) {
      const bool fwd = kind == kD;
      const int i = T.a;
      const int q = (i << 5) + lane;
      const bool act = q < w;
      const int cnt_own = min(32, w - (i << 5));
      double *const yg = V.y + (size_t)j0 * V.n;
      // this tile's own entries go to shared memory while the warp waits,
      // so[cc][lane] holding the entry lane uses at step cc.  Forward: row
      // q, column 32i + cc (lanes read consecutive rows).  Transposed:
      // column q, row 32i + c with c = cnt - 1 - cc; loaded down each column
      // (lane = row) so the reads stay coalesced, transposed on the way.
      double(*so)[32] = sm_own;
      stage_tile(so, M, ld, w, i, i, cnt_own, fwd, true, lane);
      double d = 1.0, y = 1.0;
      if (act) {
        d = __ldg(M + (size_t)q * ld + q);
        y = __drcp_rn(d);
      }
      sn_wait(V.in + fi, V.epoch * (unsigned long long)(fwd ? V.need_in[t] : V.n_ot[t]), V.err, V.wait_cycles);
      double v[KR];
#pragma unroll
      for (int j = 0; j < KR; ++j) v[j] = (act && j < kr) ? __ldcg(xg + (size_t)j * V.n + c0 + q) : 0.0;
      if (fwd && act) {
        // the sources' products, in increasing source order, 8 loads at a time
        const int p1 = V.pull_ptr[c0 + q + 1];
        for (int p = V.pull_ptr[c0 + q]; p < p1; p += 8) {
          size_t ci[8];
#pragma unroll
          for (int b = 0; b < 8; ++b) ci[b] = p + b < p1 ? (size_t)__ldg(V.pull_idx + p + b) : 0;
#pragma unroll
          for (int j = 0; j < KR; ++j)
            if (j < kr) {
              const double *cb = V.contrib + (size_t)(j0 + j) * V.ncontrib;
              double cv[8];
#pragma unroll
              for (int b = 0; b < 8; ++b) cv[b] = p + b < p1 ? __ldcg(cb + ci[b]) : 0.0;
#pragma unroll
              for (int b = 0; b < 8; ++b)
                if (p + b < p1) v[j] = xsub(v[j], cv[b]);
            }
        }
      }
      // earlier tiles (forward: 0..i-1; transposed: nt-1 down to i+1), each
      // column applied as soon as its value appears in the scratch copy
      const int steps = fwd ? i : nt - 1 - i;
      bool failed = false;
      for (int step = 0; step < steps; ++step) {
        const int J = fwd ? step : nt - 1 - step;
        const int cnt = min(32, w - (J << 5));
        double m[32];
        if (fwd) {
#pragma unroll
          for (int cc = 0; cc < 32; ++cc)
            m[cc] = (act && cc < cnt) ? __ldg(M + (size_t)((J << 5) + cc) * ld + q) : 0.0;
        } else {
          stage_tile(sm_app, M, ld, w, i, J, cnt, false, false, lane);
          cp_async_wait_all();
          __syncwarp();
#pragma unroll
          for (int cc = 0; cc < 32; ++cc) m[cc] = sm_app[cc][lane];
          __syncwarp();
        }
        const unsigned inside = cnt == 32 ? kFull : (1u << cnt) - 1u;
        int applied = 0;
        long long t0 = 0;
        while (applied < cnt) {
          double xl[KR];
          bool rdy = true;
#pragma unroll
          for (int j = 0; j < KR; ++j) {
            xl[j] = 0.0;
            if (j < kr && lane < cnt) {
              xl[j] = ld_rlx_f64(yg + (size_t)j * V.n + c0 + (J << 5) + lane);
              rdy = rdy && !unsolved(xl[j]);
            }
          }
          // columns ready in the order they are applied
          unsigned r = __ballot_sync(kFull, rdy) & inside;
          if (!fwd) r = __brev(r) >> (32 - cnt);
          const int pre = failed ? cnt : min(cnt, __ffs(~r) == 0 ? 32 : __ffs(~r) - 1);
#pragma unroll
          for (int cc = 0; cc < 32; ++cc) {
            if (cc >= applied && cc < pre) {
              const int c = fwd ? cc : cnt - 1 - cc;
#pragma unroll
              for (int j = 0; j < KR; ++j)
                if (j < kr) {
                  const double xc = __shfl_sync(kFull, xl[j], c);
                  if (act) v[j] = xsub(v[j], xmul(m[cc], xc));
                }
            }
          }
          if (pre == applied) {
            if (t0 == 0) t0 = __shfl_sync(kFull, clock64(), 0);
            __nanosleep(20);
            if (__any_sync(kFull, ld_relaxed(V.err) != 0)) failed = true;
            if (__shfl_sync(kFull, clock64() - t0 > V.wait_cycles, 0)) {
              if (lane == 0) atomicCAS(V.err, 0, GBSYM_ERR_TIMEOUT);
              failed = true;
            }
          }
          applied = pre;
        }
      }
      // this tile: lane c divides, the warp applies the quotient, and lane
      // c publishes it at once for the tiles that wait on it
      const DivWindow dw(d);
      cp_async_wait_all();
      __syncwarp();
#pragma unroll
      for (int cc = 0; cc < 32; ++cc) {
        if (cc < cnt_own) {
          const int c = fwd ? cc : cnt_own - 1 - cc;
          const bool upd = act && (fwd ? lane > c : lane < c);
          const double mc = so[cc][lane];
#pragma unroll
          for (int j = 0; j < KR; ++j)
            if (j < kr) {
              if (lane == c) v[j] = quotient(v[j], d, y, dw);
              const double xc = __shfl_sync(kFull, v[j], c);
              if (upd) v[j] = xsub(v[j], xmul(mc, xc));
              // (a NaN with the sentinel's bits would read as unsolved)
              if (lane == c)
                st_rlx_f64(yg + (size_t)j * V.n + c0 + q, unsolved(xc) ? __longlong_as_double(0x7ff8000000000000ll) : xc);
            }
        }
      }
      if (act) {
#pragma unroll
        for (int j = 0; j < KR; ++j)
          if (j < kr) xg[(size_t)j * V.n + c0 + q] = v[j];
      }
    } else {
      const int H = V.hsplit[t];
      const int rho = lane / H, h = lane % H;
      double acc[KR];
      bool failed = false;
      if (kind == kP) {
        // off-block rows w + a + rho: products with the supernode's solution
        const int o = T.a + rho;
        const bool act = o < ld - w;
        grouped_sum<KR, false>(w, H, rho, h, act, M + w + o, ld, nullptr, V.y + (size_t)j0 * V.n + c0, V.n, kr, acc,
                               V.err, V.wait_cycles, failed);
        if (act && h == 0) {
#pragma unroll
          for (int j = 0; j < KR; ++j)
            if (j < kr) V.contrib[(size_t)(j0 + j) * V.ncontrib + V.coff[t] + o] = acc[j];
        }
        sn_fence();
        if (lane == 0) {
          const int cnt = T.kind >> 8;
          for (int e = 0; e < cnt; ++e) red_rel64(V.in + (size_t)V.gt_tg[T.b + e] * V.groups + g);
        }
      } else {
        // columns a + rho: off-block products with the solved rows below
        const int col = T.a + rho;
        const bool act = col < w;
        grouped_sum<KR, true>(ld - w, H, rho, h, act, M + (size_t)col * ld + w, 1, V.rows + V.rb[t] + w,
                              V.y + (size_t)j0 * V.n, V.n, kr, acc, V.err, V.wait_cycles, failed);
        if (act && h == 0) {
#pragma unroll
          for (int j = 0; j < KR; ++j)
            if (j < kr) {
              double *xp = xg + (size_t)j * V.n + c0 + col;
              *xp = xsub(__ldcg(xp), acc[j]);
            }
        }
        sn_fence();
        if (lane == 0) red_rel64(V.in + fi);
      }
    }
  }
}

// Lanes per row for a product over len entries: enough that no lane sums
// more than 64 runs, at most 32.
int split_for(int len) {
  const int rem = len & 7, n4 = rem >= 4;
  const int nruns = len / 8 + n4 + (rem - 4 * n4);
  int H = 1;
  while (H < 32 && (nruns + H - 1) / H > 64) H *= 2;
  return H;
}

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

template <int KR>
int sn_grid() {
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sn<KR>, kSnWarps * 32, 0));
  return std::max(1, per_sm) * num_sms();
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
  std::vector<int> c0(nsup + 1), nr(nsup), col2sup(n);
  std::vector<long long> rb(nsup), vb(nsup), coff(nsup);
  size_t nvals = 0;
  long long ncontrib = 0;
  for (int q = 0; q < nsup; ++q) {
    const int a = sup2col[q], z = sup2col[q + 1];
    GB_CHECK(z > a, GBSYM_ERR_BAD_MATRIX);
    const size_t r0 = Li_ptr[a], r1 = Li_ptr[z];
    GB_CHECK(r1 >= r0 + (size_t)(z - a) && r1 - r0 < (size_t)1 << 30, GBSYM_ERR_BAD_MATRIX);
    c0[q] = a;
    nr[q] = (int)(r1 - r0);
    rb[q] = (long long)r0;
    vb[q] = (long long)Lp[a];
    coff[q] = ncontrib;
    ncontrib += nr[q] - (z - a);
    for (int j = 0; j < z - a; ++j) {
      GB_CHECK(Li[r0 + j] == a + j, GBSYM_ERR_BAD_MATRIX);  // the diagonal block's rows first
      col2sup[a + j] = q;
    }
    for (size_t k = r0 + (z - a); k < r1; ++k)  // off-block rows below the supernode, ascending
      GB_CHECK(Li[k] >= z && Li[k] < n && (k == r0 + (z - a) || Li[k] > Li[k - 1]), GBSYM_ERR_BAD_MATRIX);
    nvals = std::max(nvals, (size_t)Lp[a] + (r1 - r0) * (size_t)(z - a));
  }
  c0[nsup] = n;
  GB_CHECK(ncontrib < INT_MAX, GBSYM_ERR_UNSUPPORTED);
  t->ncontrib = ncontrib;
  const size_t nrows = Li_ptr[n];
  // pull lists (sources ascending) and both level schedules
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
  std::vector<int> pidx(std::max(cnt[n], 1));
  {
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int q = 0; q < nsup; ++q) {
      const int w = c0[q + 1] - c0[q];
      for (int k = w; k < nr[q]; ++k) pidx[fill[Li[rb[q] + k]]++] = (int)(coff[q] + (k - w));
    }
  }
  std::vector<int> lset, bset;
  levels_from(flev, nsup, t->h_lev_ptr, lset);
  levels_from(blev, nsup, t->h_blev_ptr, bset);
  t->nlev = (int)t->h_lev_ptr.size() - 1;
  t->nblev = (int)t->h_blev_ptr.size() - 1;
  // task lists, by supernode level.  Lanes per row (forward products) and
  // per column (transposed) live in one array, the transposed half second.
  std::vector<int> hs(2 * nsup), need_in(nsup, 0), n_ot(nsup, 0), gt_tg;
  for (int q = 0; q < nsup; ++q) {
    const int w = c0[q + 1] - c0[q];
    hs[q] = split_for(w);
    hs[nsup + q] = split_for(nr[q] - w);
  }
  std::vector<SnTask> L[4];  // forward tiles, forward products, transposed tiles, transposed products
  std::vector<int> tbs[4];
  for (int b = 0; b < nsup; ++b) {
    const int q = lset[b], w = c0[q + 1] - c0[q], nb = nr[q] - w, nt = (w + 31) / 32;
    tbs[0].push_back((int)L[0].size());
    tbs[1].push_back((int)L[1].size());
    for (int i = 0; i < nt; ++i) L[0].push_back({kD, q, i, 0});
    const int R = 32 / hs[q];
    for (int o = 0; o < nb; o += R) {
      const int start = (int)gt_tg.size();
      int prev = -1;
      for (int k = o; k < std::min(nb, o + R); ++k) {
        const int u = col2sup[Li[rb[q] + w + k]];
        if (u != prev) {
          gt_tg.push_back(u);
          need_in[u]++;
        }
        prev = u;
      }
      L[1].push_back({kP | (((int)gt_tg.size() - start) << 8), q, o, start});
    }
  }
  for (int b = 0; b < nsup; ++b) {
    const int q = bset[b], w = c0[q + 1] - c0[q], nb = nr[q] - w, nt = (w + 31) / 32;
    tbs[2].push_back((int)L[2].size());
    tbs[3].push_back((int)L[3].size());
    if (nb > 0) {
      const int R = 32 / hs[nsup + q];
      for (int a = 0; a < w; a += R, ++n_ot[q]) L[3].push_back({kO, q, a, 0});
    }
    for (int i = nt - 1; i >= 0; --i) L[2].push_back({kT, q, i, 0});
  }
  for (int l = 0; l < 4; ++l) {
    tbs[l].push_back((int)L[l].size());
    t->q[l].ntask = (int)L[l].size();
    if (L[l].empty()) L[l].push_back({kD, 0, 0, 0});  // never taken: the queue is empty
    upload(t->q[l].task, L[l].data(), L[l].size(), false, s);
    upload(t->q[l].tb, tbs[l].data(), tbs[l].size(), false, s);
  }
  upload(t->c0, c0.data(), c0.size(), false, s);
  upload(t->nr, nr.data(), nr.size(), false, s);
  upload(t->rb, rb.data(), rb.size(), false, s);
  upload(t->vb, vb.data(), vb.size(), false, s);
  upload(t->coff, coff.data(), coff.size(), false, s);
  upload(t->rows, Li, nrows, false, s);
  upload(t->vals, Lx, nvals, false, s);
  upload(t->pull_ptr, cnt.data(), cnt.size(), false, s);
  upload(t->pull_idx, pidx.data(), pidx.size(), false, s);
  upload(t->hf, hs.data(), hs.size(), false, s);
  upload(t->need_in, need_in.data(), need_in.size(), false, s);
  upload(t->n_ot, n_ot.data(), n_ot.size(), false, s);
  if (gt_tg.empty()) gt_tg.push_back(0);
  upload(t->gt_tg, gt_tg.data(), gt_tg.size(), false, s);
  t->err.alloc(2);
  GB_CUDA(cudaMemsetAsync(t->err.p, 0, 2 * sizeof(int), s));
  t->grid = sn_grid<kSnRhs>();
  GB_CUDA(cudaStreamSynchronize(s));
  return t.release();
}

// skew > 0 sets every counter target that many epochs ahead, so waits on
// counters cannot complete (the bounded-wait self-test).
void sn_launch(gbsym_sn_s *t, double *x, int k, bool transposed, cudaStream_t s, unsigned long long skew,
               long long wait_cycles) {
  if (t->n == 0 || k == 0) return;
  const int G = (k + kSnRhs - 1) / kSnRhs;
  const size_t per = (size_t)t->nsup * G;
  if (G != t->groups) {
    t->flags.alloc(4 + 2 * per);
    GB_CUDA(cudaMemsetAsync(t->flags.p, 0, t->flags.n * sizeof(unsigned long long), s));
    t->groups = G;
    t->ef = t->et = 0;
    for (auto &qq : t->q) qq.ctr = 0;
  }
  if (!transposed && t->ncontrib > 0 && t->contrib_k < (size_t)k) {
    t->contrib.alloc((size_t)t->ncontrib * k);
    t->contrib_k = k;
  }
  if (t->yscr.n < (size_t)t->n * k) t->yscr.alloc((size_t)t->n * k);
  fill_sentinel(t->yscr.p, (size_t)t->n * k * sizeof(double), s);
  const int grid = t->grid;
  SnView V{};
  V.n = t->n;
  V.k = k;
  V.groups = G;
  V.nblk = t->nsup;
  V.c0 = t->c0.p;
  V.nr = t->nr.p;
  V.hsplit = t->hf.p + (transposed ? t->nsup : 0);
  V.need_in = t->need_in.p;
  V.n_ot = t->n_ot.p;
  V.rb = t->rb.p;
  V.vb = t->vb.p;
  V.coff = t->coff.p;
  V.rows = t->rows.p;
  V.vals = t->vals.p;
  V.pull_ptr = t->pull_ptr.p;
  V.pull_idx = t->pull_idx.p;
  V.gt_tg = t->gt_tg.p;
  V.x = x;
  V.contrib = t->contrib.p;
  V.y = t->yscr.p;
  V.ncontrib = t->ncontrib;
  V.err = t->err.p;
  unsigned long long *f = t->flags.p;
  const int q0 = transposed ? 2 : 0;
  for (int role = 0; role < 2; ++role) {
    SnQueue &Q = t->q[q0 + role];
    V.ntask[role] = Q.ntask;
    V.task[role] = Q.task.p;
    V.tb[role] = Q.tb.p;
    V.ctr[role] = f + q0 + role;
    V.base[role] = Q.ctr;
    // every warp of the role takes one slot past the end
    Q.ctr += (unsigned long long)Q.ntask * G + (unsigned long long)grid * (role == 0 ? 1 : kSnWarps - 1);
  }
  V.in = f + 4 + (transposed ? per : 0);
  V.epoch = (transposed ? ++t->et : ++t->ef) + skew;
  V.wait_cycles = wait_cycles;
  k_sn<kSnRhs><<<grid, kSnWarps * 32, 0, s>>>(V);
  check_launch();
}

void sn_solve(gbsym_sn_s *t, double *x, int k, bool transposed, cudaStream_t s) {
  sn_launch(t, x, k, transposed, s, 0, kSnWaitCycles);
}

int sn_read_error(gbsym_sn_s *t, cudaStream_t s) {
  if (!t->err.p) return 0;
  int h[2] = {0, 0};
  GB_CUDA(cudaMemcpyAsync(h, t->err.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (h[0]) GB_CUDA(cudaMemsetAsync(t->err.p, 0, 2 * sizeof(int), s));
  return h[0];
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
  const int code = sn_read_error(t.get(), s);
  if (code) throw Err{code};
  GB_CUDA(cudaMemcpyAsync(x, dx.p, (size_t)n * k * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
}

// x[i] /= d[i] for every right-hand side (IEEE division, as
// parsy::scale_vec_vec, solve_phase.cpp:15-21).
__global__ void k_scale_div(double *__restrict__ x, const double *__restrict__ d, int n, int k) {
  const size_t m = (size_t)n * k;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x)
    x[i] = __ddiv_rn(x[i], d[i % n]);
}

// The LL^T (and LDL^T) solve phases: one plan, the forward solve, the
// diagonal scaling when d is given, the transposed solve.  A schedule is
// validated for both directions (the transposed solve walks it backward,
// as parsy::solve_phase_ll_blocked_parallel passes it to both,
// solve_phase.cpp:58-75).
void sn_dropin_phase(int n, const size_t *Lp, const int *Li, const double *Lx, const size_t *Li_ptr,
                     const int *sup2col, int supNo, const double *d, double *x, int k, int levels,
                     const int *level_ptr, const int *par_ptr, const int *partition) {
  GB_CHECK(k >= 0, GBSYM_ERR_SIZE);
  if (n == 0 || k == 0) return;
  GB_CHECK(x, GBSYM_ERR_NULL_ARG);
  cudaStream_t s = thread_stream();
  std::unique_ptr<gbsym_sn_s> t(sn_build(n, Lp, Li, Lx, Li_ptr, sup2col, supNo, s));
  if (par_ptr) {
    sn_validate_lbc(t.get(), Li_ptr, Li, sup2col, levels, level_ptr, par_ptr, partition, false);
    sn_validate_lbc(t.get(), Li_ptr, Li, sup2col, levels, level_ptr, par_ptr, partition, true);
  }
  DBuf<double> dx, dd;
  upload(dx, x, (size_t)n * k, false, s);
  sn_solve(t.get(), dx.p, k, false, s);
  if (d) {
    upload(dd, d, (size_t)n, false, s);
    const int grid = (int)std::min<size_t>(div_up((size_t)n * k, (size_t)256), (size_t)num_sms() * 8);
    k_scale_div<<<std::max(1, grid), 256, 0, s>>>(dx.p, dd.p, n, k);
    check_launch();
  }
  sn_solve(t.get(), dx.p, k, true, s);
  const int code = sn_read_error(t.get(), s);
  if (code) throw Err{code};
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
  gbsym::PhaseRange phase_("gbsym_sn_create");
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
  gbsym::PhaseRange phase_("gbsym_sn_solve");
  if (!t || (!x && t->n && k)) return GBSYM_ERR_NULL_ARG;
  if (k < 0) return GBSYM_ERR_SIZE;
  return guarded([&] { sn_solve(t, x, k, transposed != 0, (cudaStream_t)stream); });
}

int gbsym_sn_selftest_timeout(gbsym_sn t, long long limit_cycles, void *stream) {
  if (!t) return GBSYM_ERR_NULL_ARG;
  if (t->n == 0 || limit_cycles <= 0) return GBSYM_ERR_SIZE;
  int code = 0;
  const int st = guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    DBuf<double> x((size_t)t->n);
    GB_CUDA(cudaMemsetAsync(x.p, 0, (size_t)t->n * sizeof(double), s));
    sn_launch(t, x.p, 1, false, s, 1, limit_cycles);
    code = sn_read_error(t, s);
    // the counters no longer match any epoch: start them afresh
    if (t->flags.p) GB_CUDA(cudaMemsetAsync(t->flags.p, 0, t->flags.n * sizeof(unsigned long long), s));
    t->ef = t->et = 0;
    for (auto &qq : t->q) qq.ctr = 0;
    GB_CUDA(cudaStreamSynchronize(s));
  });
  return st != GBSYM_OK ? st : code;
}

int gbsym_sn_check(gbsym_sn t, void *stream) {
  if (!t) return GBSYM_ERR_NULL_ARG;
  int code = 0;
  const int st = guarded([&] { code = sn_read_error(t, (cudaStream_t)stream); });
  return st != GBSYM_OK ? st : code;
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

#define GBSYM_PHASE_ARGS                                                                                  \
  int *col2sup, int *sup2col, size_t *newCol, int *newRow, double *newVal, size_t *rowP, size_t nBlocks, int nnz

static int phase_n(size_t n, size_t nBlocks) {
  GB_CHECK(n <= (size_t)INT_MAX && nBlocks <= (size_t)INT_MAX, GBSYM_ERR_SIZE);
  return (int)n;
}

void gbsym_parsy_solve_phase_ll_blocked(size_t n, double *x, GBSYM_PHASE_ARGS) {
  (void)col2sup;
  (void)nnz;
  set_last_error(guarded([&] {
    sn_dropin_phase(phase_n(n, nBlocks), newCol, newRow, newVal, rowP, sup2col, (int)nBlocks, nullptr, x, 1, 0,
                    nullptr, nullptr, nullptr);
  }));
}

void gbsym_parsy_solve_phase_ll_blocked_nrhs(size_t n, double *x, int n_rhs, GBSYM_PHASE_ARGS, int max_col) {
  (void)col2sup;
  (void)nnz;
  (void)max_col;
  set_last_error(guarded([&] {
    sn_dropin_phase(phase_n(n, nBlocks), newCol, newRow, newVal, rowP, sup2col, (int)nBlocks, nullptr, x, n_rhs, 0,
                    nullptr, nullptr, nullptr);
  }));
}

void gbsym_parsy_solve_phase_ll_blocked_parallel(size_t n, double *x, GBSYM_PHASE_ARGS, int levels, int *levelPtr,
                                                 int *levelSet, int parts, int *parPtr, int *partition, int chunk) {
  (void)col2sup;
  (void)nnz;
  (void)levelSet;
  (void)parts;
  (void)chunk;
  set_last_error(guarded([&] {
    GB_CHECK(n == 0 || (levelPtr && parPtr && partition), GBSYM_ERR_NULL_ARG);
    sn_dropin_phase(phase_n(n, nBlocks), newCol, newRow, newVal, rowP, sup2col, (int)nBlocks, nullptr, x, 1, levels,
                    levelPtr, n ? parPtr : nullptr, partition);
  }));
}

void gbsym_parsy_solve_phase_ll_blocked_parallel_nrhs(size_t n, double *x, int n_rhs, GBSYM_PHASE_ARGS, int levels,
                                                      int *levelPtr, int *levelSet, int parts, int *parPtr,
                                                      int *partition, int chunk, int max_col) {
  (void)col2sup;
  (void)nnz;
  (void)levelSet;
  (void)parts;
  (void)chunk;
  (void)max_col;
  set_last_error(guarded([&] {
    GB_CHECK(n == 0 || (levelPtr && parPtr && partition), GBSYM_ERR_NULL_ARG);
    sn_dropin_phase(phase_n(n, nBlocks), newCol, newRow, newVal, rowP, sup2col, (int)nBlocks, nullptr, x, n_rhs,
                    levels, levelPtr, n ? parPtr : nullptr, partition);
  }));
}

void gbsym_parsy_solve_phase_ldl(size_t n, double *d_val, double *x, GBSYM_PHASE_ARGS) {
  (void)col2sup;
  (void)nnz;
  set_last_error(guarded([&] {
    GB_CHECK(n == 0 || d_val, GBSYM_ERR_NULL_ARG);
    sn_dropin_phase(phase_n(n, nBlocks), newCol, newRow, newVal, rowP, sup2col, (int)nBlocks, d_val, x, 1, 0,
                    nullptr, nullptr, nullptr);
  }));
}

}  // extern "C"
