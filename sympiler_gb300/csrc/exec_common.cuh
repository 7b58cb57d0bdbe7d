// exec_common.cuh -- device helpers shared by the triangular-solve
// executors (exec_level.cu, exec_sweep.cu, exec_syncfree.cu,
// exec_cluster.cu) and their
// host-side entry points (exec.cu).
#pragma once

#include <cuda_runtime.h>

#include "tri.cuh"

namespace gbsym {

// ---------------------------------------------------------------------------
// arithmetic policies.  EXACT: x -= v*x_j as a rounded product and a rounded
// difference (the reference's sequence); FUSED: one fused multiply-add per
// entry (one rounding; results differ from the reference by a few ulps).
enum { kArithExact = 0, kArithFused = 1 };

//
// The update is written as inline PTX on purpose: the slab loops guard each
// slot with "q < row length" inside a fully unrolled loop, and with plain
// arithmetic the compiler turns that guard into compute-everything-then-
// select, executing the update for all kSlabMax slots of every row.  On a
// part whose FP64 rate is this low that doubled the FP64 work of a sweep
// (measured: 8 multiplies and 8 subtractions per row on a three-entry
// triangle).  An asm statement is never executed speculatively, so the
// guard stays a branch and only real entries are computed.
//
// In FP64 both roundings of the exact update are issued as fused
// multiply-adds with a constant operand; this part runs them at the rate of
// separate multiplies and subtractions (503 G thread-op/s for either form
// over all SMs, against 597 for general three-operand FMAs: two DFMAs per SM
// per clock at most).  Both forms are bit-identical to the separate
// operations for every input, signed zeros included:  RN(v*x) = fma(v, x, -0)  (adding -0 changes neither a nonzero
// product nor the sign of a zero one) and  RN(acc - p) = fma(p, -1, acc)
// (p * -1 is exact, so one rounding of acc - p remains).
template <int AR, class T>
__device__ __forceinline__ T msub(T acc, T v, T xj) {
  T r;
  if constexpr (sizeof(T) == 8) {
    if constexpr (AR == kArithExact)
      asm("{\n\t.reg .f64 p;\n\tfma.rn.f64 p, %1, %2, 0d8000000000000000;\n\t"
          "fma.rn.f64 %0, p, 0dBFF0000000000000, %3;\n\t}"
          : "=d"(r) : "d"(v), "d"(xj), "d"(acc));
    else
      asm("{\n\t.reg .f64 nv;\n\tneg.f64 nv, %1;\n\tfma.rn.f64 %0, nv, %2, %3;\n\t}"
          : "=d"(r) : "d"(v), "d"(xj), "d"(acc));
  } else {
    if constexpr (AR == kArithExact)
      asm("{\n\t.reg .f32 p;\n\tmul.rn.f32 p, %1, %2;\n\tsub.rn.f32 %0, %3, p;\n\t}"
          : "=f"(r) : "f"(v), "f"(xj), "f"(acc));
    else
      asm("{\n\t.reg .f32 nv;\n\tneg.f32 nv, %1;\n\tfma.rn.f32 %0, nv, %2, %3;\n\t}"
          : "=f"(r) : "f"(v), "f"(xj), "f"(acc));
  }
  return r;
}

// Correctly rounded a / b given y = RN(1/b).  Markstein's method (P.
// Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990): for a faithful
// quotient q = RN(a*y), the remainder a - q*b is exact under one fused
// multiply-add and q + (a - q*b)*y rounds to a/b.  The theorem needs every
// intermediate normal, so operands whose exponents could under- or
// overflow the remainder or the quotient (and zeros, infinities, NaNs) take
// IEEE division instead.  Three dependent FP64 operations replace a
// division that costs about seven FMAs of issue and 280 ns of latency on
// this part.  The IEEE division is a call out of line: inlined, its code
// lengthened the common path by about 100 cycles even when not taken (one
// warp, a dependent chain of divisions: 360 cycles each inlined, 284 out of
// line, 256 with no range test at all).
static __device__ __noinline__ double div_ieee(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double div_by(double a, double b, double y) {
  // biased exponents from the high words; the same ranges as
  // 63 <= ea <= 2043, 3 <= eb <= 2043, |ea - eb| <= 1000
  const int ea = (__double2hiint(a) >> 20) & 0x7ff, eb = (__double2hiint(b) >> 20) & 0x7ff;
  const bool ok = (unsigned)(ea - 63) <= 1980u && (unsigned)(eb - 3) <= 2040u &&
                  (unsigned)(ea - eb + 1000) <= 2000u;
  if (__builtin_expect(!ok, 0)) return div_ieee(a, b);
  double q;  // RN(a*y), issued as an FMA (asm: the compiler would fold it back into a multiply)
  asm("fma.rn.f64 %0, %1, %2, 0d8000000000000000;" : "=d"(q) : "d"(a), "d"(y));
  const double r = __fma_rn(-q, b, a);
  return __fma_rn(r, y, q);
}
__device__ __forceinline__ float div_by(float a, float b, float /*y*/) { return __fdiv_rn(a, b); }

__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// L2-coherent loads for values other blocks write while a launch runs.
__device__ __forceinline__ double ldx(const double *p) { return __ldcg(p); }
__device__ __forceinline__ float ldx(const float *p) { return __ldcg(p); }
template <class T, bool CG>
__device__ __forceinline__ T ldv(const T *p) {
  return CG ? ldx(p) : *p;
}

// ---------------------------------------------------------------------------
// Static part of a row: everything that does not depend on x.  All loads
// are independent of each other (slab entries are addressed by the packed
// row index alone), so they are in flight together.
// S is the slab capacity the registers hold; it must be at least A.K.  A
// kernel compiled for a narrow slab (S = 4 covers every stencil factor up
// to three off-diagonals per row) keeps far fewer registers live.
template <class T, int S = kSlabMax>
struct RowStatic {
  int orig, len, ovb;
  T d, y;
  int c[S];
  T v[S];
};

template <class T, int S>
__device__ __forceinline__ void load_row(const TriView<T> &A, int row, RowStatic<T, S> &r) {
  r.orig = A.perm[row];
  r.len = A.len[row];
  r.d = A.dg ? A.dg[row] : T(1);
  r.y = A.dg ? A.rc[row] : T(1);
  r.ovb = A.ovp ? A.ovp[row] : 0;
#pragma unroll
  for (int q = 0; q < S; ++q)
    if (q < A.K) {
      r.c[q] = A.sci[(size_t)q * A.npad + row];
      r.v[q] = A.sv[(size_t)q * A.npad + row];
    }
}

// acc - sum_q v_q x[c_q] in storage order; the slab gathers are issued
// together before the first subtraction.
template <class T, bool CG, int AR>
__device__ __forceinline__ T row_accumulate(const TriView<T> &A, const RowStatic<T> &r, const T *x,
                                            T acc) {
  T xv[kSlabMax];
#pragma unroll
  for (int q = 0; q < kSlabMax; ++q)
    if (q < A.K && q < r.len) xv[q] = ldv<T, CG>(x + r.c[q]);
#pragma unroll
  for (int q = 0; q < kSlabMax; ++q)
    if (q < A.K && q < r.len) acc = msub<AR>(acc, r.v[q], xv[q]);
  for (int t = A.K; t < r.len; ++t) {
    const int e = r.ovb + t - A.K;
    acc = msub<AR>(acc, A.ov[e], ldv<T, CG>(x + A.oci[e]));
  }
  return acc;
}

template <class T, int S>
__device__ __forceinline__ T row_finish(const TriView<T> &A, const RowStatic<T, S> &r, T acc) {
  return A.dg ? div_by(acc, r.d, r.y) : acc;
}

template <class T, int VEC> struct VecT;
template <> struct VecT<double, 1> { using t = double; };
template <> struct VecT<double, 2> { using t = double2; };
template <> struct VecT<float, 1> { using t = float; };
template <> struct VecT<float, 2> { using t = float2; };
template <> struct VecT<float, 4> { using t = float4; };

template <class T, int VEC, bool CG>
__device__ __forceinline__ void vload(const T *p, T (&v)[VEC]) {
  using V = typename VecT<T, VEC>::t;
  const V t = CG ? __ldcg(reinterpret_cast<const V *>(p)) : *reinterpret_cast<const V *>(p);
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

// k right-hand sides of one row, row-major x[i*k + r]: this lane's VEC-wide
// slices r = lane*VEC, lane*VEC + G*VEC, ...; all slab gathers of a slice
// are issued before the in-order accumulation.
template <class T, int G, int VEC, bool CG, int AR>
__device__ __forceinline__ void row_mrhs(const TriView<T> &A, const RowStatic<T> &rs, T *x, int k,
                                         int lane) {
  const size_t orig = (size_t)rs.orig;
  for (int r = lane * VEC; r < k; r += G * VEC) {
    T acc[VEC];
    vload<T, VEC, CG>(x + orig * k + r, acc);
    T xv[kSlabMax][VEC];
#pragma unroll
    for (int q = 0; q < kSlabMax; ++q)
      if (q < A.K && q < rs.len) vload<T, VEC, CG>(x + (size_t)rs.c[q] * k + r, xv[q]);
#pragma unroll
    for (int q = 0; q < kSlabMax; ++q)
      if (q < A.K && q < rs.len) {
#pragma unroll
        for (int u = 0; u < VEC; ++u) acc[u] = msub<AR>(acc[u], rs.v[q], xv[q][u]);
      }
    for (int t = A.K; t < rs.len; ++t) {
      const int e = rs.ovb + t - A.K;
      const T v = A.ov[e];
      T y[VEC];
      vload<T, VEC, CG>(x + (size_t)A.oci[e] * k + r, y);
#pragma unroll
      for (int u = 0; u < VEC; ++u) acc[u] = msub<AR>(acc[u], v, y[u]);
    }
#pragma unroll
    for (int u = 0; u < VEC; ++u) acc[u] = row_finish(A, rs, acc[u]);
    vstore<T, VEC>(x + orig * k + r, acc);
  }
}

// lanes per row: enough to cover k with 2-wide (FP64) / 4-wide (FP32) loads
inline int lanes_for(int k, int dsize) {
  const int per = dsize == 8 ? 2 : 4;
  const int need = div_up(k, per);
  int g = 2;
  while (g < need && g < 32) g <<= 1;
  return g;
}

template <class T>
inline TriView<T> view_of(const gbsym_tri_s *t);
template <>
inline TriView<double> view_of<double>(const gbsym_tri_s *t) { return t->view64(); }
template <>
inline TriView<float> view_of<float>(const gbsym_tri_s *t) { return t->view32(); }
template <class T>
inline TriView<T> view_packed_of(const gbsym_tri_s *t);
template <>
inline TriView<double> view_packed_of<double>(const gbsym_tri_s *t) { return t->view64_packed(); }
template <>
inline TriView<float> view_packed_of<float>(const gbsym_tri_s *t) { return t->view32_packed(); }

// Host entry points of the executors (one translation unit each).
template <class T>
void run_levelset(gbsym_tri_s *t, T *x, const T *b, int k, int dtype, cudaStream_t s);
template <class T>
void run_persist(gbsym_tri_s *t, T *x, int k, cudaStream_t s);
template <class T>
void run_oneblock(gbsym_tri_s *t, T *x, cudaStream_t s);
// b non-null: out of place, x = L^-1 b with b left unchanged; the solution
// is published straight into x (sentinel-filled first) instead of into the
// plan's scratch copy.
template <class T>
void run_syncfree(gbsym_tri_s *t, T *x, int k, cudaStream_t s, const T *b);
template <class T>
void run_part(gbsym_tri_s *t, T *x, cudaStream_t s);
template <class T>
void run_cluster(gbsym_tri_s *t, T *x, int k, cudaStream_t s);

}  // namespace gbsym
