// adjoint.cu -- reverse mode of X = L^{-1} B.
//
// With G = dloss/dX, the cotangent of B is G_B = L^{-T} G: the transposed
// (backward) solve, run by the same level-packed executor on the plan of
// L^T (the CSC of L read as an upper CSR with the diagonal first, the
// layout of ltsolve, sparse_blas/sptrsv_lt.cpp:11-20).  The cotangent of a
// stored entry L_ij is -sum_r G_B[i,r] X[j,r] (dX = -L^{-1} dL X), formed
// only on L's sparsity pattern, so memory stays O(nnz + n k): X is kept
// from the forward solve and nothing is recomputed.
#include <cstdint>

#include "common.cuh"
#include "tri.cuh"

namespace gbsym {

// Any k: one thread per row i of L (CSR, diagonal last), each stored
// entry's k-term product in four interleaved partial sums.  Lanes across rows keep
// every FP64 instruction full: a lane-per-right-hand-side layout needs a
// five-step shuffle reduction per entry, six warp FP64 instructions for
// one instruction's worth of products, and this part's FP64 issue rate is
// the bound.  G_B's row is re-read from L1 for each entry.
__global__ void __launch_bounds__(256)
k_value_grad(int n, const int *__restrict__ Lp, const int *__restrict__ Li,
             const double *__restrict__ X, const double *__restrict__ GB, int k,
             double *__restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *gi = GB + (size_t)i * k;
  for (int e = Lp[i]; e < Lp[i + 1]; ++e) {
    const double *xj = X + (size_t)Li[e] * k;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int r = 0;
    for (; r + 4 <= k; r += 4) {
      s0 = __fma_rn(__ldg(gi + r), __ldg(xj + r), s0);
      s1 = __fma_rn(__ldg(gi + r + 1), __ldg(xj + r + 1), s1);
      s2 = __fma_rn(__ldg(gi + r + 2), __ldg(xj + r + 2), s2);
      s3 = __fma_rn(__ldg(gi + r + 3), __ldg(xj + r + 3), s3);
    }
    for (; r < k; ++r) s0 = __fma_rn(__ldg(gi + r), __ldg(xj + r), s0);
    grad[e] = -((s0 + s1) + (s2 + s3));
  }
}

// Four lanes per row for k a multiple of 8 (up to 64): lane q keeps the
// row's G_B values 2q, 2q+1, 2q+8, 2q+9, ... in registers, and for each
// entry reads the same positions of X's row j as 16-byte vectors, so the
// row's four lanes read 64 contiguous bytes per step and every load
// instruction is coalesced (one thread per row leaves its lanes a row
// apart, 32 sectors per load).  The partial sums meet in two shuffle steps
// among the row's four lanes, which run the same entries in lock step.
template <int K>
__global__ void __launch_bounds__(256)
k_value_grad4(int n, const int *__restrict__ Lp, const int *__restrict__ Li, const double *__restrict__ X,
              const double *__restrict__ GB, double *__restrict__ grad) {
  static_assert(K % 8 == 0 && K <= 64, "four lanes of two-value slices");
  constexpr int S = K / 8;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= 4LL * n) return;  // whole rows only: the grid is a multiple of 4 lanes
  const int i = (int)(t >> 2), q = (int)(t & 3);
  const unsigned grp = 0xfu << (threadIdx.x & 28);
  double2 g[S];
#pragma unroll
  for (int c = 0; c < S; ++c) g[c] = __ldg(reinterpret_cast<const double2 *>(GB + (size_t)i * K + 2 * q + 8 * c));
  const int e1 = Lp[i + 1];
  for (int e = Lp[i]; e < e1; ++e) {
    const double *xj = X + (size_t)Li[e] * K + 2 * q;
    double a0 = 0.0, a1 = 0.0;
#pragma unroll
    for (int c = 0; c < S; ++c) {
      const double2 v = __ldg(reinterpret_cast<const double2 *>(xj + 8 * c));
      a0 = __fma_rn(g[c].x, v.x, a0);
      a1 = __fma_rn(g[c].y, v.y, a1);
    }
    double sum = a0 + a1;
    sum += __shfl_xor_sync(grp, sum, 1);
    sum += __shfl_xor_sync(grp, sum, 2);
    if (q == 0) grad[e] = -sum;
  }
}

template <int K>
static void launch_grad4(int n, const int *Lp, const int *Li, const double *X, const double *g, double *grad,
                         cudaStream_t s) {
  k_value_grad4<K><<<div_up(4LL * n, 256), 256, 0, s>>>(n, Lp, Li, X, g, grad);
}

void tri_adjoint(gbsym_tri_s *Lt, int n, const int *Lp, const int *Li, const double *X, double *g,
                 int k, double *grad, cudaStream_t s) {
  GB_CHECK(Lt->n == n && k >= 1, GBSYM_ERR_SIZE);
  GB_CHECK(kind_is_upper(Lt->kind), GBSYM_ERR_UNSUPPORTED);
  if (n == 0) return;
  tri_solve_rowmajor(Lt, g, nullptr, k, GBSYM_F64, s);
  const bool vec = ((uintptr_t)X % 16 == 0) && ((uintptr_t)g % 16 == 0);
  if (vec && k == 8) launch_grad4<8>(n, Lp, Li, X, g, grad, s);
  else if (vec && k == 16) launch_grad4<16>(n, Lp, Li, X, g, grad, s);
  else if (vec && k == 32) launch_grad4<32>(n, Lp, Li, X, g, grad, s);
  else if (vec && k == 64) launch_grad4<64>(n, Lp, Li, X, g, grad, s);
  else k_value_grad<<<div_up(n, 256), 256, 0, s>>>(n, Lp, Li, X, g, k, grad);
  check_launch();
}

}  // namespace gbsym

using namespace gbsym;

extern "C" int gbsym_tri_adjoint(gbsym_tri Lt, int n, const int *Lp, const int *Li, const double *X,
                                 double *g, int k, double *grad, void *stream) {
  gbsym::PhaseRange phase_("gbsym_tri_adjoint");
  if (!Lt || (n && (!Lp || !Li || !X || !g || !grad))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    tri_adjoint(Lt, n, Lp, Li, X, g, k, grad, (cudaStream_t)stream);
  });
}
