// adjoint.cu -- reverse mode of X = L^{-1} B.
//
// With G = dloss/dX, the cotangent of B is G_B = L^{-T} G: the transposed
// (backward) solve, run by the same level-packed executor on the plan of
// L^T (the CSC of L read as an upper CSR with the diagonal first, the
// layout of ltsolve, sparse_blas/sptrsv_lt.cpp:11-20).  The cotangent of a
// stored entry L_ij is -sum_r G_B[i,r] X[j,r] (dX = -L^{-1} dL X), formed
// only on L's sparsity pattern, so memory stays O(nnz + n k): X is kept
// from the forward solve and nothing is recomputed.
#include "common.cuh"
#include "tri.cuh"

namespace gbsym {

// One thread per row i of L (CSR, diagonal last), each stored entry's
// k-term product in four interleaved partial sums.  Lanes across rows keep
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

void tri_adjoint(gbsym_tri_s *Lt, int n, const int *Lp, const int *Li, const double *X, double *g,
                 int k, double *grad, cudaStream_t s) {
  GB_CHECK(Lt->n == n && k >= 1, GBSYM_ERR_SIZE);
  GB_CHECK(kind_is_upper(Lt->kind), GBSYM_ERR_UNSUPPORTED);
  if (n == 0) return;
  tri_solve_rowmajor(Lt, g, nullptr, k, GBSYM_F64, s);
  k_value_grad<<<div_up(n, 256), 256, 0, s>>>(n, Lp, Li, X, g, k, grad);
  check_launch();
}

}  // namespace gbsym

using namespace gbsym;

extern "C" int gbsym_tri_adjoint(gbsym_tri Lt, int n, const int *Lp, const int *Li, const double *X,
                                 double *g, int k, double *grad, void *stream) {
  if (!Lt || (n && (!Lp || !Li || !X || !g || !grad))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    tri_adjoint(Lt, n, Lp, Li, X, g, k, grad, (cudaStream_t)stream);
  });
}
