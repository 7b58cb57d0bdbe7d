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

// One warp per row i of L (CSR, diagonal last).  Lanes hold G_B[i, :] and
// reduce the k-term products of each stored entry.
__global__ void __launch_bounds__(256)
k_value_grad(int n, const int *__restrict__ Lp, const int *__restrict__ Li,
             const double *__restrict__ X, const double *__restrict__ GB, int k,
             double *__restrict__ grad) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n) return;
  const double *gi = GB + (size_t)i * k;
  for (int e = Lp[i]; e < Lp[i + 1]; ++e) {
    const double *xj = X + (size_t)Li[e] * k;
    double s = 0.0;
    for (int r = lane; r < k; r += 32) s += gi[r] * xj[r];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) grad[e] = -s;
  }
}

void tri_adjoint(gbsym_tri_s *Lt, int n, const int *Lp, const int *Li, const double *X, double *g,
                 int k, double *grad, cudaStream_t s) {
  GB_CHECK(Lt->n == n && k >= 1, GBSYM_ERR_SIZE);
  GB_CHECK(kind_is_upper(Lt->kind), GBSYM_ERR_UNSUPPORTED);
  if (n == 0) return;
  tri_solve_rowmajor(Lt, g, nullptr, k, GBSYM_F64, s);
  k_value_grad<<<div_up(n, 8), 256, 0, s>>>(n, Lp, Li, X, g, k, grad);
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
