// exec_syncfree.cu -- SYNCFREE executor, host side: the warp units, the
// sentinel fill of the scratch copy and the choice of the kernel compiled
// for the plan's slab width.  The sweep itself is described and defined in
// exec_syncfree_kernel.cuh.
#include <algorithm>
#include <cstdlib>
#include <vector>

#include "exec_syncfree.cuh"

namespace gbsym {

Units sf_units(gbsym_tri_s *t, int rpw) {
  for (auto &e : t->sf_units)
    if (e.rpw == rpw) return {e.row.p, e.cnt.p, e.n};
  std::vector<int> row, cnt;
  for (int l = 0; l < t->nlev; ++l)
    for (int a = t->h_lev_ptr[l]; a < t->h_lev_ptr[l + 1]; a += rpw) {
      row.push_back(a);
      cnt.push_back(std::min(rpw, t->h_lev_ptr[l + 1] - a));
    }
  gbsym_tri_s::SfUnits e;
  e.rpw = rpw;
  e.n = (int)row.size();
  e.row.alloc(row.size());
  e.cnt.alloc(cnt.size());
  GB_CUDA(cudaMemcpy(e.row.p, row.data(), row.size() * sizeof(int), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(e.cnt.p, cnt.data(), cnt.size() * sizeof(int), cudaMemcpyHostToDevice));
  t->sf_units.push_back(std::move(e));
  const auto &b = t->sf_units.back();
  return {b.row.p, b.cnt.p, b.n};
}

// Every published slot starts as the sentinel (all bits set): 16-byte
// stores over the 16-byte multiple, 4-byte stores over the remainder.
__global__ void k_fill_sentinel(uint4 *__restrict__ p, size_t n16, unsigned *__restrict__ tail, int ntail) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += stride)
    p[i] = make_uint4(~0u, ~0u, ~0u, ~0u);
  if (blockIdx.x == 0 && (int)threadIdx.x < ntail) tail[threadIdx.x] = ~0u;
}

void fill_sentinel(void *y, size_t bytes, cudaStream_t s) {
  const size_t n16 = bytes / 16;
  const int ntail = (int)((bytes - n16 * 16) / 4);
  const int grid = (int)std::max<size_t>(1, std::min<size_t>(div_up(n16, (size_t)256), (size_t)num_sms() * 8));
  k_fill_sentinel<<<grid, 256, 0, s>>>(reinterpret_cast<uint4 *>(y), n16,
                                       reinterpret_cast<unsigned *>(static_cast<char *>(y) + n16 * 16), ntail);
  check_launch();
}

template <class T>
void run_syncfree(gbsym_tri_s *t, T *x, int k, cudaStream_t s, const T *b) {
  if (k == 1 && !b && t->sf_lookthrough && sf_lookthrough_ok(t)) {
    run_syncfree_lt<T>(t, x, s);
    return;
  }
  if (k > 1 && !b && t->sf_lt_mrhs && sf_lookthrough_ok(t)) {
    run_syncfree_lt_mrhs<T>(t, x, k, s);
    return;
  }
  const size_t bytes = (size_t)t->n * k * sizeof(T);
  T *y = x;
  if (!b) {
    t->sfy.reserve(bytes);
    y = reinterpret_cast<T *>(t->sfy.p);
  }
  fill_sentinel(y, bytes, s);
  const bool ov = t->nov > 0;
  switch (t->K) {
    case 0:
    case 1:
    case 2: ov ? sf_run_ks<T, 2, true>(t, x, y, b, k, s) : sf_run_ks<T, 2, false>(t, x, y, b, k, s); break;
    case 3: ov ? sf_run_ks<T, 3, true>(t, x, y, b, k, s) : sf_run_ks<T, 3, false>(t, x, y, b, k, s); break;
    case 4: ov ? sf_run_ks<T, 4, true>(t, x, y, b, k, s) : sf_run_ks<T, 4, false>(t, x, y, b, k, s); break;
    default:
      ov ? sf_run_ks<T, kSlabMax, true>(t, x, y, b, k, s) : sf_run_ks<T, kSlabMax, false>(t, x, y, b, k, s);
      break;
  }
}

template void run_syncfree<double>(gbsym_tri_s *, double *, int, cudaStream_t, const double *);
template void run_syncfree<float>(gbsym_tri_s *, float *, int, cudaStream_t, const float *);

}  // namespace gbsym
