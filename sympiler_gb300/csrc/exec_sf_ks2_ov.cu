// exec_sf_ks2_ov.cu -- the sync-free sweep's kernels compiled for a two-
// entry slab (plans with t->K <= 2) with rows longer than the slab (their
// extra entries are polled and accumulated in groups).
#include "exec_syncfree_kernel.cuh"

namespace gbsym {

template void sf_run_ks<double, 2, true>(gbsym_tri_s *, double *, double *, const double *, int, cudaStream_t);
template void sf_run_ks<float, 2, true>(gbsym_tri_s *, float *, float *, const float *, int, cudaStream_t);

}  // namespace gbsym
