// exec_sf_ks3_ov.cu -- the sync-free sweep's kernels compiled for a three-
// entry slab (plans with t->K == 3) with rows longer than the slab (their
// extra entries are polled and accumulated in groups).
#include "exec_syncfree_kernel.cuh"

namespace gbsym {

template void sf_run_ks<double, 3, true>(gbsym_tri_s *, double *, double *, const double *, int, cudaStream_t);
template void sf_run_ks<float, 3, true>(gbsym_tri_s *, float *, float *, const float *, int, cudaStream_t);

}  // namespace gbsym
