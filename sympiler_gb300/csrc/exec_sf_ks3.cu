// exec_sf_ks3.cu -- the sync-free sweep's kernels compiled for a three-entry
// slab (plans with t->K == 3) whose rows all fit in the slab.
#include "exec_syncfree_kernel.cuh"

namespace gbsym {

template void sf_run_ks<double, 3, false>(gbsym_tri_s *, double *, double *, const double *, int, cudaStream_t);
template void sf_run_ks<float, 3, false>(gbsym_tri_s *, float *, float *, const float *, int, cudaStream_t);

}  // namespace gbsym
