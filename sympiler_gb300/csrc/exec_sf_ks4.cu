// exec_sf_ks4.cu -- the sync-free sweep's kernels compiled for a four-entry
// slab (plans with t->K == 4) whose rows all fit in the slab.
#include "exec_syncfree_kernel.cuh"

namespace gbsym {

template void sf_run_ks<double, 4, false>(gbsym_tri_s *, double *, double *, const double *, int, cudaStream_t);
template void sf_run_ks<float, 4, false>(gbsym_tri_s *, float *, float *, const float *, int, cudaStream_t);

}  // namespace gbsym
