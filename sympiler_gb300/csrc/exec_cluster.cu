// exec_cluster.cu -- CLUSTER executor: thread-block clusters sweep the
// wavefront levels, separated by hardware cluster barriers.
//
// On this part a cluster barrier costs about a quarter of a microsecond for
// up to 16 blocks, well under a kernel boundary or a software grid barrier,
// and it cannot hang: every block of a cluster executes the same number of
// barriers.  Levels are therefore swept inside one cluster: the rows of a
// level are spread over the cluster's threads, each thread arrives at the
// barrier (release) right after its stores, loads the static part of its
// next row while the others finish, then waits (acquire) and gathers x
// through L2.
//
// Right-hand sides are independent, so with k > 1 the columns are split
// into equal slices and each cluster sweeps all levels for its own slice --
// as many clusters as are co-resident, which puts the whole GPU's FP64
// pipes to work on a solve whose levels are individually too small to.
#include <cooperative_groups.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "exec_common.cuh"

namespace cg = cooperative_groups;

namespace gbsym {

constexpr int kClusterThreads = 512;

__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// One row, columns [0, kw) of a window whose row stride is k (x points at
// the window's first column).
template <class T, int G, int VEC, int AR>
__device__ __forceinline__ void row_window(const TriView<T> &A, const RowStatic<T> &rs, T *x, int k,
                                           int kw, int lane) {
  const size_t orig = (size_t)rs.orig;
  for (int r = lane * VEC; r < kw; r += G * VEC) {
    T acc[VEC];
    vload<T, VEC, true>(x + orig * k + r, acc);
    T xv[kSlabMax][VEC];
#pragma unroll
    for (int q = 0; q < kSlabMax; ++q)
      if (q < A.K && q < rs.len) vload<T, VEC, true>(x + (size_t)rs.c[q] * k + r, xv[q]);
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
      vload<T, VEC, true>(x + (size_t)A.oci[e] * k + r, y);
#pragma unroll
      for (int u = 0; u < VEC; ++u) acc[u] = msub<AR>(acc[u], v, y[u]);
    }
#pragma unroll
    for (int u = 0; u < VEC; ++u) acc[u] = row_finish(A, rs, acc[u]);
    vstore<T, VEC>(x + orig * k + r, acc);
  }
}

// G lanes per row, VEC columns per lane step; cluster q sweeps the column
// slice [q*kc, min(k, (q+1)*kc)).
template <class T, int G, int VEC, int AR>
__global__ void __launch_bounds__(kClusterThreads)
k_cluster_sweep(TriView<T> A, T *__restrict__ x, int k, int kc, const int *__restrict__ lev_ptr,
                int nlev) {
  cg::cluster_group cl = cg::this_cluster();
  const int csize = (int)cl.num_blocks();
  const int crank = (int)cl.block_rank();
  const int cid = blockIdx.x / csize;
  const int c0 = cid * kc;
  const int kw = min(k, c0 + kc) - c0;
  if (kw <= 0) return;  // the whole cluster leaves together
  T *xw = x + c0;
  const int ngroups = csize * kClusterThreads / G;
  const int gid = (crank * kClusterThreads + threadIdx.x) / G;
  const int lane = threadIdx.x % G;
  RowStatic<T> rs;
  int r0 = lev_ptr[0], r1 = lev_ptr[1];
  if (r0 + gid < r1) load_row(A, r0 + gid, rs);
  for (int l = 0; l < nlev; ++l) {
    int row = r0 + gid;
    if (row < r1) {
      if (G == 1 && VEC == 1 && k == 1) {
        T acc = ldx(xw + rs.orig);
        acc = row_accumulate<T, true, AR>(A, rs, xw, acc);
        xw[rs.orig] = row_finish(A, rs, acc);
      } else {
        row_window<T, G, VEC, AR>(A, rs, xw, k, kw, lane);
      }
    }
    for (row += ngroups; row < r1; row += ngroups) {
      RowStatic<T> r2;
      load_row(A, row, r2);
      if (G == 1 && VEC == 1 && k == 1) {
        T acc = ldx(xw + r2.orig);
        acc = row_accumulate<T, true, AR>(A, r2, xw, acc);
        xw[r2.orig] = row_finish(A, r2, acc);
      } else {
        row_window<T, G, VEC, AR>(A, r2, xw, k, kw, lane);
      }
    }
    if (l + 1 < nlev) {
      cluster_arrive();
      const int n0 = r1, n1 = lev_ptr[l + 2];
      if (n0 + gid < n1) load_row(A, n0 + gid, rs);
      cluster_wait();
      r0 = n0;
      r1 = n1;
    }
  }
}

// Cluster shape: up to 16 blocks per cluster (fewer for narrow systems),
// and as many clusters as the device holds at once, each taking a column
// slice of even width (so 16-byte loads stay aligned).
struct ClusterShape {
  int csize, nclusters, kc;
};

// co-resident clusters per (kernel, cluster size, device), queried once
static int max_clusters(const void *kernel, int csize, cudaLaunchConfig_t &cfg) {
  static std::mutex mu;
  static std::map<std::tuple<const void *, int, int>, int> cache;
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  const auto key = std::make_tuple(kernel, csize, dev);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int maxc = 0;
  if (cudaOccupancyMaxActiveClusters(&maxc, kernel, &cfg) != cudaSuccess) {
    cudaGetLastError();
    maxc = 0;
  }
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = maxc;
  return maxc;
}

template <class K>
static ClusterShape cluster_shape(gbsym_tri_s *t, K kernel, int k, int lanes) {
  // blocks needed to give every row of the widest level its own group
  const long long want = div_up((long long)t->max_level_rows * lanes, kClusterThreads);
  int csize = 16;
  while (csize > 1 && csize / 2 >= want) csize /= 2;
  if (t->cluster_blocks > 0) csize = std::min(csize, t->cluster_blocks);
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(kClusterThreads);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int maxc = 1;
  for (;;) {
    cfg.gridDim = dim3(csize);
    maxc = max_clusters((const void *)kernel, csize, cfg);
    if (maxc >= 1) break;
    if (csize == 1) {
      maxc = 1;
      break;
    }
    csize /= 2;
    at[0].val.clusterDim.x = csize;
  }
  ClusterShape sh;
  sh.csize = csize;
  if (k == 1) {
    sh.nclusters = 1;
    sh.kc = 1;
  } else {
    int kc = div_up(k, std::max(1, maxc));
    if (kc % 2) ++kc;
    sh.kc = std::min(kc, k % 2 ? k + 1 : k);
    sh.nclusters = div_up(k, sh.kc);
  }
  return sh;
}

template <class K, class... Args>
static void launch_cluster(K kernel, const ClusterShape &sh, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(sh.csize * sh.nclusters);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = sh.csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  GB_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
  check_launch();
}

template <class T, int G, int VEC, int AR>
static void cluster_go(gbsym_tri_s *t, T *x, int k, cudaStream_t s) {
  auto kern = k_cluster_sweep<T, G, VEC, AR>;
  GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  const ClusterShape sh = cluster_shape(t, kern, k, G);
  launch_cluster(kern, sh, s, view_of<T>(t), x, k, sh.kc, (const int *)t->lev_ptr.p, t->nlev);
}

// lanes per row for a column slice of width kc
template <class T, int AR>
static void cluster_ar(gbsym_tri_s *t, T *x, int k, cudaStream_t s) {
  if (k == 1) {
    cluster_go<T, 1, 1, AR>(t, x, 1, s);
    return;
  }
  // the slice width depends on the cluster count; size lanes for the
  // widest slice a 16-cluster split can give (k / 8 rounded up, even)
  int kc = div_up(k, 8);
  if (kc % 2) ++kc;
  const bool aligned = (k % 2 == 0) && ((uintptr_t)x % (2 * sizeof(T)) == 0);
  if (!aligned) {
    cluster_go<T, 4, 1, AR>(t, x, k, s);
    return;
  }
  const int need = div_up(kc, 2);
  if (need <= 1) cluster_go<T, 1, 2, AR>(t, x, k, s);
  else if (need <= 2) cluster_go<T, 2, 2, AR>(t, x, k, s);
  else if (need <= 4) cluster_go<T, 4, 2, AR>(t, x, k, s);
  else if (need <= 8) cluster_go<T, 8, 2, AR>(t, x, k, s);
  else cluster_go<T, 16, 2, AR>(t, x, k, s);
}

template <class T>
void run_cluster(gbsym_tri_s *t, T *x, int k, cudaStream_t s) {
  if (t->arith == kArithFused) cluster_ar<T, kArithFused>(t, x, k, s);
  else cluster_ar<T, kArithExact>(t, x, k, s);
}

template void run_cluster<double>(gbsym_tri_s *, double *, int, cudaStream_t);
template void run_cluster<float>(gbsym_tri_s *, float *, int, cudaStream_t);

}  // namespace gbsym
