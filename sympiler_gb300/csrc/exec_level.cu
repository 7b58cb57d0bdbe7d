// exec_level.cu -- LEVELSET executor: one launch per wavefront level,
// captured once into a CUDA graph and replayed.
//
// The level kernels use programmatic dependent launch: a kernel starts while
// its predecessor runs, loads the static part of its rows (permutation,
// length, divisor, reciprocal and the slab columns and values -- independent
// coalesced loads), and only then waits for the previous level
// (griddepcontrol.wait) before gathering x, with all of a row's gathers in
// flight at once.  This is the reference's per-level parallel-for
// (sptrsv_csr_levelset, sparse_blas/sptrsv.cpp:40-55) with the fork/join
// replaced by a kernel boundary that overlaps the next level's loads.
#include <algorithm>

#include "exec_common.cuh"

namespace gbsym {

constexpr int kLvlBlock = 64;  // narrow blocks spread a level over more SMs

template <class T, bool REDUNDANT, int AR>
__global__ void __launch_bounds__(kLvlBlock)
k_level_1rhs(TriView<T> A, T *__restrict__ x, const T *__restrict__ b, int r_begin, int r_end) {
  pdl_trigger();
  const int row = r_begin + blockIdx.x * kLvlBlock + threadIdx.x;
  const bool active = row < r_end;
  RowStatic<T> r;
  if (active) load_row(A, row, r);
  pdl_wait();  // the previous level's x is complete and visible from here
  if (!active) return;
  T acc = REDUNDANT ? T(0) : x[r.orig];
  acc = row_accumulate<T, false, AR>(A, r, x, acc);
  if (REDUNDANT) acc = add_rn(acc, b[r.orig]);
  x[r.orig] = row_finish(A, r, acc);
}

template <class T, int G, int VEC, int AR>
__global__ void __launch_bounds__(256)
k_level_mrhs(TriView<T> A, T *__restrict__ x, int k, int r_begin, int r_end) {
  pdl_trigger();
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int lane = threadIdx.x % G;
  const int row = r_begin + gid;
  const bool active = row < r_end;
  RowStatic<T> rs;
  if (active) load_row(A, row, rs);
  pdl_wait();
  if (!active) return;
  row_mrhs<T, G, VEC, false, AR>(A, rs, x, k, lane);
}

template <class K, class... Args>
static void launch_pdl(K kernel, dim3 grid, dim3 block, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  GB_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
  check_launch();
}

template <class T, int G, int AR>
static void launch_level_mrhs(const TriView<T> &A, T *x, int k, int a, int z, cudaStream_t s) {
  const int grid = div_up(z - a, 256 / G);
  const bool v4 = sizeof(T) == 4 && (k % 4 == 0) && ((uintptr_t)x % 16 == 0);
  const bool v2 = (k % 2 == 0) && ((uintptr_t)x % (2 * sizeof(T)) == 0);
  if (v4)
    launch_pdl(k_level_mrhs<T, G, (sizeof(T) == 4 ? 4 : 2), AR>, dim3(grid), dim3(256), s, A, x, k, a, z);
  else if (v2)
    launch_pdl(k_level_mrhs<T, G, 2, AR>, dim3(grid), dim3(256), s, A, x, k, a, z);
  else
    launch_pdl(k_level_mrhs<T, G, 1, AR>, dim3(grid), dim3(256), s, A, x, k, a, z);
}

template <class T, int AR>
static void launch_level(const TriView<T> &A, T *x, const T *b, int k, int a, int z, cudaStream_t s) {
  if (z <= a) return;
  if (k == 1) {
    const int grid = div_up(z - a, kLvlBlock);
    if (b)
      launch_pdl(k_level_1rhs<T, true, AR>, dim3(grid), dim3(kLvlBlock), s, A, x, b, a, z);
    else
      launch_pdl(k_level_1rhs<T, false, AR>, dim3(grid), dim3(kLvlBlock), s, A, x, (const T *)nullptr, a, z);
    return;
  }
  switch (lanes_for(k, sizeof(T))) {
    case 2: launch_level_mrhs<T, 2, AR>(A, x, k, a, z, s); break;
    case 4: launch_level_mrhs<T, 4, AR>(A, x, k, a, z, s); break;
    case 8: launch_level_mrhs<T, 8, AR>(A, x, k, a, z, s); break;
    case 16: launch_level_mrhs<T, 16, AR>(A, x, k, a, z, s); break;
    default: launch_level_mrhs<T, 32, AR>(A, x, k, a, z, s); break;
  }
}

template <class T>
static void issue_levels(gbsym_tri_s *t, T *x, const T *b, int k, cudaStream_t s) {
  const TriView<T> A = view_of<T>(t);
  for (int l = 0; l < t->nlev; ++l) {
    if (t->arith == kArithFused)
      launch_level<T, kArithFused>(A, x, b, k, t->h_lev_ptr[l], t->h_lev_ptr[l + 1], s);
    else
      launch_level<T, kArithExact>(A, x, b, k, t->h_lev_ptr[l], t->h_lev_ptr[l + 1], s);
  }
}

// Level launches are captured once per (x, b, k, dtype, arithmetic) into a
// CUDA graph and replayed; the plan keeps the eight most recent.
template <class T>
void run_levelset(gbsym_tri_s *t, T *x, const T *b, int k, int dtype, cudaStream_t s) {
  if (t->nlev <= 2) {
    issue_levels<T>(t, x, b, k, s);
    return;
  }
  GraphEntry *hit = nullptr;
  for (auto &g : t->graphs)
    if (g.x == x && g.b == b && g.k == k && g.dtype == dtype && g.exec == t->arith) hit = &g;
  if (!hit) {
    if (t->graphs.size() >= 8) {
      auto old = std::min_element(t->graphs.begin(), t->graphs.end(),
                                  [](const GraphEntry &a, const GraphEntry &c) { return a.stamp < c.stamp; });
      cudaGraphExecDestroy(old->exec_graph);
      t->graphs.erase(old);
    }
    GraphEntry g;
    g.x = x;
    g.b = b;
    g.k = k;
    g.dtype = dtype;
    g.exec = t->arith;
    cudaGraph_t graph;
    GB_CUDA(cudaStreamBeginCapture(t->cap_stream, cudaStreamCaptureModeThreadLocal));
    const unsigned long long before = g_launches.load();
    try {
      issue_levels<T>(t, x, b, k, t->cap_stream);
    } catch (...) {
      cudaStreamEndCapture(t->cap_stream, &graph);
      throw;
    }
    g.nodes = g_launches.load() - before;
    g_launches.fetch_sub(g.nodes);  // counted when replayed
    GB_CUDA(cudaStreamEndCapture(t->cap_stream, &graph));
    GB_CUDA(cudaGraphInstantiate(&g.exec_graph, graph, 0));
    cudaGraphDestroy(graph);
    t->graphs.push_back(g);
    hit = &t->graphs.back();
  }
  hit->stamp = ++t->graph_clock;
  GB_CUDA(cudaGraphLaunch(hit->exec_graph, s));
  count_launch(hit->nodes);
}

template void run_levelset<double>(gbsym_tri_s *, double *, const double *, int, int, cudaStream_t);
template void run_levelset<float>(gbsym_tri_s *, float *, const float *, int, int, cudaStream_t);

}  // namespace gbsym
