// noalloc.cu -- a forward triangular solve that allocates nothing.
//
// Some callers cannot allocate device memory: a host application that
// hands all device memory to its own pool allocator (a framework's caching
// allocator, a memory-budgeted service) and cannot accept foreign
// cudaMalloc/cudaFree calls, which also synchronise the whole device; or a
// latency-critical loop where such a synchronisation is not acceptable.
// The plan API allocates its packed copy of the matrix and its scratch, so
// those callers get this entry point instead: it runs the sync-free
// executor's algorithm directly on the caller's CSR arrays, and the only
// memory it needs beyond the caller's inputs and outputs -- the published
// solution values and an error word -- lives in one file-scope static
// device array of fixed size.  Every GPU that loads this library holds that
// array (4 MiB plus a few words) until the process exits.
//
// Rows are processed in natural order, which is a topological order of a
// lower-triangular solve: warp units of 32 consecutive rows are dealt to
// warps round-robin, each warp walking its units in increasing order, in a
// cooperative launch (every warp co-resident), so the smallest unfinished
// row can always proceed.  A finished row publishes its value into the
// static array, pre-filled with an all-ones bit pattern; dependent rows
// poll those values with relaxed loads.  Each row is accumulated in storage
// order with separately rounded multiply and subtract and an IEEE division,
// the reference's sptrsv_csr sequence (sparse_blas/sptrsv.cpp:17-25).
// Waits are bounded; a malformed row (a column outside [0, row)) is
// reported, not followed.
//
// The first call on a device does that device's set-up: it looks up the
// device address of the static array (cudaGetSymbolAddress, with that
// device current) and the kernel's resident blocks per SM, and remembers
// both.  Every call clears the part of the array it uses, runs the sweep
// and copies the error word back to the host, and returns only after the
// solve has finished on its stream, so no call can be captured into a CUDA
// graph.  All calls share the array and the last call's contents stay in
// it, so calls that overlap on the GPU (different streams, or different
// host threads on one device) race: serialise them.
//
// The caller's row pointers must be valid: Lp[0..n] non-decreasing and
// every Lp[i+1] within Li and Lx, since the kernel reads
// Li[Lp[i] .. Lp[i+1]) without knowing the arrays' lengths.  Column
// indices are checked before use.  After GBSYM_ERR_BAD_MATRIX or
// GBSYM_ERR_TIMEOUT the contents of x are undefined (rows finished before
// the error keep their solved values).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace gbsym {
namespace {

constexpr int kNoAllocMaxRows = 1 << 19;  // 524,288 rows
constexpr int kNoAllocTail = 32;           // error word (and padding)
constexpr int kNaBlock = 256;

// published values (one 8-byte slot per row), then the error word
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocMaxRows + kNoAllocTail];

struct DeviceScratch {
  unsigned long long *ptr = nullptr;  // device address of g_noalloc_scratch
  int per_sm = 0;                     // resident blocks of the sweep per SM
  bool ready = false;
};
static std::mutex g_na_mu;
static DeviceScratch g_na_dev[64];

__device__ __forceinline__ double na_ld_rlx(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return __longlong_as_double((long long)v);
}
__device__ __forceinline__ void na_st_rlx(unsigned long long *p, double d) {
  unsigned long long v = (unsigned long long)__double_as_longlong(d);
  if (v == ~0ull) v = 0x7ff8000000000000ull;  // never publish the sentinel
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__global__ void __launch_bounds__(kNaBlock)
k_noalloc_forward(int n, const int *__restrict__ Lp, const int *__restrict__ Li,
                  const double *__restrict__ Lx, double *__restrict__ x, unsigned long long *scratch) {
  constexpr unsigned FULL = 0xffffffffu;
  int *err = reinterpret_cast<int *>(scratch + kNoAllocMaxRows);
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nunits = (n + 31) >> 5;
  for (int u = warp; u < nunits; u += nwarps) {
    const int i = (u << 5) + lane;
    bool done = i >= n;
    int j = 0, end = 0;
    double acc = 0.0;
    if (!done) {
      j = Lp[i];
      end = Lp[i + 1] - 1;  // the diagonal is the last entry of the row
      acc = x[i];
      if (end < j) {        // an empty row has no diagonal
        atomicCAS(err, 0, GBSYM_ERR_BAD_MATRIX);
        done = true;
      }
    }
    long long t0 = clock64();
    int rounds = 0;
    while (__any_sync(FULL, !done)) {
      bool moved = false;
      if (!done) {
        while (j < end) {
          const int c = Li[j];
          if (c < 0 || c >= i) {  // not a dependency of a lower triangle
            atomicCAS(err, 0, GBSYM_ERR_BAD_MATRIX);
            j = end;
            done = true;
            break;
          }
          const double v = na_ld_rlx(scratch + c);
          if (__double_as_longlong(v) == -1ll) break;  // not published yet
          acc = __dsub_rn(acc, __dmul_rn(Lx[j], v));
          ++j;
          moved = true;
        }
        if (!done && j >= end) {
          acc = __ddiv_rn(acc, Lx[end]);
          x[i] = acc;
          na_st_rlx(scratch + i, acc);
          done = true;
          moved = true;
        }
        if (moved) t0 = clock64();
      }
      if (!__any_sync(FULL, moved)) __nanosleep(32);
      if ((++rounds & 63) == 0) {
        if (!done && clock64() - t0 > (1ll << 32)) {
          atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
          done = true;
        }
        const int e = lane == 0 ? ld_relaxed(err) : 0;
        if (__shfl_sync(FULL, e, 0) != 0) return;
      }
    }
  }
}

// Device address of the static array for the current device and the
// sweep's resident blocks per SM, looked up once per device (with that
// device current) and remembered.
static DeviceScratch scratch_for_current_device() {
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CHECK(dev >= 0 && dev < 64, GBSYM_ERR_UNSUPPORTED);
  std::lock_guard<std::mutex> lk(g_na_mu);
  DeviceScratch &d = g_na_dev[dev];
  if (!d.ready) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      std::fprintf(stderr, "gbsym: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      throw Err{GBSYM_ERR_CUDA};
    }
    int per_sm = 0;
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_noalloc_forward, kNaBlock, 0));
    d.ptr = static_cast<unsigned long long *>(p);
    d.per_sm = per_sm;
    d.ready = true;
  }
  return d;
}

}  // namespace
}  // namespace gbsym

using namespace gbsym;

extern "C" int gbsym_sptrsv_csr_noalloc(int n, const int *Lp, const int *Li, const double *Lx,
                                        double *x, void *stream) {
  if (n < 0 || n > kNoAllocMaxRows) {
    std::fprintf(stderr, "gbsym_sptrsv_csr_noalloc: n = %d is outside [0, %d]\n", n, kNoAllocMaxRows);
    return GBSYM_ERR_SIZE;
  }
  if (n == 0) return GBSYM_OK;
  if (!Lp || !Li || !Lx || !x) return GBSYM_ERR_NULL_ARG;
  int code = GBSYM_OK;
  const int st = guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    const DeviceScratch d = scratch_for_current_device();
    // the cooperative sweep needs one resident block on every SM
    GB_CHECK(d.per_sm >= 1, GBSYM_ERR_UNSUPPORTED);
    unsigned long long *scratch = d.ptr;
    // published values start as the sentinel; the error word starts at zero
    GB_CUDA(cudaMemsetAsync(scratch, 0xff, (size_t)n * sizeof(unsigned long long), s));
    GB_CUDA(cudaMemsetAsync(scratch + kNoAllocMaxRows, 0, sizeof(int), s));
    const int grid = num_sms();
    void *params[] = {(void *)&n, (void *)&Lp, (void *)&Li, (void *)&Lx, (void *)&x, (void *)&scratch};
    GB_CUDA(cudaLaunchCooperativeKernel((const void *)k_noalloc_forward, dim3(grid), dim3(kNaBlock), params,
                                        0, s));
    check_launch();
    GB_CUDA(cudaMemcpyAsync(&code, scratch + kNoAllocMaxRows, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
  });
  return st ? st : code;
}
