// common.cuh -- shared internals of the gbsym library: status plumbing,
// separately-rounded arithmetic, device buffers, launch accounting.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gbsym.h"
#include "nvtx3/nvToolsExt.h"

namespace gbsym {

// ---------------------------------------------------------------------------
// status
struct Err {
  int code;
};

void set_last_error(int code);
int last_error();

#define GB_CUDA(call)                                                     \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) {                                              \
      std::fprintf(stderr, "gbsym: %s failed at %s:%d: %s\n", #call,      \
                   __FILE__, __LINE__, cudaGetErrorString(e_));           \
      throw ::gbsym::Err{GBSYM_ERR_CUDA};                                 \
    }                                                                     \
  } while (0)

#define GB_CHECK(cond, code)                 \
  do {                                       \
    if (!(cond)) throw ::gbsym::Err{(code)}; \
  } while (0)

// Runs f() and converts thrown Err / std::bad_alloc into a status code.
template <class F>
int guarded(F &&f) {
  try {
    f();
    return GBSYM_OK;
  } catch (const Err &e) {
    return e.code;
  } catch (const std::bad_alloc &) {
    return GBSYM_ERR_SIZE;
  }
}

// A named NVTX range around one call of a library phase (plan build,
// factorisation, solve, Krylov iteration, batch), so that Nsight timelines
// show where a caller's time goes.  Header-only NVTX: without a tool
// attached a push or pop is a check of a function pointer.
struct PhaseRange {
  explicit PhaseRange(const char *name) { nvtxRangePushA(name); }
  ~PhaseRange() { nvtxRangePop(); }
  PhaseRange(const PhaseRange &) = delete;
  PhaseRange &operator=(const PhaseRange &) = delete;
};

// Every kernel launch made by the library goes through this counter.
extern std::atomic<unsigned long long> g_launches;
inline void count_launch(unsigned long long k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }
inline void check_launch() {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "gbsym: kernel launch failed: %s\n", cudaGetErrorString(e));
    throw Err{GBSYM_ERR_CUDA};
  }
}

// ---------------------------------------------------------------------------
// Separately rounded arithmetic.  The reference accumulates each row as
// x -= a*b with a rounded product and a rounded subtraction; these intrinsics
// keep nvcc from contracting the pair into one fused multiply-add.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double sqrt_rn(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float sqrt_rn(float a) { return __fsqrt_rn(a); }

// Relaxed device-scope loads/stores for values other threads publish while
// a kernel runs (level numbers, ready flags).
__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(int *p, int v) {
  asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded waits: a wait that sees no progress for this long records
// GBSYM_ERR_TIMEOUT in the launch's error word and returns.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s
constexpr long long kWaitLimitIters = 1ll << 26;

// ---------------------------------------------------------------------------
// Device buffer (owning).
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) GB_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
  }
  // grow-only reuse
  void reserve(size_t count) {
    if (count > n) alloc(count);
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

// Library-owned non-blocking stream of the calling host thread (drop-ins).
cudaStream_t thread_stream();
int num_sms();

// Copies host or device data of `count` elements into a fresh device buffer.
template <class T>
void upload(DBuf<T> &dst, const T *src, size_t count, bool on_device, cudaStream_t s) {
  dst.alloc(count);
  if (count)
    GB_CUDA(cudaMemcpyAsync(dst.p, src, count * sizeof(T),
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
}

}  // namespace gbsym
