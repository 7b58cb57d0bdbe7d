// spmv.cu -- CSR sparse matrix-vector products on the GPU.
//
// Reference: spmv_csr / spmv_csr_parallel (sparse_blas/spmv.cpp:12-21,
// 37-57) and the accumulate form spmv_csr(..., y, z, a, b) (spmv.cpp:
// 23-34).  Each row is summed by one thread in storage order with
// separately rounded multiply and add, the order the reference uses, so
// FP64 results match it bit for bit.
#include <algorithm>
#include <memory>

#include "csr.cuh"

namespace gbsym {

constexpr int kSpmvRows = 256;

// acc + RN(v * x), both roundings separate (the reference's order), issued
// in FP64 as fused multiply-adds with a constant operand: RN(v*x) =
// fma(v, x, -0) and RN(acc + p) = fma(p, 1, acc) are bit-identical to the
// separate operations for every input, and run at their rate.  Inline PTX
// keeps the compiler from folding the two into one FMA.
__device__ __forceinline__ double madd_exact(double acc, double v, double x) {
  double r;
  asm("{\n\t.reg .f64 p;\n\tfma.rn.f64 p, %1, %2, 0d8000000000000000;\n\t"
      "fma.rn.f64 %0, p, 0d3FF0000000000000, %3;\n\t}"
      : "=d"(r) : "d"(v), "d"(x), "d"(acc));
  return r;
}
__device__ __forceinline__ float madd_exact(float acc, float v, float x) { return add_rn(acc, mul_rn(v, x)); }

// MODE 0: y = A x.  MODE 1: z = alpha (z + A x) + beta y.
// One thread per row, loading its entries directly: on this part the
// exact FP64 sum is bound by the FP64 pipe (two DFMAs per entry; ncu on the
// 96^3 convection-diffusion operator: FP64 pipe 72% active, DRAM 36%), so
// the kernel keeps many independent rows in flight with no barrier in the
// way.  Staging each block's entries through shared memory measured 5-10%
// slower; staging each warp's products (coalesced loads, then each lane's
// ordered sum from shared memory) 29% slower; preloading eight entries per
// thread before the sum 0-6% slower on that operator.
template <class T, int MODE>
__global__ void __launch_bounds__(kSpmvRows)
k_spmv(int n, const int *__restrict__ p, const int *__restrict__ ci, const T *__restrict__ val,
       const T *__restrict__ x, const T *__restrict__ yin, T *__restrict__ out, T alpha, T beta) {
  const int row = blockIdx.x * kSpmvRows + threadIdx.x;
  if (row >= n) return;
  const int lo = p[row], hi = p[row + 1];
  T acc = MODE == 1 ? out[row] : T(0);
  for (int e = lo; e < hi; ++e) acc = madd_exact(acc, val[e], x[ci[e]]);
  if (MODE == 1) acc = add_rn(mul_rn(alpha, acc), mul_rn(beta, yin[row]));
  out[row] = acc;
}

template <class T>
void spmv_typed(const gbsym_csr_s *a, const T *x, T *y, cudaStream_t s) {
  if (a->n == 0) return;
  const T *val = nullptr;
  if constexpr (sizeof(T) == 8) val = (const T *)a->x64.p; else val = (const T *)a->x32.p;
  k_spmv<T, 0><<<div_up(a->n, kSpmvRows), kSpmvRows, 0, s>>>(a->n, a->p.p, a->i.p, val, x, nullptr,
                                                            y, T(0), T(0));
  check_launch();
}

void csr_spmv(const gbsym_csr_s *a, const void *x, void *y, int dtype, cudaStream_t s) {
  if (dtype == GBSYM_F64) {
    GB_CHECK(a->x64.p || a->nnz == 0, GBSYM_ERR_UNSUPPORTED);
    spmv_typed<double>(a, (const double *)x, (double *)y, s);
  } else {
    GB_CHECK(a->x32.p || a->nnz == 0, GBSYM_ERR_UNSUPPORTED);
    spmv_typed<float>(a, (const float *)x, (float *)y, s);
  }
}

void csr_spmv_axpby(const gbsym_csr_s *a, const double *x, const double *y, double *z,
                    double alpha, double beta, cudaStream_t s) {
  if (a->n == 0) return;
  GB_CHECK(a->x64.p || a->nnz == 0, GBSYM_ERR_UNSUPPORTED);
  k_spmv<double, 1><<<div_up(a->n, kSpmvRows), kSpmvRows, 0, s>>>(a->n, a->p.p, a->i.p, a->x64.p,
                                                                  x, y, z, alpha, beta);
  check_launch();
}

__global__ void k_validate_csr(int n, int ncols, const int *__restrict__ p,
                               const int *__restrict__ ci, int *err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int a = p[i], z = p[i + 1];
    bool bad = z < a;
    for (int e = a; !bad && e < z; ++e) bad = ci[e] < 0 || ci[e] >= ncols;
    if (bad && atomicCAS(err, 0, GBSYM_ERR_BAD_MATRIX) == 0) err[1] = i;
  }
}

gbsym_csr_s *csr_build(int n, int ncols, const int *p, const int *i, const double *x, int vdtype,
                       bool on_device, cudaStream_t s) {
  GB_CHECK(n >= 0 && ncols >= 0, GBSYM_ERR_SIZE);
  GB_CHECK(vdtype == GBSYM_F64 || vdtype == GBSYM_F32, GBSYM_ERR_UNSUPPORTED);
  std::unique_ptr<gbsym_csr_s> a(new gbsym_csr_s());
  a->n = n;
  a->ncols = ncols;
  a->vdtype = vdtype;
  int nnz = 0;
  if (on_device) {
    if (n) {
      GB_CUDA(cudaMemcpyAsync(&nnz, p + n, sizeof(int), cudaMemcpyDeviceToHost, s));
      GB_CUDA(cudaStreamSynchronize(s));
    }
  } else {
    nnz = n ? p[n] : 0;
  }
  a->nnz = nnz;
  upload(a->p, p, n + 1, on_device, s);
  upload(a->i, i, nnz, on_device, s);
  if (vdtype == GBSYM_F64) {
    upload(a->x64, x, nnz, on_device, s);
  } else {
    DBuf<double> tmp;
    upload(tmp, x, nnz, on_device, s);
    a->x32.alloc(nnz);
    convert_f64_f32(tmp.p, a->x32.p, nnz, s);
    GB_CUDA(cudaStreamSynchronize(s));
  }
  if (n) {
    DBuf<int> err(2);
    GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
    k_validate_csr<<<std::min(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(n, ncols, a->p.p,
                                                                           a->i.p, err.p);
    check_launch();
    int h[2];
    GB_CUDA(cudaMemcpyAsync(h, err.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (h[0]) throw Err{h[0]};
  }
  return a.release();
}

__global__ void k_f64_to_f32(const double *__restrict__ a, float *__restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}
__global__ void k_f32_to_f64(const float *__restrict__ a, double *__restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

void convert_f64_f32(const double *a, float *b, long long n, cudaStream_t s) {
  if (!n) return;
  k_f64_to_f32<<<(int)std::min<long long>(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(a, b, n);
  check_launch();
}
void convert_f32_f64(const float *a, double *b, long long n, cudaStream_t s) {
  if (!n) return;
  k_f32_to_f64<<<(int)std::min<long long>(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(a, b, n);
  check_launch();
}

}  // namespace gbsym

using namespace gbsym;

extern "C" int gbsym_csr_create(gbsym_csr *out, int n, int ncols, const int *p, const int *i,
                                const double *x, int value_dtype, int on_device, void *stream) {
  if (!out || (n > 0 && (!p || !i || !x))) return GBSYM_ERR_NULL_ARG;
  *out = nullptr;
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    *out = csr_build(n, ncols, p, i, x, value_dtype, on_device != 0, s);
  });
}

extern "C" int gbsym_csr_destroy(gbsym_csr a) {
  delete a;
  return GBSYM_OK;
}

extern "C" int gbsym_csr_spmv(gbsym_csr a, const void *x, void *y, int dtype, void *stream) {
  gbsym::PhaseRange phase_("gbsym_csr_spmv");
  if (!a || (a->n && (!x || !y))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    csr_spmv(a, x, y, dtype, (cudaStream_t)stream);
  });
}

extern "C" int gbsym_csr_spmv_axpby(gbsym_csr a, const double *x, const double *y, double *z,
                                    double alpha, double beta, void *stream) {
  if (!a || (a->n && (!x || !y || !z))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    csr_spmv_axpby(a, x, y, z, alpha, beta, (cudaStream_t)stream);
  });
}
