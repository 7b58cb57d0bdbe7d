// csr.cuh -- device CSR matrix plan (gbsym_csr) and SpMV entry points.
#pragma once

#include "common.cuh"

struct gbsym_csr_s {
  int n = 0, ncols = 0, vdtype = GBSYM_F64;
  long long nnz = 0;
  gbsym::DBuf<int> p, i;
  gbsym::DBuf<double> x64;
  gbsym::DBuf<float> x32;
};

namespace gbsym {
void csr_spmv(const gbsym_csr_s *a, const void *x, void *y, int dtype, cudaStream_t s);
void csr_spmv_axpby(const gbsym_csr_s *a, const double *x, const double *y, double *z,
                    double alpha, double beta, cudaStream_t s);
gbsym_csr_s *csr_build(int n, int ncols, const int *p, const int *i, const double *x, int vdtype,
                       bool on_device, cudaStream_t s);
void convert_f64_f32(const double *a, float *b, long long n, cudaStream_t s);
void convert_f32_f64(const float *a, double *b, long long n, cudaStream_t s);
}  // namespace gbsym
