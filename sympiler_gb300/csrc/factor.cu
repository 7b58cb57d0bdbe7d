// factor.cu -- incomplete factorisations on the GPU, level-scheduled.
//
// ILU0 restates spilu0_csr (sparse_blas/spilu0.cpp:11-51): row i, in order
// over its lower entries j, takes the multiplier l_ij = l_ij / u_jj and
// subtracts l_ij * u_j* from the entries of row i that are in its pattern.
// Rows only read finished rows, so rows of one wavefront level of the lower
// pattern are independent: one warp per row, the j loop sequential (the
// reference's order), the pattern-matched updates of one j spread over the
// lanes (they touch distinct entries).
//
// IC0 restates spic0_csr (sparse_blas/spic0.cpp:106-128), which is
// right-looking on the upper CSR of A.  The same values come out of a
// left-looking sweep: row c receives its updates from the earlier rows i
// that hold column c, in ascending i (see k_ic0_rows for which entry each
// such row updates), then the diagonal takes its square root and the
// off-diagonals are divided by it.  The rows i feeding row c are the column
// c of the upper pattern, found through its transpose; rows run one warp
// each, one launch per wavefront level.
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "tri.cuh"

namespace gbsym {

__device__ __forceinline__ int find_col(const int *__restrict__ ci, int a, int z, int col) {
  int lo = a, hi = z;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (ci[mid] < col) lo = mid + 1; else hi = mid;
  }
  return (lo < z && ci[lo] == col) ? lo : -1;
}

__global__ void k_check_sorted(int n, const int *__restrict__ p, const int *__restrict__ ci,
                               const int *__restrict__ dg, int need_diag_first, int *err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int a = p[i], z = p[i + 1];
    bool bad = z <= a;
    for (int e = a; !bad && e < z; ++e) {
      bad = ci[e] < 0 || ci[e] >= n || (e > a && ci[e] <= ci[e - 1]);
    }
    if (!bad && dg) bad = dg[i] < a || dg[i] >= z || ci[dg[i]] != i;
    if (!bad && need_diag_first) bad = ci[a] != i;
    if (bad && atomicCAS(err, 0, GBSYM_ERR_BAD_MATRIX) == 0) err[1] = i;
  }
}

static void check_sorted(int n, const int *p, const int *ci, const int *dg, bool diag_first,
                         cudaStream_t s) {
  if (!n) return;
  DBuf<int> err(2);
  GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
  k_check_sorted<<<std::min(div_up(n, 256), num_sms() * 8), 256, 0, s>>>(n, p, ci, dg,
                                                                         diag_first ? 1 : 0, err.p);
  check_launch();
  int h[2];
  GB_CUDA(cudaMemcpyAsync(h, err.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (h[0]) throw Err{h[0]};
}

__global__ void k_ilu0_rows(const int *__restrict__ p, const int *__restrict__ ci,
                            const int *__restrict__ dg, double *l, const int *__restrict__ order,
                            int r0, int r1, int *err) {
  const int lane = threadIdx.x & 31;
  const int k = r0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (k >= r1) return;
  const int i = order[k];
  const int a = p[i], z = p[i + 1], di = dg[i];
  for (int j = a; j < di; ++j) {
    const int jrow = ci[j];
    double tl = 0.0;
    if (lane == 0) {
      tl = div_rn(l[j], l[dg[jrow]]);
      l[j] = tl;
    }
    tl = __shfl_sync(0xffffffffu, tl, 0);
    const int end = p[jrow + 1];
    for (int jj = dg[jrow] + 1 + lane; jj < end; jj += 32) {
      const int jw = find_col(ci, a, z, ci[jj]);
      if (jw >= 0) l[jw] = sub_rn(l[jw], mul_rn(tl, l[jj]));
    }
    __syncwarp();
  }
  if (lane == 0 && l[di] == 0.0 && atomicCAS(err, 0, GBSYM_ERR_PIVOT) == 0) err[1] = i;
}

void ilu0_device(int n, const int *Ap, const int *Ai, const double *Ax, const int *A_diag,
                 double *l, cudaStream_t s) {
  if (n == 0) return;
  check_sorted(n, Ap, Ai, A_diag, false, s);
  int nnz = 0;
  GB_CUDA(cudaMemcpyAsync(&nnz, Ap + n, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  GB_CUDA(cudaMemcpyAsync(l, Ax, (size_t)nnz * sizeof(double), cudaMemcpyDeviceToDevice, s));
  DBuf<int> lp, ls, err(2);
  const int nlev = build_levels_device(n, Ap, Ai, A_diag, GBSYM_ILU_UNIT_LOWER, lp, ls, s);
  std::vector<int> h(nlev + 1);
  GB_CUDA(cudaMemcpyAsync(h.data(), lp.p, (nlev + 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
  GB_CUDA(cudaStreamSynchronize(s));
  for (int lv = 0; lv < nlev; ++lv) {
    const int rows = h[lv + 1] - h[lv];
    k_ilu0_rows<<<div_up(rows, 8), 256, 0, s>>>(Ap, Ai, A_diag, l, ls.p, h[lv], h[lv + 1], err.p);
    check_launch();
  }
  int he[2];
  GB_CUDA(cudaMemcpyAsync(he, err.p, sizeof(he), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (he[0]) throw Err{he[0]};
}

// ---- IC0 -------------------------------------------------------------------
__global__ void k_row_ids(int n, const int *__restrict__ p, int *rowid) {
  const int lane = threadIdx.x & 31;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n;
       i += (gridDim.x * blockDim.x) >> 5)
    for (int e = p[i] + lane; e < p[i + 1]; e += 32) rowid[e] = i;
}

__global__ void k_gather_int(long long m, const int *__restrict__ src, const int *__restrict__ idx,
                             int *dst) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m;
       t += (long long)gridDim.x * blockDim.x)
    dst[t] = src[idx[t]];
}

__global__ void k_row_bounds(int n, long long m, const int *__restrict__ sorted_rows, int *rp) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m;
       t += (long long)gridDim.x * blockDim.x) {
    const int r = sorted_rows[t];
    const int prev = t ? sorted_rows[t - 1] : -1;
    for (int q = prev + 1; q <= r; ++q) rp[q] = (int)t;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int last = m ? sorted_rows[m - 1] : -1;
    for (int q = last + 1; q <= n; ++q) rp[q] = (int)m;
  }
}

__global__ void k_iota_ll(long long m, int *v) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m;
       t += (long long)gridDim.x * blockDim.x)
    v[t] = (int)t;
}

// Transpose of a CSR pattern: for every entry e (row r, col c) of the input,
// output row c lists (col r, src e), r ascending (a stable radix sort of the
// entries by column keeps the input's row order).
void transpose_pattern(int n, int nnz, const int *p, const int *ci, Transposed &out,
                       cudaStream_t s) {
  out.rp.alloc(n + 1);
  out.ci.alloc(nnz);
  out.src.alloc(nnz);
  if (nnz == 0) {
    GB_CUDA(cudaMemsetAsync(out.rp.p, 0, (n + 1) * sizeof(int), s));
    return;
  }
  DBuf<int> rowid(nnz), keys_out(nnz), iota(nnz);
  const int g = std::max(1, std::min(div_up(std::max(nnz, n), 256), num_sms() * 8));
  k_row_ids<<<g, 256, 0, s>>>(n, p, rowid.p);
  check_launch();
  k_iota_ll<<<g, 256, 0, s>>>(nnz, iota.p);
  check_launch();
  int end_bit = 1;
  while ((1 << end_bit) < n && end_bit < 31) ++end_bit;
  size_t tmp_bytes = 0;
  GB_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, (const unsigned *)ci,
                                          (unsigned *)keys_out.p, iota.p, out.src.p, nnz, 0,
                                          end_bit, s));
  DBuf<char> tmp(tmp_bytes);
  GB_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, (const unsigned *)ci,
                                          (unsigned *)keys_out.p, iota.p, out.src.p, nnz, 0,
                                          end_bit, s));
  count_launch(4);
  k_gather_int<<<g, 256, 0, s>>>(nnz, rowid.p, out.src.p, out.ci.p);
  check_launch();
  k_row_bounds<<<g, 256, 0, s>>>(n, nnz, keys_out.p, out.rp.p);
  check_launch();
}

// Row c of the upper factor.  The reference's inner scan
// (spic0.cpp:117-123: `for (l = m; l < Lp[i+1] && Li[l+1] <= Li[k]; l++)
// if (Li[l] == Li[k]) ...`) tests the NEXT column before the match, so
// within row i it reaches a matching position only when that position is
// the last entry of row i (the following read is the next row's diagonal,
// i+1 <= Li[k]).  Row i therefore updates exactly one entry of row c: the
// one in the column of row i's last entry, if row c holds it.  Lanes find
// those targets and form the products for up to 32 rows i at a time; lane
// 0 applies the subtractions in ascending i, the reference's order.
__global__ void k_ic0_rows(const int *__restrict__ up, const int *__restrict__ ui, double *val,
                           const int *__restrict__ lp, const int *__restrict__ li,
                           const int *__restrict__ lsrc, const int *__restrict__ order, int r0,
                           int r1, int *err) {
  const int lane = threadIdx.x & 31;
  const int kk = r0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (kk >= r1) return;
  const int c = order[kk];
  const int a = up[c], z = up[c + 1];
  // transposed row c: rows i <= c holding column c; the last one is c itself
  const int t_end = lp[c + 1] - 1;
  for (int t0 = lp[c]; t0 < t_end; t0 += 32) {
    const int t = t0 + lane;
    int kpos = -1;
    double prod = 0.0;
    if (t < t_end) {
      const int i = li[t];
      const int m = lsrc[t];
      const int last = up[i + 1] - 1;
      kpos = find_col(ui, a, z, ui[last]);
      if (kpos >= 0) prod = mul_rn(val[m], val[last]);
    }
    const int cnt = min(32, t_end - t0);
    for (int q = 0; q < cnt; ++q) {
      const int kp = __shfl_sync(0xffffffffu, kpos, q);
      const double pr = __shfl_sync(0xffffffffu, prod, q);
      if (lane == 0 && kp >= 0) val[kp] = sub_rn(val[kp], pr);
    }
    __syncwarp();
  }
  double d = 0.0;
  if (lane == 0) {
    const double piv = val[a];
    if (!(piv > 0.0) && atomicCAS(err, 0, GBSYM_ERR_PIVOT) == 0) err[1] = c;
    d = sqrt_rn(piv);
    val[a] = d;
  }
  d = __shfl_sync(0xffffffffu, d, 0);
  for (int k = a + 1 + lane; k < z; k += 32) val[k] = div_rn(val[k], d);
}

void ic0_device(int n, double *val, const int *up, const int *ui, cudaStream_t s) {
  if (n == 0) return;
  check_sorted(n, up, ui, nullptr, true, s);
  int nnz = 0;
  GB_CUDA(cudaMemcpyAsync(&nnz, up + n, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  Transposed L;  // CSR of the lower factor: row c, columns i <= c, diagonal last
  transpose_pattern(n, nnz, up, ui, L, s);
  DBuf<int> lvp, lvs, err(2);
  const int nlev = build_levels_device(n, L.rp.p, L.ci.p, nullptr, GBSYM_LOWER_DIAG_LAST, lvp, lvs, s);
  std::vector<int> h(nlev + 1);
  GB_CUDA(cudaMemcpyAsync(h.data(), lvp.p, (nlev + 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), s));
  GB_CUDA(cudaStreamSynchronize(s));
  for (int lv = 0; lv < nlev; ++lv) {
    const int rows = h[lv + 1] - h[lv];
    k_ic0_rows<<<div_up(rows, 8), 256, 0, s>>>(up, ui, val, L.rp.p, L.ci.p, L.src.p, lvs.p, h[lv],
                                               h[lv + 1], err.p);
    check_launch();
  }
  int he[2];
  GB_CUDA(cudaMemcpyAsync(he, err.p, sizeof(he), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (he[0]) throw Err{he[0]};
}

}  // namespace gbsym

using namespace gbsym;

extern "C" int gbsym_ilu0_device(int n, const int *Ap, const int *Ai, const double *Ax,
                                 const int *A_diag, double *l, void *stream) {
  gbsym::PhaseRange phase_("gbsym_ilu0_device");
  if (n > 0 && (!Ap || !Ai || !Ax || !A_diag || !l)) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    ilu0_device(n, Ap, Ai, Ax, A_diag, l, (cudaStream_t)stream);
  });
}

extern "C" int gbsym_ic0_device(int n, double *val, const int *rowPtr, const int *rowIdx,
                                void *stream) {
  gbsym::PhaseRange phase_("gbsym_ic0_device");
  if (n > 0 && (!val || !rowPtr || !rowIdx)) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    ic0_device(n, val, rowPtr, rowIdx, (cudaStream_t)stream);
  });
}
