// krylov.cu -- IC0-preconditioned CG and ILU0-right-preconditioned
// restarted GMRES on the device.
//
// PCG follows Saad, Iterative Methods for Sparse Linear Systems (2nd ed.),
// Algorithm 9.1; the reference has no CG, but its IC-style solve pair
// (Cholesky::solve, sparse_blas/linear_solver/Cholesky.cpp:32-37: forward
// solve on L, then the transposed solve) is the preconditioner apply.
//
// GMRES follows pmgmres_ldlt_cr (sparse_blas/parsy/gmres/mgmres.cpp:
// 839-987): modified Gram-Schmidt Arnoldi, the re-orthogonalisation test
// (av + delta*h == av, delta = 1e-3), Givens rotations and back
// substitution on the small Hessenberg matrix (kept on the host), stop on
// |g[k+1]| <= tol * ||r0||.  It differs in two chosen ways: the system
// product is a general CSR SpMV (the nonsymmetric operator), and the ILU0
// preconditioner (lus_cr, mgmres.cpp:598-689) is applied on the right, in
// FP32 or FP64 as the factor plans store it.  All vector work is FP64.
//
// Dot products reduce in a fixed order (per-block partial sums, then one
// block), so a solve is deterministic run to run.
#include <chrono>
#include <cmath>
#include <memory>
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "csr.cuh"
#include "tri.cuh"

namespace gbsym {

constexpr int kRedThreads = 256;

static int red_blocks(long long n) { return std::max(1, std::min(div_up(n, 2048), num_sms() * 4)); }

__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  return v;
}

// partial[blockIdx] = sum a.b over this block's grid-stride range
__global__ void __launch_bounds__(kRedThreads)
k_dot_partial(long long n, const double *__restrict__ a, const double *__restrict__ b,
              double *__restrict__ partial) {
  __shared__ double sh[32];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s += a[i] * b[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Final reduction of m partials into out[0]; op selects what is stored:
// 0: sum; 1: sum and ratio out[1] = num[0] / sum (alpha = rz / pq);
// 2: sum and ratio out[1] = sum / den[0], then den[0] = sum (beta update).
__global__ void __launch_bounds__(kRedThreads)
k_reduce_final(int m, const double *__restrict__ partial, double *out, int op, double *aux) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) s += partial[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) {
    out[0] = s;
    if (op == 1) out[1] = aux[0] / s;
    if (op == 2) {
      out[1] = s / aux[0];
      aux[0] = s;
    }
  }
}

struct Reducer {
  DBuf<double> partial;
  int blocks = 0;
  void dot(long long n, const double *a, const double *b, double *out, int op, double *aux,
           cudaStream_t s) {
    blocks = red_blocks(n);
    partial.reserve(blocks);
    k_dot_partial<<<blocks, kRedThreads, 0, s>>>(n, a, b, partial.p);
    check_launch();
    k_reduce_final<<<1, kRedThreads, 0, s>>>(blocks, partial.p, out, op, aux);
    check_launch();
  }
};

// ---- PCG kernels ----------------------------------------------------------
// x += alpha p ; r -= alpha q ; partial ||r||^2
__global__ void __launch_bounds__(kRedThreads)
k_pcg_update(long long n, const double *__restrict__ alpha_ptr, const double *__restrict__ p,
             const double *__restrict__ q, double *__restrict__ x, double *__restrict__ r,
             double *__restrict__ partial) {
  __shared__ double sh[32];
  const double alpha = *alpha_ptr;
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    s += ri * ri;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// p = z + beta p
__global__ void k_pcg_p(long long n, const double *__restrict__ beta_ptr, const double *__restrict__ z,
                        double *__restrict__ p) {
  const double beta = *beta_ptr;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

// r = b - r
__global__ void k_residual(long long n, const double *__restrict__ b, double *__restrict__ r) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}

static int ew_blocks(long long n) { return std::max(1, std::min(div_up(n, 256), num_sms() * 8)); }

static void apply_ic0(gbsym_tri_s *L, gbsym_tri_s *Lt, double *z, cudaStream_t s) {
  tri_solve_rowmajor(L, z, nullptr, 1, GBSYM_F64, s);
  tri_solve_rowmajor(Lt, z, nullptr, 1, GBSYM_F64, s);
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// scalar slots
enum { S_BB = 0, S_RR, S_RZ, S_PQ, S_ALPHA, S_RZN, S_BETA, S_COUNT = 8 };

void pcg(gbsym_csr_s *A, gbsym_tri_s *L, gbsym_tri_s *Lt, const double *b, double *x, double tol,
         int maxit, gbsym_krylov_result *res, cudaStream_t s) {
  const int n = A->n;
  GB_CHECK(L->n == n && Lt->n == n, GBSYM_ERR_SIZE);
  const double t0 = now_s();
  DBuf<double> r(n), z(n), p(n), q(n), sc(S_COUNT);
  Reducer red;
  double *hs = nullptr;
  GB_CUDA(cudaMallocHost((void **)&hs, S_COUNT * sizeof(double)));
  std::unique_ptr<double, void (*)(double *)> hs_guard(hs, [](double *v) { cudaFreeHost(v); });
  const int eb = ew_blocks(n);
  // r = b - A x ; z = M^-1 r ; p = z
  csr_spmv(A, x, r.p, GBSYM_F64, s);
  k_residual<<<eb, 256, 0, s>>>(n, b, r.p);
  check_launch();
  red.dot(n, b, b, sc.p + S_BB, 0, nullptr, s);
  red.dot(n, r.p, r.p, sc.p + S_RR, 0, nullptr, s);
  GB_CUDA(cudaMemcpyAsync(z.p, r.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  apply_ic0(L, Lt, z.p, s);
  GB_CUDA(cudaMemcpyAsync(p.p, z.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  red.dot(n, r.p, z.p, sc.p + S_RZ, 0, nullptr, s);
  GB_CUDA(cudaMemcpyAsync(hs, sc.p, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  const double bnorm = hs[S_BB] > 0 ? std::sqrt(hs[S_BB]) : 1.0;
  double rel = std::sqrt(hs[S_RR]) / bnorm;
  int it = 0;
  while (rel > tol && it < maxit) {
    csr_spmv(A, p.p, q.p, GBSYM_F64, s);
    // pq -> S_PQ, alpha = rz / pq -> S_ALPHA
    red.dot(n, p.p, q.p, sc.p + S_PQ, 1, sc.p + S_RZ, s);
    k_pcg_update<<<red.blocks, kRedThreads, 0, s>>>(n, sc.p + S_ALPHA, p.p, q.p, x, r.p, red.partial.p);
    check_launch();
    k_reduce_final<<<1, kRedThreads, 0, s>>>(red.blocks, red.partial.p, sc.p + S_RR, 0, nullptr);
    check_launch();
    GB_CUDA(cudaMemcpyAsync(hs + S_RR, sc.p + S_RR, sizeof(double), cudaMemcpyDeviceToHost, s));
    // speculatively continue with the preconditioner while the norm travels
    GB_CUDA(cudaMemcpyAsync(z.p, r.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    apply_ic0(L, Lt, z.p, s);
    GB_CUDA(cudaStreamSynchronize(s));
    ++it;
    rel = std::sqrt(hs[S_RR]) / bnorm;
    if (rel <= tol) break;
    // rz_new -> S_RZN, beta = rz_new / rz -> S_BETA, rz = rz_new
    red.dot(n, r.p, z.p, sc.p + S_RZN, 2, sc.p + S_RZ, s);
    k_pcg_p<<<eb, 256, 0, s>>>(n, sc.p + S_BETA, z.p, p.p);
    check_launch();
  }
  GB_CUDA(cudaStreamSynchronize(s));
  // true residual in FP64
  csr_spmv(A, x, r.p, GBSYM_F64, s);
  k_residual<<<eb, 256, 0, s>>>(n, b, r.p);
  check_launch();
  red.dot(n, r.p, r.p, sc.p + S_RR, 0, nullptr, s);
  GB_CUDA(cudaMemcpyAsync(hs + S_RR, sc.p + S_RR, sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (res) {
    res->iterations = it;
    res->restarts = 0;
    res->relres = std::sqrt(hs[S_RR]) / bnorm;
    res->seconds = now_s() - t0;
    res->status = rel <= tol ? GBSYM_OK : GBSYM_ERR_NOT_CONVERGED;
  }
}

// ---- GMRES kernels ----------------------------------------------------------
// v = alpha * u
__global__ void k_scale(long long n, double alpha, const double *__restrict__ u, double *__restrict__ v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    v[i] = alpha * u[i];
}

// The sum of m block partials, as k_reduce_final forms it (same threads,
// same order), by the block that arrives last: every block publishes its
// partials, then takes a ticket; the block holding the last ticket reads
// them back through L2, stores the sums and resets the ticket for the next
// launch.  One launch instead of three, the same bits.
__device__ __forceinline__ void last_block_sums(int m, const double *pdot, double *out_dot, const double *pnorm,
                                                double *out_norm, unsigned *ticket, double *sh) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (out_dot) {
    double t = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) t += __ldcg(pdot + i);
    t = block_sum(t, sh);
    if (threadIdx.x == 0) out_dot[0] = t;
  }
  if (out_norm) {
    double t = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) t += __ldcg(pnorm + i);
    t = block_sum(t, sh);
    if (threadIdx.x == 0) out_norm[0] = t;
  }
  if (threadIdx.x == 0) *ticket = 0;
}

// One fused modified Gram-Schmidt pass over v, its reductions finished in
// the same launch:
//   if vprev: v -= h[jprev] * vprev  (the previous projection)
//   *out_dot  = v . vnext            (the next projection), if out_dot
//   *out_norm = v . v                (if out_norm)
__global__ void __launch_bounds__(kRedThreads)
k_mgs_pass_sum(long long n, double *__restrict__ v, const double *__restrict__ vprev,
               const double *__restrict__ hprev, const double *__restrict__ vnext, double *__restrict__ pdot,
               double *__restrict__ pnorm, double *out_dot, double *out_norm, unsigned *ticket) {
  __shared__ double sh[32];
  const double h = vprev ? *hprev : 0.0;
  double sd = 0.0, sn = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double vi = v[i];
    if (vprev) {
      vi = vi - h * vprev[i];
      v[i] = vi;
    }
    if (vnext) sd += vi * vnext[i];
    sn += vi * vi;
  }
  if (out_dot) {
    sd = block_sum(sd, sh);
    if (threadIdx.x == 0) pdot[blockIdx.x] = sd;
  }
  if (out_norm) {
    sn = block_sum(sn, sh);
    if (threadIdx.x == 0) pnorm[blockIdx.x] = sn;
  }
  last_block_sums(gridDim.x, pdot, out_dot, pnorm, out_norm, ticket, sh);
}

// w = sum_j y[j] V[j]
__global__ void k_combine(long long n, int m, const double *__restrict__ V, long long ld,
                          const double *__restrict__ y, double *__restrict__ w) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int j = 0; j < m; ++j) t += V[j * ld + i] * y[j];
    w[i] = t;
  }
}

__global__ void k_add(long long n, const double *__restrict__ a, double *__restrict__ x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] += a[i];
}

struct Precond {
  gbsym_tri_s *Lu, *U;
  DBuf<float> z32;
  void apply(const double *in, double *out, long long n, cudaStream_t s) {
    if (Lu->vdtype == GBSYM_F32) {
      z32.reserve(n);
      convert_f64_f32(in, z32.p, n, s);
      tri_solve_rowmajor(Lu, z32.p, nullptr, 1, GBSYM_F32, s);
      tri_solve_rowmajor(U, z32.p, nullptr, 1, GBSYM_F32, s);
      convert_f32_f64(z32.p, out, n, s);
    } else {
      if (in != out)
        GB_CUDA(cudaMemcpyAsync(out, in, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      tri_solve_rowmajor(Lu, out, nullptr, 1, GBSYM_F64, s);
      tri_solve_rowmajor(U, out, nullptr, 1, GBSYM_F64, s);
    }
  }
};

static void mult_givens(double c, double sn, int k, double *g) {
  const double g1 = c * g[k] - sn * g[k + 1];
  const double g2 = sn * g[k] + c * g[k + 1];
  g[k] = g1;
  g[k + 1] = g2;
}

void gmres(gbsym_csr_s *A, gbsym_tri_s *Lu, gbsym_tri_s *U, const double *b, double *x, int mr,
           int maxit, double tol, gbsym_krylov_result *res, cudaStream_t s) {
  const long long n = A->n;
  GB_CHECK(mr >= 1 && Lu->n == n && U->n == n && Lu->vdtype == U->vdtype, GBSYM_ERR_SIZE);
  const double t0 = now_s();
  const double delta = 1.0e-03;
  DBuf<double> V((size_t)(mr + 1) * n), r(n), w(n), sc(2 * (mr + 2)), dy(mr + 1);
  DBuf<double> pd, pn;
  DBuf<unsigned> ticket(1);
  Reducer red;
  Precond M{Lu, U, {}};
  const int blocks = red_blocks(n);
  pd.alloc(blocks);
  pn.alloc(blocks);
  GB_CUDA(cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), s));
  double *hs = nullptr;
  GB_CUDA(cudaMallocHost((void **)&hs, 2 * (mr + 2) * sizeof(double)));
  std::unique_ptr<double, void (*)(double *)> hs_guard(hs, [](double *v) { cudaFreeHost(v); });
  std::vector<double> H((size_t)(mr + 1) * mr), c(mr + 1), sn(mr + 1), g(mr + 1), y(mr + 1);
  auto Hm = [&](int i, int j) -> double & { return H[(size_t)i * mr + j]; };
  auto Vj = [&](int j) { return V.p + (size_t)j * n; };
  const int eb = ew_blocks(n);
  // ||b||
  red.dot(n, b, b, sc.p, 0, nullptr, s);
  GB_CUDA(cudaMemcpyAsync(hs, sc.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  const double bnorm = std::sqrt(hs[0]);
  int itr_used = 0, restarts = 0;
  double rho = 0.0, rho_tol = 0.0;
  bool converged = false, breakdown = false;
  for (int itr = 0; itr < maxit && !converged && !breakdown; ++itr) {
    csr_spmv(A, x, r.p, GBSYM_F64, s);
    k_residual<<<eb, 256, 0, s>>>(n, b, r.p);
    check_launch();
    red.dot(n, r.p, r.p, sc.p, 0, nullptr, s);
    GB_CUDA(cudaMemcpyAsync(hs, sc.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    rho = std::sqrt(hs[0]);
    if (itr == 0) rho_tol = rho * tol;
    if (rho <= rho_tol || rho == 0.0) {
      converged = true;
      break;
    }
    ++restarts;
    k_scale<<<eb, 256, 0, s>>>(n, 1.0 / rho, r.p, Vj(0));
    check_launch();
    g.assign(mr + 1, 0.0);
    g[0] = rho;
    std::fill(H.begin(), H.end(), 0.0);
    int k = 0, k_copy = 0;
    for (k = 0; k < mr; ++k) {
      k_copy = k;
      // v_{k+1} = A M^-1 v_k
      M.apply(Vj(k), w.p, n, s);
      csr_spmv(A, w.p, Vj(k + 1), GBSYM_F64, s);
      double *v = Vj(k + 1);
      // pass j (0..k): apply projection j-1, dot with v_j; pass k+1: apply
      // projection k, norm.  sc[j] <- h[j][k]; sc[k+1] <- ||v||^2 ;
      // sc[mr+1] <- ||v||^2 before orthogonalisation (av).
      for (int j = 0; j <= k + 1; ++j) {
        const double *vprev = j > 0 ? Vj(j - 1) : nullptr;
        const double *vnext = j <= k ? Vj(j) : nullptr;
        const bool norm = j == 0 || j == k + 1;
        k_mgs_pass_sum<<<blocks, kRedThreads, 0, s>>>(n, v, vprev, sc.p + (j > 0 ? j - 1 : 0), vnext, pd.p, pn.p,
                                                      vnext ? sc.p + j : nullptr,
                                                      norm ? sc.p + (j == 0 ? mr + 1 : k + 1) : nullptr, ticket.p);
        check_launch();
      }
      GB_CUDA(cudaMemcpyAsync(hs, sc.p, (mr + 2) * sizeof(double), cudaMemcpyDeviceToHost, s));
      GB_CUDA(cudaStreamSynchronize(s));
      const double av = std::sqrt(hs[mr + 1]);
      for (int j = 0; j <= k; ++j) Hm(j, k) = hs[j];
      Hm(k + 1, k) = std::sqrt(hs[k + 1]);
      if (av + delta * Hm(k + 1, k) == av) {
        // re-orthogonalise once more, accumulating into h
        for (int j = 0; j <= k + 1; ++j) {
          const double *vprev = j > 0 ? Vj(j - 1) : nullptr;
          const double *vnext = j <= k ? Vj(j) : nullptr;
          k_mgs_pass_sum<<<blocks, kRedThreads, 0, s>>>(n, v, vprev, sc.p + (j > 0 ? j - 1 : 0), vnext, pd.p,
                                                        pn.p, vnext ? sc.p + j : nullptr,
                                                        j == k + 1 ? sc.p + k + 1 : nullptr, ticket.p);
          check_launch();
        }
        GB_CUDA(cudaMemcpyAsync(hs, sc.p, (mr + 2) * sizeof(double), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
        for (int j = 0; j <= k; ++j) Hm(j, k) += hs[j];
        Hm(k + 1, k) = std::sqrt(hs[k + 1]);
      }
      if (Hm(k + 1, k) != 0.0) {
        k_scale<<<eb, 256, 0, s>>>(n, 1.0 / Hm(k + 1, k), v, v);
        check_launch();
      }
      if (k > 0) {
        for (int i = 0; i < k + 2; ++i) y[i] = Hm(i, k);
        for (int j = 0; j < k; ++j) mult_givens(c[j], sn[j], j, y.data());
        for (int i = 0; i < k + 2; ++i) Hm(i, k) = y[i];
      }
      const double mu = std::sqrt(Hm(k, k) * Hm(k, k) + Hm(k + 1, k) * Hm(k + 1, k));
      if (mu == 0.0) {  // the reference returns here without updating x
        breakdown = true;
        break;
      }
      c[k] = Hm(k, k) / mu;
      sn[k] = -Hm(k + 1, k) / mu;
      Hm(k, k) = c[k] * Hm(k, k) - sn[k] * Hm(k + 1, k);
      Hm(k + 1, k) = 0.0;
      mult_givens(c[k], sn[k], k, g.data());
      rho = std::fabs(g[k + 1]);
      ++itr_used;
      if (rho <= rho_tol) {
        converged = true;
        break;
      }
    }
    if (breakdown) break;
    k = std::min(k_copy, mr - 1);
    y[k] = g[k] / Hm(k, k);
    for (int i = k - 1; i >= 0; --i) {
      y[i] = g[i];
      for (int j = i + 1; j < k + 1; ++j) y[i] -= Hm(i, j) * y[j];
      y[i] /= Hm(i, i);
    }
    GB_CUDA(cudaMemcpyAsync(dy.p, y.data(), (k + 1) * sizeof(double), cudaMemcpyHostToDevice, s));
    k_combine<<<eb, 256, 0, s>>>(n, k + 1, V.p, n, dy.p, r.p);
    check_launch();
    M.apply(r.p, w.p, n, s);
    k_add<<<eb, 256, 0, s>>>(n, w.p, x);
    check_launch();
    GB_CUDA(cudaStreamSynchronize(s));  // y is reused on the host
  }
  // final FP64 residual
  csr_spmv(A, x, r.p, GBSYM_F64, s);
  k_residual<<<eb, 256, 0, s>>>(n, b, r.p);
  check_launch();
  red.dot(n, r.p, r.p, sc.p, 0, nullptr, s);
  GB_CUDA(cudaMemcpyAsync(hs, sc.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (res) {
    res->iterations = itr_used;
    res->restarts = restarts;
    res->relres = std::sqrt(hs[0]) / (bnorm > 0 ? bnorm : 1.0);
    res->seconds = now_s() - t0;
    res->status = converged ? GBSYM_OK : GBSYM_ERR_NOT_CONVERGED;
  }
}

}  // namespace gbsym

using namespace gbsym;

extern "C" int gbsym_pcg(gbsym_csr A, gbsym_tri L, gbsym_tri Lt, const double *b, double *x,
                         double tol, int maxit, gbsym_krylov_result *res, void *stream) {
  if (!A || !L || !Lt || (A->n && (!b || !x))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    pcg(A, L, Lt, b, x, tol, maxit, res, (cudaStream_t)stream);
  });
}

extern "C" int gbsym_gmres(gbsym_csr A, gbsym_tri Lu, gbsym_tri U, const double *b, double *x,
                           int mr, int maxit, double tol, gbsym_krylov_result *res, void *stream) {
  if (!A || !Lu || !U || (A->n && (!b || !x))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    gmres(A, Lu, U, b, x, mr, maxit, tol, res, (cudaStream_t)stream);
  });
}
