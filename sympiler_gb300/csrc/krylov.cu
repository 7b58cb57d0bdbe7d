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
// substitution on the small Hessenberg matrix, stop on |g[k+1]| <= tol *
// ||r0||.  All of it runs on the device: each Gram-Schmidt round is one
// cooperative launch, the Hessenberg column, the re-orthogonalisation
// decision, the rotations and the back substitution are single-thread
// kernels, and the host reads each step's residual estimate one step late
// (gmres() below).  It differs in two chosen ways: the system
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
  cudaEvent_t rr_ready = nullptr;
  GB_CUDA(cudaEventCreateWithFlags(&rr_ready, cudaEventDisableTiming));
  std::unique_ptr<CUevent_st, void (*)(cudaEvent_t)> ev_guard(rr_ready, [](cudaEvent_t e) { cudaEventDestroy(e); });
  while (rel > tol && it < maxit) {
    csr_spmv(A, p.p, q.p, GBSYM_F64, s);
    // pq -> S_PQ, alpha = rz / pq -> S_ALPHA
    red.dot(n, p.p, q.p, sc.p + S_PQ, 1, sc.p + S_RZ, s);
    k_pcg_update<<<red.blocks, kRedThreads, 0, s>>>(n, sc.p + S_ALPHA, p.p, q.p, x, r.p, red.partial.p);
    check_launch();
    k_reduce_final<<<1, kRedThreads, 0, s>>>(red.blocks, red.partial.p, sc.p + S_RR, 0, nullptr);
    check_launch();
    GB_CUDA(cudaMemcpyAsync(hs + S_RR, sc.p + S_RR, sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaEventRecord(rr_ready, s));
    // continue with the preconditioner while the norm travels; the host
    // waits only for the norm, so the GPU keeps working on the two sweeps
    // while the host checks it and queues the rest of the iteration
    GB_CUDA(cudaMemcpyAsync(z.p, r.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    apply_ic0(L, Lt, z.p, s);
    GB_CUDA(cudaEventSynchronize(rr_ready));
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

// ---- one whole Gram-Schmidt round in one cooperative launch --------------
// The passes of a round depend on each other only through their dot
// products, so instead of one launch per pass (and a kernel boundary
// between passes) one launch runs them all: after a pass every block
// publishes its partial sums, meets the others at a grid barrier, and sums
// all partials itself in the same fixed order as k_reduce_final (so every
// block holds the same bits).  Partials alternate between two buffers, so a block
// that runs ahead into pass j+1 never overwrites a partial a slower block
// still reads for pass j (all blocks have read pass j's before any can
// pass barrier j+1).
__device__ __forceinline__ unsigned ld_acquire_b32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Bounded grid barrier on a counter that only grows (wrap-around compare);
// false (and GBSYM_ERR_TIMEOUT in err) when the wait ran out.
__device__ __forceinline__ bool gs_barrier(unsigned *bar, unsigned target, int *err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    int ok = 1;
    long long it = 0;
    const unsigned long long t0 = globaltimer_ns();
    while ((int)(ld_acquire_b32(bar) - target) < 0) {
      ++it;
      if (it > kWaitLimitIters || ((it & 255) == 0 && globaltimer_ns() - t0 > kWaitLimitNs) ||
          ((it & 255) == 0 && ld_relaxed(err) != 0)) {
        atomicCAS(err, 0, GBSYM_ERR_TIMEOUT);
        ok = 0;
        break;
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The sum of m partials in k_reduce_final's order, broadcast to the block.
__device__ __forceinline__ double all_sum(int m, const double *p, double *sh, double *bcast) {
  double t = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) t += __ldcg(p + i);
  t = block_sum(t, sh);
  if (threadIdx.x == 0) *bcast = t;
  __syncthreads();
  t = *bcast;
  __syncthreads();
  return t;
}

// Round of Arnoldi step k over v = V_{k+1} (V's columns ld apart):
// pass j = 0..k applies projection j-1 (with the dot of pass j-1) and
// takes the dot with V_j into sc[j]; pass k+1 applies projection k and
// takes ||v||^2 into sc[k+1].  The first round also stores ||v||^2 before
// any projection into sc[mr+1].  A second round (re-orthogonalisation)
// runs only when *run_if is set; otherwise block 0 advances the barrier
// counter by the arrivals the round would have made, and all return.
constexpr int kMgsThreads = 256;

__global__ void __launch_bounds__(kMgsThreads)
k_mgs_round(long long n, double *V, long long ld, int k, int mr, double *sc, int second,
            const int *run_if, double *part, unsigned *bar, unsigned base, int *err) {
  __shared__ double sh[32];
  __shared__ double bc;
  if (run_if && *run_if == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(bar, (unsigned)(k + 2) * gridDim.x);
    return;
  }
  double *v = V + (size_t)(k + 1) * ld;
  const int m = gridDim.x;
  double h = 0.0;
  for (int j = 0; j <= k + 1; ++j) {
    const double *vprev = j > 0 ? V + (size_t)(j - 1) * ld : nullptr;
    const double *vnext = j <= k ? V + (size_t)j * ld : nullptr;
    const bool want_norm = second ? j == k + 1 : (j == 0 || j == k + 1);
    double sd = 0.0, sn = 0.0;
    // the thread's elements i, i + S, i + 2S, ... in that order (so the
    // sums are those of a plain grid-stride loop), four at a time with all
    // their loads issued before the first store: the stores to v would
    // otherwise keep every load of the next element behind them, one
    // memory round trip per element
    constexpr int U = 4;
    const long long S = (long long)gridDim.x * blockDim.x;
    for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n; i0 += U * S) {
      double a[U], p[U], q[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long i = i0 + u * S;
        if (i < n) {
          a[u] = v[i];
          if (vprev) p[u] = vprev[i];
          if (vnext) q[u] = vnext[i];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long i = i0 + u * S;
        if (i < n) {
          double vi = a[u];
          if (vprev) {
            vi = vi - h * p[u];
            v[i] = vi;
          }
          if (vnext) sd += vi * q[u];
          if (want_norm) sn += vi * vi;  // only the passes that report a norm pay for it
        }
      }
    }
    double *pd = part + (size_t)(j & 1) * 2 * m, *pn = pd + m;
    if (vnext) {
      sd = block_sum(sd, sh);
      if (threadIdx.x == 0) pd[blockIdx.x] = sd;
    }
    if (want_norm) {
      sn = block_sum(sn, sh);
      if (threadIdx.x == 0) pn[blockIdx.x] = sn;
    }
    if (!gs_barrier(bar, base + (unsigned)(j + 1) * m, err)) return;
    if (vnext) {
      h = all_sum(m, pd, sh, &bc);
      if (blockIdx.x == 0 && threadIdx.x == 0) sc[j] = h;
    }
    if (want_norm) {
      const double t = all_sum(m, pn, sh, &bc);
      if (blockIdx.x == 0 && threadIdx.x == 0) sc[second || j == k + 1 ? k + 1 : mr + 1] = t;
    }
  }
}

// v = alpha[0] * v, alpha read on the device
__global__ void k_scale_by(long long n, const double *__restrict__ alpha, double *__restrict__ v) {
  const double a = *alpha;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    v[i] = a * v[i];
}

// ---- the small Hessenberg problem, on the device ---------------------------
// One thread; at most mr + 1 = 31 rows.  Every product and sum is rounded
// separately (no contraction), as the reference's host code computes it.
//
// State (doubles): H[(mr+1) x mr] row-major, c[mr+1], sn[mr+1], g[mr+1],
// y[mr+1], then the per-step words below.
enum { GW_SCALE = 0, GW_RHO, GW_CONV, GW_BREAK, GW_COUNT };
constexpr int kGmresMaxRestart = 1024;

struct GmresState {
  double *H, *c, *sn, *g, *y, *w;  // w: GW_COUNT words
  int *reorth;                     // re-orthogonalise this step (0/1)
  int mr;
};

__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }

// After the first Gram-Schmidt round of step k: column k of H from the
// dots, and the re-orthogonalisation test av + delta * h(k+1,k) == av
// (mgmres.cpp:901-925).
__global__ void k_gm_column(GmresState st, int k, const double *__restrict__ sc, double delta) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int mr = st.mr;
  const double av = sqrt(sc[mr + 1]);
  for (int j = 0; j <= k; ++j) st.H[j * mr + k] = sc[j];
  const double h = sqrt(sc[k + 1]);
  st.H[(k + 1) * mr + k] = h;
  *st.reorth = add_(av, mul_(delta, h)) == av ? 1 : 0;
}

// After the (possibly skipped) second round: its dots added to column k,
// the scale of v_{k+1}, the earlier rotations applied to column k, the new
// rotation (mgmres.cpp:927-958, mult_givens 186-251), |g[k+1]| and the
// convergence and breakdown words.  The block first loads everything the
// step reads into shared memory (one round trip instead of one per value
// on the single thread's dependent chain); thread 0 then computes.
// Dynamic shared memory: 3(k+2) + 2k doubles.
__global__ void k_gm_givens(GmresState st, int k, const double *__restrict__ sc, double rho_tol) {
  extern __shared__ double gsh[];
  const int mr = st.mr;
  double *col = gsh, *ad = col + (k + 2), *cs = ad + (k + 2), *sns = cs + k, *gg = sns + k;
  const bool reo = *st.reorth != 0;
  for (int j = threadIdx.x; j <= k + 1; j += blockDim.x) {
    col[j] = st.H[j * mr + k];
    ad[j] = reo ? sc[j] : 0.0;
  }
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    cs[j] = st.c[j];
    sns[j] = st.sn[j];
  }
  if (threadIdx.x < 2) gg[threadIdx.x] = st.g[k + threadIdx.x];
  __syncthreads();
  if (threadIdx.x == 0) {
    if (reo) {
      for (int j = 0; j <= k; ++j) col[j] = add_(col[j], ad[j]);
      col[k + 1] = sqrt(ad[k + 1]);
    }
    const double hn = col[k + 1];
    st.w[GW_SCALE] = hn != 0.0 ? 1.0 / hn : 1.0;
    for (int j = 0; j < k; ++j) {
      const double a = col[j], b = col[j + 1];
      col[j] = sub_(mul_(cs[j], a), mul_(sns[j], b));
      col[j + 1] = add_(mul_(sns[j], a), mul_(cs[j], b));
    }
    const double mu = sqrt(add_(mul_(col[k], col[k]), mul_(col[k + 1], col[k + 1])));
    if (mu == 0.0) {
      st.w[GW_BREAK] = 1.0;
      st.w[GW_CONV] = 0.0;
    } else {
      const double ck = col[k] / mu, sk = -col[k + 1] / mu;
      st.c[k] = ck;
      st.sn[k] = sk;
      col[k] = sub_(mul_(ck, col[k]), mul_(sk, col[k + 1]));
      col[k + 1] = 0.0;
      const double g1 = sub_(mul_(ck, gg[0]), mul_(sk, gg[1]));
      const double g2 = add_(mul_(sk, gg[0]), mul_(ck, gg[1]));
      st.g[k] = g1;
      st.g[k + 1] = g2;
      const double rho = fabs(g2);
      st.w[GW_RHO] = rho;
      st.w[GW_CONV] = rho <= rho_tol ? 1.0 : 0.0;
      st.w[GW_BREAK] = 0.0;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j <= k + 1; j += blockDim.x) st.H[j * mr + k] = col[j];
}

// Restart set-up: g = rho e_1 (mgmres.cpp:878-886); H, c, sn need no
// clearing (every entry is written before it is read).
__global__ void k_gm_start(GmresState st, const double *__restrict__ rr) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i <= st.mr; ++i) st.g[i] = 0.0;
  st.g[0] = sqrt(rr[0]);
}

// Back substitution on the rotated H (mgmres.cpp:960-972) into y[0..k].
// With `staged`, the block first copies H's leading (k+1) x (k+1) block and
// g into shared memory ((k+1)(k+2) doubles of dynamic shared memory), so
// thread 0's dependent chain reads no global memory.
__global__ void k_gm_backsub(GmresState st, int k, int staged) {
  extern __shared__ double bsh[];
  const int mr = st.mr, w = k + 1;
  if (staged) {
    for (int t = threadIdx.x; t < w * w; t += blockDim.x) bsh[t] = st.H[(t / w) * mr + t % w];
    for (int t = threadIdx.x; t < w; t += blockDim.x) bsh[w * w + t] = st.g[t];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  auto Hm = [&](int i, int j) { return staged ? bsh[i * w + j] : st.H[i * mr + j]; };
  auto g = [&](int i) { return staged ? bsh[w * w + i] : st.g[i]; };
  st.y[k] = g(k) / Hm(k, k);
  for (int i = k - 1; i >= 0; --i) {
    double t = g(i);
    for (int j = i + 1; j < k + 1; ++j) t = sub_(t, mul_(Hm(i, j), st.y[j]));
    st.y[i] = t / Hm(i, i);
  }
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

// GMRES(mr) with the Arnoldi step's small problem on the device.  Per step
// k the host only launches: the preconditioner and the SpMV, the Gram-
// Schmidt passes (the second round's passes run only when k_gm_column asked
// for them), k_gm_givens and the scaling of v_{k+1}; then it copies step
// k's three words (rho, converged, breakdown) to pinned memory.  The host
// reads step k-1's words after launching step k, so the GPU never waits for
// the host inside a restart cycle; when step k-1 has converged the already
// queued step k does no harm (it touches H's column k, g[k+1..k+2] and
// v_{k+1}, none of which the back substitution of step k-1 reads) and its
// time is the cost of the one-step lag.
void gmres(gbsym_csr_s *A, gbsym_tri_s *Lu, gbsym_tri_s *U, const double *b, double *x, int mr,
           int maxit, double tol, gbsym_krylov_result *res, cudaStream_t s) {
  const long long n = A->n;
  GB_CHECK(mr >= 1 && Lu->n == n && U->n == n && Lu->vdtype == U->vdtype, GBSYM_ERR_SIZE);
  // the rotation step stages column k in shared memory (5 mr + 6 doubles)
  GB_CHECK(mr <= kGmresMaxRestart, GBSYM_ERR_UNSUPPORTED);
  const double t0 = now_s();
  const double delta = 1.0e-03;
  DBuf<double> V((size_t)(mr + 1) * n), r(n), w(n), sc(2 * (mr + 2));
  DBuf<double> st_buf((size_t)(mr + 1) * mr + 4 * (mr + 1) + GW_COUNT);
  DBuf<int> reorth(1);
  Reducer red;
  Precond M{Lu, U, {}};
  const int blocks = red_blocks(n);
  GmresState st;
  st.H = st_buf.p;
  st.c = st.H + (size_t)(mr + 1) * mr;
  st.sn = st.c + (mr + 1);
  st.g = st.sn + (mr + 1);
  st.y = st.g + (mr + 1);
  st.w = st.y + (mr + 1);
  st.reorth = reorth.p;
  st.mr = mr;
  // pinned words: [0] the residual norm^2 of a restart, then GW_COUNT per step
  double *hs = nullptr;
  const size_t hwords = 1 + (size_t)GW_COUNT * mr;
  GB_CUDA(cudaMallocHost((void **)&hs, hwords * sizeof(double)));
  std::unique_ptr<double, void (*)(double *)> hs_guard(hs, [](double *v) { cudaFreeHost(v); });
  std::vector<cudaEvent_t> ev(mr, nullptr);
  struct EvGuard {
    std::vector<cudaEvent_t> &e;
    ~EvGuard() {
      for (auto x : e)
        if (x) cudaEventDestroy(x);
    }
  } ev_guard{ev};
  for (auto &e : ev) GB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
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
  // one Gram-Schmidt round over v = v_{k+1}: pass j (0..k) applies
  // projection j-1 and dots with v_j, pass k+1 applies projection k and
  // takes the norm.  First round: sc[j] <- h[j][k], sc[k+1] <- ||v||^2,
  // sc[mr+1] <- ||v||^2 before orthogonalisation (av).  Second round (only
  // if k_gm_column set the flag): the same without av.
  // the round's passes run in one cooperative launch (k_mgs_round); its
  // grid barrier counts arrivals on gbar, whose expected value the host
  // tracks in `base`
  int rs_per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rs_per_sm, k_mgs_round, kMgsThreads, 0));
  GB_CHECK(rs_per_sm >= 1, GBSYM_ERR_UNSUPPORTED);
  // two blocks per SM: the round's grid barriers cost more with more blocks
  // and its streaming needs enough of them (C3 GMRES, FP32 preconditioner:
  // 0.1378 / 0.1258 / 0.1278 / 0.1353 s at 1 / 2 / 4 / 8 blocks per SM)
  const int rblocks = std::max(1, std::min(blocks, std::min(rs_per_sm, 2) * num_sms()));
  DBuf<double> part(4 * (size_t)rblocks);
  DBuf<unsigned> gbar(1);
  DBuf<int> gerr(1);
  GB_CUDA(cudaMemsetAsync(gbar.p, 0, sizeof(unsigned), s));
  GB_CUDA(cudaMemsetAsync(gerr.p, 0, sizeof(int), s));
  unsigned base = 0;
  auto mgs_round = [&](int k, bool second) {
    long long nn = n, ld = n;
    double *Vp = V.p, *scp = sc.p, *partp = part.p;
    int kk = k, mrr = mr, sec = second ? 1 : 0;
    const int *run_if = second ? reorth.p : nullptr;
    unsigned *barp = gbar.p;
    int *errp = gerr.p;
    void *args[] = {&nn, &Vp, &ld, &kk, &mrr, &scp, &sec, &run_if, &partp, &barp, &base, &errp};
    GB_CUDA(cudaLaunchCooperativeKernel((const void *)k_mgs_round, dim3(rblocks), dim3(kMgsThreads), args, 0, s));
    check_launch();
    base += (unsigned)(k + 2) * rblocks;
  };
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
    k_gm_start<<<1, 32, 0, s>>>(st, sc.p);
    check_launch();
    int k_last = -1;    // last step launched
    int k_stop = -1;    // step that converged, or -1
    int k_break = -1;   // step that broke down, or -1
    auto inspect = [&](int k) {
      GB_CUDA(cudaEventSynchronize(ev[k]));
      const double *hw = hs + 1 + (size_t)GW_COUNT * k;
      if (hw[GW_BREAK] != 0.0) k_break = k;
      else if (hw[GW_CONV] != 0.0) k_stop = k;
      if (hw[GW_BREAK] == 0.0) rho = hw[GW_RHO];
    };
    for (int k = 0; k < mr; ++k) {
      // v_{k+1} = A M^-1 v_k
      M.apply(Vj(k), w.p, n, s);
      csr_spmv(A, w.p, Vj(k + 1), GBSYM_F64, s);
      mgs_round(k, false);
      k_gm_column<<<1, 32, 0, s>>>(st, k, sc.p, delta);
      check_launch();
      mgs_round(k, true);
      k_gm_givens<<<1, 32, (size_t)(5 * k + 6) * sizeof(double), s>>>(st, k, sc.p, rho_tol);
      check_launch();
      k_scale_by<<<eb, 256, 0, s>>>(n, st.w + GW_SCALE, Vj(k + 1));
      check_launch();
      GB_CUDA(cudaMemcpyAsync(hs + 1 + (size_t)GW_COUNT * k, st.w, GW_COUNT * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
      GB_CUDA(cudaEventRecord(ev[k], s));
      k_last = k;
      if (k > 0) {
        inspect(k - 1);  // step k is queued behind it
        if (k_stop >= 0 || k_break >= 0) break;
      }
    }
    if (k_stop < 0 && k_break < 0) inspect(k_last);
    if (k_break >= 0) {  // the reference returns here without updating x
      itr_used += k_break;
      breakdown = true;
      break;
    }
    const int kk = k_stop >= 0 ? k_stop : k_last;
    itr_used += kk + 1;
    if (k_stop >= 0) converged = true;
    {
      const size_t bs = (size_t)(kk + 1) * (kk + 2) * sizeof(double);
      const bool staged = bs <= 48 * 1024;
      k_gm_backsub<<<1, 256, staged ? bs : 0, s>>>(st, kk, staged ? 1 : 0);
    }
    check_launch();
    k_combine<<<eb, 256, 0, s>>>(n, kk + 1, V.p, n, st.y, r.p);
    check_launch();
    M.apply(r.p, w.p, n, s);
    k_add<<<eb, 256, 0, s>>>(n, w.p, x);
    check_launch();
  }
  // final FP64 residual
  csr_spmv(A, x, r.p, GBSYM_F64, s);
  k_residual<<<eb, 256, 0, s>>>(n, b, r.p);
  check_launch();
  red.dot(n, r.p, r.p, sc.p, 0, nullptr, s);
  GB_CUDA(cudaMemcpyAsync(hs, sc.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  int werr = 0;
  GB_CUDA(cudaMemcpyAsync(&werr, gerr.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (werr) throw Err{werr};  // a Gram-Schmidt barrier gave up
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
  gbsym::PhaseRange phase_("gbsym_pcg");
  if (!A || !L || !Lt || (A->n && (!b || !x))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    pcg(A, L, Lt, b, x, tol, maxit, res, (cudaStream_t)stream);
  });
}

extern "C" int gbsym_gmres(gbsym_csr A, gbsym_tri Lu, gbsym_tri U, const double *b, double *x,
                           int mr, int maxit, double tol, gbsym_krylov_result *res, void *stream) {
  gbsym::PhaseRange phase_("gbsym_gmres");
  if (!A || !Lu || !U || (A->n && (!b || !x))) return GBSYM_ERR_NULL_ARG;
  return guarded([&] {
    gmres(A, Lu, U, b, x, mr, maxit, tol, res, (cudaStream_t)stream);
  });
}
