// batch.cu -- many independent lower-triangular systems of uneven sizes in
// one executor pass.
//
// The systems are packed into one device pool as a block-diagonal triangle
// (system s occupies rows off[s] .. off[s+1]).  Rows of different systems
// never depend on each other, so the wavefront levels of the pool are the
// union of the systems' own levels: level l holds the level-l rows of every
// system still that deep.  One level-packed plan over the pool therefore
// solves all systems with max-depth launches (or one block sweep), each
// launch covering every system's work at that depth, instead of one solve
// per system.  Right-hand sides are the systems' row-major n_s x k blocks
// laid end to end, which is exactly the pool's row-major (sum n_s) x k.
#include <memory>
#include <vector>

#include "common.cuh"
#include "tri.cuh"

struct gbsym_batch_s {
  int nsys = 0;
  std::vector<long long> off;  // row offsets, nsys + 1
  std::unique_ptr<gbsym_tri_s> pool;
};

using namespace gbsym;

// Packs the systems into one block-diagonal pool on the device.  kind is
// GBSYM_LOWER_DIAG_LAST (lower CSR, diagonal last in each row) or
// GBSYM_LOWER_CSC (lower CSC, diagonal first in each column: the upper CSR
// an IC0 factor is computed in), which the pool plan transposes on the
// device as gbsym_tri_create does for one system.  Every column index is
// checked against its own system's size on the host while packing, so no
// entry can reach into another system.
static int batch_create(gbsym_batch *out, int nsys, const int *n, const int *const *Lp,
                        const int *const *Li, const double *const *Lx, int kind, int value_dtype,
                        void *stream) {
  if (!out || nsys < 0 || (nsys > 0 && (!n || !Lp || !Li || !Lx))) return GBSYM_ERR_NULL_ARG;
  *out = nullptr;
  if (kind != GBSYM_LOWER_DIAG_LAST && kind != GBSYM_LOWER_CSC) return GBSYM_ERR_UNSUPPORTED;
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    std::unique_ptr<gbsym_batch_s> b(new gbsym_batch_s());
    b->nsys = nsys;
    b->off.assign(nsys + 1, 0);
    long long nnz = 0;
    for (int q = 0; q < nsys; ++q) {
      GB_CHECK(n[q] >= 0 && (n[q] == 0 || (Lp[q] && Li[q] && Lx[q])), GBSYM_ERR_NULL_ARG);
      b->off[q + 1] = b->off[q] + n[q];
      if (n[q]) {
        GB_CHECK(Lp[q][0] == 0 && Lp[q][n[q]] >= 0, GBSYM_ERR_BAD_MATRIX);
        nnz += Lp[q][n[q]];
      }
    }
    GB_CHECK(b->off[nsys] < (1ll << 31) && nnz < (1ll << 31), GBSYM_ERR_SIZE);
    const int N = (int)b->off[nsys];
    std::vector<int> P(N + 1), I(nnz);
    std::vector<double> X(nnz);
    long long e = 0;
    for (int q = 0; q < nsys; ++q) {
      const int rows = n[q];
      const int base = (int)b->off[q];
      for (int r = 0; r < rows; ++r) {
        P[base + r] = (int)e;
        GB_CHECK(Lp[q][r] <= Lp[q][r + 1], GBSYM_ERR_BAD_MATRIX);
        for (int t = Lp[q][r]; t < Lp[q][r + 1]; ++t, ++e) {
          const int c = Li[q][t];
          GB_CHECK(c >= 0 && c < rows, GBSYM_ERR_BAD_MATRIX);
          I[e] = c + base;
          X[e] = Lx[q][t];
        }
      }
    }
    P[N] = (int)e;
    DBuf<int> dp, di;
    DBuf<double> dx;
    upload(dp, P.data(), N + 1, false, s);
    upload(di, I.data(), e, false, s);
    upload(dx, X.data(), e, false, s);
    gbsym_tri pool = nullptr;
    const int st = gbsym_tri_create(&pool, N, dp.p, di.p, dx.p, nullptr, kind, value_dtype, 1, nullptr,
                                    nullptr, 0, s);
    if (st != GBSYM_OK) throw Err{st};
    b->pool.reset(pool);
    GB_CUDA(cudaStreamSynchronize(s));  // the packed plan no longer needs the staging copies
    *out = b.release();
  });
}

extern "C" int gbsym_batch_create(gbsym_batch *out, int nsys, const int *n, const int *const *Lp,
                                  const int *const *Li, const double *const *Lx, int value_dtype,
                                  void *stream) {
  gbsym::PhaseRange phase_("gbsym_batch_create");
  return batch_create(out, nsys, n, Lp, Li, Lx, GBSYM_LOWER_DIAG_LAST, value_dtype, stream);
}

extern "C" int gbsym_batch_create_kind(gbsym_batch *out, int nsys, const int *n, const int *const *Lp,
                                       const int *const *Li, const double *const *Lx, int kind,
                                       int value_dtype, void *stream) {
  gbsym::PhaseRange phase_("gbsym_batch_create_kind");
  return batch_create(out, nsys, n, Lp, Li, Lx, kind, value_dtype, stream);
}

extern "C" int gbsym_batch_destroy(gbsym_batch b) {
  delete b;
  return GBSYM_OK;
}

extern "C" int gbsym_batch_solve(gbsym_batch b, void *x, int k, int dtype, void *stream) {
  gbsym::PhaseRange phase_("gbsym_batch_solve");
  if (!b || (!x && b->off.back() && k)) return GBSYM_ERR_NULL_ARG;
  if (k < 1) return GBSYM_ERR_SIZE;
  return guarded([&] {
    tri_solve_rowmajor(b->pool.get(), x, nullptr, k, dtype,
                       (cudaStream_t)stream);
  });
}

extern "C" int gbsym_batch_solve_host(gbsym_batch b, void *x, int k, int dtype) {
  gbsym::PhaseRange phase_("gbsym_batch_solve_host");
  if (!b || (!x && b->off.back() && k)) return GBSYM_ERR_NULL_ARG;
  if (k < 1) return GBSYM_ERR_SIZE;
  return guarded([&] { tri_solve_host_rowmajor(b->pool.get(), x, k, dtype); });
}

extern "C" int gbsym_batch_autotune(gbsym_batch b, int k, int dtype, void *stream, int *chosen) {
  gbsym::PhaseRange phase_("gbsym_batch_autotune");
  if (!b) return GBSYM_ERR_NULL_ARG;
  return gbsym_tri_autotune(b->pool.get(), k, dtype, stream, chosen);
}

extern "C" int gbsym_batch_check(gbsym_batch b, void *stream) {
  if (!b) return GBSYM_ERR_NULL_ARG;
  return gbsym_tri_check(b->pool.get(), stream);
}

extern "C" int gbsym_batch_get_info(gbsym_batch b, gbsym_tri_info *info) {
  if (!b) return GBSYM_ERR_NULL_ARG;
  return gbsym_tri_get_info(b->pool.get(), info);
}

extern "C" int gbsym_batch_get_tuning(gbsym_batch b, int k, int *tuning) {
  if (!b) return GBSYM_ERR_NULL_ARG;
  return gbsym_tri_get_tuning(b->pool.get(), k, tuning);
}

extern "C" int gbsym_batch_row_offsets(gbsym_batch b, long long *offsets) {
  if (!b || !offsets) return GBSYM_ERR_NULL_ARG;
  for (int q = 0; q <= b->nsys; ++q) offsets[q] = b->off[q];
  return GBSYM_OK;
}
