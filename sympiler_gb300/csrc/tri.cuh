// tri.cuh -- the level-packed triangle (gbsym_tri) shared by the solve,
// Krylov, adjoint and batched translation units.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "common.cuh"

namespace gbsym {

// Device view of a level-packed triangle in sliced-ELL form.
//
// Packed row k is original row perm[k]; rows of level l occupy packed
// positions lev_ptr[l] .. lev_ptr[l+1].  Row k has len[k] off-diagonal
// entries, in the caller's storage order: the first min(len, K) of them
// sit in a column-interleaved slab (entry q of row k at sci/sv[q*npad + k],
// so a warp reading entry q of 32 consecutive rows reads one contiguous
// run), the rest in an overflow CSR at ovp[k] (entry q >= K at
// oci/ov[ovp[k] + q - K]).  Column indices keep the ORIGINAL numbering, so
// x is addressed in the caller's order.  dg[k] is the row's divisor; dg is
// null for a unit triangle; rc[k] = RN(1 / dg[k]).  Every static load of a row is independent of
// the others (no row-pointer indirection for the slab), which is what lets
// a level kernel finish them before it waits on the previous level.
constexpr int kSlabMax = 8;

template <class T>
struct TriView {
  int K;     // slab width, 0 .. kSlabMax
  int npad;  // slab stride (>= n)
  const int *__restrict__ perm;
  const int *__restrict__ len;
  const int *__restrict__ sci;
  const T *__restrict__ sv;
  const int *__restrict__ ovp;  // null when no row overflows
  const int *__restrict__ oci;
  const T *__restrict__ ov;
  const T *__restrict__ dg;
  const T *__restrict__ rc;  // RN(1/dg), for the exact Markstein division
};

// Internal kinds used only by the schedule builders: every stored entry on
// the dependency side of the diagonal is a dependency, wherever it sits in
// the row, and the diagonal need not be present.
constexpr int kKindStrictLower = 100;
constexpr int kKindStrictUpper = 101;

inline bool kind_is_upper(int kind) {
  return kind == GBSYM_UPPER_DIAG_FIRST || kind == GBSYM_ILU_UPPER || kind == kKindStrictUpper;
}
inline bool kind_is_unit(int kind) { return kind == GBSYM_ILU_UNIT_LOWER; }

struct GraphEntry {
  const void *x = nullptr;
  const void *b = nullptr;
  int k = 0, dtype = 0, exec = 0;
  cudaGraphExec_t exec_graph = nullptr;
  unsigned long long nodes = 0;
  unsigned long long stamp = 0;
};

}  // namespace gbsym

struct gbsym_tri_s {
  int n = 0;
  int nlev = 0;
  int kind = 0;
  int vdtype = GBSYM_F64;
  long long nnz_off = 0;
  int max_level_rows = 0;
  int exec = GBSYM_EXEC_LEVELSET;       // chosen executor for k = 1
  int exec_mrhs = GBSYM_EXEC_LEVELSET;  // chosen executor for k > 1
  int exec_forced = GBSYM_EXEC_AUTO;
  int persist_blocks = 0;               // cap on the persistent grid (0: none)
  int cluster_blocks = 0;               // cap on blocks per cluster (0: none)
  std::vector<int> h_lev_ptr;        // packed level boundaries (host copy)
  int K = 0, npad = 0;               // slab width and stride
  long long nov = 0;                 // overflow entries
  gbsym::DBuf<int> lev_ptr, perm, len, sci, ovp, oci;
  gbsym::DBuf<int> scp, ocp;         // sci / oci in packed-row numbering (sync-free scratch order)
  gbsym::DBuf<double> sv64, ov64, dg64, rc64;
  gbsym::DBuf<float> sv32, ov32, dg32, rc32;
  int arith = GBSYM_ARITH_EXACT;      // GBSYM_ARITH_EXACT or GBSYM_ARITH_FUSED
  gbsym::DBuf<int> err;              // device error word(s): code, where
  gbsym::DBuf<unsigned> bar;         // grid-barrier arrival counter
  gbsym::DBuf<char> sfy;             // sync-free published values (sentinel-filled)
  gbsym::DBuf<char> sfb;             // look-through sweep: right-hand side in packed order
  struct SfUnits {
    int rpw = 0, n = 0;
    gbsym::DBuf<int> row, cnt;       // level-aligned warp units
  };
  std::vector<SfUnits> sf_units;
  int sf_blocks_per_sm = 0;          // sync-free grid, forced for every k (0: default)
  int sf_bps_tuned[2] = {0, 0};      // sync-free blocks per SM the autotuner chose, k = 1 and k > 1 (0: default)
  int sf_alt_lanes = 0;              // k > 1, 1: the other lane layout (FP64: two values per
                                     // lane; FP32: two), the autotuner's choice
  int sf_deal = 0;                   // sync-free unit dealing: SM count to spread over (0: plain order)
  int sf_lookthrough = 1;            // k = 1: spare lanes recompute each row's dependencies (1),
                                     // and theirs (2), so rows wait two (three) levels back
                                     // (exec_sf_lt.cu); plans whose rows fit a three-entry slab;
                                     // 0: the plain sweep
  int sf_lt_mrhs = 0;                // k > 1: the look-through sweep for several right-hand
                                     // sides (the autotuner's choice; in place only)
  struct PartPlan {
    int R = 0, nparts = 0, ngroups = 0;  // rows per partition (0: not built)
    gbsym::DBuf<int> part_group, group_ptr, rows;
  };
  PartPlan part;                     // partitioned executor's schedule
  int part_rows_pref = 0;            // partition size (0: default)
  gbsym::DBuf<char> scratch;         // layout-conversion scratch
  gbsym::DBuf<char> io;              // device copy for host-memory solves
  cudaStream_t cap_stream = nullptr; // private stream for graph capture
  std::vector<gbsym::GraphEntry> graphs;
  unsigned long long graph_clock = 0;

  gbsym::TriView<double> view64() const {
    return {K, npad, perm.p, len.p, sci.p, sv64.p, nov ? ovp.p : nullptr, oci.p, ov64.p,
            kind == GBSYM_ILU_UNIT_LOWER ? nullptr : dg64.p, rc64.p};
  }
  gbsym::TriView<float> view32() const {
    return {K, npad, perm.p, len.p, sci.p, sv32.p, nov ? ovp.p : nullptr, oci.p, ov32.p,
            kind == GBSYM_ILU_UNIT_LOWER ? nullptr : dg32.p, rc32.p};
  }
  // The same views with dependency columns in packed-row numbering.
  gbsym::TriView<double> view64_packed() const {
    gbsym::TriView<double> v = view64();
    v.sci = scp.p;
    v.oci = ocp.p;
    return v;
  }
  gbsym::TriView<float> view32_packed() const {
    gbsym::TriView<float> v = view32();
    v.sci = scp.p;
    v.oci = ocp.p;
    return v;
  }
  ~gbsym_tri_s();
};

namespace gbsym {
// Solve on device memory, row-major n x k (k >= 1), in place.  b non-null
// selects the "redundant" row formula (k == 1, FP64 only).
void tri_solve_rowmajor(gbsym_tri_s *t, void *x, const void *b, int k, int dtype,
                        cudaStream_t s);
// Row-major host memory (FP64 or FP32 as the plan), in place over the
// CPU-GPU link where the buffer allows it, else staged; synchronises.
void tri_solve_host_rowmajor(gbsym_tri_s *t, void *x, int k, int dtype);
// Out of place on device memory, row-major n x k: x = L^-1 b, b unchanged
// (b and x must not overlap).
void tri_solve_into(gbsym_tri_s *t, const void *b, void *x, int k, int dtype, cudaStream_t s);
// Executor selection (exec.cu).
void choose_exec(gbsym_tri_s *t);
int effective_exec(const gbsym_tri_s *t, int k, bool redundant);
// Synchronises s and returns (and clears) the plan's sticky device error.
int tri_read_error(gbsym_tri_s *t, cudaStream_t s);
// Build a plan from device arrays (validates matrix and schedule).
gbsym_tri_s *tri_build(int n, const int *d_p, const int *d_i, const double *d_x,
                       const int *d_diags, int kind, int vdtype,
                       const int *h_level_ptr, const int *d_level_set, int levels,
                       cudaStream_t s);
// Sync-free level computation on device arrays: returns the level count,
// fills d_level_ptr (levels+1) and d_level_set (n).  Used by the plan and
// by the schedule-builder drop-ins.
int build_levels_device(int n, const int *d_p, const int *d_i, const int *d_diags,
                        int kind, DBuf<int> &d_level_ptr, DBuf<int> &d_level_set,
                        cudaStream_t s);
// Transpose of a square CSR pattern: for every entry e (row r, col c) of the
// input, output row c lists (col r, src e) with r ascending.
struct Transposed {
  DBuf<int> rp, ci, src;
};
void transpose_pattern(int n, int nnz, const int *p, const int *ci, Transposed &out,
                       cudaStream_t s);
// Incomplete factorisations on device arrays (factor.cu).
void ilu0_device(int n, const int *Ap, const int *Ai, const double *Ax, const int *A_diag,
                 double *l, cudaStream_t s);
void ic0_device(int n, double *val, const int *up, const int *ui, cudaStream_t s);
// Checks that (p, i, diags) is a well-formed triangle of the given kind.
void validate_matrix(int n, const int *d_p, const int *d_i, const int *d_diags,
                     int kind, cudaStream_t s);
// Checks an LBC schedule (coarse levels -> partitions -> rows) against the
// DAG of the triangle: every dependency of a row lies in an earlier coarse
// level or earlier in the same partition.
void validate_lbc(int n, const int *d_p, const int *d_i, const int *d_diags, int kind,
                  int level_no, const int *h_level_ptr, const int *h_par_ptr,
                  const int *h_partition, cudaStream_t s);
}  // namespace gbsym
