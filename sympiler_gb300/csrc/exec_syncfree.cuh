// exec_syncfree.cuh -- declarations shared by the SYNCFREE executor's host
// side (exec_syncfree.cu) and its kernels.  The kernels are compiled once
// per slab width, each width in its own translation unit (exec_sf_ks*.cu),
// so that the widths build in parallel.
#pragma once

#include "exec_common.cuh"

namespace gbsym {

constexpr int kSfBlock = 256;

// Warp units of `rpw` rows cut per level: unit u covers packed rows
// row[u] .. row[u] + cnt[u], all in one level.  Built once per rows-per-unit.
struct Units {
  const int *row, *cnt;
  int n;
};

Units sf_units(gbsym_tri_s *t, int rpw);

// The sweep of a plan whose slab is at most KS entries wide (KS >= t->K),
// into the sentinel-filled y; OV: the plan has rows longer than its slab.
// In place (b null) y is the plan's scratch copy and x receives every value
// as well; out of place y is x itself and the right-hand sides come from b.
template <class T, int KS, bool OV>
void sf_run_ks(gbsym_tri_s *t, T *x, T *y, const T *b, int k, cudaStream_t s);

// One right-hand side, in place, with look-through (exec_sf_lt.cu): plans
// whose rows all fit a slab of at most three entries.
inline bool sf_lookthrough_ok(const gbsym_tri_s *t) { return t->K <= 3 && t->nov == 0; }
template <class T>
void run_syncfree_lt(gbsym_tri_s *t, T *x, cudaStream_t s);
// k > 1 right-hand sides, in place, with look-through (exec_sf_lt.cu)
template <class T>
void run_syncfree_lt_mrhs(gbsym_tri_s *t, T *x, int k, cudaStream_t s);

}  // namespace gbsym
