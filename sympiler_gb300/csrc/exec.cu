// exec.cu -- executor dispatch, default choice and the autotuner.
//
// The reference has one executor per schedule kind and a fixed OpenMP
// thread count (sptrsv_demo.cpp:36-65).  Here five GPU executors run any
// level-packed plan (exec_level.cu, exec_sweep.cu, exec_syncfree.cu,
// exec_cluster.cu);
// which is fastest depends on the wavefront depth, the level width, the
// row length, the number of right-hand sides and the arithmetic.  The
// default choice is a heuristic; gbsym_tri_autotune times the candidates on
// the plan itself and remembers the winner for the plan and, process-wide,
// for plans with the same key (level count, mean row length, k, dtype).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "exec_syncfree.cuh"

namespace gbsym {

using TuneKey = std::tuple<int, int, int, int, int>;  // levels, mean len x4, k, dtype, arith
static std::map<TuneKey, int> g_tuned;
static std::mutex g_tuned_mu;

static TuneKey tune_key(const gbsym_tri_s *t, int k, int dtype) {
  const int mean4 = t->n ? (int)(4.0 * (double)t->nnz_off / t->n + 0.5) : 0;
  return TuneKey(t->nlev, mean4, std::min(k, 64), dtype, t->arith);
}

int effective_exec(const gbsym_tri_s *t, int k, bool redundant) {
  int e = t->exec_forced != GBSYM_EXEC_AUTO ? t->exec_forced : (k == 1 ? t->exec : t->exec_mrhs);
  if (redundant) e = GBSYM_EXEC_LEVELSET;
  if ((e == GBSYM_EXEC_ONEBLOCK || e == GBSYM_EXEC_PARTITIONED) && k != 1) e = GBSYM_EXEC_SYNCFREE;
  if (t->nlev <= 1) e = GBSYM_EXEC_LEVELSET;
  return e;
}

// Default executor before any tuning: the sync-free sweep (no level
// barriers) unless the levels are narrow enough for one block.
void choose_exec(gbsym_tri_s *t) {
  const double mean_rows = (double)t->n / std::max(1, t->nlev);
  t->exec = (t->max_level_rows <= 512 && mean_rows <= 256.0) ? GBSYM_EXEC_ONEBLOCK : GBSYM_EXEC_SYNCFREE;
  t->exec_mrhs = GBSYM_EXEC_SYNCFREE;
  {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    auto it1 = g_tuned.find(tune_key(t, 1, t->vdtype));
    if (it1 != g_tuned.end()) t->exec = it1->second;
  }
  if (const char *force = std::getenv("GBSYM_TRI_EXEC")) {
    int e = -1;
    if (!std::strcmp(force, "levelset")) e = GBSYM_EXEC_LEVELSET;
    else if (!std::strcmp(force, "persistent")) e = GBSYM_EXEC_PERSISTENT;
    else if (!std::strcmp(force, "oneblock")) e = GBSYM_EXEC_ONEBLOCK;
    else if (!std::strcmp(force, "syncfree")) e = GBSYM_EXEC_SYNCFREE;
    else if (!std::strcmp(force, "cluster")) e = GBSYM_EXEC_CLUSTER;
    else if (!std::strcmp(force, "partitioned")) e = GBSYM_EXEC_PARTITIONED;
    if (e >= 0) {
      t->exec = e;
      t->exec_mrhs = (e == GBSYM_EXEC_ONEBLOCK || e == GBSYM_EXEC_PARTITIONED) ? GBSYM_EXEC_SYNCFREE : e;
    }
  }
  if (const char *pr = std::getenv("GBSYM_PART_ROWS")) t->part_rows_pref = std::atoi(pr);
  if (const char *pb = std::getenv("GBSYM_PERSIST_BLOCKS")) t->persist_blocks = std::atoi(pb);
  if (const char *cb = std::getenv("GBSYM_CLUSTER_BLOCKS")) t->cluster_blocks = std::atoi(cb);
  if (const char *sb = std::getenv("GBSYM_SF_BLOCKS_PER_SM")) t->sf_blocks_per_sm = std::atoi(sb);
  if (const char *al = std::getenv("GBSYM_SF_ALT_LANES")) t->sf_alt_lanes = std::atoi(al) == 1;
  if (const char *lt = std::getenv("GBSYM_SF_LOOKTHROUGH")) t->sf_lookthrough = std::max(0, std::min(2, std::atoi(lt)));
  if (const char *lm = std::getenv("GBSYM_SF_LT_MRHS")) t->sf_lt_mrhs = std::atoi(lm) != 0;
  t->sf_deal = num_sms();
  if (const char *sd = std::getenv("GBSYM_SF_DEAL")) t->sf_deal = std::atoi(sd);
}

template <class T>
static void solve_as(gbsym_tri_s *t, int e, T *x, const T *b, int k, int dtype, cudaStream_t s) {
  switch (e) {
    case GBSYM_EXEC_ONEBLOCK: run_oneblock<T>(t, x, s); break;
    case GBSYM_EXEC_PERSISTENT: run_persist<T>(t, x, k, s); break;
    case GBSYM_EXEC_SYNCFREE: run_syncfree<T>(t, x, k, s, nullptr); break;
    case GBSYM_EXEC_CLUSTER: run_cluster<T>(t, x, k, s); break;
    case GBSYM_EXEC_PARTITIONED: run_part<T>(t, x, s); break;
    default: run_levelset<T>(t, x, b, k, dtype, s); break;
  }
}

template <class T>
static void solve_typed(gbsym_tri_s *t, T *x, const T *b, int k, int dtype, cudaStream_t s) {
  if (t->n == 0 || k == 0) return;
  solve_as<T>(t, effective_exec(t, k, b != nullptr), x, b, k, dtype, s);
}

void tri_solve_rowmajor(gbsym_tri_s *t, void *x, const void *b, int k, int dtype, cudaStream_t s) {
  if (dtype == GBSYM_F64) {
    GB_CHECK(t->vdtype == GBSYM_F64, GBSYM_ERR_UNSUPPORTED);
    solve_typed<double>(t, (double *)x, (const double *)b, k, dtype, s);
  } else {
    GB_CHECK(t->vdtype == GBSYM_F32 && b == nullptr, GBSYM_ERR_UNSUPPORTED);
    solve_typed<float>(t, (float *)x, nullptr, k, dtype, s);
  }
}

void tri_solve_into(gbsym_tri_s *t, const void *b, void *x, int k, int dtype, cudaStream_t s) {
  if (t->n == 0 || k == 0) return;
  GB_CHECK((dtype == GBSYM_F64) == (t->vdtype == GBSYM_F64), GBSYM_ERR_UNSUPPORTED);
  // With many right-hand sides the sweep reads b and publishes each result
  // straight into x (one write of the solution instead of two; C2 factor,
  // 64 RHS: 299 MB of DRAM traffic per solve against 407 MB).  With few,
  // a row's values are too short for that to matter and the in-place
  // sweep's scratch in packed row order, whose runs are contiguous, is
  // faster (C2 factor, one RHS: 236 us publishing into x against 212 us
  // for the copy and the in-place solve).
  if (k >= 32 && effective_exec(t, k, false) == GBSYM_EXEC_SYNCFREE &&
      !(t->sf_lt_mrhs && sf_lookthrough_ok(t))) {
    if (dtype == GBSYM_F64) run_syncfree<double>(t, (double *)x, k, s, (const double *)b);
    else run_syncfree<float>(t, (float *)x, k, s, (const float *)b);
    return;
  }
  const size_t es = dtype == GBSYM_F64 ? sizeof(double) : sizeof(float);
  GB_CUDA(cudaMemcpyAsync(x, b, (size_t)t->n * k * es, cudaMemcpyDeviceToDevice, s));
  tri_solve_rowmajor(t, x, nullptr, k, dtype, s);
}

int tri_read_error(gbsym_tri_s *t, cudaStream_t s) {
  int h[2] = {0, 0};
  GB_CUDA(cudaMemcpyAsync(h, t->err.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (h[0]) GB_CUDA(cudaMemsetAsync(t->err.p, 0, 2 * sizeof(int), s));
  return h[0];
}

template <class T>
__global__ void k_fill_tune(T *x, long long m) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = T(1) + T(i % 7) * T(0.125);
}

template <class T>
static int autotune_typed(gbsym_tri_s *t, int k, int dtype, cudaStream_t s) {
  const long long m = (long long)t->n * k;
  DBuf<T> buf(m);
  // (executor, parameter) candidates: the sync-free sweep is tried at one,
  // two and three blocks per SM (parameter bits 0-2) and, for several
  // right-hand sides, with its other lane layout (bit 3: two values per
  // lane in FP64 instead of one, two in FP32 instead of four); the
  // partitioned executor (k = 1 only) at
  // several partition sizes
  std::vector<std::pair<int, int>> cands = {{GBSYM_EXEC_LEVELSET, 0}, {GBSYM_EXEC_PERSISTENT, 0},
                                            {GBSYM_EXEC_SYNCFREE, 1}, {GBSYM_EXEC_SYNCFREE, 2},
                                            {GBSYM_EXEC_SYNCFREE, 3}, {GBSYM_EXEC_CLUSTER, 0}};
  if (k > 1)
    for (int b = 1; b <= 3; ++b) cands.push_back({GBSYM_EXEC_SYNCFREE, b | 8});
  // one right-hand side on a plan that allows it: the look-through sweep
  // over one level (bits 4-5 = 1) and over two (= 2) beside the plain one
  if (k == 1 && sf_lookthrough_ok(t))
    for (int lv = 1; lv <= 2; ++lv)
      for (int b = 1; b <= 3; ++b) cands.push_back({GBSYM_EXEC_SYNCFREE, b | (lv << 4)});
  // several right-hand sides: the look-through sweep (bit 5) where it may
  // pay, a wavefront deeper than it is wide per lane group
  if (k > 1 && sf_lookthrough_ok(t))
    for (int b = 1; b <= 3; ++b) cands.push_back({GBSYM_EXEC_SYNCFREE, b | 32});
  if (k == 1 && t->max_level_rows <= 4096) cands.push_back({GBSYM_EXEC_ONEBLOCK, 0});
  if (k == 1) {
    std::vector<int> sizes;
    for (int parts : {num_sms() / 4, num_sms() / 2, num_sms(), 2 * num_sms(), 4 * num_sms()}) {
      const int r = std::min(std::max(64, div_up(t->n, std::max(1, parts))), (200 * 1024) / (int)sizeof(T));
      if (std::find(sizes.begin(), sizes.end(), r) == sizes.end()) sizes.push_back(r);
    }
    for (int r : sizes) cands.push_back({GBSYM_EXEC_PARTITIONED, r});
  }
  // caches are flushed between timed runs, as between solves of a longer
  // computation
  int l2 = 0, dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
  DBuf<char> flush((size_t)std::max(l2, 1 << 20) * 2);
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  int best = -1, best_rows = 0;
  float best_ms = 0;
  const int saved_rows = t->part_rows_pref;
  const int kk = k > 1 ? 1 : 0;
  const int saved_bps = t->sf_bps_tuned[kk], saved_alt = t->sf_alt_lanes, saved_lt = t->sf_lookthrough;
  const int saved_ltm = t->sf_lt_mrhs;
  for (const auto &cand : cands) {
    const int e = cand.first;
    if (e == GBSYM_EXEC_PARTITIONED) t->part_rows_pref = cand.second;
    if (e == GBSYM_EXEC_SYNCFREE) {
      t->sf_bps_tuned[kk] = cand.second & 7;
      if (k > 1) {
        t->sf_alt_lanes = (cand.second >> 3) & 1;
        t->sf_lt_mrhs = (cand.second >> 5) & 1;
      } else {
        t->sf_lookthrough = (cand.second >> 4) & 3;
      }
    }
    std::vector<float> ms;
    for (int rep = 0; rep < 4; ++rep) {
      k_fill_tune<T><<<(int)std::min<long long>(div_up(m, 256), num_sms() * 8), 256, 0, s>>>(buf.p, m);
      check_launch();
      GB_CUDA(cudaMemsetAsync(flush.p, rep, flush.n, s));
      GB_CUDA(cudaEventRecord(e0, s));
      solve_as<T>(t, e, buf.p, nullptr, k, dtype, s);
      GB_CUDA(cudaEventRecord(e1, s));
      GB_CUDA(cudaEventSynchronize(e1));
      float v = 0;
      GB_CUDA(cudaEventElapsedTime(&v, e0, e1));
      if (rep) ms.push_back(v);  // the first run builds graphs and warms caches
    }
    if (tri_read_error(t, s)) continue;  // a candidate that timed out is skipped
    std::sort(ms.begin(), ms.end());
    const float med = ms[ms.size() / 2];
    if (best < 0 || med < best_ms) {
      best = e;
      best_rows = cand.second;
      best_ms = med;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  t->part_rows_pref = saved_rows;
  t->sf_bps_tuned[kk] = saved_bps;
  t->sf_alt_lanes = saved_alt;
  t->sf_lookthrough = saved_lt;
  t->sf_lt_mrhs = saved_ltm;
  if (best < 0) throw Err{GBSYM_ERR_TIMEOUT};
  if (best == GBSYM_EXEC_PARTITIONED) t->part_rows_pref = best_rows;
  if (best == GBSYM_EXEC_SYNCFREE) {
    t->sf_bps_tuned[kk] = best_rows & 7;
    if (k > 1) {
      t->sf_alt_lanes = (best_rows >> 3) & 1;
      t->sf_lt_mrhs = (best_rows >> 5) & 1;
    } else {
      t->sf_lookthrough = (best_rows >> 4) & 3;
    }
  }
  if (k == 1) t->exec = best; else t->exec_mrhs = best;
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  g_tuned[tune_key(t, k, dtype)] = best;
  return best;
}

}  // namespace gbsym

using namespace gbsym;

extern "C" int gbsym_tri_autotune(gbsym_tri t, int k, int dtype, void *stream, int *chosen) {
  gbsym::PhaseRange phase_("gbsym_tri_autotune");
  if (!t) return GBSYM_ERR_NULL_ARG;
  if (k < 1) return GBSYM_ERR_SIZE;
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    int e = GBSYM_EXEC_LEVELSET;
    if (t->n > 0 && t->nlev > 1) {
      if (dtype == GBSYM_F64) {
        GB_CHECK(t->vdtype == GBSYM_F64, GBSYM_ERR_UNSUPPORTED);
        e = autotune_typed<double>(t, k, dtype, s);
      } else {
        GB_CHECK(t->vdtype == GBSYM_F32, GBSYM_ERR_UNSUPPORTED);
        e = autotune_typed<float>(t, k, dtype, s);
      }
    }
    if (chosen) *chosen = e;
  });
}

extern "C" int gbsym_tri_get_tuning(gbsym_tri t, int k, int *tuning) {
  if (!t || !tuning) return GBSYM_ERR_NULL_ARG;
  if (k < 1) return GBSYM_ERR_SIZE;
  tuning[0] = effective_exec(t, k, false);
  tuning[1] = t->sf_blocks_per_sm > 0 ? t->sf_blocks_per_sm : t->sf_bps_tuned[k > 1 ? 1 : 0];
  const int lt_ok = sf_lookthrough_ok(t) ? 1 : 0;
  tuning[2] = k > 1 ? (t->sf_alt_lanes | ((t->sf_lt_mrhs && lt_ok) ? 2 : 0))
                    : (lt_ok ? t->sf_lookthrough : 0);
  return GBSYM_OK;
}

extern "C" int gbsym_tri_set_arith(gbsym_tri t, int arith) {
  if (!t) return GBSYM_ERR_NULL_ARG;
  if (arith != GBSYM_ARITH_EXACT && arith != GBSYM_ARITH_FUSED) return GBSYM_ERR_UNSUPPORTED;
  t->arith = arith;
  return GBSYM_OK;
}
