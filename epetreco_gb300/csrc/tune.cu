// tune.cu -- the row-kernel autotuner.
//
// A product kernel's best launch shape depends on the matrix: rows of a few
// dozen entries want small lane groups, the long columns of the transposed
// system matrix want full warps and deep unrolling, and a persistent grid
// can beat one block per tile when tiles are short.  tune_rows times the
// candidates on the caller's own matrix and remembers the winner for the
// process.  Candidates: G in {g/2, g, 2g} (g = the heuristic group size for
// the mean row length) with 16-byte chunks per lane (U in {1, 2, 4}) or
// interleaved entries; then, for the fastest, a persistent grid of 4 and 8
// blocks per SM.  Each candidate runs once to
// warm up and is then timed over three runs with CUDA events.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "spmv.cuh"

namespace epet {

namespace {

using TuneKey = std::tuple<int, int, int64_t, int64_t, int64_t>;  // dev, kind, rows, nnz, cols

std::mutex g_tune_mu;
std::map<TuneKey, RowPlan> g_tune_cache;

epet_status time_plan(const RowPlan& p, const std::function<epet_status(const RowPlan&)>& run,
                      cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, float* ms) {
  EPET_CHECK(run(p));
  EPET_CUDA(cudaEventRecord(e0, st));
  constexpr int kReps = 3;
  for (int r = 0; r < kReps; r++) EPET_CHECK(run(p));
  EPET_CUDA(cudaEventRecord(e1, st));
  EPET_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  EPET_CUDA(cudaEventElapsedTime(&t, e0, e1));
  *ms = t / kReps;
  return EPET_OK;
}

}  // namespace

bool tune_lookup(int kind, int64_t nrows, int64_t nnz, int64_t ncols, RowPlan* out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune_cache.find(TuneKey{dev, kind, nrows, nnz, ncols});
  if (it == g_tune_cache.end()) return false;
  *out = it->second;
  return true;
}

epet_status tune_rows(int kind, int64_t nrows, int64_t nnz, int64_t ncols, double avg,
                      const std::function<epet_status(const RowPlan&)>& run, cudaStream_t st,
                      RowPlan* out) {
  int dev = 0, sms = 0;
  EPET_CUDA(cudaGetDevice(&dev));
  EPET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const TuneKey key{dev, kind, nrows, nnz, ncols};
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune_cache.find(key);
  if (it != g_tune_cache.end()) {
    *out = it->second;
    return EPET_OK;
  }
  const RowPlan base = default_plan(avg);
  if (nrows <= 0 || nnz <= 0) {
    *out = base;
    return EPET_OK;
  }
  std::vector<RowPlan> cands;
  for (int g : {base.G / 2, base.G, base.G * 2}) {
    if (g < 4 || g > 32) continue;
    for (int u : {1, 2, 4}) cands.push_back(RowPlan{g, u, 0, true});
    cands.push_back(RowPlan{g, 1, 0, false});
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  EPET_CUDA(cudaEventCreate(&e0));
  EPET_CUDA(cudaEventCreate(&e1));
  RowPlan best = base;
  float best_ms = 3.4e38f;
  epet_status rc = EPET_OK;
  auto try_plan = [&](const RowPlan& p) {
    float ms = 0.f;
    if (rc == EPET_OK) rc = time_plan(p, run, st, e0, e1, &ms);
    if (rc == EPET_OK && ms < best_ms) {
      best_ms = ms;
      best = p;
    }
  };
  for (const RowPlan& p : cands) try_plan(p);
  const RowPlan one_per_tile = best;
  for (int per_sm : {4, 8}) {
    RowPlan p = one_per_tile;
    p.grid = per_sm * sms;
    if (plan_tiles(p, nrows) > p.grid) try_plan(p);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != EPET_OK) return rc;
  g_tune_cache[key] = best;
  *out = best;
  return EPET_OK;
}

}  // namespace epet
