// batch.cu -- many independent reconstructions iterated by batched launches.
//
// Each problem is an ordinary epet_mlem (its own matrix, CSC copy, counts,
// sensitivity and image, all in separate allocations).  The batch adds a
// device array of per-problem descriptors and tile tables, and runs every
// step of an iteration as ONE launch over all problems: a tile of rows (or
// voxels) finds its problem by binary search in the tile table, then works
// on that problem's arrays.  The four launches of an iteration (five with
// wide row groups) are captured
// in one CUDA graph.  Partial image sums are written per tile; a problem's
// tiles are contiguous, so its image sum is a fixed-order sum over its own
// tile range (deterministic, as in the single-problem driver).
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "mlem_internal.h"
#include "rows.cuh"
#include "spmv.cuh"

namespace epet {

// One problem's arrays, device-resident.
struct BatchDesc {
  const int64_t* row_ptr;
  const int32_t* col;
  const float* val;
  const int64_t* col_ptr;
  const int32_t* row;
  const float* cval;
  const float* y;
  float* e;
  float* ybar;
  const float* s;
  float* x;
  float* xnew;
  int64_t m, V;
};

constexpr int kNormTile = 256;  // voxels per tile of the normalisation launch

// Tile tables: for each rows-per-tile choice (8, 16, 32, 64 rows: G = 32,
// 16, 8, 4) the exclusive prefix of per-problem tile counts, nprob + 1
// entries each, for the forward rows and the transpose columns; plus one
// table of normalisation tiles.
inline int rpt_index(int G) { return G == 32 ? 0 : G == 16 ? 1 : G == 8 ? 2 : 3; }

__device__ __forceinline__ int find_problem(const int64_t* __restrict__ tiles, int np,
                                            int64_t t) {
  int lo = 0, hi = np;  // tiles[lo] <= t < tiles[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(tiles + mid) <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Forward (FWD) or transpose product of every problem, MLEM epilogues fused.
template <int G, int U, bool VEC, bool FWD>
__global__ void __launch_bounds__(kSpmvThreads)
k_batch_rows(const BatchDesc* __restrict__ desc, const int64_t* __restrict__ tiles, int np,
             double* __restrict__ partial) {
  constexpr int RPT = kSpmvThreads / G;
  __shared__ double red[kSpmvThreads / 32];
  const int lg = threadIdx.x % G;
  const int64_t ntiles = tiles[np];
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int p = find_problem(tiles, np, tile);
    const BatchDesc& d = desc[p];
    const int64_t r = (tile - tiles[p]) * RPT + threadIdx.x / G;
    double part = 0.0;
    if constexpr (FWD) {
      if (r < d.m) {
        const float v = row_dot<G, U, VEC>(d.col, d.val, d.x, d.row_ptr[r], d.row_ptr[r + 1], lg);
        if (lg == 0) EpiMlemForward{d.y, d.e, d.ybar}(r, v);
      }
    } else {
      if (r < d.V) {
        const float c = row_dot<G, U, VEC>(d.row, d.cval, d.e, d.col_ptr[r], d.col_ptr[r + 1], lg);
        if (lg == 0) part = EpiMlemUpdate{d.x, d.s, d.xnew, nullptr}(r, c);
      }
      block_sum_to(part, red, partial + tile);
    }
  }
}

// sums[p] = fixed-order sum of partial over problem p's transpose tiles.
__global__ void k_batch_sums(const double* __restrict__ partial,
                             const int64_t* __restrict__ tiles, double* __restrict__ sums) {
  __shared__ double red[kSpmvThreads / 32];
  const int p = blockIdx.x;
  double s = 0.0;
  for (int64_t i = tiles[p] + threadIdx.x; i < tiles[p + 1]; i += kSpmvThreads) s += partial[i];
  block_sum_to(s, red, sums + p);
}

// x = xnew * float(1 / sum) per problem (reco.cu:277-281).
__global__ void k_batch_normalise(const BatchDesc* __restrict__ desc,
                                  const int64_t* __restrict__ tiles, int np,
                                  const double* __restrict__ sums) {
  const int64_t tile = blockIdx.x;
  const int p = find_problem(tiles, np, tile);
  const BatchDesc& d = desc[p];
  const int64_t v = (tile - tiles[p]) * kNormTile + threadIdx.x;
  if (v < d.V) d.x[v] = fmul((float)(1.0 / sums[p]), d.xnew[v]);
}

}  // namespace epet

using namespace epet;

struct epet_mlem_batch {
  std::vector<epet_mlem*> probs;
  epet_mlem_options opt{};
  BatchDesc* desc = nullptr;       // device, nprob
  int64_t* tiles = nullptr;        // device: fwd[4][np+1], bwd[4][np+1], norm[np+1]
  std::vector<int64_t> tiles_h;    // host copy
  double* partial = nullptr;       // transpose tiles (most of any plan)
  double* sums = nullptr;          // nprob
  RowPlan plan_fwd, plan_bwd;
  int64_t nnz = 0, rows = 0, voxels = 0;
  // grouped layout: one pass over all problems' row groups replaces the
  // forward launch; the transpose launch sums each problem's slots
  bool grouped = false;
  void* gdesc = nullptr;      // device, nprob descriptors of the pass
  int64_t* gstart = nullptr;  // device, prefix of the problems' group counts
  int64_t total_groups = 0;
  int32_t* gwide = nullptr;   // device, global ids of the wide groups
  int64_t nwide = 0;
  int graph_kernels = 0;      // kernels in the captured iteration
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;

  int np() const { return (int)probs.size(); }
  const int64_t* fwd_tiles(int G) const { return tiles + rpt_index(G) * (np() + 1); }
  const int64_t* bwd_tiles(int G) const { return tiles + (4 + rpt_index(G)) * (np() + 1); }
  const int64_t* norm_tiles() const { return tiles + 8 * (np() + 1); }
  int64_t host_total(int table) const { return tiles_h[table * (np() + 1) + np()]; }
};

namespace {

void batch_free(epet_mlem_batch* h) {
  if (!h) return;
  cudaDeviceSynchronize();
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  for (epet_mlem* p : h->probs) epet_mlem_destroy(p);
  for (void* b : {(void*)h->desc, (void*)h->tiles, (void*)h->partial, (void*)h->sums,
                  h->gdesc, (void*)h->gstart, (void*)h->gwide})
    if (b) dev_free(b, 0);
  delete h;
}

epet_status launch_batch_rows(const epet_mlem_batch* h, const RowPlan& plan, bool fwd,
                              cudaStream_t st) {
  const int G = plan.G;
  const int64_t nt = h->host_total((fwd ? 0 : 4) + rpt_index(G));
  if (nt <= 0) return EPET_OK;
  const unsigned grid = (unsigned)(plan.grid > 0 ? std::min<int64_t>(nt, plan.grid) : nt);
  const int64_t* tiles = fwd ? h->fwd_tiles(G) : h->bwd_tiles(G);
  dispatch_plan(plan, true, [&](auto g, auto u, auto v) {
    if (fwd)
      k_batch_rows<decltype(g)::value, decltype(u)::value, decltype(v)::value, true>
          <<<grid, kSpmvThreads, 0, st>>>(h->desc, tiles, h->np(), nullptr);
    else
      k_batch_rows<decltype(g)::value, decltype(u)::value, decltype(v)::value, false>
          <<<grid, kSpmvThreads, 0, st>>>(h->desc, tiles, h->np(), h->partial);
  });
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status batch_iteration(const epet_mlem_batch* h, cudaStream_t st) {
  if (h->grouped)
    EPET_CHECK(grouped_pass_batch(h->gdesc, h->gstart, h->np(), h->total_groups, h->gwide,
                                  h->nwide, st));
  else
    EPET_CHECK(launch_batch_rows(h, h->plan_fwd, true, st));
  EPET_CHECK(launch_batch_rows(h, h->plan_bwd, false, st));
  k_batch_sums<<<h->np(), kSpmvThreads, 0, st>>>(h->partial, h->bwd_tiles(h->plan_bwd.G),
                                                 h->sums);
  EPET_LAUNCHED();
  const int64_t nt = h->host_total(8);
  if (nt > 0) {
    k_batch_normalise<<<(unsigned)nt, kNormTile, 0, st>>>(h->desc, h->norm_tiles(), h->np(),
                                                          h->sums);
    EPET_LAUNCHED();
  }
  return EPET_OK;
}

}  // namespace

extern "C" {

epet_status epet_mlem_batch_create(int32_t nprob, const epet_problem* problems,
                                   const int32_t* const* rows_d, const int64_t* m,
                                   const float* const* y_d, const float* const* s_d,
                                   const epet_mlem_options* opt, epet_mlem_batch** out,
                                   epet_stream_t stream) {
  if (nprob <= 0 || !problems || !rows_d || !m || !y_d || !s_d || !out)
    return set_error(EPET_ERR_INVALID, "bad arguments");
  epet_mlem_options o{};
  if (opt) o = *opt;
  if (o.matrix_free)
    return set_error(EPET_ERR_INVALID, "batched reconstructions store their matrices "
                                       "(matrix_free is not supported)");
  if (o.value_format != EPET_VALUES_FP32)
    return set_error(EPET_ERR_INVALID, "batched reconstructions hold FP32 values");
  cudaStream_t st = (cudaStream_t)stream;
  epet_mlem_batch* h = new epet_mlem_batch();
  h->opt = o;
  auto fail = [&](epet_status rc) {
    batch_free(h);
    return rc;
  };
  epet_mlem_options po = o;  // members iterated alone: graph as asked, heuristic shapes
  po.autotune = 0;
  // every member in the grouped layout where all support it (6 bytes per
  // entry), else every member with its CSR and column-major copy
  bool all_grouped = o.layout != EPET_LAYOUT_CSC;
  for (int i = 0; i < nprob && all_grouped; i++) {
    const epet_grid& g = problems[i].grid;
    all_grouped = grouped_supported((int64_t)g.n[0] * g.n[1] * g.n[2], m[i]);
  }
  if (o.layout == EPET_LAYOUT_GROUPED && !all_grouped)
    return set_error(EPET_ERR_UNSUPPORTED, "batch: a problem too large for the grouped layout");
  po.layout = all_grouped ? EPET_LAYOUT_GROUPED : EPET_LAYOUT_CSC;
  for (int i = 0; i < nprob; i++) {
    epet_mlem* p = nullptr;
    epet_status rc = epet_mlem_create(&problems[i], rows_d[i], y_d[i], m[i], s_d[i], &po, &p,
                                      stream);
    if (rc != EPET_OK) return fail(rc);
    h->probs.push_back(p);
    h->nnz += p->A.nnz;
    h->rows += p->m;
    h->voxels += p->V;
  }
  const int np = nprob;
  std::vector<BatchDesc> dh(np);
  h->tiles_h.assign(9 * (np + 1), 0);
  h->grouped = all_grouped;
  std::vector<unsigned char> gd_h(all_grouped ? np * grouped_batch_desc_bytes() : 0);
  std::vector<int64_t> gs_h(np + 1, 0);
  std::vector<int32_t> gw_h;  // global ids of the wide groups
  for (int i = 0; i < np; i++) {
    epet_mlem* p = h->probs[i];
    if (all_grouped) {
      // the transpose launch sums the problem's slots: the slot lists as
      // "columns", the ones as values, the slots' corrections gathered
      const epet_status rc = grouped_ones(&p->G, st);
      if (rc != EPET_OK) return fail(rc);
      dh[i] = BatchDesc{nullptr, nullptr, nullptr, p->G.cg_ptr, p->G.cg_slot, p->G.ones,
                        p->y, p->G.partial, p->ybar, p->s, p->x, p->xnew, p->m, p->V};
      grouped_batch_desc(p->G, p->x, p->y, p->ybar, gd_h.data() + i * grouped_batch_desc_bytes());
      for (int32_t w : p->G.wide_h) gw_h.push_back((int32_t)(gs_h[i] + w));
      gs_h[i + 1] = gs_h[i] + p->G.ngroups;
      if (!aligned16(p->G.cg_slot, p->G.ones))
        return fail(set_error(EPET_ERR_UNSUPPORTED, "batch: slot streams not 16-byte aligned"));
    } else {
      dh[i] = BatchDesc{p->A.row_ptr, p->A.col, p->A.val, p->At.col_ptr, p->At.row, p->At.val,
                        p->y, p->e, p->ybar, p->s, p->x, p->xnew, p->m, p->V};
      if (!aligned16(p->A.col, p->A.val) || !aligned16(p->At.row, p->At.val))
        return fail(set_error(EPET_ERR_UNSUPPORTED, "batch: matrix streams not 16-byte aligned"));
    }
    for (int k = 0; k < 4; k++) {
      const int64_t rpt = int64_t(8) << k;
      int64_t* f = &h->tiles_h[k * (np + 1)];
      int64_t* b = &h->tiles_h[(4 + k) * (np + 1)];
      f[i + 1] = f[i] + ceil_div(p->m, rpt);
      b[i + 1] = b[i] + ceil_div(p->V, rpt);
    }
    int64_t* nrm = &h->tiles_h[8 * (np + 1)];
    nrm[i + 1] = nrm[i] + ceil_div(p->V, (int64_t)kNormTile);
  }
#define ALLOC(ptr, bytes)                                                    \
  do {                                                                       \
    cudaError_t e_ = dev_alloc((void**)&(ptr), std::max<size_t>(bytes, 8), st); \
    if (e_ != cudaSuccess) return fail(cuda_status(e_, "allocation " #ptr)); \
  } while (0)
  ALLOC(h->desc, np * sizeof(BatchDesc));
  ALLOC(h->tiles, h->tiles_h.size() * 8);
  ALLOC(h->partial, std::max<int64_t>(h->host_total(4), 1) * 8);  // 8 rows per tile: most
  ALLOC(h->sums, np * 8);
  if (all_grouped) {
    ALLOC(h->gdesc, gd_h.size());
    ALLOC(h->gstart, (np + 1) * 8);
    h->total_groups = gs_h[np];
    if (h->total_groups > INT32_MAX)
      return fail(set_error(EPET_ERR_UNSUPPORTED, "batch: more than 2^31 row groups"));
    h->nwide = (int64_t)gw_h.size();
    if (h->nwide > 0) ALLOC(h->gwide, h->nwide * 4);
  }
#undef ALLOC
  cudaError_t e = cudaMemcpyAsync(h->desc, dh.data(), np * sizeof(BatchDesc),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->tiles, h->tiles_h.data(), h->tiles_h.size() * 8,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && all_grouped)
    e = cudaMemcpyAsync(h->gdesc, gd_h.data(), gd_h.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && all_grouped)
    e = cudaMemcpyAsync(h->gstart, gs_h.data(), (np + 1) * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && h->nwide > 0)
    e = cudaMemcpyAsync(h->gwide, gw_h.data(), h->nwide * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(cuda_status(e, "batch descriptors"));

  const double avg_row = h->rows ? (double)h->nnz / h->rows : 0.0;
  int64_t nslots = 0;
  for (const epet_mlem* p : h->probs) nslots += p->G.nslots;
  const double avg_col = h->voxels ? (double)(all_grouped ? nslots : h->nnz) / h->voxels : 0.0;
  h->plan_fwd = default_plan(avg_row);
  h->plan_bwd = default_plan(avg_col);
  if (o.autotune) {
    // kinds 5 / 6 / 7 keep batch plans apart from single-matrix plans
    epet_status rc = EPET_OK;
    if (all_grouped) {
      // one pass fills the slots (unless the plan is cached); the slot
      // sums' candidates rerun the (idempotent) update epilogue
      if (!tune_lookup(7, h->voxels, nslots, np, &h->plan_bwd))
        rc = grouped_pass_batch(h->gdesc, h->gstart, np, h->total_groups, h->gwide, h->nwide,
                                st);
      if (rc == EPET_OK)
        rc = tune_rows(
            7, h->voxels, nslots, np, avg_col,
            [&](const RowPlan& pl) { return launch_batch_rows(h, pl, false, st); }, st,
            &h->plan_bwd);
    } else {
      rc = tune_rows(
          5, h->rows, h->nnz, np, avg_row,
          [&](const RowPlan& pl) { return launch_batch_rows(h, pl, true, st); }, st,
          &h->plan_fwd);
      if (rc == EPET_OK)
        rc = tune_rows(
            6, h->voxels, h->nnz, np, avg_col,
            [&](const RowPlan& pl) { return launch_batch_rows(h, pl, false, st); }, st,
            &h->plan_bwd);
    }
    if (rc != EPET_OK) return fail(rc);
  }
  *out = h;
  return EPET_OK;
}

epet_status epet_mlem_batch_destroy(epet_mlem_batch* h) {
  if (h) cudaDeviceSynchronize();
  batch_free(h);
  return EPET_OK;
}

epet_status epet_mlem_batch_iterate(epet_mlem_batch* h, int32_t nit, double* loglik_h,
                                    epet_stream_t stream) {
  if (!h || nit < 0) return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  if (h->opt.use_graph) {
    if (!h->exec) {
      cudaStream_t cap = nullptr;
      EPET_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
      epet_status rc = EPET_OK;
      cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
      const long long k0 = epet_launch_count();
      if (e == cudaSuccess) rc = batch_iteration(h, cap);
      // (capturing counted the kernels; the replays below count them again)
      h->graph_kernels = (int)(epet_launch_count() - k0);
      note_launch(-h->graph_kernels);
      cudaError_t e2 = cudaStreamEndCapture(cap, &h->graph);
      cudaStreamDestroy(cap);
      if (e != cudaSuccess) return cuda_status(e, "begin capture");
      if (rc != EPET_OK) return rc;
      if (e2 != cudaSuccess) return cuda_status(e2, "end capture");
      EPET_CUDA(cudaGraphInstantiate(&h->exec, h->graph, 0));
    }
    for (int it = 0; it < nit; it++) {
      EPET_CUDA(cudaGraphLaunch(h->exec, st));
      note_launch(h->graph_kernels);  // the kernels of the captured iteration
    }
  } else {
    for (int it = 0; it < nit; it++) EPET_CHECK(batch_iteration(h, st));
  }
  if (loglik_h) {
    for (int i = 0; i < h->np(); i++) {
      EPET_CHECK(epet_mlem_iterate(h->probs[i], 0, &loglik_h[i], stream));
    }
  }
  return EPET_OK;
}

epet_status epet_mlem_batch_get_image(const epet_mlem_batch* h, int32_t i, float* x_d,
                                      epet_stream_t stream) {
  if (!h || i < 0 || i >= h->np()) return set_error(EPET_ERR_INVALID, "bad arguments");
  return epet_mlem_get_image(h->probs[i], x_d, stream);
}

epet_mlem* epet_mlem_batch_member(epet_mlem_batch* h, int32_t i) {
  if (!h || i < 0 || i >= h->np()) {
    set_error(EPET_ERR_INVALID, "bad arguments");
    return nullptr;
  }
  return h->probs[i];
}

epet_status epet_mlem_batch_stats(const epet_mlem_batch* h, int64_t* nnz_h,
                                  int64_t* bytes_per_iter_h, int32_t plan_h[6]) {
  if (!h) return set_error(EPET_ERR_INVALID, "bad arguments");
  if (nnz_h) *nnz_h = h->nnz;
  if (bytes_per_iter_h) {
    int64_t tot = 0;
    for (const epet_mlem* p : h->probs) {
      int64_t b = 0;
      EPET_CHECK(epet_mlem_stats(p, nullptr, &b));
      tot += b;
    }
    *bytes_per_iter_h = tot;
  }
  if (plan_h) {
    const RowPlan* ps[2] = {&h->plan_fwd, &h->plan_bwd};
    for (int k = 0; k < 2; k++) {
      plan_h[3 * k + 0] = ps[k]->G;
      plan_h[3 * k + 1] = ps[k]->vec ? ps[k]->U : 0;
      plan_h[3 * k + 2] = ps[k]->grid;
    }
  }
  return EPET_OK;
}

}  // extern "C"
