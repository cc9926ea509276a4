// mlem.cu -- the reconstruction driver (reco.cu:32-332 without MPI/HDF5).
//
// One epet_mlem holds a reconstruction on the device: the measured rows and
// their counts (reordered by crystal pairs, see order_rows), the system matrix built once by the fused kernel (it is
// deterministic, so the reference's rebuild in every iteration is not
// needed), its column-major copy, the normalised sensitivity and the image.
// An iteration is four kernels: forward product fused with e = y/(Ax);
// transpose product fused with x*c/s; the fixed-order image sum (block
// partials); the normalisation (which reduces the partials itself).  With use_graph the four are captured once in a CUDA
// graph and replayed.  The Poisson log-likelihood of the last forward
// projection is reduced in fp64 on request.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "spmv.cuh"

#include "mlem_internal.h"

using namespace epet;

static void mlem_free(epet_mlem* h) {
  if (!h) return;
  cudaDeviceSynchronize();  // nothing in flight uses the arrays
  grouped_free(&h->G, 0);
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  void* bufs[] = {h->A16.row_ptr, h->A16.base, h->A16.scale, h->A16.delta, h->A16.q,
                  h->At16.row_ptr, h->At16.base, h->At16.scale, h->At16.delta, h->At16.q,
                  h->rows, h->y, h->ybar, h->e16, h->s, h->x, h->xnew, h->e, h->A.row_ptr, h->A.col,
                  h->A.val,
                  h->At.col_ptr, h->At.row, h->At.val, h->part_ll, h->part_x, h->sums, h->c64};
  for (void* b : bufs)
    if (b) dev_free(b, 0);
  delete h;
}

// x*c/s (dividesMultiplies, mlemOperations.hpp:38-79, with s == 0 -> 1), the
// arithmetic of EpiMlemUpdate, from a correction image held apart: the fp64
// one of the matrix-free schedule (rounded to fp32 as the reference's float
// c) or the fp32 one summed across the shards of a row-sharded
// reconstruction.
template <typename CT>
__global__ void k_update_c(const float* __restrict__ x, const CT* __restrict__ cimg,
                           const float* __restrict__ s, int64_t V, float* __restrict__ xnew) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  const float c = (float)cimg[v];
  float dvs = s[v];
  dvs = __fadd_rn(dvs, (float)(dvs == 0.f));
  xnew[v] = __fdiv_rn(__fmul_rn(x[v], c), dvs);
}

__global__ void k_f64_to_f32_vec(const double* __restrict__ a, int64_t n, float* __restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// The reference's schedule: the chords recomputed in every iteration (one
// walk per row gives A x, e and the row's share of A^T e), then the update
// and the normalisation.
static epet_status mlem_iteration_free(epet_mlem* h, cudaStream_t st) {
  EPET_CUDA(cudaMemsetAsync(h->c64, 0, h->V * 8, st));
  EPET_CHECK(epet_project_mlem(&h->p, h->rows, h->m, h->x, h->y, h->ybar, h->c64,
                               h->opt.max_row_nnz, nullptr, 0, st));
  k_update_c<double><<<ceil_div(h->V, 256), 256, 0, st>>>(h->x, h->c64, h->s, h->V, h->xnew);
  EPET_LAUNCHED();
  return launch_sum_normalise(h->xnew, h->V, h->part_x, h->x, st);
}

// c = A^T (y / A x) over this object's rows, without the update (the
// forward product keeps ybar and e as in the iteration).
static epet_status mlem_correction(epet_mlem* h, float* c, cudaStream_t st) {
  if (h->grouped) {
    EPET_CHECK(grouped_pass(h->G, h->x, h->y, h->ybar, st));
    return launch_sums(h->G.plan_cols, h->G.cg_ptr, h->G.cg_slot, h->G.partial, h->V,
                       EpiKeep{c}, nullptr, st);
  }
  if (h->opt.matrix_free) {
    EPET_CUDA(cudaMemsetAsync(h->c64, 0, h->V * 8, st));
    EPET_CHECK(epet_project_mlem(&h->p, h->rows, h->m, h->x, h->y, h->ybar, h->c64,
                                 h->opt.max_row_nnz, nullptr, 0, st));
    k_f64_to_f32_vec<<<ceil_div(h->V, 256), 256, 0, st>>>(h->c64, h->V, c);
    EPET_LAUNCHED();
    return EPET_OK;
  }
  if (h->opt.value_format != EPET_VALUES_FP32) {
    EPET_CHECK((launch_rows16<EpiMlemForward16, float>(
        &h->A16, h->x, EpiMlemForward16{h->y, h->e16, h->ybar}, nullptr, st)));
    return launch_rows16<EpiKeep, uint16_t>(&h->At16, h->e16, EpiKeep{c}, nullptr, st);
  }
  EPET_CHECK(launch_rows(h->plan_fwd, h->A.row_ptr, h->A.col, h->A.val, h->x, h->m,
                         EpiMlemForward{h->y, h->e, h->ybar}, nullptr, st));
  return launch_rows(h->plan_bwd, h->At.col_ptr, h->At.row, h->At.val, h->e, h->V, EpiKeep{c},
                     nullptr, st);
}

// The grouped layout: one pass over the entries (A x, e, the groups' shares
// of A^T e), the fixed-order slot sums per column fused with x*c/s, the
// image sum and the normalisation.
static epet_status mlem_iteration_grouped(epet_mlem* h, cudaStream_t st) {
  EPET_CHECK(grouped_pass(h->G, h->x, h->y, h->ybar, st));
  EPET_CHECK(launch_sums(h->G.plan_cols, h->G.cg_ptr, h->G.cg_slot, h->G.partial,
                         h->V, EpiMlemUpdate{h->x, h->s, h->xnew, nullptr}, nullptr, st));
  return launch_sum_normalise(h->xnew, h->V, h->part_x, h->x, st);
}

static epet_status mlem_iteration(epet_mlem* h, cudaStream_t st) {
  if (h->opt.matrix_free) return mlem_iteration_free(h, st);
  if (h->grouped) return mlem_iteration_grouped(h, st);
  if (h->opt.value_format != EPET_VALUES_FP32) {
    EPET_CHECK((launch_rows16<EpiMlemForward16, float>(
        &h->A16, h->x, EpiMlemForward16{h->y, h->e16, h->ybar}, nullptr, st)));
    EPET_CHECK((launch_rows16<EpiMlemUpdate, uint16_t>(
        &h->At16, h->e16, EpiMlemUpdate{h->x, h->s, h->xnew, nullptr}, nullptr, st)));
    return launch_sum_normalise(h->xnew, h->V, h->part_x, h->x, st);
  }
  EPET_CHECK(launch_rows(h->plan_fwd, h->A.row_ptr, h->A.col, h->A.val, h->x, h->m,
                         EpiMlemForward{h->y, h->e, h->ybar}, nullptr, st));
  EPET_CHECK(launch_rows(h->plan_bwd, h->At.col_ptr, h->At.row, h->At.val, h->e, h->V,
                         EpiMlemUpdate{h->x, h->s, h->xnew, nullptr}, nullptr, st));
  return launch_sum_normalise(h->xnew, h->V, h->part_x, h->x, st);
}

// Order of the measured rows inside a reconstruction.  A line through a
// voxel joins crystals of the two heads whose y indices, and whose z indices,
// add up to about twice the voxel's position on that axis (the heads face
// each other with parallel y and z axes), so keys ordered by angle, then by
// the two index sums, then by the first crystal, make the channels through
// one voxel a few contiguous runs.  Each column of the column-major copy
// lists its rows in this order, so the transpose product's gathers of
// e = y / (A x) read far fewer cache sectors; each column sum has the same
// terms in another order.  Channels outside the setup get the largest key
// (the build reports them as before).
__global__ void k_pair_keys(epet_setup s, const int32_t* __restrict__ rows, int64_t m,
                            int32_t nch, int32_t kmax, int32_t* __restrict__ key,
                            int32_t* __restrict__ idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int32_t c = rows[i];
  int32_t k = kmax;
  if (c >= 0 && c < nch) {
    int id[5];  // angle, crystal 0 (z, y), crystal 1 (z, y)
    channel_decode(s, c, id);
    const int SY = s.n0y + s.n1y - 1, SZ = s.n0z + s.n1z - 1;
    k = (((id[0] * SY + id[2] + id[4]) * SZ + id[1] + id[3]) * s.n0y + id[2]) * s.n0z + id[1];
  }
  key[i] = k;
  idx[i] = (int32_t)i;
}

__global__ void k_gather_i32(const int32_t* __restrict__ src, const int32_t* __restrict__ idx,
                             int64_t m, int32_t* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) dst[i] = src[idx[i]];
}

// h->rows / h->y = the measured rows and counts in the order above (a
// stable sort of the keys, which carries y along); list order when the keys
// do not fit 31 bits.  *idx_out (caller frees; null in list order) = the
// list index of each row in the new order.
static epet_status order_rows(const epet_problem* p, const int32_t* rows_d, int64_t m,
                              epet_mlem* h, cudaStream_t st, int32_t** idx_out) {
  *idx_out = nullptr;
  const epet_setup& s = p->setup;
  const int64_t SY = (int64_t)s.n0y + s.n1y - 1, SZ = (int64_t)s.n0z + s.n1z - 1;
  const int64_t kmax = (int64_t)s.na * SY * SZ * s.n0y * s.n0z;
  const int64_t nch = (int64_t)s.na * s.n0z * s.n0y * s.n1z * s.n1y;
  if (m < 2 || m > INT32_MAX || kmax >= INT32_MAX || nch > INT32_MAX) {
    if (m > 0)
      EPET_CUDA(cudaMemcpyAsync(h->rows, rows_d, m * 4, cudaMemcpyDeviceToDevice, st));
    return EPET_OK;
  }
  int32_t *key = nullptr, *idx = nullptr;
  EPET_CUDA(dev_alloc((void**)&key, m * 4, st));
  cudaError_t e = dev_alloc((void**)&idx, m * 4, st);
  if (e != cudaSuccess) {
    dev_free(key, st);
    return cuda_status(e, "allocation of the row order");
  }
  k_pair_keys<<<ceil_div(m, 256), 256, 0, st>>>(s, rows_d, m, (int32_t)nch, (int32_t)kmax, key,
                                                idx);
  note_launch();
  epet_status rc = cudaGetLastError() == cudaSuccess
                       ? epet_coo_sort(h->y, key, idx, m, nullptr, 0, st)
                       : set_error(EPET_ERR_CUDA, "row order keys");
  if (rc == EPET_OK) {
    k_gather_i32<<<ceil_div(m, 256), 256, 0, st>>>(rows_d, idx, m, h->rows);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) rc = set_error(EPET_ERR_CUDA, "row order gather");
  }
  dev_free(key, st);
  if (rc == EPET_OK) *idx_out = idx;
  else dev_free(idx, st);
  return rc;
}

__global__ void k_perm_len(const int64_t* __restrict__ rp0, const int32_t* __restrict__ idx,
                           int64_t m, int64_t* __restrict__ len) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) len[i] = rp0[idx[i] + 1] - rp0[idx[i]];
}

// Row i of the CSR = built row idx[i], read from the segment of its chunk
// (chunks of ch rows); a warp per row.
__global__ void k_perm_rows(const int64_t* __restrict__ rp0, const SegDev* __restrict__ seg,
                            int64_t ch, const int32_t* __restrict__ idx, int64_t m,
                            const int64_t* __restrict__ rp, int32_t* __restrict__ col,
                            float* __restrict__ val) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= m) return;
  const int64_t j = idx[i];
  const SegDev sg = seg[j / ch];
  const int64_t b = rp0[j] - sg.e0, n = rp0[j + 1] - rp0[j], d = rp[i];
  for (int64_t k = lane; k < n; k += 32) {
    col[d + k] = sg.col[b + k];
    val[d + k] = sg.val[b + k];
  }
}

// The system matrix of the rows h->rows (the crystal-pair order), built
// over the rows in list order (rows_d: neighbouring rows are near-parallel
// lines, which the walk handles faster) into one allocation per chunk
// (chunks of a uniform row count).  rp0 (m + 1, list order) gets the row
// pointers; segd (device) the chunk table.
struct ListBuild {
  std::vector<CsrSegment> segs;
  int64_t* rp0 = nullptr;
  SegDev* segd = nullptr;
  int64_t ch = 1, nnz = 0;
  void release(cudaStream_t st) {
    for (const CsrSegment& sg : segs) {
      dev_free(sg.col, st);
      dev_free(sg.val, st);
    }
    segs.clear();
    for (void* q : {(void*)rp0, (void*)segd})
      if (q) dev_free(q, st);
    rp0 = nullptr;
    segd = nullptr;
  }
};

static epet_status build_list_order(const epet_problem* p, const int32_t* rows_d, int64_t m,
                                    int32_t max_row_nnz, ListBuild* b, cudaStream_t st) {
  EPET_CUDA(dev_alloc((void**)&b->rp0, (m + 1) * 8, st));
  EPET_CHECK(build_csr_segments(p, rows_d, m, b->rp0, &b->segs, &b->nnz, max_row_nnz, st));
  b->ch = b->segs.empty() ? 1 : b->segs[0].nr;
  for (size_t k = 0; k < b->segs.size(); k++)
    if (b->segs[k].r0 != (int64_t)k * b->ch || (k + 1 < b->segs.size() && b->segs[k].nr != b->ch))
      return set_error(EPET_ERR_INVALID, "internal: uneven build chunks");
  std::vector<SegDev> hs;
  for (const CsrSegment& sg : b->segs) hs.push_back({sg.col, sg.val, sg.e0});
  EPET_CUDA(dev_alloc((void**)&b->segd, std::max<size_t>(hs.size(), 1) * sizeof(SegDev), st));
  if (!hs.empty())
    EPET_CUDA(cudaMemcpyAsync(b->segd, hs.data(), hs.size() * sizeof(SegDev),
                              cudaMemcpyHostToDevice, st));
  return EPET_OK;
}

// The list-order build moved row by row into h->A in the crystal-pair order
// (exact size; no growth copies).
static epet_status move_to_pair_order(const ListBuild& lb, const int32_t* idx, epet_mlem* h,
                                      cudaStream_t st) {
  const int64_t m = h->m;
  const int64_t nnz = lb.nnz;
  int64_t *len = nullptr, *tmp = nullptr;
  epet_csr B{m, h->V, 0, nullptr, nullptr, nullptr};
  epet_status rc = EPET_OK;
  auto cu = [&](cudaError_t e, const char* what) {
    if (rc == EPET_OK && e != cudaSuccess) rc = cuda_status(e, what);
  };
  cu(dev_alloc((void**)&B.row_ptr, (m + 1) * 8, st), "allocation of A");
  cu(dev_alloc((void**)&B.col, (nnz + 4) * 4, st), "allocation of A");
  cu(dev_alloc((void**)&B.val, (nnz + 4) * 4, st), "allocation of A");
  cu(dev_alloc((void**)&len, std::max<int64_t>(m, 1) * 8, st), "allocation of the row move");
  cu(dev_alloc((void**)&tmp, scan_tmp_elems(m) * 8, st), "allocation of the row move");
  if (rc == EPET_OK && m > 0) {
    k_perm_len<<<ceil_div(m, 256), 256, 0, st>>>(lb.rp0, idx, m, len);
    note_launch();
    rc = exclusive_scan_i64(len, B.row_ptr, m, tmp, st);
    if (rc == EPET_OK) {
      k_perm_rows<<<ceil_div(m * 32, 256), 256, 0, st>>>(lb.rp0, lb.segd, lb.ch, idx, m,
                                                       B.row_ptr, B.col, B.val);
      note_launch();
      cu(cudaGetLastError(), "row move");
    }
  } else if (rc == EPET_OK) {
    cu(cudaMemsetAsync(B.row_ptr, 0, 8, st), "row move");
  }
  // the copies must finish before the caller releases the segments
  cu(cudaStreamSynchronize(st), "row move");
  for (void* q : {(void*)len, (void*)tmp})
    if (q) dev_free(q, st);
  if (rc != EPET_OK) {
    for (void* q : {(void*)B.row_ptr, (void*)B.col, (void*)B.val})
      if (q) dev_free(q, st);
    return rc;
  }
  B.nnz = nnz;
  h->A = B;
  h->capA = nnz;
  return EPET_OK;
}

// s *= num / den where den > 0 (the 16-bit forms' sensitivity).
__global__ void k_scale_by_ratio(float* __restrict__ s, const float* __restrict__ num,
                                 const float* __restrict__ den, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && den[i] > 0.f) s[i] = __fmul_rn(s[i], __fdiv_rn(num[i], den[i]));
}

__global__ void k_fill_u16(uint16_t* x, int64_t n, uint16_t v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

__global__ void k_fill(float* x, int64_t n, float v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

__global__ void k_f64_to_f32(const double* a, int64_t n, float* b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

extern "C" {

epet_status epet_mlem_create(const epet_problem* p, const int32_t* rows_d, const float* y_d,
                             int64_t m, const float* s_d, const epet_mlem_options* opt,
                             epet_mlem** out, epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (!out || m < 0 || (m > 0 && (!rows_d || !y_d)) || !s_d)
    return set_error(EPET_ERR_INVALID, "bad arguments");
  epet_mlem_options o{};
  if (opt) o = *opt;
  if (o.value_format != EPET_VALUES_FP32 && o.value_format != EPET_VALUES_BF16 &&
      o.value_format != EPET_VALUES_FP16)
    return set_error(EPET_ERR_INVALID, "value_format %d", o.value_format);
  cudaStream_t st = (cudaStream_t)stream;
  epet_mlem* h = new epet_mlem();
  h->p = *p;
  h->opt = o;
  h->m = m;
  h->V = (int64_t)p->grid.n[0] * p->grid.n[1] * p->grid.n[2];
  const int64_t V = h->V;
  auto fail = [&](epet_status rc) {
    mlem_free(h);
    return rc;
  };
#define ALLOC(ptr, bytes)                                                    \
  do {                                                                       \
    cudaError_t e_ = dev_alloc((void**)&(ptr), std::max<size_t>(bytes, 8), st); \
    if (e_ != cudaSuccess) return fail(cuda_status(e_, "allocation " #ptr)); \
  } while (0)
  ALLOC(h->rows, m * 4);
  ALLOC(h->y, m * 4);
  ALLOC(h->e, m * 4);
  ALLOC(h->ybar, m * 4);
  if (o.value_format != EPET_VALUES_FP32) ALLOC(h->e16, m * 2);
  ALLOC(h->s, V * 4);
  ALLOC(h->x, V * 4);
  ALLOC(h->xnew, V * 4);
  ALLOC(h->sums, 64);
  if (m > 0) cudaMemcpyAsync(h->y, y_d, m * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(h->s, s_d, V * 4, cudaMemcpyDeviceToDevice, st);
  // sensitivity normalised to sum 1 (reco.cu:181-183)
  {
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(V, 256), 1024));
    double* part = nullptr;
    ALLOC(part, nb * 8);
    epet_status rc = sum_f64(h->s, V, part, nb, h->sums + 2, st);
    if (rc == EPET_OK) rc = launch_normalise(h->s, h->sums + 2, V, h->s, st);
    dev_free(part, st);
    if (rc != EPET_OK) return fail(rc);
  }
  // x = ones / sum(ones) (reco.cu:126-136)
  k_fill<<<ceil_div(V, 256), 256, 0, st>>>(h->x, V, (float)(1.0 / (double)(float)V));
  note_launch();
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(EPET_ERR_CUDA, "fill"));

  if (o.matrix_free) {
    // nothing stored: rows and counts in list order, the fp64 correction image
    if (o.value_format != EPET_VALUES_FP32)
      return fail(set_error(EPET_ERR_INVALID, "matrix_free needs FP32 values"));
    h->opt.use_graph = 0;
    h->opt.autotune = 0;
    if (m > 0) cudaMemcpyAsync(h->rows, rows_d, m * 4, cudaMemcpyDeviceToDevice, st);
    ALLOC(h->c64, V * 8);
    ALLOC(h->part_ll, 1024 * 8);
    ALLOC(h->part_x, sum_blocks(V) * 8);
    h->plan_fwd = default_plan(0.0);
    h->plan_bwd = default_plan(0.0);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(cuda_status(e, "mlem create"));
    *out = h;
    return EPET_OK;
  }
  int32_t* idx = nullptr;  // list index of each row in the new order
  {
    epet_status rc = order_rows(p, rows_d, m, h, st, &idx);
    if (rc != EPET_OK) return fail(rc);
  }
  if (o.layout != EPET_LAYOUT_AUTO && o.layout != EPET_LAYOUT_GROUPED &&
      o.layout != EPET_LAYOUT_CSC) {
    if (idx) dev_free(idx, st);
    return fail(set_error(EPET_ERR_INVALID, "layout %d", o.layout));
  }
  const bool grouped_ok = grouped_supported(V, m);
  if (o.layout == EPET_LAYOUT_GROUPED && !grouped_ok) {
    if (idx) dev_free(idx, st);
    return fail(set_error(EPET_ERR_UNSUPPORTED, "grouped layout: %lld voxels (at most 819,200)",
                          (long long)V));
  }
  // AUTO: the grouped layout for FP32 values; the 16-bit forms keep the
  // CSR and the column-major copy (their grouped pass is bound by shared
  // memory, not by the bytes it saves, and runs slower)
  const bool want_grouped = o.layout == EPET_LAYOUT_GROUPED ||
                            (o.layout == EPET_LAYOUT_AUTO && o.value_format == EPET_VALUES_FP32);
  // the system matrix (rows in the crystal-pair order): the grouped layout
  // reads the list-order build's chunks directly; the CSC layout moves them
  // into one CSR, then makes the column-major copy
  epet_status rc = EPET_OK;
  if (idx) {
    ListBuild lb;
    rc = build_list_order(p, rows_d, m, o.max_row_nnz, &lb, st);
    if (rc == EPET_OK && want_grouped && grouped_ok) {
      RowSource src{lb.rp0, nullptr, nullptr, lb.segd, lb.ch, idx};
      rc = grouped_build(src, m, V, lb.nnz, o.value_format, &h->G, st);
      if (rc == EPET_OK) {
        cudaError_t e = cudaStreamSynchronize(st);  // before the chunks go
        if (e != cudaSuccess) rc = cuda_status(e, "grouped layout");
      }
      h->A = epet_csr{m, V, lb.nnz, nullptr, nullptr, nullptr};
    } else if (rc == EPET_OK) {
      rc = move_to_pair_order(lb, idx, h, st);
    }
    lb.release(st);
    dev_free(idx, st);
  } else {
    rc = build_csr_growable(p, h->rows, m, &h->A, &h->capA, o.max_row_nnz, st);
    if (rc == EPET_OK && want_grouped && grouped_ok)
      rc = grouped_build(RowSource{h->A.row_ptr, h->A.col, h->A.val, nullptr, 1, nullptr}, m, V,
                         h->A.nnz, o.value_format, &h->G, st);
  }
  if (rc != EPET_OK) return fail(rc);
  const int64_t nnz = h->A.nnz;
  if (want_grouped && grouped_ok) {
    if (o.value_format != EPET_VALUES_FP32 && V > 0) {
      // The iterations run with the 16-bit values, whose column sums differ
      // from the FP32 ones by the rounding of the values; an MLEM update
      // x*c/s with s from the FP32 matrix would then drift by that ratio in
      // every iteration.  s is scaled per column by (sum of 16-bit values) /
      // (sum of FP32 values) over the measured rows, the sensitivity of the
      // matrix the iterations use.
      float *q = nullptr, *f = nullptr;
      ALLOC(q, V * 4);
      ALLOC(f, V * 4);
      rc = grouped_column_sums(h->G, true, q, st);
      if (rc == EPET_OK) rc = grouped_column_sums(h->G, false, f, st);
      if (rc == EPET_OK) {
        k_scale_by_ratio<<<ceil_div(V, 256), 256, 0, st>>>(h->s, q, f, V);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) rc = set_error(EPET_ERR_CUDA, "sensitivity ratio");
      }
      dev_free(q, st);
      dev_free(f, st);
      if (rc != EPET_OK) return fail(rc);
    }
    grouped_drop_fp32(&h->G, st);
    EPET_CUDA(cudaStreamSynchronize(st));
    h->grouped = true;
    // the grouped layout holds the matrix: the CSR's arrays go (nnz stays)
    for (void** q : {(void**)&h->A.row_ptr, (void**)&h->A.col, (void**)&h->A.val}) {
      if (*q) dev_free(*q, st);
      *q = nullptr;
    }
    h->plan_fwd = RowPlan{32, 1, num_sms(), false};  // reported: one warp per group
    h->plan_bwd = h->G.plan_cols;
    ALLOC(h->part_ll, 1024 * 8);
    ALLOC(h->part_x, sum_blocks(V) * 8);
    if (o.autotune) {
      // the slot sums' launch shape (from the cache when this shape was
      // tuned before; else one pass fills the slots, then the candidates
      // run the real, idempotent, epilogue)
      const double avg = V ? (double)h->G.nslots / V : 0.0;
      if (!tune_lookup(4, V, h->G.nslots, h->G.ngroups, &h->G.plan_cols))
        rc = grouped_pass(h->G, h->x, h->y, h->ybar, st);
      if (rc == EPET_OK)
        rc = tune_rows(
            4, V, h->G.nslots, h->G.ngroups, avg,
            [&](const RowPlan& pl) {
              return launch_sums(pl, h->G.cg_ptr, h->G.cg_slot, h->G.partial, h->V,
                                 EpiMlemUpdate{h->x, h->s, h->xnew, nullptr}, nullptr, st);
            },
            st, &h->G.plan_cols);
      if (rc != EPET_OK) return fail(rc);
      h->plan_bwd = h->G.plan_cols;
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(cuda_status(e, "mlem create"));
    *out = h;
    return EPET_OK;
  }
  ALLOC(h->At.col_ptr, (V + 1) * 8);
  ALLOC(h->At.row, nnz * 4);
  ALLOC(h->At.val, nnz * 4);
  rc = epet_csr_to_csc(&h->A, &h->At, nullptr, 0, stream);
  if (rc != EPET_OK) return fail(rc);
  if (o.value_format != EPET_VALUES_FP32) {
    // 16-bit forms of A and A^T (the column-major copy viewed as A^T's CSR);
    // the 32-bit arrays are released afterwards
    epet_csr At_as_csr{V, m, nnz, h->At.col_ptr, h->At.row, h->At.val};
    struct {
      const epet_csr* src;
      epet_csr16* dst;
      int64_t rows;
    } jobs[2] = {{&h->A, &h->A16, m}, {&At_as_csr, &h->At16, V}};
    for (auto& j : jobs) {
      int64_t* cnt = nullptr;
      ALLOC(cnt, (j.rows + 1) * 8);
      int64_t n16 = 0;
      rc = epet_csr16_count(j.src, cnt, &n16, stream);
      dev_free(cnt, st);
      if (rc != EPET_OK) return fail(rc);
      ALLOC(j.dst->row_ptr, (j.rows + 1) * 8);
      ALLOC(j.dst->base, csr16_capacity(n16) / 8 * 4);  // one base per 8-entry chunk
      ALLOC(j.dst->scale, j.rows * 4);
      ALLOC(j.dst->delta, csr16_capacity(n16) * 2);
      ALLOC(j.dst->q, csr16_capacity(n16) * 2);
      j.dst->nnz = csr16_capacity(n16);
      rc = epet_csr_compress(j.src, o.value_format, j.dst, stream);
      if (rc != EPET_OK) return fail(rc);
    }
    // The transpose product uses the 16-bit column-major values; scale s by
    // the ratio of their column sums to the FP32 ones over the measured
    // rows, so the update x*c/s does not drift by the rounding of the values
    // (see the grouped layout above).
    if (V > 0 && m > 0) {
      float *ones = nullptr, *q = nullptr, *f = nullptr;
      uint16_t* ones16 = nullptr;
      ALLOC(ones, m * 4);
      ALLOC(ones16, m * 2);
      ALLOC(q, V * 4);
      ALLOC(f, V * 4);
      k_fill<<<ceil_div(m, 256), 256, 0, st>>>(ones, m, 1.f);
      note_launch();
      k_fill_u16<<<ceil_div(m, 256), 256, 0, st>>>(ones16, m, (uint16_t)0x3f80u);  // BF16 1.0
      note_launch();
      rc = launch_rows(default_plan((double)nnz / V), h->At.col_ptr, h->At.row, h->At.val, ones, V,
                       EpiKeep{f}, nullptr, st);
      if (rc == EPET_OK)
        rc = launch_rows16<EpiKeep, uint16_t>(&h->At16, ones16, EpiKeep{q}, nullptr, st);
      if (rc == EPET_OK) {
        k_scale_by_ratio<<<ceil_div(V, 256), 256, 0, st>>>(h->s, q, f, V);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) rc = set_error(EPET_ERR_CUDA, "sensitivity ratio");
      }
      EPET_CUDA(cudaStreamSynchronize(st));
      for (void* b : {(void*)ones, (void*)ones16, (void*)q, (void*)f}) dev_free(b, st);
      if (rc != EPET_OK) return fail(rc);
    }
    EPET_CUDA(cudaStreamSynchronize(st));
    dev_free(h->A.col, st); h->A.col = nullptr;
    dev_free(h->A.val, st); h->A.val = nullptr;
    dev_free(h->At.row, st); h->At.row = nullptr;
    dev_free(h->At.val, st); h->At.val = nullptr;
  }
  h->plan_fwd = default_plan(m ? (double)nnz / m : 0.0);
  h->plan_bwd = default_plan(V ? (double)nnz / V : 0.0);
  ALLOC(h->part_ll, 1024 * 8);
  ALLOC(h->part_x, sum_blocks(V) * 8);
  if (o.autotune && o.value_format == EPET_VALUES_FP32) {
    // both products are idempotent (they write e / ybar and xnew / partials
    // from x, y, s): the candidates run the real epilogues
    rc = tune_rows(
        0, m, nnz, V, m ? (double)nnz / m : 0.0,
        [&](const RowPlan& pl) {
          return launch_rows(pl, h->A.row_ptr, h->A.col, h->A.val, h->x, h->m,
                             EpiMlemForward{h->y, h->e, h->ybar}, nullptr, st);
        },
        st, &h->plan_fwd);
    if (rc == EPET_OK)
      rc = tune_rows(
          1, V, nnz, m, V ? (double)nnz / V : 0.0,
          [&](const RowPlan& pl) {
            return launch_rows(pl, h->At.col_ptr, h->At.row, h->At.val, h->e, h->V,
                               EpiMlemUpdate{h->x, h->s, h->xnew, nullptr}, nullptr, st);
          },
          st, &h->plan_bwd);
    if (rc != EPET_OK) return fail(rc);
  }
#undef ALLOC
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(cuda_status(e, "mlem create"));
  *out = h;
  return EPET_OK;
}

epet_status epet_mlem_destroy(epet_mlem* h) {
  if (h) cudaDeviceSynchronize();
  mlem_free(h);
  return EPET_OK;
}

epet_status epet_mlem_iterate(epet_mlem* h, int32_t nit, double* loglik_h,
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
      if (e == cudaSuccess) rc = mlem_iteration(h, cap);
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
    for (int it = 0; it < nit; it++) EPET_CHECK(mlem_iteration(h, st));
  }
  if (loglik_h) {
    if (h->m > 0) {
      const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(h->m, 256), 1024));
      EPET_CHECK(poisson_loglik(h->y, h->ybar, h->m, h->part_ll, nb, h->sums + 0, st));
    } else {
      EPET_CUDA(cudaMemsetAsync(h->sums, 0, 8, st));
    }
    double s0 = 0.0;
    EPET_CUDA(cudaMemcpyAsync(&s0, h->sums, 8, cudaMemcpyDeviceToHost, st));
    EPET_CUDA(cudaStreamSynchronize(st));
    *loglik_h = s0;
  }
  return EPET_OK;
}

epet_status epet_mlem_correction(epet_mlem* h, float* c_d, epet_stream_t stream) {
  if (!h || !c_d) return set_error(EPET_ERR_INVALID, "bad arguments");
  return mlem_correction(h, c_d, (cudaStream_t)stream);
}

epet_status epet_mlem_update(epet_mlem* h, const float* c_d, epet_stream_t stream) {
  if (!h || !c_d) return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  k_update_c<float><<<ceil_div(h->V, 256), 256, 0, st>>>(h->x, c_d, h->s, h->V, h->xnew);
  EPET_LAUNCHED();
  return launch_sum_normalise(h->xnew, h->V, h->part_x, h->x, st);
}

epet_status epet_mlem_loglik(epet_mlem* h, double* loglik_h, epet_stream_t stream) {
  if (!h || !loglik_h) return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  if (h->m > 0) {
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(h->m, 256), 1024));
    EPET_CHECK(poisson_loglik(h->y, h->ybar, h->m, h->part_ll, nb, h->sums + 0, st));
  } else {
    EPET_CUDA(cudaMemsetAsync(h->sums, 0, 8, st));
  }
  double s0 = 0.0;
  EPET_CUDA(cudaMemcpyAsync(&s0, h->sums, 8, cudaMemcpyDeviceToHost, st));
  EPET_CUDA(cudaStreamSynchronize(st));
  *loglik_h = s0;
  return EPET_OK;
}

float* epet_mlem_image(epet_mlem* h) { return h ? h->x : nullptr; }

epet_status epet_mlem_get_image(const epet_mlem* h, float* x_d, epet_stream_t stream) {
  if (!h || !x_d) return set_error(EPET_ERR_INVALID, "bad arguments");
  EPET_CUDA(cudaMemcpyAsync(x_d, h->x, h->V * 4, cudaMemcpyDeviceToDevice,
                            (cudaStream_t)stream));
  return EPET_OK;
}

epet_status epet_mlem_set_image(epet_mlem* h, const float* x_d, epet_stream_t stream) {
  if (!h || !x_d) return set_error(EPET_ERR_INVALID, "bad arguments");
  EPET_CUDA(cudaMemcpyAsync(h->x, x_d, h->V * 4, cudaMemcpyDeviceToDevice,
                            (cudaStream_t)stream));
  return EPET_OK;
}

epet_status epet_mlem_stats(const epet_mlem* h, int64_t* nnz_h, int64_t* bytes_h) {
  if (!h) return set_error(EPET_ERR_INVALID, "bad arguments");
  if (nnz_h) *nnz_h = h->A.nnz;
  if (bytes_h && h->grouped) {
    // pass: values (4 or 2 bytes) and ranks (2) per entry, row pointers,
    // y, ybar, row scales (16-bit), per slot the table, the x gather and
    // the correction written; slot sums: column pointers, per slot the slot
    // index, a one and the correction, x and s read, xnew written; image
    // sum and normalisation: xnew read twice, x written
    const int64_t np = h->G.npad, m = h->m, V = h->V, ns = h->G.nslots;  // (padded entries)
    const int64_t bv = h->G.fmt == EPET_VALUES_FP32 ? 4 : 2;
    *bytes_h = (bv + 2) * np + 8 * (m + 1) + 8 * m + (bv == 2 ? 4 * m : 0) + 12 * ns +
               8 * (V + 1) + 12 * ns + 8 * V + 4 * V + 8 * V + 4 * V;
  } else if (bytes_h && h->opt.matrix_free) {
    // no matrix: the pass writes and reads the rays (24 bytes each) and the
    // channel geometry (224 bytes per row), reads y and writes ybar, reads x
    // and the fp64 c (zeroed, accumulated), writes xnew, then sums and scales
    const int64_t m = h->m, V = h->V, R = h->p.nrays;
    *bytes_h = 2 * 24 * R * m + 2 * 224 * m + 8 * m + 4 * V + 3 * 8 * V + 4 * V + 4 * V +
               4 * V + 4 * V;
  } else if (bytes_h && h->opt.value_format != EPET_VALUES_FP32) {
    // per stored entry 4 bytes (offset + value) and a 4-byte base per 8;
    // per row a pointer and a scale (12 bytes); vectors as in FP32
    const int64_t m = h->m, V = h->V;
    // (e written and gathered as 2-byte BF16)
    *bytes_h = 4 * h->A16.nnz + h->A16.nnz / 2 + 12 * m + 4 * m + 4 * V + 2 * m + 4 * m +
               4 * h->At16.nnz + h->At16.nnz / 2 + 12 * V + 2 * m + 4 * V + 4 * V + 4 * V +
               4 * V + 4 * V;
  } else if (bytes_h) {
    // forward: values+columns, row pointers, y, x (once), e written;
    // transpose: values+rows, column pointers, e (once), x, s, xnew written;
    // sum/normalise: xnew read, x written.
    const int64_t nnz = h->A.nnz, m = h->m, V = h->V;
    *bytes_h = 8 * nnz + 8 * (m + 1) + 4 * m + 4 * V + 4 * m +
               8 * nnz + 8 * (V + 1) + 4 * m + 4 * V + 4 * V + 4 * V +
               4 * V + 4 * V;
  }
  return EPET_OK;
}

epet_status epet_mlem_plan(const epet_mlem* h, int32_t plan_h[6]) {
  if (!h || !plan_h) return set_error(EPET_ERR_INVALID, "bad arguments");
  const RowPlan* ps[2] = {&h->plan_fwd, &h->plan_bwd};
  for (int k = 0; k < 2; k++) {
    plan_h[3 * k + 0] = ps[k]->G;
    plan_h[3 * k + 1] = ps[k]->vec ? ps[k]->U : 0;
    plan_h[3 * k + 2] = ps[k]->grid;
  }
  return EPET_OK;
}

epet_status epet_mlem_layout(const epet_mlem* h, int32_t* layout_h) {
  if (!h || !layout_h) return set_error(EPET_ERR_INVALID, "bad arguments");
  *layout_h = h->opt.matrix_free ? -1 : (h->grouped ? EPET_LAYOUT_GROUPED : EPET_LAYOUT_CSC);
  return EPET_OK;
}

epet_status epet_trim_memory(size_t keep_bytes) { return trim_memory(keep_bytes); }

epet_status epet_sensitivity(const epet_problem* p, const int32_t* rows_d, int64_t m,
                             float* s_d, double* s64_d, int32_t max_row_nnz, void* ws,
                             size_t ws_bytes, epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (!s_d || m < 0 || (m > 0 && !rows_d)) return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t V = (int64_t)p->grid.n[0] * p->grid.n[1] * p->grid.n[2];
  double* s64 = s64_d;
  if (!s64) EPET_CUDA(dev_alloc((void**)&s64, V * 8, st));
  EPET_CUDA(cudaMemsetAsync(s64, 0, V * 8, st));
  epet_status rc = column_sums(p, rows_d, m, s64, max_row_nnz, ws, ws_bytes, st);
  if (rc == EPET_OK) {
    k_f64_to_f32<<<ceil_div(V, 256), 256, 0, st>>>(s64, V, s_d);
    note_launch();
    // normalised to sum 1 as backprojection.cu:157-161
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(V, 256), 1024));
    double* part = nullptr;
    cudaError_t e = dev_alloc((void**)&part, (nb + 1) * 8, st);
    rc = e == cudaSuccess ? sum_f64(s_d, V, part, nb, part + nb, st)
                          : cuda_status(e, "allocation of the sum");
    if (rc == EPET_OK) rc = launch_normalise(s_d, part + nb, V, s_d, st);
    if (part) dev_free(part, st);
  }
  if (!s64_d) dev_free(s64, st);
  return rc;
}

}  // extern "C"
