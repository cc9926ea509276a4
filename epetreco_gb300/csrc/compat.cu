// compat.cu -- int32-index variants of the sparse operators, for callers
// that hold the reference's int row pointers (ECSR int[m+1], wrappers.hpp:
// 64-74), and the constant-geometry slot of the C++ drop-in header.
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "internal.h"
#include "spmv.cuh"

namespace epet {

__global__ void k_coo2csr_i32(const int32_t* __restrict__ row, int64_t nnz, int64_t m,
                              int32_t* __restrict__ csr) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r > m) return;
  int64_t lo = 0, hi = nnz;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (row[mid] < r) lo = mid + 1;
    else hi = mid;
  }
  csr[r] = (int32_t)lo;
}

__global__ void k_csr2ecsr_i32(int32_t* ecsr, const int32_t* yrow, int64_t nnzr,
                               const int32_t* csr, int64_t m) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nnzr) ecsr[i] = csr[yrow[i]];
  if (i == nnzr) ecsr[nnzr] = csr[m];
}

__global__ void k_ptr_i32_to_i64(const int32_t* a, int64_t n, int64_t* b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

__global__ void k_ptr_i64_to_i32(const int64_t* a, int64_t n, int32_t* b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (int32_t)a[i];
}

// Row ids of every entry: out[k] = rows[i] for k in [ptr[i], ptr[i+1]).
__global__ void k_expand_channels(const int64_t* __restrict__ ptr, int64_t m,
                                  const int32_t* __restrict__ rows, int32_t* __restrict__ out) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= m) return;
  const int32_t c = rows[i];
  for (int64_t k = ptr[i] + lane; k < ptr[i + 1]; k += 32) out[k] = c;
}

}  // namespace epet

using namespace epet;

// The process-global geometry of epet_set_constant_geometry (the reference's
// __constant__ symbols are process-global too); read and written under a lock.
static std::mutex g_const_mu;
static epet_problem g_const_problem;
static bool g_const_set = false;

extern "C" {

epet_status epet_coo2csr_i32(const int32_t* row_d, int64_t nnz, int64_t m, int32_t* csr_d,
                             epet_stream_t stream) {
  if (nnz < 0 || m < 0 || !csr_d || (nnz > 0 && !row_d) || nnz > INT32_MAX)
    return set_error(EPET_ERR_INVALID, "bad arguments");
  k_coo2csr_i32<<<ceil_div(m + 1, 256), 256, 0, (cudaStream_t)stream>>>(row_d, nnz, m, csr_d);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status epet_csr2ecsr_i32(int32_t* ecsr_d, const int32_t* yrow_d, int64_t nnzr,
                              const int32_t* csr_d, int64_t m, epet_stream_t stream) {
  if (nnzr < 0 || m < 0 || !ecsr_d || !csr_d || (nnzr > 0 && !yrow_d))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  k_csr2ecsr_i32<<<ceil_div(nnzr + 1, 256), 256, 0, (cudaStream_t)stream>>>(ecsr_d, yrow_d,
                                                                             nnzr, csr_d, m);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status epet_index_i64_to_i32(const int64_t* a_d, int64_t n, int32_t* b_d,
                                  epet_stream_t stream) {
  if (n < 0 || (n > 0 && (!a_d || !b_d))) return set_error(EPET_ERR_INVALID, "bad arguments");
  if (n == 0) return EPET_OK;
  k_ptr_i64_to_i32<<<ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(a_d, n, b_d);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status epet_index_i32_to_i64(const int32_t* a_d, int64_t n, int64_t* b_d,
                                  epet_stream_t stream) {
  if (n < 0 || (n > 0 && (!a_d || !b_d))) return set_error(EPET_ERR_INVALID, "bad arguments");
  if (n == 0) return EPET_OK;
  k_ptr_i32_to_i64<<<ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(a_d, n, b_d);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status epet_csr_expand_rows(const int64_t* row_ptr_d, int64_t m, const int32_t* rows_d,
                                 int32_t* out_d, epet_stream_t stream) {
  if (m < 0 || (m > 0 && (!row_ptr_d || !rows_d || !out_d)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  if (m == 0) return EPET_OK;
  k_expand_channels<<<ceil_div(m * 32, 256), 256, 0, (cudaStream_t)stream>>>(row_ptr_d, m,
                                                                              rows_d, out_d);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status epet_csrmv_i32(int trans, int64_t m, int64_t n, int64_t nnz, float alpha,
                           const float* val_d, const int32_t* row_ptr_d, const int32_t* col_d,
                           const float* x_d, float beta, float* y_d, epet_stream_t stream) {
  if (m < 0 || n < 0 || nnz < 0 || !row_ptr_d || !x_d || !y_d || (nnz > 0 && (!val_d || !col_d)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  int64_t* rp = nullptr;
  EPET_CUDA(dev_alloc((void**)&rp, (m + 1) * 8, st));
  k_ptr_i32_to_i64<<<ceil_div(m + 1, 256), 256, 0, st>>>(row_ptr_d, m + 1, rp);
  note_launch();
  epet_csr a{m, n, nnz, rp, const_cast<int32_t*>(col_d), const_cast<float*>(val_d)};
  epet_status rc = epet_csrmv(trans, &a, nullptr, alpha, x_d, beta, y_d, stream);
  dev_free(rp, st);
  return rc;
}

epet_status epet_set_constant_geometry(const epet_setup* setup, const epet_grid* grid,
                                       int32_t nrays) {
  if (!setup || !grid) return set_error(EPET_ERR_INVALID, "bad arguments");
  epet_problem p{};
  p.setup = *setup;
  p.grid = *grid;
  p.nrays = nrays;
  p.seed = 1251;
  EPET_CHECK(epet_problem_validate(&p));
  std::lock_guard<std::mutex> lock(g_const_mu);
  g_const_problem = p;
  g_const_set = true;
  return EPET_OK;
}

epet_status epet_get_constant_geometry(epet_problem* out) {
  if (!out) return set_error(EPET_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lock(g_const_mu);
  if (!g_const_set)
    return set_error(EPET_ERR_INVALID, "no constant geometry set (epet_set_constant_geometry)");
  *out = g_const_problem;
  return EPET_OK;
}

}  // extern "C"
