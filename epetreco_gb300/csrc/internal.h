// internal.h -- host-side declarations shared between the library's units.
#pragma once
#include "common.cuh"

namespace epet {

Geo make_geo(const epet_problem& p);
epet_status launch_rays(const Geo& G, const int32_t* rows, int64_t m,
                        float* out, bool uniforms_only, cudaStream_t st);

// Exclusive scan of int64 counts (n entries) into out[n+1]; out[n] = total.
// tmp must hold scan_tmp_elems(n) int64.
size_t scan_tmp_elems(int64_t n);
epet_status exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n,
                               int64_t* tmp, cudaStream_t st);

// Radix sort histogram size (int64 entries) for n items (sort.cu).
size_t radix_hist_elems(int64_t n);
// The column-major order of a CSR's entries (nnz entries, n columns, at
// most 2^31 - 1 entries): each column's entries' positions, ascending, at
// pos[col_ptr[v] ..]; col_ptr has n + 1 entries.  Neither rows nor values
// are read.
epet_status csr_to_csc_positions(int64_t nnz, int64_t n, const int32_t* col, int64_t* col_ptr,
                                 uint32_t* pos, cudaStream_t st);

// Row walk configuration chosen for a problem (per-row accumulator size).
int auto_row_capacity(const epet_problem& p);
int64_t exact_rows_total();
int64_t overflow_rows_total();

// Candidate compaction and per-candidate values (workqueue.cu).
epet_status launch_workqueue_count(const Geo& G, const int32_t* rows, int64_t m,
                                   int64_t* row_count, cudaStream_t st);
epet_status launch_workqueue_fill(const Geo& G, const int32_t* rows, int64_t m,
                                  const int64_t* row_off, int32_t* cnl, int32_t* vxl,
                                  cudaStream_t st);
epet_status launch_values(const Geo& G, const float* rays, int64_t m,
                          const int64_t* row_ptr, const int32_t* col, float* val,
                          bool exact, cudaStream_t st);
// Rows left to the per-candidate path: in CSR mode (mode 0) each row's kept
// entries go to compact buffers (row i of the list at off[i], any length),
// row_len[row] is set and src_idx[row] = -2 - i tells the row gather to read
// them there; the caller frees the buffers (release()) after that gather.
struct ExactRows {
  int64_t* off = nullptr;
  int32_t* col = nullptr;
  float* val = nullptr;
  void release(cudaStream_t st);
};
epet_status exact_rows_apply(const Geo& G, const int32_t* rows, const int32_t* ex_rows,
                             int64_t n_ex, int mode, int32_t* row_len, int32_t* src_idx,
                             ExactRows* keep, const float* x, float* y, const float* e,
                             float* c, double* s64, const float* ycnt, double* c64,
                             cudaStream_t st);
epet_status column_sums(const epet_problem* p, const int32_t* rows_d, int64_t m,
                        double* s64, int32_t max_row_nnz, void* ws, size_t ws_bytes,
                        cudaStream_t st);

}  // namespace epet
