// mlem_internal.h -- the reconstruction object shared by mlem.cu (one
// problem) and batch.cu (many problems iterated by batched launches).
#pragma once
#include <vector>
#include "common.cuh"
#include "spmv.cuh"

struct epet_mlem {
  epet_problem p;
  epet_mlem_options opt;
  int64_t m = 0, V = 0;
  int32_t* rows = nullptr;
  float *y = nullptr, *s = nullptr, *x = nullptr, *xnew = nullptr, *e = nullptr;
  float* ybar = nullptr;  // last forward projection
  uint16_t* e16 = nullptr;  // ratio e as BF16 bits (16-bit forms)
  epet_csr A{};
  epet_csc At{};
  epet_csr16 A16{}, At16{};  // 16-bit forms (value_format != FP32)
  int64_t capA = 0;
  double *part_ll = nullptr, *part_x = nullptr, *sums = nullptr;
  double* c64 = nullptr;  // correction image of the matrix-free schedule
  epet::RowPlan plan_fwd, plan_bwd;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace epet {
// A chunk of a system matrix built into its own allocation: rows r0 ..
// r0+nr-1, global entries e0 .. e0+n-1 at col[0..n) / val[0..n).
struct CsrSegment {
  int64_t r0, nr, e0, n;
  int32_t* col;
  float* val;
};
// Build of the rows with each chunk's entries in a new allocation (no
// growth copies); row_ptr (m+1, caller-allocated) gets the global row
// pointers.  On failure the segments made so far are still listed.
epet_status build_csr_segments(const epet_problem* p, const int32_t* rows, int64_t m,
                               int64_t* row_ptr, std::vector<CsrSegment>* segs, int64_t* nnz,
                               int32_t max_row_nnz, cudaStream_t st);
epet_status build_csr_growable(const epet_problem* p, const int32_t* rows, int64_t m,
                               epet_csr* out, int64_t* cap, int32_t max_row_nnz,
                               cudaStream_t st);
}

