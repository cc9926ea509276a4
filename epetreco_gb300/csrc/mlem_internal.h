// mlem_internal.h -- the reconstruction object shared by mlem.cu (one
// problem) and batch.cu (many problems iterated by batched launches).
#pragma once
#include <vector>
#include "common.cuh"
#include "spmv.cuh"

namespace epet {
// Grouped layout of a reconstruction's matrix (grouped.cu): consecutive rows
// in groups whose distinct columns fit a per-warp shared table.
constexpr int kGroupCap = 1536;  // distinct columns of a group held in shared memory
constexpr int kGroupWarps = 16;  // warps (groups in flight) per block of the iteration
struct GroupDesc {
  int32_t r0, r1;  // rows [r0, r1)
  int32_t tb, nd;  // table slots [tb, tb + nd)
};
struct GroupedMatrix {
  int fmt = 0;  // EPET_VALUES_*
  int64_t n = 0;                // columns (voxels)
  int64_t ngroups = 0, nslots = 0, npad = 0;
  GroupDesc* groups = nullptr;
  int32_t* table = nullptr;     // each group's distinct columns, ascending
  int64_t* row_ptr = nullptr;   // rows padded to whole 4-entry chunks
  float* val32 = nullptr;       // values (FP32 form; 16-bit forms: until the sensitivity is fixed)
  uint16_t* val16 = nullptr;    // 16-bit forms: values / row scale
  float* scale = nullptr;
  uint16_t* loc = nullptr;      // per entry: rank of its column in its group's table
  int64_t* cg_ptr = nullptr;    // per column: its slots (group order) at cg_slot[cg_ptr[v] ..]
  int32_t* cg_slot = nullptr;
  float* ones = nullptr;        // nslots ones (batched form: its slot sums run on the row kernel)
  float* partial = nullptr;     // per slot: the group's share of c = A^T e
  int32_t* wide = nullptr;      // ids of the groups of one row wider than the shared tables
  int64_t nwide = 0;
  std::vector<int32_t> wide_h;  // the same on the host
  RowPlan plan_cols;
};
bool grouped_supported(int64_t V, int64_t m);
// One chunk of a build held in its own allocation (entries e0 onwards).
struct SegDev {
  const int32_t* col;
  const float* val;
  int64_t e0;
};
// Where the grouped build reads row r of the matrix (rows in the
// reconstruction's order): a CSR (segs null: entries rp[r] .. rp[r+1] of
// col / val), or the chunks of a build over the rows in another order (row r
// is built row q = idx[r], entries rp[q] .. rp[q+1] of the chunk q / ch).
struct RowSource {
  const int64_t* rp;
  const int32_t* col;
  const float* val;
  const SegDev* segs;
  int64_t ch;
  const int32_t* idx;
};
// Builds the grouped layout of an m x n matrix with nnz entries; the source
// is left as it is (the caller may release it afterwards).
epet_status grouped_build(const RowSource& A, int64_t m, int64_t n, int64_t nnz,
                          int value_format, GroupedMatrix* G, cudaStream_t st);
// ybar = A x, e = y / ybar and the groups' shares of A^T e into G.partial
// (one kernel, two when the matrix has wide groups: grouped_pass_kernels).
int grouped_pass_kernels(const GroupedMatrix& G);
epet_status grouped_pass(const GroupedMatrix& G, const float* x, const float* y, float* ybar,
                         cudaStream_t st);
void grouped_free(GroupedMatrix* G, cudaStream_t st);
// Allocates and fills G->ones (the batched form's slot sums) if not yet there.
epet_status grouped_ones(GroupedMatrix* G, cudaStream_t st);
// Releases the FP32 values of a 16-bit form.
void grouped_drop_fp32(GroupedMatrix* G, cudaStream_t st);
// Column sums of the values over the matrix's rows into out[V]: the stored
// 16-bit values dequantised (quantised) or the FP32 values (while they
// exist); fixed summation order.
epet_status grouped_column_sums(const GroupedMatrix& G, bool quantised, float* out,
                                cudaStream_t st);
// Batched form: a descriptor per problem (grouped_batch_desc_bytes() each,
// written by grouped_batch_desc into a host buffer and copied to the
// device) and one pass over all problems' groups (gstart: device prefix of
// the problems' group counts, np + 1 entries; wide: the global ids of the
// wide groups, nwide of them, passed by a second kernel).
size_t grouped_batch_desc_bytes();
void grouped_batch_desc(const GroupedMatrix& G, const float* x, const float* y, float* ybar,
                        void* out);
epet_status grouped_pass_batch(const void* desc, const int64_t* gstart, int np,
                               int64_t total_groups, const int32_t* wide, int64_t nwide,
                               cudaStream_t st);
}  // namespace epet

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
  bool grouped = false;   // the matrix in the grouped layout (no column-major copy)
  epet::GroupedMatrix G;
  epet::RowPlan plan_fwd, plan_bwd;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_kernels = 0;  // kernels in the captured iteration
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

