/* epet_oracle.h -- CPU restatement of the epetreco MLEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA library is
 * compared against; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline legs load it.  The product never links or calls it.
 *
 * Every function follows a reference file:line (paths relative to the
 * reference's src/ tree).  Floating-point expressions keep the reference's
 * operand order and are compiled without contraction (-ffp-contract=off), so
 * each float operation rounds once, as the reference's host build does.
 * Parity of this restatement is pinned against the reference's own code
 * built for the host (oracle/ref/, see tests/test_oracle_vs_ref.py) and
 * against the fixtures in tests/golden/.
 *
 * Two places where the reference's float results depend on the build:
 *  - sinf/cosf of the rotation angle: the CUDA library computes the per-angle
 *    table on the device; the oracle takes that table as an input (eo_trig
 *    NULL -> computed here with the host libm);
 *  - the cuRAND uniforms: supplied by the caller (dumped from the device by
 *    the library's epet_dump_uniforms), never generated here. */
#ifndef EPET_ORACLE_H
#define EPET_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* DefaultMeasurementSetup<T> field set (MeasurementSetup.hpp:124-164). */
typedef struct {
  float pos0x, pos1x;
  int na, n0z, n0y, n1z, n1y;
  float da, segx, segy, segz;
} eo_setup;

/* DefaultVoxelGrid<T> field set (VoxelGrid.hpp:88-200). */
typedef struct {
  float o[3], d[3];
  int n[3];
} eo_grid;

/* ---- linear index maps (MeasurementSetupLinIndex.hpp, VoxelGridLinIndex.hpp) */
void eo_channel_decode(const eo_setup* s, int cnl, int out5[5]); /* ida,0z,0y,1z,1y */
int eo_channel_encode(const eo_setup* s, int ida, int id0z, int id0y, int id1z,
                      int id1y);
int64_t eo_nchannels(const eo_setup* s);
void eo_voxel_decode(const eo_grid* g, int vxl, int out3[3]);
int eo_voxel_encode(const eo_grid* g, int ix, int iy, int iz);

/* ---- geometry */
/* sin/cos of each angle, interleaved [na][2]; host libm. */
void eo_trig_table(const eo_setup* s, float* sc);
/* Crystal box coordinates -> world (MeasurementSetupTrafo2CartCoord.hpp:56-104
 * for det 0, :219-270 for det 1).  sc = {sin, cos} of the channel's angle. */
void eo_trafo(const eo_setup* s, const float sc[2], int det, int iz, int iy,
              const float box[3], float out[3]);
/* Candidate test: distance of the voxel centre from the crystal-centre line
 * below half the summed diagonals (getSystemMatrixDeviceOnly.cu:25-77,
 * getWorkqueue.hpp:50-79, distancePointLine.h:19-73). */
int eo_candidate(const eo_setup* s, const eo_grid* g, const float* trig,
                 int cnl, int vxl);
/* Slab chord length of a line with a box (getSystemMatrixFromWorkqueue.cu:
 * 24-69; identical copy getSystemMatrixDeviceOnly.cu:88-133).  Axes where the
 * two ray points coincide are left out of the slab test, as in the
 * reference (its masked min/max, ChordsCalc_lowlevel.hpp:30-156). */
float eo_intersection_length(const float vxl6[6], const float ray6[6]);
/* Rays of one channel from its uniforms rnd[nrays][6]: r0..r2 -> crystal 0,
 * r3..r5 -> crystal 1 (getSystemMatrixFromWorkqueue.cu:196-230). */
void eo_rays(const eo_setup* s, const float* trig, int cnl, int nrays,
             const float* rnd, float* rays);
/* Voxel box corners (getSystemMatrixFromWorkqueue.cu:150-160). */
void eo_voxel_box(const eo_grid* g, int vxl, float box6[6]);

/* ---- system matrix */
#define EO_SUM_SEQUENTIAL 0 /* a += len_r in ray order, fp32 (the reference) */
#define EO_SUM_EXACT 1      /* exact sum of the fp32 lengths, rounded once */

/* Element (cnl, vxl) from the channel's rays[nrays][6] (the workqueue kernel
 * body, getSystemMatrixFromWorkqueue.cu:160-244). */
float eo_sm_value(const eo_grid* g, const float* rays, int nrays, int vxl,
                  int sum_mode);

/* Candidate scan over a measurement list and the whole grid, list-major and
 * voxel-minor (getWorkqueue.hpp:187-223).  Writes up to cap pairs; returns
 * the total number found. */
int64_t eo_workqueue(const eo_setup* s, const eo_grid* g, const float* trig,
                     const int32_t* list, int64_t n_list, int32_t* out_cnl,
                     int32_t* out_vxl, int64_t cap);
/* Per-row candidate counts (row_count[n_list]); returns the total. */
int64_t eo_workqueue_counts(const eo_setup* s, const eo_grid* g,
                            const float* trig, const int32_t* list,
                            int64_t n_list, int64_t* row_count);

/* Values for a workqueue: rnd_rows[n_list][nrays][6] are the uniforms of each
 * list row; wq_row[i] is the list row of entry i. */
void eo_sm_values_wq(const eo_setup* s, const eo_grid* g, const float* trig,
                     const int32_t* list, int nrays, const float* rnd_rows,
                     int64_t n_wq, const int32_t* wq_row,
                     const int32_t* wq_vxl, int sum_mode, float* out_val);

/* Full build over a measurement list: rows = list entries, columns = voxel
 * ids ascending, entries = candidates whose value is non-zero (the
 * reference's getSystemMatrix + cooSort + coo2csr + csr2ecsr pipeline with
 * stored zeros dropped).  row_ptr[n_list+1]; writes up to cap entries;
 * returns nnz. */
int64_t eo_sm_build_csr(const eo_setup* s, const eo_grid* g, const float* trig,
                        const int32_t* list, int64_t n_list, int nrays,
                        const float* rnd_rows, int sum_mode, int64_t* row_ptr,
                        int32_t* col, float* val, int64_t cap);
/* One-pass form of eo_sm_build_csr: start returns a handle and the nnz;
 * finish writes row_ptr[n_list+1], col, val and frees the handle. */
void* eo_sm_build_start(const eo_setup* s, const eo_grid* g, const float* trig,
                        const int32_t* list, int64_t n_list, int nrays,
                        const float* rnd_rows, int sum_mode, int64_t* nnz_out);
void eo_sm_build_finish(void* h, int64_t* row_ptr, int32_t* col, float* val);

/* ---- sparse format conversions */
/* Stable lexicographic (row, col) sort carrying values (cooSort.hpp:26-71). */
void eo_coo_sort(float* val, int32_t* row, int32_t* col, int64_t n);
/* Row pointer of a row-sorted COO (cusparseWrapper.hpp:38-45). */
void eo_coo2csr(const int32_t* row, int64_t nnz, int64_t m, int64_t* csr);
/* ecsr[i] = csr[yRowId[i]], ecsr[nnzr] = csr[m] (convertCsr2Ecsr.hpp:34-47). */
void eo_csr2ecsr(int64_t* ecsr, const int32_t* yRowId, int64_t nnzr,
                 const int64_t* csr, int64_t m);

/* ---- SpMV (csrmv.hpp:25-36 semantics): y = alpha*op(A)*x + beta*y.
 * Dot products accumulate in double and round once to float. */
void eo_csrmv(int trans, int64_t m, int64_t n, const int64_t* row_ptr,
              const int32_t* col, const float* val, float alpha,
              const float* x, float beta, float* y);
void eo_csrmv_f64(int trans, int64_t m, int64_t n, const int64_t* row_ptr,
                  const int32_t* col, const float* val, double alpha,
                  const double* x, double beta, double* y);

/* ---- MLEM element-wise operations (mlemOperations.hpp:22-139) */
void eo_divides(float* r, const float* a, const float* b, int64_t n);
void eo_divides_multiplies(float* r, const float* a, const float* b,
                           const float* c, int64_t n);
void eo_scales(float* x, float alpha, int64_t n);
double eo_sum(const float* x, int64_t n); /* double accumulation */

/* MLEM (reco.cu:209-281): per iteration c = A^T (y / A x) over the rows,
 * x = x*c/s (s==0 -> 1), x /= sum(x).  s must be normalised by the caller.
 * fp32 arithmetic with double dot products; rows with A x == 0 contribute
 * nothing (the reference divides without a guard, mlemOperations.hpp:31). */
void eo_mlem(int64_t m, int64_t V, const int64_t* row_ptr, const int32_t* col,
             const float* val, const float* y, const float* s, float* x,
             int nit);
void eo_mlem_f64(int64_t m, int64_t V, const int64_t* row_ptr,
                 const int32_t* col, const float* val, const double* y,
                 const double* s, double* x, int nit);
void eo_mlem_f64_trace(int64_t m, int64_t V, const int64_t* rp, const int32_t* col,
                       const float* val, const double* y, const double* s, double* x,
                       int nit, double* trace);
/* s = A^T 1 normalised to sum 1 (backprojection.cu:113-161 with an all-ones
 * measurement). */
void eo_sensitivity(int64_t m, int64_t V, const int64_t* row_ptr,
                    const int32_t* col, const float* val, float* s);
/* Poisson log-likelihood sum_i y_i log(ybar_i) - ybar_i over ybar_i > 0. */
double eo_poisson_loglik(int64_t m, const float* y, const float* ybar);

/* ---- chunking helpers (wrappers.hpp:410-446) */
int64_t eo_n_in_chunk(int64_t id_chunk, int64_t n_all, int64_t n_full_chunk);
int64_t eo_chunk_ptr(int64_t id_chunk, int64_t n_full_chunk);
int64_t eo_n_chunks(int64_t max_nnz, int64_t max_n_chunk);

#ifdef __cplusplus
}
#endif
#endif
