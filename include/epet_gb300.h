/* epet_gb300.h -- C ABI of the GB300 (sm_103a) implementation of epetreco's
 * MLEM hot path.
 *
 * The reference has no plugin or FFI layer: its operator surface is a set of
 * header templates called directly by its drivers (reco.cu, backprojection.cu,
 * pureSMCalculation.cu) plus three __constant__ symbols.  Each entry point
 * below names the reference interface it replaces (file:line, relative to
 * the reference's src/ tree).  include/epet_gb300_shim.hpp re-exposes the
 * reference's own C++ names on top of this ABI.
 *
 * Conventions
 *  - Every function returns an epet_status and never throws or exits;
 *    epet_last_error() gives a message for the calling thread.
 *  - Pointers named *_d are device pointers; the caller owns every buffer.
 *    Calls are stream-ordered on the given stream (0 = legacy default) and
 *    do not synchronise unless documented ("synchronous").
 *  - Functions taking (void* ws, size_t ws_bytes) need device scratch: pass
 *    a caller buffer of at least the size reported by the matching
 *    *_workspace_size(), or ws = NULL to let the library allocate it
 *    stream-ordered (cudaMallocAsync) and free it before returning.  The
 *    system-matrix calls take extra stream-ordered memory from the library's
 *    pool for the rows they redo (a window over capacity, an axis-parallel
 *    ray), whose count is known only during the call; epet_coo_sort_noalloc
 *    allocates nothing.
 *  - Index types: channel and voxel ids int32, element counts and row
 *    pointers int64 (the reference's int counts overflow at the full 52^3 x
 *    5.1M-channel size). */
#ifndef EPET_GB300_H
#define EPET_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* epet_stream_t; /* == cudaStream_t */

typedef enum {
  EPET_OK = 0,
  EPET_ERR_INVALID = 1,     /* bad argument */
  EPET_ERR_CAPACITY = 2,    /* output too small; required size reported */
  EPET_ERR_CUDA = 3,        /* CUDA runtime error */
  EPET_ERR_UNSUPPORTED = 4, /* geometry/format outside the supported range */
  EPET_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
  EPET_ERR_OVERFLOW = 6     /* reserved: no call returns it (rows over the
                               window capacity are redone at their size) */
} epet_status;

/* DefaultMeasurementSetup<float> (MeasurementSetup.hpp:124-164): two planar
 * heads of n0z x n0y and n1z x n1y crystals of seg{x,y,z} metres, centres at
 * x = pos0x / pos1x, rotated about y in na steps of da degrees. */
typedef struct {
  float pos0x, pos1x;
  int32_t na, n0z, n0y, n1z, n1y;
  float da, segx, segy, segz;
} epet_setup;

/* DefaultVoxelGrid<float> (VoxelGrid.hpp:88-200): origin o, pitch d, count n. */
typedef struct {
  float o[3];
  float d[3];
  int32_t n[3];
} epet_grid;

/* Ray generators (RayGenerators.hpp): EPET_RAYS_RANDOM is RandRayGen (:15-40),
 * six cuRAND uniforms per ray from the channel's generator; EPET_RAYS_REGULAR
 * is ReguRayGen (:46-66), every coordinate 0.5, i.e. each of the nrays rays is
 * the line between the two crystal centres (nrays = 1 gives the same matrix up
 * to the rounding of the mean, at 1/nrays of the cost). */
enum { EPET_RAYS_RANDOM = 0, EPET_RAYS_REGULAR = 1 };

/* Replaces the process-global __constant__ grid_const / setup_const /
 * nrays_const (device_constant_memory.hpp:14-26) with a value passed to each
 * call; seed is RANDOM_SEED (1251 in getSystemMatrixFromWorkqueue.cu:22).
 * ray_mode (EPET_RAYS_*) picks the generator the reference selects with the
 * RayGen template argument of systemMatrixCalculation (wrappers.hpp:172); it
 * fills what would otherwise be padding, and 0 (a zero-initialised struct)
 * is the random generator. */
typedef struct {
  epet_setup setup;
  epet_grid grid;
  int32_t nrays;
  int32_t ray_mode;
  uint64_t seed;
} epet_problem;

/* CSR over a measurement list ("ECSR": row i is channel rows[i]).  col holds
 * voxel ids ascending within each row. */
typedef struct {
  int64_t m;        /* rows */
  int64_t n;        /* columns (voxels) */
  int64_t nnz;
  int64_t* row_ptr; /* m+1, device */
  int32_t* col;     /* nnz, device */
  float* val;       /* nnz, device */
} epet_csr;

/* 16-bit storage of a CSR (value_format 1 = BF16, 2 = FP16): about 4.5 bytes
 * per entry.  A row is stored as chunks of 8 entries (rows padded with
 * zero-valued entries of offset 0): chunk c has a column base base[c] (its
 * smallest column), the entries' 16-bit offsets delta (col = base[c] +
 * delta_k) and 16-bit values q (value = scale[r] * q_k, scale = the row's
 * largest value).  Columns need not ascend within a row; a chunk ends early
 * before an entry that would widen its column range to 65536.  row_ptr
 * counts stored entries (multiples of 8).  delta and q are read with 16-byte
 * loads: 16-byte aligned; nnz = their capacity in entries, base holds nnz/8
 * chunks, scale m rows. */
#define EPET_VALUES_FP32 0
#define EPET_VALUES_BF16 1
#define EPET_VALUES_FP16 2
typedef struct {
  int64_t m, n;
  int64_t nnz;       /* in: capacity of delta/q (entries); out: stored entries */
  int64_t* row_ptr;  /* m+1 */
  int32_t* base;     /* nnz / 8 (one per chunk) */
  float* scale;      /* m */
  uint16_t* delta;
  uint16_t* q;
  int32_t format;
} epet_csr16;

/* Column-major copy of an epet_csr: col_ptr[n+1], row ids ascending within a
 * column (used by the scatter-free back-projection). */
typedef struct {
  int64_t m, n, nnz;
  int64_t* col_ptr;
  int32_t* row;
  float* val;
} epet_csc;

/* ------------------------------------------------------------- runtime */
const char* epet_last_error(void);
const char* epet_version(void);
/* Number of kernels this library has launched in the process (CUDA-graph
 * replays count the kernels they contain); for launch accounting. */
long long epet_launch_count(void);
/* Number of device allocations the library has made itself in the process
 * (from its memory pool; caller workspaces are not counted).  For
 * accounting and tests; no counterpart in the reference. */
long long epet_device_allocations(void);
/* Fault injection for tests of the error paths (no counterpart in the
 * reference): after `after` more device allocations every allocation the
 * library makes fails with EPET_ERR_CUDA (out of memory), on the host side,
 * without touching the device; after < 0 switches it off. */
epet_status epet_debug_fail_allocations(long long after);
/* Problem checks: index ranges fit int32, nrays >= 1, positive pitches,
 * ray_mode one of EPET_RAYS_*. */
epet_status epet_problem_validate(const epet_problem* p);

/* ------------------------------------------------------------- geometry */
/* sin/cos of each angle, interleaved [na][2], computed on the device as the
 * reference's transform does (MeasurementSetupTrafo2CartCoord.hpp:67-68). */
epet_status epet_trig_table(const epet_problem* p, float* sc_d,
                            epet_stream_t stream);
/* The cuRAND uniforms of each listed channel, out_d[m][nrays][6]
 * (curand_init(seed, channel, 0) then 6 curand_uniform per ray, as in
 * getSystemMatrixFromWorkqueue.cu:189-204); 0.5 everywhere for
 * EPET_RAYS_REGULAR. */
epet_status epet_dump_uniforms(const epet_problem* p, const int32_t* rows_d,
                               int64_t m, float* out_d, epet_stream_t stream);
/* Diagnostics (no counterpart in the reference): rows of system-matrix builds
 * since the library was loaded whose window exceeded the shared-memory
 * capacity and were redone with their exact size, and rows handed to the
 * per-candidate path (a ray with two equal coordinates). */
epet_status epet_build_counters(int64_t* overflow_rows_h, int64_t* exact_rows_h);
/* Work measure of the chord walk (no counterpart in the reference): the
 * total over the listed channels' rays of the grid cells each ray crosses
 * (1 + the grid planes it passes inside the grid), in *steps_h and, when
 * row_steps_d != NULL, per row in row_steps_d[m].  Synchronous. */
epet_status epet_ray_steps(const epet_problem* p, const int32_t* rows_d, int64_t m,
                           int64_t* row_steps_d, int64_t* steps_h, epet_stream_t stream);
/* Library self-test (no counterpart in the reference): compares the walk
 * kernel's reciprocal-based correctly rounded division with the hardware's
 * IEEE division on n seeded operand pairs; *mismatches_h counts differing
 * results (0 expected).  Synchronous. */
epet_status epet_selftest_division(int64_t n, uint64_t seed, int64_t* mismatches_h,
                                   epet_stream_t stream);
/* World-coordinate rays out_d[m][nrays][6] (RandRayGen, RayGenerators.hpp:
 * 15-40 with the per-channel seeding of getSystemMatrixFromWorkqueue.cu;
 * ReguRayGen, :46-66, for EPET_RAYS_REGULAR). */
epet_status epet_rays(const epet_problem* p, const int32_t* rows_d, int64_t m,
                      float* out_d, epet_stream_t stream);

/* ------------------------------------------------ candidate compaction */
/* Replaces getWorkqueue (getWorkqueue.hpp:187-223) and the candidate test +
 * compaction of getSystemMatrix (getSystemMatrixDeviceOnly.cu:25-77,
 * :304-491): all (channel, voxel) pairs with dist(voxel centre, crystal-
 * centre line) < sum of half diagonals, list-major and voxel-minor.
 * row_count_d[m] receives per-row counts; *total_h the sum (synchronous). */
epet_status epet_workqueue_count(const epet_problem* p, const int32_t* rows_d,
                                 int64_t m, int64_t* row_count_d,
                                 int64_t* total_h, epet_stream_t stream);
/* Fills the pairs given row_off_d[m+1] (exclusive scan of the counts). */
epet_status epet_workqueue_fill(const epet_problem* p, const int32_t* rows_d,
                                int64_t m, const int64_t* row_off_d,
                                int32_t* wq_cnl_d, int32_t* wq_vxl_d,
                                epet_stream_t stream);
/* Values for a row-grouped workqueue (CSR pattern over the list): each
 * element is the mean over nrays of the slab chord length, summed in ray
 * order in fp32 exactly as getSystemMatrixFromWorkqueue (:96-261), so it is
 * bit-identical to the reference's per-channel-seeded values. */
epet_status epet_sm_values(const epet_problem* p, const int32_t* rows_d,
                           int64_t m, const int64_t* row_ptr_d,
                           const int32_t* col_d, float* val_d, void* ws,
                           size_t ws_bytes, epet_stream_t stream);
size_t epet_sm_values_workspace_size(const epet_problem* p, int64_t m);

/* ------------------------------------------------ system matrix (hot path) */
/* Replaces systemMatrixCalculation (wrappers.hpp:166-247: getSystemMatrix +
 * cooSort + coo2csr + csr2ecsr) with one fused build: per channel the rays
 * are traced through the grid, chord lengths accumulate exactly per voxel,
 * candidates with a non-zero value are emitted in voxel order straight into
 * CSR (rows = rows_d, in order).  Stored zeros of the reference are dropped.
 * out->row_ptr/col/val are caller buffers; cap = capacity of col/val.
 * Synchronous.  On EPET_ERR_CAPACITY *nnz_h holds the required nnz and
 * row_ptr is complete.  max_row_nnz: the walk's per-row window capacity in
 * cells (0 = sized from a sample of the rows); rows with a larger window are
 * redone with their own size, so it changes speed and memory, not results
 * (EPET_ERR_UNSUPPORTED if a window does not fit in shared memory). */
epet_status epet_sm_build(const epet_problem* p, const int32_t* rows_d,
                          int64_t m, epet_csr* out, int64_t cap,
                          int64_t* nnz_h, int32_t max_row_nnz, void* ws,
                          size_t ws_bytes, epet_stream_t stream);
size_t epet_sm_build_workspace_size(const epet_problem* p, int64_t m,
                                    int32_t max_row_nnz);
/* Matrix-free projections (no matrix stored): y_d[m] = A x_d (forward), or
 * c_d[V] += A^T e_d (back-projection, fp32 atomics).  Same element values as
 * epet_sm_build. */
epet_status epet_project_forward(const epet_problem* p, const int32_t* rows_d,
                                 int64_t m, const float* x_d, float* y_d,
                                 int32_t max_row_nnz, void* ws,
                                 size_t ws_bytes, epet_stream_t stream);
epet_status epet_project_back(const epet_problem* p, const int32_t* rows_d,
                              int64_t m, const float* e_d, float* c_d,
                              int32_t max_row_nnz, void* ws, size_t ws_bytes,
                              epet_stream_t stream);
/* One MLEM pass without a stored matrix, the reference's schedule of a
 * system matrix rebuilt in every iteration (reco.cu:216-254: the chunk's
 * matrix, csrmv, divides, transposed csrmv with beta = 1) done by one chord
 * walk per row: ybar = A x (into ybar_d, may be NULL), e = y / ybar (0 where
 * ybar == 0), c64_d[V] += A^T e accumulated in fp64 (the caller zeroes it).
 * Same element values and the same A x as epet_project_forward. */
epet_status epet_project_mlem(const epet_problem* p, const int32_t* rows_d,
                              int64_t m, const float* x_d, const float* y_d,
                              float* ybar_d, double* c64_d, int32_t max_row_nnz,
                              void* ws, size_t ws_bytes, epet_stream_t stream);
/* Sensitivity image (backprojection.cu:113-161 fed an all-ones measurement):
 * s_d[V] = column sums of A over the listed channels, accumulated in fp64
 * (s64_d, may be NULL) and normalised to sum 1 in s_d. */
epet_status epet_sensitivity(const epet_problem* p, const int32_t* rows_d,
                             int64_t m, float* s_d, double* s64_d,
                             int32_t max_row_nnz, void* ws, size_t ws_bytes,
                             epet_stream_t stream);

/* ------------------------------------------------------ sparse formats */
/* cooSort (cooSort.hpp:53-71): stable in-place sort of COO triples by
 * (row, col), values follow. */
epet_status epet_coo_sort(float* val_d, int32_t* row_d, int32_t* col_d,
                          int64_t n, void* ws, size_t ws_bytes,
                          epet_stream_t stream);
size_t epet_coo_sort_workspace_size(int64_t n);
/* epet_coo_sort for callers that cannot let the library allocate device
 * memory: a host application whose own allocator owns all of the device's
 * memory, or an integration whose memory budget is fixed at start-up.  No
 * counterpart in the reference.  Allocates nothing: its scratch is a
 * file-scope device array of 7 MiB, held by every GPU that loads the library
 * until the process exits, so n is limited to 262,144 triples
 * (EPET_ERR_CAPACITY above that).  Stream-ordered, and nothing is read back
 * to the host: ids sort in signed order (negative ids included, as the
 * reference's comparator orders them), where epet_coo_sort rejects negative
 * ids.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current, and again when another
 * context has been made current; make that first call before any stream
 * capture begins.  The address is not looked up again after cudaDeviceReset
 * of a device whose context handle stays the same: do not use this call on a
 * device after resetting it in the same process.  All calls share the one
 * array, which keeps the last call's contents (the call initialises what it
 * reads): calls that overlap on the GPU (different streams, or several host
 * threads) race on it and must be serialised by the caller. */
epet_status epet_coo_sort_noalloc(float* val_d, int32_t* row_d, int32_t* col_d,
                                  int64_t n, epet_stream_t stream);
/* convertCoo2Csr (cusparseWrapper.hpp:38-45): row pointer of row-sorted COO. */
epet_status epet_coo2csr(const int32_t* row_d, int64_t nnz, int64_t m,
                         int64_t* csr_d, epet_stream_t stream);
/* convertCsr2Ecsr (convertCsr2Ecsr.hpp:34-47): ecsr[i] = csr[yRowId[i]],
 * ecsr[nnzr] = csr[m]; one gather kernel instead of 3 copies per row. */
epet_status epet_csr2ecsr(int64_t* ecsr_d, const int32_t* yrow_d, int64_t nnzr,
                          const int64_t* csr_d, int64_t m,
                          epet_stream_t stream);
/* Column-major copy (stable: row ids ascending within each column). */
epet_status epet_csr_to_csc(const epet_csr* a, epet_csc* out, void* ws,
                            size_t ws_bytes, epet_stream_t stream);
size_t epet_csr_to_csc_workspace_size(int64_t m, int64_t n, int64_t nnz);

/* ---------------------------------------------------------------- SpMV */
/* CSRmv<float>::operator() (csrmv.hpp:25-36): y = alpha*op(A)*x + beta*y,
 * trans = 0 (NON_TRANSPOSE) or 1 (TRANSPOSE).  The transpose reads the CSC
 * when csc != NULL (scatter-free, deterministic), else scatters with fp32
 * atomics into y.  The launch shape of the row products comes from the
 * autotuner: the first call for a matrix shape (rows, nnz, columns) times
 * the candidate shapes into scratch memory (y is written once) and the
 * process keeps the winner; while the stream is being captured, or with
 * EPET_AUTOTUNE=0 in the environment, a fixed heuristic shape is used
 * (results then depend on the inputs alone; shapes change fp32 rounding
 * only). */
epet_status epet_csrmv(int trans, const epet_csr* a, const epet_csc* csc,
                       float alpha, const float* x_d, float beta, float* y_d,
                       epet_stream_t stream);

/* 16-bit layout: per-row stored-entry counts (row_len16_d[m]) and their
 * total. */
epet_status epet_csr16_count(const epet_csr* a, int64_t* row_len16_d,
                             int64_t* nnz16_h, epet_stream_t stream);
/* Converts a CSR (or, given a column-major copy viewed as the CSR of A^T,
 * the transpose) into the 16-bit layout; out->nnz = capacity on input. */
epet_status epet_csr_compress(const epet_csr* a, int32_t format, epet_csr16* out,
                              epet_stream_t stream);
/* y = alpha * A x + beta * y over the 16-bit layout (FP32 accumulation). */
epet_status epet_csr16_mv(const epet_csr16* a, float alpha, const float* x_d,
                          float beta, float* y_d, epet_stream_t stream);

/* -------------------------------------------------- MLEM element-wise ops */
/* divides (mlemOperations.hpp:22-32): r = a / b, no guard (as reference). */
epet_status epet_divides(float* r_d, const float* a_d, const float* b_d,
                         int64_t n, epet_stream_t stream);
/* dividesMultiplies (mlemOperations.hpp:38-79): r = a*b/c, c == 0 -> 1. */
epet_status epet_divides_multiplies(float* r_d, const float* a_d,
                                    const float* b_d, const float* c_d,
                                    int64_t n, epet_stream_t stream);
/* scales (mlemOperations.hpp:85-124): x *= alpha. */
epet_status epet_scales(float* x_d, float alpha, int64_t n,
                        epet_stream_t stream);
/* sum (mlemOperations.hpp:133-139) in fp64 into a device scalar. */
epet_status epet_sum_f64(const float* x_d, int64_t n, double* out_d,
                         epet_stream_t stream);

/* ------------------------------------------- int32-index compatibility */
/* For callers holding the reference's int row pointers (mallocD_SystemMatrix,
 * wrappers.hpp:64-74).  Same semantics as the int64 forms above. */
epet_status epet_coo2csr_i32(const int32_t* row_d, int64_t nnz, int64_t m,
                             int32_t* csr_d, epet_stream_t stream);
epet_status epet_csr2ecsr_i32(int32_t* ecsr_d, const int32_t* yrow_d,
                              int64_t nnzr, const int32_t* csr_d, int64_t m,
                              epet_stream_t stream);
/* CSRmv<float>::operator() with the reference's argument list (csrmv.hpp:
 * 25-36): int32 row pointer; the transpose scatters with fp32 atomics. */
epet_status epet_csrmv_i32(int trans, int64_t m, int64_t n, int64_t nnz,
                           float alpha, const float* val_d,
                           const int32_t* row_ptr_d, const int32_t* col_d,
                           const float* x_d, float beta, float* y_d,
                           epet_stream_t stream);
epet_status epet_index_i64_to_i32(const int64_t* a_d, int64_t n, int32_t* b_d,
                                  epet_stream_t stream);
epet_status epet_index_i32_to_i64(const int32_t* a_d, int64_t n, int64_t* b_d,
                                  epet_stream_t stream);
/* out_d[k] = rows_d[i] for every entry k of row i (the COO row ids that
 * systemMatrixCalculation leaves in aCnlId_devi, wrappers.hpp:172-247). */
epet_status epet_csr_expand_rows(const int64_t* row_ptr_d, int64_t m,
                                 const int32_t* rows_d, int32_t* out_d,
                                 epet_stream_t stream);
/* Process-wide geometry for drivers written against the reference's
 * __constant__ grid_const/setup_const/nrays_const (device_constant_memory.hpp:
 * 14-26, set with cudaMemcpyToSymbol in reco.cu:64-72); seed 1251. */
epet_status epet_set_constant_geometry(const epet_setup* setup,
                                       const epet_grid* grid, int32_t nrays);
epet_status epet_get_constant_geometry(epet_problem* out);

/* ------------------------------------------------------------- memory */
/* Device memory the library allocates itself (reconstruction objects,
 * workspaces not passed by the caller) comes from a stream-ordered pool per
 * device that keeps freed memory reserved, so setting up a reconstruction of
 * the same size again maps no new memory.  This call returns the reserve
 * above keep_bytes to the device (synchronises every device the library
 * used).  No counterpart in the reference (it allocates with cudaMalloc and
 * frees nothing between iterations). */
epet_status epet_trim_memory(size_t keep_bytes);

/* ---------------------------------------------------------- MLEM driver */
/* One reconstruction (reco.cu:209-281) held on the device: measured rows,
 * their counts, the system matrix (in the layout of opt->layout, or none
 * with opt->matrix_free), sensitivity and image. */
typedef struct epet_mlem epet_mlem;

typedef struct {
  int32_t max_row_nnz; /* 0 = auto */
  int32_t use_graph;   /* capture one iteration in a CUDA graph */
  int32_t value_format; /* EPET_VALUES_FP32 / _BF16 / _FP16 (16-bit values + row scale) */
  int32_t autotune;    /* 1: time candidate launch shapes of the two products on this
                          matrix at create (cached per matrix shape for the process);
                          0: a fixed heuristic shape (results then depend only on the
                          inputs, not on timings).  FP32 values only. */
  int32_t matrix_free; /* 1: store no matrix; every iteration recomputes the chords
                          (epet_project_mlem), as the reference rebuilds its matrix in
                          every iteration.  FP32 values; use_graph and autotune are
                          ignored (the pass reads per-chunk counters back). */
  int32_t layout;      /* EPET_LAYOUT_*: how a stored matrix is held */
} epet_mlem_options;

/* Layouts of a reconstruction's stored matrix.  GROUPED: rows cut into
 * groups of consecutive rows (crystal-pair order) whose distinct columns fit
 * a per-warp table in shared memory; each entry keeps its value and a 2-byte
 * rank of its column in the group's table (6 bytes per entry in FP32, 4 in
 * BF16/FP16); one pass over the entries per iteration gives A x, the ratio
 * and A^T e, the latter summed per column in a fixed order; supported up to
 * 819,200 voxels.  CSC: the CSR and its column-major copy (16 bytes per entry
 * in FP32), the transpose product over the copy.  AUTO: GROUPED for FP32
 * values where supported, else CSC (the 16-bit forms run faster in CSC: their
 * grouped pass is bound by shared memory).  Both are deterministic.  The
 * 16-bit forms scale the sensitivity per column by the ratio of the column
 * sums of the values their transpose product uses to the FP32 column sums
 * (over the measured rows), so the iterations do not drift by the rounding
 * of the values. */
enum { EPET_LAYOUT_AUTO = 0, EPET_LAYOUT_GROUPED = 1, EPET_LAYOUT_CSC = 2 };

/* Builds the system matrix for the measured rows (rows_d channel ids, in
 * any order, with y_d > 0), keeps y, s (normalised here) and x = ones/V.
 * Internally the rows are stored in crystal-pair order (angle, then the sums
 * of the two crystals' y and z indices, then the first crystal), so a
 * shuffled row list gives the same object.  Synchronous. */
epet_status epet_mlem_create(const epet_problem* p, const int32_t* rows_d,
                             const float* y_d, int64_t m, const float* s_d,
                             const epet_mlem_options* opt, epet_mlem** out,
                             epet_stream_t stream);
epet_status epet_mlem_destroy(epet_mlem* h);
/* Runs nit iterations: c = A^T (y / A x); x = x*c/s; x /= sum(x).  With
 * loglik_h != NULL the fp64 Poisson log-likelihood of the last forward
 * projection is returned (synchronous then). */
epet_status epet_mlem_iterate(epet_mlem* h, int32_t nit, double* loglik_h,
                              epet_stream_t stream);
/* Row-sharded reconstructions (reco.cu:216-260: row chunks dealt to the MPI
 * ranks, the correction image summed with MPI_Allreduce, then the update on
 * every rank).  epet_mlem_correction runs the forward product (e = y / A x,
 * ybar kept) and writes c_d[V] = A^T e over this object's rows, leaving the
 * image unchanged; the caller sums c_d over the shards (e.g. an all-reduce);
 * epet_mlem_update then applies x = x*c/s (s == 0 -> 1) and x /= sum(x).  On
 * one shard, correction + update is one iteration, bit for bit.
 * epet_mlem_loglik: the fp64 Poisson log-likelihood of the last forward
 * projection over this object's rows (synchronous); shards add theirs. */
epet_status epet_mlem_correction(epet_mlem* h, float* c_d, epet_stream_t stream);
epet_status epet_mlem_update(epet_mlem* h, const float* c_d, epet_stream_t stream);
epet_status epet_mlem_loglik(epet_mlem* h, double* loglik_h, epet_stream_t stream);
/* Image access (device pointer valid until destroy), copy-out, statistics
 * (with matrix_free: nnz 0, and the bytes of the pass's rays, channel
 * geometry and vectors). */
float* epet_mlem_image(epet_mlem* h);
epet_status epet_mlem_get_image(const epet_mlem* h, float* x_d, epet_stream_t stream);
epet_status epet_mlem_set_image(epet_mlem* h, const float* x_d,
                                epet_stream_t stream);
epet_status epet_mlem_stats(const epet_mlem* h, int64_t* nnz_h,
                            int64_t* bytes_per_iter_h);
/* Launch shapes of the two products: plan_h[0..2] = forward lanes per row,
 * 16-byte chunks per lane and round (0 = lanes interleave single entries),
 * persistent grid (0 = one block per tile); plan_h[3..5] the same for the
 * transpose. */
epet_status epet_mlem_plan(const epet_mlem* h, int32_t plan_h[6]);
/* The layout the matrix is held in (EPET_LAYOUT_GROUPED or EPET_LAYOUT_CSC;
 * -1 with matrix_free). */
epet_status epet_mlem_layout(const epet_mlem* h, int32_t* layout_h);

/* ---------------------------------------------- batched reconstructions */
/* Many independent reconstructions (each its own geometry, grid, rays,
 * measured rows and sensitivity) iterated together: every step of an
 * iteration is ONE kernel launch over all problems' rows or voxels, and the
 * iteration (forward product + e = y/(Ax), transpose product + x*c/s,
 * per-problem fp64 image sums, normalisation: four launches, five when a
 * grouped-layout problem has a row wider than the shared tables) is captured in
 * one CUDA graph.  Launch shapes come from the autotuner unless
 * opt->autotune == 0.  The reference runs one reconstruction per process
 * (reco.cu:209-281); there is no batched counterpart.  FP32 values. */
typedef struct epet_mlem_batch epet_mlem_batch;

/* Arrays of nprob entries on the host; rows_d[i], y_d[i], s_d[i] are device
 * pointers as for epet_mlem_create.  Synchronous. */
epet_status epet_mlem_batch_create(int32_t nprob, const epet_problem* problems,
                                   const int32_t* const* rows_d, const int64_t* m,
                                   const float* const* y_d, const float* const* s_d,
                                   const epet_mlem_options* opt, epet_mlem_batch** out,
                                   epet_stream_t stream);
epet_status epet_mlem_batch_destroy(epet_mlem_batch* h);
/* nit iterations of every problem; loglik_h (nprob entries or NULL) as in
 * epet_mlem_iterate. */
epet_status epet_mlem_batch_iterate(epet_mlem_batch* h, int32_t nit, double* loglik_h,
                                    epet_stream_t stream);
epet_status epet_mlem_batch_get_image(const epet_mlem_batch* h, int32_t i, float* x_d,
                                      epet_stream_t stream);
/* Problem i as a single reconstruction (owned by the batch: do not destroy);
 * iterating it alone runs the plain per-problem kernels on the same arrays. */
epet_mlem* epet_mlem_batch_member(epet_mlem_batch* h, int32_t i);
/* Totals over the problems; plan_h as epet_mlem_plan (may be NULL). */
epet_status epet_mlem_batch_stats(const epet_mlem_batch* h, int64_t* nnz_h,
                                  int64_t* bytes_per_iter_h, int32_t plan_h[6]);

/* ---------------------------------------------------------------- HDF5 files
 * The reference's file formats without libhdf5 (host code, host buffers).
 * Reading: superblocks of version 0-3, groups as symbol tables or compact
 * links, datasets with contiguous or compact storage of IEEE floats or
 * integers of either byte order (converted to float); other files return
 * EPET_ERR_UNSUPPORTED.  Writing: superblock 0, the root group as a symbol
 * table, one contiguous little-endian float dataset, as libhdf5 writes it. */

/* Shape of dataset `name` ("a/b" for nested groups): *ndims_h and up to 8
 * entries of dims_h (either may be NULL). */
epet_status epet_h5_dataset_shape(const char* path, const char* name, int32_t* ndims_h,
                                  int64_t* dims_h);
/* All n elements of dataset `name` as float, in the file's (row-major)
 * order; EPET_ERR_CAPACITY if n is not its element count.  H5Reader::read
 * (H5Reader.hpp:39-70) reads the measurement "messung" this way. */
epet_status epet_h5_read_f32(const char* path, const char* name, float* out_h, int64_t n);
/* readHDF5_MeasVct (wrappers.hpp:311-333): the channels of "messung" whose
 * value is not zero, ascending, as row ids rows_h and values y_h (up to
 * `capacity` of each); *m_h = their number, *nchannels_h = the dataset's
 * element count (either may be NULL).  With rows_h or y_h NULL only the
 * counts are returned; EPET_ERR_CAPACITY when m > capacity. */
epet_status epet_h5_read_measurement(const char* path, int32_t* rows_h, float* y_h,
                                     int64_t capacity, int64_t* m_h, int64_t* nchannels_h);
/* A measurement file: the 1-D float dataset "messung" of n counts (the
 * reference reads it through H5Reader.hpp:16; it has no writer for it). */
epet_status epet_h5_write_measurement(const char* path, const float* y_h, int64_t n);
/* H5DensityWriter::write (H5DensityWriter.hpp:140-199): the 3-D float
 * dataset "density" [n0][n1][n2] of the image x_h (voxel (i,j,k) at
 * i*n1*n2 + j*n2 + k, the library's order) with float attributes xmin, ymin,
 * zmin (= grid->o) and xmax, ymax, zmax (= o + n * d), int attributes xnbin,
 * ynbin, znbin. */
epet_status epet_h5_write_density(const char* path, const float* x_h, const epet_grid* grid);
/* A restart point: the "density" file of epet_h5_write_density plus an int
 * attribute "iteration" (the iterations done).  The reference's per-iteration
 * "<it>_<out>" files (reco.cu:284-291) are its restart points, fed back as the
 * guess (reco.cu:114-137), without the count. */
epet_status epet_h5_write_checkpoint(const char* path, const float* x_h, const epet_grid* grid,
                                     int64_t iteration);
/* A numeric scalar attribute attr of dataset name, as double;
 * EPET_ERR_INVALID when the dataset has none of that name. */
epet_status epet_h5_read_attribute(const char* path, const char* name, const char* attr,
                                   double* value_h);
/* Reads a "density" file: the image (n elements; x_h may be NULL) and the
 * grid from its attributes (pitch = (max - min) / nbin; grid_h may be NULL). */
epet_status epet_h5_read_density(const char* path, float* x_h, int64_t n, epet_grid* grid_h);

#ifdef __cplusplus
}
#endif
#endif
