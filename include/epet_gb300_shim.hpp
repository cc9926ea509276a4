/* epet_gb300_shim.hpp -- the reference's C++ operator names on top of the
 * epet_gb300 C ABI, so drivers written against epetreco's headers
 * (reco.cu, backprojection.cu, pureSMCalculation.cu) build against the GB300
 * library.  Include it BEFORE any reference header: it defines the include
 * guards of the headers it replaces (cooSort.hpp, cusparseWrapper.hpp,
 * convertCsr2Ecsr.hpp, csrmv.hpp, mlemOperations.hpp), so a later include of
 * those becomes a no-op.
 *
 * Differences a driver sees (each is stated where it applies below):
 *  - geometry: call epetSetConstantGeometry(grid, setup, nrays) where the
 *    reference copies to its __constant__ symbols (reco.cu:64-72);
 *  - systemMatrixCalculation stores only non-zero values (the reference also
 *    stores zero-valued candidates); nnz_devi grows by the non-zeros;
 *  - rays are seeded per channel (curand_init(1251, channel, 0), as the
 *    reference's getSystemMatrixFromWorkqueue), so values are reproducible;
 *    the reference's production kernel seeds per thread and is not; the
 *    RayGen argument of systemMatrixCalculation selects the generator
 *    (ReguRayGen: regular rays, anything else: RandRayGen);
 *  - errors throw cudaException after printing the library's message, like
 *    HANDLE_ERROR (CUDA_HandleError.hpp:17-31).
 * Operations are synchronous where the reference's are (it synchronises after
 * every call). */
#ifndef EPET_GB300_SHIM_HPP
#define EPET_GB300_SHIM_HPP

#include <cuda_runtime.h>
#include <cusparse.h>

#include <cstdint>
#include <exception>
#include <iostream>

#include "epet_gb300.h"

/* Guards of the reference headers replaced here. */
#define COOSORT_HPP
#define CUSPARSEWRAPPER_HPP
#define CONVERTCSR2ECSR_HPP
#define CSRMV_HPP
#define MLEMOPERATIONS_HPP

#ifndef CUDA_HANDLE_ERROR
class cudaException : public std::exception {};
#endif

/* The regular generator of RayGenerators.hpp:46-66, declared so that the
 * generator a driver names can be told apart; the reference header defines it
 * with the same three parameters. */
template <typename T, typename MSTrafo0_inplace, typename MSTrafo1_inplace>
struct ReguRayGen;

namespace epet_shim {

/* epet_problem::ray_mode of the RayGen argument: ReguRayGen is
 * EPET_RAYS_REGULAR, every other generator (RandRayGen) EPET_RAYS_RANDOM. */
template <typename RayGen>
struct ray_mode_of {
  static constexpr int value = EPET_RAYS_RANDOM;
};
template <typename T, typename A, typename B>
struct ray_mode_of<ReguRayGen<T, A, B>> {
  static constexpr int value = EPET_RAYS_REGULAR;
};

inline void check(epet_status s, const char* what) {
  if (s != EPET_OK) {
    std::cerr << what << ": " << epet_last_error() << std::endl;
    throw cudaException();
  }
}

inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::cerr << what << ": " << cudaGetErrorString(e) << std::endl;
    throw cudaException();
  }
}

inline epet_problem constant_problem() {
  epet_problem p;
  check(epet_get_constant_geometry(&p), "constant geometry");
  return p;
}

inline int64_t nchannels(const epet_problem& p) {
  const epet_setup& s = p.setup;
  return (int64_t)s.na * s.n0z * s.n0y * s.n1z * s.n1y;
}

}  // namespace epet_shim

/* Replaces the three cudaMemcpyToSymbol calls of reco.cu:64-72.  VG/MS are
 * the reference's DefaultVoxelGrid / DefaultMeasurementSetup (any type with
 * their accessors). */
template <typename VG, typename MS>
void epetSetConstantGeometry(VG const& grid, MS const& setup, int nrays) {
  epet_setup s{(float)setup.pos0x(), (float)setup.pos1x(), setup.na(),  setup.n0z(),
                setup.n0y(),         setup.n1z(),         setup.n1y(), (float)setup.da(),
                (float)setup.segx(), (float)setup.segy(), (float)setup.segz()};
  epet_grid g{{(float)grid.gridox(), (float)grid.gridoy(), (float)grid.gridoz()},
              {(float)grid.griddx(), (float)grid.griddy(), (float)grid.griddz()},
              {grid.gridnx(), grid.gridny(), grid.gridnz()}};
  epet_shim::check(epet_set_constant_geometry(&s, &g, nrays), "epetSetConstantGeometry");
}

/* systemMatrixCalculation (wrappers.hpp:166-247).  Rows = the nY_host[0]
 * channels listed at yRowId_devi.  Fills the ECSR row pointer (nY+1 ints),
 * column ids, values, the intermediate COO channel ids and the CSR over all
 * channels, and adds the number of stored entries to *nnz_devi.  The arrays
 * must hold nY*V entries, as mallocD_SystemMatrix sizes them. */
template <typename T, typename ListSizeType, typename GridSizeType, typename MemArrSizeType,
          typename RayGen>
void systemMatrixCalculation(int* const aEcsrCnlPtr_devi, GridSizeType* const aVxlId_devi,
                             T* const aVal_devi, MemArrSizeType* const nnz_devi,
                             int* const aCnlId_devi, int* const aCsrCnlPtr_devi,
                             int* const yRowId_devi, ListSizeType const* const& nY_host,
                             cusparseHandle_t const& handle) {
  static_assert(sizeof(T) == 4 && sizeof(GridSizeType) == 4, "float values, int voxel ids");
  (void)handle;
  using namespace epet_shim;
  epet_problem p = constant_problem();
  p.ray_mode = ray_mode_of<RayGen>::value;
  const int64_t m = (int64_t)nY_host[0];
  const int64_t V = (int64_t)p.grid.n[0] * p.grid.n[1] * p.grid.n[2];
  MemArrSizeType nnz0 = 0;
  check_cuda(cudaMemcpy(&nnz0, nnz_devi, sizeof(nnz0), cudaMemcpyDeviceToHost), "nnz");
  int64_t* rp = nullptr;
  check_cuda(cudaMalloc((void**)&rp, (m + 1) * sizeof(int64_t)), "cudaMalloc");
  epet_csr out{m, V, 0, rp, reinterpret_cast<int32_t*>(aVxlId_devi),
               reinterpret_cast<float*>(aVal_devi)};
  int64_t nnz = 0;
  epet_status st = epet_sm_build(&p, yRowId_devi, m, &out, m * V, &nnz, 0, nullptr, 0, 0);
  if (st == EPET_OK) st = epet_index_i64_to_i32(rp, m + 1, aEcsrCnlPtr_devi, 0);
  if (st == EPET_OK) st = epet_csr_expand_rows(rp, m, yRowId_devi, aCnlId_devi, 0);
  if (st == EPET_OK)
    st = epet_coo2csr_i32(aCnlId_devi, nnz, nchannels(p), aCsrCnlPtr_devi, 0);
  cudaFree(rp);
  check(st, "systemMatrixCalculation");
  MemArrSizeType nnz1 = nnz0 + (MemArrSizeType)nnz;
  check_cuda(cudaMemcpy(nnz_devi, &nnz1, sizeof(nnz1), cudaMemcpyHostToDevice), "nnz");
  check_cuda(cudaDeviceSynchronize(), "systemMatrixCalculation");
}

/* cooSort (cooSort.hpp:53-71). */
template <typename T>
void cooSort(T* const cooVal, int* const cooRowId, int* const cooColId, int const N) {
  static_assert(sizeof(T) == 4, "float values");
  epet_shim::check(epet_coo_sort(reinterpret_cast<float*>(cooVal), cooRowId, cooColId, N,
                                 nullptr, 0, 0),
                   "cooSort");
}

/* cusparseWrapper.hpp:21-45: the descriptor is not used by the library. */
inline cusparseStatus_t customizeMatDescr(cusparseMatDescr_t& descr,
                                          cusparseHandle_t const& handle) {
  (void)descr;
  (void)handle;
  return CUSPARSE_STATUS_SUCCESS;
}

inline cusparseStatus_t convertCoo2Csr(int* const csrRowPtr, int const* const cooRowId,
                                       cusparseHandle_t const& handle, int const nnz,
                                       int const m) {
  (void)handle;
  return epet_coo2csr_i32(cooRowId, nnz, m, csrRowPtr, 0) == EPET_OK
             ? CUSPARSE_STATUS_SUCCESS
             : CUSPARSE_STATUS_EXECUTION_FAILED;
}

/* convertCsr2Ecsr.hpp:34-47 (one gather kernel, synchronous). */
inline void convertCsr2Ecsr(int* const ecsrRowPtr, int* const yRowId, int const nnzr,
                            int* const csrRowPtr, int const m) {
  epet_shim::check(epet_csr2ecsr_i32(ecsrRowPtr, yRowId, nnzr, csrRowPtr, m, 0),
                   "convertCsr2Ecsr");
  epet_shim::check_cuda(cudaDeviceSynchronize(), "convertCsr2Ecsr");
}

namespace epet_shim {

/* Column-major copies registered for CSRs (keyed by the CSR's value array):
 * a transposed CSRmv on a registered matrix reads its copy (scatter-free,
 * deterministic) instead of scattering with atomics.  One host thread, as
 * the reference's drivers. */
struct TransposeEntry {
  const float* csr_val;
  int m, n, nnz;
  epet_csc csc;
};
inline TransposeEntry* transposes() {
  static TransposeEntry table[16];
  return table;
}
inline int& transpose_count() {
  static int n = 0;
  return n;
}
inline TransposeEntry* find_transpose(const float* val, int m, int n, int nnz) {
  TransposeEntry* t = transposes();
  for (int i = 0; i < transpose_count(); i++)
    if (t[i].csr_val == val && t[i].m == m && t[i].n == n && t[i].nnz == nnz) return &t[i];
  return nullptr;
}

}  // namespace epet_shim

/* No counterpart in the reference: builds the column-major copy of an
 * m x n CSR with int row pointers (device arrays, as CSRmv takes them) and
 * registers it, so later CSRmv(CUSPARSE_OPERATION_TRANSPOSE) calls on this
 * matrix (same value array and sizes) use the scatter-free product.  Worth
 * it when a matrix is transposed in several iterations (a driver that keeps
 * its matrix); release with epetReleaseTranspose before freeing the CSR. */
inline void epetBuildTranspose(int m, int n, int nnz, float* const csrValA,
                               int* const csrRowPtrA, int* const csrColIdA) {
  using namespace epet_shim;
  if (find_transpose(csrValA, m, n, nnz)) return;
  TransposeEntry* t = transposes();
  if (transpose_count() == 16) check(EPET_ERR_CAPACITY, "epetBuildTranspose: 16 registered");
  TransposeEntry e{csrValA, m, n, nnz, epet_csc{}};
  int64_t* rp = nullptr;
  check_cuda(cudaMalloc((void**)&rp, ((size_t)m + 1) * sizeof(int64_t)), "cudaMalloc");
  check_cuda(cudaMalloc((void**)&e.csc.col_ptr, ((size_t)n + 1) * sizeof(int64_t)), "cudaMalloc");
  check_cuda(cudaMalloc((void**)&e.csc.row, ((size_t)nnz + 1) * sizeof(int32_t)), "cudaMalloc");
  check_cuda(cudaMalloc((void**)&e.csc.val, ((size_t)nnz + 1) * sizeof(float)), "cudaMalloc");
  epet_status st = epet_index_i32_to_i64(csrRowPtrA, (int64_t)m + 1, rp, 0);
  epet_csr a{m, n, nnz, rp, csrColIdA, csrValA};
  if (st == EPET_OK) st = epet_csr_to_csc(&a, &e.csc, nullptr, 0, 0);
  check_cuda(cudaDeviceSynchronize(), "epetBuildTranspose");
  cudaFree(rp);
  check(st, "epetBuildTranspose");
  t[transpose_count()++] = e;
}

inline void epetReleaseTranspose(float* const csrValA) {
  using namespace epet_shim;
  TransposeEntry* t = transposes();
  for (int i = 0; i < transpose_count(); i++)
    if (t[i].csr_val == csrValA) {
      cudaFree(t[i].csc.col_ptr);
      cudaFree(t[i].csc.row);
      cudaFree(t[i].csc.val);
      t[i] = t[--transpose_count()];
      return;
    }
}

/* CSRmv<float> (csrmv.hpp:18-36); alpha/beta are host pointers as in the
 * reference; the transpose reads the column-major copy registered with
 * epetBuildTranspose for this matrix, else scatters with atomics. */
template <typename T>
struct CSRmv;

template <>
struct CSRmv<float> {
  void operator()(cusparseHandle_t handle, cusparseOperation_t transA, int m, int n, int nnz,
                  float* const alpha, cusparseMatDescr_t descrA, float* const csrValA,
                  int* const csrRowPtrA, int* const csrColIdA, float* const x,
                  float* const beta, float* const y) {
    (void)handle;
    (void)descrA;
    const int trans = transA == CUSPARSE_OPERATION_NON_TRANSPOSE ? 0 : 1;
    if (trans) {
      if (const epet_shim::TransposeEntry* e =
              epet_shim::find_transpose(csrValA, m, n, nnz)) {
        epet_csr a{m, n, nnz, nullptr, csrColIdA, csrValA};
        epet_shim::check(epet_csrmv(1, &a, &e->csc, *alpha, x, *beta, y, 0), "CSRmv");
        return;
      }
    }
    epet_shim::check(epet_csrmv_i32(trans, m, n, nnz, *alpha, csrValA, csrRowPtrA, csrColIdA, x,
                                    *beta, y, 0),
                     "CSRmv");
  }
};

/* mlemOperations.hpp:22-139. */
template <typename T>
void divides(T* const& result, T* const& dividend, T* const& divisor, int const n) {
  static_assert(sizeof(T) == 4, "float");
  epet_shim::check(epet_divides(result, dividend, divisor, n, 0), "divides");
}

template <typename T>
void dividesMultiplies(T* const& result, T* const& a, T* const& b, T* const& c, int const n) {
  static_assert(sizeof(T) == 4, "float");
  epet_shim::check(epet_divides_multiplies(result, a, b, c, n, 0), "dividesMultiplies");
}

template <typename T>
void scales(T* const& x, T const alpha, int const n) {
  static_assert(sizeof(T) == 4, "float");
  epet_shim::check(epet_scales(x, alpha, n, 0), "scales");
}

/* Returns the sum on the host (synchronising), accumulated in fp64. */
template <typename T>
T sum(T* const& x, int const n) {
  static_assert(sizeof(T) == 4, "float");
  double* d = nullptr;
  epet_shim::check_cuda(cudaMalloc((void**)&d, sizeof(double)), "cudaMalloc");
  epet_status st = epet_sum_f64(x, n, d, 0);
  double h = 0.0;
  if (st == EPET_OK) cudaMemcpy(&h, d, sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d);
  epet_shim::check(st, "sum");
  return (T)h;
}

/* Chunk helpers (wrappers.hpp:410-446). */
template <typename ListSizeType, typename ChunkGridSizeType>
ListSizeType nInChunk(ChunkGridSizeType idChunk, ListSizeType const nAll,
                      ListSizeType const nFullChunk) {
  if (idChunk < ChunkGridSizeType((nAll + nFullChunk - 1) / nFullChunk)) {
    if (idChunk < ChunkGridSizeType(nAll / nFullChunk)) return nFullChunk;
    return (nAll % nFullChunk);
  }
  return 0;
}

template <typename ListSizeType, typename ChunkGridSizeType>
ListSizeType chunkPtr(ChunkGridSizeType const chunkId, ListSizeType const nFullChunk) {
  return chunkId * nFullChunk;
}

template <typename ChunkGridSizeType, typename MemArrSizeType>
ChunkGridSizeType nChunks(MemArrSizeType const maxNnz, MemArrSizeType const maxNChunk) {
  return ChunkGridSizeType((maxNnz + maxNChunk - 1) / maxNChunk);
}

#endif
