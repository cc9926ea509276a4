// spmv.cuh -- fused MLEM epilogues of the row kernels (spmv.cu).
#pragma once
#include <functional>

#include "common.cuh"
#include "rows.cuh"

namespace epet {

// Forward projection epilogue: yb = A x (row r), e[r] = y[r] / yb with the
// reference's divides (mlemOperations.hpp:22-32) but 0 where yb == 0 (the
// reference would produce inf/NaN there); keeps yb for the log-likelihood,
// which a separate kernel evaluates when asked for.
struct EpiMlemForward {
  const float* y;
  float* e;
  float* ybar;
  __device__ double operator()(int64_t r, float d) const {
    ybar[r] = d;
    e[r] = d > 0.f ? __fdiv_rn(y[r], d) : 0.f;
    return 0.0;
  }
};

// The same for the 16-bit forms: e is kept as BF16 bits (relative error
// <= 2^-9), which halves the bytes of the transpose product's gathers.
struct EpiMlemForward16 {
  const float* y;
  uint16_t* e16;
  float* ybar;
  __device__ double operator()(int64_t r, float d) const {
    ybar[r] = d;
    const float ev = d > 0.f ? __fdiv_rn(y[r], d) : 0.f;
    // round to nearest even on the upper 16 bits (e is finite and >= 0)
    const uint32_t b = __float_as_uint(ev);
    e16[r] = (uint16_t)((b + 0x7fffu + ((b >> 16) & 1u)) >> 16);
    return 0.0;
  }
};

// Back-projection epilogue (column v, c = (A^T e)[v]): the reference's
// dividesMultiplies (mlemOperations.hpp:38-79): xnew = x*c/s with s == 0 -> 1;
// returns xnew for the image sum.
struct EpiMlemUpdate {
  const float* x;
  const float* s;
  float* xnew;
  float* c_out;  // optional
  __device__ double operator()(int64_t v, float c) const {
    if (c_out) c_out[v] = c;
    float dvs = s[v];
    dvs = __fadd_rn(dvs, (float)(dvs == 0.f));
    const float xn = __fdiv_rn(__fmul_rn(x[v], c), dvs);
    xnew[v] = xn;
    return (double)xn;
  }
};

// Store the product (c = (A^T e)[v] of a row-sharded reconstruction, summed
// across shards before the update).
struct EpiKeep {
  float* out;
  __device__ double operator()(int64_t r, float d) const {
    out[r] = d;
    return 0.0;
  }
};

int pick_group(double avg_len);
RowPlan default_plan(double avg_len);

template <class Epi>
epet_status launch_rows(const RowPlan& plan, const int64_t* ptr, const int32_t* idx,
                        const float* val, const float* x, int64_t nrows, Epi epi,
                        double* partial, cudaStream_t st);

// The same with every value 1 and no value stream: out = Epi(row, sum of
// x over the row's indices), equal to launch_rows with values 1.
template <class Epi>
epet_status launch_sums(const RowPlan& plan, const int64_t* ptr, const int32_t* idx,
                        const float* x, int64_t nrows, Epi epi, double* partial,
                        cudaStream_t st);

// Autotuner: times run(plan) over candidate plans around default_plan(avg)
// (group sizes, unroll depths, persistent grids) and returns the fastest.
// Results are cached per (device, kind, rows, nnz, cols) for the life of the
// process (mutex-guarded).  run must be idempotent; the stream must not be
// capturing.
epet_status tune_rows(int kind, int64_t nrows, int64_t nnz, int64_t ncols, double avg,
                      const std::function<epet_status(const RowPlan&)>& run, cudaStream_t st,
                      RowPlan* out);
// The cached plan of (kind, rows, nnz, cols) on the current device, if any.
bool tune_lookup(int kind, int64_t nrows, int64_t nnz, int64_t ncols, RowPlan* out);
template <class Epi, class XT>
epet_status launch_rows16(const epet_csr16* a, const XT* x, Epi epi, double* partial,
                          cudaStream_t st);
inline int64_t csr16_capacity(int64_t nnz16) { return nnz16; }
epet_status launch_sum_partials(const double* p, int64_t n, double* out, cudaStream_t st);
// x = xnew / sum(xnew), the sum in fp64 and in a fixed order: block
// partials (part holds sum_blocks(n) doubles), then the scaling launch.
int sum_blocks(int64_t n);
epet_status launch_sum_normalise(const float* xnew, int64_t n, double* part, float* x,
                                 cudaStream_t st);
epet_status launch_normalise(const float* xnew, const double* sum, int64_t n, float* x,
                             cudaStream_t st);
epet_status sum_f64(const float* x, int64_t n, double* partial, int nblocks, double* out,
                    cudaStream_t st);
// sum_i y_i log(ybar_i) - ybar_i over ybar_i > 0, fp64, fixed order.
epet_status poisson_loglik(const float* y, const float* ybar, int64_t m, double* partial,
                           int nblocks, double* out, cudaStream_t st);

}  // namespace epet
