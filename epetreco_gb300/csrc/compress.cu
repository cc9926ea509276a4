// compress.cu -- 16-bit system-matrix storage: BF16/FP16 values with a per-row
// FP32 scale and 16-bit column steps (4 bytes per entry instead of 8), and
// the products over it.
//
// Row r holds entries k = 0..len-1: col_k = base[r] + sum_{j<=k} delta_j
// (delta_0 = 0) and value_k = scale[r] * q_k, q_k the 16-bit float of
// value_k / scale[r], scale[r] = max value of the row.  A step wider than
// 65535 is split by zero-valued entries of step 65535, so every matrix is
// representable; at 52^3 voxels no step in a row exceeds ny*nz = 2704.
// The same layout over the column-major copy stores A^T, so one kernel serves
// both products.  The products accumulate in FP32.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "spmv.cuh"

namespace epet {

constexpr uint32_t kMaxStep = 65535u;

// Entries a row needs (escapes included).
__global__ void k_c16_count(const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            int64_t m, int64_t* __restrict__ cnt) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= m) return;
  const int64_t b = ptr[r], e = ptr[r + 1];
  int64_t extra = 0;
  for (int64_t k = b + 1 + lane; k < e; k += 32) {
    const uint32_t d = (uint32_t)(idx[k] - idx[k - 1]);
    extra += (d - 1u) / kMaxStep;
  }
  for (int o = 16; o > 0; o >>= 1) extra += __shfl_xor_sync(0xffffffffu, extra, o);
  if (lane == 0) cnt[r] = (e - b) + extra;
}

template <int FMT>
__device__ __forceinline__ uint16_t to_q(float v) {
  if (FMT == 1) return __bfloat16_as_ushort(__float2bfloat16_rn(v));
  return __half_as_ushort(__float2half_rn(v));
}

template <int FMT>
__device__ __forceinline__ float from_q(uint32_t q) {
  if (FMT == 1) return __uint_as_float(q << 16);
  return __half2float(__ushort_as_half((unsigned short)q));
}

// Fill: warp per row; chunks of 32 entries, escapes placed by a warp scan.
template <int FMT>
__global__ void k_c16_fill(const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                           const float* __restrict__ val, int64_t m,
                           const int64_t* __restrict__ ptr16, int32_t* __restrict__ base,
                           float* __restrict__ scale, uint16_t* __restrict__ delta,
                           uint16_t* __restrict__ q) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= m) return;
  const int64_t b = ptr[r], e = ptr[r + 1];
  // row scale: max value
  float mx = 0.f;
  for (int64_t k = b + lane; k < e; k += 32) mx = fmaxf(mx, fabsf(val[k]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const float sc = mx > 0.f ? mx : 1.f;
  if (lane == 0) {
    scale[r] = sc;
    base[r] = e > b ? idx[b] : 0;
  }
  int64_t out = ptr16[r];
  for (int64_t k0 = b; k0 < e; k0 += 32) {
    const int64_t k = k0 + lane;
    uint32_t d = 0, ex = 0;
    if (k < e && k > b) {
      d = (uint32_t)(idx[k] - idx[k - 1]);
      ex = (d - 1u) / kMaxStep;
    }
    uint32_t inc = ex;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    const uint32_t tot = __shfl_sync(0xffffffffu, inc, 31);
    if (k < e) {
      int64_t o = out + (k - k0) + (inc - ex);
      for (uint32_t j = 0; j < ex; j++) {  // escape entries
        delta[o] = (uint16_t)kMaxStep;
        q[o] = 0;
        o++;
      }
      delta[o] = (uint16_t)(d - ex * kMaxStep);
      q[o] = to_q<FMT>(__fdiv_rn(val[k], sc));
    }
    const int64_t nthis = e - k0 < 32 ? e - k0 : 32;
    out += nthis + tot;
  }
}

// Product over the 16-bit layout: a group of G lanes per row, each lane
// reading 8 consecutive entries (16-byte loads of steps and values) per
// round; columns come from the group-wide prefix sum of the steps.
template <int G, int FMT, class Epi>
__global__ void __launch_bounds__(kSpmvThreads)
k_rows16(const int64_t* __restrict__ ptr, const int32_t* __restrict__ base,
         const float* __restrict__ scale, const uint16_t* __restrict__ delta,
         const uint16_t* __restrict__ q, const float* __restrict__ x, int64_t nrows, Epi epi,
         double* __restrict__ partial) {
  constexpr int RPB = kSpmvThreads / G;
  __shared__ double red[kSpmvThreads / 32];
  const int lg = threadIdx.x % G;
  const int64_t row = (int64_t)blockIdx.x * RPB + threadIdx.x / G;
  double part = 0.0;
  // all lanes of a group take part in the group shuffles
  const bool live = row < nrows;
  const int64_t b = live ? ptr[row] : 0, e = live ? ptr[row + 1] : 0;
  int32_t col = live ? base[row] : 0;  // column of the entry before the chunk
  float acc = 0.f;
  // round-aligned start (8-entry, 16-byte boundaries)
  const int64_t a0 = b & ~int64_t(7);
  const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (threadIdx.x & 31 & ~(G - 1)));
  // software pipeline: the next round's loads are issued before this
  // round's scan and gathers
  uint4 dv = make_uint4(0, 0, 0, 0), qv = make_uint4(0, 0, 0, 0);
  if (a0 + 8 * lg < e) {
    dv = __ldcs(reinterpret_cast<const uint4*>(delta + a0 + 8 * lg));
    qv = __ldcs(reinterpret_cast<const uint4*>(q + a0 + 8 * lg));
  }
  for (int64_t c0 = a0; c0 < e; c0 += 8 * G) {
    const int64_t k = c0 + 8 * lg;  // this lane's first entry
    uint4 dn = make_uint4(0, 0, 0, 0), qn = make_uint4(0, 0, 0, 0);
    if (k + 8 * G < e) {
      dn = __ldcs(reinterpret_cast<const uint4*>(delta + k + 8 * G));
      qn = __ldcs(reinterpret_cast<const uint4*>(q + k + 8 * G));
    }
    // entries j of this lane's chunk with lo <= j < hi lie in [b, e)
    const int64_t dl = b - k, dh = e - k;
    const int lo = dl > 0 ? (int)dl : 0;
    const int hi = dh < 8 ? (dh > 0 ? (int)dh : 0) : 8;
    uint32_t dd[8], qq[8];
    dd[0] = dv.x & 0xffffu; dd[1] = dv.x >> 16; dd[2] = dv.y & 0xffffu; dd[3] = dv.y >> 16;
    dd[4] = dv.z & 0xffffu; dd[5] = dv.z >> 16; dd[6] = dv.w & 0xffffu; dd[7] = dv.w >> 16;
    qq[0] = qv.x & 0xffffu; qq[1] = qv.x >> 16; qq[2] = qv.y & 0xffffu; qq[3] = qv.y >> 16;
    qq[4] = qv.z & 0xffffu; qq[5] = qv.z >> 16; qq[6] = qv.w & 0xffffu; qq[7] = qv.w >> 16;
    // entries outside [b, e) do not step
    uint32_t lsum = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if (j < lo || j >= hi) dd[j] = 0;
      lsum += dd[j];
    }
    // group exclusive scan of the lane sums
    uint32_t inc = lsum;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) {
      const uint32_t t = __shfl_up_sync(gmask, inc, o, G);
      if (lg >= o) inc += t;
    }
    const uint32_t total = __shfl_sync(gmask, inc, G - 1, G);
    int32_t c = col + (int32_t)(inc - lsum);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      c += (int32_t)dd[j];
      if (j >= lo && j < hi) acc = fmaf(from_q<FMT>(qq[j]), __ldg(x + c), acc);
    }
    col += (int32_t)total;
    dv = dn;
    qv = qn;
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o, G);
  if (live && lg == 0) part = epi(row, acc * scale[row]);
  if (partial) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kSpmvThreads / 32; w++) t += red[w];
      partial[blockIdx.x] = t;
    }
  }
}

struct EpiStore {  // y = alpha*d + beta*y
  float alpha, beta;
  float* y;
  __device__ double operator()(int64_t r, float d) const {
    y[r] = beta == 0.f ? alpha * d : alpha * d + beta * y[r];
    return 0.0;
  }
};

template <int FMT, class Epi>
static epet_status launch16_fmt(int G, const epet_csr16* a, const float* x, Epi epi,
                                double* partial, cudaStream_t st) {
  const int rpb = kSpmvThreads / G;
  const unsigned nb = (unsigned)((a->m + rpb - 1) / rpb);
  switch (G) {
    case 32: k_rows16<32, FMT, Epi><<<nb, kSpmvThreads, 0, st>>>(a->row_ptr, a->base, a->scale, a->delta, a->q, x, a->m, epi, partial); break;
    case 16: k_rows16<16, FMT, Epi><<<nb, kSpmvThreads, 0, st>>>(a->row_ptr, a->base, a->scale, a->delta, a->q, x, a->m, epi, partial); break;
    case 8: k_rows16<8, FMT, Epi><<<nb, kSpmvThreads, 0, st>>>(a->row_ptr, a->base, a->scale, a->delta, a->q, x, a->m, epi, partial); break;
    default: k_rows16<4, FMT, Epi><<<nb, kSpmvThreads, 0, st>>>(a->row_ptr, a->base, a->scale, a->delta, a->q, x, a->m, epi, partial); break;
  }
  EPET_LAUNCHED();
  return EPET_OK;
}

int pick_group16(double avg_len) {
  if (avg_len >= 256) return 32;
  if (avg_len >= 96) return 16;
  if (avg_len >= 40) return 8;
  return 4;
}

template <class Epi>
epet_status launch_rows16(const epet_csr16* a, const float* x, Epi epi, double* partial,
                          cudaStream_t st) {
  if (a->m <= 0) return EPET_OK;
  if (((reinterpret_cast<uintptr_t>(a->delta) | reinterpret_cast<uintptr_t>(a->q)) & 15) != 0)
    return set_error(EPET_ERR_INVALID, "16-bit matrix: delta and q must be 16-byte aligned");
  const int G = pick_group16(a->m ? (double)a->nnz / a->m : 0.0);
  if (a->format == EPET_VALUES_BF16) return launch16_fmt<1>(G, a, x, epi, partial, st);
  if (a->format == EPET_VALUES_FP16) return launch16_fmt<2>(G, a, x, epi, partial, st);
  return set_error(EPET_ERR_INVALID, "unknown value format %d", a->format);
}

template epet_status launch_rows16<EpiMlemForward>(const epet_csr16*, const float*,
                                                   EpiMlemForward, double*, cudaStream_t);
template epet_status launch_rows16<EpiMlemUpdate>(const epet_csr16*, const float*,
                                                  EpiMlemUpdate, double*, cudaStream_t);

int64_t rows16_blocks(const epet_csr16* a) {
  const int G = pick_group16(a->m ? (double)a->nnz / a->m : 0.0);
  const int rpb = kSpmvThreads / G;
  return (a->m + rpb - 1) / rpb;
}

}  // namespace epet

using namespace epet;

extern "C" {

epet_status epet_csr16_count(const epet_csr* a, int64_t* row_len16_d, int64_t* nnz16_h,
                             epet_stream_t stream) {
  if (!a || !row_len16_d || !nnz16_h) return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  *nnz16_h = 0;
  if (a->m == 0) return EPET_OK;
  k_c16_count<<<ceil_div(a->m * 32, 256), 256, 0, st>>>(a->row_ptr, a->col, a->m, row_len16_d);
  EPET_LAUNCHED();
  int64_t* tmp = nullptr;
  int64_t* off = nullptr;
  EPET_CUDA(dev_alloc((void**)&tmp, scan_tmp_elems(a->m + 1) * 8, st));
  EPET_CUDA(dev_alloc((void**)&off, (a->m + 1) * 8, st));
  epet_status rc = exclusive_scan_i64(row_len16_d, off, a->m, tmp, st);
  if (rc == EPET_OK) {
    cudaError_t e = cudaMemcpyAsync(nnz16_h, off + a->m, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_status(e, "csr16 count");
  }
  dev_free(tmp, st);
  dev_free(off, st);
  return rc;
}

epet_status epet_csr_compress(const epet_csr* a, int32_t format, epet_csr16* out,
                              epet_stream_t stream) {
  if (!a || !out || !out->row_ptr || (a->m > 0 && (!out->base || !out->scale)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  if (format != EPET_VALUES_BF16 && format != EPET_VALUES_FP16)
    return set_error(EPET_ERR_INVALID, "format must be EPET_VALUES_BF16 or EPET_VALUES_FP16");
  cudaStream_t st = (cudaStream_t)stream;
  out->m = a->m;
  out->n = a->n;
  out->format = format;
  if (a->m == 0) {
    out->nnz = 0;
    EPET_CUDA(cudaMemsetAsync(out->row_ptr, 0, 8, st));
    return EPET_OK;
  }
  int64_t* cnt = nullptr;
  EPET_CUDA(dev_alloc((void**)&cnt, (a->m + 1) * 8, st));
  int64_t nnz16 = 0;
  epet_status rc = epet_csr16_count(a, cnt, &nnz16, stream);
  if (rc == EPET_OK && nnz16 > out->nnz && out->nnz >= 0 && (out->delta || out->q)) {
    // caller buffers too small
    rc = set_error(EPET_ERR_CAPACITY, "16-bit layout needs %lld entries", (long long)nnz16);
  }
  if (rc == EPET_OK && nnz16 > 0 && (!out->delta || !out->q))
    rc = set_error(EPET_ERR_INVALID, "delta/q buffers missing");
  if (rc == EPET_OK) {
    int64_t* tmp = nullptr;
    dev_alloc((void**)&tmp, scan_tmp_elems(a->m + 1) * 8, st);
    rc = exclusive_scan_i64(cnt, out->row_ptr, a->m, tmp, st);
    dev_free(tmp, st);
  }
  if (rc == EPET_OK) {
    const unsigned nb = (unsigned)ceil_div(a->m * 32, 256);
    if (format == EPET_VALUES_BF16)
      k_c16_fill<1><<<nb, 256, 0, st>>>(a->row_ptr, a->col, a->val, a->m, out->row_ptr,
                                        out->base, out->scale, out->delta, out->q);
    else
      k_c16_fill<2><<<nb, 256, 0, st>>>(a->row_ptr, a->col, a->val, a->m, out->row_ptr,
                                        out->base, out->scale, out->delta, out->q);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_status(e, "k_c16_fill");
    out->nnz = nnz16;
  }
  dev_free(cnt, st);
  return rc;
}

epet_status epet_csr16_mv(const epet_csr16* a, float alpha, const float* x_d, float beta,
                          float* y_d, epet_stream_t stream) {
  if (!a || (a->m > 0 && !y_d) || (a->n > 0 && !x_d))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  return launch_rows16(a, x_d, EpiStore{alpha, beta, y_d}, nullptr, (cudaStream_t)stream);
}

}  // extern "C"
