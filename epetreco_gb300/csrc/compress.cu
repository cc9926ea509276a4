// compress.cu -- 16-bit system-matrix storage: BF16/FP16 values with a per-row
// FP32 scale and 16-bit column offsets (4.5 bytes per entry instead of 8),
// and the products over it.
//
// A row is stored as chunks of 8 entries: chunk c has a 32-bit column base
// cbase[c] (the smallest column of its entries), 16-bit offsets
// (col = cbase[c] + offset) and 16-bit values (value = scale[r] * q, q the
// 16-bit float of value / scale[r], scale[r] = the row's largest value).
// Rows are padded to whole chunks with zero-valued entries of offset 0, so a
// chunk never mixes rows and a lane decodes its chunk alone: no scan over
// steps, no masks.  Columns need not ascend within a row; a chunk ends early
// (and is padded) before an entry that would widen its column range to
// 65536 or more, so every matrix is representable; at 52^3 voxels 8
// consecutive entries of a row span far less.  The same
// layout over the column-major copy stores A^T, so one kernel serves both
// products.  The products accumulate in FP32.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "spmv.cuh"

namespace epet {

constexpr int kChunk = 8;
constexpr int32_t kMaxSpan = 65535;

// True (warp-uniform) when the fixed chunks [b + 8c, b + 8c + 8) of row
// [b, e) all span at most kMaxSpan columns (largest - smallest).
__device__ __forceinline__ bool fixed_chunks(const int32_t* __restrict__ idx, int64_t b,
                                             int64_t e, int lane) {
  bool ok = true;
  for (int64_t k = b + (int64_t)kChunk * lane; k < e; k += 32 * kChunk) {
    const int64_t last = k + kChunk - 1 < e ? k + kChunk - 1 : e - 1;
    int32_t mn = idx[k], mx = mn;
    for (int64_t j = k + 1; j <= last; j++) {
      mn = min(mn, idx[j]);
      mx = max(mx, idx[j]);
    }
    if (mx - mn > kMaxSpan) ok = false;
  }
  return __all_sync(0xffffffffu, ok);
}

// Greedy chunks of row [b, e) (one thread): a chunk takes up to 8 entries
// whose columns span at most kMaxSpan.  Returns the number of chunks; with
// out pointers given, writes them.
template <int FMT>
__device__ int64_t greedy_chunks(const int32_t* __restrict__ idx, const float* __restrict__ val,
                                 int64_t b, int64_t e, float sc, int64_t out,
                                 int32_t* cbase, uint16_t* off, uint16_t* q);

// Stored entries of every row (multiples of 8).
__global__ void k_c16_count(const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            int64_t m, int64_t* __restrict__ cnt) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= m) return;
  const int64_t b = ptr[r], e = ptr[r + 1];
  if (fixed_chunks(idx, b, e, lane)) {
    if (lane == 0) cnt[r] = (e - b + kChunk - 1) / kChunk * kChunk;
  } else if (lane == 0) {
    cnt[r] = greedy_chunks<1>(idx, nullptr, b, e, 1.f, -1, nullptr, nullptr, nullptr) * kChunk;
  }
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

template <int FMT>
__device__ int64_t greedy_chunks(const int32_t* __restrict__ idx, const float* __restrict__ val,
                                 int64_t b, int64_t e, float sc, int64_t out, int32_t* cbase,
                                 uint16_t* off, uint16_t* q) {
  int64_t n = 0;
  int64_t k = b;
  while (k < e) {
    int32_t mn = idx[k], mx = idx[k];
    int j = 1;
    for (; j < kChunk && k + j < e; j++) {
      const int32_t c = idx[k + j];
      if (max(mx, c) - min(mn, c) > kMaxSpan) break;
      mn = min(mn, c);
      mx = max(mx, c);
    }
    if (out >= 0) {
      for (int t = 0; t < j; t++) {
        off[out + n * kChunk + t] = (uint16_t)(idx[k + t] - mn);
        q[out + n * kChunk + t] = to_q<FMT>(__fdiv_rn(val[k + t], sc));
      }
      cbase[(out >> 3) + n] = mn;
      for (int p = j; p < kChunk; p++) {
        off[out + n * kChunk + p] = 0;
        q[out + n * kChunk + p] = 0;
      }
    }
    k += j;
    n++;
  }
  return n;
}

// Fill: warp per row; fixed chunks lane-parallel, otherwise lane 0 greedy.
template <int FMT>
__global__ void k_c16_fill(const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                           const float* __restrict__ val, int64_t m,
                           const int64_t* __restrict__ ptr16, int32_t* __restrict__ cbase,
                           float* __restrict__ scale, uint16_t* __restrict__ off,
                           uint16_t* __restrict__ q) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= m) return;
  const int64_t b = ptr[r], e = ptr[r + 1];
  // row scale: largest value
  float mx = 0.f;
  for (int64_t k = b + lane; k < e; k += 32) mx = fmaxf(mx, fabsf(val[k]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const float sc = mx > 0.f ? mx : 1.f;
  if (lane == 0) scale[r] = sc;
  const int64_t out = ptr16[r];
  if (fixed_chunks(idx, b, e, lane)) {
    const int64_t len = e - b, padded = (len + kChunk - 1) / kChunk * kChunk;
    for (int64_t p0 = 0; p0 < padded; p0 += 32) {
      const int64_t p = p0 + lane;
      const bool real = p < len;
      const int32_t col = real ? idx[b + p] : INT32_MAX;
      // smallest column of the chunk (lanes lane & ~7 .. +7; a chunk's first
      // entry is real, padding lanes hold INT32_MAX)
      int32_t base = col;
      for (int o = 1; o < kChunk; o <<= 1) base = min(base, __shfl_xor_sync(0xffffffffu, base, o));
      if (p < padded) {
        off[out + p] = real ? (uint16_t)(col - base) : (uint16_t)0;
        q[out + p] = real ? to_q<FMT>(__fdiv_rn(val[b + p], sc)) : (uint16_t)0;
        if ((p & (kChunk - 1)) == 0) cbase[(out + p) >> 3] = base;
      }
    }
  } else if (lane == 0) {
    greedy_chunks<FMT>(idx, val, b, e, sc, out, cbase, off, q);
  }
}

// The gathered vector: FP32, or BF16 bits (the MLEM ratio e of the 16-bit
// forms: half the gather traffic of the transpose product).
__device__ __forceinline__ float ld_x(const float* __restrict__ x, int32_t i) {
  return __ldg(x + i);
}
__device__ __forceinline__ float ld_x(const uint16_t* __restrict__ x, int32_t i) {
  return __uint_as_float((uint32_t)__ldg(reinterpret_cast<const unsigned short*>(x) + i) << 16);
}

// Product over the 16-bit layout: a group of G lanes per row; lane l takes
// the entry pairs l, l + G, ... of the row (32-bit loads of offsets and
// values), so the lanes of a group gather x at consecutive entries of the
// row (neighbouring columns share cache sectors); P pairs per round, and the
// next round's loads are issued before this round's gathers.  Indices are
// 32-bit and relative to the row's first stored entry (a row holds fewer
// than 2^31 entries).
template <int G, int P, int FMT, class Epi, class XT>
__global__ void __launch_bounds__(kSpmvThreads)
k_rows16(const int64_t* __restrict__ ptr, const int32_t* __restrict__ cbase,
         const float* __restrict__ scale, const uint16_t* __restrict__ off,
         const uint16_t* __restrict__ q, const XT* __restrict__ x, int64_t nrows, Epi epi,
         double* __restrict__ partial) {
  constexpr int RPT = kSpmvThreads / G;
  __shared__ double red[kSpmvThreads / 32];
  const int lg = threadIdx.x % G;
  const int64_t row = (int64_t)blockIdx.x * RPT + threadIdx.x / G;
  const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (threadIdx.x & 31 & ~(G - 1)));
  double part = 0.0;
  const bool live = row < nrows;
  const int64_t s0 = live ? ptr[row] : 0;                      // a multiple of 8
  const int n = live ? (int)((ptr[row + 1] - s0) >> 1) : 0;    // pairs
  const uint32_t* __restrict__ o2 = reinterpret_cast<const uint32_t*>(off + s0);
  const uint32_t* __restrict__ q2 = reinterpret_cast<const uint32_t*>(q + s0);
  const int32_t* __restrict__ cb = cbase + (s0 >> 3);          // 4 pairs per chunk
  float acc[P];
  uint32_t oc[P], vc[P];
  int32_t bc[P];
#pragma unroll
  for (int u = 0; u < P; u++) {
    acc[u] = 0.f;
    const int i = lg + u * G;
    oc[u] = 0u; vc[u] = 0u; bc[u] = 0;
    if (i < n) {
      oc[u] = __ldcs(o2 + i);
      vc[u] = __ldcs(q2 + i);
      bc[u] = __ldg(cb + (i >> 2));
    }
  }
  for (int i0 = lg; i0 < n; i0 += P * G) {
    uint32_t on[P], vn[P];
    int32_t bn[P];
#pragma unroll
    for (int u = 0; u < P; u++) {
      const int i = i0 + (P + u) * G;
      on[u] = 0u; vn[u] = 0u; bn[u] = 0;
      if (i < n) {
        on[u] = __ldcs(o2 + i);
        vn[u] = __ldcs(q2 + i);
        bn[u] = __ldg(cb + (i >> 2));
      }
    }
#pragma unroll
    for (int u = 0; u < P; u++) {
      if (i0 + u * G < n) {
        const XT* xb = x + bc[u];
        acc[u] = fmaf(from_q<FMT>(vc[u] & 0xffffu), ld_x(xb, (int32_t)(oc[u] & 0xffffu)), acc[u]);
        acc[u] = fmaf(from_q<FMT>(vc[u] >> 16), ld_x(xb, (int32_t)(oc[u] >> 16)), acc[u]);
      }
      oc[u] = on[u]; vc[u] = vn[u]; bc[u] = bn[u];
    }
  }
  float a = 0.f;
#pragma unroll
  for (int u = 0; u < P; u++) a += acc[u];
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) a += __shfl_xor_sync(gmask, a, o, G);
  if (live && lg == 0) part = epi(row, a * scale[row]);
  if (partial) block_sum_to(part, red, partial + blockIdx.x);
}

struct EpiStore {  // y = alpha*d + beta*y
  float alpha, beta;
  float* y;
  __device__ double operator()(int64_t r, float d) const {
    y[r] = beta == 0.f ? alpha * d : alpha * d + beta * y[r];
    return 0.0;
  }
};

template <int FMT, class Epi, class XT>
static epet_status launch16_fmt(int G, const epet_csr16* a, const XT* x, Epi epi,
                                double* partial, cudaStream_t st) {
  const int rpb = kSpmvThreads / G;
  const unsigned nb = (unsigned)((a->m + rpb - 1) / rpb);
  switch (G) {  // pairs in flight per lane: 8 with whole warps (long rows), else 4
    case 32: k_rows16<32, 8, FMT, Epi, XT><<<nb, kSpmvThreads, 0, st>>>(a->row_ptr, a->base, a->scale, a->delta, a->q, x, a->m, epi, partial); break;
    case 16: k_rows16<16, 4, FMT, Epi, XT><<<nb, kSpmvThreads, 0, st>>>(a->row_ptr, a->base, a->scale, a->delta, a->q, x, a->m, epi, partial); break;
    case 8: k_rows16<8, 4, FMT, Epi, XT><<<nb, kSpmvThreads, 0, st>>>(a->row_ptr, a->base, a->scale, a->delta, a->q, x, a->m, epi, partial); break;
    default: k_rows16<4, 4, FMT, Epi, XT><<<nb, kSpmvThreads, 0, st>>>(a->row_ptr, a->base, a->scale, a->delta, a->q, x, a->m, epi, partial); break;
  }
  EPET_LAUNCHED();
  return EPET_OK;
}

// Lanes per row from the mean stored entries per row (a lane takes two
// entries per step): whole warps with 8 pairs in flight for rows of
// thousands of entries (the transpose), else groups with 4 pairs in flight
// (measured at 52^3 voxels: rows of ~390 entries run fastest with 16 lanes).
int pick_group16(double avg_len) {
  if (avg_len >= 2048) return 32;
  if (avg_len >= 96) return 16;
  if (avg_len >= 32) return 8;
  return 4;
}

template <class Epi, class XT>
epet_status launch_rows16(const epet_csr16* a, const XT* x, Epi epi, double* partial,
                          cudaStream_t st) {
  if (a->m <= 0) return EPET_OK;
  if (((reinterpret_cast<uintptr_t>(a->delta) | reinterpret_cast<uintptr_t>(a->q)) & 15) != 0)
    return set_error(EPET_ERR_INVALID, "16-bit matrix: delta and q must be 16-byte aligned");
  if (!a->base || !a->scale || !a->row_ptr)
    return set_error(EPET_ERR_INVALID, "16-bit matrix: missing arrays");
  const int G = pick_group16(a->m ? (double)a->nnz / a->m : 0.0);
  if (a->format == EPET_VALUES_BF16) return launch16_fmt<1>(G, a, x, epi, partial, st);
  if (a->format == EPET_VALUES_FP16) return launch16_fmt<2>(G, a, x, epi, partial, st);
  return set_error(EPET_ERR_INVALID, "unknown value format %d", a->format);
}

template epet_status launch_rows16<EpiMlemForward16, float>(const epet_csr16*, const float*,
                                                            EpiMlemForward16, double*,
                                                            cudaStream_t);
template epet_status launch_rows16<EpiMlemUpdate, uint16_t>(const epet_csr16*, const uint16_t*,
                                                            EpiMlemUpdate, double*, cudaStream_t);
template epet_status launch_rows16<EpiKeep, uint16_t>(const epet_csr16*, const uint16_t*,
                                                      EpiKeep, double*, cudaStream_t);

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
    cudaError_t e = dev_alloc((void**)&tmp, scan_tmp_elems(a->m + 1) * 8, st);
    rc = e == cudaSuccess ? exclusive_scan_i64(cnt, out->row_ptr, a->m, tmp, st)
                          : cuda_status(e, "allocation of the scan");
    if (tmp) dev_free(tmp, st);
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
  return launch_rows16<EpiStore, float>(a, x_d, EpiStore{alpha, beta, y_d}, nullptr,
                                       (cudaStream_t)stream);
}

}  // extern "C"
