// rows.cuh -- the row dot products shared by the single and batched
// product kernels (spmv.cu, batch.cu).
#pragma once
#include <type_traits>

#include "common.cuh"

namespace epet {

constexpr int kSpmvThreads = 256;

// Launch plan of a row kernel: G lanes per row; vec: each lane reads 16-byte
// chunks of 4 consecutive entries, U chunks per round (else the lanes
// interleave single entries, which keeps a warp's gathers of x on
// neighbouring columns); grid = 0 for one block per tile of kSpmvThreads / G
// rows, else a persistent grid of that many blocks striding over the tiles.
struct RowPlan {
  int G = 32, U = 2, grid = 0;
  bool vec = true;  // 16-byte chunks per lane (else lanes interleave entries)
};
inline int plan_rows_per_tile(const RowPlan& p) { return kSpmvThreads / p.G; }
inline int64_t plan_tiles(const RowPlan& p, int64_t nrows) {
  const int rpt = plan_rows_per_tile(p);
  return nrows > 0 ? (nrows + rpt - 1) / rpt : 0;
}

// Matrix streams are read once per product: streaming (evict-first) loads.
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int32_t* p) { return __ldcs(p); }

// Dot product of row [beg, end) with x by a group of G lanes, element-wise
// loads (any alignment of idx / val).
template <int G>
__device__ __forceinline__ float group_dot_scalar(const int32_t* __restrict__ idx,
                                                  const float* __restrict__ val,
                                                  const float* __restrict__ x, int64_t beg,
                                                  int64_t end, int lg) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  int64_t k = beg + lg;
  for (; k + 3 * G < end; k += 4 * G) {
    const float v0 = ld_stream(val + k), v1 = ld_stream(val + k + G);
    const float v2 = ld_stream(val + k + 2 * G), v3 = ld_stream(val + k + 3 * G);
    const int c0 = ld_stream(idx + k), c1 = ld_stream(idx + k + G);
    const int c2 = ld_stream(idx + k + 2 * G), c3 = ld_stream(idx + k + 3 * G);
    a0 = fmaf(v0, __ldg(x + c0), a0);
    a1 = fmaf(v1, __ldg(x + c1), a1);
    a2 = fmaf(v2, __ldg(x + c2), a2);
    a3 = fmaf(v3, __ldg(x + c3), a3);
  }
  for (; k < end; k += G) a0 = fmaf(ld_stream(val + k), __ldg(x + ld_stream(idx + k)), a0);
  float a = (a0 + a1) + (a2 + a3);
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o, G);
  return a;
}

// The same with 16-byte loads; idx and val must be 16-byte aligned.  The
// row splits into a head (entries before the first 16-byte boundary, at most
// 3), a body of 4-entry chunks (float4 / int4 loads) and a tail (at most 3
// entries).  Lane l takes body chunks l, l + G, ...; a round covers U chunks
// per lane and the next round's loads are issued before this round's
// gathers, so up to 64*U bytes per lane of the matrix stream are in flight.
template <int G, int U>
__device__ __forceinline__ float group_dot_vec(const int32_t* __restrict__ idx,
                                               const float* __restrict__ val,
                                               const float* __restrict__ x, int64_t beg,
                                               int64_t end, int lg) {
  const int64_t h = min(end, (beg + 3) & ~int64_t(3));
  const int64_t t = max(h, end & ~int64_t(3));
  float acc[U];
#pragma unroll
  for (int u = 0; u < U; u++) acc[u] = 0.f;
  if (lg < h - beg) acc[0] = ld_stream(val + beg + lg) * __ldg(x + ld_stream(idx + beg + lg));
  if (lg < end - t) acc[U - 1] = fmaf(ld_stream(val + t + lg), __ldg(x + ld_stream(idx + t + lg)), acc[U - 1]);
  const float4* __restrict__ v4 = reinterpret_cast<const float4*>(val + h);
  const int4* __restrict__ c4 = reinterpret_cast<const int4*>(idx + h);
  const int64_t nc = (t - h) >> 2;
  // software pipeline: the loads of round r + 1 are issued before the
  // gathers of round r, so the matrix stream stays in flight while the
  // gathers wait
  float4 v[U];
  int4 c[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int64_t jj = lg + u * G;
    if (jj < nc) {
      v[u] = __ldcs(v4 + jj);
      c[u] = __ldcs(c4 + jj);
    }
  }
  for (int64_t j = lg; j < nc; j += U * G) {
    float4 vn[U];
    int4 cn[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t jj = j + (U + u) * G;
      if (jj < nc) {
        vn[u] = __ldcs(v4 + jj);
        cn[u] = __ldcs(c4 + jj);
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (j + u * G < nc) {
        acc[u] = fmaf(v[u].x, __ldg(x + c[u].x), acc[u]);
        acc[u] = fmaf(v[u].y, __ldg(x + c[u].y), acc[u]);
        acc[u] = fmaf(v[u].z, __ldg(x + c[u].z), acc[u]);
        acc[u] = fmaf(v[u].w, __ldg(x + c[u].w), acc[u]);
      }
      v[u] = vn[u];
      c[u] = cn[u];
    }
  }
  float a = acc[0];
#pragma unroll
  for (int u = 1; u < U; u++) a += acc[u];
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o, G);
  return a;
}

// The same sums with every value 1 (no value stream): sum of x over the
// row's indices, in the same order as the dot products above (a product by
// 1 is exact, so the results equal theirs).
template <int G>
__device__ __forceinline__ float group_sum_scalar(const int32_t* __restrict__ idx,
                                                  const float* __restrict__ x, int64_t beg,
                                                  int64_t end, int lg) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  int64_t k = beg + lg;
  for (; k + 3 * G < end; k += 4 * G) {
    const int c0 = ld_stream(idx + k), c1 = ld_stream(idx + k + G);
    const int c2 = ld_stream(idx + k + 2 * G), c3 = ld_stream(idx + k + 3 * G);
    a0 += __ldg(x + c0);
    a1 += __ldg(x + c1);
    a2 += __ldg(x + c2);
    a3 += __ldg(x + c3);
  }
  for (; k < end; k += G) a0 += __ldg(x + ld_stream(idx + k));
  float a = (a0 + a1) + (a2 + a3);
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o, G);
  return a;
}

template <int G, int U>
__device__ __forceinline__ float group_sum_vec(const int32_t* __restrict__ idx,
                                               const float* __restrict__ x, int64_t beg,
                                               int64_t end, int lg) {
  const int64_t h = min(end, (beg + 3) & ~int64_t(3));
  const int64_t t = max(h, end & ~int64_t(3));
  float acc[U];
#pragma unroll
  for (int u = 0; u < U; u++) acc[u] = 0.f;
  if (lg < h - beg) acc[0] = 1.f * __ldg(x + ld_stream(idx + beg + lg));
  if (lg < end - t) acc[U - 1] += __ldg(x + ld_stream(idx + t + lg));
  const int4* __restrict__ c4 = reinterpret_cast<const int4*>(idx + h);
  const int64_t nc = (t - h) >> 2;
  int4 c[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int64_t jj = lg + u * G;
    if (jj < nc) c[u] = __ldcs(c4 + jj);
  }
  for (int64_t j = lg; j < nc; j += U * G) {
    int4 cn[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t jj = j + (U + u) * G;
      if (jj < nc) cn[u] = __ldcs(c4 + jj);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (j + u * G < nc) {
        acc[u] += __ldg(x + c[u].x);
        acc[u] += __ldg(x + c[u].y);
        acc[u] += __ldg(x + c[u].z);
        acc[u] += __ldg(x + c[u].w);
      }
      c[u] = cn[u];
    }
  }
  float a = acc[0];
#pragma unroll
  for (int u = 1; u < U; u++) a += acc[u];
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o, G);
  return a;
}

// Row dot product in the form the template arguments select.
template <int G, int U, bool VEC>
__device__ __forceinline__ float row_dot(const int32_t* __restrict__ idx,
                                         const float* __restrict__ val,
                                         const float* __restrict__ x, int64_t beg, int64_t end,
                                         int lg) {
  if constexpr (VEC) return group_dot_vec<G, U>(idx, val, x, beg, end, lg);
  else return group_dot_scalar<G>(idx, val, x, beg, end, lg);
}
template <int G, int U, bool VEC>
__device__ __forceinline__ float row_sum(const int32_t* __restrict__ idx,
                                         const float* __restrict__ x, int64_t beg, int64_t end,
                                         int lg) {
  if constexpr (VEC) return group_sum_vec<G, U>(idx, x, beg, end, lg);
  else return group_sum_scalar<G>(idx, x, beg, end, lg);
}

// Fixed-order block sum of one double per thread into *out (thread 0);
// red holds kSpmvThreads / 32 doubles; ends with a barrier so red can be
// reused.
__device__ __forceinline__ void block_sum_to(double part, double* red, double* out) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kSpmvThreads / 32; w++) t += red[w];
    *out = t;
  }
  __syncthreads();
}

// Calls f(integral_constant<G>, integral_constant<U>, bool_constant<VEC>)
// for the plan's values (the interleaved form has one unroll; it is also the
// form for streams not on 16-byte boundaries).
template <class F>
void dispatch_plan(const RowPlan& p, bool aligned, F&& f) {
  using std::integral_constant;
  const bool vec = aligned && p.vec;
  auto with_u = [&](auto g) {
    if (!vec) return f(g, integral_constant<int, 1>{}, std::false_type{});
    switch (p.U) {
      case 1: return f(g, integral_constant<int, 1>{}, std::true_type{});
      case 4: return f(g, integral_constant<int, 4>{}, std::true_type{});
      default: return f(g, integral_constant<int, 2>{}, std::true_type{});
    }
  };
  switch (p.G) {
    case 32: return with_u(integral_constant<int, 32>{});
    case 16: return with_u(integral_constant<int, 16>{});
    case 8: return with_u(integral_constant<int, 8>{});
    default: return with_u(integral_constant<int, 4>{});
  }
}

inline bool aligned16(const void* a, const void* b) {
  return ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0;
}

}  // namespace epet
