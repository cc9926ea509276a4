// sort.cu -- scan, stable LSD radix sort, and the sparse-format operators
// built on them: cooSort, coo2csr, csr2ecsr and the column-major copy.
//
// The reference sorts COO triples with thrust's comparison sort_by_key
// (cooSort.hpp:53-71, a merge sort) and converts with cusparseXcoo2csr
// (cusparseWrapper.hpp:38-45) and a host loop of three synchronous copies per
// row (convertCsr2Ecsr.hpp:34-47).  Here: an 8-bit-digit LSD radix sort on a
// packed (row, col) key, stable within each tile by warp-ordered ranking
// (__match_any_sync), a histogram+scan row pointer, and one gather kernel.
#include <algorithm>
#include <type_traits>
#include <mutex>

#include <cuda.h>

#include "common.cuh"
#include "internal.h"

namespace epet {

// ------------------------------------------------------------------ scan
constexpr int kScanThreads = 256, kScanItems = 8,
              kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads)
k_scan_tile(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
            int64_t* __restrict__ tile_sums) {
  __shared__ int64_t warp_tot[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  // block exclusive scan of s
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    int64_t t = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
    int64_t ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t u = __shfl_up_sync(0xffffffffu, ti, o);
      if (lane >= o) ti += u;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = ti - t;
    if (lane == kScanThreads / 32 - 1) tile_sums[blockIdx.x] = ti;
  }
  __syncthreads();
  int64_t run = warp_tot[w] + inc - s;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n,
                           const int64_t* __restrict__ tile_off) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_off[i / kScanTile];
}

__global__ void k_set_total(int64_t* out, int64_t n, const int64_t* tile_sums_scanned,
                            int64_t ntiles) {
  // out[n] = exclusive offset of the last tile + its sum; the scanned tile
  // array has ntiles+1 entries, the last one being the total.
  out[n] = tile_sums_scanned[ntiles];
}

size_t scan_tmp_elems(int64_t n) {
  size_t t = 0;
  int64_t k = n;
  while (true) {
    int64_t tiles = (k + kScanTile - 1) / kScanTile;
    if (tiles < 1) tiles = 1;
    t += 2 * (size_t)(tiles + 1);
    if (tiles == 1) break;
    k = tiles;
  }
  return t + 2;
}

epet_status exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n,
                               int64_t* tmp, cudaStream_t st) {
  if (n <= 0) {
    EPET_CUDA(cudaMemsetAsync(out, 0, 8, st));
    return EPET_OK;
  }
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  int64_t* sums = tmp;
  int64_t* sums_scan = tmp + (tiles + 1);
  k_scan_tile<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums);
  EPET_LAUNCHED();
  if (tiles == 1) {
    EPET_CUDA(cudaMemcpyAsync(out + n, sums, 8, cudaMemcpyDeviceToDevice, st));
    return EPET_OK;
  }
  EPET_CHECK(exclusive_scan_i64(sums, sums_scan, tiles, tmp + 2 * (tiles + 1), st));
  k_scan_add<<<ceil_div(n, 256), 256, 0, st>>>(out, n, sums_scan);
  EPET_LAUNCHED();
  k_set_total<<<1, 1, 0, st>>>(out, n, sums_scan, tiles);
  EPET_LAUNCHED();
  return EPET_OK;
}

static int bits_for(int64_t maxval) {
  int b = 0;
  while (b < 63 && (int64_t(1) << b) <= maxval) b++;
  return b;
}

// ------------------------------------------------------------ radix sort
//
// Stable LSD radix sort with BITS-bit digits, reduce-then-scan over chunks:
// the input is cut into nchunks equal runs of whole tiles (a few per SM);
// the histogram kernel counts each chunk's digits (BINS x nchunks counts),
// an exclusive scan of the digit-major counts gives every (digit, chunk) its
// output start, and the scatter kernel walks its chunk's tiles in order,
// keeping a running output offset per digit.  Within a tile, items are
// ranked stably -- warp w owns items [w*512, (w+1)*512) and ranks them in 16
// rounds of 32 consecutive items with __match_any_sync -- and staged in
// shared memory in digit order, so each digit's global writes are
// contiguous runs.  Input and output go through adapters, so the first pass
// of the column-major copy reads a CSR directly and the last one writes the
// CSC arrays and its column starts.
constexpr int kRsThreads = 256, kRsItems = 16, kRsTile = kRsThreads * kRsItems;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsMaxChunks = 2048;

struct RsGrid {
  int64_t tiles, tpc;  // tiles, tiles per chunk
  int nchunks;
};
static RsGrid rs_grid(int64_t n) {
  RsGrid g;
  g.tiles = std::max<int64_t>(1, (n + kRsTile - 1) / kRsTile);
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = std::min<int64_t>(kRsMaxChunks, 3 * (int64_t)sms);
  g.tpc = (g.tiles + want - 1) / want;
  g.nchunks = (int)((g.tiles + g.tpc - 1) / g.tpc);
  return g;
}

// A pass whose digit is the same in every key is the identity permutation.
// `vary` (device, optional) holds the OR and the AND of all keys; where
// given, a pass over a digit with no varying bit only copies its input.
__device__ __forceinline__ bool pass_active(const uint64_t* vary, int shift, unsigned mask) {
  return !vary || ((unsigned)((vary[0] ^ vary[1]) >> shift) & mask) != 0u;
}

template <int BITS, typename In>
__global__ void __launch_bounds__(kRsThreads)
k_radix_hist(In in, int64_t n, int shift, int64_t tpc, int nchunks, int64_t* __restrict__ hist,
             const uint64_t* __restrict__ vary) {
  constexpr int BINS = 1 << BITS;
  if (!pass_active(vary, shift, BINS - 1)) {
    for (int d = threadIdx.x; d < BINS; d += kRsThreads) hist[(int64_t)d * nchunks + blockIdx.x] = 0;
    return;
  }
  __shared__ unsigned cnt[BINS];
  for (int d = threadIdx.x; d < BINS; d += kRsThreads) cnt[d] = 0;
  __syncthreads();
  const int64_t beg = (int64_t)blockIdx.x * tpc * kRsTile;
  const int64_t end = min(n, beg + tpc * kRsTile);
  for (int64_t i = beg + threadIdx.x; i < end; i += kRsThreads)
    atomicAdd(&cnt[(unsigned)(in.key(i) >> shift) & (BINS - 1)], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < BINS; d += kRsThreads)
    hist[(int64_t)d * nchunks + blockIdx.x] = cnt[d];
}

// Plain arrays in / out.
template <typename K, typename V>
struct ArrIn {
  const K* k;
  const V* v;
  __device__ K key(int64_t i) const { return k[i]; }
  __device__ V val(int64_t i) const { return v[i]; }
};
template <typename K, typename V>
struct ArrOut {
  K* k;
  V* v;
  __device__ void put(int64_t pos, K key, V val, bool) const {
    k[pos] = key;
    v[pos] = val;
  }
};

// CSR in, with the row of every entry precomputed (k_row_ids): key =
// column, value = (row << 32) | value bits.
struct CsrIn {
  const int32_t* col;
  const int32_t* row;
  const float* vals;
  __device__ uint32_t key(int64_t i) const { return (uint32_t)col[i]; }
  __device__ uint64_t val(int64_t i) const {
    return ((uint64_t)(uint32_t)row[i] << 32) | __float_as_uint(vals[i]);
  }
};
// The columns of a CSR with each entry's position as its value (the
// positions' column-major order: no rows, no values read).
struct PosIn {
  const int32_t* col;
  __device__ uint32_t key(int64_t i) const { return (uint32_t)col[i]; }
  __device__ uint32_t val(int64_t i) const { return (uint32_t)i; }
};
// CSR-ordered keys (runs of ascending columns): ranked by ballots.
template <typename In>
struct IsCsrIn : std::false_type {};
template <>
struct IsCsrIn<CsrIn> : std::true_type {};
template <>
struct IsCsrIn<PosIn> : std::true_type {};

// Row id of every CSR entry (a warp per row).
__global__ void k_row_ids(const int64_t* __restrict__ row_ptr, int64_t m,
                          int32_t* __restrict__ row) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= m) return;
  for (int64_t k = row_ptr[r] + (threadIdx.x & 31); k < row_ptr[r + 1]; k += 32)
    row[k] = (int32_t)r;
}

// Positions in column-major order out, with the column starts (as CscOut).
struct PosCscOut {
  uint32_t* pos;
  int64_t* col_first;
  __device__ void put(int64_t p, uint32_t k, uint32_t v, bool first) const {
    pos[p] = v;
    if (first) atomicMin(reinterpret_cast<unsigned long long*>(col_first + k),
                         (unsigned long long)p);
  }
};

// CSC out: row and value arrays; the first position of every column goes to
// col_first (atomicMin, initialised to nnz; empty columns are filled in
// afterwards by a suffix minimum).  Only the last pass writes this form, so
// a staged run of one digit is sorted by the full key.
struct CscOut {
  int32_t* row;
  float* val;
  int64_t* col_first;
  __device__ void put(int64_t pos, uint32_t k, uint64_t v, bool first) const {
    row[pos] = (int32_t)(v >> 32);
    val[pos] = __uint_as_float((uint32_t)v);
    if (first) atomicMin(reinterpret_cast<unsigned long long*>(col_first + k),
                         (unsigned long long)pos);
  }
};

template <int BITS, typename K, typename V, typename In, typename Out>
__global__ void __launch_bounds__(kRsThreads, 3)
k_radix_scatter(In in, Out out, int64_t n, int shift, int64_t tpc, int nchunks,
                const int64_t* __restrict__ offs, const uint64_t* __restrict__ vary) {
  constexpr int BINS = 1 << BITS;
  if (!pass_active(vary, shift, BINS - 1)) {
    const int64_t beg = (int64_t)blockIdx.x * tpc * kRsTile;
    const int64_t end = min(n, beg + tpc * kRsTile);
    for (int64_t i = beg + threadIdx.x; i < end; i += kRsThreads)
      out.put(i, in.key(i), in.val(i), false);
    return;
  }
  __shared__ unsigned wcnt[kRsWarps][BINS];
  __shared__ unsigned dstart[BINS + 1];
  __shared__ unsigned warp_tot[kRsWarps];
  __shared__ int64_t run[BINS];  // output position of the chunk's next item of each digit
  extern __shared__ __align__(16) unsigned char rs_dyn[];  // staged tile
  V* sv = reinterpret_cast<V*>(rs_dyn);
  K* sk = reinterpret_cast<K*>(rs_dyn + sizeof(V) * kRsTile);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < BINS; d += kRsThreads) run[d] = offs[(int64_t)d * nchunks + blockIdx.x];
  constexpr int DPT = (BINS + kRsThreads - 1) / kRsThreads;  // digits per thread
  const unsigned lt = (1u << lane) - 1u;
  for (int64_t t = 0; t < tpc; t++) {
    const int64_t tile0 = ((int64_t)blockIdx.x * tpc + t) * kRsTile;
    if (tile0 >= n) break;
    const int tile_n = (int)(n - tile0 < kRsTile ? n - tile0 : kRsTile);
    for (int d = lane; d < BINS; d += 32) wcnt[w][d] = 0;
    __syncwarp();
    const int64_t wbase = tile0 + (int64_t)w * (kRsItems * 32);
    // keys only in registers (ranking); values are read once, when staged
    K kk[kRsItems];
    unsigned rank[kRsItems];
#pragma unroll
    for (int r = 0; r < kRsItems; r++) {
      const int64_t i = wbase + r * 32 + lane;
      kk[r] = i < n ? in.key(i) : K(0);
    }
#pragma unroll
    for (int r = 0; r < kRsItems; r++) {
      const int64_t i = wbase + r * 32 + lane;
      const bool ok = i < n;
      const unsigned dig = ok ? ((unsigned)(kk[r] >> shift) & (BINS - 1)) : BINS + lane;
      unsigned peers;
      if constexpr (IsCsrIn<In>::value) {
        // rows of a CSR: consecutive columns, up to 32 distinct digits per
        // round, where one ballot per digit bit is cheaper than a match
        peers = __ballot_sync(0xffffffffu, ok);
        peers = ok ? peers : (1u << lane);
#pragma unroll
        for (int b = 0; b < BITS; b++) {
          const bool bit = (dig >> b) & 1u;
          const unsigned bal = __ballot_sync(0xffffffffu, bit);
          peers &= bit ? bal : ~bal;
        }
      } else {
        peers = __match_any_sync(0xffffffffu, dig);
      }
      unsigned before = 0;
      if (ok) before = wcnt[w][dig];
      rank[r] = before + __popc(peers & lt);
      __syncwarp();
      const int leader = 31 - __clz(peers);
      if (ok && lane == leader) wcnt[w][dig] = before + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // per digit: warp offsets (exclusive over warps) and the digit total
    unsigned tot[DPT];
    unsigned mysum = 0;
#pragma unroll
    for (int q = 0; q < DPT; q++) {
      const int d = threadIdx.x * DPT + q;
      unsigned acc = 0;
      if (d < BINS) {
        for (int ww = 0; ww < kRsWarps; ww++) {
          const unsigned c = wcnt[ww][d];
          wcnt[ww][d] = acc;
          acc += c;
        }
      }
      tot[q] = acc;
      mysum += acc;
    }
    // exclusive scan of the digit totals (block-wide, digits in thread order)
    unsigned inc = mysum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned u = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += u;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
      const unsigned u = lane < kRsWarps ? warp_tot[lane] : 0u;
      unsigned ti = u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned x = __shfl_up_sync(0xffffffffu, ti, o);
        if (lane >= o) ti += x;
      }
      if (lane < kRsWarps) warp_tot[lane] = ti - u;
    }
    __syncthreads();
    {
      unsigned acc = warp_tot[w] + inc - mysum;
#pragma unroll
      for (int q = 0; q < DPT; q++) {
        const int d = threadIdx.x * DPT + q;
        if (d < BINS) dstart[d] = acc;
        acc += tot[q];
      }
      if (threadIdx.x == kRsThreads - 1) dstart[BINS] = acc;
    }
    __syncthreads();
    // stage in digit order
#pragma unroll
    for (int r = 0; r < kRsItems; r++) {
      const int64_t i = wbase + r * 32 + lane;
      if (i < n) {
        const unsigned dig = (unsigned)(kk[r] >> shift) & (BINS - 1);
        const unsigned lp = dstart[dig] + wcnt[w][dig] + rank[r];
        sk[lp] = kk[r];
        sv[lp] = in.val(i);
      }
    }
    __syncthreads();
    // contiguous runs per digit
    for (int j = threadIdx.x; j < tile_n; j += kRsThreads) {
      const K key = sk[j];
      const unsigned dig = (unsigned)(key >> shift) & (BINS - 1);
      const bool first = (unsigned)j == dstart[dig] || sk[j - 1] != key;
      out.put(run[dig] + (j - (int)dstart[dig]), key, sv[j], first);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < BINS; d += kRsThreads) run[d] += dstart[d + 1] - dstart[d];
    __syncthreads();
  }
}

size_t radix_hist_elems(int64_t n) {
  const int64_t tiles = std::max<int64_t>(1, (n + kRsTile - 1) / kRsTile);
  return (size_t)512 * (size_t)std::min<int64_t>(tiles, kRsMaxChunks);
}

// One pass: histogram of `in`'s keys, scan, scatter from `in` to `out`.
template <int BITS, typename K, typename V, typename In, typename Out>
epet_status radix_pass(In in, Out out, int64_t n, int shift, int64_t* hist, int64_t* hist_scan,
                       int64_t* scan_tmp, cudaStream_t st, const uint64_t* vary = nullptr) {
  const RsGrid g = rs_grid(n);
  k_radix_hist<BITS, In><<<(unsigned)g.nchunks, kRsThreads, 0, st>>>(in, n, shift, g.tpc,
                                                                     g.nchunks, hist, vary);
  EPET_LAUNCHED();
  EPET_CHECK(exclusive_scan_i64(hist, hist_scan, (int64_t)(1 << BITS) * g.nchunks, scan_tmp, st));
  const size_t dyn = (sizeof(K) + sizeof(V)) * (size_t)kRsTile;
  EPET_CUDA(cudaFuncSetAttribute(k_radix_scatter<BITS, K, V, In, Out>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  k_radix_scatter<BITS, K, V, In, Out><<<(unsigned)g.nchunks, kRsThreads, dyn, st>>>(
      in, out, n, shift, g.tpc, g.nchunks, hist_scan, vary);
  EPET_LAUNCHED();
  return EPET_OK;
}

// Sorts (keys, vals) in place on the low `bits` bits (8-bit digits).
template <typename K, typename Vt>
epet_status radix_sort(K* keys, Vt* vals, K* alt_keys, Vt* alt_vals, int64_t n, int bits,
                       int64_t* hist, int64_t* hist_scan, int64_t* scan_tmp,
                       cudaStream_t st) {
  if (n <= 1 || bits <= 0) return EPET_OK;
  K *src_k = keys, *dst_k = alt_keys;
  Vt *src_v = vals, *dst_v = alt_vals;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += 8, passes++) {
    EPET_CHECK((radix_pass<8, K, Vt>(ArrIn<K, Vt>{src_k, src_v}, ArrOut<K, Vt>{dst_k, dst_v},
                                      n, shift, hist, hist_scan, scan_tmp, st)));
    std::swap(src_k, dst_k);
    std::swap(src_v, dst_v);
  }
  if (passes & 1) {
    EPET_CUDA(cudaMemcpyAsync(keys, src_k, n * sizeof(K), cudaMemcpyDeviceToDevice, st));
    EPET_CUDA(cudaMemcpyAsync(vals, src_v, n * sizeof(Vt), cudaMemcpyDeviceToDevice, st));
  }
  return EPET_OK;
}

// ----------------------------------------------------------- COO helpers
__global__ void k_pack_coo(const int32_t* row, const int32_t* col, const float* val,
                           int64_t n, int colbits, uint64_t* key, uint32_t* v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    key[i] = ((uint64_t)(uint32_t)row[i] << colbits) | (uint32_t)col[i];
    v[i] = __float_as_uint(val[i]);
  }
}

__global__ void k_unpack_coo(const uint64_t* key, const uint32_t* v, int64_t n, int colbits,
                             int32_t* row, int32_t* col, float* val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    row[i] = (int32_t)(key[i] >> colbits);
    col[i] = (int32_t)(key[i] & ((uint64_t(1) << colbits) - 1));
    val[i] = __uint_as_float(v[i]);
  }
}

__global__ void k_max2(const int32_t* a, const int32_t* b, int64_t n, int* out) {
  int ma = 0, mb = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    ma = max(ma, a[i]);
    mb = max(mb, b[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ma = max(ma, __shfl_xor_sync(0xffffffffu, ma, o));
    mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], ma);
    atomicMax(&out[1], mb);
  }
}

__global__ void k_min2(const int32_t* a, const int32_t* b, int64_t n, int* out) {
  int ma = 0, mb = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    ma = min(ma, a[i]);
    mb = min(mb, b[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ma = min(ma, __shfl_xor_sync(0xffffffffu, ma, o));
    mb = min(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out[0], ma);
    atomicMin(&out[1], mb);
  }
}

// Row pointer from row-sorted ids: csr[r] = #entries with row < r
// (lower bound per r).
__global__ void k_coo2csr(const int32_t* __restrict__ row, int64_t nnz, int64_t m,
                          int64_t* __restrict__ csr) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r > m) return;
  int64_t lo = 0, hi = nnz;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (row[mid] < r) lo = mid + 1;
    else hi = mid;
  }
  csr[r] = lo;
}

__global__ void k_csr2ecsr(int64_t* ecsr, const int32_t* yrow, int64_t nnzr,
                           const int64_t* csr, int64_t m) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nnzr) ecsr[i] = csr[yrow[i]];
  if (i == nnzr) ecsr[nnzr] = csr[m];
}

__global__ void k_fill_i64(int64_t* p, int64_t n, int64_t v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// p[i] = min(p[i..n-1]) by one block: per-thread chunk minima, a block-wide
// suffix scan of them, then the chunks.
__global__ void __launch_bounds__(1024) k_suffix_min_i64(int64_t* p, int64_t n) {
  __shared__ int64_t cm[1024];
  const int t = threadIdx.x;
  const int64_t per = (n + 1023) / 1024;
  const int64_t b = min(n, t * per), e = min(n, b + per);
  int64_t m = INT64_MAX;
  for (int64_t i = e - 1; i >= b; i--) m = min(m, p[i]);
  cm[t] = m;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int64_t v = t + o < 1024 ? cm[t + o] : INT64_MAX;
    __syncthreads();
    cm[t] = min(cm[t], v);
    __syncthreads();
  }
  int64_t run = t + 1 < 1024 ? cm[t + 1] : INT64_MAX;
  for (int64_t i = e - 1; i >= b; i--) {
    run = min(run, p[i]);
    p[i] = run;
  }
}

}  // namespace epet

using namespace epet;

extern "C" {

size_t epet_coo_sort_workspace_size(int64_t n) {
  const size_t hist = radix_hist_elems(n);
  return 2 * align256(n * 8) + 2 * align256(n * 4) + align256(hist * 8) +
         align256((hist + 1) * 8) + align256(scan_tmp_elems(hist) * 8) + 256;
}

epet_status epet_coo_sort(float* val_d, int32_t* row_d, int32_t* col_d, int64_t n,
                          void* ws, size_t ws_bytes, epet_stream_t stream) {
  if (n < 0 || (n > 0 && (!val_d || !row_d || !col_d)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  if (n <= 1) return EPET_OK;
  cudaStream_t st = (cudaStream_t)stream;
  Scratch scr;
  EPET_CHECK(scr.init(ws, ws_bytes, epet_coo_sort_workspace_size(n), st));
  uint64_t* key = scr.take<uint64_t>(n);
  uint64_t* key2 = scr.take<uint64_t>(n);
  uint32_t* v = scr.take<uint32_t>(n);
  uint32_t* v2 = scr.take<uint32_t>(n);
  const size_t hn = radix_hist_elems(n);
  int64_t* hist = scr.take<int64_t>(hn);
  int64_t* hist_scan = scr.take<int64_t>(hn + 1);
  int64_t* tmp = scr.take<int64_t>(scan_tmp_elems(hn));
  int* mx = scr.take<int>(4);
  if (scr.overrun) return set_error(EPET_ERR_INVALID, "internal: workspace size");
  // index ranges (ids must be non-negative)
  int h_mx[2] = {0, 0}, h_mn[2] = {0, 0};
  EPET_CUDA(cudaMemsetAsync(mx, 0, 16, st));
  k_max2<<<std::min(ceil_div(n, 256), 1024), 256, 0, st>>>(row_d, col_d, n, mx);
  EPET_LAUNCHED();
  k_min2<<<std::min(ceil_div(n, 256), 1024), 256, 0, st>>>(row_d, col_d, n, mx + 2);
  EPET_LAUNCHED();
  EPET_CUDA(cudaMemcpyAsync(h_mx, mx, 8, cudaMemcpyDeviceToHost, st));
  EPET_CUDA(cudaMemcpyAsync(h_mn, mx + 2, 8, cudaMemcpyDeviceToHost, st));
  EPET_CUDA(cudaStreamSynchronize(st));
  if (h_mn[0] < 0 || h_mn[1] < 0)
    return set_error(EPET_ERR_INVALID, "negative row/column index");
  const int colbits = std::max(1, bits_for(h_mx[1]));
  const int rowbits = std::max(1, bits_for(h_mx[0]));
  const int T = 256;
  k_pack_coo<<<ceil_div(n, T), T, 0, st>>>(row_d, col_d, val_d, n, colbits, key, v);
  EPET_LAUNCHED();
  EPET_CHECK((radix_sort<uint64_t, uint32_t>(key, v, key2, v2, n, colbits + rowbits, hist,
                                             hist_scan, tmp, st)));
  k_unpack_coo<<<ceil_div(n, T), T, 0, st>>>(key, v, n, colbits, row_d, col_d, val_d);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status epet_coo2csr(const int32_t* row_d, int64_t nnz, int64_t m, int64_t* csr_d,
                         epet_stream_t stream) {
  if (nnz < 0 || m < 0 || !csr_d || (nnz > 0 && !row_d))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  k_coo2csr<<<ceil_div(m + 1, 256), 256, 0, (cudaStream_t)stream>>>(row_d, nnz, m, csr_d);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status epet_csr2ecsr(int64_t* ecsr_d, const int32_t* yrow_d, int64_t nnzr,
                          const int64_t* csr_d, int64_t m, epet_stream_t stream) {
  if (nnzr < 0 || m < 0 || !ecsr_d || !csr_d || (nnzr > 0 && !yrow_d))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  k_csr2ecsr<<<ceil_div(nnzr + 1, 256), 256, 0, (cudaStream_t)stream>>>(ecsr_d, yrow_d, nnzr,
                                                                         csr_d, m);
  EPET_LAUNCHED();
  return EPET_OK;
}

// Radix passes of the column-major copy: one 9-bit pass up to 2^9 columns,
// an 8/9-bit and a 9-bit pass up to 2^18, then 9-bit passes (ping-pong
// through a second key/value pair) up to the int32 column range.
static int csc_passes(int64_t n) {
  const int bits = std::max(1, bits_for(n - 1));
  return bits <= 18 ? (bits <= 9 ? 1 : 2) : (bits + 8) / 9;
}

size_t epet_csr_to_csc_workspace_size(int64_t m, int64_t n, int64_t nnz) {
  (void)m;
  const size_t hist = radix_hist_elems(nnz);
  const size_t pair = csc_passes(n) > 2 ? 2 : 1;  // key/value pairs between passes
  return 2 * align256(nnz * 4) + align256(nnz * 8) + (pair - 1) * (align256(nnz * 4) +
         align256(nnz * 8)) + align256(hist * 8) + align256((hist + 1) * 8) +
         align256(scan_tmp_elems(hist) * 8) + 256;
}

}  // extern "C"

namespace epet {
// The column-major copy of a CSR.
static epet_status csr_to_csc_impl(const epet_csr* a, epet_csc* out, void* ws, size_t ws_bytes,
                                   epet_stream_t stream) {
  if (!a || !out || !out->col_ptr || (a->nnz > 0 && (!out->row || !out->val)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  if (a->n < 0 || a->n > (int64_t)INT32_MAX + 1)
    return set_error(EPET_ERR_INVALID, "column count %lld", (long long)a->n);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nnz = a->nnz;
  out->m = a->m;
  out->n = a->n;
  out->nnz = nnz;
  if (nnz == 0) {
    EPET_CUDA(cudaMemsetAsync(out->col_ptr, 0, (a->n + 1) * 8, st));
    return EPET_OK;
  }
  Scratch scr;
  EPET_CHECK(scr.init(ws, ws_bytes, epet_csr_to_csc_workspace_size(a->m, a->n, nnz), st));
  const int passes = csc_passes(a->n);
  uint32_t* key = scr.take<uint32_t>(nnz);
  uint64_t* pv = scr.take<uint64_t>(nnz);
  uint32_t* key2 = passes > 2 ? scr.take<uint32_t>(nnz) : nullptr;
  uint64_t* pv2 = passes > 2 ? scr.take<uint64_t>(nnz) : nullptr;
  const size_t hn = radix_hist_elems(nnz);
  int64_t* hist = scr.take<int64_t>(hn);
  int64_t* hist_scan = scr.take<int64_t>(hn + 1);
  int64_t* tmp = scr.take<int64_t>(scan_tmp_elems(hn));
  int32_t* rid = scr.take<int32_t>(nnz);
  if (scr.overrun) return set_error(EPET_ERR_INVALID, "internal: workspace size");
  const int bits = std::max(1, bits_for(a->n - 1));
  k_row_ids<<<ceil_div(a->m * 32, 256), 256, 0, st>>>(a->row_ptr, a->m, rid);
  EPET_LAUNCHED();
  CsrIn in{a->col, rid, a->val};
  CscOut co{out->row, out->val, out->col_ptr};
  k_fill_i64<<<ceil_div(a->n + 1, 256), 256, 0, st>>>(out->col_ptr, a->n + 1, nnz);
  EPET_LAUNCHED();
  if (passes == 1) {
    // one pass: CSR -> CSC
    EPET_CHECK((radix_pass<9, uint32_t, uint64_t>(in, co, nnz, 0, hist, hist_scan, tmp, st)));
  } else if (passes == 2) {
    // low digits: CSR -> (key, row|val); high digits -> CSC
    const int b0 = bits - 9;
    ArrOut<uint32_t, uint64_t> mid{key, pv};
    ArrIn<uint32_t, uint64_t> mid_in{key, pv};
    if (b0 <= 8) EPET_CHECK((radix_pass<8, uint32_t, uint64_t>(in, mid, nnz, 0, hist, hist_scan, tmp, st)));
    else EPET_CHECK((radix_pass<9, uint32_t, uint64_t>(in, mid, nnz, 0, hist, hist_scan, tmp, st)));
    EPET_CHECK((radix_pass<9, uint32_t, uint64_t>(mid_in, co, nnz, b0 <= 8 ? 8 : 9, hist,
                                                  hist_scan, tmp, st)));
  } else {
    // 9-bit digits from the least significant: CSR -> pair 0, pair k%2 ->
    // pair (k+1)%2, the last one -> CSC
    uint32_t* ks[2] = {key, key2};
    uint64_t* vs[2] = {pv, pv2};
    EPET_CHECK((radix_pass<9, uint32_t, uint64_t>(in, ArrOut<uint32_t, uint64_t>{ks[0], vs[0]},
                                                  nnz, 0, hist, hist_scan, tmp, st)));
    for (int k = 1; k < passes; k++) {
      ArrIn<uint32_t, uint64_t> src{ks[(k - 1) & 1], vs[(k - 1) & 1]};
      if (k + 1 < passes)
        EPET_CHECK((radix_pass<9, uint32_t, uint64_t>(src, ArrOut<uint32_t, uint64_t>{ks[k & 1],
                                                      vs[k & 1]}, nnz, 9 * k, hist, hist_scan,
                                                      tmp, st)));
      else
        EPET_CHECK((radix_pass<9, uint32_t, uint64_t>(src, co, nnz, 9 * k, hist, hist_scan, tmp,
                                                      st)));
    }
  }
  // empty columns start where the next non-empty one does
  k_suffix_min_i64<<<1, 1024, 0, st>>>(out->col_ptr, a->n + 1);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status csr_to_csc_positions(int64_t nnz, int64_t n, const int32_t* col, int64_t* col_ptr,
                                 uint32_t* pos, cudaStream_t st) {
  if (n < 0 || n > (int64_t)INT32_MAX + 1 || nnz < 0 || nnz > (int64_t)INT32_MAX)
    return set_error(EPET_ERR_INVALID, "positions: %lld entries, %lld columns", (long long)nnz,
                     (long long)n);
  if (nnz == 0) {
    EPET_CUDA(cudaMemsetAsync(col_ptr, 0, (n + 1) * 8, st));
    return EPET_OK;
  }
  const int passes = csc_passes(n);
  const size_t hn = radix_hist_elems(nnz);
  Scratch scr;
  EPET_CHECK(scr.init(nullptr, 0,
                      2 * (passes > 2 ? 2 : 1) * align256(nnz * 4) + align256(hn * 8) +
                          align256((hn + 1) * 8) + align256(scan_tmp_elems(hn) * 8) + 256,
                      st));
  uint32_t* ks[2] = {scr.take<uint32_t>(nnz), passes > 2 ? scr.take<uint32_t>(nnz) : nullptr};
  uint32_t* vs[2] = {scr.take<uint32_t>(nnz), passes > 2 ? scr.take<uint32_t>(nnz) : nullptr};
  int64_t* hist = scr.take<int64_t>(hn);
  int64_t* hist_scan = scr.take<int64_t>(hn + 1);
  int64_t* tmp = scr.take<int64_t>(scan_tmp_elems(hn));
  if (scr.overrun) return set_error(EPET_ERR_INVALID, "internal: workspace size");
  const int bits = std::max(1, bits_for(n - 1));
  PosIn in{col};
  PosCscOut co{pos, col_ptr};
  k_fill_i64<<<ceil_div(n + 1, 256), 256, 0, st>>>(col_ptr, n + 1, nnz);
  EPET_LAUNCHED();
  using K = uint32_t;
  using V = uint32_t;
  if (passes == 1) {
    EPET_CHECK((radix_pass<9, K, V>(in, co, nnz, 0, hist, hist_scan, tmp, st)));
  } else if (passes == 2) {
    const int b0 = bits - 9;
    ArrOut<K, V> mid{ks[0], vs[0]};
    if (b0 <= 8) EPET_CHECK((radix_pass<8, K, V>(in, mid, nnz, 0, hist, hist_scan, tmp, st)));
    else EPET_CHECK((radix_pass<9, K, V>(in, mid, nnz, 0, hist, hist_scan, tmp, st)));
    EPET_CHECK((radix_pass<9, K, V>(ArrIn<K, V>{ks[0], vs[0]}, co, nnz, b0 <= 8 ? 8 : 9, hist,
                                    hist_scan, tmp, st)));
  } else {
    EPET_CHECK((radix_pass<9, K, V>(in, ArrOut<K, V>{ks[0], vs[0]}, nnz, 0, hist, hist_scan, tmp,
                                    st)));
    for (int k = 1; k < passes; k++) {
      ArrIn<K, V> src{ks[(k - 1) & 1], vs[(k - 1) & 1]};
      if (k + 1 < passes)
        EPET_CHECK((radix_pass<9, K, V>(src, ArrOut<K, V>{ks[k & 1], vs[k & 1]}, nnz, 9 * k,
                                        hist, hist_scan, tmp, st)));
      else
        EPET_CHECK((radix_pass<9, K, V>(src, co, nnz, 9 * k, hist, hist_scan, tmp, st)));
    }
  }
  k_suffix_min_i64<<<1, 1024, 0, st>>>(col_ptr, n + 1);
  EPET_LAUNCHED();
  return EPET_OK;
}
}  // namespace epet

extern "C" epet_status epet_csr_to_csc(const epet_csr* a, epet_csc* out, void* ws,
                                       size_t ws_bytes, epet_stream_t stream) {
  return csr_to_csc_impl(a, out, ws, ws_bytes, stream);
}

// ----------------------------------------------- allocation-free cooSort
//
// For callers that must not allocate device memory from inside the library
// call: a host process whose own allocator owns all device memory, an
// integration whose memory budget is fixed at start-up, or a loop that must
// not wait on the allocator.  The sort's scratch lives in a file-scope device
// array sized for kNoAllocCooSortMax entries (7 MiB), which every GPU that
// loads this library holds until the process exits.
//
// Unlike epet_coo_sort, this path reads nothing back to the host: the keys
// are (row, col) with the sign bits flipped (so unsigned order is the signed
// order of the reference's comparator, negative ids included), all eight
// 8-bit digits get a pass, and a pass over a digit that no key varies in
// (found on the device from the OR and AND of the keys) only copies.

namespace epet {
constexpr int64_t kNoAllocCooSortMax = int64_t(1) << 18;  // 262,144 triples
constexpr size_t kNoAllocScratchBytes = size_t(7) << 20;  // 7 MiB
static __device__ __align__(256) unsigned char g_coo_sort_scratch[kNoAllocScratchBytes];

__global__ void k_pack_coo_signed(const int32_t* row, const int32_t* col, const float* val,
                                  int64_t n, uint64_t* key, uint32_t* v, uint64_t* vary) {
  uint64_t o = 0, a = ~uint64_t(0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = ((uint64_t)((uint32_t)row[i] ^ 0x80000000u) << 32) |
                       ((uint32_t)col[i] ^ 0x80000000u);
    key[i] = k;
    v[i] = __float_as_uint(val[i]);
    o |= k;
    a &= k;
  }
  for (int s = 16; s > 0; s >>= 1) {
    o |= __shfl_xor_sync(0xffffffffu, o, s);
    a &= __shfl_xor_sync(0xffffffffu, a, s);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicOr(reinterpret_cast<unsigned long long*>(vary), (unsigned long long)o);
    atomicAnd(reinterpret_cast<unsigned long long*>(vary + 1), (unsigned long long)a);
  }
}

__global__ void k_unpack_coo_signed(const uint64_t* key, const uint32_t* v, int64_t n,
                                    int32_t* row, int32_t* col, float* val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    row[i] = (int32_t)((uint32_t)(key[i] >> 32) ^ 0x80000000u);
    col[i] = (int32_t)((uint32_t)key[i] ^ 0x80000000u);
    val[i] = __uint_as_float(v[i]);
  }
}

static size_t noalloc_scratch_need(int64_t n) {
  const size_t hn = radix_hist_elems(n);
  return 2 * align256(n * 8) + 2 * align256(n * 4) + align256(hn * 8) + align256((hn + 1) * 8) +
         align256(scan_tmp_elems(hn) * 8) + align256(16);
}

// Device address of the array, per device, for the context it was looked up
// in (a caller that makes another context current gets it looked up again).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[256];
static CUcontext g_noalloc_ctx[256];

static epet_status noalloc_scratch(void** out) {
  static CtxGetCurrentFn ctx_get = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(fn);
  }();
  int dev = 0;
  EPET_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return set_error(EPET_ERR_UNSUPPORTED, "device index %d", dev);
  // cudaGetDevice made the device's primary context current if none was
  CUcontext ctx = nullptr;
  if (ctx_get) ctx_get(&ctx);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev] || g_noalloc_ctx[dev] != ctx) {
    // the array's host-side name is a stand-in, not a device address
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_coo_sort_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_coo_sort_scratch)");
    g_noalloc_ptr[dev] = p;
    g_noalloc_ctx[dev] = ctx;
  }
  *out = g_noalloc_ptr[dev];
  return EPET_OK;
}
}  // namespace epet

extern "C" epet_status epet_coo_sort_noalloc(float* val_d, int32_t* row_d, int32_t* col_d,
                                             int64_t n, epet_stream_t stream) {
  using namespace epet;
  if (n < 0 || (n > 0 && (!val_d || !row_d || !col_d)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  if (n > kNoAllocCooSortMax)
    return set_error(EPET_ERR_CAPACITY,
                     "epet_coo_sort_noalloc sorts at most %lld triples (%lld given); use "
                     "epet_coo_sort with a workspace for larger inputs",
                     (long long)kNoAllocCooSortMax, (long long)n);
  if (n <= 1) return EPET_OK;
  if (noalloc_scratch_need(n) > kNoAllocScratchBytes)
    return set_error(EPET_ERR_INVALID, "internal: static scratch too small (%zu > %zu)",
                     noalloc_scratch_need(n), kNoAllocScratchBytes);
  void* scratch = nullptr;
  EPET_CHECK(noalloc_scratch(&scratch));
  cudaStream_t st = (cudaStream_t)stream;
  Scratch scr;  // carves the array; owns nothing
  EPET_CHECK(scr.init(scratch, kNoAllocScratchBytes, noalloc_scratch_need(n), st));
  uint64_t* key = scr.take<uint64_t>(n);
  uint64_t* key2 = scr.take<uint64_t>(n);
  uint32_t* v = scr.take<uint32_t>(n);
  uint32_t* v2 = scr.take<uint32_t>(n);
  const size_t hn = radix_hist_elems(n);
  int64_t* hist = scr.take<int64_t>(hn);
  int64_t* hist_scan = scr.take<int64_t>(hn + 1);
  int64_t* tmp = scr.take<int64_t>(scan_tmp_elems(hn));
  uint64_t* vary = scr.take<uint64_t>(2);
  if (scr.overrun) return set_error(EPET_ERR_INVALID, "internal: workspace size");
  // the array keeps the previous call's contents: the OR starts at 0, the AND at all ones
  EPET_CUDA(cudaMemsetAsync(vary, 0x00, 8, st));
  EPET_CUDA(cudaMemsetAsync(vary + 1, 0xff, 8, st));
  const int T = 256;
  k_pack_coo_signed<<<std::min(ceil_div(n, T), 1024), T, 0, st>>>(row_d, col_d, val_d, n, key,
                                                                   v, vary);
  EPET_LAUNCHED();
  // eight passes (an even count: the result ends in key / v)
  uint64_t *sk = key, *dk = key2;
  uint32_t *sv = v, *dv = v2;
  for (int shift = 0; shift < 64; shift += 8) {
    EPET_CHECK((radix_pass<8, uint64_t, uint32_t>(ArrIn<uint64_t, uint32_t>{sk, sv},
                                                  ArrOut<uint64_t, uint32_t>{dk, dv}, n, shift,
                                                  hist, hist_scan, tmp, st, vary)));
    std::swap(sk, dk);
    std::swap(sv, dv);
  }
  k_unpack_coo_signed<<<ceil_div(n, T), T, 0, st>>>(key, v, n, row_d, col_d, val_d);
  EPET_LAUNCHED();
  return EPET_OK;
}
