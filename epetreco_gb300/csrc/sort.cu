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

// ------------------------------------------------------------ radix sort
constexpr int kRsThreads = 256, kRsItems = 16, kRsTile = kRsThreads * kRsItems;
constexpr int kRsWarps = kRsThreads / 32;

template <typename K>
__global__ void __launch_bounds__(kRsThreads)
k_radix_hist(const K* __restrict__ keys, int64_t n, int shift, int64_t ntiles,
             int64_t* __restrict__ hist) {
  __shared__ unsigned cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
#pragma unroll 4
  for (int k = 0; k < kRsItems; k++) {
    const int64_t i = base + k * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(unsigned)(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter: warp w ranks items [w*512, (w+1)*512) of the tile in 16
// rounds of 32 consecutive items; ranks follow (warp, round, lane) order.
template <typename K, typename Vt>
__global__ void __launch_bounds__(kRsThreads)
k_radix_scatter(const K* __restrict__ keys, const Vt* __restrict__ vals, int64_t n,
                int shift, int64_t ntiles, const int64_t* __restrict__ offs,
                K* __restrict__ okeys, Vt* __restrict__ ovals) {
  __shared__ unsigned wcnt[kRsWarps][256];
  __shared__ int64_t base_off[256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int d = lane; d < 256; d += 32) wcnt[w][d] = 0;
  base_off[threadIdx.x] = offs[(int64_t)threadIdx.x * ntiles + blockIdx.x];
  __syncwarp();
  const int64_t wbase = (int64_t)blockIdx.x * kRsTile + (int64_t)w * (kRsItems * 32);
  K kk[kRsItems];
  unsigned rank[kRsItems];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < kRsItems; r++) {
    const int64_t i = wbase + r * 32 + lane;
    const bool ok = i < n;
    kk[r] = ok ? keys[i] : K(0);
    const unsigned dig = ok ? ((unsigned)(kk[r] >> shift) & 255u) : 256u + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, dig);
    unsigned before = 0;
    if (ok) before = wcnt[w][dig];
    rank[r] = before + __popc(peers & lt);
    __syncwarp();
    const int leader = 31 - __clz(peers);
    if (ok && lane == leader) wcnt[w][dig] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // exclusive prefix over warps per digit
  {
    const int d = threadIdx.x;
    unsigned run = 0;
    for (int ww = 0; ww < kRsWarps; ww++) {
      unsigned c = wcnt[ww][d];
      wcnt[ww][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRsItems; r++) {
    const int64_t i = wbase + r * 32 + lane;
    if (i < n) {
      const unsigned dig = (unsigned)(kk[r] >> shift) & 255u;
      const int64_t pos = base_off[dig] + wcnt[w][dig] + rank[r];
      okeys[pos] = kk[r];
      ovals[pos] = vals[i];
    }
  }
}

size_t radix_hist_elems(int64_t n) {
  const int64_t tiles = std::max<int64_t>(1, (n + kRsTile - 1) / kRsTile);
  return (size_t)256 * tiles;
}

template <typename K, typename Vt>
epet_status radix_sort(K* keys, Vt* vals, K* alt_keys, Vt* alt_vals, int64_t n, int bits,
                       int64_t* hist, int64_t* hist_scan, int64_t* scan_tmp,
                       cudaStream_t st) {
  if (n <= 1 || bits <= 0) return EPET_OK;
  const int64_t ntiles = (n + kRsTile - 1) / kRsTile;
  K *src_k = keys, *dst_k = alt_keys;
  Vt *src_v = vals, *dst_v = alt_vals;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += 8, passes++) {
    k_radix_hist<K><<<(unsigned)ntiles, kRsThreads, 0, st>>>(src_k, n, shift, ntiles, hist);
    EPET_LAUNCHED();
    EPET_CHECK(exclusive_scan_i64(hist, hist_scan, 256 * ntiles, scan_tmp, st));
    k_radix_scatter<K, Vt><<<(unsigned)ntiles, kRsThreads, 0, st>>>(
        src_k, src_v, n, shift, ntiles, hist_scan, dst_k, dst_v);
    EPET_LAUNCHED();
    std::swap(src_k, dst_k);
    std::swap(src_v, dst_v);
  }
  if (passes & 1) {
    EPET_CUDA(cudaMemcpyAsync(keys, src_k, n * sizeof(K), cudaMemcpyDeviceToDevice, st));
    EPET_CUDA(cudaMemcpyAsync(vals, src_v, n * sizeof(Vt), cudaMemcpyDeviceToDevice, st));
  }
  return EPET_OK;
}

static int bits_for(int64_t maxval) {
  int b = 0;
  while (b < 63 && (int64_t(1) << b) <= maxval) b++;
  return b;
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

// CSR -> (key = column, value = row<<32 | value bits), rows ascending.
__global__ void k_csr_to_pairs(const int64_t* __restrict__ row_ptr, int64_t m,
                               const int32_t* __restrict__ col, const float* __restrict__ val,
                               uint32_t* __restrict__ key, uint64_t* __restrict__ pv) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= m) return;
  for (int64_t k = row_ptr[row] + lane; k < row_ptr[row + 1]; k += 32) {
    key[k] = (uint32_t)col[k];
    pv[k] = ((uint64_t)(uint32_t)row << 32) | __float_as_uint(val[k]);
  }
}

__global__ void k_pairs_to_csc(const uint64_t* __restrict__ pv, int64_t nnz,
                               int32_t* __restrict__ row, float* __restrict__ val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nnz) {
    row[i] = (int32_t)(pv[i] >> 32);
    val[i] = __uint_as_float((uint32_t)pv[i]);
  }
}

__global__ void k_colptr_from_sorted(const uint32_t* __restrict__ key, int64_t nnz,
                                     int64_t n, int64_t* __restrict__ col_ptr) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c > n) return;
  int64_t lo = 0, hi = nnz;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if ((int64_t)key[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  col_ptr[c] = lo;
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

size_t epet_csr_to_csc_workspace_size(int64_t m, int64_t n, int64_t nnz) {
  (void)m;
  (void)n;
  const size_t hist = radix_hist_elems(nnz);
  return 2 * align256(nnz * 4) + 2 * align256(nnz * 8) + align256(hist * 8) +
         align256((hist + 1) * 8) + align256(scan_tmp_elems(hist) * 8) + 256;
}

epet_status epet_csr_to_csc(const epet_csr* a, epet_csc* out, void* ws, size_t ws_bytes,
                            epet_stream_t stream) {
  if (!a || !out || !out->col_ptr || (a->nnz > 0 && (!out->row || !out->val)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
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
  uint32_t* key = scr.take<uint32_t>(nnz);
  uint32_t* key2 = scr.take<uint32_t>(nnz);
  uint64_t* pv = scr.take<uint64_t>(nnz);
  uint64_t* pv2 = scr.take<uint64_t>(nnz);
  const size_t hn = radix_hist_elems(nnz);
  int64_t* hist = scr.take<int64_t>(hn);
  int64_t* hist_scan = scr.take<int64_t>(hn + 1);
  int64_t* tmp = scr.take<int64_t>(scan_tmp_elems(hn));
  if (scr.overrun) return set_error(EPET_ERR_INVALID, "internal: workspace size");
  const int T = 256;
  k_csr_to_pairs<<<ceil_div(a->m * 32, T), T, 0, st>>>(a->row_ptr, a->m, a->col, a->val, key,
                                                        pv);
  EPET_LAUNCHED();
  EPET_CHECK((radix_sort<uint32_t, uint64_t>(key, pv, key2, pv2, nnz,
                                             std::max(1, bits_for(a->n - 1)), hist, hist_scan,
                                             tmp, st)));
  k_pairs_to_csc<<<ceil_div(nnz, T), T, 0, st>>>(pv, nnz, out->row, out->val);
  EPET_LAUNCHED();
  k_colptr_from_sorted<<<ceil_div(a->n + 1, T), T, 0, st>>>(key, nnz, a->n, out->col_ptr);
  EPET_LAUNCHED();
  return EPET_OK;
}

}  // extern "C"
