// workqueue.cu -- candidate compaction and per-candidate values.
//
// Candidates of a channel are the voxels whose centre lies closer than the
// sum of half diagonals to the crystal-centre line (getSystemMatrixDeviceOnly
// .cu:25-77; CPU form getWorkqueue.hpp:33-113).  The reference tests all
// m x V pairs; here a warp handles one channel and tests only the voxels of
// each (ix, iy) column whose z range can pass (a float superset from the
// line-cylinder quadratic with a 1% radius margin and one voxel of padding),
// then applies the exact test.  Output order is the reference's: list-major,
// voxel-minor (ascending voxel id).
//
// Values (epet_sm_values) follow the workqueue kernel exactly
// (getSystemMatrixFromWorkqueue.cu:96-261): per element, the chord lengths of
// the channel's rays are added in ray order in fp32 and divided by nrays, so
// the results are bit-identical to the reference's per-channel-seeded
// values.  The rays of a channel are generated once and kept in shared
// memory for all its elements.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace epet {

constexpr int kWqWarps = 4;

// z-index range [zlo, zhi] of the candidates of column (ix, iy); empty when
// zlo > zhi.  Conservative (superset of the exact test).
__device__ __forceinline__ void column_z_range(const Geo& G, const ChannelLine& L,
                                               const float u[3], float R2, int ix,
                                               int iy, int* zlo, int* zhi) {
  const epet_grid& g = G.p.grid;
  const int nz = g.n[2];
  const float wx = voxel_centre(g, 0, ix) - L.a[0];
  const float wy = voxel_centre(g, 1, iy) - L.a[1];
  const float k = u[0] * wx + u[1] * wy;
  const float A = 1.f - u[2] * u[2];
  if (A < 1e-3f) {  // line within ~2 degrees of z: take the whole column
    *zlo = 0;
    *zhi = nz - 1;
    return;
  }
  // dist^2(t) = A t^2 - 2 k uz t + (wx^2 + wy^2 - k^2), t = z - a_z
  const float B = -2.f * k * u[2];
  const float C = wx * wx + wy * wy - k * k - R2;
  const float D = B * B - 4.f * A * C;
  if (D < 0.f) {
    *zlo = 1; *zhi = 0;
    return;
  }
  const float sq = sqrtf(D);
  const float t0 = (-B - sq) / (2.f * A), t1 = (-B + sq) / (2.f * A);
  const float z0 = L.a[2] + t0, z1 = L.a[2] + t1;
  // centres o + (i + 0.5) d inside [z0, z1], padded by one index
  int i0 = (int)ceilf((z0 - g.o[2]) / g.d[2] - 0.5f) - 1;
  int i1 = (int)floorf((z1 - g.o[2]) / g.d[2] - 0.5f) + 1;
  *zlo = max(i0, 0);
  *zhi = min(i1, nz - 1);
}

__device__ __forceinline__ void line_unit(const ChannelLine& L, float u[3]) {
  const float n = sqrtf(L.ab[0] * L.ab[0] + L.ab[1] * L.ab[1] + L.ab[2] * L.ab[2]);
  u[0] = L.ab[0] / n;
  u[1] = L.ab[1] / n;
  u[2] = L.ab[2] / n;
}

// Warp per channel.  kFill = false: row_count[row] = number of candidates.
// kFill = true: writes the pairs from row_off[row] on, in voxel order.
template <bool kFill>
__global__ void __launch_bounds__(32 * kWqWarps)
k_workqueue(Geo G, const int32_t* __restrict__ rows, int64_t m,
            int64_t* __restrict__ row_count, const int64_t* __restrict__ row_off,
            int32_t* __restrict__ out_cnl, int32_t* __restrict__ out_vxl) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * kWqWarps + (threadIdx.x >> 5);
  if (row >= m) return;
  const int cnl = rows[row];
  ChannelLine L;
  CrystalMat m0, m1;
  channel_line(G, cnl, &L, nullptr, &m0, &m1);
  float u[3];
  line_unit(L, u);
  const float Reff = G.sum_radii * 1.01f + 1e-6f;
  const float R2 = Reff * Reff;
  const epet_grid& g = G.p.grid;
  const int ny = g.n[1];
  const int ncol = g.n[0] * ny;
  int64_t base = kFill ? row_off[row] : 0;
  int64_t count = 0;
  for (int q0 = 0; q0 < ncol; q0 += 32) {
    const int q = q0 + lane;
    int zlo = 1, zhi = 0, ix = 0, iy = 0;
    int c = 0;
    if (q < ncol) {
      ix = q / ny;
      iy = q - ix * ny;
      column_z_range(G, L, u, R2, ix, iy, &zlo, &zhi);
      for (int iz = zlo; iz <= zhi; iz++) c += is_candidate(G, L, ix, iy, iz);
    }
    const int inc = warp_incl_scan(c);
    const int tot = __shfl_sync(0xffffffffu, inc, 31);
    if (kFill && c > 0) {
      int64_t o = base + count + (inc - c);
      const int vb = ix * G.nyz + iy * g.n[2];
      for (int iz = zlo; iz <= zhi; iz++)
        if (is_candidate(G, L, ix, iy, iz)) {
          out_cnl[o] = cnl;
          out_vxl[o] = vb + iz;
          o++;
        }
    }
    count += tot;
  }
  if (!kFill && lane == 0) row_count[row] = count;
}

// Slab chord length of a ray in the box of voxel (ix,iy,iz), as
// intersectionLength (getSystemMatrixFromWorkqueue.cu:24-69): axes where the
// ray's two points coincide are left out of the entry/exit max/min.
__device__ __forceinline__ float isect_len(const epet_grid& g, int ix, int iy,
                                           int iz, const float* r) {
  const int id[3] = {ix, iy, iz};
  bool any = false;
  float amin = 0.f, amax = 0.f;
  bool good = false;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (r[d] == r[3 + d]) continue;
    any = true;
    const float den = fsub(r[3 + d], r[d]);
    float lo = fdiv(fsub(voxel_plane(g, d, id[d]), r[d]), den);
    float hi = fdiv(fsub(voxel_plane(g, d, id[d] + 1), r[d]), den);
    if (hi < lo) {
      float t = lo;
      lo = hi;
      hi = t;
    }
    if (!good) {
      amin = lo;
      amax = hi;
      good = true;
    } else {
      amin = fmaxf(amin, lo);
      amax = fminf(amax, hi);
    }
  }
  if (!any) return 0.f;
  if (!(amin < amax)) return 0.f;
  const float dx = fsub(r[3], r[0]), dy = fsub(r[4], r[1]), dz = fsub(r[5], r[2]);
  return fmul(fsub(amax, amin), norm3(dx, dy, dz));
}

constexpr int kValThreads = 128;

// CTA (row, slice): the row's rays in shared memory, the slice's threads
// over every gridDim.y-th group of kValThreads elements (few rows get many
// slices, so a short list of long rows still fills the device).
// Exact = false: the fp32 sum in ray order of getSystemMatrixFromWorkqueue.
// Exact = true: the fused build's exact sum -- each positive chord as
// max(1, round(chord * 2^s)) fixed-point units, the 64-bit total scaled back
// and divided by nrays with the same operations as the ray walk -- so rows
// the walk hands to this path get values of the same definition.
template <bool Exact>
__global__ void __launch_bounds__(kValThreads)
k_values(Geo G, const float* __restrict__ rays, int64_t m,
         const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
         float* __restrict__ val) {
  extern __shared__ float sray[];
  const int64_t row = blockIdx.x;
  if (row >= m) return;
  const int64_t b = row_ptr[row], e = row_ptr[row + 1];
  const int64_t first = b + (int64_t)blockIdx.y * kValThreads;
  if (first >= e) return;  // uniform across the block
  const int R = G.p.nrays;
  const float* src = rays + row * (int64_t)R * 6;
  for (int i = threadIdx.x; i < R * 6; i += kValThreads) sray[i] = src[i];
  __syncthreads();
  const epet_grid& g = G.p.grid;
  for (int64_t k = first + threadIdx.x; k < e; k += (int64_t)gridDim.y * kValThreads) {
    const int v = col[k];
    const int ix = v / G.nyz, rem = v - ix * G.nyz;
    const int iy = rem / g.n[2], iz = rem - iy * g.n[2];
    if (Exact) {
      unsigned long long u = 0ull;
      for (int r = 0; r < R; r++) {
        const float c = isect_len(g, ix, iy, iz, &sray[6 * r]);
        if (c > 0.f) u += __float2ull_rn(fmaxf(fmul(c, G.fx_scale), 1.f));
      }
      const float fR = (float)R;
      val[k] = div_cr(fmul(__ull2float_rn(u), G.fx_inv), fR, __frcp_rn(fR));
    } else {
      float a = 0.f;
      for (int r = 0; r < R; r++) a = fadd(a, isect_len(g, ix, iy, iz, &sray[6 * r]));
      val[k] = fdiv(a, (float)R);
    }
  }
}

// Per-candidate path for the rows the walk leaves out (see sm_build.cu):
// candidates -> values in reference order -> drop zeros.
// kMode as in sm_build.cu: 0 CSR staging, 1 forward, 2 back, 3 column sums,
// 5 one MLEM pass (forward into y, then c64 += A^T (ycnt / y)).
template <int kMode>
__global__ void k_apply_exact(int64_t n_ex, const int32_t* __restrict__ ex_rows,
                              const int64_t* __restrict__ wq_off,
                              const int32_t* __restrict__ wq_vxl,
                              const float* __restrict__ wq_val, int32_t* out_col,
                              float* out_val, int32_t* row_len, int32_t* src_idx,
                              const float* x, float* y, const float* e, float* c,
                              double* s64, const float* ycnt, double* c64) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n_ex) return;
  const int64_t row = ex_rows[i];
  const int64_t b = wq_off[i], n = wq_off[i + 1] - b;
  int64_t o = 0;
  float fsum = 0.f;
  for (int64_t k0 = 0; k0 < n; k0 += 32) {
    const int64_t k = k0 + lane;
    const float v = k < n ? wq_val[b + k] : 0.f;
    const unsigned nzm = __ballot_sync(0xffffffffu, v != 0.f);
    if (v != 0.f) {
      const int vox = wq_vxl[b + k];
      const int64_t pos = o + __popc(nzm & ((1u << lane) - 1u));
      if (kMode == 0) {  // kept entries compacted in place (at most the candidates)
        out_col[b + pos] = vox;
        out_val[b + pos] = v;
      }
      if (kMode == 2 && e[row] != 0.f) atomicAdd(&c[vox], fmul(v, e[row]));
      if (kMode == 3) atomicAdd(&s64[vox], (double)v);
    }
    if (kMode == 1 || kMode == 5) {
      // ordered: lane contributions in element order via the warp
      float t = v != 0.f ? fmul(v, x[wq_vxl[b + k < b + n ? b + k : b]]) : 0.f;
      for (int l = 0; l < 32; l++) fsum = fadd(fsum, __shfl_sync(0xffffffffu, t, l));
    }
    o += __popc(nzm);
  }
  if (lane == 0) {
    if (kMode == 0) {
      row_len[row] = (int32_t)o;
      src_idx[row] = (int32_t)(-2 - i);
    }
    if ((kMode == 1 || kMode == 5) && y) y[row] = fsum;
  }
  if (kMode == 5) {
    // every lane holds the same fsum (the warp-ordered sum)
    const float ev = fsum > 0.f ? __fdiv_rn(ycnt[row], fsum) : 0.f;
    if (ev != 0.f)
      for (int64_t k = lane; k < n; k += 32) {
        const float v = wq_val[b + k];
        if (v != 0.f) atomicAdd(&c64[wq_vxl[b + k]], (double)fmul(v, ev));
      }
  }
}

__global__ void k_gather_i32(const int32_t* src, const int32_t* idx, int64_t n,
                             int32_t* dst) {  // dst[i] = src[idx[i]]
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

__global__ void k_expand_rows(const int64_t* __restrict__ row_ptr, int64_t m,
                              int32_t* __restrict__ out) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= m) return;
  for (int64_t k = row_ptr[row] + lane; k < row_ptr[row + 1]; k += 32) out[k] = (int32_t)row;
}

epet_status launch_workqueue_count(const Geo& G, const int32_t* rows, int64_t m,
                                   int64_t* row_count, cudaStream_t st) {
  if (m == 0) return EPET_OK;
  k_workqueue<false><<<ceil_div(m, kWqWarps), 32 * kWqWarps, 0, st>>>(
      G, rows, m, row_count, nullptr, nullptr, nullptr);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status launch_workqueue_fill(const Geo& G, const int32_t* rows, int64_t m,
                                  const int64_t* row_off, int32_t* cnl, int32_t* vxl,
                                  cudaStream_t st) {
  if (m == 0) return EPET_OK;
  k_workqueue<true><<<ceil_div(m, kWqWarps), 32 * kWqWarps, 0, st>>>(
      G, rows, m, nullptr, row_off, cnl, vxl);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status launch_values(const Geo& G, const float* rays, int64_t m,
                          const int64_t* row_ptr, const int32_t* col, float* val,
                          bool exact, cudaStream_t st) {
  if (m == 0) return EPET_OK;
  const size_t smem = (size_t)G.p.nrays * 6 * sizeof(float);
  if (smem > 200 * 1024)
    return set_error(EPET_ERR_UNSUPPORTED, "nrays too large for the values kernel");
  const unsigned slices = (unsigned)std::min<int64_t>(64, std::max<int64_t>(1, 4096 / m));
  const dim3 grid((unsigned)m, slices);
  if (exact) {
    EPET_CUDA(cudaFuncSetAttribute(k_values<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    k_values<true><<<grid, kValThreads, smem, st>>>(G, rays, m, row_ptr, col, val);
  } else {
    EPET_CUDA(cudaFuncSetAttribute(k_values<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    k_values<false><<<grid, kValThreads, smem, st>>>(G, rays, m, row_ptr, col, val);
  }
  EPET_LAUNCHED();
  return EPET_OK;
}

void ExactRows::release(cudaStream_t st) {
  if (off) dev_free(off, st);
  if (col) dev_free(col, st);
  if (val) dev_free(val, st);
  off = nullptr;
  col = nullptr;
  val = nullptr;
}

// Per-candidate path for a few rows (list ex_rows of indices into rows).
epet_status exact_rows_apply(const Geo& G, const int32_t* rows, const int32_t* ex_rows,
                             int64_t n_ex, int mode, int32_t* row_len, int32_t* src_idx,
                             ExactRows* keep, const float* x, float* y, const float* e,
                             float* c, double* s64, const float* ycnt, double* c64,
                             cudaStream_t st) {
  if (n_ex == 0) return EPET_OK;
  if (mode == 0 && (!keep || keep->off)) return set_error(EPET_ERR_INVALID, "internal: exact rows");
  // off/col/val: handed to the caller in CSR mode, else released here; the
  // temporaries live in owned scratch blocks; all freed on every return path
  struct Local {
    ExactRows bufs;
    cudaStream_t s;
    ~Local() { bufs.release(s); }
  } local{ExactRows{}, st};
  ExactRows& out = mode == 0 ? *keep : local.bufs;
  Scratch t1;
  EPET_CHECK(t1.init(nullptr, 0, align256((size_t)n_ex * 4) + align256((size_t)(n_ex + 1) * 8) +
                                     align256(scan_tmp_elems(n_ex + 1) * 8), st));
  int32_t* cnl = t1.take<int32_t>(n_ex);
  int64_t* cnt = t1.take<int64_t>(n_ex + 1);
  int64_t* tmp = t1.take<int64_t>(scan_tmp_elems(n_ex + 1));
  if (t1.overrun) return set_error(EPET_ERR_INVALID, "internal: exact-row workspace size");
  EPET_CUDA(dev_alloc((void**)&out.off, (n_ex + 1) * 8, st));
  k_gather_i32<<<ceil_div(n_ex, 256), 256, 0, st>>>(rows, ex_rows, n_ex, cnl);
  EPET_LAUNCHED();
  EPET_CHECK(launch_workqueue_count(G, cnl, n_ex, cnt, st));
  EPET_CHECK(exclusive_scan_i64(cnt, out.off, n_ex, tmp, st));
  int64_t total = 0;
  EPET_CUDA(cudaMemcpyAsync(&total, out.off + n_ex, 8, cudaMemcpyDeviceToHost, st));
  EPET_CUDA(cudaStreamSynchronize(st));
  const int64_t tt = std::max<int64_t>(total, 1);
  Scratch t2;
  EPET_CHECK(t2.init(nullptr, 0, 2 * align256((size_t)tt * 4) +
                                     align256((size_t)n_ex * G.p.nrays * 24), st));
  int32_t* wv = t2.take<int32_t>(tt);
  float* wval = t2.take<float>(tt);
  float* rays = t2.take<float>((size_t)n_ex * G.p.nrays * 6);
  if (t2.overrun) return set_error(EPET_ERR_INVALID, "internal: exact-row workspace size");
  // candidate channels; in CSR mode the kept columns then overwrite them
  EPET_CUDA(dev_alloc((void**)&out.col, tt * 4, st));
  if (mode == 0) EPET_CUDA(dev_alloc((void**)&out.val, tt * 4, st));
  EPET_CHECK(launch_workqueue_fill(G, cnl, n_ex, out.off, out.col, wv, st));
  EPET_CHECK(launch_rays(G, cnl, n_ex, rays, false, st));
  EPET_CHECK(launch_values(G, rays, n_ex, out.off, wv, wval, true, st));
  const int T = 128;
  const int nb = ceil_div(n_ex * 32, T);
#define EPET_APPLY(K)                                                                    \
  k_apply_exact<K><<<nb, T, 0, st>>>(n_ex, ex_rows, out.off, wv, wval, out.col, out.val, row_len, \
                                     src_idx, x, y, e, c, s64, ycnt, c64)
  switch (mode) {
    case 0: EPET_APPLY(0); break;
    case 1: EPET_APPLY(1); break;
    case 2: EPET_APPLY(2); break;
    case 5: EPET_APPLY(5); break;
    default: EPET_APPLY(3); break;
  }
#undef EPET_APPLY
  EPET_LAUNCHED();
  return EPET_OK;
}

}  // namespace epet

using namespace epet;

extern "C" {

epet_status epet_workqueue_count(const epet_problem* p, const int32_t* rows_d,
                                 int64_t m, int64_t* row_count_d,
                                 int64_t* total_h, epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (m < 0 || (m > 0 && (!rows_d || !row_count_d)))
    return set_error(EPET_ERR_INVALID, "bad rows/counts");
  cudaStream_t st = (cudaStream_t)stream;
  Geo G = make_geo(*p);
  EPET_CHECK(launch_workqueue_count(G, rows_d, m, row_count_d, st));
  if (total_h) {
    *total_h = 0;
    if (m > 0) {
      int64_t *off = nullptr, *tmp = nullptr;
      EPET_CUDA(dev_alloc((void**)&off, (m + 1) * 8, st));
      EPET_CUDA(dev_alloc((void**)&tmp, scan_tmp_elems(m + 1) * 8, st));
      epet_status rc = exclusive_scan_i64(row_count_d, off, m, tmp, st);
      if (rc == EPET_OK) {
        EPET_CUDA(cudaMemcpyAsync(total_h, off + m, 8, cudaMemcpyDeviceToHost, st));
      }
      dev_free(off, st);
      dev_free(tmp, st);
      EPET_CUDA(cudaStreamSynchronize(st));
      if (rc != EPET_OK) return rc;
    }
  }
  return EPET_OK;
}

epet_status epet_workqueue_fill(const epet_problem* p, const int32_t* rows_d,
                                int64_t m, const int64_t* row_off_d,
                                int32_t* wq_cnl_d, int32_t* wq_vxl_d,
                                epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (m < 0 || (m > 0 && (!rows_d || !row_off_d || !wq_cnl_d || !wq_vxl_d)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  return launch_workqueue_fill(make_geo(*p), rows_d, m, row_off_d, wq_cnl_d, wq_vxl_d,
                               (cudaStream_t)stream);
}

size_t epet_sm_values_workspace_size(const epet_problem* p, int64_t m) {
  if (epet_problem_validate(p) != EPET_OK) return 0;
  const int64_t ch = std::min<int64_t>(std::max<int64_t>(m, 1), 65536);
  return align256((size_t)ch * p->nrays * 24);
}

epet_status epet_sm_values(const epet_problem* p, const int32_t* rows_d,
                           int64_t m, const int64_t* row_ptr_d,
                           const int32_t* col_d, float* val_d, void* ws,
                           size_t ws_bytes, epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (m < 0 || (m > 0 && (!rows_d || !row_ptr_d)))
    return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  Geo G = make_geo(*p);
  Scratch scr;
  EPET_CHECK(scr.init(ws, ws_bytes, epet_sm_values_workspace_size(p, m), st));
  const int64_t ch = std::min<int64_t>(std::max<int64_t>(m, 1), 65536);
  float* rays = scr.take<float>((size_t)ch * p->nrays * 6);
  if (scr.overrun) return set_error(EPET_ERR_INVALID, "internal: workspace size");
  for (int64_t c0 = 0; c0 < m; c0 += ch) {
    const int64_t mc = std::min(ch, m - c0);
    EPET_CHECK(launch_rays(G, rows_d + c0, mc, rays, false, st));
    EPET_CHECK(launch_values(G, rays, mc, row_ptr_d + c0, col_d, val_d, false, st));
  }
  return EPET_OK;
}

}  // extern "C"
