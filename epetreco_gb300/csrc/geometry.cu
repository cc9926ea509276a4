// geometry.cu -- per-angle trig table, cuRAND uniforms and world rays.
//
// Rays follow RandRayGen with the per-channel seeding of the workqueue
// kernel: curand_init(seed, channel, 0) and six curand_uniform draws per ray,
// the first three placing the start point in crystal 0 and the last three
// the end point in crystal 1 (getSystemMatrixFromWorkqueue.cu:189-230).
// With EPET_RAYS_REGULAR they follow ReguRayGen (RayGenerators.hpp:46-66):
// the six box coordinates are 0.5, so every ray joins the crystal centres,
// and no generator is seeded.
#include <curand_kernel.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace epet {

__global__ void k_trig(epet_setup s, float* sc) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < s.na) angle_sincos(s, a, &sc[2 * a], &sc[2 * a + 1]);
}

// Six box coordinates of one ray: cuRAND uniforms, or 0.5 each for regular rays.
__device__ __forceinline__ void draw6(curandState& st, bool regular, float* u) {
#pragma unroll
  for (int k = 0; k < 6; k++) u[k] = regular ? 0.5f : curand_uniform(&st);
}

// One thread per channel: the cuRAND stream of a channel is sequential, so a
// channel's 6*nrays draws stay on one thread; channels spread over threads.
// The uniforms-only form (a test and debugging interface) seeds every
// channel with curand_init(seed, channel, 0) directly.
__device__ __forceinline__ void emit_rays(const Geo& G, int cnl, curandState st, bool uniforms,
                                          float2* o) {
  const bool regular = G.p.ray_mode == EPET_RAYS_REGULAR;
  int id[5];
  channel_decode(G.p.setup, cnl, id);
  float sn, cs;
  angle_sincos(G.p.setup, id[0], &sn, &cs);
  const CrystalMat m0 = crystal_matrix(G.p.setup, sn, cs, 0, id[1], id[2]);
  const CrystalMat m1 = crystal_matrix(G.p.setup, sn, cs, 1, id[3], id[4]);
  // rays in pairs: 48 bytes as three 16-byte stores when the row's block is
  // 16-byte aligned (half as many scattered stores as 8-byte ones)
  const bool wide = (reinterpret_cast<uintptr_t>(o) & 15) == 0;
  for (int r = 0; r < G.p.nrays; r++) {
    float u[6];
    draw6(st, regular, u);
    float w[6];
    if (uniforms) {
#pragma unroll
      for (int k = 0; k < 6; k++) w[k] = u[k];
    } else {
      crystal_apply(m0, u[0], u[1], u[2], w);
      crystal_apply(m1, u[3], u[4], u[5], w + 3);
    }
    if (wide && r + 1 < G.p.nrays) {
      float u2[6], w2[6];
      draw6(st, regular, u2);
      if (uniforms) {
#pragma unroll
        for (int k = 0; k < 6; k++) w2[k] = u2[k];
      } else {
        crystal_apply(m0, u2[0], u2[1], u2[2], w2);
        crystal_apply(m1, u2[3], u2[4], u2[5], w2 + 3);
      }
      float4* q = reinterpret_cast<float4*>(o + 3 * r);
      q[0] = make_float4(w[0], w[1], w[2], w[3]);
      q[1] = make_float4(w[4], w[5], w2[0], w2[1]);
      q[2] = make_float4(w2[2], w2[3], w2[4], w2[5]);
      r++;
    } else {
      o[3 * r + 0] = make_float2(w[0], w[1]);
      o[3 * r + 1] = make_float2(w[2], w[3]);
      o[3 * r + 2] = make_float2(w[4], w[5]);
    }
  }
}

__global__ void __launch_bounds__(128) k_uniforms(Geo G, const int32_t* __restrict__ rows,
                                                  int64_t m, float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  curandState st = {};
  if (G.p.ray_mode != EPET_RAYS_REGULAR)
    curand_init(G.p.seed, (unsigned long long)rows[i], 0ull, &st);
  emit_rays(G, rows[i], st, true,
            reinterpret_cast<float2*>(out + i * (int64_t)G.p.nrays * 6));
}

// World rays.  Thread t handles rows t*K .. t*K+K-1: the first channel's
// generator comes from curand_init, the next ones from the previous
// channel's initial state advanced by the channel difference in
// subsequences (skipahead_sequence): curand_init(seed, c, 0) is the seeded
// state advanced c subsequences, so this yields the same states while a
// typical step (consecutive channel ids) applies one jump matrix instead of
// one per set bit of the channel id.
constexpr int kRaysPerThread = 4;
__global__ void __launch_bounds__(128) k_rays(Geo G, const int32_t* __restrict__ rows,
                                              int64_t m, float* __restrict__ out) {
  const int64_t i0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kRaysPerThread;
  if (i0 >= m) return;
  const int64_t i1 = i0 + kRaysPerThread < m ? i0 + kRaysPerThread : m;
  const bool regular = G.p.ray_mode == EPET_RAYS_REGULAR;
  curandState base = {};
  int prev = rows[i0];
  if (!regular) curand_init(G.p.seed, (unsigned long long)prev, 0ull, &base);
  for (int64_t i = i0; i < i1; i++) {
    const int cnl = rows[i];
    if (i > i0 && !regular) {
      if (cnl > prev) skipahead_sequence((unsigned long long)(cnl - prev), &base);
      else if (cnl != prev) curand_init(G.p.seed, (unsigned long long)cnl, 0ull, &base);
      prev = cnl;
    }
    emit_rays(G, cnl, base, false,
              reinterpret_cast<float2*>(out + i * (int64_t)G.p.nrays * 6));
  }
}

Geo make_geo(const epet_problem& p) {
  Geo G;
  G.p = p;
  // 0.5*(absolute(vxlEdges)+absolute(pxlEdges)) with absolute = sqrtf of the
  // left-to-right sum of squares (getSystemMatrixDeviceOnly.cu:55-58); this
  // file is compiled with host contraction disabled.
  volatile float a0 = p.grid.d[0] * p.grid.d[0];
  volatile float a1 = p.grid.d[1] * p.grid.d[1];
  volatile float a2 = p.grid.d[2] * p.grid.d[2];
  volatile float av = sqrtf((a0 + a1) + a2);
  volatile float b0 = p.setup.segx * p.setup.segx;
  volatile float b1 = p.setup.segy * p.setup.segy;
  volatile float b2 = p.setup.segz * p.setup.segz;
  volatile float bv = sqrtf((b0 + b1) + b2);
  volatile float sr = av + bv;
  G.sum_radii = 0.5f * sr;
  G.V = p.grid.n[0] * p.grid.n[1] * p.grid.n[2];
  G.nyz = p.grid.n[1] * p.grid.n[2];
  // Fixed-point chord sums: a cell gets at most nrays chords (one per ray),
  // each split as hi * 2^b + lo with lo < 2^b; b and the scale 2^s are chosen
  // so that nrays * 2^b <= 2^32 and nrays * max(hi) < 2^32, i.e. both halves
  // sum in 32 bits without carries, exactly and in any order.  A chord is at
  // most the voxel diagonal (av, +1% for rounding).
  int lg = 0;
  while ((1ll << lg) < (long long)p.nrays + 1) lg++;  // ceil(log2(nrays + 1))
  const int b = 32 - lg;                               // lo bits
  const int units_bits = 64 - 2 * lg;                  // chord units < 2^units_bits
  int s = (int)floor(log2(ldexp(1.0, units_bits) / ((double)av * 1.01 + 1e-30)));
  if (s > 100) s = 100;
  G.fx_scale = ldexpf(1.0f, s);
  G.fx_inv = ldexpf(1.0f, -s);
  G.fx_split = b;
  return G;
}

epet_status launch_rays(const Geo& G, const int32_t* rows, int64_t m, float* out,
                        bool uniforms_only, cudaStream_t st) {
  if (m == 0) return EPET_OK;
  const int T = 128;
  if (uniforms_only)
    k_uniforms<<<ceil_div(m, T), T, 0, st>>>(G, rows, m, out);
  else
    k_rays<<<ceil_div(ceil_div(m, kRaysPerThread), T), T, 0, st>>>(G, rows, m, out);
  EPET_LAUNCHED();
  return EPET_OK;
}

// Self-test of div_cr against the correctly rounded division: n seeded
// operand pairs, a with exponents in [2^-40, 2^5), b in [2^-20, 2^5), random
// signs and mantissas; counts bitwise differences.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void k_selftest_div(int64_t n, uint64_t seed, unsigned long long* bad) {
  unsigned long long mine = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r = splitmix64(seed ^ (uint64_t)i * 0x2545f4914f6cdd1dull);
    const uint32_t ea = 127 - 40 + (uint32_t)((r >> 23) % 45u);
    const uint32_t eb = 127 - 20 + (uint32_t)((r >> 46) % 25u);
    const float a = (r & 0xfffff) == 0 ? 0.f
                    : __uint_as_float(((uint32_t)(r >> 63) << 31) | (ea << 23) |
                                      ((uint32_t)r & 0x7fffffu));
    const float b = __uint_as_float(((uint32_t)(r >> 62 & 1u) << 31) | (eb << 23) |
                                    ((uint32_t)(r >> 32) & 0x7fffffu));
    if (__float_as_uint(div_cr(a, b, __frcp_rn(b))) != __float_as_uint(__fdiv_rn(a, b))) mine++;
  }
  if (mine) atomicAdd(bad, mine);
}

}  // namespace epet

using namespace epet;

// Work measure of the walk: the cells a ray crosses inside the grid, i.e. 1
// + the grid planes it passes between its entry and exit (per axis, the
// distance between the entry and exit cell indices).  Entry and exit cells
// are taken a little inside the ray's grid interval, so a ray that only
// grazes a plane counts the cells on one side of it.
__global__ void k_ray_steps(Geo G, const float* __restrict__ rays, int64_t n,
                            unsigned long long* __restrict__ total,
                            unsigned long long* __restrict__ per_row) {
  const epet_grid& g = G.p.grid;
  unsigned long long mine = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float* r = rays + 6 * i;
    float a_in = 0.f, a_out = 1.f;
    bool hit = true;
    for (int a = 0; a < 3; a++) {
      const float p0 = r[a], dp = r[a + 3] - r[a];
      const float lo = g.o[a], hi = g.o[a] + g.n[a] * g.d[a];
      if (dp == 0.f) {
        hit = hit && p0 > lo && p0 < hi;
      } else {
        const float t0 = (lo - p0) / dp, t1 = (hi - p0) / dp;
        a_in = fmaxf(a_in, fminf(t0, t1));
        a_out = fminf(a_out, fmaxf(t0, t1));
      }
    }
    if (!hit || !(a_in < a_out)) continue;
    const float span = a_out - a_in, t_in = a_in + 1e-6f * span, t_out = a_out - 1e-6f * span;
    unsigned long long st = 1;
    for (int a = 0; a < 3; a++) {
      const float dp = r[a + 3] - r[a];
      const int c0 = min(max((int)floorf((r[a] + t_in * dp - g.o[a]) / g.d[a]), 0), g.n[a] - 1);
      const int c1 = min(max((int)floorf((r[a] + t_out * dp - g.o[a]) / g.d[a]), 0), g.n[a] - 1);
      st += (unsigned long long)abs(c1 - c0);
    }
    mine += st;
    if (per_row) atomicAdd(per_row + i / G.p.nrays, st);
  }
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(total, mine);
}

extern "C" {

epet_status epet_build_counters(int64_t* overflow_rows_h, int64_t* exact_rows_h) {
  if (overflow_rows_h) *overflow_rows_h = overflow_rows_total();
  if (exact_rows_h) *exact_rows_h = exact_rows_total();
  return EPET_OK;
}

epet_status epet_selftest_division(int64_t n, uint64_t seed, int64_t* mismatches_h,
                                   epet_stream_t stream) {
  if (n < 0 || !mismatches_h) return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* bad = nullptr;
  EPET_CUDA(dev_alloc((void**)&bad, 8, st));
  EPET_CUDA(cudaMemsetAsync(bad, 0, 8, st));
  k_selftest_div<<<1024, 256, 0, st>>>(n, seed, bad);
  EPET_LAUNCHED();
  unsigned long long h = 0;
  EPET_CUDA(cudaMemcpyAsync(&h, bad, 8, cudaMemcpyDeviceToHost, st));
  EPET_CUDA(dev_free(bad, st));
  EPET_CUDA(cudaStreamSynchronize(st));
  *mismatches_h = (int64_t)h;
  return EPET_OK;
}

epet_status epet_ray_steps(const epet_problem* p, const int32_t* rows_d, int64_t m,
                           int64_t* row_steps_d, int64_t* steps_h, epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (m < 0 || (m > 0 && !rows_d) || !steps_h) return set_error(EPET_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  const Geo G = make_geo(*p);
  // rays of chunks of rows (about 256 MB per chunk)
  const int64_t ch = std::max<int64_t>(1, std::min<int64_t>(m, (int64_t(256) << 20) /
                                                                   ((int64_t)p->nrays * 24)));
  Scratch scr;
  EPET_CHECK(scr.init(nullptr, 0, align256((size_t)ch * p->nrays * 24) + 256, st));
  float* rays = scr.take<float>((size_t)ch * p->nrays * 6);
  unsigned long long* tot = scr.take<unsigned long long>(1);
  if (scr.overrun) return set_error(EPET_ERR_INVALID, "internal: workspace size");
  EPET_CUDA(cudaMemsetAsync(tot, 0, 8, st));
  if (row_steps_d && m > 0) EPET_CUDA(cudaMemsetAsync(row_steps_d, 0, m * 8, st));
  for (int64_t c0 = 0; c0 < m; c0 += ch) {
    const int64_t mc = std::min(ch, m - c0);
    EPET_CHECK(launch_rays(G, rows_d + c0, mc, rays, false, st));
    const int64_t nr = mc * p->nrays;
    k_ray_steps<<<std::min<int64_t>(ceil_div(nr, 256), 8 * (int64_t)num_sms()), 256, 0, st>>>(
        G, rays, nr, tot,
        row_steps_d ? reinterpret_cast<unsigned long long*>(row_steps_d + c0) : nullptr);
    EPET_LAUNCHED();
  }
  unsigned long long h = 0;
  EPET_CUDA(cudaMemcpyAsync(&h, tot, 8, cudaMemcpyDeviceToHost, st));
  EPET_CUDA(cudaStreamSynchronize(st));
  *steps_h = (int64_t)h;
  return EPET_OK;
}

epet_status epet_trig_table(const epet_problem* p, float* sc_d,
                            epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (!sc_d) return set_error(EPET_ERR_INVALID, "sc_d is NULL");
  k_trig<<<ceil_div(p->setup.na, 128), 128, 0, (cudaStream_t)stream>>>(p->setup, sc_d);
  EPET_LAUNCHED();
  return EPET_OK;
}

epet_status epet_dump_uniforms(const epet_problem* p, const int32_t* rows_d,
                               int64_t m, float* out_d, epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (m < 0 || (m > 0 && (!rows_d || !out_d)))
    return set_error(EPET_ERR_INVALID, "bad rows/out");
  return launch_rays(make_geo(*p), rows_d, m, out_d, true, (cudaStream_t)stream);
}

epet_status epet_rays(const epet_problem* p, const int32_t* rows_d, int64_t m,
                      float* out_d, epet_stream_t stream) {
  EPET_CHECK(epet_problem_validate(p));
  if (m < 0 || (m > 0 && (!rows_d || !out_d)))
    return set_error(EPET_ERR_INVALID, "bad rows/out");
  return launch_rays(make_geo(*p), rows_d, m, out_d, false, (cudaStream_t)stream);
}

}  // extern "C"
