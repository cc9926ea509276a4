// common.cuh -- shared device code of the epet_gb300 library.
//
// Geometry functions reproduce the reference's float operation sequence with
// explicit round-to-nearest intrinsics (__fmul_rn, __fadd_rn, ...), which the
// compiler may not contract into FMAs.  The reference's host build rounds
// every operation once (no contraction), and these functions give the same
// bits, so candidate sets and chord lengths are reproducible across builds.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/epet_gb300.h"

namespace epet {

// ------------------------------------------------------------ error state
epet_status set_error(epet_status st, const char* fmt, ...);
epet_status cuda_status(cudaError_t e, const char* what);
#define EPET_CUDA(call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return epet::cuda_status(e_, #call); \
  } while (0)
// After a kernel launch: count it and surface launch errors.
#define EPET_LAUNCHED()                                   \
  do {                                                    \
    epet::note_launch();                                  \
    EPET_CUDA(cudaGetLastError());                        \
  } while (0)
#define EPET_CHECK(call)              \
  do {                                \
    epet_status s_ = (call);          \
    if (s_ != EPET_OK) return s_;     \
  } while (0)

// Scratch memory: the caller's workspace when given, else stream-ordered
// allocations released by the destructor (after the work queued on stream).
struct Scratch {
  char* base = nullptr;
  size_t size = 0, used = 0;
  bool owned = false;
  cudaStream_t stream = 0;
  epet_status init(void* ws, size_t ws_bytes, size_t need, cudaStream_t s);
  // Carves the next 256-byte-aligned piece; nullptr (and `overrun` set) if
  // the workspace size computed for the call was too small.
  template <typename T>
  T* take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    if (used + bytes > size) {
      overrun = true;
      return nullptr;
    }
    char* p = base + used;
    used += bytes;
    return reinterpret_cast<T*>(p);
  }
  bool overrun = false;
  ~Scratch();
};
__host__ __device__ inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
int num_sms();
// Library device memory (a stream-ordered pool per device, see runtime.cu).
cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t st);
cudaError_t dev_free(void* p, cudaStream_t st);
epet_status trim_memory(size_t keep_bytes);
// Counts the library's kernel launches (graph replays count their kernels).
void note_launch(int n = 1);

// ------------------------------------------------------------ geometry

// Per-problem constants shared by the kernels (passed by value).
struct Geo {
  epet_problem p;
  float sum_radii;   // 0.5*(|voxel diagonal| + |crystal diagonal|)
  int32_t V;         // voxels
  int32_t nyz;       // n[1]*n[2]
  float fx_scale;    // 2^s: chord length -> fixed point units
  float fx_inv;      // 2^-s
  int fx_split;      // units = hi * 2^fx_split + lo, both parts summed in 32 bits
};

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// Correctly rounded quotient a / b from inv = RN(1/b), by Markstein's
// theorem (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990): q0 = RN(a*inv)
// lies within one ulp of a/b, the residual r = a - b*q0 is exact in one fma,
// and RN(q0 + r*inv) = RN(a/b) for operands away from overflow and
// underflow (the ray parameters here are of order 1).  One reciprocal per
// ray and axis replaces a division per plane crossing.
__device__ __forceinline__ float div_cr(float a, float b, float inv) {
  const float q0 = __fmul_rn(a, inv);
  const float r = __fmaf_rn(-q0, b, a);
  return __fmaf_rn(r, inv, q0);
}

// sqrtf(a0*a0 + a1*a1 + a2*a2) (distancePointLine.h:19-24).
__device__ __forceinline__ float norm3(float a0, float a1, float a2) {
  return fsqrt(fadd(fadd(fmul(a0, a0), fmul(a1, a1)), fmul(a2, a2)));
}

// Angle of index ida: T(M_PI)*ida*(meas->da())/T(180.0) evaluated left to
// right in float (MeasurementSetupTrafo2CartCoord.hpp:67-68).
__device__ __forceinline__ void angle_sincos(const epet_setup& s, int ida,
                                             float* sn, float* cs) {
  float a = fmul(3.14159265358979323846f, (float)ida);
  a = fmul(a, s.da);
  a = fdiv(a, 180.0f);
  *sn = sinf(a);
  *cs = cosf(a);
}

// The non-zero entries of the 3x4 crystal transform
// (MeasurementSetupTrafo2CartCoord.hpp:70-90); rows apply as
//   x = (t00*b0 + t02*b2) + t03,  y = t11*b1 + t13,  z = (t20*b0 + t22*b2) + t23
// which equals the reference's four-term sums because the dropped terms are
// exact zeros added to non-zero values.
struct CrystalMat {
  float t00, t02, t03, t11, t13, t20, t22, t23;
};

__device__ __forceinline__ CrystalMat crystal_matrix(const epet_setup& s,
                                                     float sn, float cs,
                                                     int det, int iz, int iy) {
  const float e0 = s.segx, e1 = s.segy, e2 = s.segz;
  const int ny = det == 0 ? s.n0y : s.n1y;
  const int nz = det == 0 ? s.n0z : s.n1z;
  const float pos0 = det == 0 ? s.pos0x : s.pos1x;
  // pos[1] = (id - T(.5)*(n-1))*edge (MeasurementSetupTrafo2CartCoord.hpp:64-65)
  const float pos1 = fmul(fsub((float)iy, fmul(0.5f, (float)(ny - 1))), e1);
  const float pos2 = fmul(fsub((float)iz, fmul(0.5f, (float)(nz - 1))), e2);
  const float X = fsub(pos0, fmul(0.5f, e0));
  const float Z = fsub(pos2, fmul(0.5f, e2));
  CrystalMat m;
  m.t00 = fmul(cs, e0);
  m.t02 = fmul(sn, e2);
  m.t03 = fadd(fmul(cs, X), fmul(sn, Z));
  m.t11 = e1;
  m.t13 = fsub(pos1, fmul(0.5f, e1));
  m.t20 = fmul(-sn, e0);
  m.t22 = fmul(cs, e2);
  m.t23 = fadd(fmul(-sn, X), fmul(cs, Z));
  return m;
}

__device__ __forceinline__ void crystal_apply(const CrystalMat& m, float b0,
                                              float b1, float b2, float* o) {
  o[0] = fadd(fadd(fmul(m.t00, b0), fmul(m.t02, b2)), m.t03);
  o[1] = fadd(fmul(m.t11, b1), m.t13);
  o[2] = fadd(fadd(fmul(m.t20, b0), fmul(m.t22, b2)), m.t23);
}

// Channel id -> (ida, id0z, id0y, id1z, id1y) (MeasurementSetupLinIndex.hpp).
__device__ __forceinline__ void channel_decode(const epet_setup& s, int cnl,
                                               int* id) {
  int t = cnl;
  id[4] = t % s.n1y;
  t /= s.n1y;
  id[3] = t % s.n1z;
  t /= s.n1z;
  id[2] = t % s.n0y;
  t /= s.n0y;
  id[1] = t % s.n0z;
  id[0] = t / s.n0z;
}

// Voxel centre o + (i + T(0.5))*d (getSystemMatrixDeviceOnly.cu:67-69).
__device__ __forceinline__ float voxel_centre(const epet_grid& g, int d, int i) {
  return fadd(g.o[d], fmul(fadd((float)i, 0.5f), g.d[d]));
}
// Voxel plane o + k*d (getSystemMatrixFromWorkqueue.cu:155-160; plane k is
// the low face of voxel k and the high face of voxel k-1, same float).
__device__ __forceinline__ float voxel_plane(const epet_grid& g, int d, int k) {
  return fadd(g.o[d], fmul((float)k, g.d[d]));
}

// Candidate line of one channel: crystal centres a, b; ab = b - a; |ab|; and
// the exact threshold on |ab x ap|^2 (see candidate_threshold).
struct ChannelLine {
  float a[3], ab[3];
  float s_max;  // candidate iff cross2 < s_max
};

// The reference test is rn(rn(sqrt(S)) / |ab|) < sum_radii where S is the
// float |ab x ap|^2.  That expression is non-decreasing in S, so the set of
// passing S is a prefix of the non-negative floats: find its end by
// bisection on the float bit patterns.  Afterwards each voxel costs one
// comparison, with the same outcome as the full expression.
__device__ __forceinline__ float candidate_threshold(float nab, float sr) {
  uint32_t lo = 0u, hi = 0x7f800000u;  // [0, +inf]
  // invariant: pass(lo) (when lo == 0 check separately), !pass(hi)
  auto pass = [&](uint32_t bits) {
    return fdiv(fsqrt(__uint_as_float(bits)), nab) < sr;
  };
  if (!pass(0u)) return 0.0f;  // nothing passes
  while (hi - lo > 1u) {
    uint32_t mid = lo + (hi - lo) / 2u;
    if (pass(mid)) lo = mid;
    else hi = mid;
  }
  return __uint_as_float(hi);  // first failing value
}

// The same threshold found by one warp: each round the 32 lanes test 32
// points of [lo, hi] and keep the sub-interval where the outcome changes.
// Must be called by all 32 lanes of a warp.
__device__ __forceinline__ float candidate_threshold_warp(float nab, float sr) {
  const int lane = threadIdx.x & 31;
  auto pass = [&](uint32_t bits) {
    return fdiv(fsqrt(__uint_as_float(bits)), nab) < sr;
  };
  if (!pass(0u)) return 0.0f;
  uint32_t lo = 0u, hi = 0x7f800000u;  // pass(lo), !pass(hi)
  while (hi - lo > 1u) {
    const uint32_t span = hi - lo;
    // lane l tests lo + ceil(span*(l+1)/33); strictly inside (lo, hi]
    uint32_t pt = lo + (uint32_t)(((uint64_t)span * (uint32_t)(lane + 1) + 32u) / 33u);
    if (pt <= lo) pt = lo + 1u;
    if (pt > hi) pt = hi;
    const unsigned okm = __ballot_sync(0xffffffffu, pt < hi && pass(pt));
    // points are increasing in the lane index and pass() is monotone:
    // the passing lanes form a prefix
    const int npass = __popc(okm);
    const uint32_t new_lo = npass ? __shfl_sync(0xffffffffu, pt, npass - 1) : lo;
    uint32_t new_hi = npass < 32 ? __shfl_sync(0xffffffffu, pt, npass < 32 ? npass : 31) : hi;
    if (new_hi > hi) new_hi = hi;
    lo = new_lo;
    hi = new_hi;
  }
  return __uint_as_float(hi);
}

__device__ __forceinline__ void channel_line(const Geo& G, int cnl,
                                             ChannelLine* L, int* ida_out,
                                             CrystalMat* m0, CrystalMat* m1) {
  int id[5];
  channel_decode(G.p.setup, cnl, id);
  float sn, cs;
  angle_sincos(G.p.setup, id[0], &sn, &cs);
  *m0 = crystal_matrix(G.p.setup, sn, cs, 0, id[1], id[2]);
  *m1 = crystal_matrix(G.p.setup, sn, cs, 1, id[3], id[4]);
  float b[3];
  crystal_apply(*m0, 0.5f, 0.5f, 0.5f, L->a);
  crystal_apply(*m1, 0.5f, 0.5f, 0.5f, b);
  for (int d = 0; d < 3; d++) L->ab[d] = fsub(b[d], L->a[d]);
  float nab = norm3(L->ab[0], L->ab[1], L->ab[2]);
  L->s_max = candidate_threshold(nab, G.sum_radii);
  if (ida_out) *ida_out = id[0];
}

// |ab x ap|^2 for a point p (distancePointLine.h:46-72, before the sqrt).
__device__ __forceinline__ float cross2(const ChannelLine& L, float p0, float p1,
                                        float p2) {
  const float ap0 = fsub(p0, L.a[0]), ap1 = fsub(p1, L.a[1]),
              ap2 = fsub(p2, L.a[2]);
  const float c0 = fsub(fmul(L.ab[1], ap2), fmul(L.ab[2], ap1));
  const float c1 = fsub(fmul(L.ab[2], ap0), fmul(L.ab[0], ap2));
  const float c2 = fsub(fmul(L.ab[0], ap1), fmul(L.ab[1], ap0));
  return fadd(fadd(fmul(c0, c0), fmul(c1, c1)), fmul(c2, c2));
}

__device__ __forceinline__ bool is_candidate(const Geo& G, const ChannelLine& L,
                                             int ix, int iy, int iz) {
  const float s = cross2(L, voxel_centre(G.p.grid, 0, ix),
                         voxel_centre(G.p.grid, 1, iy),
                         voxel_centre(G.p.grid, 2, iz));
  return s < L.s_max;
}

// Warp helpers.
__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

}  // namespace epet
