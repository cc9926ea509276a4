// sm_build.cu -- fused on-the-fly system matrix: ray walks -> exact per-voxel
// sums -> candidate filter -> CSR rows in voxel order.
//
// Semantics (what the reference computes, getSystemMatrixFromWorkqueue.cu:
// 96-261 over the candidates of getSystemMatrixDeviceOnly.cu:25-77):
//   A[c,v] = (1/nrays) * sum_r len_r(v)  for candidate voxels v of channel c,
// len_r(v) the slab chord length of ray r in voxel v (:24-69).  Entries with
// A[c,v] == 0 are not stored (the reference stores them).
//
// GB300 design:
//  * one CTA per channel; its rays come from a thread-per-channel cuRAND
//    kernel (geometry.cu), so the sequential XORWOW stream of a channel is
//    drawn once instead of once per candidate voxel;
//  * each thread walks a ray voxel by voxel (Siddon order).  The entry/exit
//    parameters are the reference's own correctly rounded quotients
//    (plane - r0)/(r1 - r0), shared between neighbouring voxels, so each
//    chord length is bit-identical to intersectionLength(); a voxel is never
//    evaluated more than once per ray;
//  * chords accumulate in a dense shared-memory window covering the ray
//    bundle slab by slab along x (bounded by the 64 crystal-corner lines, an
//    exact convex-hull bound), as 64-bit fixed-point integers: the sum is
//    exact and independent of the order of the atomic adds, so results are
//    deterministic; it is rounded once to float.  Versus the reference's
//    sequential fp32 sum the difference is below (nrays-1)*2^-24 relative;
//  * window cells are ordered by voxel id (x slabs ascending, then y, z), so
//    extraction is an ordered compaction: no sort;
//  * candidates are tested with an exact threshold on |ab x ap|^2 that
//    reproduces the reference's float test bit for bit (common.cuh).
#include <curand_kernel.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "mlem_internal.h"

namespace epet {

constexpr int kWalkThreads = 128;
constexpr int kGeomFloats = 56;  // per-channel geometry record (k_channel_geom)
constexpr int kMaxSlabs = 1024;  // nx limit of the walk kernel
constexpr float kWinPad = 1e-3f;  // window padding margin, in voxels (slab_window)

enum WalkMode { kModeCsr = 0, kModeForward = 1, kModeBack = 2, kModeColSum = 3,
                kModeWindow = 4, kModeMlem = 5 };

struct WalkArgs {
  Geo G;
  const int32_t* rows;  // this launch's rows
  int64_t m;
  const float* rays;    // [m][nrays][6]
  const float* geom;    // [m][kGeomFloats] channel geometry (k_channel_geom)
  int cap_cells;        // window capacity (cells) of this launch
  // CSR staging (row i writes stage_col/val[i*stride ...], row_len[i])
  int64_t stride;
  int32_t* stage_col;
  float* stage_val;
  int32_t* row_len;
  // projections
  const float* x;  // forward input (voxels)
  float* y;        // forward output (rows)
  const float* e;  // back-projection input (rows)
  float* c;        // back-projection output (voxels)
  double* s64;     // column sums
  // one MLEM pass (kModeMlem): ybar = A x into y, c64 += A^T (ycnt / ybar)
  const float* ycnt;  // measured counts (rows)
  double* c64;        // correction image (voxels), fp64
  // window sizes (kModeWindow) and overflow reporting
  int32_t* win_cells;      // per row window cells
  int32_t* overflow_rows;  // list of rows whose window exceeded cap_cells
  int32_t* overflow_count;
  int32_t* hit_outside;    // rows with hits outside the window (must stay 0)
  int32_t* exact_rows;     // rows left to the per-candidate path
  int32_t* exact_count;
  // redo launch over rows whose window exceeded the first launch's capacity:
  // block b handles chunk row sel[b] and stages at b*stride; ovf_idx[row] = b
  const int32_t* sel;
  int32_t* ovf_idx;
};

// Dynamic shared memory of the walk kernel: the grid-plane table, the per-row
// z terms of the candidate test and the pool, each on a 256-byte boundary.
// The pool holds, per channel, the window's column table (8 bytes per
// column, border included) followed by the two 32-bit sum words of every
// window cell and of the two trash cells (8 bytes per cell): a channel needs
// columns + cells + 2 <= cap_cells.
struct WalkLayout {
  size_t planes, ztab, pool, pext, lines, slabs, total;
};
constexpr int kHullLines = 64;  // crystal-corner pair lines of the hull
// nplanes: grid planes of all three axes (n0 + n1 + n2 + 3); nz: z cells.
// The pool holds the column table and the cells.  Three arrays that die
// early share it: the hull extents at the slab planes (pext, at its start)
// and the hull lines' parameters after them are read only while the slab
// windows are built, and the slab windows (slabs, at its end) only until the
// column table is built, so the table must end before them and the cells,
// written afterwards, may run over them.
__host__ __device__ inline WalkLayout walk_layout(int nslab, int nplanes, int nz, int cap_cells) {
  WalkLayout L;
  L.planes = 0;
  L.ztab = L.planes + align256((size_t)(nplanes + 2) * 4);  // + a guard entry at each end
  L.pool = L.ztab + align256((size_t)nz * 8);
  const size_t pext_b = ((size_t)(nslab + 1) * 16 + 15) & ~size_t(15);
  const size_t slab_b = ((size_t)20 * nslab + 15) & ~size_t(15);
  const size_t line_b = (size_t)6 * kHullLines * 4;
  size_t pool_b = (size_t)cap_cells * 8;
  if (pool_b < pext_b + line_b + slab_b) pool_b = pext_b + line_b + slab_b;
  pool_b = (pool_b + 15) & ~size_t(15);
  L.pext = L.pool;
  L.lines = L.pool + pext_b;
  L.slabs = L.pool + pool_b - slab_b;
  L.total = L.pool + align256(pool_b);
  return L;
}

// Slab metadata in shared memory.
// The window is sliced along the slab axis sa (x or z, whichever the
// channel's line follows more closely); within slab i the cells form the
// rectangle [p0, p0+wp) x [q0, q0+wq) over the other two axes
// (sa = 0: p = y, q = z; sa = 2: p = x, q = y).
struct Slab {
  int off;  // first cell
  int p0, wp;
  int q0, wq;
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

// Block-wide exclusive scan of one int per thread (kWalkThreads threads).
__device__ __forceinline__ int block_excl_scan(int v, int* warp_tot, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = warp_incl_scan(v);
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    int t = lane < (kWalkThreads / 32) ? warp_tot[lane] : 0;
    int ti = warp_incl_scan(t);
    if (lane < (kWalkThreads / 32)) warp_tot[lane] = ti - t;
    if (lane == (kWalkThreads / 32) - 1) *total = ti;
  }
  __syncthreads();
  int r = warp_tot[w] + inc - v;
  __syncthreads();
  return r;
}

// Order-preserving float <-> int keys for warp min/max reductions.
__device__ __forceinline__ int fkey(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fval(int k) {
  return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff);
}

// Index window of slab i along axis sa from the hull's cross-sections at its
// two planes (pext[k] = {pmin, pmax, qmin, qmax} keys at plane k) and the
// hull vertices (crystal corners) inside the slab.  An index range is
// widened by one only on a side whose extreme lies within kWinPad (in
// voxels) of a grid plane, where the rounding of the hull's or a ray's
// arithmetic could put a hit in the neighbouring cell (both are ~1e-6 voxel
// here); the window then holds about 1.7x a row's non-zeros instead of 3.9x
// with a voxel of padding on every side (channels of the full workload).
// A hit outside the window is still counted and reported (hit_outside).
__device__ void slab_window(const Geo& G, const float (*c0)[3], const float (*c1)[3],
                            const int4* pext, int sa, int i, Slab* out) {
  const epet_grid& g = G.p.grid;
  const int pa = sa == 0 ? 1 : 0, qa = sa == 0 ? 2 : 1;
  const float P0 = voxel_plane(g, sa, i), P1 = voxel_plane(g, sa, i + 1);
  int plo = min(pext[i].x, pext[i + 1].x), phi = max(pext[i].y, pext[i + 1].y);
  int qlo = min(pext[i].z, pext[i + 1].z), qhi = max(pext[i].w, pext[i + 1].w);
  for (int k = 0; k < 8; k++) {
    if (c0[k][sa] >= P0 && c0[k][sa] <= P1) {
      plo = min(plo, fkey(c0[k][pa])); phi = max(phi, fkey(c0[k][pa]));
      qlo = min(qlo, fkey(c0[k][qa])); qhi = max(qhi, fkey(c0[k][qa]));
    }
    if (c1[k][sa] >= P0 && c1[k][sa] <= P1) {
      plo = min(plo, fkey(c1[k][pa])); phi = max(phi, fkey(c1[k][pa]));
      qlo = min(qlo, fkey(c1[k][qa])); qhi = max(qhi, fkey(c1[k][qa]));
    }
  }
  out->p0 = out->q0 = 0;
  out->wp = out->wq = 0;
  if (plo > phi) return;  // the bundle does not reach this slab
  const float pmin = fval(plo), pmax = fval(phi), qmin = fval(qlo), qmax = fval(qhi);
  const int np = g.n[pa], nq = g.n[qa];
  auto lo_index = [](float f) {
    const float fl = floorf(f);
    return (int)fl - (f - fl < kWinPad ? 1 : 0);
  };
  auto hi_index = [](float f) {
    const float fl = floorf(f);
    return (int)fl + (f - fl > 1.f - kWinPad ? 1 : 0);
  };
  int a0 = lo_index((pmin - g.o[pa]) / g.d[pa]);
  int a1 = hi_index((pmax - g.o[pa]) / g.d[pa]);
  int b0 = lo_index((qmin - g.o[qa]) / g.d[qa]);
  int b1 = hi_index((qmax - g.o[qa]) / g.d[qa]);
  if (a1 < 0 || a0 > np - 1 || b1 < 0 || b0 > nq - 1) return;
  a0 = clampi(a0, 0, np - 1); a1 = clampi(a1, 0, np - 1);
  b0 = clampi(b0, 0, nq - 1); b1 = clampi(b1, 0, nq - 1);
  out->p0 = a0; out->wp = a1 - a0 + 1;
  out->q0 = b0; out->wq = b1 - b0 + 1;
}

// The window: the cells of a channel's hull, as a table over the columns
// (ix, iy) of its (x, y) bounding box, each column a run of zn consecutive
// z cells from zlo; cells are stored column after column (x major, then y,
// then z), which is voxel-id order.  Each cell holds its exact fixed-point
// sum as two 32-bit words: every chord's units are split as
// hi * 2^fx_split + lo and the halves are summed separately with
// fire-and-forget 32-bit shared atomics; the split is sized (make_geo) so
// neither half can overflow.  The total (hi_sum << fx_split) + lo_sum is
// exact and independent of the order of the adds.
struct Window {
  uint2* cell;  // per cell {lo, hi} sum words
  // per column: {first cell, zlo | zn << 16}; empty: zn 0.  The table has
  // (wbx + 1) x (wby + 1) entries (row stride wbyp = wby + 1): the last
  // column of each row and the last row are empty and stand for every
  // column outside the box.
  const int2* cols;
  const float* planes;  // grid planes: x at [0, n0], y at poff1 + [0, n1], z at poff2 + ...
  int poff1, poff2;
  int bx0, by0, wbx, wby, wbyp;
  int split;
  int trash;      // cell W: absorbs the adds of steps with nothing to add (never read)
  int trash_out;  // cell W + 1: counts (in lo) hits outside the window (must stay 0)
};

// A lane's cached column: first cell, first z, number of z cells.
struct Col {
  int off, zlo, zn;
};
// Column (cx, cy) relative to the box corner; outside the box: an empty
// border entry (both indices clamped, unsigned, to the border).
__device__ __forceinline__ Col load_col(const Window& w, int cx, int cy) {
  const unsigned ux = min((unsigned)cx, (unsigned)w.wbx), uy = min((unsigned)cy, (unsigned)w.wby);
  const int2 e = w.cols[ux * w.wbyp + uy];
  Col c;
  c.off = e.x;
  c.zlo = e.y & 0xffff;
  c.zn = e.y >> 16;
  return c;
}

// One axis of a ray walk: the ray's parameter at grid plane k is the
// reference's quotient (plane_k - r0)/(r1 - r0), correctly rounded.
struct WalkAxis {
  const float* P;           // plane positions o + k*d, k = 0..n (the shared table)
  float o, d, r0, dr, inv;  // ray at r0 + a*dr; inv = RN(1/dr)
  int n, step;
  float lo, hi;  // parameter interval of the current cell along this axis
  int kn;        // index of the plane at hi (cell + 1 ascending, cell descending)
  __device__ __forceinline__ float alpha(int k) const { return div_cr(fsub(P[k], r0), dr, inv); }
  // cell with lo <= a < hi (a inside the axis' grid range); the first
  // guess only starts the search, which corrects it either way; the
  // parameters of the cell's two planes are carried along the search
  __device__ __forceinline__ void enter(float a) {
    int i = clampi((int)floorf(__fdividef(r0 + a * dr - o, d)), 0, n - 1);
    float ai = alpha(i), ai1 = alpha(i + 1);
    if (step > 0) {  // interval of cell i: [alpha(i), alpha(i+1)]
      while (i > 0 && ai > a) { i--; ai1 = ai; ai = alpha(i); }
      while (i < n - 1 && ai1 <= a) { i++; ai = ai1; ai1 = alpha(i + 1); }
      lo = ai;
      hi = ai1;
      kn = i + 1;
    } else {         // interval of cell i: [alpha(i+1), alpha(i)]
      while (i < n - 1 && ai1 > a) { i++; ai = ai1; ai1 = alpha(i + 1); }
      while (i > 0 && ai <= a) { i--; ai1 = ai; ai = alpha(i); }
      lo = ai1;
      hi = ai;
      kn = i;
    }
  }
};

// Walk one ray through the grid and add its chord lengths to the window.
// Voxel interval = [max lo, min hi] over the axes; length = (aMax - aMin) *
// |r1 - r0| (getSystemMatrixFromWorkqueue.cu:24-69).  The walk starts in the
// cell containing the parameter fraction `frac` of the ray's grid range,
// runs to the exit, re-enters at the entry and stops at the starting cell
// (the first cell entered at or after its entry parameter), all in one loop:
// the lanes of a warp walk rays of one channel, each from a different
// starting point (fewer atomic collisions), and stay converged.  Each step
// is branch-free: the axis whose plane comes first is selected and advanced
// with one division.
//
// With npieces > 1 the lane walks only piece `piece` of the ray: the cells
// entered in [a_lo, a_hi), the piece's share of the grid range (no wrap).
// The pieces of a ray compute their common bounds with the same expression,
// so every cell belongs to exactly one piece.  Whole rays and pieces share
// one loop (one copy of its code).
__device__ __forceinline__ void walk_ray(const Geo& G, const float* ray, const Window& w, int* needs_exact,
                         float frac, int piece, int npieces) {
  const epet_grid& g = G.p.grid;
  if (ray[0] == ray[3] && ray[1] == ray[4] && ray[2] == ray[5]) return;
  if (ray[0] == ray[3] || ray[1] == ray[4] || ray[2] == ray[5]) {
    // A ray with equal coordinates on an axis: the reference leaves that
    // axis out of its slab test, so the chord reaches every candidate along
    // it, possibly beyond the bundle window.  Such (rare) rows are redone by
    // the per-candidate path.
    *needs_exact = 1;
    return;
  }
  WalkAxis X, Y, Z;
  X.P = w.planes; Y.P = w.planes + w.poff1; Z.P = w.planes + w.poff2;
  X.o = g.o[0]; X.d = g.d[0]; X.r0 = ray[0]; X.dr = fsub(ray[3], ray[0]); X.n = g.n[0];
  Y.o = g.o[1]; Y.d = g.d[1]; Y.r0 = ray[1]; Y.dr = fsub(ray[4], ray[1]); Y.n = g.n[1];
  Z.o = g.o[2]; Z.d = g.d[2]; Z.r0 = ray[2]; Z.dr = fsub(ray[5], ray[2]); Z.n = g.n[2];
  X.inv = __frcp_rn(X.dr);
  Y.inv = __frcp_rn(Y.dr);
  Z.inv = __frcp_rn(Z.dr);
  X.step = X.dr > 0.f ? 1 : -1;
  Y.step = Y.dr > 0.f ? 1 : -1;
  Z.step = Z.dr > 0.f ? 1 : -1;
  const float L = norm3(X.dr, Y.dr, Z.dr);
  // grid parameter range
  float a_in, a_out;
  {
    const float x0 = X.alpha(0), x1 = X.alpha(X.n);
    const float y0 = Y.alpha(0), y1 = Y.alpha(Y.n);
    const float z0 = Z.alpha(0), z1 = Z.alpha(Z.n);
    a_in = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fminf(z0, z1));
    a_out = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
  }
  if (!(a_in < a_out)) return;
  const float span = fsub(a_out, a_in);
  // a_lim: the walk stops after the cell whose exit parameter reaches it
  // (the grid's exit, the piece's end, or after the wrap the start cell's
  // entry)
  float a_s, a_lo = -INFINITY, a_lim = a_out;
  // entry state of the second part: plane indices, their parameters, and
  // the entry parameter of the grid's first cell
  int ekpx = 0, ekpy = 0, ekpz = 0;
  float ehx = 0.f, ehy = 0.f, ehz = 0.f, eamin = 0.f;
  bool second;
  if (npieces > 1) {
    if (piece > 0) a_lo = fadd(a_in, fmul(span, (float)piece / (float)npieces));
    if (piece + 1 < npieces) a_lim = fadd(a_in, fmul(span, (float)(piece + 1) / (float)npieces));
    a_s = piece > 0 ? a_lo : a_in;
    if (!(a_s < a_out) || !(a_lo < a_lim)) return;  // an empty piece (rounding)
    second = true;  // no wrap
  } else {
    a_s = a_in + span * frac;
    if (!(a_s >= a_in && a_s < a_out)) a_s = a_in;
    // entry state of the second part (the cells before the starting cell),
    // computed up front by all lanes together: the switch in the loop is
    // then a register copy, not a divergent search
    X.enter(a_in);
    Y.enter(a_in);
    Z.enter(a_in);
    ekpx = X.kn; ekpy = w.poff1 + Y.kn; ekpz = w.poff2 + Z.kn;
    ehx = X.hi; ehy = Y.hi; ehz = Z.hi;
    eamin = fmaxf(fmaxf(X.lo, Y.lo), Z.lo);
    second = !(a_s > a_in);  // nothing before the starting cell
  }
  X.enter(a_s);
  Y.enter(a_s);
  Z.enter(a_s);
  const float a_start = fmaxf(fmaxf(X.lo, Y.lo), Z.lo);  // entry of the starting cell
  // Per axis the walk keeps kp, the plane table index of the plane at which
  // it leaves the current cell along that axis (the axis' table offset plus
  // the plane index kn), and h, that plane's parameter; the cell index is
  // kn - 1 (ascending) or kn (descending).  The entry parameter of the
  // current cell is always the latest crossing (the largest of the axes'
  // lo), so it is carried as one value; the cell whose exit parameter reaches
  // a_out is the last before the grid's exit, so no axis steps past its last
  // plane.
  int kpx = X.kn, kpy = w.poff1 + Y.kn, kpz = w.poff2 + Z.kn;
  float hx = X.hi, hy = Y.hi, hz = Z.hi;
  float amin = a_start;
  // a piece's first cell entered before a_lo is the previous piece's: walked
  // as a zero-length cell (every later cell is entered at or after a_lo)
  if (amin < a_lo) amin = fminf(fminf(hx, hy), hz);
  const int ox = (X.step > 0 ? 1 : 0) + w.bx0;  // column = (kp_x - ox, kp_y - oy)
  const int oy = w.poff1 + (Y.step > 0 ? 1 : 0) + w.by0;
  const int oz = w.poff2 + (Z.step > 0 ? 1 : 0);  // z cell = kp_z - oz
  Col col = load_col(w, kpx - ox, kpy - oy);
  // chord units = RN((amax - amin) * L) * 2^s = RN((amax - amin) * (L * 2^s)):
  // scaling by a power of two is exact
  const float Ls = fmul(L, G.fx_scale);
  const uint32_t lo_mask = (1u << w.split) - 1u;
  const int budget = g.n[0] + g.n[1] + g.n[2] + 4;
  for (int steps = 0; steps < budget; steps++) {
    // the axis whose plane comes first (ties: x, then y, then z)
    const float amax = fminf(fminf(hx, hy), hz);
    const bool mx = hx == amax;
    const bool my = !mx && hy == amax;
    const bool mz = !mx && !my;
    {
      // Branch-free add: a step with nothing to add (a zero-length cell, the
      // previous piece's cell) adds to the trash cell, a hit outside the
      // window adds one to the outside cell's count.
      const bool add = amin < amax;
      const unsigned dz = (unsigned)(kpz - oz - col.zlo);
      const bool inwin = dz < (unsigned)col.zn;
      const int c = add ? (inwin ? col.off + (int)dz : w.trash_out) : w.trash;
      // units = RN_int(max(len * scale, 1)) (< 2^64 by the choice of scale:
      // a positive chord counts at least one unit), split as hi * 2^split + lo
      const unsigned long long u = __float2ull_rn(fmaxf(fmul(fsub(amax, amin), Ls), 1.f));
      const uint32_t h = (uint32_t)(u >> w.split);
      const uint32_t l = inwin ? (uint32_t)u & lo_mask : 1u;
      atomicAdd(&w.cell[c].x, l);
      atomicAdd(&w.cell[c].y, h);
    }
    if (amax >= a_lim) {
      // last cell: the part before the starting cell, if any
      if (second || !(eamin < a_start)) break;
      second = true;
      a_lim = a_start;
      kpx = ekpx; kpy = ekpy; kpz = ekpz;
      hx = ehx; hy = ehy; hz = ehz;
      amin = eamin;
      col = load_col(w, kpx - ox, kpy - oy);
      continue;
    }
    // advance the axis whose plane comes first: its next plane's parameter
    // is the reference's quotient over the tabulated plane position
    const int st = mx ? X.step : (my ? Y.step : Z.step);
    const int kp = (mx ? kpx : (my ? kpy : kpz)) + st;
    const float P = w.planes[kp];  // in the table or a guard entry
    const float r0 = mx ? X.r0 : (my ? Y.r0 : Z.r0), dr = mx ? X.dr : (my ? Y.dr : Z.dr);
    const float inv = mx ? X.inv : (my ? Y.inv : Z.inv);
    const float h = div_cr(fsub(P, r0), dr, inv);
    hx = mx ? h : hx; kpx = mx ? kp : kpx;
    hy = my ? h : hy; kpy = my ? kp : kpy;
    hz = mz ? h : hz; kpz = mz ? kp : kpz;
    amin = amax;
    col = load_col(w, kpx - ox, kpy - oy);
  }
}

// Per-channel geometry for the walk, one thread per channel: the 16 crystal
// corners (8 per crystal), the crystal-centre line a, ab, and the exact
// candidate threshold on |ab x ap|^2.  Laid out as kGeomFloats floats per row
// (corners of crystal 0, of crystal 1, a, ab, threshold, padding).
__global__ void k_channel_geom(Geo G, const int32_t* __restrict__ rows, int64_t m,
                               float* __restrict__ geom) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  int id[5];
  channel_decode(G.p.setup, rows[i], id);
  float sn, cs;
  angle_sincos(G.p.setup, id[0], &sn, &cs);
  const CrystalMat m0 = crystal_matrix(G.p.setup, sn, cs, 0, id[1], id[2]);
  const CrystalMat m1 = crystal_matrix(G.p.setup, sn, cs, 1, id[3], id[4]);
  float g[kGeomFloats];
  for (int k = 0; k < 8; k++) {
    crystal_apply(m0, (float)(k & 1), (float)((k >> 1) & 1), (float)(k >> 2), &g[3 * k]);
    crystal_apply(m1, (float)(k & 1), (float)((k >> 1) & 1), (float)(k >> 2), &g[24 + 3 * k]);
  }
  float b[3];
  crystal_apply(m0, 0.5f, 0.5f, 0.5f, &g[48]);
  crystal_apply(m1, 0.5f, 0.5f, 0.5f, b);
  for (int d = 0; d < 3; d++) g[51 + d] = fsub(b[d], g[48 + d]);
  g[54] = candidate_threshold(norm3(g[51], g[52], g[53]), G.sum_radii);
  g[55] = 0.f;
  float4* o = reinterpret_cast<float4*>(geom + i * kGeomFloats);
#pragma unroll
  for (int q = 0; q < kGeomFloats / 4; q++)
    o[q] = make_float4(g[4 * q], g[4 * q + 1], g[4 * q + 2], g[4 * q + 3]);
}

static epet_status launch_channel_geom(const Geo& G, const int32_t* rows, int64_t m, float* geom,
                                       cudaStream_t st) {
  if (m == 0) return EPET_OK;
  k_channel_geom<<<ceil_div(m, 128), 128, 0, st>>>(G, rows, m, geom);
  EPET_LAUNCHED();
  return EPET_OK;
}

template <int kMode>
__global__ void __launch_bounds__(kWalkThreads)
k_walk(WalkArgs args) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Geo& G = args.G;
  const epet_grid& g = G.p.grid;
  const int nx = g.n[0];
  const int nplanes = g.n[0] + g.n[1] + g.n[2] + 3;
  const WalkLayout lay = walk_layout(max(g.n[0], g.n[2]), nplanes, g.n[2], args.cap_cells);
  Slab* slabs = reinterpret_cast<Slab*>(smem + lay.slabs);
  Window win;
  win.split = G.fx_split;
  __shared__ __align__(16) float s_geom[kGeomFloats];
  const float(*c0)[3] = reinterpret_cast<const float(*)[3]>(s_geom);
  const float(*c1)[3] = reinterpret_cast<const float(*)[3]>(s_geom + 24);
  const ChannelLine& line = *reinterpret_cast<const ChannelLine*>(s_geom + 48);
  __shared__ int warp_tot[kWalkThreads / 32];
  __shared__ int s_total, s_exact, s_box[4];
  __shared__ double red_d[kWalkThreads / 32];
  __shared__ float red_f[kWalkThreads / 32];
  __shared__ float s_e;

  if ((int64_t)blockIdx.x >= args.m) return;
  const int64_t row = args.sel ? (int64_t)args.sel[blockIdx.x] : (int64_t)blockIdx.x;
  const int64_t slot = blockIdx.x;  // staging slot

  // ---- channel geometry (k_channel_geom): corners, line, threshold
  if (threadIdx.x < kGeomFloats / 4)
    reinterpret_cast<float4*>(s_geom)[threadIdx.x] =
        reinterpret_cast<const float4*>(args.geom + row * kGeomFloats)[threadIdx.x];
  if (threadIdx.x == 0) {
    s_exact = 0;
    s_box[0] = INT_MAX; s_box[1] = INT_MIN; s_box[2] = INT_MAX; s_box[3] = INT_MIN;
  }
  __syncthreads();
  // slabs along the axis the line follows more closely (x or z)
  const int sa = fabsf(line.ab[2]) > fabsf(line.ab[0]) ? 2 : 0;
  const int pa = sa == 0 ? 1 : 0, qa = sa == 0 ? 2 : 1;
  const int ns = g.n[sa];  // slabs

  // ---- hull cross-section at every slab plane: the 64 crystal-corner pair
  // lines' parameters in shared memory (a thread per line), then two threads
  // per plane, each taking the extremes over 32 of the lines, combined with
  // one shuffle
  int4* pext = reinterpret_cast<int4*>(smem + lay.pext);
  {
    constexpr int kLines = kHullLines;
    // ax, ay, az, inv (0: parallel to the planes), dy, dz of each line
    float(*s_line)[kLines] = reinterpret_cast<float(*)[kLines]>(smem + lay.lines);
    __shared__ int s_nospan;
    if (threadIdx.x == 0) s_nospan = 0;
    __syncthreads();
    if (threadIdx.x < kLines) {
      const int a = threadIdx.x >> 3, b = threadIdx.x & 7;
      const float ax = c0[a][sa], ay = c0[a][pa], az = c0[a][qa];
      const float dx = c1[b][sa] - ax;
      const bool ok = dx != 0.f;
      const float inv = ok ? __frcp_rn(dx) : 0.f;
      s_line[0][threadIdx.x] = ax;
      s_line[1][threadIdx.x] = ay;
      s_line[2][threadIdx.x] = az;
      s_line[3][threadIdx.x] = inv;
      s_line[4][threadIdx.x] = c1[b][pa] - ay;
      s_line[5][threadIdx.x] = c1[b][qa] - az;
      // t is monotone in the plane position: when every line meets the
      // first and the last plane within its segment it meets all of them
      // (the usual case, the grid lying between the heads), and the
      // per-plane tests drop
      const float X0 = voxel_plane(g, sa, 0), X1 = voxel_plane(g, sa, ns);
      const float t0 = (X0 - ax) * inv, t1 = (X1 - ax) * inv;
      if (!(ok && t0 >= 0.f && t0 <= 1.f && t1 >= 0.f && t1 <= 1.f)) s_nospan = 1;
    }
    __syncthreads();
    const bool all_span = s_nospan == 0;
    const int half = threadIdx.x & 1, l0 = half * (kLines / 2);
    for (int k0 = 0; k0 <= ns; k0 += kWalkThreads / 2) {
      const int k = k0 + (threadIdx.x >> 1);
      const float X = voxel_plane(g, sa, min(k, ns));
      float ylo = INFINITY, yhi = -INFINITY, zlo = INFINITY, zhi = -INFINITY;
      bool any = false;
      if (all_span) {
#pragma unroll 8
        for (int l = l0; l < l0 + kLines / 2; l++) {
          const float t = (X - s_line[0][l]) * s_line[3][l];
          const float y = s_line[1][l] + t * s_line[4][l], z = s_line[2][l] + t * s_line[5][l];
          ylo = fminf(ylo, y); yhi = fmaxf(yhi, y);
          zlo = fminf(zlo, z); zhi = fmaxf(zhi, z);
        }
        any = true;
      } else {
        for (int l = l0; l < l0 + kLines / 2; l++) {
          const float inv = s_line[3][l];
          const float t = (X - s_line[0][l]) * inv;
          if (inv != 0.f && t >= 0.f && t <= 1.f) {
            const float y = s_line[1][l] + t * s_line[4][l], z = s_line[2][l] + t * s_line[5][l];
            ylo = fminf(ylo, y); yhi = fmaxf(yhi, y);
            zlo = fminf(zlo, z); zhi = fmaxf(zhi, z);
            any = true;
          }
        }
      }
      ylo = fminf(ylo, __shfl_xor_sync(0xffffffffu, ylo, 1));
      yhi = fmaxf(yhi, __shfl_xor_sync(0xffffffffu, yhi, 1));
      zlo = fminf(zlo, __shfl_xor_sync(0xffffffffu, zlo, 1));
      zhi = fmaxf(zhi, __shfl_xor_sync(0xffffffffu, zhi, 1));
      // (every lane takes part in the shuffle: no short-circuit around it)
      const int any_pair = __shfl_xor_sync(0xffffffffu, (int)any, 1);
      any = any || any_pair != 0;
      if (half == 0 && k <= ns)
        pext[k] = any ? make_int4(fkey(ylo), fkey(yhi), fkey(zlo), fkey(zhi))
                      : make_int4(INT_MAX, INT_MIN, INT_MAX, INT_MIN);
    }
  }
  __syncthreads();

  // ---- per-slab windows (rectangles over the other two axes), their
  // flattened offsets, and the (x, y) bounding box of all of them
  int my_cells = 0;
  const int per = (ns + kWalkThreads - 1) / kWalkThreads;
  const int sbeg = threadIdx.x * per, send = min(ns, sbeg + per);
  {
    int xlo = INT_MAX, xhi = INT_MIN, ylo = INT_MAX, yhi = INT_MIN;
    for (int i = sbeg; i < send; i++) {
      Slab sl;
      slab_window(G, c0, c1, pext, sa, i, &sl);
      slabs[i] = sl;
      my_cells += sl.wp * sl.wq;
      if (sl.wp > 0 && sl.wq > 0) {
        if (sa == 0) {  // slab = x, rectangle over (y, z)
          xlo = min(xlo, i); xhi = max(xhi, i);
          ylo = min(ylo, sl.p0); yhi = max(yhi, sl.p0 + sl.wp - 1);
        } else {        // slab = z, rectangle over (x, y)
          xlo = min(xlo, sl.p0); xhi = max(xhi, sl.p0 + sl.wp - 1);
          ylo = min(ylo, sl.q0); yhi = max(yhi, sl.q0 + sl.wq - 1);
        }
      }
    }
    if (xlo <= xhi) {
      atomicMin(&s_box[0], xlo); atomicMax(&s_box[1], xhi);
      atomicMin(&s_box[2], ylo); atomicMax(&s_box[3], yhi);
    }
  }
  int n_rect = 0;  // cells of all slab rectangles (z slabs only: offsets for the table)
  if (sa == 2) {   // uniform across the block
    const int excl = block_excl_scan(my_cells, warp_tot, &s_total);
    int o = excl;
    for (int i = sbeg; i < send; i++) {
      slabs[i].off = o;
      o += slabs[i].wp * slabs[i].wq;
    }
  }
  __syncthreads();
  if (sa == 2) n_rect = s_total;
  win.bx0 = s_box[0];
  win.by0 = s_box[2];
  win.wbx = s_box[1] >= s_box[0] ? s_box[1] - s_box[0] + 1 : 0;
  win.wby = s_box[3] >= s_box[2] ? s_box[3] - s_box[2] + 1 : 0;
  win.wbyp = win.wby + 1;
  const int A = (win.wbx + 1) * win.wbyp;  // table entries (with the empty border)
  // z range of column k = (ix, iy): for x slabs the range of slab ix's
  // rectangle at iy; for z slabs the first and last slab whose rectangle
  // holds (ix, iy)
  auto col_range_scan = [&](int k, int* zlo, int* zhi) {  // z slabs, no storage
    const int ix = win.bx0 + k / win.wbyp, iy = win.by0 + k % win.wbyp;
    int lo = INT_MAX, hi = INT_MIN;
    for (int iz = 0; iz < ns; iz++) {
      const Slab sl = slabs[iz];
      if ((unsigned)(ix - sl.p0) < (unsigned)sl.wp && (unsigned)(iy - sl.q0) < (unsigned)sl.wq) {
        lo = min(lo, iz);
        hi = iz;
      }
    }
    *zlo = lo;
    *zhi = hi;
  };
  auto col_range_x = [&](int k, int* zlo, int* zhi) {  // x slabs
    const int cx = k / win.wbyp, cy = k % win.wbyp;
    const int ix = win.bx0 + cx, iy = win.by0 + cy;
    const Slab sl = slabs[cx < win.wbx ? ix : win.bx0];  // the border column is empty
    if (cx < win.wbx && cy < win.wby && (unsigned)(iy - sl.p0) < (unsigned)sl.wp) {
      *zlo = sl.q0;
      *zhi = sl.q0 + sl.wq - 1;
    } else {
      *zlo = INT_MAX;
      *zhi = INT_MIN;
    }
  };
  const int kper = (A + kWalkThreads - 1) / kWalkThreads;
  const int kbeg = min(A, (int)threadIdx.x * kper), kend = min(A, kbeg + kper);
  if (kMode == kModeWindow) {
    // columns + cells, computed without the table
    int n = 0;
    for (int k = kbeg; k < kend; k++) {
      int zlo, zhi;
      if (sa == 0) col_range_x(k, &zlo, &zhi);
      else col_range_scan(k, &zlo, &zhi);
      if (zhi >= zlo) n += zhi - zlo + 1;
    }
    block_excl_scan(n, warp_tot, &s_total);
    // + the two trash cells
    if (threadIdx.x == 0) args.win_cells[row] = A + s_total + 2;
    return;
  }
  int2* cols = reinterpret_cast<int2*>(smem + lay.pool);
  const bool table_fits = (size_t)A * 8 <= lay.slabs - lay.pool;  // ends before the slabs
  if (table_fits) {
    if (sa == 0) {
      for (int k = kbeg; k < kend; k++) {
        int zlo, zhi;
        col_range_x(k, &zlo, &zhi);
        cols[k] = make_int2(zlo, zhi);
      }
    } else {
      for (int k = threadIdx.x; k < A; k += kWalkThreads) cols[k] = make_int2(INT_MAX, INT_MIN);
      __syncthreads();
      // every rectangle cell widens its column's range (shared atomics)
      const int rpt = (n_rect + kWalkThreads - 1) / kWalkThreads;
      const int rbeg = min(n_rect, (int)threadIdx.x * rpt), rend = min(n_rect, rbeg + rpt);
      if (rbeg < rend) {
        int lo_s = 0, hi_s = ns - 1;  // last slab with off <= rbeg
        while (lo_s < hi_s) {
          const int mid = (lo_s + hi_s + 1) >> 1;
          if (slabs[mid].off <= rbeg) lo_s = mid;
          else hi_s = mid - 1;
        }
        int iz = lo_s;
        Slab sl = slabs[iz];
        int jp = (rbeg - sl.off) / max(sl.wq, 1), jq = rbeg - sl.off - jp * sl.wq;
        for (int r = rbeg; r < rend; r++) {
          while (r >= sl.off + sl.wp * sl.wq) {
            sl = slabs[++iz];
            jp = 0;
            jq = 0;
          }
          const int k = (sl.p0 + jp - win.bx0) * win.wbyp + (sl.q0 + jq - win.by0);
          atomicMin(&cols[k].x, iz);
          atomicMax(&cols[k].y, iz);
          if (++jq == sl.wq) {
            jq = 0;
            ++jp;
          }
        }
      }
    }
  }
  __syncthreads();
  // column lengths -> first cells (exclusive scan), packed ranges
  int n_mine = 0;
  if (table_fits)
    for (int k = kbeg; k < kend; k++)
      if (cols[k].y >= cols[k].x) n_mine += cols[k].y - cols[k].x + 1;
  const int cexcl = block_excl_scan(n_mine, warp_tot, &s_total);
  const int W = s_total;  // window cells
  if (!table_fits || A + W + 2 > args.cap_cells) {
    if (threadIdx.x == 0) {
      int k = atomicAdd(args.overflow_count, 1);
      args.overflow_rows[k] = (int32_t)row;
      if (kMode == kModeCsr) args.row_len[row] = -1;
    }
    return;
  }
  {
    int o = cexcl;
    for (int k = kbeg; k < kend; k++) {
      const int2 r = cols[k];
      if (r.y >= r.x) {
        cols[k] = make_int2(o, r.x | ((r.y - r.x + 1) << 16));
        o += r.y - r.x + 1;
      } else {
        cols[k] = make_int2(o, 0);  // empty: zn 0
      }
    }
  }
  win.cols = cols;
  // 8A + 8(W + 2) <= pool
  win.cell = reinterpret_cast<uint2*>(smem + lay.pool + (size_t)A * 8);
  win.trash = W;
  win.trash_out = W + 1;
  // grid planes o + k d of the three axes (the walk's quotients read them)
  float* planes = reinterpret_cast<float*>(smem + lay.planes) + 1;  // guards at -1 and nplanes
  win.planes = planes;
  win.poff1 = g.n[0] + 1;
  win.poff2 = g.n[0] + g.n[1] + 2;
  if (threadIdx.x == 0) planes[-1] = planes[nplanes] = 0.f;
  for (int i = threadIdx.x; i < nplanes; i += kWalkThreads) {
    const int a = i < win.poff1 ? 0 : (i < win.poff2 ? 1 : 2);
    planes[i] = voxel_plane(g, a, i - (a == 0 ? 0 : (a == 1 ? win.poff1 : win.poff2)));
  }
  // per z cell the candidate test's z terms ab1 * ap2 and ab0 * ap2
  // (ap = voxel centre - a; the other terms are constant along a column)
  float2* ztab = reinterpret_cast<float2*>(smem + lay.ztab);
  for (int iz = threadIdx.x; iz < g.n[2]; iz += kWalkThreads) {
    const float ap2 = fsub(voxel_centre(g, 2, iz), line.a[2]);
    ztab[iz] = make_float2(fmul(line.ab[1], ap2), fmul(line.ab[0], ap2));
  }
  // ---- zero the window, walk the rays
  for (int i = threadIdx.x; i <= W + 1; i += kWalkThreads) {  // the window and the trash cells
    win.cell[i] = make_uint2(0u, 0u);
  }
  __syncthreads();
  const int R = G.p.nrays;
  const float* rays = args.rays + row * (int64_t)R * 6;
  // Rays to lanes: whole rays, one per lane, in rounds of kWalkThreads;
  // in the last round, whole warps take one ray per lane and the remaining
  // rays are cut into equal pieces over the remaining lanes (100 rays: 3
  // warps of whole rays, 4 rays in 8 pieces each on the fourth warp).
  {
    auto walk = [&](int r, int piece, int np) {
      float ray[6];
      const float2* rp = reinterpret_cast<const float2*>(rays + 6 * r);
      const float2 a = rp[0], b = rp[1], c = rp[2];
      ray[0] = a.x; ray[1] = a.y; ray[2] = b.x; ray[3] = b.y; ray[4] = c.x; ray[5] = c.y;
      // golden-ratio spread of the starting points of whole rays
      const float frac = (float)r * 0.6180339887f - floorf((float)r * 0.6180339887f);
      walk_ray(G, ray, win, &s_exact, frac, piece, np);
    };
    // one call site, so each form of the walk loop is compiled once
    const int t = threadIdx.x;
    const int rounds = R / kWalkThreads;
    const int rr = R - rounds * kWalkThreads, r0 = rounds * kWalkThreads;
    const int fw = rr / 32;  // warps of whole rays in the last round
    for (int k = 0; k <= rounds; k++) {
      int r = k * kWalkThreads + t, piece = 0, np = 1;
      bool act = true;
      if (k == rounds) {
        if (t < fw * 32) {
          r = r0 + t;
        } else {
          const int rem = rr - fw * 32, lanes = kWalkThreads - fw * 32;
          np = rem > 0 ? lanes / rem : 1;
          const int l = t - fw * 32;
          act = rem > 0 && l < rem * np;
          r = r0 + fw * 32 + l / np;
          piece = l % np;
        }
      }
      if (act) walk(r, piece, np);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && win.cell[win.trash_out].x != 0u) atomicAdd(args.hit_outside, 1);
  if (s_exact) {  // uniform across the block
    if (threadIdx.x == 0) {
      int k = atomicAdd(args.exact_count, 1);
      args.exact_rows[k] = (int32_t)row;
      if (kMode == kModeCsr) args.row_len[row] = 0;
    }
    return;
  }

  // ---- ordered extraction: the cells are stored in voxel-id order, thread
  // t takes a contiguous range of them (odd length: the lanes' concurrent
  // reads fall in distinct shared-memory banks)
  const int cpt = ((W + kWalkThreads - 1) / kWalkThreads) | 1;
  const int cbeg = min(W, (int)threadIdx.x * cpt), cend = min(W, cbeg + cpt);
  // Visits the thread's range in order: fcol(ix, iy) on entering a column,
  // f(cell, ix, iy, iz) per cell.
  auto for_cells = [&](auto&& fcol, auto&& f) {
    if (cbeg >= cend) return;
    int lo_k = 0, hi_k = A - 1;  // last column with first cell <= cbeg
    while (lo_k < hi_k) {
      const int mid = (lo_k + hi_k + 1) >> 1;
      if (cols[mid].x <= cbeg) lo_k = mid;
      else hi_k = mid - 1;
    }
    int k = lo_k;
    int2 e = cols[k];
    int zhi = (e.y & 0xffff) + (e.y >> 16) - 1;
    int cx = k / win.wbyp, cy = k - cx * win.wbyp;
    int iz = (e.y & 0xffff) + (cbeg - e.x);
    fcol(win.bx0 + cx, win.by0 + cy);
    for (int cidx = cbeg; cidx < cend; cidx++) {
      if (iz > zhi) {
        do {  // next non-empty column
          ++k;
          if (++cy == win.wbyp) {
            cy = 0;
            ++cx;
          }
          e = cols[k];
          iz = e.y & 0xffff;
          zhi = iz + (e.y >> 16) - 1;
        } while (iz > zhi);
        fcol(win.bx0 + cx, win.by0 + cy);
      }
      f(cidx, win.bx0 + cx, win.by0 + cy, iz);
      ++iz;
    }
  };
  const ChannelLine L = line;
  const float fR = (float)R;
  // pass 1: candidate filter, count, projections
  // (every cell takes the same instructions: the candidate test and the
  // value are computed for all of them and the result selected).  The
  // candidate test is the reference's |ab x ap|^2 with the same operations:
  // its x and y terms come per column, its z terms from the table.
  int cnt = 0;
  float fsum = 0.f;
  const float inv_fR = __frcp_rn(fR);
  float K0 = 0.f, K1 = 0.f, c2sq = 0.f;
  int colvox = 0;
  for_cells(
      [&](int ix, int iy) {
        const float ap0 = fsub(voxel_centre(g, 0, ix), L.a[0]);
        const float ap1 = fsub(voxel_centre(g, 1, iy), L.a[1]);
        K0 = fmul(L.ab[2], ap1);
        K1 = fmul(L.ab[2], ap0);
        const float c2 = fsub(fmul(L.ab[0], ap1), fmul(L.ab[1], ap0));
        c2sq = fmul(c2, c2);
        colvox = ix * G.nyz + iy * g.n[2];
      },
      [&](int cidx, int ix, int iy, int iz) {
    const uint2 cu = win.cell[cidx];
    const unsigned long long u = ((unsigned long long)cu.y << win.split) + (unsigned long long)cu.x;
    const float2 zt = ztab[iz];
    const float c0 = fsub(zt.x, K0), c1 = fsub(K1, zt.y);
    // not a candidate: dropped
    const bool cand = fadd(fadd(fmul(c0, c0), fmul(c1, c1)), c2sq) < L.s_max;
    const bool keep = (u != 0ull) & cand;
    const float v = div_cr(fmul(__ull2float_rn(u), G.fx_inv), fR, inv_fR);
    if (kMode == kModeCsr || kMode == kModeMlem) {
      // kept entries compacted at the start of the thread's range: the slot
      // written is this cell's or an earlier one, already read
      win.cell[cbeg + cnt] = make_uint2(__float_as_uint(v), (uint32_t)(colvox + iz));
    }
    cnt += keep ? 1 : 0;
    if (kMode != kModeCsr && keep) {
      const int vox = colvox + iz;
      if (kMode == kModeForward || kMode == kModeMlem) fsum = fadd(fsum, fmul(v, args.x[vox]));
      if (kMode == kModeBack) {
        const float ev = args.e[row];
        if (ev != 0.f) atomicAdd(&args.c[vox], fmul(v, ev));
      }
      if (kMode == kModeColSum) atomicAdd(&args.s64[vox], (double)v);
    }
  });
  if (kMode == kModeCsr) {
    const int pos = block_excl_scan(cnt, warp_tot, &s_total);
    const int64_t o = slot * args.stride + pos;
    for (int j = 0; j < cnt; j++) {
      const uint2 e = win.cell[cbeg + j];
      args.stage_col[o + j] = (int32_t)e.y;
      args.stage_val[o + j] = __uint_as_float(e.x);
    }
    if (threadIdx.x == 0) {
      args.row_len[row] = s_total;
      if (args.sel) args.ovf_idx[row] = (int32_t)slot;
    }
  } else if (kMode == kModeForward || kMode == kModeMlem) {
    // deterministic block reduction in thread order
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float v = fsum;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fadd(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) red_f[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int k = 0; k < kWalkThreads / 32; k++) t = fadd(t, red_f[k]);
      if (args.y) args.y[row] = t;
      // e = y / (A x) (mlemOperations.hpp:22-32, 0 where A x == 0)
      if (kMode == kModeMlem) s_e = t > 0.f ? __fdiv_rn(args.ycnt[row], t) : 0.f;
    }
    if (kMode == kModeMlem) {
      // the row's share of A^T e: its kept entries, compacted in pass 1
      __syncthreads();
      const float ev = s_e;
      if (ev != 0.f)
        for (int j = 0; j < cnt; j++) {
          const uint2 en = win.cell[cbeg + j];
          atomicAdd(&args.c64[en.y], (double)fmul(__uint_as_float(en.x), ev));
        }
    }
  }
  (void)red_d;
}

// Gather staged rows into their final CSR positions (warp per row).
// Rows redone with a larger window (ovf_idx[row] >= 0) come from the second
// staging area.
// Row sources: ovf_idx[row] = -1: the walk's stage (row * stride);
// >= 0: the redo's stage (slot * stride2); <= -2: row -2 - ovf_idx[row] of
// the per-candidate path's compact buffers (at ex.off[i]).
__global__ void k_gather_rows(const int32_t* __restrict__ stage_col,
                              const float* __restrict__ stage_val, int64_t stride,
                              const int32_t* __restrict__ ovf_idx,
                              const int32_t* __restrict__ stage2_col,
                              const float* __restrict__ stage2_val, int64_t stride2,
                              ExactRows ex, const int64_t* __restrict__ row_ptr, int64_t m,
                              int32_t* __restrict__ col, float* __restrict__ val,
                              int64_t cap) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= m) return;
  const int64_t b = row_ptr[row], n = row_ptr[row + 1] - b;
  if (b + n > cap) return;
  const int32_t oi = ovf_idx ? ovf_idx[row] : -1;
  const int32_t* sc;
  const float* sv;
  if (oi <= -2) {
    const int64_t o = ex.off[-2 - oi];
    sc = ex.col + o;
    sv = ex.val + o;
  } else {
    sc = oi >= 0 ? stage2_col + oi * stride2 : stage_col + row * stride;
    sv = oi >= 0 ? stage2_val + oi * stride2 : stage_val + row * stride;
  }
  for (int64_t k = lane; k < n; k += 32) {
    col[b + k] = sc[k];
    val[b + k] = sv[k];
  }
}

__global__ void k_gather_i32(const int32_t* src, const int32_t* idx, int64_t n,
                             int32_t* dst);

__global__ void k_len_to_i64(const int32_t* len, int64_t* out, int64_t m) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = len[i] < 0 ? 0 : len[i];
}

__global__ void k_offset_rowptr(int64_t* rp, int64_t n, const int64_t* base) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rp[i] += *base;
}

// ------------------------------------------------------------------ host

static size_t walk_smem(const Geo& G, int cap_cells) {
  static_assert(sizeof(Slab) == 20, "walk_layout assumes 20-byte slabs");
  return walk_layout(std::max(G.p.grid.n[0], G.p.grid.n[2]),
                     G.p.grid.n[0] + G.p.grid.n[1] + G.p.grid.n[2] + 3, G.p.grid.n[2], cap_cells)
      .total;
}

// Dynamic shared memory a walk CTA may use on the current device (cached per
// device; any thread).
static int max_dyn_smem() {
  static std::atomic<int> cache[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int>* slot = dev >= 0 && dev < 64 ? &cache[dev] : nullptr;
  int v = slot ? slot->load(std::memory_order_relaxed) : 0;
  if (v == 0) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    v -= 4096;  // static shared memory of the kernel
    if (slot) slot->store(v, std::memory_order_relaxed);
  }
  return v;
}

template <int kMode>
static epet_status launch_walk(WalkArgs a, size_t smem, cudaStream_t st) {
  if (a.m == 0) return EPET_OK;
  EPET_CUDA(cudaFuncSetAttribute(k_walk<kMode>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  k_walk<kMode><<<(unsigned)a.m, kWalkThreads, smem, st>>>(a);
  EPET_LAUNCHED();
  return EPET_OK;
}

// Rows processed per chunk (rays and staging are chunk-sized).
static int64_t chunk_rows(const Geo& G, int cap_cells) {
  const int64_t per_row = (int64_t)G.p.nrays * 24 + (int64_t)cap_cells * 8 + 64;
  int64_t c = ((int64_t)8 << 30) / per_row;  // ~8 GiB of chunk buffers
  c = std::max<int64_t>(1024, std::min<int64_t>(c, 4194304));
  return c;
}

// Window capacity for a problem from a sample of channels spread over all
// angles.  Rows whose window exceeds it are reported and redone with their
// exact size.
static epet_status sample_capacity(const Geo& G, cudaStream_t st, int* cap_out) {
  const epet_setup& s = G.p.setup;
  const int64_t nch = (int64_t)s.na * s.n0z * s.n0y * s.n1z * s.n1y;
  const int64_t per_angle = nch / s.na;
  std::vector<int32_t> sample;
  const int pick = 64;
  for (int a = 0; a < s.na; a++)
    for (int k = 0; k < pick; k++) {
      int64_t c = (int64_t)a * per_angle + (per_angle * k) / pick + (k * 7919) % std::max<int64_t>(1, per_angle / pick);
      sample.push_back((int32_t)std::min<int64_t>(c, nch - 1));
    }
  // the most oblique crystal pairs: every index at an end of its range
  for (int a = 0; a < s.na; a++)
    for (int k = 0; k < 16; k++) {
      const int i0z = (k & 1) ? s.n0z - 1 : 0, i0y = (k & 2) ? s.n0y - 1 : 0;
      const int i1z = (k & 4) ? s.n1z - 1 : 0, i1y = (k & 8) ? s.n1y - 1 : 0;
      const int64_t c = (((((int64_t)a * s.n0z + i0z) * s.n0y + i0y) * s.n1z + i1z) * s.n1y) + i1y;
      sample.push_back((int32_t)c);
    }
  const int64_t n = (int64_t)sample.size();
  int32_t *d_rows = nullptr, *d_cells = nullptr;
  float* d_geom = nullptr;
  EPET_CUDA(dev_alloc((void**)&d_rows, n * 4, st));
  EPET_CUDA(dev_alloc((void**)&d_cells, n * 4, st));
  EPET_CUDA(dev_alloc((void**)&d_geom, n * kGeomFloats * 4, st));
  EPET_CUDA(cudaMemcpyAsync(d_rows, sample.data(), n * 4, cudaMemcpyHostToDevice, st));
  WalkArgs a{};
  a.G = G;
  a.rows = d_rows;
  a.m = n;
  a.win_cells = d_cells;
  a.geom = d_geom;
  epet_status rc = launch_channel_geom(G, d_rows, n, d_geom, st);
  if (rc == EPET_OK) rc = launch_walk<kModeWindow>(a, walk_smem(G, 0), st);
  std::vector<int32_t> cells(n);
  if (rc == EPET_OK) {
    cudaError_t e = cudaMemcpyAsync(cells.data(), d_cells, n * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_status(e, "window sample");
  }
  dev_free(d_rows, st);
  dev_free(d_cells, st);
  dev_free(d_geom, st);
  if (rc != EPET_OK) return rc;
  // Sized for the 90th percentile of the sample, not its maximum: every CTA
  // reserves the capacity in shared memory, so a smaller one keeps more
  // channels resident per SM; the few larger windows are redone with their
  // exact size (redo_overflow).
  std::sort(cells.begin(), cells.end());
  const int p90 = cells.empty() ? 0 : cells[(cells.size() * 9) / 10];
  int cap = std::max(256, (int)(p90 * 1.10) + 64);
  // If a capacity at most 15 % smaller keeps one more CTA resident per SM,
  // take the largest such: the occupancy gain outweighs the few more rows
  // redone.
  auto resident = [&](int c) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_walk<kModeCsr>, kWalkThreads,
                                                      walk_smem(G, c)) != cudaSuccess)
      n = 0;
    return n;
  };
  const int n0 = resident(cap), lo = std::max(256, (int)(cap * 0.85));
  if (n0 > 0 && resident(lo) > n0) {
    int a = lo, b = cap;  // resident(a) > n0 >= resident(b)
    while (b - a > 1) {
      const int mid = (a + b) / 2;
      if (resident(mid) > n0) a = mid;
      else b = mid;
    }
    cap = a;
  }
  *cap_out = cap;
  return EPET_OK;
}

int auto_row_capacity(const epet_problem& p) {
  (void)p;
  return 0;
}

// Rows redone by the per-candidate path / with a larger window since load.
static std::atomic<int64_t> n_exact_rows_{0};
static std::atomic<int64_t> n_overflow_rows_{0};
int64_t exact_rows_total() { return n_exact_rows_.load(); }
int64_t overflow_rows_total() { return n_overflow_rows_.load(); }

// Generic driver: runs mode kMode over all rows in chunks.  For kModeCsr the
// rows are staged and gathered into out (capacity cap).
struct BuildOut {
  epet_csr* csr = nullptr;
  int64_t cap = 0;
  cudaStream_t stream = nullptr;  // stream of the build (growth is ordered on it)
  // optional growth of csr->col/val: returns false on failure; must keep the
  // first `keep` entries and update csr->col/val and cap
  bool (*grow)(BuildOut* self, int64_t need, int64_t keep, int64_t rows_done,
               int64_t rows_total) = nullptr;
  int64_t nnz = 0;
  const float* x = nullptr;
  float* y = nullptr;
  const float* e = nullptr;
  float* c = nullptr;
  double* s64 = nullptr;
  const float* ycnt = nullptr;  // kModeMlem: counts in; c64 out
  double* c64 = nullptr;
  // optional destination of each chunk's entries instead of csr->col/val
  // (rows c0 .. c0+mc-1, n entries in row order from index 0); returns false
  // on failure.  csr->row_ptr still receives the global row pointers.
  bool (*chunk_dst)(BuildOut* self, int64_t c0, int64_t mc, int64_t n, int32_t** col,
                    float** val) = nullptr;
  std::vector<CsrSegment>* segs = nullptr;
};

size_t walk_workspace_size(const Geo& G, int64_t m, int cap_cells, bool csr) {
  const int64_t ch = std::min<int64_t>(std::max<int64_t>(m, 1), chunk_rows(G, cap_cells));
  size_t b = 2 * align256((size_t)ch * G.p.nrays * 24);     // rays (two chunks)
  b += 2 * align256((size_t)ch * kGeomFloats * 4);          // channel geometry (two chunks)
  if (csr) {
    b += 2 * align256((size_t)ch * cap_cells * 4);          // staging col/val
    b += align256((size_t)ch * 4);                          // row_len
    b += align256((size_t)(ch + 1) * 8) * 2;                // counts + rowptr chunk
    b += align256(scan_tmp_elems(ch + 1) * 8);
  }
  b += 3 * align256((size_t)ch * 4) + 256;                  // overflow/exact rows, ovf_idx, flags
  return b;
}

// Second launch over the rows listed in ovf_rows (chunk-local indices): their
// window sizes are measured, the walk reruns with exactly that capacity; CSR
// rows stage into a separate area (stride *cap2) indexed through ovf_idx.
template <int kMode>
static epet_status redo_overflow(WalkArgs a, const int32_t* ovf_rows, int n, int* cap2,
                                 int32_t** s2c, float** s2v, int32_t* ovf_idx,
                                 cudaStream_t st) {
  // temporaries in one owned block, released on every return path
  Scratch tmp;
  EPET_CHECK(tmp.init(nullptr, 0, 3 * align256((size_t)n * 4) +
                                      align256((size_t)n * kGeomFloats * 4), st));
  int32_t* sel = tmp.take<int32_t>(n);
  int32_t* cnl = tmp.take<int32_t>(n);
  int32_t* cells = tmp.take<int32_t>(n);
  float* geom = tmp.take<float>((size_t)n * kGeomFloats);
  if (tmp.overrun) return set_error(EPET_ERR_INVALID, "internal: redo workspace size");
  EPET_CUDA(cudaMemcpyAsync(sel, ovf_rows, n * 4, cudaMemcpyDeviceToDevice, st));
  k_gather_i32<<<ceil_div(n, 256), 256, 0, st>>>(a.rows, sel, n, cnl);
  EPET_LAUNCHED();
  EPET_CHECK(launch_channel_geom(a.G, cnl, n, geom, st));
  WalkArgs w{};
  w.G = a.G;
  w.rows = cnl;
  w.m = n;
  w.win_cells = cells;
  w.geom = geom;
  EPET_CHECK(launch_walk<kModeWindow>(w, walk_smem(a.G, 0), st));
  std::vector<int32_t> h(n);
  EPET_CUDA(cudaMemcpyAsync(h.data(), cells, n * 4, cudaMemcpyDeviceToHost, st));
  EPET_CUDA(cudaStreamSynchronize(st));
  int mx = 0;
  for (int v : h) mx = std::max(mx, v);
  *cap2 = std::max(mx, 1);
  if (walk_smem(a.G, *cap2) > (size_t)max_dyn_smem())
    return set_error(EPET_ERR_UNSUPPORTED, "per-row window of %d cells exceeds shared memory",
                     *cap2);
  WalkArgs b = a;
  b.sel = sel;
  b.m = n;
  b.cap_cells = *cap2;
  b.stride = *cap2;
  b.ovf_idx = ovf_idx;
  if (kMode == kModeCsr) {
    EPET_CUDA(dev_alloc((void**)s2c, (size_t)n * *cap2 * 4, st));
    EPET_CUDA(dev_alloc((void**)s2v, (size_t)n * *cap2 * 4, st));
    b.stage_col = *s2c;
    b.stage_val = *s2v;
  }
  EPET_CUDA(cudaMemsetAsync(a.overflow_count, 0, 4, st));
  EPET_CHECK(launch_walk<kMode>(b, walk_smem(a.G, *cap2), st));
  return EPET_OK;
}

template <int kMode>
static epet_status run_walk(const Geo& G, const int32_t* rows, int64_t m,
                            int cap_cells, BuildOut* out, void* ws, size_t ws_bytes,
                            cudaStream_t st) {
  const bool csr = kMode == kModeCsr;
  const int64_t ch = std::min<int64_t>(std::max<int64_t>(m, 1), chunk_rows(G, cap_cells));
  Scratch scr;
  EPET_CHECK(scr.init(ws, ws_bytes, walk_workspace_size(G, m, cap_cells, csr), st));
  // rays and geometry of two chunks: the next chunk's are generated on a
  // side stream while the current chunk is walked
  float* rays_b[2] = {scr.take<float>((size_t)ch * G.p.nrays * 6),
                      scr.take<float>((size_t)ch * G.p.nrays * 6)};
  float* geom_b[2] = {scr.take<float>((size_t)ch * kGeomFloats),
                      scr.take<float>((size_t)ch * kGeomFloats)};
  int32_t *stage_col = nullptr, *row_len = nullptr;
  float* stage_val = nullptr;
  int64_t *cnt = nullptr, *rp_chunk = nullptr, *scan_tmp = nullptr;
  if (csr) {
    stage_col = scr.take<int32_t>((size_t)ch * cap_cells);
    stage_val = scr.take<float>((size_t)ch * cap_cells);
    row_len = scr.take<int32_t>(ch);
    cnt = scr.take<int64_t>(ch + 1);
    rp_chunk = scr.take<int64_t>(ch + 1);
    scan_tmp = scr.take<int64_t>(scan_tmp_elems(ch + 1));
  }
  int32_t* ovf_rows = scr.take<int32_t>(ch);
  int32_t* ex_rows = scr.take<int32_t>(ch);
  int32_t* ovf_idx = scr.take<int32_t>(ch);
  int32_t* flags = scr.take<int32_t>(64);  // [0] overflow, [1] hits outside, [2] exact rows
  if (scr.overrun) return set_error(EPET_ERR_INVALID, "internal: workspace size");

  EPET_CUDA(cudaMemsetAsync(flags, 0, 64 * 4, st));
  if (csr) EPET_CUDA(cudaMemsetAsync(out->csr->row_ptr, 0, 8, st));
  // ready[b]: buffer b holds its chunk's rays; done[b]: the last kernel that
  // reads buffer b has run (recorded on st).  The side stream is drained
  // before the scratch memory is released, on every return path.
  struct Side {
    cudaStream_t s = nullptr;
    cudaEvent_t start = nullptr, ready[2] = {nullptr, nullptr}, done[2] = {nullptr, nullptr};
    ~Side() {
      if (s) cudaStreamSynchronize(s);
      for (cudaEvent_t e : {start, ready[0], ready[1], done[0], done[1]})
        if (e) cudaEventDestroy(e);
      if (s) cudaStreamDestroy(s);
    }
  } side;
  EPET_CUDA(cudaStreamCreateWithFlags(&side.s, cudaStreamNonBlocking));
  for (cudaEvent_t* e : {&side.start, &side.ready[0], &side.ready[1], &side.done[0], &side.done[1]})
    EPET_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  EPET_CUDA(cudaEventRecord(side.start, st));  // the scratch memory is ready
  EPET_CUDA(cudaStreamWaitEvent(side.s, side.start, 0));
  auto prepare = [&](int64_t c0, int b) -> epet_status {
    const int64_t mc = std::min(ch, m - c0);
    EPET_CUDA(cudaStreamWaitEvent(side.s, side.done[b], 0));
    EPET_CHECK(launch_rays(G, rows + c0, mc, rays_b[b], false, side.s));
    EPET_CHECK(launch_channel_geom(G, rows + c0, mc, geom_b[b], side.s));
    EPET_CUDA(cudaEventRecord(side.ready[b], side.s));
    return EPET_OK;
  };
  if (m > 0) EPET_CHECK(prepare(0, 0));
  int64_t total_nnz = 0;
  for (int64_t c0 = 0, k = 0; c0 < m; c0 += ch, k++) {
    const int64_t mc = std::min(ch, m - c0);
    const int b = (int)(k & 1);
    EPET_CUDA(cudaStreamWaitEvent(st, side.ready[b], 0));
    if (c0 + ch < m) EPET_CHECK(prepare(c0 + ch, b ^ 1));
    float* rays = rays_b[b];
    float* geom = geom_b[b];
    WalkArgs a{};
    a.G = G;
    a.rows = rows + c0;
    a.m = mc;
    a.rays = rays;
    a.geom = geom;
    a.cap_cells = cap_cells;
    a.stride = cap_cells;
    a.stage_col = stage_col;
    a.stage_val = stage_val;
    a.row_len = row_len;
    a.x = out->x;
    a.y = out->y ? out->y + c0 : nullptr;
    a.e = out->e ? out->e + c0 : nullptr;
    a.c = out->c;
    a.s64 = out->s64;
    a.ycnt = out->ycnt ? out->ycnt + c0 : nullptr;
    a.c64 = out->c64;
    a.overflow_rows = ovf_rows;
    a.overflow_count = flags;
    a.hit_outside = flags + 1;
    a.exact_rows = ex_rows;
    a.exact_count = flags + 2;
    EPET_CUDA(cudaMemsetAsync(flags, 0, 4, st));
    EPET_CUDA(cudaMemsetAsync(flags + 2, 0, 4, st));
    EPET_CHECK(launch_walk<kMode>(a, walk_smem(G, cap_cells), st));
    int32_t fl[3] = {0, 0, 0};
    EPET_CUDA(cudaMemcpyAsync(fl, flags, 12, cudaMemcpyDeviceToHost, st));
    EPET_CUDA(cudaStreamSynchronize(st));
    // the chunk's second-stage buffers (redone rows, axis-parallel rows),
    // released on every return path
    struct ChunkExtra {
      cudaStream_t s;
      int32_t* stage2_col = nullptr;
      float* stage2_val = nullptr;
      ExactRows exr;
      ~ChunkExtra() {
        if (stage2_col) dev_free(stage2_col, s);
        if (stage2_val) dev_free(stage2_val, s);
        exr.release(s);
      }
    } extra{st};
    int32_t*& stage2_col = extra.stage2_col;
    float*& stage2_val = extra.stage2_val;
    ExactRows& exr = extra.exr;
    // rows whose window exceeded the capacity: redo them with their exact size
    int cap2 = 0;
    if (csr) EPET_CUDA(cudaMemsetAsync(ovf_idx, 0xff, mc * 4, st));
    if (fl[0] > 0) {
      EPET_CHECK(redo_overflow<kMode>(a, ovf_rows, fl[0], &cap2, &stage2_col, &stage2_val, ovf_idx,
                                      st));
      n_overflow_rows_ += fl[0];
      // the redone rows can add to the list of rows with an axis-parallel ray
      EPET_CUDA(cudaMemcpyAsync(&fl[2], flags + 2, 4, cudaMemcpyDeviceToHost, st));
      EPET_CUDA(cudaStreamSynchronize(st));
    }
    if (fl[2] > 0) {
      // rows with an axis-parallel ray: per-candidate path
      EPET_CHECK(exact_rows_apply(G, rows + c0, ex_rows, fl[2], kMode, row_len,
                                  csr ? ovf_idx : nullptr, &exr, a.x, a.y, a.e, a.c, a.s64,
                                  a.ycnt, a.c64, st));
      n_exact_rows_ += fl[2];
    }
    if (csr) {
      const int T = 256;
      k_len_to_i64<<<ceil_div(mc, T), T, 0, st>>>(row_len, cnt, mc);
      EPET_LAUNCHED();
      EPET_CHECK(exclusive_scan_i64(cnt, rp_chunk, mc, scan_tmp, st));
      // global row pointers: chunk scan + running total
      int64_t* rp = out->csr->row_ptr + c0;
      EPET_CUDA(cudaMemcpyAsync(rp + 1, rp_chunk + 1, mc * 8, cudaMemcpyDeviceToDevice, st));
      k_offset_rowptr<<<ceil_div(mc, T), T, 0, st>>>(rp + 1, mc, rp);
      EPET_LAUNCHED();
      int64_t chunk_total = 0;
      EPET_CUDA(cudaMemcpyAsync(&chunk_total, rp_chunk + mc, 8, cudaMemcpyDeviceToHost, st));
      EPET_CUDA(cudaStreamSynchronize(st));
      if (out->chunk_dst) {
        int32_t* dcol = nullptr;
        float* dval = nullptr;
        if (!out->chunk_dst(out, c0, mc, chunk_total, &dcol, &dval))
          return set_error(EPET_ERR_CUDA, "could not allocate a system-matrix chunk");
        k_gather_rows<<<ceil_div(mc * 32, T), T, 0, st>>>(
            stage_col, stage_val, cap_cells, ovf_idx, stage2_col, stage2_val, cap2, exr, rp_chunk,
            mc, dcol, dval, chunk_total);
      } else {
        if (total_nnz + chunk_total > out->cap && out->grow &&
            !out->grow(out, total_nnz + chunk_total, total_nnz, c0 + mc, m))
          return set_error(EPET_ERR_CUDA, "could not grow the system-matrix buffers");
        k_gather_rows<<<ceil_div(mc * 32, T), T, 0, st>>>(
            stage_col, stage_val, cap_cells, ovf_idx, stage2_col, stage2_val, cap2, exr, rp, mc,
            out->csr->col, out->csr->val, out->cap);
      }
      EPET_LAUNCHED();
      total_nnz += chunk_total;
    }
    EPET_CUDA(cudaEventRecord(side.done[b], st));  // buffer b free for chunk k + 2
  }
  int32_t outside = 0;
  EPET_CUDA(cudaMemcpyAsync(&outside, flags + 1, 4, cudaMemcpyDeviceToHost, st));
  EPET_CUDA(cudaStreamSynchronize(st));
  if (outside)
    return set_error(EPET_ERR_UNSUPPORTED,
                     "%d rows had ray-voxel hits outside the crystal-hull window (ray "
                     "endpoints inside the grid are not supported)", outside);
  out->nnz = total_nnz;
  return EPET_OK;
}

static bool grow_device(BuildOut* self, int64_t need, int64_t keep, int64_t rows_done,
                        int64_t rows_total) {
  // extrapolate the final size from the rows done so far
  double est = (double)need * (double)rows_total / (double)std::max<int64_t>(rows_done, 1);
  int64_t ncap = std::max<int64_t>(need, (int64_t)(est * 1.03) + 1024);
  int32_t* col = nullptr;
  float* val = nullptr;
  const cudaStream_t st = self->stream;
  if (dev_alloc((void**)&col, ncap * 4, st) != cudaSuccess) return false;
  if (dev_alloc((void**)&val, ncap * 4, st) != cudaSuccess) {
    dev_free(col, st);
    return false;
  }
  if (keep > 0) {
    cudaMemcpyAsync(col, self->csr->col, keep * 4, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(val, self->csr->val, keep * 4, cudaMemcpyDeviceToDevice, st);
  }
  if (self->csr->col) dev_free(self->csr->col, st);
  if (self->csr->val) dev_free(self->csr->val, st);
  self->csr->col = col;
  self->csr->val = val;
  self->cap = ncap;
  return true;
}

static bool segment_device(BuildOut* self, int64_t c0, int64_t mc, int64_t n, int32_t** col,
                           float** val) {
  CsrSegment sg{c0, mc, self->segs->empty() ? 0 : self->segs->back().e0 + self->segs->back().n,
                n, nullptr, nullptr};
  const cudaStream_t st = self->stream;
  if (dev_alloc((void**)&sg.col, std::max<int64_t>(n, 1) * 4, st) != cudaSuccess) return false;
  if (dev_alloc((void**)&sg.val, std::max<int64_t>(n, 1) * 4, st) != cudaSuccess) {
    dev_free(sg.col, st);
    return false;
  }
  self->segs->push_back(sg);
  *col = sg.col;
  *val = sg.val;
  return true;
}

static epet_status resolve_capacity(const Geo& G, int32_t max_row_nnz, cudaStream_t st,
                                    int* cap) {
  if (max_row_nnz > 0) {
    *cap = max_row_nnz;
  } else {
    EPET_CHECK(sample_capacity(G, st, cap));
  }
  if (walk_smem(G, *cap) > (size_t)max_dyn_smem())
    return set_error(EPET_ERR_UNSUPPORTED,
                     "per-row window of %d cells exceeds shared memory", *cap);
  if (G.p.grid.n[0] > kMaxSlabs || G.p.grid.n[2] > kMaxSlabs)
    return set_error(EPET_ERR_UNSUPPORTED, "grid nx or nz > %d", kMaxSlabs);
  return EPET_OK;
}

}  // namespace epet

using namespace epet;

static epet_status check_rows(const epet_problem* p, const int32_t* rows, int64_t m) {
  EPET_CHECK(epet_problem_validate(p));
  if (m < 0 || (m > 0 && !rows)) return set_error(EPET_ERR_INVALID, "bad rows");
  return EPET_OK;
}

extern "C" {

size_t epet_sm_build_workspace_size(const epet_problem* p, int64_t m,
                                    int32_t max_row_nnz) {
  if (epet_problem_validate(p) != EPET_OK || max_row_nnz <= 0) return 0;
  return walk_workspace_size(make_geo(*p), m, max_row_nnz, true);
}

epet_status epet_sm_build(const epet_problem* p, const int32_t* rows_d,
                          int64_t m, epet_csr* out, int64_t cap,
                          int64_t* nnz_h, int32_t max_row_nnz, void* ws,
                          size_t ws_bytes, epet_stream_t stream) {
  EPET_CHECK(check_rows(p, rows_d, m));
  if (!out || !out->row_ptr || (cap > 0 && (!out->col || !out->val)) || cap < 0)
    return set_error(EPET_ERR_INVALID, "bad output CSR");
  cudaStream_t st = (cudaStream_t)stream;
  Geo G = make_geo(*p);
  int capc = 0;
  EPET_CHECK(resolve_capacity(G, max_row_nnz, st, &capc));
  if (ws && max_row_nnz <= 0)
    return set_error(EPET_ERR_INVALID, "a caller workspace needs an explicit max_row_nnz");
  BuildOut bo;
  bo.csr = out;
  bo.cap = cap;
  epet_status rc = run_walk<kModeCsr>(G, rows_d, m, capc, &bo, ws, ws_bytes, st);
  if (rc != EPET_OK) return rc;
  out->m = m;
  out->n = G.V;
  out->nnz = bo.nnz;
  if (nnz_h) *nnz_h = bo.nnz;
  if (bo.nnz > cap)
    return set_error(EPET_ERR_CAPACITY, "nnz %lld exceeds capacity %lld",
                     (long long)bo.nnz, (long long)cap);
  return EPET_OK;
}

epet_status epet_project_forward(const epet_problem* p, const int32_t* rows_d,
                                 int64_t m, const float* x_d, float* y_d,
                                 int32_t max_row_nnz, void* ws,
                                 size_t ws_bytes, epet_stream_t stream) {
  EPET_CHECK(check_rows(p, rows_d, m));
  if (!x_d || !y_d) return set_error(EPET_ERR_INVALID, "x/y NULL");
  cudaStream_t st = (cudaStream_t)stream;
  Geo G = make_geo(*p);
  int capc = 0;
  EPET_CHECK(resolve_capacity(G, max_row_nnz, st, &capc));
  BuildOut bo;
  bo.x = x_d;
  bo.y = y_d;
  return run_walk<kModeForward>(G, rows_d, m, capc, &bo, ws, ws_bytes, st);
}

epet_status epet_project_back(const epet_problem* p, const int32_t* rows_d,
                              int64_t m, const float* e_d, float* c_d,
                              int32_t max_row_nnz, void* ws, size_t ws_bytes,
                              epet_stream_t stream) {
  EPET_CHECK(check_rows(p, rows_d, m));
  if (!e_d || !c_d) return set_error(EPET_ERR_INVALID, "e/c NULL");
  cudaStream_t st = (cudaStream_t)stream;
  Geo G = make_geo(*p);
  int capc = 0;
  EPET_CHECK(resolve_capacity(G, max_row_nnz, st, &capc));
  BuildOut bo;
  bo.e = e_d;
  bo.c = c_d;
  return run_walk<kModeBack>(G, rows_d, m, capc, &bo, ws, ws_bytes, st);
}

epet_status epet_project_mlem(const epet_problem* p, const int32_t* rows_d, int64_t m,
                              const float* x_d, const float* y_d, float* ybar_d,
                              double* c64_d, int32_t max_row_nnz, void* ws, size_t ws_bytes,
                              epet_stream_t stream) {
  EPET_CHECK(check_rows(p, rows_d, m));
  if (!x_d || (m > 0 && !y_d) || !c64_d) return set_error(EPET_ERR_INVALID, "x/y/c64 NULL");
  cudaStream_t st = (cudaStream_t)stream;
  Geo G = make_geo(*p);
  int capc = 0;
  EPET_CHECK(resolve_capacity(G, max_row_nnz, st, &capc));
  BuildOut bo;
  bo.x = x_d;
  bo.y = ybar_d;
  bo.ycnt = y_d;
  bo.c64 = c64_d;
  return run_walk<kModeMlem>(G, rows_d, m, capc, &bo, ws, ws_bytes, st);
}

}  // extern "C"

namespace epet {
// CSR build into library-owned buffers (from the library pool, grown as
// needed).
epet_status build_csr_growable(const epet_problem* p, const int32_t* rows, int64_t m,
                               epet_csr* out, int64_t* cap, int32_t max_row_nnz,
                               cudaStream_t st) {
  Geo G = make_geo(*p);
  int capc = 0;
  EPET_CHECK(resolve_capacity(G, max_row_nnz, st, &capc));
  if (!out->row_ptr) EPET_CUDA(dev_alloc((void**)&out->row_ptr, (m + 1) * 8, st));
  BuildOut bo;
  bo.csr = out;
  bo.stream = st;
  bo.cap = *cap;
  bo.grow = grow_device;
  epet_status rc = run_walk<kModeCsr>(G, rows, m, capc, &bo, nullptr, 0, st);
  *cap = bo.cap;
  if (rc != EPET_OK) return rc;
  out->m = m;
  out->n = G.V;
  out->nnz = bo.nnz;
  return EPET_OK;
}

epet_status build_csr_segments(const epet_problem* p, const int32_t* rows, int64_t m,
                               int64_t* row_ptr, std::vector<CsrSegment>* segs, int64_t* nnz,
                               int32_t max_row_nnz, cudaStream_t st) {
  Geo G = make_geo(*p);
  int capc = 0;
  EPET_CHECK(resolve_capacity(G, max_row_nnz, st, &capc));
  epet_csr csr{m, G.V, 0, row_ptr, nullptr, nullptr};
  BuildOut bo;
  bo.csr = &csr;
  bo.stream = st;
  bo.chunk_dst = segment_device;
  bo.segs = segs;
  EPET_CHECK(run_walk<kModeCsr>(G, rows, m, capc, &bo, nullptr, 0, st));
  *nnz = bo.nnz;
  return EPET_OK;
}

epet_status column_sums(const epet_problem* p, const int32_t* rows_d, int64_t m,
                        double* s64, int32_t max_row_nnz, void* ws, size_t ws_bytes,
                        cudaStream_t st) {
  Geo G = make_geo(*p);
  int capc = 0;
  EPET_CHECK(resolve_capacity(G, max_row_nnz, st, &capc));
  BuildOut bo;
  bo.s64 = s64;
  return run_walk<kModeColSum>(G, rows_d, m, capc, &bo, ws, ws_bytes, st);
}
}  // namespace epet
