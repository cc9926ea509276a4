/* epet_oracle.c -- CPU restatement of the epetreco MLEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see epet_oracle.h): the checker for the CUDA
 * library, never part of the product path.  Compiled with -ffp-contract=off
 * so that every float operation below rounds once, in the reference's order.
 * OpenMP parallelises the per-row loops; results do not depend on the thread
 * count (each row is computed by one thread, reductions are per row). */
#include "epet_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ indices */

/* MeasurementSetupLinIndex.hpp:58-165: angle slowest, id1y fastest. */
void eo_channel_decode(const eo_setup* s, int cnl, int out5[5]) {
  int n4 = s->n1y * s->n1z * s->n0y * s->n0z;
  int n3 = s->n1y * s->n1z * s->n0y;
  int n2 = s->n1y * s->n1z;
  int n1 = s->n1y;
  int t = cnl;
  out5[0] = t / n4;
  t %= n4;
  out5[1] = t / n3;
  t %= n3;
  out5[2] = t / n2;
  t %= n2;
  out5[3] = t / n1;
  out5[4] = t % n1;
}

/* MeasurementSetupLinIndex.hpp:32-45. */
int eo_channel_encode(const eo_setup* s, int ida, int id0z, int id0y, int id1z,
                      int id1y) {
  return ida * (s->n1y * s->n1z * s->n0y * s->n0z) +
         id0z * (s->n1y * s->n1z * s->n0y) + id0y * (s->n1y * s->n1z) +
         id1z * s->n1y + id1y;
}

int64_t eo_nchannels(const eo_setup* s) {
  return (int64_t)s->na * s->n0z * s->n0y * s->n1z * s->n1y;
}

/* VoxelGridLinIndex.hpp:33-35 (x slowest, z fastest) and :52-114. */
void eo_voxel_decode(const eo_grid* g, int vxl, int out3[3]) {
  int nyz = g->n[1] * g->n[2];
  out3[0] = vxl / nyz;
  int t = vxl % nyz;
  out3[1] = t / g->n[2];
  out3[2] = t % g->n[2];
}

int eo_voxel_encode(const eo_grid* g, int ix, int iy, int iz) {
  return ix * (g->n[2] * g->n[1]) + iy * g->n[2] + iz;
}

/* ----------------------------------------------------------------- geometry */

/* Angle argument exactly as MeasurementSetupTrafo2CartCoord.hpp:67-68:
 * T(M_PI)*ida*(meas->da())/T(180.0), evaluated left to right in float. */
static float angle_arg(const eo_setup* s, int ida) {
  float a = (float)M_PI * (float)ida;
  a = a * s->da;
  return a / 180.0f;
}

void eo_trig_table(const eo_setup* s, float* sc) {
  for (int a = 0; a < s->na; a++) {
    float arg = angle_arg(s, a);
    sc[2 * a + 0] = sinf(arg);
    sc[2 * a + 1] = cosf(arg);
  }
}

static void trig_of(const eo_setup* s, const float* trig, int ida, float sc[2]) {
  if (trig) {
    sc[0] = trig[2 * ida];
    sc[1] = trig[2 * ida + 1];
  } else {
    float arg = angle_arg(s, ida);
    sc[0] = sinf(arg);
    sc[1] = cosf(arg);
  }
}

/* MeasurementSetupTrafo2CartCoord.hpp:56-104 (first crystal) and :219-270
 * (second): translate by -1/2, scale by the crystal edges, place the crystal,
 * rotate about y.  The 3x4 matrix and its application keep the reference's
 * operand order; terms multiplied by an exact zero are kept. */
void eo_trafo(const eo_setup* s, const float sc[2], int det, int iz, int iy,
              const float box[3], float out[3]) {
  float edges[3] = {s->segx, s->segy, s->segz};
  int ny = det == 0 ? s->n0y : s->n1y;
  int nz = det == 0 ? s->n0z : s->n1z;
  float pos[3];
  pos[0] = det == 0 ? s->pos0x : s->pos1x;
  pos[1] = (iy - 0.5f * (ny - 1)) * edges[1];
  pos[2] = (iz - 0.5f * (nz - 1)) * edges[2];
  float sin_ = sc[0], cos_ = sc[1];
  float t[12];
  t[0 * 4 + 0] = cos_ * edges[0];
  t[0 * 4 + 1] = 0.f;
  t[0 * 4 + 2] = sin_ * edges[2];
  t[0 * 4 + 3] =
      cos_ * (pos[0] - 0.5f * edges[0]) + sin_ * (pos[2] - 0.5f * edges[2]);
  t[1 * 4 + 0] = 0.f;
  t[1 * 4 + 1] = edges[1];
  t[1 * 4 + 2] = 0.f;
  t[1 * 4 + 3] = pos[1] - 0.5f * edges[1];
  t[2 * 4 + 0] = -sin_ * edges[0];
  t[2 * 4 + 1] = 0.f;
  t[2 * 4 + 2] = cos_ * edges[2];
  t[2 * 4 + 3] =
      -sin_ * (pos[0] - 0.5f * edges[0]) + cos_ * (pos[2] - 0.5f * edges[2]);
  float b0 = box[0], b1 = box[1], b2 = box[2];
  for (int r = 0; r < 3; r++)
    out[r] = t[r * 4 + 0] * b0 + t[r * 4 + 1] * b1 + t[r * 4 + 2] * b2 +
             t[r * 4 + 3] * 1.f;
}

/* distancePointLine.h:19-24 */
static float absolute3(const float* a) {
  return sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
}

/* distancePointLine.h:57-73: |ab x ap| / |ab|. */
static float distance_point_line(const float* a, const float* b,
                                 const float* p) {
  float ap[3], ab[3], c[3];
  for (int d = 0; d < 3; d++) {
    ap[d] = p[d] - a[d];
    ab[d] = b[d] - a[d];
  }
  for (int d = 0; d < 3; d++)
    c[d] = ab[(d + 1) % 3] * ap[(d + 2) % 3] - ab[(d + 2) % 3] * ap[(d + 1) % 3];
  return absolute3(c) / absolute3(ab);
}

static float sum_radii(const eo_setup* s, const eo_grid* g) {
  float ve[3] = {g->d[0], g->d[1], g->d[2]};
  float pe[3] = {s->segx, s->segy, s->segz};
  return 0.5f * (absolute3(ve) + absolute3(pe));
}

typedef struct {
  float a[3], b[3]; /* crystal centres */
  float sr;         /* sum of radii */
} eo_line;

static void channel_line(const eo_setup* s, const eo_grid* g, const float* trig,
                         int cnl, eo_line* L) {
  int id[5];
  eo_channel_decode(s, cnl, id);
  float sc[2];
  trig_of(s, trig, id[0], sc);
  float c[3] = {0.5f, 0.5f, 0.5f};
  eo_trafo(s, sc, 0, id[1], id[2], c, L->a);
  eo_trafo(s, sc, 1, id[3], id[4], c, L->b);
  L->sr = sum_radii(s, g);
}

static int line_candidate(const eo_grid* g, const eo_line* L, int vxl) {
  int iv[3];
  eo_voxel_decode(g, vxl, iv);
  float p[3];
  for (int d = 0; d < 3; d++) p[d] = g->o[d] + (iv[d] + 0.5f) * g->d[d];
  return distance_point_line(L->a, L->b, p) < L->sr;
}

int eo_candidate(const eo_setup* s, const eo_grid* g, const float* trig,
                 int cnl, int vxl) {
  eo_line L;
  channel_line(s, g, trig, cnl, &L);
  return line_candidate(g, &L, vxl);
}

/* getSystemMatrixFromWorkqueue.cu:24-69.  Masked axes (equal ray
 * coordinates) do not take part in the entry/exit max/min. */
float eo_intersection_length(const float v[6], const float r[6]) {
  int sects[3];
  for (int d = 0; d < 3; d++) sects[d] = r[d] != r[3 + d];
  if (!(sects[0] || sects[1] || sects[2])) return 0.f;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int d = 0; d < 3; d++) {
    if (sects[d]) {
      lo[d] = (v[d] - r[d]) / (r[3 + d] - r[d]);
      hi[d] = (v[3 + d] - r[d]) / (r[3 + d] - r[d]);
      if (hi[d] < lo[d]) {
        float t = lo[d];
        lo[d] = hi[d];
        hi[d] = t;
      }
    }
  }
  int good = 0;
  float amin = 0.f, amax = 0.f;
  for (int d = 0; d < 3; d++) {
    if (!sects[d]) continue;
    if (!good) {
      amin = lo[d];
      amax = hi[d];
      good = 1;
    } else {
      amin = amin > lo[d] ? amin : lo[d];
      amax = amax < hi[d] ? amax : hi[d];
    }
  }
  if (!(amin < amax)) return 0.f;
  float dx = r[3] - r[0], dy = r[4] - r[1], dz = r[5] - r[2];
  return (amax - amin) * sqrtf(dx * dx + dy * dy + dz * dz);
}

void eo_rays(const eo_setup* s, const float* trig, int cnl, int nrays,
             const float* rnd, float* rays) {
  int id[5];
  eo_channel_decode(s, cnl, id);
  float sc[2];
  trig_of(s, trig, id[0], sc);
  for (int r = 0; r < nrays; r++) {
    eo_trafo(s, sc, 0, id[1], id[2], &rnd[6 * r + 0], &rays[6 * r + 0]);
    eo_trafo(s, sc, 1, id[3], id[4], &rnd[6 * r + 3], &rays[6 * r + 3]);
  }
}

/* getSystemMatrixFromWorkqueue.cu:150-160: corners o + i*d and o + (i+1)*d. */
void eo_voxel_box(const eo_grid* g, int vxl, float box[6]) {
  int iv[3];
  eo_voxel_decode(g, vxl, iv);
  for (int d = 0; d < 3; d++) {
    box[d] = g->o[d] + iv[d] * g->d[d];
    box[3 + d] = g->o[d] + (iv[d] + 1) * g->d[d];
  }
}

/* Exact sum of floats: TwoSum-compensated double accumulation (the terms are
 * non-negative chord lengths), rounded once to float. */
static float exact_sum_round(const float* t, int n) {
  double s = 0.0, e = 0.0;
  for (int i = 0; i < n; i++) {
    double a = s, b = (double)t[i];
    double sum = a + b;
    double bb = sum - a;
    e += (a - (sum - bb)) + (b - bb);
    s = sum;
  }
  return (float)(s + e);
}

float eo_sm_value(const eo_grid* g, const float* rays, int nrays, int vxl,
                  int sum_mode) {
  float box[6];
  eo_voxel_box(g, vxl, box);
  if (sum_mode == EO_SUM_SEQUENTIAL) {
    float a = 0.f;
    for (int r = 0; r < nrays; r++)
      a += eo_intersection_length(box, &rays[6 * r]);
    a /= nrays;
    return a;
  }
  float stack[256];
  float* t = nrays <= 256 ? stack : (float*)malloc(sizeof(float) * nrays);
  for (int r = 0; r < nrays; r++) t[r] = eo_intersection_length(box, &rays[6 * r]);
  float a = exact_sum_round(t, nrays);
  if (t != stack) free(t);
  return a / (float)nrays;
}

/* ------------------------------------------------------------- workqueue */

static int64_t grid_size(const eo_grid* g) {
  return (int64_t)g->n[0] * g->n[1] * g->n[2];
}

int64_t eo_workqueue_counts(const eo_setup* s, const eo_grid* g,
                            const float* trig, const int32_t* list,
                            int64_t n_list, int64_t* row_count) {
  int64_t V = grid_size(g), total = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total)
  for (int64_t i = 0; i < n_list; i++) {
    eo_line L;
    channel_line(s, g, trig, list[i], &L);
    int64_t c = 0;
    for (int64_t v = 0; v < V; v++) c += line_candidate(g, &L, (int)v);
    row_count[i] = c;
    total += c;
  }
  return total;
}

int64_t eo_workqueue(const eo_setup* s, const eo_grid* g, const float* trig,
                     const int32_t* list, int64_t n_list, int32_t* out_cnl,
                     int32_t* out_vxl, int64_t cap) {
  int64_t* cnt = (int64_t*)malloc(sizeof(int64_t) * (n_list + 1));
  int64_t total = eo_workqueue_counts(s, g, trig, list, n_list, cnt);
  int64_t* off = (int64_t*)malloc(sizeof(int64_t) * (n_list + 1));
  off[0] = 0;
  for (int64_t i = 0; i < n_list; i++) off[i + 1] = off[i] + cnt[i];
  int64_t V = grid_size(g);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t i = 0; i < n_list; i++) {
    if (off[i] >= cap) continue;
    eo_line L;
    channel_line(s, g, trig, list[i], &L);
    int64_t k = off[i];
    for (int64_t v = 0; v < V && k < cap; v++) {
      if (line_candidate(g, &L, (int)v)) {
        out_cnl[k] = list[i];
        out_vxl[k] = (int32_t)v;
        k++;
      }
    }
  }
  free(cnt);
  free(off);
  return total;
}

void eo_sm_values_wq(const eo_setup* s, const eo_grid* g, const float* trig,
                     const int32_t* list, int nrays, const float* rnd_rows,
                     int64_t n_wq, const int32_t* wq_row,
                     const int32_t* wq_vxl, int sum_mode, float* out_val) {
#pragma omp parallel
  {
    float* rays = (float*)malloc(sizeof(float) * 6 * nrays);
    int32_t cur = -1;
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n_wq; i++) {
      if (wq_row[i] != cur) {
        cur = wq_row[i];
        eo_rays(s, trig, list[cur], nrays, &rnd_rows[(int64_t)cur * nrays * 6],
                rays);
      }
      out_val[i] = eo_sm_value(g, rays, nrays, wq_vxl[i], sum_mode);
    }
    free(rays);
  }
}

/* Rows independent; each row scans the grid in ascending voxel order, so the
 * output is already in cooSort's (row, col) order. */
int64_t eo_sm_build_csr(const eo_setup* s, const eo_grid* g, const float* trig,
                        const int32_t* list, int64_t n_list, int nrays,
                        const float* rnd_rows, int sum_mode, int64_t* row_ptr,
                        int32_t* col, float* val, int64_t cap) {
  int64_t V = grid_size(g);
  /* pass 1: per-row non-zero counts */
  int64_t* cnt = (int64_t*)calloc((size_t)n_list + 1, sizeof(int64_t));
#pragma omp parallel
  {
    float* rays = (float*)malloc(sizeof(float) * 6 * nrays);
#pragma omp for schedule(dynamic, 1)
    for (int64_t i = 0; i < n_list; i++) {
      eo_line L;
      channel_line(s, g, trig, list[i], &L);
      eo_rays(s, trig, list[i], nrays, &rnd_rows[i * nrays * 6], rays);
      int64_t c = 0;
      for (int64_t v = 0; v < V; v++)
        if (line_candidate(g, &L, (int)v) &&
            eo_sm_value(g, rays, nrays, (int)v, sum_mode) != 0.f)
          c++;
      cnt[i] = c;
    }
    free(rays);
  }
  row_ptr[0] = 0;
  for (int64_t i = 0; i < n_list; i++) row_ptr[i + 1] = row_ptr[i] + cnt[i];
  free(cnt);
  /* pass 2: fill */
#pragma omp parallel
  {
    float* rays = (float*)malloc(sizeof(float) * 6 * nrays);
#pragma omp for schedule(dynamic, 1)
    for (int64_t i = 0; i < n_list; i++) {
      if (row_ptr[i] >= cap) continue;
      eo_line L;
      channel_line(s, g, trig, list[i], &L);
      eo_rays(s, trig, list[i], nrays, &rnd_rows[i * nrays * 6], rays);
      int64_t k = row_ptr[i];
      for (int64_t v = 0; v < V && k < cap; v++) {
        if (!line_candidate(g, &L, (int)v)) continue;
        float a = eo_sm_value(g, rays, nrays, (int)v, sum_mode);
        if (a != 0.f) {
          col[k] = (int32_t)v;
          val[k] = a;
          k++;
        }
      }
    }
    free(rays);
  }
  return row_ptr[n_list];
}

/* The same rows in one pass: each thread appends its rows' entries to its own
 * growable buffers; eo_sm_build_finish lays them out as a CSR (row order of
 * the list) and frees the handle.  Test infrastructure: identical results to
 * eo_sm_build_csr at a third of its cost. */
typedef struct {
  int64_t n_list, nnz;
  int nthreads;
  int32_t** tcol;
  float** tval;
  int64_t *tlen, *tcap;
  int32_t* row_t;    /* thread that built the row */
  int64_t* row_off;  /* offset in that thread's buffers */
  int64_t* row_cnt;
} eo_build;

void* eo_sm_build_start(const eo_setup* s, const eo_grid* g, const float* trig,
                        const int32_t* list, int64_t n_list, int nrays,
                        const float* rnd_rows, int sum_mode, int64_t* nnz_out) {
  eo_build* b = (eo_build*)calloc(1, sizeof(eo_build));
  const int64_t V = grid_size(g);
  b->n_list = n_list;
  b->nthreads = omp_get_max_threads();
  b->tcol = (int32_t**)calloc((size_t)b->nthreads, sizeof(int32_t*));
  b->tval = (float**)calloc((size_t)b->nthreads, sizeof(float*));
  b->tlen = (int64_t*)calloc((size_t)b->nthreads, sizeof(int64_t));
  b->tcap = (int64_t*)calloc((size_t)b->nthreads, sizeof(int64_t));
  b->row_t = (int32_t*)calloc((size_t)n_list + 1, sizeof(int32_t));
  b->row_off = (int64_t*)calloc((size_t)n_list + 1, sizeof(int64_t));
  b->row_cnt = (int64_t*)calloc((size_t)n_list + 1, sizeof(int64_t));
#pragma omp parallel num_threads(b->nthreads)
  {
    const int t = omp_get_thread_num();
    float* rays = (float*)malloc(sizeof(float) * 6 * nrays);
#pragma omp for schedule(dynamic, 1)
    for (int64_t i = 0; i < n_list; i++) {
      eo_line L;
      channel_line(s, g, trig, list[i], &L);
      eo_rays(s, trig, list[i], nrays, &rnd_rows[i * nrays * 6], rays);
      b->row_t[i] = t;
      b->row_off[i] = b->tlen[t];
      for (int64_t v = 0; v < V; v++) {
        if (!line_candidate(g, &L, (int)v)) continue;
        const float a = eo_sm_value(g, rays, nrays, (int)v, sum_mode);
        if (a == 0.f) continue;
        if (b->tlen[t] == b->tcap[t]) {
          b->tcap[t] = b->tcap[t] ? 2 * b->tcap[t] : 4096;
          b->tcol[t] = (int32_t*)realloc(b->tcol[t], sizeof(int32_t) * (size_t)b->tcap[t]);
          b->tval[t] = (float*)realloc(b->tval[t], sizeof(float) * (size_t)b->tcap[t]);
        }
        b->tcol[t][b->tlen[t]] = (int32_t)v;
        b->tval[t][b->tlen[t]] = a;
        b->tlen[t]++;
      }
      b->row_cnt[i] = b->tlen[t] - b->row_off[i];
    }
    free(rays);
  }
  int64_t nnz = 0;
  for (int64_t i = 0; i < n_list; i++) nnz += b->row_cnt[i];
  b->nnz = nnz;
  *nnz_out = nnz;
  return b;
}

void eo_sm_build_finish(void* h, int64_t* row_ptr, int32_t* col, float* val) {
  eo_build* b = (eo_build*)h;
  row_ptr[0] = 0;
  for (int64_t i = 0; i < b->n_list; i++) row_ptr[i + 1] = row_ptr[i] + b->row_cnt[i];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < b->n_list; i++) {
    const int t = b->row_t[i];
    memcpy(col + row_ptr[i], b->tcol[t] + b->row_off[i], sizeof(int32_t) * (size_t)b->row_cnt[i]);
    memcpy(val + row_ptr[i], b->tval[t] + b->row_off[i], sizeof(float) * (size_t)b->row_cnt[i]);
  }
  for (int t = 0; t < b->nthreads; t++) {
    free(b->tcol[t]);
    free(b->tval[t]);
  }
  free(b->tcol); free(b->tval); free(b->tlen); free(b->tcap);
  free(b->row_t); free(b->row_off); free(b->row_cnt);
  free(b);
}

/* ----------------------------------------------------------- sparse formats */

typedef struct {
  int32_t row, col;
  float val;
  int64_t pos;
} coo_ent;

static int coo_cmp(const void* pa, const void* pb) {
  const coo_ent* a = (const coo_ent*)pa;
  const coo_ent* b = (const coo_ent*)pb;
  if (a->row != b->row) return a->row < b->row ? -1 : 1;
  if (a->col != b->col) return a->col < b->col ? -1 : 1;
  return a->pos < b->pos ? -1 : (a->pos > b->pos); /* stable */
}

/* cooSort.hpp:26-71: (row, col) lexicographic; equal keys keep input order
 * (thrust's comparison sort_by_key is a stable merge sort). */
void eo_coo_sort(float* val, int32_t* row, int32_t* col, int64_t n) {
  coo_ent* e = (coo_ent*)malloc(sizeof(coo_ent) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; i++) {
    e[i].row = row[i];
    e[i].col = col[i];
    e[i].val = val[i];
    e[i].pos = i;
  }
  qsort(e, (size_t)n, sizeof(coo_ent), coo_cmp);
  for (int64_t i = 0; i < n; i++) {
    row[i] = e[i].row;
    col[i] = e[i].col;
    val[i] = e[i].val;
  }
  free(e);
}

/* cusparseXcoo2csr semantics (cusparseWrapper.hpp:38-45): csr[r] = number of
 * entries with row < r, for r = 0..m. */
void eo_coo2csr(const int32_t* row, int64_t nnz, int64_t m, int64_t* csr) {
  for (int64_t r = 0; r <= m; r++) csr[r] = 0;
  for (int64_t i = 0; i < nnz; i++) csr[row[i] + 1]++;
  for (int64_t r = 0; r < m; r++) csr[r + 1] += csr[r];
}

/* convertCsr2Ecsr.hpp:34-47 */
void eo_csr2ecsr(int64_t* ecsr, const int32_t* yRowId, int64_t nnzr,
                 const int64_t* csr, int64_t m) {
  for (int64_t i = 0; i < nnzr; i++) ecsr[i] = csr[yRowId[i]];
  ecsr[nnzr] = csr[m];
}

/* ------------------------------------------------------------------- SpMV */

void eo_csrmv(int trans, int64_t m, int64_t n, const int64_t* rp,
              const int32_t* col, const float* val, float alpha,
              const float* x, float beta, float* y) {
  if (!trans) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; i++) {
      double acc = 0.0;
      for (int64_t k = rp[i]; k < rp[i + 1]; k++)
        acc += (double)val[k] * (double)x[col[k]];
      float ax = (float)acc;
      y[i] = beta == 0.f ? alpha * ax : alpha * ax + beta * y[i];
    }
  } else {
    /* per-thread fp64 column sums over static row ranges, added in thread
     * order, rounded once */
    const int nt = omp_get_max_threads();
    double* acc = (double*)calloc((size_t)n * (size_t)nt, sizeof(double));
#pragma omp parallel num_threads(nt)
    {
      double* a = acc + (size_t)omp_get_thread_num() * (size_t)n;
#pragma omp for schedule(static)
      for (int64_t i = 0; i < m; i++)
        for (int64_t k = rp[i]; k < rp[i + 1]; k++) a[col[k]] += (double)val[k] * (double)x[i];
    }
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
      double t = 0.0;
      for (int q = 0; q < nt; q++) t += acc[(size_t)q * (size_t)n + (size_t)j];
      const float ax = (float)t;
      y[j] = beta == 0.f ? alpha * ax : alpha * ax + beta * y[j];
    }
    free(acc);
  }
}

void eo_csrmv_f64(int trans, int64_t m, int64_t n, const int64_t* rp,
                  const int32_t* col, const float* val, double alpha,
                  const double* x, double beta, double* y) {
  if (!trans) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; i++) {
      double acc = 0.0;
      for (int64_t k = rp[i]; k < rp[i + 1]; k++)
        acc += (double)val[k] * x[col[k]];
      y[i] = beta == 0.0 ? alpha * acc : alpha * acc + beta * y[i];
    }
  } else {
    /* per-thread column sums over static row ranges, added in thread order */
    const int nt = omp_get_max_threads();
    double* acc = (double*)calloc((size_t)n * (size_t)nt, sizeof(double));
#pragma omp parallel num_threads(nt)
    {
      double* a = acc + (size_t)omp_get_thread_num() * (size_t)n;
#pragma omp for schedule(static)
      for (int64_t i = 0; i < m; i++)
        for (int64_t k = rp[i]; k < rp[i + 1]; k++) a[col[k]] += (double)val[k] * x[i];
    }
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
      double t = 0.0;
      for (int q = 0; q < nt; q++) t += acc[(size_t)q * (size_t)n + (size_t)j];
      y[j] = beta == 0.0 ? alpha * t : alpha * t + beta * y[j];
    }
    free(acc);
  }
}

/* ------------------------------------------------------------ MLEM ops */

/* mlemOperations.hpp:22-32: r = a / b, no guard. */
void eo_divides(float* r, const float* a, const float* b, int64_t n) {
  for (int64_t i = 0; i < n; i++) r[i] = a[i] / b[i];
}

/* mlemOperations.hpp:38-79: r = a*b/c with c==0 -> c=1. */
void eo_divides_multiplies(float* r, const float* a, const float* b,
                           const float* c, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    float dvs = c[i];
    dvs += (float)(dvs == 0.f);
    r[i] = a[i] * b[i] / dvs;
  }
}

/* mlemOperations.hpp:85-124 */
void eo_scales(float* x, float alpha, int64_t n) {
  for (int64_t i = 0; i < n; i++) x[i] = alpha * x[i];
}

/* mlemOperations.hpp:133-139, accumulated in double. */
double eo_sum(const float* x, int64_t n) {
  double s = 0.0;
  for (int64_t i = 0; i < n; i++) s += x[i];
  return s;
}

/* reco.cu:209-281 over one chunk holding all measured rows. */
void eo_mlem(int64_t m, int64_t V, const int64_t* rp, const int32_t* col,
             const float* val, const float* y, const float* s, float* x,
             int nit) {
  float* yt = (float*)malloc(sizeof(float) * (m > 0 ? m : 1));
  float* e = (float*)malloc(sizeof(float) * (m > 0 ? m : 1));
  float* c = (float*)malloc(sizeof(float) * V);
  float* xx = (float*)malloc(sizeof(float) * V);
  for (int it = 0; it < nit; it++) {
    for (int64_t j = 0; j < V; j++) c[j] = 0.f;
    eo_csrmv(0, m, V, rp, col, val, 1.f, x, 0.f, yt);
    for (int64_t i = 0; i < m; i++) e[i] = yt[i] > 0.f ? y[i] / yt[i] : 0.f;
    eo_csrmv(1, m, V, rp, col, val, 1.f, e, 1.f, c);
    eo_divides_multiplies(xx, x, c, s, V);
    memcpy(x, xx, sizeof(float) * V);
    double norm = eo_sum(x, V);
    eo_scales(x, (float)(1. / norm), V);
  }
  free(yt);
  free(e);
  free(c);
  free(xx);
}

void eo_mlem_f64(int64_t m, int64_t V, const int64_t* rp, const int32_t* col,
                 const float* val, const double* y, const double* s, double* x,
                 int nit) {
  eo_mlem_f64_trace(m, V, rp, col, val, y, s, x, nit, NULL);
}

/* The same, keeping the image after every iteration in trace[it][V]. */
void eo_mlem_f64_trace(int64_t m, int64_t V, const int64_t* rp, const int32_t* col,
                       const float* val, const double* y, const double* s, double* x,
                       int nit, double* trace) {
  double* yt = (double*)malloc(sizeof(double) * (m > 0 ? m : 1));
  double* e = (double*)malloc(sizeof(double) * (m > 0 ? m : 1));
  double* c = (double*)malloc(sizeof(double) * V);
  for (int it = 0; it < nit; it++) {
    for (int64_t j = 0; j < V; j++) c[j] = 0.0;
    eo_csrmv_f64(0, m, V, rp, col, val, 1.0, x, 0.0, yt);
    for (int64_t i = 0; i < m; i++) e[i] = yt[i] > 0.0 ? y[i] / yt[i] : 0.0;
    eo_csrmv_f64(1, m, V, rp, col, val, 1.0, e, 1.0, c);
    double norm = 0.0;
    for (int64_t j = 0; j < V; j++) {
      double dvs = s[j] == 0.0 ? 1.0 : s[j];
      x[j] = x[j] * c[j] / dvs;
      norm += x[j];
    }
    for (int64_t j = 0; j < V; j++) x[j] = x[j] / norm;
    if (trace) memcpy(trace + (size_t)it * (size_t)V, x, sizeof(double) * (size_t)V);
  }
  free(yt);
  free(e);
  free(c);
}

void eo_sensitivity(int64_t m, int64_t V, const int64_t* rp, const int32_t* col,
                    const float* val, float* s) {
  float* ones = (float*)malloc(sizeof(float) * (m > 0 ? m : 1));
  for (int64_t i = 0; i < m; i++) ones[i] = 1.f;
  eo_csrmv(1, m, V, rp, col, val, 1.f, ones, 0.f, s);
  double norm = eo_sum(s, V);
  eo_scales(s, (float)(1. / norm), V);
  free(ones);
}

double eo_poisson_loglik(int64_t m, const float* y, const float* ybar) {
  double ll = 0.0;
  for (int64_t i = 0; i < m; i++)
    if (ybar[i] > 0.f) ll += (double)y[i] * log((double)ybar[i]) - ybar[i];
  return ll;
}

/* ------------------------------------------------------------ chunking */

/* wrappers.hpp:410-421 */
int64_t eo_n_in_chunk(int64_t id_chunk, int64_t n_all, int64_t n_full) {
  if (id_chunk < (n_all + n_full - 1) / n_full) {
    if (id_chunk < n_all / n_full) return n_full;
    return n_all % n_full;
  }
  return 0;
}

/* wrappers.hpp:428-432 */
int64_t eo_chunk_ptr(int64_t id_chunk, int64_t n_full) {
  return id_chunk * n_full;
}

/* wrappers.hpp:440-446 */
int64_t eo_n_chunks(int64_t max_nnz, int64_t max_n_chunk) {
  return (max_nnz + max_n_chunk - 1) / max_n_chunk;
}
