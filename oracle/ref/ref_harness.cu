/* Reference harness: a C ABI over the reference's OWN host-callable code,
 * compiled from the reference headers where they lie (include path set by
 * oracle/Makefile), never copied.  Test infrastructure only: it pins the
 * oracle (oracle/epet_oracle.c) and generates the golden fixtures under
 * tests/golden/.  It is built only where the reference tree exists; nothing
 * in the product links it.
 *
 * Everything numeric below is the reference's code: the geometry functors
 * (VoxelGrid.hpp, VoxelGridLinIndex.hpp, MeasurementSetup.hpp,
 * MeasurementSetupLinIndex.hpp, MeasurementSetupTrafo2CartCoord.hpp), the
 * candidate scan (getWorkqueue.hpp:33-113), the slab chord length
 * (getSystemMatrixFromWorkqueue.cu:24-69), cooSort (cooSort.hpp:53-71),
 * convertCsr2Ecsr (convertCsr2Ecsr.hpp:34-47) and the MLEM element-wise ops
 * (mlemOperations.hpp:22-139); the thrust-based ones are built by g++ in
 * ref_harness_thrust.cpp on thrust's CPP (host) backend.  The only glue logic is the
 * per-element value loop, which mirrors the body of the workqueue kernel
 * (getSystemMatrixFromWorkqueue.cu:160-244) with the uniforms supplied by
 * the caller instead of drawn from cuRAND. */
#include <cstdint>
#include <cstdio>
#include <vector>

#include "typedefs.hpp"
#include "getSystemMatrixFromWorkqueue.cu"
#include "getWorkqueue.hpp"
#include "VoxelGridLinIndex.hpp"
#include "MeasurementSetupLinIndex.hpp"

static VG g_grid;
static MS g_setup;

extern "C" {

void ref_setup(float pos0x, float pos1x, int na, int n0z, int n0y, int n1z,
               int n1y, float da, float segx, float segy, float segz,
               float gox, float goy, float goz, float gdx, float gdy,
               float gdz, int gnx, int gny, int gnz) {
  g_setup = MS(pos0x, pos1x, na, n0z, n0y, n1z, n1y, da, segx, segy, segz);
  g_grid = VG(gox, goy, goz, gdx, gdy, gdz, gnx, gny, gnz);
}

/* Channel linear id -> (ida, id0z, id0y, id1z, id1y); and back. */
void ref_channel_decode(int cnl, int* out5) {
  out5[0] = Ida()(cnl, &g_setup);
  out5[1] = Id0z()(cnl, &g_setup);
  out5[2] = Id0y()(cnl, &g_setup);
  out5[3] = Id1z()(cnl, &g_setup);
  out5[4] = Id1y()(cnl, &g_setup);
}
int ref_channel_encode(int ida, int id0z, int id0y, int id1z, int id1y) {
  return DefaultMeasurementSetupLinId<MS>()(id0z, id0y, id1z, id1y, ida,
                                            &g_setup);
}
void ref_voxel_decode(int vxl, int* out3) {
  out3[0] = Idx()(vxl, &g_grid);
  out3[1] = Idy()(vxl, &g_grid);
  out3[2] = Idz()(vxl, &g_grid);
}
int ref_voxel_encode(int idx, int idy, int idz) {
  return DefaultVoxelGridLinId<VG>()(idx, idy, idz, &g_grid);
}

/* Box coordinates in [0,1]^3 of a crystal -> world coordinates. */
void ref_trafo0(const float* box3, int id0z, int id0y, int ida, float* out3) {
  Trafo0()(out3, box3, id0z, id0y, ida, &g_setup);
}
void ref_trafo1(const float* box3, int id1z, int id1y, int ida, float* out3) {
  Trafo1()(out3, box3, id1z, id1y, ida, &g_setup);
}

/* Slab chord length of the line through ray[0..2], ray[3..5] in the box
 * vxl[0..2]-vxl[3..5]. */
float ref_intersection_length(const float* vxl6, const float* ray6) {
  return intersectionLength<float>(vxl6, ray6);
}

/* Candidate scan over the given measurement list (channel ids) and the whole
 * grid, list-major and voxel-minor; returns the number of entries written
 * (at most cap), and the total found in *n_total. */
long long ref_workqueue(const int* cnl_list, int n_list, int* out_cnl,
                        int* out_vxl, long long cap, long long* n_total) {
  ML list(n_list);
  for (int i = 0; i < n_list; i++) list.set(i, cnl_list[i], 1.f);
  int listId = 0, vxlId = 0;
  int fc, fv;
  long long n = 0;
  while (getWorkqueueEntry<val_t, ML, VG, Idx, Idy, Idz, MS, Id0z, Id0y, Id1z,
                           Id1y, Ida, Trafo0, Trafo1>(
             &fc, &fv, listId, vxlId, &list, &g_grid, &g_setup) == 1) {
    if (n < cap) {
      out_cnl[n] = fc;
      out_vxl[n] = fv;
    }
    n++;
  }
  *n_total = n;
  return n < cap ? n : cap;
}

/* Bounded variant of the scan (getWorkqueue.hpp:129-171): at most n entries,
 * resuming from (*listId, *vxlId). */
int ref_workqueue_bounded(const int* cnl_list, int n_list, int* listId,
                          int* vxlId, int n, int* out_cnl, int* out_vxl) {
  ML list(n_list);
  for (int i = 0; i < n_list; i++) list.set(i, cnl_list[i], 1.f);
  std::vector<int> c, v;
  int found = getWorkqueue<val_t, ML, VG, Idx, Idy, Idz, MS, Id0z, Id0y, Id1z,
                           Id1y, Ida, Trafo0, Trafo1>(c, v, *listId, *vxlId,
                                                      &list, &g_grid, &g_setup,
                                                      n);
  for (int i = 0; i < found; i++) {
    out_cnl[i] = c[i];
    out_vxl[i] = v[i];
  }
  return found;
}

/* System-matrix element for (cnl, vxl) with the caller's uniforms
 * rnd[nrays][6] (the kernel draws them with curand_uniform): the voxel box,
 * the two crystal transforms and the chord sum exactly as the workqueue
 * kernel body does, then the division by nrays. */
float ref_sm_value(int cnl, int vxl, int nrays, const float* rnd) {
  float vxlCoord[6];
  int sep[3] = {Idx()(vxl, &g_grid), Idy()(vxl, &g_grid), Idz()(vxl, &g_grid)};
  vxlCoord[0] = g_grid.gridox() + sep[0] * (g_grid.griddx());
  vxlCoord[1] = g_grid.gridoy() + sep[1] * (g_grid.griddy());
  vxlCoord[2] = g_grid.gridoz() + sep[2] * (g_grid.griddz());
  vxlCoord[3] = g_grid.gridox() + (sep[0] + 1) * (g_grid.griddx());
  vxlCoord[4] = g_grid.gridoy() + (sep[1] + 1) * (g_grid.griddy());
  vxlCoord[5] = g_grid.gridoz() + (sep[2] + 1) * (g_grid.griddz());
  float a(0);
  for (int r = 0; r < nrays; r++) {
    float rayCoord[6];
    int id0z = Id0z()(cnl, &g_setup), id0y = Id0y()(cnl, &g_setup);
    int id1z = Id1z()(cnl, &g_setup), id1y = Id1y()(cnl, &g_setup);
    int ida = Ida()(cnl, &g_setup);
    Trafo0()(&rayCoord[0], &rnd[6 * r + 0], id0z, id0y, ida, &g_setup);
    Trafo1()(&rayCoord[3], &rnd[6 * r + 3], id1z, id1y, ida, &g_setup);
    a += intersectionLength(vxlCoord, rayCoord);
  }
  a /= nrays;
  return a;
}

}  // extern "C"
