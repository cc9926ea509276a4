/* Second reference-harness unit: the production kernel's file carries its own
 * copy of the slab chord length (getSystemMatrixDeviceOnly.cu:88-133), which
 * cannot share a translation unit with the workqueue kernel's copy.  Exposed
 * so the tests can check that both copies agree.  Test infrastructure only. */
#include "typedefs.hpp"
#include "getSystemMatrixDeviceOnly.cu"

extern "C" float ref_intersection_length_devonly(const float* vxl6,
                                                 const float* ray6) {
  return intersectionLength<float>(vxl6, ray6);
}
