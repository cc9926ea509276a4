/* Third reference-harness unit, compiled by g++ so that thrust's CPP (host)
 * backend is instantiated for the host only: the reference's cooSort
 * (cooSort.hpp:53-71), convertCsr2Ecsr (convertCsr2Ecsr.hpp:34-47) and MLEM
 * element-wise operators (mlemOperations.hpp:22-139) run on the CPU through
 * the reference's own code.  Test infrastructure only. */
#include <cuda_runtime_api.h>
#include "cooSort.hpp"
#include "convertCsr2Ecsr.hpp"
#include "mlemOperations.hpp"

extern "C" {
void ref_coo_sort(float* val, int* row, int* col, int n) {
  cooSort<float>(val, row, col, n);
}
void ref_csr2ecsr(int* ecsr, int* yRowId, int nnzr, int* csr, int m) {
  convertCsr2Ecsr(ecsr, yRowId, nnzr, csr, m);
}
void ref_divides(float* r, float* a, float* b, int n) {
  divides<float>(r, a, b, n);
}
void ref_divides_multiplies(float* r, float* a, float* b, float* c, int n) {
  dividesMultiplies<float>(r, a, b, c, n);
}
void ref_scales(float* x, float alpha, int n) { scales<float>(x, alpha, n); }
float ref_sum(float* x, int n) { return sum<float>(x, n); }
}
