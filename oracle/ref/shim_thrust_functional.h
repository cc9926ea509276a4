/* Build shim for compiling the reference's thrust-based headers with CCCL 3
 * (CUDA 13), where thrust::binary_function / thrust::unary_function were
 * removed.  The reference derives its functors from these empty bases
 * (cooSort.hpp, mlemOperations.hpp); nothing else in them uses the bases.
 * Test infrastructure only: force-included into oracle/ref/ref_harness.cu. */
#pragma once
#include <thrust/functional.h>
namespace thrust {
template <typename A, typename B, typename R>
struct binary_function {
  typedef A first_argument_type;
  typedef B second_argument_type;
  typedef R result_type;
};
template <typename A, typename R>
struct unary_function {
  typedef A argument_type;
  typedef R result_type;
};
}  // namespace thrust
