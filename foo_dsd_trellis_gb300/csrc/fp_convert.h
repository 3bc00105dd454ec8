// Float -> double widening on the integer pipe.  A hardware conversion to a
// 64-bit type runs at the low FP64-class rate on this part; a kernel that
// widens every output uses a few integer instructions instead.  The function follows the IEEE 754
// formats directly and returns the hardware conversion's bits (checked over
// every binary32 pattern by dsdgpu_selftest_convert).
#pragma once
#include <cuda_runtime.h>

namespace dsdgpu {

// binary32 -> binary64, exact: the exponent rebiased (127 -> 1023), the
// significand shifted up by 29 bits.  Zeros, subnormals, infinities and NaNs
// take the hardware conversion.
__device__ __forceinline__ double widen_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const unsigned long long bits = ((unsigned long long)(u >> 31) << 63) |
                                  ((unsigned long long)(e + 896u) << 52) |
                                  ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

}  // namespace dsdgpu
