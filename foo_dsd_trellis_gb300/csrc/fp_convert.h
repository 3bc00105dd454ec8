// Float -> double widening with integer operations.  A hardware conversion
// to a 64-bit type runs at the low FP64-class rate on this part; a kernel
// that widens every output uses a few integer instructions instead.  The
// function follows the IEEE 754 formats directly and returns the hardware
// conversion's bits (checked over every binary32 pattern by
// dsdgpu_selftest_convert; NaNs compare as NaN).
#pragma once
#include <cuda_runtime.h>

namespace dsdgpu {

// binary32 -> binary64, exact, with integer operations only (no branch a
// compiler could turn into a predicated hardware conversion):
//   normal      exponent rebiased (127 -> 1023), significand shifted up 29 bits;
//   zero        the sign alone;
//   subnormal   m * 2^-149 with its leading bit at position t = 31 - clz(m):
//               biased exponent t + 874, the bits below t as the fraction;
//   inf / NaN   exponent all ones, significand shifted up (a NaN gets the
//               quiet bit, as the conversion sets it).
__device__ __forceinline__ double widen_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned m = u & 0x7fffffu;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned long long normal = ((unsigned long long)(e + 896u) << 52) |
                                    ((unsigned long long)m << 29);
  const int t = 31 - __clz((int)(m | 1u));
  const unsigned long long sub = ((unsigned long long)(t + 874) << 52) |
                                 (((unsigned long long)m << (52 - t)) & 0xfffffffffffffull);
  const unsigned long long special = (0x7ffull << 52) |
                                     ((unsigned long long)(m ? (m | 0x400000u) : 0u) << 29);
  const unsigned long long mag = e == 0xffu ? special : (e ? normal : (m ? sub : 0ull));
  return __longlong_as_double((long long)(sign | mag));
}

// The same for an output that is almost always a normal number: the normal
// case from the high and low words (high = sign | ((|u| >> 3) + (896 << 20)),
// low = u << 29: the rebiased exponent and the significand's top 20 bits, and
// its last 3 bits), everything else through widen_exact out of line, so that
// the common path is a handful of integer instructions and a uniform branch.
static __device__ __noinline__ double widen_exact_rare(float f) { return widen_exact(f); }

__device__ __forceinline__ double widen_normal_fast(float f) {
  const unsigned u = __float_as_uint(f);
  if (((u >> 23) & 0xffu) - 1u < 254u) {
    const unsigned hi = (((u & 0x7fffffffu) >> 3) + 0x38000000u) | (u & 0x80000000u);
    return __hiloint2double((int)hi, (int)(u << 29));
  }
  return widen_exact_rare(f);
}

}  // namespace dsdgpu
