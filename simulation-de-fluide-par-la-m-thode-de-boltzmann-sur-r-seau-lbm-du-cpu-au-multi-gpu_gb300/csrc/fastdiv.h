// Division of 32-bit unsigned integers by a runtime-invariant divisor with one multiply-high,
// a subtract, two adds and two shifts instead of the integer division's instruction sequence.
// Method: Granlund and Montgomery, "Division by invariant integers using multiplication"
// (PLDI 1994), figure 4.1: with l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1,
//   t = mulhi(m, n),  n / d = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0)
// for every 32-bit n and every divisor d >= 1. Plain C++ so that host code (and the host tests)
// use the same arithmetic.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define FASTDIV_HD __host__ __device__ __forceinline__
#else
#define FASTDIV_HD inline
#endif

namespace lbm_b200 {

struct FastDiv {
  uint32_t d = 1, m = 1, s1 = 0, s2 = 0;

  FastDiv() = default;
  explicit FastDiv(uint32_t divisor) : d(divisor) {
    uint32_t l = 0;
    while (l < 32 && (uint64_t(1) << l) < divisor) ++l;
    m = static_cast<uint32_t>(((uint64_t(1) << 32) * ((uint64_t(1) << l) - divisor)) / divisor + 1);
    s1 = l < 1 ? l : 1;
    s2 = l > 1 ? l - 1 : 0;
  }

  FASTDIV_HD uint32_t div(uint32_t n) const {
#if defined(__CUDA_ARCH__)
    const uint32_t t = __umulhi(m, n);
#else
    const uint32_t t = static_cast<uint32_t>((static_cast<uint64_t>(m) * n) >> 32);
#endif
    return (t + ((n - t) >> s1)) >> s2;
  }
};

}  // namespace lbm_b200
