// Host check of FastDiv (csrc/fastdiv.h): n / d by multiply-high and shifts equals the integer
// division for every divisor 1 .. 4096, selected large divisors, and dividends at the edges
// (0, multiples of d and their neighbours, 2^31 - 1, 2^32 - 1) plus seeded random ones.
// Exit status 0 when every quotient is equal.
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#include "fastdiv.h"

int main() {
  std::mt19937_64 rng(12345);
  std::vector<uint32_t> divisors;
  for (uint32_t d = 1; d <= 4096; ++d) divisors.push_back(d);
  for (uint32_t d : {65535u, 65536u, 65537u, 1000003u, 16777216u, 2147483647u, 2147483648u, 2147483649u,
                     4294967295u})
    divisors.push_back(d);
  for (int k = 0; k < 2000; ++k) divisors.push_back(static_cast<uint32_t>(rng()) | 1u);
  long bad = 0, checked = 0;
  for (uint32_t d : divisors) {
    const lbm_b200::FastDiv f(d);
    std::vector<uint32_t> ns = {0u, 1u, d - 1, d, d + 1, 2147483647u, 2147483648u, 4294967295u, 4294967294u};
    for (uint32_t q : {1u, 2u, 3u, 1000u, 65536u}) {
      const uint64_t m = static_cast<uint64_t>(q) * d;
      if (m + 1 <= 0xffffffffull) {
        ns.push_back(static_cast<uint32_t>(m - 1));
        ns.push_back(static_cast<uint32_t>(m));
        ns.push_back(static_cast<uint32_t>(m + 1));
      }
    }
    for (int k = 0; k < 200; ++k) ns.push_back(static_cast<uint32_t>(rng()));
    for (int k = 0; k < 200; ++k) ns.push_back(static_cast<uint32_t>(rng() % (1u << 24)));
    for (uint32_t n : ns) {
      ++checked;
      if (f.div(n) != n / d) {
        if (bad < 10) std::printf("mismatch: %u / %u = %u, fastdiv %u\n", n, d, n / d, f.div(n));
        ++bad;
      }
    }
  }
  std::printf("fastdiv: %ld mismatches in %ld quotients\n", bad, checked);
  return bad == 0 ? 0 : 1;
}
