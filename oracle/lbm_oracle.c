/*
 * CPU oracle for the D2Q9 pull stream-collide path.
 *
 * TEST INFRASTRUCTURE ONLY: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load this library, and only as the checker (or as the timed CPU port of the reference).
 * The product path (the CUDA library) never links, loads or calls it.
 *
 * What it restates (reference paths are relative to the reference project):
 *   - the sequential solver v0: push streaming on the array-of-structures state
 *     g[(y*nx+x)*9+i] (src/v0_cpu/solver_v0.cpp:26-135), with the open-x rules of
 *     src/common/boundary.hpp:26-70;
 *   - the OpenMP solver v1: pull streaming on structure-of-arrays planes r[i*N+cell]
 *     (src/v1_omp/solver_v1.cpp:18-67,136-175), bitwise identical to v0;
 *   - the layout conversions between the two (preimage by streaming, pull gather).
 * Pinning: tests/test_oracle.py checks these functions bit for bit against golden vectors that
 * tests/golden/make_golden.py produced by running the reference's own v0 and v1 sources
 * (compiled from the reference tree by oracle/Makefile into oracle/_ref/).
 *
 * Build: gcc -std=c11 -O3 -ffp-contract=off -fno-trapping-math -fopenmp -fPIC -shared
 * (oracle/build_oracle.py). -ffp-contract=off is required: a fused multiply-add changes the
 * rounding and breaks bit-exactness, and FMA contraction is on by default for GCC on aarch64.
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* D2Q9 direction order 0: rest, 1: +x, 2: +y, 3: -x, 4: -y, 5: (+,+), 6: (-,+), 7: (-,-),
 * 8: (+,-) (src/common/d2q9.hpp:14-25). */
static const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

/* Counter-based SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
 * generators", OOPSLA 2014): element k of the stream of `seed` is the SplitMix64 finaliser applied
 * to seed + (k + 1) * 0x9E3779B97F4A7C15. Mapped to [-amp, amp) through the top 53 bits. This is
 * the seeded initial-state generator of the at-scale channel workloads; the Python side restates
 * it with numpy uint64 arithmetic. */
static inline uint64_t splitmix64_at(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double oracle_seeded_uniform(uint64_t seed, uint64_t k, double amp) {
  const double u = (double)(splitmix64_at(seed, k) >> 11) * 0x1.0p-53;
  return -amp + 2.0 * amp * u;
}

void oracle_seeded_fill(uint64_t seed, double amp, uint64_t count, double* out) {
  for (uint64_t k = 0; k < count; ++k) out[k] = oracle_seeded_uniform(seed, k, amp);
}

#define REAL float
#define FN(name) name##_f32
#include "lbm_oracle_impl.h"
#undef REAL
#undef FN

#define REAL double
#define FN(name) name##_f64
#include "lbm_oracle_impl.h"
#undef REAL
#undef FN

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
