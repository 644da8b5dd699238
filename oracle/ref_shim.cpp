// C-linkage access shim over the reference's own CPU solvers, compiled together with the
// UNMODIFIED reference sources (src/v0_cpu/solver_v0.cpp, src/v1_omp/solver_v1.cpp,
// src/common/geometry.cpp) by oracle/Makefile into oracle/_ref/libref_{f32,f64}.so.
//
// TEST AND MEASUREMENT INFRASTRUCTURE ONLY: used by tests/golden/make_golden.py (to produce
// golden vectors from the reference itself), by the CPU tests that pin the oracle, and by
// bench.py's CPU baseline (the reference's own solvers timed on the host cores). Never part of
// the product.
//
// The reference API sets a state only through init_equilibrium() (src/v0_cpu/solver_v0.hpp:21,
// src/v1_omp/solver_v1.hpp:30). Seeded random initial states need direct access to the
// population arrays, so this translation unit opens the classes' private members: the standard
// headers are included first (so they are unaffected), then `private` is redefined for the
// reference headers only. v0 receives the post-streaming state as is (its own layout); v1
// receives its preimage by streaming, computed by the oracle's oracle_s_to_r. The golden
// generator checks v0 == v1 bit for bit on every case, which also checks that preimage.
#include <omp.h>

#include <chrono>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#define private public
#include "solver_v0.hpp"
#include "solver_v1.hpp"
#undef private

extern "C" {
void oracle_s_to_r_f32(int nx, int ny, const uint8_t* solid, int open_x, const float* s, float* r);
void oracle_s_to_r_f64(int nx, int ny, const uint8_t* solid, int open_x, const double* s,
                       double* r);
}

namespace {

using lbm::real;

void s_to_r(int nx, int ny, const uint8_t* solid, int open_x, const real* s, real* r) {
  if constexpr (sizeof(real) == sizeof(float))
    oracle_s_to_r_f32(nx, ny, solid, open_x, reinterpret_cast<const float*>(s),
                      reinterpret_cast<float*>(r));
  else
    oracle_s_to_r_f64(nx, ny, solid, open_x, reinterpret_cast<const double*>(s),
                      reinterpret_cast<double*>(r));
}

template <class Solver>
void finish(const Solver& solver, std::size_t n, real* s, real* rho, real* ux, real* uy,
            double* mass) {
  const auto& g = solver.populations();
  std::memcpy(s, g.data(), n * 9 * sizeof(real));
  std::vector<real> r, u, v;
  solver.macroscopic(r, u, v);
  std::memcpy(rho, r.data(), n * sizeof(real));
  std::memcpy(ux, u.data(), n * sizeof(real));
  std::memcpy(uy, v.data(), n * sizeof(real));
  *mass = solver.total_mass();
}

}  // namespace

extern "C" {

// Size of the reference's `real` as compiled (4 or 8).
int ref_real_size() { return static_cast<int>(sizeof(real)); }

// The reference's mask builders (src/common/geometry.cpp:5-23), row-major nx*ny bytes.
void ref_make_channel(int nx, int ny, uint8_t* out) {
  const lbm::Mask m = lbm::make_channel(nx, ny);
  std::memcpy(out, m.data(), m.size());
}
void ref_make_cylinder(int nx, int ny, double xc, double yc, double d, uint8_t* out) {
  const lbm::Mask m = lbm::make_cylinder(nx, ny, xc, yc, d);
  std::memcpy(out, m.data(), m.size());
}
// The reference's Poiseuille body force (src/common/geometry.hpp:24-26), in `real`.
real ref_poiseuille_force(int h, real tau, real u_max) { return lbm::poiseuille_force(h, tau, u_max); }

// Runs the reference v0 solver. init_eq != 0: init_equilibrium(rho0, ux0, uy0); otherwise s
// (v0 layout, solid cells 0) is injected as the initial post-streaming state. On return s holds
// populations(), rho/ux/uy hold macroscopic(), *mass holds total_mass(). Returns 0, or 1 if the
// reference threw (bad arguments).
int ref_v0_run(int nx, int ny, const uint8_t* solid, real tau, real fx, real fy, int open_x,
               real u_in, int init_eq, real rho0, real ux0, real uy0, real* s, int steps,
               real* rho, real* ux, real* uy, double* mass) {
  try {
    const std::size_t n = static_cast<std::size_t>(nx) * ny;
    lbm::SolverV0 solver(nx, ny, tau, fx, fy, lbm::Mask(solid, solid + n));
    if (open_x) solver.set_inflow_outflow(u_in);
    if (init_eq) {
      solver.init_equilibrium(rho0, ux0, uy0);
    } else {
      solver.g_.assign(s, s + n * 9);
      solver.g_new_ = solver.g_;
    }
    solver.run(steps);
    finish(solver, n, s, rho, ux, uy, mass);
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

// Same contract with the reference v1 (OpenMP, pull, SoA) solver; threads > 0 sets the OpenMP
// thread count.
int ref_v1_run(int nx, int ny, const uint8_t* solid, real tau, real fx, real fy, int open_x,
               real u_in, int init_eq, real rho0, real ux0, real uy0, real* s, int steps,
               real* rho, real* ux, real* uy, double* mass, int threads) {
  try {
    if (threads > 0) omp_set_num_threads(threads);
    const std::size_t n = static_cast<std::size_t>(nx) * ny;
    lbm::SolverV1 solver(nx, ny, tau, fx, fy, lbm::Mask(solid, solid + n));
    if (open_x) solver.set_inflow_outflow(u_in);
    if (init_eq) {
      solver.init_equilibrium(rho0, ux0, uy0);
    } else {
      s_to_r(nx, ny, solid, open_x, s, solver.g_.get());
      std::memcpy(solver.g_new_.get(), solver.g_.get(), n * 9 * sizeof(real));
    }
    solver.run(steps);
    finish(solver, n, s, rho, ux, uy, mass);
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

// Times a reference CPU solver on an injected state: `warmup` steps, then `reps` repetitions of
// Solver::run(steps), each timed with std::chrono::steady_clock; seconds[k] receives the k-th.
// v1 uses `threads` OpenMP threads (0: the OpenMP default). Returns 0, or 1 if the reference
// threw.
int ref_v0_bench(int nx, int ny, const uint8_t* solid, real tau, real fx, real fy, const real* s,
                 int warmup, int steps, int reps, double* seconds) {
  try {
    const std::size_t n = static_cast<std::size_t>(nx) * ny;
    lbm::SolverV0 solver(nx, ny, tau, fx, fy, lbm::Mask(solid, solid + n));
    solver.g_.assign(s, s + n * 9);
    solver.g_new_ = solver.g_;
    solver.run(warmup);
    for (int k = 0; k < reps; ++k) {
      const auto t0 = std::chrono::steady_clock::now();
      solver.run(steps);
      seconds[k] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

int ref_v1_bench(int nx, int ny, const uint8_t* solid, real tau, real fx, real fy, const real* s,
                 int warmup, int steps, int reps, int threads, double* seconds) {
  try {
    if (threads > 0) omp_set_num_threads(threads);
    const std::size_t n = static_cast<std::size_t>(nx) * ny;
    lbm::SolverV1 solver(nx, ny, tau, fx, fy, lbm::Mask(solid, solid + n));
    s_to_r(nx, ny, solid, 0, s, solver.g_.get());
    std::memcpy(solver.g_new_.get(), solver.g_.get(), n * 9 * sizeof(real));
    solver.run(warmup);
    for (int k = 0; k < reps; ++k) {
      const auto t0 = std::chrono::steady_clock::now();
      solver.run(steps);
      seconds[k] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

}  // extern "C"
