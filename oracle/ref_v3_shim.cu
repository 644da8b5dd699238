// C-linkage access shim over the reference's own GPU solver v3 (src/v3_cuda_opt/solver_v3.cu),
// compiled together with the UNMODIFIED reference source, with the reference's Release CUDA
// flags (-O3 -DNDEBUG --fmad=false) for sm_103a, by oracle/Makefile into
// oracle/_ref/libref_v3_{f32,f64}.so.
//
// TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the GPU tests run the reference's kernel through it
// on the same inputs as the library's kernels, and bench.py times it beside them on the same
// GPU. Never part of the product.
//
// As in ref_shim.cpp, the class's private members are opened (the standard headers first, then
// `private` redefined for the reference header only) so that a seeded state can be injected:
// the reference sets a state only through init_equilibrium() (solver_v3.cu:194-226). The pull
// state it keeps is the preimage by streaming of the post-streaming state, computed by the
// oracle's oracle_s_to_r (the same conversion the reference's init_equilibrium applies to a
// uniform state); it is copied into both of the solver's buffers, as init_equilibrium does.
// The reference aborts the process on a CUDA error (src/common/cuda_check.hpp:17-27).
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#define private public
#include "solver_v3.hpp"
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

// Selects the reference's kernel variant (read by the SolverV3 constructor from
// LBM_V3_VARIANT, solver_v3.cu:137-143); null or "" keeps the reference's default.
void select_variant(const char* variant) {
  if (variant && *variant)
    setenv("LBM_V3_VARIANT", variant, 1);
  else
    unsetenv("LBM_V3_VARIANT");
}

void inject(lbm::SolverV3& solver, int nx, int ny, const uint8_t* solid, int open_x,
            const real* s) {
  const std::size_t n = static_cast<std::size_t>(nx) * ny * 9;
  std::vector<real> r(n);
  s_to_r(nx, ny, solid, open_x, s, r.data());
  if (cudaMemcpy(solver.g_d_, r.data(), n * sizeof(real), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(solver.g_new_d_, r.data(), n * sizeof(real), cudaMemcpyHostToDevice) != cudaSuccess)
    throw std::runtime_error("state upload failed");
}

}  // namespace

extern "C" {

// Size of the reference's `real` as compiled (4 or 8).
int ref_v3_real_size() { return static_cast<int>(sizeof(real)); }

// Runs the reference v3 solver, same contract as ref_v0_run (ref_shim.cpp): init_eq != 0:
// init_equilibrium(rho0, ux0, uy0); otherwise s (v0 layout, solid cells 0) is injected as the
// initial post-streaming state. On return s holds populations(), rho/ux/uy hold macroscopic(),
// *mass holds total_mass(). Returns 0, or 1 if the reference threw (bad arguments).
int ref_v3_run(int nx, int ny, const uint8_t* solid, real tau, real fx, real fy, int open_x,
               real u_in, int init_eq, real rho0, real ux0, real uy0, real* s, int steps,
               real* rho, real* ux, real* uy, double* mass, const char* variant) {
  try {
    select_variant(variant);
    const std::size_t n = static_cast<std::size_t>(nx) * ny;
    lbm::SolverV3 solver(nx, ny, tau, fx, fy, lbm::Mask(solid, solid + n));
    if (open_x) solver.set_inflow_outflow(u_in);
    if (init_eq)
      solver.init_equilibrium(rho0, ux0, uy0);
    else
      inject(solver, nx, ny, solid, open_x, s);
    solver.run(steps);
    const std::vector<real> g = solver.populations();
    std::memcpy(s, g.data(), n * 9 * sizeof(real));
    std::vector<real> r, u, v;
    solver.macroscopic(r, u, v);
    std::memcpy(rho, r.data(), n * sizeof(real));
    std::memcpy(ux, u.data(), n * sizeof(real));
    std::memcpy(uy, v.data(), n * sizeof(real));
    *mass = solver.total_mass();
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

// Times the reference v3 solver on a state: injects s (v0 layout), runs `warmup` steps
// (SolverV3::run, which synchronises), then `reps` times SolverV3::timed_run(steps) (CUDA
// events around `steps` step() calls on the legacy default stream, solver_v3.cu:285-298);
// seconds[k] receives the k-th repetition. If `digest_out` is not null it receives the
// populations() after all steps (v0 layout, nx*ny*9 values). info receives bench_info().
int ref_v3_bench(int nx, int ny, const uint8_t* solid, real tau, real fx, real fy, const real* s,
                 int warmup, int steps, int reps, double* seconds, real* state_out, char* info,
                 size_t info_size, const char* variant) {
  try {
    select_variant(variant);
    const std::size_t n = static_cast<std::size_t>(nx) * ny;
    lbm::SolverV3 solver(nx, ny, tau, fx, fy, lbm::Mask(solid, solid + n));
    inject(solver, nx, ny, solid, 0, s);
    solver.run(warmup);
    for (int k = 0; k < reps; ++k) seconds[k] = solver.timed_run(steps);
    if (state_out) {
      const std::vector<real> g = solver.populations();
      std::memcpy(state_out, g.data(), n * 9 * sizeof(real));
    }
    if (info && info_size) std::snprintf(info, info_size, "%s", solver.bench_info().c_str());
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

}  // extern "C"
