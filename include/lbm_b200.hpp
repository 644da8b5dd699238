// lbm_b200.hpp - header-only C++17 drop-in for the reference's GPU solver class.
//
// lbm::SolverB200 has exactly the member set of lbm::SolverV3 (reference
// src/v3_cuda_opt/solver_v3.hpp:27-57), implemented on the C ABI of lbm_b200.h, so that the
// reference's templated consumers compile against it unchanged:
//   run_driver<Solver>           (src/common/driver.hpp:255-300),
//   poiseuille::run_all<Solver>  (tests/poiseuille_check.hpp:128-158),
//   cylinder_case::run<Solver>   (tests/cylinder_case.hpp:33-41),
//   run<Solver> of tests/test_v3_vs_v0.cu:30-37.
// Inside the reference tree it uses the reference's lbm::real and lbm::Mask (include
// "geometry.hpp" from src/common). Define LBM_B200_STANDALONE to use it without that tree
// (lbm::real is float, or double with LBM_REAL_DOUBLE).
//
// Error semantics follow the reference: bad arguments throw std::invalid_argument
// (solver_v3.cu:169-170); CUDA failures, which abort in the reference (cuda_check.hpp:17-27),
// throw std::runtime_error here.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "lbm_b200.h"

#ifdef LBM_B200_STANDALONE
namespace lbm {
#ifdef LBM_REAL_DOUBLE
using real = double;
#else
using real = float;
#endif
using Mask = std::vector<std::uint8_t>;
}  // namespace lbm
#else
#include "geometry.hpp"
#endif

namespace lbm {

class SolverB200 {
 public:
  // Storage form as compiled: the reference's `real` selects FP32 or FP64 (both bit-exact
  // with v0).
  static constexpr int kPrecision = sizeof(real) == sizeof(double) ? LBM_FP64 : LBM_FP32;

  SolverB200(int nx, int ny, real tau, real force_x, real force_y, Mask solid)
      : nx_(nx), ny_(ny), solid_(std::move(solid)) {
    if (solid_.size() != static_cast<std::size_t>(nx) * static_cast<std::size_t>(ny))
      throw std::invalid_argument("solid mask size does not match the grid");
    if (tau <= real(0.5)) throw std::invalid_argument("tau must be > 0.5");
    check(lbm_create(nx, ny, solid_.data(), static_cast<double>(tau),
                     static_cast<double>(force_x), static_cast<double>(force_y), kPrecision, &h_),
          "lbm_create");
  }
  ~SolverB200() { lbm_destroy(h_); }
  SolverB200(const SolverB200&) = delete;
  SolverB200& operator=(const SolverB200&) = delete;

  void init_equilibrium(real rho0, real ux0, real uy0) {
    check(lbm_init_equilibrium(h_, rho0, ux0, uy0), "init_equilibrium");
  }
  // Opens the domain in x (inlet (u_in, 0) at x = 0, outflow at x = nx - 1); call before
  // init_equilibrium(), as with the reference.
  void set_inflow_outflow(real u_in) { check(lbm_set_inflow_outflow(h_, u_in), "set_inflow_outflow"); }
  void step() { check(lbm_step(h_, 1), "step"); }
  void run(int steps) { check(lbm_run(h_, steps), "run"); }
  double timed_run(int steps) {
    double t = 0.0;
    check(lbm_timed_run(h_, steps, &t), "timed_run");
    return t;
  }

  void macroscopic(std::vector<real>& rho, std::vector<real>& ux, std::vector<real>& uy) const {
    const std::size_t n = cells();
    rho.assign(n, real(0));
    ux.assign(n, real(0));
    uy.assign(n, real(0));
    check(lbm_macroscopic(h_, rho.data(), ux.data(), uy.data()), "macroscopic");
  }
  double total_mass() const {
    double m = 0.0;
    check(lbm_total_mass(h_, &m), "total_mass");
    return m;
  }
  std::vector<real> populations() const {
    std::vector<real> g(cells() * 9);
    check(lbm_get_populations(h_, g.data()), "populations");
    return g;
  }
  void populations_at(int x, int y, real* out) const {
    check(lbm_populations_at(h_, x, y, out), "populations_at");
  }

  int threads() const { return 0; }
  std::string bench_info() const {
    char buf[1024];
    check(lbm_device_info(h_, buf, sizeof buf), "bench_info");
    return buf;
  }

  int nx() const { return nx_; }
  int ny() const { return ny_; }
  const Mask& solid() const { return solid_; }

  // Extensions beyond the SolverV3 member set.
  void set_populations(const std::vector<real>& s) {
    if (s.size() != cells() * 9) throw std::invalid_argument("populations size");
    check(lbm_set_populations(h_, s.data()), "set_populations");
  }
  lbm_solver* handle() const { return h_; }

 private:
  std::size_t cells() const { return static_cast<std::size_t>(nx_) * static_cast<std::size_t>(ny_); }
  void check(int rc, const char* what) const {
    if (rc == LBM_OK) return;
    static const char* const names[] = {"ok", "invalid argument", "CUDA error", "out of memory",
                                        "diverged", "unsupported", "timeout"};
    const std::string detail = h_ ? lbm_last_error(h_) : "";
    const std::string msg = std::string(what) + ": " +
                            (rc >= 0 && rc <= 6 ? names[rc] : "error") +
                            (detail.empty() ? "" : " (" + detail + ")");
    if (rc == LBM_ERR_INVALID_ARG) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
  }

  int nx_, ny_;
  Mask solid_;
  lbm_solver* h_ = nullptr;
};

}  // namespace lbm
