// Per-storage-form choices shared by the solver and the strip engine: the physics policy of the
// step kernels (exact for plain FP32 / FP64, fast for the 16-bit forms), its packed twin, the
// arithmetic of the moment pass, the per-launch constants, and the host equilibrium.
#pragma once

#include "collide.h"
#include "lbm_device.cuh"
#include "step_kernel.cuh"

namespace lbm_b200 {

template <class ST>
struct Form;
template <>
struct Form<float> {
  using A = ExactF32;
  using Phys = ExactPhys<ExactF32>;
  using PackedPhys = ExactPhysF32x2;
  static Phys::Consts consts(double tau, double fx, double fy) {
    return make_collide_consts<float>(float(tau), float(fx), float(fy));
  }
};
template <>
struct Form<double> {
  using A = ExactF64;
  using Phys = ExactPhys<ExactF64>;
  using PackedPhys = Phys;
  static Phys::Consts consts(double tau, double fx, double fy) {
    return make_collide_consts<double>(tau, fx, fy);
  }
};
template <>
struct Form<__half> {
  using A = ExactF32;  // moment pass
  using Phys = FastPhys;
  using PackedPhys = Phys;  // already packed
  static Phys::Consts consts(double tau, double fx, double fy) {
    return make_fast_consts(float(tau), float(fx), float(fy), kStoreScale16);
  }
};
template <>
struct Form<__nv_bfloat16> {
  using A = ExactF32;
  using Phys = FastPhys;
  using PackedPhys = Phys;  // already packed
  static Phys::Consts consts(double tau, double fx, double fy) {
    return make_fast_consts(float(tau), float(fx), float(fy), kStoreScale16);
  }
};

inline constexpr int kCx[kQ] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
inline constexpr int kCy[kQ] = {0, 0, 1, 0, -1, 1, 1, -1, -1};

// Shifted equilibrium of (rho0, ux0, uy0) in T, the reference's expressions and order
// (src/common/boundary.hpp:26-34, src/common/d2q9.hpp:40-42).
template <class T>
inline Eq9<T> host_equilibrium(T rho0, T ux0, T uy0) {
  Eq9<T> e{};
  const T usq = ux0 * ux0 + uy0 * uy0;
  const T drho0 = rho0 - T(1);
  for (int i = 0; i < kQ; ++i) {
    const T cu = kCx[i] * ux0 + kCy[i] * uy0;
    e.v[i] = weight<T>(i) * (drho0 + rho0 * (T(3) * cu + T(4.5) * cu * cu - T(1.5) * usq));
  }
  return e;
}

}  // namespace lbm_b200
