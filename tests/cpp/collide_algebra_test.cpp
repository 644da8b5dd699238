// Host check of the simplified exact collision (csrc/collide.h) against the literal collision
// of the reference's v0 (src/v0_cpu/solver_v0.cpp:86-99,127-143, src/common/d2q9.hpp:40-50),
// on random states, in float and double, with and without the adjoint form's Brinkman drag
// (collide_exact_drag). Exit status 0 when every output value is equal.
// Compile with -ffp-contract=off.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "collide.h"

namespace {

constexpr int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
constexpr int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};

template <class T>
void literal(const T* g, T omega, T fp, T fx, T fy, T* out) {
  T m0 = 0, mx = 0, my = 0;
  for (int i = 0; i < 9; ++i) {
    m0 += g[i];
    mx += CX[i] * g[i];
    my += CY[i] * g[i];
  }
  const T drho = m0, rho = T(1) + drho;
  const T ux = (mx + T(0.5) * fx) / rho, uy = (my + T(0.5) * fy) / rho;
  const T usq = ux * ux + uy * uy;
  for (int i = 0; i < 9; ++i) {
    const T wi = lbm_b200::weight<T>(i);
    const T cu = CX[i] * ux + CY[i] * uy;
    const T geq = wi * (drho + rho * (T(3) * cu + T(4.5) * cu * cu - T(1.5) * usq));
    const T cxi = T(CX[i]), cyi = T(CY[i]);
    const T cu2 = cxi * ux + cyi * uy, cf = cxi * fx + cyi * fy;
    const T guo = wi * (T(3) * ((cxi - ux) * fx + (cyi - uy) * fy) + T(9) * cu2 * cf);
    out[i] = g[i] - omega * (g[i] - geq) + fp * guo;
  }
}

// The literal collision with a Brinkman drag (F_tot = F - (alpha rho) u, u = (m + F/2) / d,
// d = rho (1 + 0.5 alpha)), the forward model of the adjoint form.
template <class T>
T literal_drag(const T* g, T omega, T fp, T fx, T fy, T alpha, T* out) {
  T m0 = 0, mx = 0, my = 0;
  for (int i = 0; i < 9; ++i) {
    m0 += g[i];
    mx += CX[i] * g[i];
    my += CY[i] * g[i];
  }
  const T drho = m0, rho = T(1) + drho;
  const T kf = T(1) + T(0.5) * alpha, d = rho * kf;
  const T ux = (mx + T(0.5) * fx) / d, uy = (my + T(0.5) * fy) / d;
  const T Fx = fx - (alpha * rho) * ux, Fy = fy - (alpha * rho) * uy;
  const T usq = ux * ux + uy * uy;
  for (int i = 0; i < 9; ++i) {
    const T wi = lbm_b200::weight<T>(i);
    const T cxi = T(CX[i]), cyi = T(CY[i]);
    const T cu = cxi * ux + cyi * uy;
    const T geq = wi * (drho + rho * (T(3) * cu + T(4.5) * cu * cu - T(1.5) * usq));
    const T cf = cxi * Fx + cyi * Fy;
    const T guo = wi * (T(3) * ((cxi - ux) * Fx + (cyi - uy) * Fy) + T(9) * cu * cf);
    out[i] = g[i] - omega * (g[i] - geq) + fp * guo;
  }
  return ux;
}

template <class T>
long check(long trials, unsigned seed) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  long bad = 0;
  for (long t = 0; t < trials; ++t) {
    const double scale = std::pow(10.0, -1.0 - 5.0 * (0.5 + 0.5 * u(rng)));  // 1e-1 .. 1e-6
    T g[9];
    for (int i = 0; i < 9; ++i) g[i] = T(scale * u(rng) * lbm_b200::weight<double>(i) * 9.0);
    if (t % 7 == 0) g[t % 9] = T(0);
    const T tau = T(0.5 + 1e-3 + 1.5 * (0.5 + 0.5 * u(rng)));
    T fx = T(1e-4 * u(rng)), fy = T(1e-4 * u(rng));
    if (t % 5 == 0) fy = T(0);
    if (t % 11 == 0) fx = T(0);
    const auto k = lbm_b200::make_collide_consts<T>(tau, fx, fy);
    T a[9], b[9];
    literal<T>(g, k.omega, k.force_prefactor, fx, fy, a);
    lbm_b200::collide_exact<lbm_b200::HostArith<T>>(g, k, b);
    for (int i = 0; i < 9; ++i)
      if (!(a[i] == b[i])) {
        if (bad < 5)
          std::printf("mismatch trial %ld dir %d: %.17g vs %.17g\n", t, i, (double)a[i], (double)b[i]);
        ++bad;
      }
    // Brinkman drag (alpha in [0, 0.1], zero for some states)
    const T alpha = t % 3 == 0 ? T(0) : T(0.05 + 0.05 * u(rng));
    const T ua = literal_drag<T>(g, k.omega, k.force_prefactor, fx, fy, alpha, a);
    const T ub = lbm_b200::collide_exact_drag<lbm_b200::HostArith<T>>(g, k, alpha, b);
    if (!(ua == ub)) ++bad;
    for (int i = 0; i < 9; ++i)
      if (!(a[i] == b[i])) {
        if (bad < 5)
          std::printf("drag mismatch trial %ld dir %d: %.17g vs %.17g\n", t, i, (double)a[i], (double)b[i]);
        ++bad;
      }
    // moments
    T r1, u1, v1;
    lbm_b200::moments_exact<lbm_b200::HostArith<T>>(g, k.hfx, k.hfy, r1, u1, v1);
    T m0 = 0, mx = 0, my = 0;
    for (int i = 0; i < 9; ++i) { m0 += g[i]; mx += CX[i] * g[i]; my += CY[i] * g[i]; }
    const T rho = T(1) + m0;
    if (!(r1 == rho && u1 == (mx + T(0.5) * fx) / rho && v1 == (my + T(0.5) * fy) / rho)) ++bad;
  }
  return bad;
}

// collide_fast (FP32, regrouped, FMA) against the literal collision in double: relative error
// of each output with respect to the largest |output| of the cell.
double check_fast(long trials) {
  std::mt19937_64 rng(3);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  double worst = 0.0;
  for (long t = 0; t < trials; ++t) {
    float g[9];
    double gd[9];
    for (int i = 0; i < 9; ++i) {
      g[i] = float(0.05 * u(rng) * lbm_b200::weight<double>(i) * 9.0);
      gd[i] = g[i];
    }
    const float tau = float(0.51 + 1.4 * (0.5 + 0.5 * u(rng)));
    const float fx = float(1e-4 * u(rng)), fy = float(1e-4 * u(rng));
    // The fast collision takes and returns values scaled by the 16-bit storage scale.
    const float scale = 32768.0f;
    const auto kf = lbm_b200::make_fast_consts(tau, fx, fy, scale);
    const double omega = 1.0 / double(tau);
    double a[9];
    literal<double>(gd, omega, 1.0 - 0.5 * omega, double(fx), double(fy), a);
    float gs[9], b[9];
    for (int i = 0; i < 9; ++i) gs[i] = g[i] * scale;
    lbm_b200::collide_fast(gs, kf, b);
    double amax = 0.0;
    for (int i = 0; i < 9; ++i) amax = std::fmax(amax, std::fabs(a[i]));
    for (int i = 0; i < 9; ++i) worst = std::fmax(worst, std::fabs(a[i] - double(b[i]) / scale) / amax);
  }
  return worst;
}

}  // namespace

int main(int argc, char** argv) {
  const long trials = argc > 1 ? std::atol(argv[1]) : 100000;
  const long bf = check<float>(trials, 1), bd = check<double>(trials, 2);
  std::printf("collide_exact vs literal v0: float %ld / double %ld mismatching values in %ld states\n",
              bf, bd, trials);
  const double fast = check_fast(trials / 4);
  std::printf("collide_fast vs literal (double): worst relative error %.3e\n", fast);
  return (bf == 0 && bd == 0 && fast < 2e-6) ? 0 : 1;
}
