// D2Q9 lattice helpers and the BGK + Guo collision of one cell, shared by every kernel of the
// library. Plain C++17 with an LBM_HD annotation so that the same source also compiles for the
// host (tests/cpp/collide_algebra_test.cpp checks its algebra there against the oracle).
//
// Conventions (reference src/common/d2q9.hpp:14-50):
//   direction order 0: rest, 1: +x, 2: +y, 3: -x, 4: -y, 5: (+,+), 6: (-,+), 7: (-,-), 8: (+,-);
//   populations are stored shifted, g_i = f_i - w_i;
//   g_eq_i = w_i [drho + rho (3 cu + 4.5 cu^2 - 1.5 |u|^2)],
//   guo_i  = w_i [3 ((c_i - u).F) + 9 (c_i.u)(c_i.F)],
//   g_post = g - omega (g - g_eq) + (1 - omega/2) guo.
#pragma once

#if defined(__CUDACC__)
#define LBM_HD __host__ __device__ __forceinline__
#else
#define LBM_HD inline
#endif

namespace lbm_b200 {

constexpr int kQ = 9;

LBM_HD constexpr int dir_cx(int i) { return (i == 1 || i == 5 || i == 8) ? 1 : ((i == 3 || i == 6 || i == 7) ? -1 : 0); }
LBM_HD constexpr int dir_cy(int i) { return (i == 2 || i == 5 || i == 6) ? 1 : ((i == 4 || i == 7 || i == 8) ? -1 : 0); }
LBM_HD constexpr int dir_opp(int i) { return i == 0 ? 0 : (i <= 4 ? ((i + 1) % 4) + 1 : ((i - 5 + 2) % 4) + 5); }

static_assert(dir_opp(1) == 3 && dir_opp(2) == 4 && dir_opp(3) == 1 && dir_opp(4) == 2, "opp");
static_assert(dir_opp(5) == 7 && dir_opp(6) == 8 && dir_opp(7) == 5 && dir_opp(8) == 6, "opp");

// Weights rounded in T exactly as the reference's `real(4) / 9`, `real(1) / 9`, `real(1) / 36`.
template <class T>
LBM_HD constexpr T weight(int i) {
  return i == 0 ? T(4) / T(9) : (i <= 4 ? T(1) / T(9) : T(1) / T(36));
}

// Per-launch constants of the exact collision, computed on the host in the solver precision T
// with the reference's expressions (src/v3_cuda_opt/solver_v3.cu:252-253 and d2q9.hpp:46-50).
template <class T>
struct CollideConsts {
  T omega;            // real(1) / tau
  T force_prefactor;  // real(1) - real(0.5) * omega
  T fx, fy;           // body force
  T hfx, hfy;         // real(0.5) * fx, real(0.5) * fy  (Guo half-force velocity shift)
  T cf_x, cf_y;       // c.F of directions 1 (= fx) and 2 (= fy)
  T cf_p, cf_q;       // c.F of directions 5 (fx + fy) and 6 ((-fx) + fy)
};

template <class T>
inline CollideConsts<T> make_collide_consts(T tau, T fx, T fy) {
  CollideConsts<T> c;
  c.omega = T(1) / tau;
  c.force_prefactor = T(1) - T(0.5) * c.omega;
  c.fx = fx;
  c.fy = fy;
  c.hfx = T(0.5) * fx;
  c.hfy = T(0.5) * fy;
  c.cf_x = fx;
  c.cf_y = fy;
  c.cf_p = fx + fy;
  c.cf_q = fy - fx;
  return c;
}

// Bit-exact collision of one cell (A: arithmetic policy with add/sub/mul/div of type A::T,
// each one IEEE round-to-nearest operation that is never fused).
//
// The result equals the reference's v0 collision (src/v0_cpu/solver_v0.cpp:86-99,127-143)
// value for value on every finite state. It evaluates the same IEEE operations on the same
// operands and skips only those whose result is known exactly:
//   * products by the lattice integers c_i in {-1, 0, 1}: 1*a = a and (-1)*a = -a exactly, and a
//     0*a term adds a zero, which leaves a non-zero sum unchanged;
//   * opposite directions share values: RN(-a) = -RN(a), so cu_opp = -cu, 3 cu_opp = -(3 cu),
//     (4.5 cu_opp) cu_opp = (4.5 cu) cu, (9 cu_opp) cf_opp = (9 cu) cf, and each such value is
//     computed once;
//   * (0 - u) f = -(u f) and a + (-b) = a - b are the same IEEE operation.
// Only the sign of an exact zero can differ from v0 (numerically equal: the reference's tests
// compare with `!=`). A state holding inf or NaN has diverged; results then differ from v0 only
// in which non-finite value they hold.
template <class A>
LBM_HD void collide_exact(const typename A::T (&g)[kQ], const CollideConsts<typename A::T>& k,
                          typename A::T (&out)[kQ]) {
  using T = typename A::T;
  using S = typename A::S;
  // Moments, sequential over i = 0..8 as in v0 (zero-coefficient terms dropped).
  T m0 = g[0];
  m0 = A::add(m0, g[1]);
  m0 = A::add(m0, g[2]);
  m0 = A::add(m0, g[3]);
  m0 = A::add(m0, g[4]);
  m0 = A::add(m0, g[5]);
  m0 = A::add(m0, g[6]);
  m0 = A::add(m0, g[7]);
  m0 = A::add(m0, g[8]);
  T mx = A::sub(g[1], g[3]);
  mx = A::add(mx, g[5]);
  mx = A::sub(mx, g[6]);
  mx = A::sub(mx, g[7]);
  mx = A::add(mx, g[8]);
  T my = A::sub(g[2], g[4]);
  my = A::add(my, g[5]);
  my = A::add(my, g[6]);
  my = A::sub(my, g[7]);
  my = A::sub(my, g[8]);

  const T drho = m0;
  const T rho = A::add(A::k(S(1)), drho);
  const T ux = A::div(A::add(mx, k.hfx), rho);
  const T uy = A::div(A::add(my, k.hfy), rho);
  const T usq = A::add(A::mul(ux, ux), A::mul(uy, uy));
  const T s15 = A::mul(A::k(S(1.5)), usq);

  // Distinct c.u values: a (dir 1), b (dir 2), p (dir 5), q (dir 6); the others are negations.
  const T a = ux, b = uy;
  const T p = A::add(ux, uy);
  const T q = A::sub(uy, ux);
  const T three = A::k(S(3)), four5 = A::k(S(4.5)), nine = A::k(S(9));
  const T a3 = A::mul(three, a), b3 = A::mul(three, b), p3 = A::mul(three, p), q3 = A::mul(three, q);
  const T ka = A::mul(A::mul(four5, a), a);
  const T kb = A::mul(A::mul(four5, b), b);
  const T kp = A::mul(A::mul(four5, p), p);
  const T kq = A::mul(A::mul(four5, q), q);
  // 3 cu + 4.5 cu^2 - 1.5 usq per direction (direction 0: -1.5 usq).
  T bracket[kQ];
  bracket[1] = A::sub(A::add(a3, ka), s15);
  bracket[3] = A::sub(A::sub(ka, a3), s15);
  bracket[2] = A::sub(A::add(b3, kb), s15);
  bracket[4] = A::sub(A::sub(kb, b3), s15);
  bracket[5] = A::sub(A::add(p3, kp), s15);
  bracket[7] = A::sub(A::sub(kp, p3), s15);
  bracket[6] = A::sub(A::add(q3, kq), s15);
  bracket[8] = A::sub(A::sub(kq, q3), s15);

  T geq[kQ];
  geq[0] = A::mul(A::k(weight<S>(0)), A::sub(drho, A::mul(rho, s15)));
#if defined(__CUDACC__)
#pragma unroll
#endif
  for (int i = 1; i < kQ; ++i) geq[i] = A::mul(A::k(weight<S>(i)), A::add(drho, A::mul(rho, bracket[i])));

  // Guo source: t_i = (cx_i - ux) fx + (cy_i - uy) fy from six products, P_i = (9 cu_i) cf_i.
  const T axp = A::mul(A::sub(A::k(S(1)), ux), k.fx);
  const T axm = A::mul(A::sub(A::k(S(-1)), ux), k.fx);
  const T ax0 = A::neg(A::mul(ux, k.fx));
  const T ayp = A::mul(A::sub(A::k(S(1)), uy), k.fy);
  const T aym = A::mul(A::sub(A::k(S(-1)), uy), k.fy);
  const T ay0 = A::neg(A::mul(uy, k.fy));
  T t[kQ];
  t[0] = A::add(ax0, ay0);
  t[1] = A::add(axp, ay0);
  t[2] = A::add(ax0, ayp);
  t[3] = A::add(axm, ay0);
  t[4] = A::add(ax0, aym);
  t[5] = A::add(axp, ayp);
  t[6] = A::add(axm, ayp);
  t[7] = A::add(axm, aym);
  t[8] = A::add(axp, aym);
  const T pa = A::mul(A::mul(nine, a), k.cf_x);
  const T pb = A::mul(A::mul(nine, b), k.cf_y);
  const T pp = A::mul(A::mul(nine, p), k.cf_p);
  const T pq = A::mul(A::mul(nine, q), k.cf_q);
  T guo[kQ];
  guo[0] = A::mul(A::k(weight<S>(0)), A::mul(three, t[0]));
  guo[1] = A::mul(A::k(weight<S>(1)), A::add(A::mul(three, t[1]), pa));
  guo[3] = A::mul(A::k(weight<S>(3)), A::add(A::mul(three, t[3]), pa));
  guo[2] = A::mul(A::k(weight<S>(2)), A::add(A::mul(three, t[2]), pb));
  guo[4] = A::mul(A::k(weight<S>(4)), A::add(A::mul(three, t[4]), pb));
  guo[5] = A::mul(A::k(weight<S>(5)), A::add(A::mul(three, t[5]), pp));
  guo[7] = A::mul(A::k(weight<S>(7)), A::add(A::mul(three, t[7]), pp));
  guo[6] = A::mul(A::k(weight<S>(6)), A::add(A::mul(three, t[6]), pq));
  guo[8] = A::mul(A::k(weight<S>(8)), A::add(A::mul(three, t[8]), pq));

#if defined(__CUDACC__)
#pragma unroll
#endif
  for (int i = 0; i < kQ; ++i)
    out[i] = A::add(A::sub(g[i], A::mul(k.omega, A::sub(g[i], geq[i]))),
                    A::mul(k.force_prefactor, guo[i]));
}

// Moments of the reference's macroscopic() for one cell (src/v0_cpu/solver_v0.cpp:26-39,
// 111-123): rho = 1 + sum g, u = (sum c g + F/2) / rho, same operation order as collide_exact.
template <class A>
LBM_HD void moments_exact(const typename A::T (&g)[kQ], typename A::T hfx, typename A::T hfy,
                          typename A::T& rho, typename A::T& ux, typename A::T& uy) {
  using T = typename A::T;
  using S = typename A::S;
  T m0 = g[0];
#if defined(__CUDACC__)
#pragma unroll
#endif
  for (int i = 1; i < kQ; ++i) m0 = A::add(m0, g[i]);
  T mx = A::sub(g[1], g[3]);
  mx = A::add(mx, g[5]);
  mx = A::sub(mx, g[6]);
  mx = A::sub(mx, g[7]);
  mx = A::add(mx, g[8]);
  T my = A::sub(g[2], g[4]);
  my = A::add(my, g[5]);
  my = A::add(my, g[6]);
  my = A::sub(my, g[7]);
  my = A::sub(my, g[8]);
  rho = A::add(A::k(S(1)), m0);
  ux = A::div(A::add(mx, hfx), rho);
  uy = A::div(A::add(my, hfy), rho);
}

// ---------------------------------------------------------------------------------------------
// Fast FP32 collision of the 16-bit storage forms (not bit-exact; FMA, one reciprocal).
//
// omega g_eq_i + fp guo_i (fp = 1 - omega/2) regrouped per direction as
//   w_i [ A + 3 fp cf_i + cu_i (B + 9 fp cf_i + C cu_i) ],
//   A = omega drho - 1.5 omega rho |u|^2 - 3 fp (u.F),  B = 3 omega rho,  C = 4.5 omega rho,
// which is the same polynomial as the reference's geq/guo (d2q9.hpp:40-50) with
// (c_i - u).F = cf_i - u.F; out_i = (1 - omega) g_i + that.
// ---------------------------------------------------------------------------------------------
struct FastConsts {
  float omega, one_minus_omega;
  float hfx, hfy;      // F / 2
  float fp3fx, fp3fy;  // 3 fp F
  float k3[kQ];        // 3 fp cf_i
  float k9[kQ];        // 9 fp cf_i
};

inline FastConsts make_fast_consts(float tau, float fx, float fy) {
  FastConsts c{};
  c.omega = 1.0f / tau;
  c.one_minus_omega = 1.0f - c.omega;
  const float fp = 1.0f - 0.5f * c.omega;
  c.hfx = 0.5f * fx;
  c.hfy = 0.5f * fy;
  c.fp3fx = 3.0f * fp * fx;
  c.fp3fy = 3.0f * fp * fy;
  for (int i = 0; i < kQ; ++i) {
    const float cf = static_cast<float>(dir_cx(i)) * fx + static_cast<float>(dir_cy(i)) * fy;
    c.k3[i] = 3.0f * fp * cf;
    c.k9[i] = 9.0f * fp * cf;
  }
  return c;
}

// Scalar arithmetic of the fast collision (FMA allowed, one reciprocal).
struct FastF32 {
  using T = float;
  static LBM_HD float k(float v) { return v; }
  static LBM_HD float neg(float a) { return -a; }
  static LBM_HD float add(float a, float b) { return a + b; }
  static LBM_HD float sub(float a, float b) { return a - b; }
  static LBM_HD float mul(float a, float b) { return a * b; }
  static LBM_HD float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return a * b + c;
#endif
  }
  static LBM_HD float rcp(float a) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(a);
#else
    return 1.0f / a;
#endif
  }
};

template <class P>
LBM_HD void collide_fast_t(const typename P::T (&g)[kQ], const FastConsts& kc,
                           typename P::T (&out)[kQ]) {
  using T = typename P::T;
  const T m0 = P::add(P::add(P::add(P::add(g[0], g[1]), P::add(g[2], g[3])),
                             P::add(P::add(g[4], g[5]), P::add(g[6], g[7]))), g[8]);
  const T mx = P::add(P::add(P::sub(g[1], g[3]), P::sub(g[5], g[6])), P::sub(g[8], g[7]));
  const T my = P::sub(P::add(P::sub(g[2], g[4]), P::add(g[5], g[6])), P::add(g[7], g[8]));
  const T rho = P::add(P::k(1.0f), m0);
  const T inv = P::rcp(rho);
  const T ux = P::mul(P::add(mx, P::k(kc.hfx)), inv);
  const T uy = P::mul(P::add(my, P::k(kc.hfy)), inv);
  const T usq = P::fma(ux, ux, P::mul(uy, uy));
  const T orho = P::mul(P::k(kc.omega), rho);
  const T uf = P::fma(P::k(kc.fp3fx), ux, P::mul(P::k(kc.fp3fy), uy));
  const T a = P::fma(P::k(kc.omega), m0, P::fma(P::mul(P::k(-1.5f), orho), usq, P::neg(uf)));
  const T b = P::mul(P::k(3.0f), orho), c = P::mul(P::k(4.5f), orho);
  const T p = P::add(ux, uy), q = P::sub(uy, ux);
  const T cu[kQ] = {P::k(0.0f), ux, uy, P::neg(ux), P::neg(uy), p, q, P::neg(p), P::neg(q)};
  const T om1 = P::k(kc.one_minus_omega);
  out[0] = P::fma(P::k(weight<float>(0)), a, P::mul(om1, g[0]));
#if defined(__CUDACC__)
#pragma unroll
#endif
  for (int i = 1; i < kQ; ++i) {
    const T t = P::fma(P::fma(c, cu[i], P::add(b, P::k(kc.k9[i]))), cu[i], P::add(a, P::k(kc.k3[i])));
    out[i] = P::fma(P::k(weight<float>(i)), t, P::mul(om1, g[i]));
  }
}

LBM_HD void collide_fast(const float (&g)[kQ], const FastConsts& k, float (&out)[kQ]) {
  collide_fast_t<FastF32>(g, k, out);
}

// Host arithmetic policy (plain IEEE operators; compile with -ffp-contract=off).
template <class TT>
struct HostArith {
  using T = TT;
  using S = TT;
  static inline T k(S v) { return v; }
  static inline T neg(T a) { return -a; }
  static inline T add(T a, T b) { return a + b; }
  static inline T sub(T a, T b) { return a - b; }
  static inline T mul(T a, T b) { return a * b; }
  static inline T div(T a, T b) { return a / b; }
};

}  // namespace lbm_b200
