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
// Moments m0 = sum g, mx = sum c_x g, my = sum c_y g, sequential over i = 0..8 as in v0
// (zero-coefficient terms dropped).
template <class A>
LBM_HD void moments_seq(const typename A::T (&g)[kQ], typename A::T& m0, typename A::T& mx,
                        typename A::T& my) {
  m0 = g[0];
  m0 = A::add(m0, g[1]);
  m0 = A::add(m0, g[2]);
  m0 = A::add(m0, g[3]);
  m0 = A::add(m0, g[4]);
  m0 = A::add(m0, g[5]);
  m0 = A::add(m0, g[6]);
  m0 = A::add(m0, g[7]);
  m0 = A::add(m0, g[8]);
  mx = A::sub(g[1], g[3]);
  mx = A::add(mx, g[5]);
  mx = A::sub(mx, g[6]);
  mx = A::sub(mx, g[7]);
  mx = A::add(mx, g[8]);
  my = A::sub(g[2], g[4]);
  my = A::add(my, g[5]);
  my = A::add(my, g[6]);
  my = A::sub(my, g[7]);
  my = A::sub(my, g[8]);
}

// Equilibrium, Guo source and BGK relaxation of one cell given its density, velocity and the
// force acting on it (fx, fy; cf_p = fx + fy and cf_q = fy - fx, the c.F of directions 5 and 6).
template <class A>
LBM_HD void collide_exact_post(const typename A::T (&g)[kQ], typename A::T omega,
                               typename A::T force_prefactor, typename A::T drho, typename A::T rho,
                               typename A::T ux, typename A::T uy, typename A::T fx, typename A::T fy,
                               typename A::T cf_p, typename A::T cf_q, typename A::T (&out)[kQ]) {
  using T = typename A::T;
  using S = typename A::S;
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
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int i = 1; i < kQ; ++i) geq[i] = A::mul(A::k(weight<S>(i)), A::add(drho, A::mul(rho, bracket[i])));

  // Guo source: t_i = (cx_i - ux) fx + (cy_i - uy) fy from six products, P_i = (9 cu_i) cf_i.
  const T axp = A::mul(A::sub(A::k(S(1)), ux), fx);
  const T axm = A::mul(A::sub(A::k(S(-1)), ux), fx);
  const T ax0 = A::neg(A::mul(ux, fx));
  const T ayp = A::mul(A::sub(A::k(S(1)), uy), fy);
  const T aym = A::mul(A::sub(A::k(S(-1)), uy), fy);
  const T ay0 = A::neg(A::mul(uy, fy));
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
  const T pa = A::mul(A::mul(nine, a), fx);
  const T pb = A::mul(A::mul(nine, b), fy);
  const T pp = A::mul(A::mul(nine, p), cf_p);
  const T pq = A::mul(A::mul(nine, q), cf_q);
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

#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int i = 0; i < kQ; ++i)
    out[i] = A::add(A::sub(g[i], A::mul(omega, A::sub(g[i], geq[i]))), A::mul(force_prefactor, guo[i]));
}

template <class A>
LBM_HD void collide_exact(const typename A::T (&g)[kQ], const CollideConsts<typename A::T>& k,
                          typename A::T (&out)[kQ]) {
  using T = typename A::T;
  using S = typename A::S;
  T m0, mx, my;
  moments_seq<A>(g, m0, mx, my);
  const T drho = m0;
  const T rho = A::add(A::k(S(1)), drho);
  const T ux = A::div(A::add(mx, k.hfx), rho);
  const T uy = A::div(A::add(my, k.hfy), rho);
  collide_exact_post<A>(g, k.omega, k.force_prefactor, drho, rho, ux, uy, k.cf_x, k.cf_y, k.cf_p,
                        k.cf_q, out);
}

// The same collision with a Brinkman drag: the force on the cell is F_tot = F - alpha rho u and
// the Guo velocity u = (m + F/2) / (rho (1 + alpha/2)) solves rho u = m + F_tot / 2; the
// reference's literal order of these extra operations is kept (kf = 1 + 0.5 alpha, d = rho kf,
// F_tot = F - (alpha rho) u), so alpha = 0 gives collide_exact's values (kf = 1, d = rho,
// F_tot = F). Returns u_x.
template <class A>
LBM_HD typename A::T collide_exact_drag(const typename A::T (&g)[kQ], const CollideConsts<typename A::T>& k,
                                        typename A::T alpha, typename A::T (&out)[kQ]) {
  using T = typename A::T;
  using S = typename A::S;
  T m0, mx, my;
  moments_seq<A>(g, m0, mx, my);
  const T drho = m0;
  const T rho = A::add(A::k(S(1)), drho);
  const T kf = A::add(A::k(S(1)), A::mul(A::k(S(0.5)), alpha));
  const T d = A::mul(rho, kf);
  const T ux = A::div(A::add(mx, k.hfx), d);
  const T uy = A::div(A::add(my, k.hfy), d);
  const T ar = A::mul(alpha, rho);
  const T fx = A::sub(k.fx, A::mul(ar, ux));
  const T fy = A::sub(k.fy, A::mul(ar, uy));
  collide_exact_post<A>(g, k.omega, k.force_prefactor, drho, rho, ux, uy, fx, fy, A::add(fx, fy),
                        A::sub(fy, fx), out);
  return ux;
}

// Moments of the reference's macroscopic() for one cell (src/v0_cpu/solver_v0.cpp:26-39,
// 111-123): rho = 1 + sum g, u = (sum c g + F/2) / rho, same operation order as collide_exact.
template <class A>
LBM_HD void moments_exact(const typename A::T (&g)[kQ], typename A::T hfx, typename A::T hfy,
                          typename A::T& rho, typename A::T& ux, typename A::T& uy) {
  using T = typename A::T;
  using S = typename A::S;
  T m0 = g[0];
#if defined(__CUDA_ARCH__)
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
// Works on scaled populations G_i = S g_i (S a power of two, the storage scale of every plane)
// and returns scaled results, so that no per-value rescaling is spent on loads and stores:
// power-of-two scaling commutes with rounding, m = sum G_i / S and u = (m_x' + S F_x / 2) *
// (1 / (S rho)) are the unscaled moments exactly, and S w_i folds into the per-direction
// constants. The post-collision value omega g_eq_i + fp guo_i (fp = 1 - omega/2) is the
// reference's geq/guo polynomial (d2q9.hpp:40-50) regrouped per pair of opposite directions
// (c_j = -c_i, so cu_j = -cu_i, cf_j = -cf_i, w_j = w_i):
//   S w_i t_i = E + N + O,  S w_j t_j = E + N - O,
//   E = S w (a + c cu^2),  N = S w 9 fp cf_i cu,  O = S w (b cu + 3 fp cf_i),
//   a = omega drho - 1.5 omega rho |u|^2 - 3 fp (u.F),  b = 3 omega rho,  c = 4.5 omega rho,
// using (c_i - u).F = cf_i - u.F; out_i = (1 - omega) G_i + S w_i t_i.
// ---------------------------------------------------------------------------------------------
struct FastConsts {
  float omega, one_minus_omega;
  float inv_scale;     // 1 / S
  float shfx, shfy;    // S F / 2
  float fp3fx, fp3fy;  // 3 fp F
  float w0, wax, wdg;  // S w_0, S w_axis, S w_diagonal
  float wk3[kQ];       // S w_i 3 fp cf_i
  float wk9[kQ];       // S w_i 9 fp cf_i
};

inline FastConsts make_fast_consts(float tau, float fx, float fy, float scale = 1.0f) {
  FastConsts c{};
  c.omega = 1.0f / tau;
  c.one_minus_omega = 1.0f - c.omega;
  const float fp = 1.0f - 0.5f * c.omega;
  c.inv_scale = 1.0f / scale;
  c.shfx = scale * (0.5f * fx);
  c.shfy = scale * (0.5f * fy);
  c.fp3fx = 3.0f * fp * fx;
  c.fp3fy = 3.0f * fp * fy;
  c.w0 = scale * weight<float>(0);
  c.wax = scale * weight<float>(1);
  c.wdg = scale * weight<float>(5);
  for (int i = 0; i < kQ; ++i) {
    const float cf = static_cast<float>(dir_cx(i)) * fx + static_cast<float>(dir_cy(i)) * fy;
    const float w = scale * weight<float>(i);
    c.wk3[i] = w * (3.0f * fp * cf);
    c.wk9[i] = w * (9.0f * fp * cf);
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

// Outputs of one pair of opposite directions i (cu) and j (-cu) of weight class (wa, wb, wc).
template <class P>
LBM_HD void fast_pair(const typename P::T (&g)[kQ], const FastConsts& kc, int i, int j,
                      typename P::T cu, typename P::T wa, typename P::T wb, typename P::T wc,
                      typename P::T om1, typename P::T (&out)[kQ]) {
  using T = typename P::T;
  const T e = P::fma(P::mul(wc, cu), cu, wa);
  const T o = P::fma(wb, cu, P::k(kc.wk3[i]));
  const T en = P::fma(P::k(kc.wk9[i]), cu, e);
  out[i] = P::fma(om1, g[i], P::add(en, o));
  out[j] = P::fma(om1, g[j], P::sub(en, o));
}

template <class P>
LBM_HD void collide_fast_t(const typename P::T (&g)[kQ], const FastConsts& kc,
                           typename P::T (&out)[kQ]) {
  using T = typename P::T;
  const T m0s = P::add(P::add(P::add(P::add(g[0], g[1]), P::add(g[2], g[3])),
                              P::add(P::add(g[4], g[5]), P::add(g[6], g[7]))), g[8]);
  const T mxs = P::add(P::add(P::sub(g[1], g[3]), P::sub(g[5], g[6])), P::sub(g[8], g[7]));
  const T mys = P::sub(P::add(P::sub(g[2], g[4]), P::add(g[5], g[6])), P::add(g[7], g[8]));
  const T m0 = P::mul(m0s, P::k(kc.inv_scale));
  const T rho = P::add(P::k(1.0f), m0);
  const T invs = P::mul(P::rcp(rho), P::k(kc.inv_scale));
  const T ux = P::mul(P::add(mxs, P::k(kc.shfx)), invs);
  const T uy = P::mul(P::add(mys, P::k(kc.shfy)), invs);
  const T usq = P::fma(ux, ux, P::mul(uy, uy));
  const T orho = P::mul(P::k(kc.omega), rho);
  const T uf = P::fma(P::k(kc.fp3fx), ux, P::mul(P::k(kc.fp3fy), uy));
  const T a = P::fma(P::k(kc.omega), m0, P::fma(P::mul(P::k(-1.5f), orho), usq, P::neg(uf)));
  const T b = P::mul(P::k(3.0f), orho), c = P::mul(P::k(4.5f), orho);
  const T om1 = P::k(kc.one_minus_omega);
  out[0] = P::fma(om1, g[0], P::mul(P::k(kc.w0), a));
  const T wa = P::mul(P::k(kc.wax), a), wb = P::mul(P::k(kc.wax), b), wc = P::mul(P::k(kc.wax), c);
  fast_pair<P>(g, kc, 1, 3, ux, wa, wb, wc, om1, out);
  fast_pair<P>(g, kc, 2, 4, uy, wa, wb, wc, om1, out);
  const T da = P::mul(P::k(kc.wdg), a), db = P::mul(P::k(kc.wdg), b), dc = P::mul(P::k(kc.wdg), c);
  fast_pair<P>(g, kc, 5, 7, P::add(ux, uy), da, db, dc, om1, out);
  fast_pair<P>(g, kc, 6, 8, P::sub(uy, ux), da, db, dc, om1, out);
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
