/*
 * Oracle body, instantiated once per floating-point type by lbm_oracle.c with
 *   REAL      float or double (the reference's compile-time `lbm::real`),
 *   FN(name)  name with the type suffix (_f32 or _f64).
 *
 * TEST INFRASTRUCTURE ONLY. This is a CPU restatement of the reference solver, used by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker. The
 * product (the CUDA library) never links, loads or calls it.
 *
 * Every floating-point expression below keeps the operand order of the reference, because the
 * GPU kernels must match it bit for bit. The file is compiled with -ffp-contract=off (no fused
 * multiply-add), as the reference's CPU build is (reference CMakeLists.txt:18-24).
 */

/* Weights w_i rounded in REAL, as `real(4) / 9` etc. (src/common/d2q9.hpp:26-27). */
static const REAL FN(W)[9] = {(REAL)4 / 9,  (REAL)1 / 9,  (REAL)1 / 9,  (REAL)1 / 9, (REAL)1 / 9,
                              (REAL)1 / 36, (REAL)1 / 36, (REAL)1 / 36, (REAL)1 / 36};

/* Shifted equilibrium g_eq = w [drho + rho (3 cu + 4.5 cu cu - 1.5 usq)]
 * (src/common/d2q9.hpp:40-42). Evaluation order: ((3*cu) + ((4.5*cu)*cu)) - (1.5*usq). */
static inline __attribute__((always_inline)) REAL FN(equilibrium_shifted)(REAL wi, REAL drho, REAL rho, REAL cu, REAL usq) {
  return wi * (drho + rho * ((REAL)3 * cu + (REAL)4.5 * cu * cu - (REAL)1.5 * usq));
}

/* Guo source without its (1 - omega/2) prefactor (src/common/d2q9.hpp:46-50):
 * w [3 ((cx - ux) fx + (cy - uy) fy) + 9 (c.u)(c.F)]. */
static inline __attribute__((always_inline)) REAL FN(guo_source)(REAL wi, REAL cxi, REAL cyi, REAL ux, REAL uy, REAL fx,
                                  REAL fy) {
  const REAL cu = cxi * ux + cyi * uy;
  const REAL cf = cxi * fx + cyi * fy;
  return wi * ((REAL)3 * ((cxi - ux) * fx + (cyi - uy) * fy) + (REAL)9 * cu * cf);
}

/* Inlet equilibrium of (rho0, ux0, uy0) (src/common/boundary.hpp:26-34). */
void FN(oracle_equilibrium_state)(REAL rho0, REAL ux0, REAL uy0, REAL* eq) {
  const REAL usq = ux0 * ux0 + uy0 * uy0;
  const REAL drho0 = rho0 - (REAL)1;
  for (int i = 0; i < 9; ++i) {
    const REAL cu = CX[i] * ux0 + CY[i] * uy0;
    eq[i] = FN(equilibrium_shifted)(FN(W)[i], drho0, rho0, cu, usq);
  }
}

/* Uniform equilibrium on every fluid cell, zero on solid cells, v0 layout s[(y*nx+x)*9+i]
 * (src/v0_cpu/solver_v0.cpp:41-51). */
void FN(oracle_init_equilibrium)(int nx, int ny, const uint8_t* solid, REAL rho0, REAL ux0,
                                 REAL uy0, REAL* s) {
  const REAL usq = ux0 * ux0 + uy0 * uy0;
  const REAL drho0 = rho0 - (REAL)1;
  const size_t n = (size_t)nx * ny;
  for (size_t c = 0; c < n; ++c)
    for (int i = 0; i < 9; ++i) {
      const REAL cu = CX[i] * ux0 + CY[i] * uy0;
      s[c * 9 + i] = solid[c] ? (REAL)0 : FN(equilibrium_shifted)(FN(W)[i], drho0, rho0, cu, usq);
    }
}

/* Moments of one cell of the post-streaming state, v0 order: sequential sums over i = 0..8,
 * zero-weight terms included (src/v0_cpu/solver_v0.cpp:26-39). */
static inline void FN(moments)(const REAL* gc, REAL fx, REAL fy, REAL* drho, REAL* ux, REAL* uy) {
  REAL m0 = 0, mx = 0, my = 0;
  for (int i = 0; i < 9; ++i) {
    m0 += gc[i];
    mx += CX[i] * gc[i];
    my += CY[i] * gc[i];
  }
  *drho = m0;
  const REAL rho = (REAL)1 + m0;
  *ux = (mx + (REAL)0.5 * fx) / rho;
  *uy = (my + (REAL)0.5 * fy) / rho;
}

/* One push step of v0 on the AoS post-streaming state (src/v0_cpu/solver_v0.cpp:63-105), with
 * the open-x inflow/outflow rules applied to the new buffer (src/common/boundary.hpp:37-48). */
static void FN(v0_step)(int nx, int ny, const uint8_t* solid, REAL tau, REAL fx, REAL fy,
                        int open_x, const REAL* eq_in, const REAL* g, REAL* g_new) {
  const REAL omega = (REAL)1 / tau;
  const REAL force_prefactor = (REAL)1 - (REAL)0.5 * omega;
  for (int y = 0; y < ny; ++y) {
    for (int x = 0; x < nx; ++x) {
      const size_t c = (size_t)y * nx + x;
      if (solid[c]) continue;
      REAL drho, ux, uy;
      FN(moments)(&g[c * 9], fx, fy, &drho, &ux, &uy);
      const REAL rho = (REAL)1 + drho;
      const REAL usq = ux * ux + uy * uy;
      for (int i = 0; i < 9; ++i) {
        const REAL cu = CX[i] * ux + CY[i] * uy;
        const REAL geq = FN(equilibrium_shifted)(FN(W)[i], drho, rho, cu, usq);
        const REAL g_post = g[c * 9 + i] - omega * (g[c * 9 + i] - geq) +
                            force_prefactor * FN(guo_source)(FN(W)[i], (REAL)CX[i], (REAL)CY[i],
                                                             ux, uy, fx, fy);
        int xn;
        if (open_x) {
          xn = x + CX[i];
          if (xn < 0 || xn >= nx) continue;
        } else {
          xn = (x + CX[i] + nx) % nx;
        }
        const int yn = (y + CY[i] + ny) % ny;
        const size_t cn = (size_t)yn * nx + xn;
        if (solid[cn])
          g_new[c * 9 + OPP[i]] = g_post;
        else
          g_new[cn * 9 + i] = g_post;
      }
    }
  }
  if (open_x) {
    for (int y = 0; y < ny; ++y) {
      const size_t row = (size_t)y * nx;
      if (!solid[row]) {
        g_new[row * 9 + 1] = eq_in[1];
        g_new[row * 9 + 5] = eq_in[5];
        g_new[row * 9 + 8] = eq_in[8];
      }
      const size_t out = row + nx - 1, prev = row + nx - 2;
      if (!solid[out]) {
        g_new[out * 9 + 3] = g_new[prev * 9 + 3];
        g_new[out * 9 + 6] = g_new[prev * 9 + 6];
        g_new[out * 9 + 7] = g_new[prev * 9 + 7];
      }
    }
  }
}

/* Runs `steps` v0 steps in place on s (v0 layout). Returns 0, or -1 on allocation failure. */
int FN(oracle_v0_run)(int nx, int ny, const uint8_t* solid, REAL tau, REAL fx, REAL fy,
                      int open_x, REAL u_in, REAL* s, int steps) {
  const size_t n = (size_t)nx * ny * 9;
  REAL* g_new = (REAL*)malloc(n * sizeof(REAL));
  if (!g_new) return -1;
  memcpy(g_new, s, n * sizeof(REAL)); /* solid slots are never written: keep them as in s */
  REAL eq_in[9] = {0};
  if (open_x) FN(oracle_equilibrium_state)((REAL)1, u_in, (REAL)0, eq_in);
  REAL* a = s;
  REAL* b = g_new;
  for (int k = 0; k < steps; ++k) {
    FN(v0_step)(nx, ny, solid, tau, fx, fy, open_x, eq_in, a, b);
    REAL* t = a;
    a = b;
    b = t;
  }
  if (a != s) memcpy(s, a, n * sizeof(REAL));
  free(g_new);
  return 0;
}

/* rho, ux, uy of the post-streaming state; solid cells give 0 (src/v0_cpu/solver_v0.cpp:111-123). */
void FN(oracle_macroscopic)(int nx, int ny, const uint8_t* solid, REAL fx, REAL fy, const REAL* s,
                            REAL* rho, REAL* ux, REAL* uy) {
  const size_t n = (size_t)nx * ny;
  for (size_t c = 0; c < n; ++c) {
    rho[c] = 0;
    ux[c] = 0;
    uy[c] = 0;
    if (solid[c]) continue;
    REAL drho;
    FN(moments)(&s[c * 9], fx, fy, &drho, &ux[c], &uy[c]);
    rho[c] = (REAL)1 + drho;
  }
}

/* Fluid-cell count plus the sum of every fluid population, accumulated in double in v0's order
 * (src/v0_cpu/solver_v0.cpp:125-135). */
double FN(oracle_total_mass)(int nx, int ny, const uint8_t* solid, const REAL* s) {
  double drho = 0.0;
  size_t fluid = 0;
  const size_t n = (size_t)nx * ny;
  for (size_t c = 0; c < n; ++c) {
    if (solid[c]) continue;
    ++fluid;
    for (int i = 0; i < 9; ++i) drho += s[c * 9 + i];
  }
  return (double)fluid + drho;
}

/* Post-streaming populations of fluid cell (x, y) gathered from the post-collision SoA state r
 * (plane stride n = nx*ny), with the open-x rules (src/common/boundary.hpp:53-70). */
static inline void FN(gather_pull)(const REAL* r, const uint8_t* solid, int nx, int ny, int x,
                                   int y, int open_x, const REAL* eq_in, REAL* out) {
  const size_t n = (size_t)nx * ny;
  for (int i = 0; i < 9; ++i) {
    if (open_x && x == 0 && CX[i] == 1) {
      out[i] = eq_in[i];
      continue;
    }
    int xc = x;
    if (open_x && x == nx - 1 && CX[i] == -1) xc = nx - 2;
    const size_t cc = (size_t)y * nx + xc;
    const int xs = (xc - CX[i] + nx) % nx;
    const int ys = (y - CY[i] + ny) % ny;
    const size_t src = (size_t)ys * nx + xs;
    out[i] = solid[src] ? r[OPP[i] * n + cc] : r[i * n + src];
  }
}

/* Post-collision SoA state r -> post-streaming v0-layout state s (solid cells 0)
 * (src/v3_cuda_opt/solver_v3.cu:300-320 with the pull gather). */
void FN(oracle_r_to_s)(int nx, int ny, const uint8_t* solid, int open_x, REAL u_in, const REAL* r,
                       REAL* s) {
  REAL eq_in[9] = {0};
  if (open_x) FN(oracle_equilibrium_state)((REAL)1, u_in, (REAL)0, eq_in);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const size_t c = (size_t)y * nx + x;
      if (solid[c]) {
        for (int i = 0; i < 9; ++i) s[c * 9 + i] = 0;
        continue;
      }
      FN(gather_pull)(r, solid, nx, ny, x, y, open_x, eq_in, &s[c * 9]);
    }
}

/* Preimage by streaming: v0-layout s -> SoA r with stream(r) = s on every fluid slot. Slot (c, i)
 * streams to (c + e_i, i), or bounces to (c, opp i) when c + e_i is solid; in an open domain a slot
 * leaving through x = 0 or x = nx - 1 is never read and keeps s[c][i]. Generalises the uniform
 * preimage of src/v3_cuda_opt/solver_v3.cu:194-226 to any state. */
void FN(oracle_s_to_r)(int nx, int ny, const uint8_t* solid, int open_x, const REAL* s, REAL* r) {
  const size_t n = (size_t)nx * ny;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const size_t c = (size_t)y * nx + x;
      for (int i = 0; i < 9; ++i) {
        REAL v;
        if (solid[c]) {
          v = 0;
        } else {
          const int leaves = open_x && (x + CX[i] < 0 || x + CX[i] >= nx);
          const int xn = (x + CX[i] + nx) % nx;
          const int yn = (y + CY[i] + ny) % ny;
          const size_t cn = (size_t)yn * nx + xn;
          if (leaves)
            v = s[c * 9 + i];
          else if (solid[cn])
            v = s[c * 9 + OPP[i]];
          else
            v = s[cn * 9 + i];
        }
        r[i * n + c] = v;
      }
    }
}

/* BGK + Guo collision of gathered populations gin, v0 operation order; writes 9 outputs with
 * stride n (SoA) starting at out. */
static inline __attribute__((always_inline)) void FN(collide_store)(const REAL* gin, REAL omega, REAL force_prefactor, REAL fx,
                                     REAL fy, REAL* out, size_t n) {
  REAL m0 = 0, mx = 0, my = 0;
#pragma GCC unroll 9
  for (int i = 0; i < 9; ++i) {
    m0 += gin[i];
    mx += CX[i] * gin[i];
    my += CY[i] * gin[i];
  }
  const REAL drho = m0;
  const REAL rho = (REAL)1 + drho;
  const REAL ux = (mx + (REAL)0.5 * fx) / rho;
  const REAL uy = (my + (REAL)0.5 * fy) / rho;
  const REAL usq = ux * ux + uy * uy;
#pragma GCC unroll 9
  for (int i = 0; i < 9; ++i) {
    const REAL cu = CX[i] * ux + CY[i] * uy;
    const REAL geq = FN(equilibrium_shifted)(FN(W)[i], drho, rho, cu, usq);
    out[i * n] = gin[i] - omega * (gin[i] - geq) +
                 force_prefactor *
                     FN(guo_source)(FN(W)[i], (REAL)CX[i], (REAL)CY[i], ux, uy, fx, fy);
  }
}

/* Pull update of interior cell c (column x, 0 < x < nx - 1): both candidate loads are done
 * unconditionally and selected by the source mask, and the collision is computed for solid
 * cells too and stored as 0, so that the loop over x has no branch and vectorises (the
 * structure of src/v1_omp/solver_v1.cpp:18-67). */
static inline __attribute__((always_inline)) void FN(pull_cell)(
    const REAL* restrict r, REAL* restrict rn, const uint8_t* restrict solid, size_t n,
    const size_t* row, int x, REAL omega, REAL force_prefactor, REAL fx, REAL fy) {
  const size_t c = row[1] + (size_t)x;
  REAL gin[9];
#pragma GCC unroll 9
  for (int i = 0; i < 9; ++i) {
    const size_t src = row[1 - CY[i]] + (size_t)(x - CX[i]);
    const REAL streamed = r[i * n + src];
    const REAL bounced = r[OPP[i] * n + c];
    gin[i] = solid[src] ? bounced : streamed;
  }
  REAL m0 = 0, mx = 0, my = 0;
#pragma GCC unroll 9
  for (int i = 0; i < 9; ++i) {
    m0 += gin[i];
    mx += CX[i] * gin[i];
    my += CY[i] * gin[i];
  }
  const REAL drho = m0;
  const REAL rho = (REAL)1 + drho;
  const REAL ux = (mx + (REAL)0.5 * fx) / rho;
  const REAL uy = (my + (REAL)0.5 * fy) / rho;
  const REAL usq = ux * ux + uy * uy;
#pragma GCC unroll 9
  for (int i = 0; i < 9; ++i) {
    const REAL cu = CX[i] * ux + CY[i] * uy;
    const REAL geq = FN(equilibrium_shifted)(FN(W)[i], drho, rho, cu, usq);
    const REAL g_post = gin[i] - omega * (gin[i] - geq) +
                        force_prefactor * FN(guo_source)(FN(W)[i], (REAL)CX[i], (REAL)CY[i], ux,
                                                         uy, fx, fy);
    rn[i * n + c] = solid[c] ? (REAL)0 : g_post;
  }
}

/* Edge columns x = 0 and x = nx - 1: gather with the periodic wrap or the open-x rules. */
static void FN(pull_edge)(const REAL* r, REAL* rn, const uint8_t* solid, int nx, int ny, int x,
                          int y, int open_x, const REAL* eq_in, REAL omega, REAL force_prefactor,
                          REAL fx, REAL fy) {
  const size_t n = (size_t)nx * ny;
  const size_t c = (size_t)y * nx + x;
  REAL out[9] = {0};
  if (!solid[c]) {
    REAL gin[9];
    FN(gather_pull)(r, solid, nx, ny, x, y, open_x, eq_in, gin);
    FN(collide_store)(gin, omega, force_prefactor, fx, fy, out, 1);
  }
  for (int i = 0; i < 9; ++i) rn[i * n + c] = out[i];
}

/* One pull step on SoA post-collision states (r -> r_new), OpenMP over rows, restating the
 * structure of the reference's v1 solver (src/v1_omp/solver_v1.cpp:136-175): periodic rows
 * computed once per row, the two edge columns apart so that the interior loop has unit strides
 * and no branch. Solid cells get 0. */
static void FN(pull_step)(int nx, int ny, const uint8_t* solid, REAL omega, REAL force_prefactor,
                          REAL fx, REAL fy, int open_x, const REAL* eq_in,
                          const REAL* restrict r, REAL* restrict rn) {
  const size_t n = (size_t)nx * ny;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < ny; ++y) {
    const size_t row[3] = {(size_t)(y == 0 ? ny - 1 : y - 1) * nx, (size_t)y * nx,
                           (size_t)(y == ny - 1 ? 0 : y + 1) * nx};
    FN(pull_edge)(r, rn, solid, nx, ny, 0, y, open_x, eq_in, omega, force_prefactor, fx, fy);
#pragma GCC ivdep
    for (int x = 1; x < nx - 1; ++x)
      FN(pull_cell)(r, rn, solid, n, row, x, omega, force_prefactor, fx, fy);
    if (nx > 1)
      FN(pull_edge)(r, rn, solid, nx, ny, nx - 1, y, open_x, eq_in, omega, force_prefactor, fx,
                    fy);
  }
}

/* Runs `steps` pull steps ping-ponging between caller-provided SoA buffers r (input) and rn
 * (scratch, same size), with `threads` OpenMP threads (0: the OpenMP default). Returns 0 when
 * the result is in r, 1 when it is in rn. Bitwise identical to oracle_v0_run on stream(r). */
int FN(oracle_pull_steps)(int nx, int ny, const uint8_t* solid, REAL tau, REAL fx, REAL fy,
                          int open_x, REAL u_in, REAL* r, REAL* rn, int steps, int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const REAL omega = (REAL)1 / tau;
  const REAL force_prefactor = (REAL)1 - (REAL)0.5 * omega;
  REAL eq_in[9] = {0};
  if (open_x) FN(oracle_equilibrium_state)((REAL)1, u_in, (REAL)0, eq_in);
  REAL* a = r;
  REAL* b = rn;
  for (int k = 0; k < steps; ++k) {
    FN(pull_step)(nx, ny, solid, omega, force_prefactor, fx, fy, open_x, eq_in, a, b);
    REAL* t = a;
    a = b;
    b = t;
  }
  return a == r ? 0 : 1;
}

/* Zero-fills an SoA buffer with the row distribution of pull_step (first touch). */
void FN(oracle_first_touch)(int nx, int ny, REAL* r) {
  const size_t n = (size_t)nx * ny;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < ny; ++y)
    for (int i = 0; i < 9; ++i) memset(&r[i * n + (size_t)y * nx], 0, (size_t)nx * sizeof(REAL));
}

/* Runs `steps` pull steps in place on the SoA state r (allocates the second buffer). Returns 0,
 * -1 on allocation failure. */
int FN(oracle_pull_run)(int nx, int ny, const uint8_t* solid, REAL tau, REAL fx, REAL fy,
                        int open_x, REAL u_in, REAL* r, int steps, int threads) {
  const size_t n = (size_t)nx * ny * 9;
  REAL* rn = (REAL*)malloc(n * sizeof(REAL));
  if (!rn) return -1;
  FN(oracle_first_touch)(nx, ny, rn);
  if (FN(oracle_pull_steps)(nx, ny, solid, tau, fx, fy, open_x, u_in, r, rn, steps, threads))
    memcpy(r, rn, n * sizeof(REAL));
  free(rn);
  return 0;
}

/* Seeded uniform perturbation of the shifted populations: s[c*9+i] = U(-amp, amp) on fluid
 * cells, 0 on solid cells, from the counter-based SplitMix64 stream of oracle_seeded_uniform. */
void FN(oracle_seeded_state)(uint64_t seed, double amp, int nx, int ny, const uint8_t* solid,
                             REAL* s) {
  const size_t n = (size_t)nx * ny;
  for (size_t c = 0; c < n; ++c)
    for (int i = 0; i < 9; ++i)
      s[c * 9 + i] = solid[c] ? (REAL)0 : (REAL)oracle_seeded_uniform(seed, c * 9 + i, amp);
}
