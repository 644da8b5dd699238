// Adjoint of the stream-collide step: gradients of a flow objective with respect to the body
// force, tau and a per-cell Brinkman drag field, with checkpointed recomputation.
//
// Forward model (per instance b of a batch sharing geometry, tau and force; alpha differs):
//   y_t = P R_t                      pull gather (streaming + halfway bounce-back), periodic;
//   R_{t+1} = C(y_t; tau, F, alpha)  BGK + Guo collision with a Brinkman drag force
//                                    F_tot = F - alpha rho u, where the Guo velocity
//                                    u = (m + F/2) / (rho (1 + alpha/2)) solves
//                                    rho u = m + F_tot / 2 exactly.
//   alpha = 0 gives the reference's collision (src/v0_cpu/solver_v0.cpp:127-143) operation for
//   operation (kf = 1 + 0 * 0.5 = 1, rho * 1 = rho, F - 0 = F), so the forward is bit-exact with
//   the plain method there.
// Objective: J = (1/W) sum_{t = T-W+1..T} (1/N_fluid) sum_fluid u_x(y_t).
// Reverse sweep: ybar_t = J_C(y_t)^T (P^T ybar_{t+1}) + dj_t/dy_t, where P^T (the transpose of the
// pull gather) is again a gather: (P^T z)[j][c] = solid(c + e_j) ? z[opp j][c] : z[j][c + e_j].
// Parameter gradients accumulate in FP64 (per instance: omega, fx, fy; per cell: alpha).
// States are recomputed segment by segment from checkpoints stored every K steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "lbm_b200.h"
#include "lbm_device.cuh"
#include "solver_internal.h"

using namespace lbm_b200;

namespace {

constexpr int kAdjThreads = 256;

struct AdjGeom {
  int nx, ny, mask_words, batch;
  long long n;       // cells per instance (nx * ny), planes are unpadded
  long long inst;    // elements per instance state (9 n)
};

template <class T>
struct AdjParams {
  T omega, fp, fx, fy, hfx, hfy;
  const T* alpha;  // batch * n, or null (zero field)
};

__device__ __forceinline__ long long wrap_cell(const AdjGeom& g, int x, int y) {
  x = x < 0 ? g.nx - 1 : (x >= g.nx ? 0 : x);
  y = y < 0 ? g.ny - 1 : (y >= g.ny ? 0 : y);
  return static_cast<long long>(y) * g.nx + x;
}

__device__ __forceinline__ bool solid_at(const uint32_t* mask, const AdjGeom& g, long long c) {
  const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
  return mask_solid(mask, g.mask_words, x, y);
}

// Per-cell neighbour code: bit i (0..8) = the pull source c - e_i is solid, bit 9 + j = the
// transpose source c + e_j is solid, bit 31 = c itself is solid. Built once per adjoint object.
constexpr uint32_t kCodeSolid = 1u << 31;

__global__ void adj_code_kernel(const uint32_t* __restrict__ mask, const AdjGeom g,
                                uint32_t* __restrict__ code) {
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < g.n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    uint32_t k = mask_solid(mask, g.mask_words, x, y) ? kCodeSolid : 0u;
#pragma unroll
    for (int i = 0; i < kQ; ++i) {
      if (solid_at(mask, g, wrap_cell(g, x - dir_cx(i), y - dir_cy(i)))) k |= 1u << i;
      if (solid_at(mask, g, wrap_cell(g, x + dir_cx(i), y + dir_cy(i)))) k |= 1u << (9 + i);
    }
    code[c] = k;
  }
}

// Periodic neighbourhood of cell (x, y): column of x - 1, x, x + 1 and row offset (times nx) of
// y - 1, y, y + 1, so that every gather index is one add.
struct Nbhd {
  int col[3];
  int row[3];
};
__device__ __forceinline__ Nbhd nbhd(const AdjGeom& g, int x, int y) {
  Nbhd h;
  h.col[0] = x == 0 ? g.nx - 1 : x - 1;
  h.col[1] = x;
  h.col[2] = x == g.nx - 1 ? 0 : x + 1;
  h.row[0] = (y == 0 ? g.ny - 1 : y - 1) * g.nx;
  h.row[1] = y * g.nx;
  h.row[2] = (y == g.ny - 1 ? 0 : y + 1) * g.nx;
  return h;
}

// Pull gather y = P R of one cell: y_i = solid(c - e_i) ? R[opp i][c] : R[i][c - e_i].
template <class T>
__device__ __forceinline__ void gather_fwd(const T* R, uint32_t code, const AdjGeom& g, const Nbhd& h,
                                           int c, T (&out)[kQ]) {
#pragma unroll
  for (int i = 0; i < kQ; ++i) {
    const int src = ((code >> i) & 1u) ? c
                                       : h.row[1 - dir_cy(i)] + h.col[1 - dir_cx(i)];
    const int plane = ((code >> i) & 1u) ? dir_opp(i) : i;
    out[i] = R[static_cast<long long>(plane) * g.n + src];
  }
}

// Transpose of the pull gather (closed domain): (P^T Z)_j = solid(c + e_j) ? Z[opp j][c]
// : Z[j][c + e_j].
template <class T>
__device__ __forceinline__ void gather_transpose(const T* Z, uint32_t code, const AdjGeom& g,
                                                 const Nbhd& h, int c, T (&out)[kQ]) {
#pragma unroll
  for (int j = 0; j < kQ; ++j) {
    const bool bounce = (code >> (9 + j)) & 1u;
    const int src = bounce ? c : h.row[1 + dir_cy(j)] + h.col[1 + dir_cx(j)];
    const int plane = bounce ? dir_opp(j) : j;
    out[j] = Z[static_cast<long long>(plane) * g.n + src];
  }
}

// Reciprocal of the backward sweep's linearisation (rounding-level accuracy suffices there):
// FP32 uses the hardware approximation, which keeps the IEEE division's out-of-line slow path
// (and the register spills its call forces) out of the kernel.
__device__ __forceinline__ float adj_rcp(float d) { return __fdividef(1.0f, d); }
__device__ __forceinline__ double adj_rcp(double d) { return 1.0 / d; }

__device__ __forceinline__ void block_add_to(double v, double* target, double* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = lane < static_cast<int>(blockDim.x >> 5) ? smem[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0 && t != 0.0) atomicAdd(target, t);
  }
}

// One forward step R -> Rn for all instances; obj (per instance, or null) accumulates the sum of
// u_x of the input state over fluid cells. write_out = 0: objective only.
template <class A>
__global__ void __launch_bounds__(kAdjThreads, 3)
    adj_forward_kernel(const typename A::T* __restrict__ R, typename A::T* __restrict__ Rn,
                       const uint32_t* __restrict__ codes, const AdjGeom g,
                       const AdjParams<typename A::T> p, int write_out, double* __restrict__ obj) {
  using T = typename A::T;
  __shared__ double smem[32];
  const int b = blockIdx.y;
  const T* Rb = R + b * g.inst;
  T* Rnb = Rn ? Rn + b * g.inst : nullptr;
  CollideConsts<T> k{};  // the collision's constants (cf_* unused: the force is per cell)
  k.omega = p.omega;
  k.force_prefactor = p.fp;
  k.fx = p.fx;
  k.fy = p.fy;
  k.hfx = p.hfx;
  k.hfy = p.hfy;
  T usum = T(0);  // per-thread partial sum (a few cells), added in double per block below
#pragma unroll 1
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < g.n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    const uint32_t code = codes[c];
    if (code & kCodeSolid) {
      if (write_out) {
#pragma unroll
        for (int i = 0; i < kQ; ++i) Rnb[i * g.n + c] = T(0);
      }
      continue;
    }
    T yv[kQ], out[kQ];
    gather_fwd(Rb, code, g, nbhd(g, x, y), static_cast<int>(c), yv);
    const T alpha = p.alpha ? p.alpha[b * g.n + c] : T(0);
    const T ux = collide_exact_drag<A>(yv, k, alpha, out);
    if (write_out) {
#pragma unroll
      for (int i = 0; i < kQ; ++i) Rnb[i * g.n + c] = out[i];
    }
    if (obj) usum += ux;
  }
  if (obj) block_add_to(static_cast<double>(usum), obj + b, smem);
}

// One adjoint step: Ybar = J_C(y_t)^T (P^T Ynext) + obj_coef * du_x/dy_t, with y_t = P R_t.
// Ynext == null: no later step (the final state). grads: per instance {omega_bar, fx_bar,
// fy_bar}; abar: per cell alpha_bar (accumulated), or null. The linearisation point y_t comes from
// the exact forward states; the intermediates and the adjoint arithmetic use FMA (this file is
// compiled with contraction allowed), which changes the gradient only at rounding level.
// alpha_bar accumulates per segment in `aseg` (precision T; zero at the start of the sweep and
// after every flush) and is flushed into the double-precision `abar` by the segment's last
// adjoint step (flush != 0), so that the per-step update is a T add, not a double one.
template <class T>
__global__ void __launch_bounds__(kAdjThreads, 3)
    adj_backward_kernel(const T* __restrict__ R, const T* __restrict__ Ynext, T* __restrict__ Ybar,
                        const uint32_t* __restrict__ codes, const AdjGeom g, const AdjParams<T> p,
                        T obj_coef, double* __restrict__ grads, T* __restrict__ aseg,
                        double* __restrict__ abar, int flush) {
  __shared__ double smem[32];
  const int b = blockIdx.y;
  const T* Rb = R + b * g.inst;
  const T* Yn = Ynext ? Ynext + b * g.inst : nullptr;
  T* Yb = Ybar + b * g.inst;
  T g_omega = T(0), g_fx = T(0), g_fy = T(0);  // per-thread partial sums (a few cells)
#pragma unroll 1
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < g.n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    const uint32_t code = codes[c];
    if (code & kCodeSolid) {
#pragma unroll
      for (int i = 0; i < kQ; ++i) Yb[i * g.n + c] = T(0);
      continue;
    }
    const Nbhd h = nbhd(g, x, y);
    T yv[kQ];
    gather_fwd(Rb, code, g, h, static_cast<int>(c), yv);
    T v[kQ];
    if (Yn) {
      gather_transpose(Yn, code, g, h, static_cast<int>(c), v);
    } else {
#pragma unroll
      for (int i = 0; i < kQ; ++i) v[i] = T(0);
    }
    // Forward intermediates (FMA arithmetic; zero-coefficient terms dropped at compile time).
    const T alpha = p.alpha ? p.alpha[b * g.n + c] : T(0);
    const T drho = ((yv[0] + yv[1]) + (yv[2] + yv[3])) + ((yv[4] + yv[5]) + (yv[6] + yv[7])) + yv[8];
    const T mx = (yv[1] - yv[3]) + (yv[5] - yv[6]) + (yv[8] - yv[7]);
    const T my = (yv[2] - yv[4]) + (yv[5] + yv[6]) - (yv[7] + yv[8]);
    const T rho = T(1) + drho;
    const T kf = T(1) + T(0.5) * alpha;
    const T d = rho * kf;
    const T inv_d = adj_rcp(d);
    const T ux = (mx + p.hfx) * inv_d, uy = (my + p.hfy) * inv_d;
    const T Fx = p.fx - alpha * rho * ux, Fy = p.fy - alpha * rho * uy;
    const T usq = ux * ux + uy * uy;
    // Backward through post_i = y_i - omega (y_i - geq_i) + fp guo_i in closed form: every sum
    // over directions of v_i w_i times a polynomial in c_i is a weighted moment of v (c^3 = c for
    // c in {0, +-1}):
    //   V0 = sum w v, Vx = sum w v c_x, Vy, Vxx = sum w v c_x^2, Vxy = sum w v c_x c_y, Vyy.
    const T D = (v[5] + v[6]) + (v[7] + v[8]);
    const T a13 = v[1] + v[3], a24 = v[2] + v[4];
    const T w1 = T(1) / T(9), w5 = T(1) / T(36);
    const T V0 = T(4) / T(9) * v[0] + w1 * (a13 + a24) + w5 * D;
    const T Vx = w1 * (v[1] - v[3]) + w5 * ((v[5] - v[6]) + (v[8] - v[7]));
    const T Vy = w1 * (v[2] - v[4]) + w5 * ((v[5] + v[6]) - (v[7] + v[8]));
    const T Vxx = w1 * a13 + w5 * D, Vyy = w1 * a24 + w5 * D;
    const T Vxy = w5 * ((v[5] - v[6]) + (v[7] - v[8]));
    T vy = T(0);  // sum v_i y_i
#pragma unroll
    for (int i = 0; i < kQ; ++i) vy += v[i] * yv[i];
    const T uV = ux * Vx + uy * Vy;
    const T Q = ux * ux * Vxx + T(2) * ux * uy * Vxy + uy * uy * Vyy;
    const T sA = T(3) * uV + T(4.5) * Q - T(1.5) * usq * V0;  // sum w v A_i
    const T cxu = ux * Vxx + uy * Vxy, cyu = ux * Vxy + uy * Vyy;  // sum w v cu c_x, c_y
    const T cxF = Fx * Vxx + Fy * Vxy, cyF = Fx * Vxy + Fy * Vyy;  // sum w v cf c_x, c_y
    const T sgeq = drho * V0 + rho * sA;                            // sum v geq
    const T sguo = T(3) * (Fx * Vx + Fy * Vy - (ux * Fx + uy * Fy) * V0) +
                   T(9) * (ux * cxF + uy * cyF);                     // sum v guo
    const T om = sgeq - vy - T(0.5) * sguo;
    const T orho = p.omega * rho;
    T d_drho = p.omega * V0;
    T d_rho = p.omega * sA;
    const T d_usq = T(-1.5) * orho * V0;
    T d_ux = obj_coef + orho * (T(3) * Vx + T(9) * cxu) + T(9) * p.fp * cxF - T(3) * p.fp * Fx * V0 +
             T(2) * ux * d_usq;
    T d_uy = orho * (T(3) * Vy + T(9) * cyu) + T(9) * p.fp * cyF - T(3) * p.fp * Fy * V0 +
             T(2) * uy * d_usq;
    const T d_Fx = T(3) * p.fp * (Vx - ux * V0) + T(9) * p.fp * cxu;
    const T d_Fy = T(3) * p.fp * (Vy - uy * V0) + T(9) * p.fp * cyu;
    // F_tot = F - alpha rho u
    T a_b = -(d_Fx * rho * ux + d_Fy * rho * uy);
    d_rho -= alpha * (d_Fx * ux + d_Fy * uy);
    d_ux -= d_Fx * alpha * rho;
    d_uy -= d_Fy * alpha * rho;
    // u = (m + F/2) / d, d = rho kf, kf = 1 + alpha/2
    const T mxb = d_ux * inv_d, myb = d_uy * inv_d;
    const T db = -(d_ux * ux + d_uy * uy) * inv_d;
    d_rho += db * kf;
    a_b += T(0.5) * db * rho;
    // rho = 1 + drho, drho = sum y, m = sum c y
    const T dtot = d_drho + d_rho;
    const T om1 = T(1) - p.omega;
#pragma unroll
    for (int i = 0; i < kQ; ++i) {
      T o = om1 * v[i] + dtot;
      if (dir_cx(i) != 0) o += dir_cx(i) > 0 ? mxb : -mxb;
      if (dir_cy(i) != 0) o += dir_cy(i) > 0 ? myb : -myb;
      Yb[i * g.n + c] = o;
    }
    g_omega += om;
    g_fx += d_Fx + T(0.5) * mxb;
    g_fy += d_Fy + T(0.5) * myb;
    if (aseg) {
      const long long ia = b * g.n + c;
      const T acc = aseg[ia] + a_b;
      if (flush) {
        abar[ia] += static_cast<double>(acc);
        aseg[ia] = T(0);
      } else {
        aseg[ia] = acc;
      }
    }
  }
  block_add_to(static_cast<double>(g_omega), grads + 3 * b + 0, smem);
  block_add_to(static_cast<double>(g_fx), grads + 3 * b + 1, smem);
  block_add_to(static_cast<double>(g_fy), grads + 3 * b + 2, smem);
}

// Pull state of every instance from v0-layout post-streaming states (closed domain).
template <class T>
__global__ void adj_set_state_kernel(T* __restrict__ R, const uint32_t* __restrict__ mask,
                                     const AdjGeom g, const T* __restrict__ aos) {
  const int b = blockIdx.y;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < g.n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    const bool solid = mask_solid(mask, g.mask_words, x, y);
    const T* s = aos + b * g.inst;
#pragma unroll
    for (int i = 0; i < kQ; ++i) {
      T v = T(0);
      if (!solid) {
        const long long cn = wrap_cell(g, x + dir_cx(i), y + dir_cy(i));
        v = solid_at(mask, g, cn) ? s[c * kQ + dir_opp(i)] : s[cn * kQ + i];
      }
      R[b * g.inst + i * g.n + c] = v;
    }
  }
}

template <class T>
__global__ void adj_get_state_kernel(const T* __restrict__ R, const uint32_t* __restrict__ codes,
                                     const AdjGeom g, int b, T* __restrict__ aos) {
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < g.n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    T s[kQ];
    const uint32_t code = codes[c];
    if (code & kCodeSolid) {
#pragma unroll
      for (int i = 0; i < kQ; ++i) s[i] = T(0);
    } else {
      gather_fwd(R + b * g.inst, code, g, nbhd(g, x, y), static_cast<int>(c), s);
    }
#pragma unroll
    for (int i = 0; i < kQ; ++i) aos[c * kQ + i] = s[i];
  }
}

template <class T>
__global__ void cast_kernel(const double* __restrict__ in, T* __restrict__ out, long long n) {
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<long long>(gridDim.x) * blockDim.x)
    out[k] = static_cast<T>(in[k]);
}

}  // namespace

struct lbm_adjoint {
  int precision = LBM_FP32, elem = 4, batch = 1, K = 100;
  AdjGeom g{};
  std::vector<uint8_t> solid;
  long long fluid = 0;
  double tau = 0, fx = 0, fy = 0;
  uint32_t* mask_d = nullptr;
  uint32_t* codes = nullptr;     // per-cell neighbour codes
  void* alpha = nullptr;         // batch * n elements (T), null = zero field
  void* state[2] = {nullptr, nullptr};
  void* ckpt = nullptr;          // checkpoints: (T/K + 1) states
  size_t ckpt_count = 0;
  void* seg = nullptr;           // K + 1 recomputed states
  void* ybar[2] = {nullptr, nullptr};
  double* grads = nullptr;       // batch * 3
  double* abar = nullptr;        // batch * n
  void* aseg = nullptr;          // batch * n, per-segment alpha_bar in the state precision
  double* obj = nullptr;         // batch
  void* stage = nullptr;
  size_t stage_bytes = 0;
  int steps = 0, window = 0;     // of the last forward
  int fin_state = 0;             // state[] index holding R_T after the forward
  bool have_forward = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  double fwd_step_s = 0, bwd_step_s = 0;
  int sm_count = 0;
  std::string err;
};

namespace {

int adj_fail(lbm_adjoint* a, int code, const std::string& msg) {
  if (a) a->err = msg;
  return code;
}

#define ADJ_CUDA(a, call)                                                                     \
  do {                                                                                       \
    const cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                                 \
      cudaGetLastError();                                                                    \
      return adj_fail(a, e_ == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA, \
                      std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    }                                                                                        \
  } while (0)

size_t state_bytes(const lbm_adjoint* a) {
  return static_cast<size_t>(a->batch) * a->g.inst * a->elem;
}

template <class T>
AdjParams<T> params(const lbm_adjoint* a) {
  AdjParams<T> p;
  const T tau = T(a->tau);
  p.omega = T(1) / tau;
  p.fp = T(1) - T(0.5) * p.omega;
  p.fx = T(a->fx);
  p.fy = T(a->fy);
  p.hfx = T(0.5) * p.fx;
  p.hfy = T(0.5) * p.fy;
  p.alpha = static_cast<const T*>(a->alpha);
  return p;
}

// Blocks per instance (grid x) and instances (grid y): about two waves of three resident blocks
// per SM in total, so that each thread takes several cells and the per-block FP64 reductions of
// the objective and the parameter gradients are amortised.
dim3 grid2(const lbm_adjoint* a) {
  const long long want = (a->g.n + kAdjThreads - 1) / kAdjThreads;
  const long long target = (6LL * a->sm_count + a->batch - 1) / a->batch;
  const int bx = static_cast<int>(std::max<long long>(1, std::min<long long>(want, target)));
  return dim3(bx, a->batch);
}

template <class A>
int forward_t(lbm_adjoint* a, const void* s0_host, int steps, int window, double* J) {
  using T = typename A::T;
  const size_t sb = state_bytes(a);
  const size_t nckpt = static_cast<size_t>(steps / a->K) + 1;
  if (a->ckpt_count < nckpt) {
    cudaFree(a->ckpt);
    a->ckpt = nullptr;
    a->ckpt_count = 0;
    ADJ_CUDA(a, cudaMalloc(&a->ckpt, nckpt * sb));
    a->ckpt_count = nckpt;
  }
  if (s0_host) {
    if (a->stage_bytes < sb) {
      cudaFree(a->stage);
      a->stage = nullptr;
      ADJ_CUDA(a, cudaMalloc(&a->stage, sb));
      a->stage_bytes = sb;
    }
    ADJ_CUDA(a, cudaMemcpyAsync(a->stage, s0_host, sb, cudaMemcpyHostToDevice, a->stream));
    adj_set_state_kernel<T><<<grid2(a), kAdjThreads, 0, a->stream>>>(
        static_cast<T*>(a->state[0]), a->mask_d, a->g, static_cast<const T*>(a->stage));
  } else {
    ADJ_CUDA(a, cudaMemsetAsync(a->state[0], 0, sb, a->stream));  // rest: f_i - w_i = 0
  }
  ADJ_CUDA(a, cudaMemcpyAsync(a->ckpt, a->state[0], sb, cudaMemcpyDeviceToDevice, a->stream));
  ADJ_CUDA(a, cudaMemsetAsync(a->obj, 0, a->batch * sizeof(double), a->stream));
  const AdjParams<T> p = params<T>(a);
  const dim3 grid = grid2(a);
  int cur = 0;
  ADJ_CUDA(a, cudaEventRecord(a->ev[0], a->stream));
  for (int t = 0; t < steps; ++t) {
    const bool in_window = t >= steps - window + 1;
    adj_forward_kernel<A><<<grid, kAdjThreads, 0, a->stream>>>(
        static_cast<const T*>(a->state[cur]), static_cast<T*>(a->state[cur ^ 1]), a->codes, a->g,
        p, 1, in_window ? a->obj : nullptr);
    cur ^= 1;
    if ((t + 1) % a->K == 0)
      ADJ_CUDA(a, cudaMemcpyAsync(static_cast<char*>(a->ckpt) + ((t + 1) / a->K) * sb,
                                  a->state[cur], sb, cudaMemcpyDeviceToDevice, a->stream));
  }
  ADJ_CUDA(a, cudaEventRecord(a->ev[1], a->stream));
  adj_forward_kernel<A><<<grid, kAdjThreads, 0, a->stream>>>(
      static_cast<const T*>(a->state[cur]), nullptr, a->codes, a->g, p, 0, a->obj);
  ADJ_CUDA(a, cudaGetLastError());
  std::vector<double> obj(a->batch);
  ADJ_CUDA(a, cudaMemcpyAsync(obj.data(), a->obj, a->batch * sizeof(double), cudaMemcpyDeviceToHost,
                              a->stream));
  ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  float ms = 0.f;
  ADJ_CUDA(a, cudaEventElapsedTime(&ms, a->ev[0], a->ev[1]));
  a->fwd_step_s = steps > 0 ? ms * 1e-3 / steps : 0.0;
  for (int b = 0; b < a->batch; ++b) J[b] = obj[b] / (static_cast<double>(window) * a->fluid);
  a->steps = steps;
  a->window = window;
  a->have_forward = true;
  a->fin_state = cur;
  return LBM_OK;
}

template <class A>
int backward_t(lbm_adjoint* a, double* dtau, double* dfx, double* dfy, double* dalpha) {
  using T = typename A::T;
  const size_t sb = state_bytes(a);
  const int T_steps = a->steps, W = a->window, K = a->K;
  if (!a->seg) ADJ_CUDA(a, cudaMalloc(&a->seg, (K + 1) * sb));
  for (int k = 0; k < 2; ++k)
    if (!a->ybar[k]) ADJ_CUDA(a, cudaMalloc(&a->ybar[k], sb));
  ADJ_CUDA(a, cudaMemsetAsync(a->grads, 0, 3 * a->batch * sizeof(double), a->stream));
  ADJ_CUDA(a, cudaMemsetAsync(a->abar, 0, a->batch * a->g.n * sizeof(double), a->stream));
  if (!a->aseg) ADJ_CUDA(a, cudaMalloc(&a->aseg, a->batch * a->g.n * a->elem));
  ADJ_CUDA(a, cudaMemsetAsync(a->aseg, 0, a->batch * a->g.n * a->elem, a->stream));
  const AdjParams<T> p = params<T>(a);
  const dim3 grid = grid2(a);
  const T coef = T(1.0 / (static_cast<double>(W) * a->fluid));
  char* seg = static_cast<char*>(a->seg);
  int yb = 0;
  bool first = true;
  ADJ_CUDA(a, cudaEventRecord(a->ev[0], a->stream));
  const int nseg = (T_steps + K - 1) / K;
  for (int s = nseg - 1; s >= 0; --s) {
    const int t0 = s * K, t1 = std::min(T_steps, t0 + K);
    // Recompute R_{t0..t1} from checkpoint s.
    ADJ_CUDA(a, cudaMemcpyAsync(seg, static_cast<char*>(a->ckpt) + static_cast<size_t>(s) * sb, sb,
                                cudaMemcpyDeviceToDevice, a->stream));
    for (int t = t0; t < t1; ++t)
      adj_forward_kernel<A><<<grid, kAdjThreads, 0, a->stream>>>(
          reinterpret_cast<const T*>(seg + (t - t0) * sb), reinterpret_cast<T*>(seg + (t - t0 + 1) * sb),
          a->codes, a->g, p, 1, nullptr);
    // Adjoint steps t1 (only for the last segment: the final state) .. t0.
    const int top = (s == nseg - 1) ? t1 : t1 - 1;
    for (int t = top; t >= t0; --t) {
      const bool in_window = t >= T_steps - W + 1;
      adj_backward_kernel<T><<<grid, kAdjThreads, 0, a->stream>>>(
          reinterpret_cast<const T*>(seg + (t - t0) * sb),
          first ? nullptr : static_cast<const T*>(a->ybar[yb ^ 1]), static_cast<T*>(a->ybar[yb]),
          a->codes, a->g, p, in_window ? coef : T(0), a->grads,
          dalpha ? static_cast<T*>(a->aseg) : nullptr, a->abar, t == t0 ? 1 : 0);
      first = false;
      yb ^= 1;
    }
  }
  ADJ_CUDA(a, cudaEventRecord(a->ev[1], a->stream));
  ADJ_CUDA(a, cudaGetLastError());
  std::vector<double> g(3 * a->batch);
  ADJ_CUDA(a, cudaMemcpyAsync(g.data(), a->grads, g.size() * sizeof(double), cudaMemcpyDeviceToHost,
                              a->stream));
  if (dalpha)
    ADJ_CUDA(a, cudaMemcpyAsync(dalpha, a->abar, a->batch * a->g.n * sizeof(double),
                                cudaMemcpyDeviceToHost, a->stream));
  ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  float ms = 0.f;
  ADJ_CUDA(a, cudaEventElapsedTime(&ms, a->ev[0], a->ev[1]));
  a->bwd_step_s = T_steps > 0 ? ms * 1e-3 / (T_steps + 1) : 0.0;
  const double omega = 1.0 / static_cast<double>(T(a->tau));
  for (int b = 0; b < a->batch; ++b) {
    if (dtau) dtau[b] = g[3 * b] * (-omega * omega);  // d omega / d tau = -1/tau^2
    if (dfx) dfx[b] = g[3 * b + 1];
    if (dfy) dfy[b] = g[3 * b + 2];
  }
  return LBM_OK;
}

template <class T>
int get_state_t(lbm_adjoint* a, int b, void* host) {
  const size_t bytes = static_cast<size_t>(a->g.inst) * sizeof(T);
  if (a->stage_bytes < bytes) {
    cudaFree(a->stage);
    a->stage = nullptr;
    ADJ_CUDA(a, cudaMalloc(&a->stage, bytes));
    a->stage_bytes = bytes;
  }
  adj_get_state_kernel<T><<<grid2(a).x, kAdjThreads, 0, a->stream>>>(
      static_cast<const T*>(a->state[a->fin_state]), a->codes, a->g, b, static_cast<T*>(a->stage));
  ADJ_CUDA(a, cudaMemcpyAsync(host, a->stage, bytes, cudaMemcpyDeviceToHost, a->stream));
  ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_adj_create(int nx, int ny, const uint8_t* solid, double tau, double fx, double fy,
                   int precision, int batch, int checkpoint_every, lbm_adjoint** out) {
  if (!out) return LBM_ERR_INVALID_ARG;
  *out = nullptr;
  if (nx < 1 || ny < 1 || !solid || batch < 1 || checkpoint_every < 1 || !(tau > 0.5) ||
      (precision != LBM_FP32 && precision != LBM_FP64) ||
      static_cast<long long>(nx) * ny > static_cast<long long>(INT_MAX))  // 32-bit cell indices
    return LBM_ERR_INVALID_ARG;
  lbm_adjoint* a = new (std::nothrow) lbm_adjoint();
  if (!a) return LBM_ERR_OUT_OF_MEMORY;
  a->precision = precision;
  a->elem = precision == LBM_FP64 ? 8 : 4;
  a->batch = batch;
  a->K = checkpoint_every;
  a->tau = tau;
  a->fx = fx;
  a->fy = fy;
  a->g.nx = nx;
  a->g.ny = ny;
  a->g.batch = batch;
  a->g.n = static_cast<long long>(nx) * ny;
  a->g.inst = kQ * a->g.n;
  a->g.mask_words = (nx + 2 + 31) / 32 + 2;
  a->solid.assign(solid, solid + a->g.n);
  for (uint8_t v : a->solid) a->fluid += v ? 0 : 1;
  auto fail = [&](int code) {
    lbm_adj_destroy(a);
    return code;
  };
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&a->sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&a->ev[0]) != cudaSuccess || cudaEventCreate(&a->ev[1]) != cudaSuccess)
    return fail(LBM_ERR_CUDA);
  std::vector<uint32_t> words;
  pack_mask(solid, nx, ny, a->g.mask_words, words);
  const size_t sb = state_bytes(a);
  cudaError_t e = cudaMalloc(&a->mask_d, words.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpy(a->mask_d, words.data(), words.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&a->codes, a->g.n * sizeof(uint32_t));
  if (e == cudaSuccess) {
    adj_code_kernel<<<256, 256, 0, a->stream>>>(a->mask_d, a->g, a->codes);
    e = cudaStreamSynchronize(a->stream);
  }
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaMalloc(&a->state[k], sb);
  if (e == cudaSuccess) e = cudaMalloc(&a->grads, 3 * batch * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&a->abar, batch * a->g.n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&a->obj, batch * sizeof(double));
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA);
  *out = a;
  return LBM_OK;
}

int lbm_adj_destroy(lbm_adjoint* a) {
  if (!a) return LBM_OK;
  if (a->stream) cudaStreamSynchronize(a->stream);
  for (void* p : {static_cast<void*>(a->mask_d), static_cast<void*>(a->codes), a->alpha, a->state[0], a->state[1], a->ckpt, a->seg,
                  a->ybar[0], a->ybar[1], static_cast<void*>(a->grads), static_cast<void*>(a->abar), a->aseg,
                  static_cast<void*>(a->obj), a->stage})
    cudaFree(p);
  for (cudaEvent_t ev : a->ev)
    if (ev) cudaEventDestroy(ev);
  if (a->stream) cudaStreamDestroy(a->stream);
  delete a;
  return LBM_OK;
}

const char* lbm_adj_last_error(const lbm_adjoint* a) { return a ? a->err.c_str() : "null"; }

int lbm_adj_set_params(lbm_adjoint* a, double tau, double fx, double fy) {
  if (!a || !(tau > 0.5)) return adj_fail(a, LBM_ERR_INVALID_ARG, "tau must be > 0.5");
  a->tau = tau;
  a->fx = fx;
  a->fy = fy;
  a->have_forward = false;
  return LBM_OK;
}

int lbm_adj_set_alpha(lbm_adjoint* a, const double* alpha) {
  if (!a) return LBM_ERR_INVALID_ARG;
  if (!alpha) {
    cudaFree(a->alpha);
    a->alpha = nullptr;
    return LBM_OK;
  }
  const long long n = a->batch * a->g.n;
  double* tmp = nullptr;
  if (!a->alpha) ADJ_CUDA(a, cudaMalloc(&a->alpha, n * a->elem));
  ADJ_CUDA(a, cudaMalloc(&tmp, n * sizeof(double)));
  ADJ_CUDA(a, cudaMemcpy(tmp, alpha, n * sizeof(double), cudaMemcpyHostToDevice));
  if (a->precision == LBM_FP64)
    cast_kernel<double><<<256, 256, 0, a->stream>>>(tmp, static_cast<double*>(a->alpha), n);
  else
    cast_kernel<float><<<256, 256, 0, a->stream>>>(tmp, static_cast<float*>(a->alpha), n);
  const cudaError_t e = cudaStreamSynchronize(a->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return adj_fail(a, LBM_ERR_CUDA, cudaGetErrorString(e));
  a->have_forward = false;
  return LBM_OK;
}

int lbm_adj_forward(lbm_adjoint* a, const void* s0, int steps, int window, double* J) {
  if (!a || !J || steps < 1 || window < 1 || window > steps + 1)
    return adj_fail(a, LBM_ERR_INVALID_ARG, "need steps >= 1 and 1 <= window <= steps + 1");
  return a->precision == LBM_FP64 ? forward_t<ExactF64>(a, s0, steps, window, J)
                                  : forward_t<ExactF32>(a, s0, steps, window, J);
}

int lbm_adj_backward(lbm_adjoint* a, double* dtau, double* dfx, double* dfy, double* dalpha) {
  if (!a) return LBM_ERR_INVALID_ARG;
  if (!a->have_forward) return adj_fail(a, LBM_ERR_INVALID_ARG, "run lbm_adj_forward first");
  return a->precision == LBM_FP64 ? backward_t<ExactF64>(a, dtau, dfx, dfy, dalpha)
                                  : backward_t<ExactF32>(a, dtau, dfx, dfy, dalpha);
}

int lbm_adj_get_populations(lbm_adjoint* a, int instance, void* s_host) {
  if (!a || !s_host || instance < 0 || instance >= a->batch || !a->have_forward)
    return adj_fail(a, LBM_ERR_INVALID_ARG, "bad instance or no forward run");
  return a->precision == LBM_FP64 ? get_state_t<double>(a, instance, s_host)
                                  : get_state_t<float>(a, instance, s_host);
}

int lbm_adj_step_times(lbm_adjoint* a, double* forward_step_s, double* backward_step_s) {
  if (!a) return LBM_ERR_INVALID_ARG;
  if (forward_step_s) *forward_step_s = a->fwd_step_s;
  if (backward_step_s) *backward_step_s = a->bwd_step_s;
  return LBM_OK;
}

}  // extern "C"
