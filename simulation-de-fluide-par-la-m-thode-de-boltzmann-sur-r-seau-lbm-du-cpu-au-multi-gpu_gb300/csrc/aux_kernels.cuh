// Kernels around the step: building and reading the state (layout conversions between the
// reference's v0 layout and the pull state), the moment pass, the mass reduction and the probe.
// None of them is on the time-step path; they are one thread per cell.
#pragma once

#include "lbm_device.cuh"

namespace lbm_b200 {

__device__ __forceinline__ long long cell_index(const Grid2D& g, int x, int y) {
  return static_cast<long long>(y) * g.pitch + x;
}

// Post-streaming populations of fluid cell (x, y) from the pull state R: population i arrives
// from (x - cx_i, y - cy_i) (periodic), or bounces back as R[opp i] of the cell itself when that
// source is solid; open domain: inlet equilibrium at x = 0 for c_x = +1, outlet copy of column
// nx - 2 at x = nx - 1 for c_x = -1 (reference src/common/boundary.hpp:53-70).
template <class ST>
__device__ void gather_cell(const ST* __restrict__ R, const uint32_t* __restrict__ mask,
                            const Grid2D& g, int x, int y,
                            const Eq9<typename StoreTraits<ST>::T>& eq_in, const PlaneScales& sc,
                            typename StoreTraits<ST>::T (&out)[kQ]) {
#pragma unroll
  for (int i = 0; i < kQ; ++i) {
    if (g.open_x && x == 0 && dir_cx(i) == 1) {
      out[i] = eq_in.v[i];
      continue;
    }
    int xc = x;
    if (g.open_x && x == g.nx - 1 && dir_cx(i) == -1) xc = g.nx - 2;
    int xs = xc - dir_cx(i);
    xs = xs < 0 ? g.nx - 1 : (xs >= g.nx ? 0 : xs);
    int ys = y - dir_cy(i);
    ys = ys < 0 ? g.ny - 1 : (ys >= g.ny ? 0 : ys);
    if (mask_solid(mask, g.mask_words, xs, ys))
      out[i] = load_one<ST>(R + dir_opp(i) * g.plane + cell_index(g, xc, y), dir_opp(i), sc);
    else
      out[i] = load_one<ST>(R + i * g.plane + cell_index(g, xs, ys), i, sc);
  }
}

// R from a post-streaming state: the preimage by streaming. Slot (c, i) streams to (c + e_i, i),
// or bounces to (c, opp i) when c + e_i is solid; slots leaving an open domain are never read.
// src: either a v0-layout state (aos != nullptr) or the uniform equilibrium eq.
template <class ST>
__global__ void set_state_kernel(ST* __restrict__ R, const uint32_t* __restrict__ mask,
                                 const Grid2D g, const typename StoreTraits<ST>::T* __restrict__ aos,
                                 const Eq9<typename StoreTraits<ST>::T> eq, const PlaneScales sc) {
  using T = typename StoreTraits<ST>::T;
  const long long n = static_cast<long long>(g.nx) * g.ny;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    const bool solid = mask_solid(mask, g.mask_words, x, y);
#pragma unroll
    for (int i = 0; i < kQ; ++i) {
      T v = T(0);
      if (!solid) {
        const int xn_raw = x + dir_cx(i);
        const bool leaves = g.open_x && (xn_raw < 0 || xn_raw >= g.nx);
        const int xn = xn_raw < 0 ? g.nx - 1 : (xn_raw >= g.nx ? 0 : xn_raw);
        int yn = y + dir_cy(i);
        yn = yn < 0 ? g.ny - 1 : (yn >= g.ny ? 0 : yn);
        const bool bounce = !leaves && mask_solid(mask, g.mask_words, xn, yn);
        if (aos) {
          const long long cn = static_cast<long long>(yn) * g.nx + xn;
          v = leaves ? aos[c * kQ + i] : (bounce ? aos[c * kQ + dir_opp(i)] : aos[cn * kQ + i]);
        } else {
          v = bounce ? eq.v[dir_opp(i)] : eq.v[i];
        }
      }
      R[i * g.plane + cell_index(g, x, y)] = encode<ST>(v, i, sc);
    }
  }
}

// Pull state -> post-streaming state in v0 layout (solid cells 0).
template <class ST>
__global__ void get_state_kernel(const ST* __restrict__ R, const uint32_t* __restrict__ mask,
                                 const Grid2D g, const Eq9<typename StoreTraits<ST>::T> eq_in,
                                 const PlaneScales sc, typename StoreTraits<ST>::T* __restrict__ aos) {
  using T = typename StoreTraits<ST>::T;
  const long long n = static_cast<long long>(g.nx) * g.ny;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    T s[kQ];
    if (mask_solid(mask, g.mask_words, x, y)) {
#pragma unroll
      for (int i = 0; i < kQ; ++i) s[i] = T(0);
    } else {
      gather_cell<ST>(R, mask, g, x, y, eq_in, sc, s);
    }
#pragma unroll
    for (int i = 0; i < kQ; ++i) aos[c * kQ + i] = s[i];
  }
}

// Moment pass: rho, ux, uy (row-major nx*ny) of the post-streaming state, reference
// macroscopic() arithmetic (src/v0_cpu/solver_v0.cpp:111-123) under policy A.
template <class ST, class A>
__global__ void moments_kernel(const ST* __restrict__ R, const uint32_t* __restrict__ mask,
                               const Grid2D g, const Eq9<typename StoreTraits<ST>::T> eq_in,
                               const PlaneScales sc, typename A::T hfx, typename A::T hfy,
                               typename A::T* __restrict__ rho, typename A::T* __restrict__ ux,
                               typename A::T* __restrict__ uy) {
  using T = typename A::T;
  const long long n = static_cast<long long>(g.nx) * g.ny;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    T r = T(0), u = T(0), v = T(0);
    if (!mask_solid(mask, g.mask_words, x, y)) {
      T s[kQ];
      gather_cell<ST>(R, mask, g, x, y, eq_in, sc, s);
      moments_exact<A>(s, hfx, hfy, r, u, v);
    }
    rho[c] = r;
    ux[c] = u;
    uy[c] = v;
  }
}

constexpr int kReduceThreads = 256;

// Block sum of a double (fixed order for a fixed launch shape).
__device__ __forceinline__ double block_sum(double v, double* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < static_cast<int>(blockDim.x >> 5) ? smem[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// First pass of the mass reduction: per-block sums of all fluid post-streaming populations,
// accumulated in double (each cell's 9 values in order i = 0..8, then a fixed tree).
template <class ST>
__global__ void __launch_bounds__(kReduceThreads)
    mass_partial_kernel(const ST* __restrict__ R, const uint32_t* __restrict__ mask,
                        const Grid2D g, const Eq9<typename StoreTraits<ST>::T> eq_in,
                        const PlaneScales sc, double* __restrict__ partials) {
  using T = typename StoreTraits<ST>::T;
  __shared__ double smem[32];
  const long long n = static_cast<long long>(g.nx) * g.ny;
  double acc = 0.0;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    if (mask_solid(mask, g.mask_words, x, y)) continue;
    T s[kQ];
    gather_cell<ST>(R, mask, g, x, y, eq_in, sc, s);
    double cell = 0.0;
#pragma unroll
    for (int i = 0; i < kQ; ++i) cell += static_cast<double>(s[i]);
    acc += cell;
  }
  const double b = block_sum(acc, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

// Second pass: one block adds the partials in a fixed order; out[0] = fluid_cells + sum.
static __global__ void __launch_bounds__(kReduceThreads)
    mass_final_kernel(const double* __restrict__ partials, int count, double fluid_cells,
                      double* __restrict__ out) {
  __shared__ double smem[32];
  double acc = 0.0;
  for (int k = threadIdx.x; k < count; k += blockDim.x) acc += partials[k];
  const double b = block_sum(acc, smem);
  if (threadIdx.x == 0) out[0] = fluid_cells + b;
}

// Sets *flag to 1 if any fluid population slot is not finite.
template <class ST>
__global__ void finite_kernel(const ST* __restrict__ R, const uint32_t* __restrict__ mask,
                              const Grid2D g, const PlaneScales sc, int* __restrict__ flag) {
  const long long n = static_cast<long long>(g.nx) * g.ny;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    if (mask_solid(mask, g.mask_words, x, y)) continue;
    bool bad = false;
#pragma unroll
    for (int i = 0; i < kQ; ++i) {
      const ST raw = R[i * g.plane + cell_index(g, x, y)];
      bad |= !isfinite(static_cast<double>(decode<ST>(raw, i, sc))) || stored_saturated<ST>(raw);
    }
    if (bad) atomicExch(flag, 1);
  }
}

// Advances the solver's device step counter (the stochastic-rounding key) after a launch
// sequence, inside a captured graph as well. The _dep form is launched with programmatic stream
// serialisation behind the step launches (it waits for the last one to complete before the
// add), so that the next sequence's first step launch is scheduled while it runs: +0.3-0.4 %
// on the benchmark's short timed regions of 2 to 8 steps per call.
static __global__ void counter_add_kernel(uint32_t* c, uint32_t n) { *c += n; }
static __global__ void counter_add_dep_kernel(uint32_t* c, uint32_t n) {
  grid_dependency_wait();
  *c += n;
}

// Copy of n16 16-byte words with coalesced vector loads and stores (a host buffer that kernels
// can address, e.g. pinned memory over NVLink-C2C, into device memory: the SMs' loads keep more
// bytes in flight than a copy engine on some hosts).
static __global__ void copy16_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, long long n16) {
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < n16;
       k += static_cast<long long>(gridDim.x) * blockDim.x)
    dst[k] = src[k];
}

// Momentum-exchange force on a body (halfway bounce-back, stationary walls): every link from a
// fluid cell x to a body cell x + c_i carries 2 c_i f*_i(x), with f*_i(x) = R_i(x) + w_i the
// post-collision population of x leaving along c_i (the pull state holds post-collision
// values), which bounces back unchanged. Links leaving an open x boundary carry nothing. FP64
// per-block partials of (F_x, F_y).
template <class ST>
__global__ void __launch_bounds__(kReduceThreads)
    body_force_partial_kernel(const ST* __restrict__ R, const uint32_t* __restrict__ mask,
                              const uint32_t* __restrict__ body, const Grid2D g,
                              const PlaneScales sc, double* __restrict__ partials) {
  __shared__ double smem[32];
  double ax = 0.0, ay = 0.0;
  const long long n = static_cast<long long>(g.nx) * g.ny;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    if (mask_solid(mask, g.mask_words, x, y)) continue;
#pragma unroll
    for (int i = 1; i < kQ; ++i) {
      int xn = x + dir_cx(i), yn = y + dir_cy(i);
      if (g.open_x && (xn < 0 || xn >= g.nx)) continue;
      xn = xn < 0 ? g.nx - 1 : (xn >= g.nx ? 0 : xn);
      yn = yn < 0 ? g.ny - 1 : (yn >= g.ny ? 0 : yn);
      if (!mask_solid(body, g.mask_words, xn, yn)) continue;
      const double f = static_cast<double>(load_one<ST>(R + i * g.plane + cell_index(g, x, y), i, sc)) +
                       weight<double>(i);
      ax += 2.0 * dir_cx(i) * f;
      ay += 2.0 * dir_cy(i) * f;
    }
  }
  const double bx = block_sum(ax, smem);
  const double by = block_sum(ay, smem);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = bx;
    partials[2 * blockIdx.x + 1] = by;
  }
}

// Sum of `count` (x, y) partial pairs into out[0..1].
static __global__ void __launch_bounds__(kReduceThreads)
    pair_final_kernel(const double* __restrict__ partials, int count, double* __restrict__ out) {
  __shared__ double smem[32];
  double ax = 0.0, ay = 0.0;
  for (int k = threadIdx.x; k < count; k += blockDim.x) {
    ax += partials[2 * k];
    ay += partials[2 * k + 1];
  }
  const double bx = block_sum(ax, smem);
  const double by = block_sum(ay, smem);
  if (threadIdx.x == 0) {
    out[0] = bx;
    out[1] = by;
  }
}

// Gather of one cell (velocity probe).
template <class ST>
__global__ void probe_kernel(const ST* __restrict__ R, const uint32_t* __restrict__ mask,
                             const Grid2D g, const Eq9<typename StoreTraits<ST>::T> eq_in,
                             const PlaneScales sc, int x, int y,
                             typename StoreTraits<ST>::T* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  typename StoreTraits<ST>::T s[kQ];
  gather_cell<ST>(R, mask, g, x, y, eq_in, sc, s);
#pragma unroll
  for (int i = 0; i < kQ; ++i) out[i] = s[i];
}

}  // namespace lbm_b200
