// Fused pull stream-collide step: the hot path.
//
// Replaces the reference's step_kernel<kPull=true, kNoModulo=true, kOpen> (src/v3_cuda_opt/
// solver_v3.cu:45-113); same mathematics, different machine mapping:
//   * one warp owns a chunk of 32*G consecutive cells of one row, each lane G consecutive cells
//     (G = 16 bytes / stored element: 4 in FP32, 2 in FP64, 8 with 16-bit storage), so every
//     population plane is read and written with one aligned 16-byte vector per lane;
//   * in the pull scheme each stored slot is read exactly once per step, so nothing needs to be
//     staged for reuse: the shift by one cell along x is a lane-local register shift plus one warp
//     shuffle, and only the two end lanes of a chunk read one extra element (an L1/L2 hit: the
//     neighbouring chunk is processed by the neighbouring warp at the same time);
//   * the y shift is a different row of the same plane (no re-read of any row);
//   * solid neighbours come from the bit-packed mask (3 funnel-shifted words per lane); a
//     bounce-back vector load is issued only by lanes whose cells have a solid neighbour in that
//     direction (walls and obstacles only);
//   * persistent grid-stride loop over chunks, warps taking consecutive chunks;
//   * warps whose cells are all solid skip the chunk (solid slots hold 0 in both buffers).
#pragma once

#include "lbm_device.cuh"

namespace lbm_b200 {

template <class ST, class Phys>
struct StepArgs {
  using T = typename StoreTraits<ST>::T;
  const ST* __restrict__ src;
  ST* __restrict__ dst;
  const uint32_t* __restrict__ mask;
  Grid2D g;
  int cpr;    // chunks per row: ceil(nx / (32 G))
  int items;  // ny * cpr
  typename Phys::Consts k;
  T eq_in[kQ];  // inlet equilibrium (open domain)
  PlaneScales sc;
};

// Exact (bit-for-bit with v0) physics for FP32 / FP64 storage.
template <class A>
struct ExactPhys {
  using T = typename A::T;
  using Consts = CollideConsts<T>;
  static __device__ __forceinline__ void collide(const T (&g)[kQ], const Consts& k, T (&o)[kQ]) {
    collide_exact<A>(g, k, o);
  }
};

constexpr int kStepThreads = 256;

// Source row of plane i for destination row y: y - cy_i (periodic).
__device__ __forceinline__ int src_row(int i, int y, int ym, int yp) {
  return dir_cy(i) == 1 ? ym : (dir_cy(i) == -1 ? yp : y);
}

template <class ST, class Phys, bool kOpen>
__global__ void __launch_bounds__(kStepThreads)
    pull_step_kernel(const StepArgs<ST, Phys> p) {
  using T = typename StoreTraits<ST>::T;
  constexpr int G = StoreTraits<ST>::kVec;
  constexpr uint32_t kFull = (1u << G) - 1u;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nx = p.g.nx, ny = p.g.ny, pitch = p.g.pitch;
  const long long plane = p.g.plane;

  for (int item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; item < p.items; item += nwarps) {
    const int y = item / p.cpr;
    const int x0 = (item - y * p.cpr) * (32 * G) + lane * G;
    const bool active = x0 < nx;
    const int ym = y == 0 ? ny - 1 : y - 1;
    const int yp = y == ny - 1 ? 0 : y + 1;

    // Mask windows: bit j = solid(x0 - 1 + j) in rows y - 1, y, y + 1.
    const uint32_t* mrow = p.mask + static_cast<size_t>(y) * p.g.mask_words;
    const uint32_t w0 = mask_window(mrow, x0);
    const uint32_t wm = mask_window(p.mask + static_cast<size_t>(ym) * p.g.mask_words, x0);
    const uint32_t wp = mask_window(p.mask + static_cast<size_t>(yp) * p.g.mask_words, x0);
    // Cells of this lane that are solid or past the row end produce 0.
    const int valid = nx - x0;
    uint32_t own = (w0 >> 1) & kFull;
    if (valid < G) own |= valid <= 0 ? kFull : (kFull & ~((1u << valid) - 1u));
    if (__all_sync(0xffffffffu, own == kFull)) continue;

    // Streamed values: plane i, source row y - cy_i, cells x0 - cx_i .. x0 - cx_i + G - 1.
    T v[kQ][G];
#pragma unroll
    for (int i = 0; i < kQ; ++i) {
      const ST* rowp = p.src + i * plane + static_cast<long long>(src_row(i, y, ym, yp)) * pitch;
      if (active) {
        load_vec<ST>(rowp + x0, v[i], i, p.sc);
      } else {
#pragma unroll
        for (int k = 0; k < G; ++k) v[i][k] = T(0);
      }
    }
#pragma unroll
    for (int i = 1; i < kQ; ++i) {
      const ST* rowp = p.src + i * plane + static_cast<long long>(src_row(i, y, ym, yp)) * pitch;
      if (dir_cx(i) == 1) {
        // cell x0 + k reads x0 + k - 1: shift up, the first element from the lane to the left
        T left = __shfl_up_sync(0xffffffffu, v[i][G - 1], 1);
        if (lane == 0) {  // lane 0 is always active (a chunk exists only if it holds cells)
          if (!kOpen || x0 > 0) left = load_one<ST>(rowp + (x0 > 0 ? x0 - 1 : nx - 1), i, p.sc);
        }
#pragma unroll
        for (int k = G - 1; k > 0; --k) v[i][k] = v[i][k - 1];
        v[i][0] = left;
      } else if (dir_cx(i) == -1) {
        // cell x0 + k reads x0 + k + 1: shift down, the last element from the lane to the right
        T right = __shfl_down_sync(0xffffffffu, v[i][0], 1);
        if (lane == 31 && active) right = load_one<ST>(rowp + (x0 + G < nx ? x0 + G : 0), i, p.sc);
#pragma unroll
        for (int k = 0; k < G - 1; ++k) v[i][k] = v[i][k + 1];
        v[i][G - 1] = right;
        if (!kOpen) {
          // periodic wrap: cell nx - 1 reads x = 0
          const int kl = nx - 1 - x0;
          if (kl >= 0 && kl < G) {
            const T w = load_one<ST>(rowp, i, p.sc);
#pragma unroll
            for (int k = 0; k < G; ++k)
              if (k == kl) v[i][k] = w;
          }
        }
      }
    }

    // Halfway bounce-back: population i of a fluid cell whose source cell is solid is the
    // outgoing population opp(i) of the cell itself.
#pragma unroll
    for (int i = 1; i < kQ; ++i) {
      const uint32_t w = dir_cy(i) == 1 ? wm : (dir_cy(i) == -1 ? wp : w0);
      const uint32_t bounce = (w >> (1 - dir_cx(i))) & kFull & ~own;
      if (bounce) {
        T b[G];
        load_vec<ST>(p.src + dir_opp(i) * plane + static_cast<long long>(y) * pitch + x0, b,
                     dir_opp(i), p.sc);
#pragma unroll
        for (int k = 0; k < G; ++k)
          if ((bounce >> k) & 1u) v[i][k] = b[k];
      }
    }

    if (kOpen) {
      // Inlet (x = 0): populations entering with c_x = +1 are the inlet equilibrium.
      if (x0 == 0) {
        v[1][0] = p.eq_in[1];
        v[5][0] = p.eq_in[5];
        v[8][0] = p.eq_in[8];
      }
      // Outlet (x = nx - 1): populations entering with c_x = -1 are those the cell x = nx - 2
      // receives (reference src/v3_cuda_opt/solver_v3.cu:66-73).
      const int kl = nx - 1 - x0;
      if (kl >= 0 && kl < G) {
#pragma unroll
        for (int i = 1; i < kQ; ++i) {
          if (dir_cx(i) != -1) continue;
          const int r = src_row(i, y, ym, yp);
          const uint32_t w = dir_cy(i) == 1 ? wm : (dir_cy(i) == -1 ? wp : w0);
          const bool solid_src = (w >> (kl + 1)) & 1u;
          const T val = solid_src
                            ? load_one<ST>(p.src + dir_opp(i) * plane +
                                               static_cast<long long>(y) * pitch + (nx - 2),
                                           dir_opp(i), p.sc)
                            : load_one<ST>(p.src + i * plane + static_cast<long long>(r) * pitch +
                                               (nx - 1),
                                           i, p.sc);
#pragma unroll
          for (int k = 0; k < G; ++k)
            if (k == kl) v[i][k] = val;
        }
      }
    }

    // Collide each cell and store the 9 planes of the own cells.
    T out[kQ][G];
#pragma unroll
    for (int k = 0; k < G; ++k) {
      T gin[kQ], o[kQ];
#pragma unroll
      for (int i = 0; i < kQ; ++i) gin[i] = v[i][k];
      Phys::collide(gin, p.k, o);
      const bool solid = (own >> k) & 1u;
#pragma unroll
      for (int i = 0; i < kQ; ++i) out[i][k] = solid ? T(0) : o[i];
    }
    if (active) {
#pragma unroll
      for (int i = 0; i < kQ; ++i)
        store_vec<ST>(p.dst + i * plane + static_cast<long long>(y) * pitch + x0, out[i], i,
                      p.sc);
    }
  }
}

}  // namespace lbm_b200
