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
//   * persistent grid-stride loop over chunks, warps taking consecutive chunks; with kPrefetch the
//     9 plane vectors of the warp's next chunk are loaded while the current chunk is computed,
//     which keeps every warp's loads in flight through the collision;
//   * warps whose cells are all solid skip the chunk (solid slots are never read).
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
  const uint32_t* step_ctr;  // lattice steps taken before this launch sequence (device counter)
  uint32_t step_off;         // index of this launch in the sequence
  long long key_base;        // cell offset of this grid in the rounding hash (batched instances)
  // Strip engine (kernels built with kHalo): the step also writes the populations leaving the
  // strip through its top owned row (c_y = +1: 2, 5, 6) into ghost row 0 of the strip above, and
  // those leaving through its bottom owned row (c_y = -1: 4, 7, 8) into ghost row n + 1 of the
  // strip below. halo[0..3]: offset of that ghost row of the strip above from dst, its plane
  // stride, the same for the strip below (read only when a boundary row is stored).
  const long long* halo;
};

// Stochastic-rounding key of the step a launch performs (16-bit forms): the step index comes
// from a device counter plus the launch's offset, so that graph replays draw fresh keys.
template <class ST, class Phys>
__device__ __forceinline__ uint32_t step_rkey(const StepArgs<ST, Phys>& p) {
  return sr_step_key(__ldg(p.step_ctr) + p.step_off);
}

// Exact (bit-for-bit with v0) physics, one cell at a time (FP64).
template <class A>
struct ExactPhys {
  using Arith = A;
  using T = typename A::T;
  using Consts = CollideConsts<T>;
  template <int G>
  static __device__ __forceinline__ void collide_all(const T (&v)[kQ][G], const Consts& k,
                                                     T (&out)[kQ][G]) {
#pragma unroll
    for (int c = 0; c < G; ++c) {
      T g[kQ], o[kQ];
#pragma unroll
      for (int i = 0; i < kQ; ++i) g[i] = v[i][c];
      collide_exact<A>(g, k, o);
#pragma unroll
      for (int i = 0; i < kQ; ++i) out[i][c] = o[i];
    }
  }
};

// Exact FP32 physics, two cells per packed instruction: the same correctly rounded operations
// per cell as ExactPhys<ExactF32>, so the same bits.
struct ExactPhysF32x2 {
  using T = float;
  using Consts = CollideConsts<float>;
  template <int G>
  static __device__ __forceinline__ void collide_all(const float (&v)[kQ][G], const Consts& k,
                                                     float (&out)[kQ][G]) {
    static_assert(G % 2 == 0, "cells are collided in pairs");
    CollideConsts<float2> k2;
    k2.omega = make_float2(k.omega, k.omega);
    k2.force_prefactor = make_float2(k.force_prefactor, k.force_prefactor);
    k2.fx = make_float2(k.fx, k.fx);
    k2.fy = make_float2(k.fy, k.fy);
    k2.hfx = make_float2(k.hfx, k.hfx);
    k2.hfy = make_float2(k.hfy, k.hfy);
    k2.cf_x = make_float2(k.cf_x, k.cf_x);
    k2.cf_y = make_float2(k.cf_y, k.cf_y);
    k2.cf_p = make_float2(k.cf_p, k.cf_p);
    k2.cf_q = make_float2(k.cf_q, k.cf_q);
#pragma unroll
    for (int c = 0; c < G; c += 2) {
      float2 g[kQ], o[kQ];
#pragma unroll
      for (int i = 0; i < kQ; ++i) g[i] = make_float2(v[i][c], v[i][c + 1]);
      collide_exact<ExactF32x2>(g, k2, o);
#pragma unroll
      for (int i = 0; i < kQ; ++i) {
        out[i][c] = o[i].x;
        out[i][c + 1] = o[i].y;
      }
    }
  }
};

// FP32 physics of the 16-bit storage forms (FMA, one reciprocal; not bit-exact), two cells per
// packed instruction.
struct FastPhys {
  using T = float;
  using Consts = FastConsts;
  template <int G>
  static __device__ __forceinline__ void collide_all(const float (&v)[kQ][G], const Consts& k,
                                                     float (&out)[kQ][G]) {
    static_assert(G % 2 == 0, "cells are collided in pairs");
#pragma unroll
    for (int c = 0; c < G; c += 2) {
      float2 g[kQ], o[kQ];
#pragma unroll
      for (int i = 0; i < kQ; ++i) g[i] = make_float2(v[i][c], v[i][c + 1]);
      collide_fast_t<FastF32x2>(g, k, o);
#pragma unroll
      for (int i = 0; i < kQ; ++i) {
        out[i][c] = o[i].x;
        out[i][c + 1] = o[i].y;
      }
    }
  }
};

constexpr int kStepThreads = 256;

// Source row of plane i for destination row y: y - cy_i (periodic).
__device__ __forceinline__ int src_row(int i, int y, int ym, int yp) {
  return dir_cy(i) == 1 ? ym : (dir_cy(i) == -1 ? yp : y);
}

// Position of one warp chunk.
struct Chunk {
  int y, ym, yp, x0;
  bool active;  // this lane owns at least one cell
};

template <int G>
__device__ __forceinline__ Chunk chunk_at(int item, int cpr, int nx, int ny, int lane) {
  Chunk c;
  c.y = item / cpr;
  c.x0 = (item - c.y * cpr) * (32 * G) + lane * G;
  c.active = c.x0 < nx;
  c.ym = c.y == 0 ? ny - 1 : c.y - 1;
  c.yp = c.y == ny - 1 ? 0 : c.y + 1;
  return c;
}

// The 9 aligned plane vectors of a chunk: plane i, row y - cy_i, cells x0 .. x0 + G - 1.
template <class ST, class Phys, int G>
__device__ __forceinline__ void load_planes(const StepArgs<ST, Phys>& p, const Chunk& c,
                                            typename StoreTraits<ST>::T (&v)[kQ][G]) {
  using T = typename StoreTraits<ST>::T;
#pragma unroll
  for (int i = 0; i < kQ; ++i) {
    if (c.active) {
      VecIO<ST, G>::load(p.src + i * p.g.plane + static_cast<long long>(src_row(i, c.y, c.ym, c.yp)) * p.g.pitch + c.x0,
                         v[i], i, p.sc);
    } else {
#pragma unroll
      for (int k = 0; k < G; ++k) v[i][k] = T(0);
    }
  }
}

// Shift, bounce-back, open-boundary rules, collision and store of one chunk whose aligned plane
// vectors are in v (consumed).
template <class ST, class Phys, bool kOpen, int G>
__device__ __forceinline__ void process_chunk(const StepArgs<ST, Phys>& p, const Chunk& c,
                                              typename StoreTraits<ST>::T (&v)[kQ][G], int lane) {
  using T = typename StoreTraits<ST>::T;
  constexpr uint32_t kFull = (1u << G) - 1u;
  const int nx = p.g.nx, pitch = p.g.pitch, x0 = c.x0, y = c.y;
  const long long plane = p.g.plane;

  // Mask windows: bit j = solid(x0 - 1 + j) in rows y - 1, y, y + 1.
  const uint32_t w0 = mask_window(p.mask + static_cast<size_t>(y) * p.g.mask_words, x0);
  const uint32_t wm = mask_window(p.mask + static_cast<size_t>(c.ym) * p.g.mask_words, x0);
  const uint32_t wp = mask_window(p.mask + static_cast<size_t>(c.yp) * p.g.mask_words, x0);
  // Cells of this lane that are solid or past the row end produce 0.
  const int valid = nx - x0;
  uint32_t own = (w0 >> 1) & kFull;
  if (valid < G) own |= valid <= 0 ? kFull : (kFull & ~((1u << valid) - 1u));
  if (__all_sync(0xffffffffu, own == kFull)) return;

#pragma unroll
  for (int i = 1; i < kQ; ++i) {
    const ST* rowp = p.src + i * plane + static_cast<long long>(src_row(i, y, c.ym, c.yp)) * pitch;
    if (dir_cx(i) == 1) {
      // cell x0 + k reads x0 + k - 1: shift up, the first element from the lane to the left
      T left = __shfl_up_sync(0xffffffffu, v[i][G - 1], 1);
      if (lane == 0) {  // lane 0 is always active (a chunk exists only if it holds cells)
        if (!kOpen || x0 > 0) left = load_step<ST>(rowp + (x0 > 0 ? x0 - 1 : nx - 1));
      }
#pragma unroll
      for (int k = G - 1; k > 0; --k) v[i][k] = v[i][k - 1];
      v[i][0] = left;
    } else if (dir_cx(i) == -1) {
      // cell x0 + k reads x0 + k + 1: shift down, the last element from the lane to the right
      T right = __shfl_down_sync(0xffffffffu, v[i][0], 1);
      if (lane == 31 && c.active) right = load_step<ST>(rowp + (x0 + G < nx ? x0 + G : 0));
#pragma unroll
      for (int k = 0; k < G - 1; ++k) v[i][k] = v[i][k + 1];
      v[i][G - 1] = right;
      if (!kOpen) {
        // periodic wrap: cell nx - 1 reads x = 0
        const int kl = nx - 1 - x0;
        if (kl >= 0 && kl < G) {
          const T w = load_step<ST>(rowp);
#pragma unroll
          for (int k = 0; k < G; ++k)
            if (k == kl) v[i][k] = w;
        }
      }
    }
  }

  // Halfway bounce-back: population i of a fluid cell whose source cell is solid is the
  // outgoing population opp(i) of the cell itself. Chunks without any solid cell in their three
  // rows (almost all of them) skip this section as a whole warp.
  constexpr uint32_t kWin = (1u << (G + 2)) - 1u;
  if (__any_sync(0xffffffffu, ((wm | w0 | wp) & kWin) != 0u)) {
#pragma unroll
  for (int i = 1; i < kQ; ++i) {
    const uint32_t w = dir_cy(i) == 1 ? wm : (dir_cy(i) == -1 ? wp : w0);
    const uint32_t bounce = (w >> (1 - dir_cx(i))) & kFull & ~own;
    if (bounce) {
      T b[G];
      VecIO<ST, G>::load(p.src + dir_opp(i) * plane + static_cast<long long>(y) * pitch + x0, b,
                         dir_opp(i), p.sc);
#pragma unroll
      for (int k = 0; k < G; ++k)
        if ((bounce >> k) & 1u) v[i][k] = b[k];
    }
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
        const int r = src_row(i, y, c.ym, c.yp);
        const uint32_t w = dir_cy(i) == 1 ? wm : (dir_cy(i) == -1 ? wp : w0);
        const bool solid_src = (w >> (kl + 1)) & 1u;
        const T val = solid_src
                          ? load_step<ST>(p.src + dir_opp(i) * plane +
                                             static_cast<long long>(y) * pitch + (nx - 2))
                          : load_step<ST>(p.src + i * plane + static_cast<long long>(r) * pitch +
                                             (nx - 1));
#pragma unroll
        for (int k = 0; k < G; ++k)
          if (k == kl) v[i][k] = val;
      }
    }
  }

  // Collide each cell and store the 9 planes of the own cells. Solid and padding cells are
  // collided too and their slots receive whatever that gives: no kernel ever reads a solid slot
  // (a fluid cell whose source is solid bounces back instead, and every gather, moment and
  // reduction skips solid cells), so no per-cell select is spent on them.
  T out[kQ][G];
  Phys::template collide_all<G>(v, p.k, out);
  if (c.active) {
    using SS = StepStore<ST, G>;
    uint32_t ph[SS::kPairs];
    if constexpr (SS::kSr) SS::hashes(p.key_base + static_cast<long long>(y) * pitch + x0, step_rkey(p), ph);
#pragma unroll
    for (int i = 0; i < kQ; ++i)
      SS::store(p.dst + i * plane + static_cast<long long>(y) * pitch + x0, out[i], i, p.sc, ph);
  }
}

// Kernel variants (same results, different register budget / memory-level parallelism):
//   0: loads at the top of each chunk, compiler-chosen registers;
//   1: next chunk prefetched into registers, at least 2 blocks of 256 threads per SM;
//   2: loads at the top of each chunk, at least 4 blocks per SM (64 registers);
//   3: next chunk prefetched, at least 3 blocks per SM.
constexpr int kStepVariants = 4;
template <int V>
struct VariantTraits {
  static constexpr bool prefetch = (V == 1 || V == 3);
  static constexpr int min_blocks = V == 0 ? 1 : (V == 1 ? 2 : (V == 2 ? 4 : 3));
};

template <class ST, class Phys, bool kOpen, int kVariant>
__global__ void __launch_bounds__(kStepThreads, VariantTraits<kVariant>::min_blocks)
    pull_step_kernel(const StepArgs<ST, Phys> p) {
  using T = typename StoreTraits<ST>::T;
  constexpr int G = StoreTraits<ST>::kVec;
  grid_dependency_wait();
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  int item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (item >= p.items) return;
  if (!VariantTraits<kVariant>::prefetch) {
#pragma unroll 1
    for (; item < p.items; item += nwarps) {
      const Chunk c = chunk_at<G>(item, p.cpr, p.g.nx, p.g.ny, lane);
      T v[kQ][G];
      load_planes<ST, Phys, G>(p, c, v);
      process_chunk<ST, Phys, kOpen, G>(p, c, v, lane);
    }
  } else {
    Chunk c = chunk_at<G>(item, p.cpr, p.g.nx, p.g.ny, lane);
    T v[kQ][G];
    load_planes<ST, Phys, G>(p, c, v);
#pragma unroll 1
    for (; item < p.items; item += nwarps) {
      const int next = item + nwarps;
      Chunk cn = c;
      T vn[kQ][G];
      if (next < p.items) {
        cn = chunk_at<G>(next, p.cpr, p.g.nx, p.g.ny, lane);
        load_planes<ST, Phys, G>(p, cn, vn);
      }
      process_chunk<ST, Phys, kOpen, G>(p, c, v, lane);
      c = cn;
#pragma unroll
      for (int i = 0; i < kQ; ++i)
#pragma unroll
        for (int k = 0; k < G; ++k) v[i][k] = vn[i][k];
    }
  }
}

}  // namespace lbm_b200
