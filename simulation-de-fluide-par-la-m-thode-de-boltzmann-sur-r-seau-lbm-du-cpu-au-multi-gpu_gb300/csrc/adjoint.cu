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
//
// Data path: both sweeps run on the warp-specialised shared-memory ring of the step kernels
// (step_ring.cuh). States are pitched planes like the solver's (row pitch a multiple of 128
// bytes); a tile is 256 or 512 consecutive cells (one or two per consumer lane) of one row of
// one instance, the tiles of all instances form one index that the blocks stride over, and the
// producer warp stages per tile:
//   forward:  the 9 pull rows (rows y - c_y of the state, 16-byte halo each side), the 3 mask
//             rows, the periodic wrap blocks and the alpha row;
//   backward: the same pull rows, the 9 transpose rows of the next step's adjoint (rows
//             y + c_y), their wrap blocks, the alpha row and the per-segment alpha_bar row.
// Solid neighbours come from the bit-packed mask (no per-cell code array). The objective and the
// parameter gradients are summed per lane, then per warp (fixed shuffle tree) into one FP64 slot
// per (instance, block, warp), accumulated across launches and reduced per instance in a fixed
// order at the end of a sweep: sums are deterministic, no atomics, and no warp waits on another.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "lbm_b200.h"
#include "lbm_device.cuh"
#include "solver_internal.h"
#include "fastdiv.h"
#include "step_ring.cuh"

using namespace lbm_b200;

namespace {

constexpr int kAdjW = 8;            // consumer warps per block
// Producer warps per block (tile_pipeline). One: a second one, which speeds up the batched
// ensemble's many short copies, made both adjoint kernels slower (27.8 -> 28.4 us forward,
// 72.8 -> 75.6 us backward on the 512 x 128 x 32 benchmark batch).
constexpr int kAdjProd = 1;
constexpr int kAdjThreads = 32 * (kAdjW + kAdjProd);
constexpr int kAuxThreads = 256;    // state conversion, field casts, slot sums

// Geometry shared by all instances. A state is 9 pitched planes; per-cell fields (alpha and its
// adjoint) are one pitched plane per instance.
struct AdjGeom {
  int nx, ny, pitch, mask_words, batch;
  long long plane;  // cells per pitched plane (ny * pitch)
  long long inst;   // elements per instance state (9 planes)
};

// Tile shape: kC cells per lane (one at a time), a tile of TW = 256 kC cells of one row,
// 16-byte halos (RingShape with one cell per lane and pass).
template <class T, int kC>
using AdjRing = RingShape<T, kAdjW, kC>;

// Stage layouts (byte offsets; every part starts on a 16-byte boundary).
template <class T, int kC>
struct FwdStage {
  using S = AdjRing<T, kC>;
  static constexpr int kMask = S::kPlaneBytes;
  static constexpr int kWrap = kMask + S::kMaskBytes;
  static constexpr int kAlpha = kWrap + S::kWrapBytes;
  static constexpr int kBytes = kAlpha + S::TW * static_cast<int>(sizeof(T));
  static_assert(kBytes % 16 == 0, "stages must stay 16-byte aligned");
};
template <class T, int kC>
struct BwdStage {
  using S = AdjRing<T, kC>;
  static constexpr int kZ = S::kPlaneBytes;
  static constexpr int kMask = 2 * S::kPlaneBytes;
  static constexpr int kWrapR = kMask + S::kMaskBytes;
  static constexpr int kWrapZ = kWrapR + S::kWrapBytes;
  static constexpr int kAlpha = kWrapZ + S::kWrapBytes;
  static constexpr int kAseg = kAlpha + S::TW * static_cast<int>(sizeof(T));
  static constexpr int kBytes = kAseg + S::TW * static_cast<int>(sizeof(T));
  static_assert(kBytes % 16 == 0, "stages must stay 16-byte aligned");
};

constexpr size_t adj_smem_bytes(int stage_bytes, int stages) {
  return static_cast<size_t>(stages) * stage_bytes + 2 * stages * sizeof(uint64_t);
}

// Tiles of all instances in one index: tile = (b * ny + y) * tiles_per_row + tile_in_row, so
// that the load is even whatever the batch. The ring pipeline hands block k the grid-stride
// sequence k, k + G, k + 2 G, ... (G blocks); tile_pos maps its i-th element to the i-th tile of
// the block's contiguous chunk k q + min(k, r) .. (total = q G + r; both sequences have
// q + (k < r) elements), so that a block's tiles of one instance are consecutive and its
// per-instance partial sums are written once per launch.
struct AdjTiles {
  FastDiv per_inst, per_row, grid;  // tiles per instance, tiles per row, blocks
  int total, q, r;
};

struct TilePos {
  int b, y, ym, yp, tx0;
};
// reverse: the tile order is mirrored (alternate steps start on the rows the previous step
// wrote last, still in L2).
template <int kTW>
__device__ __forceinline__ TilePos tile_pos(const AdjGeom& g, const AdjTiles& at, int tile, int reverse) {
  const uint32_t i = at.grid.div(static_cast<uint32_t>(tile));
  const uint32_t k = static_cast<uint32_t>(tile) - i * at.grid.d;
  uint32_t lin = k * static_cast<uint32_t>(at.q) + min(k, static_cast<uint32_t>(at.r)) + i;
  if (reverse) lin = static_cast<uint32_t>(at.total) - 1u - lin;
  TilePos t;
  t.b = static_cast<int>(at.per_inst.div(lin));
  const uint32_t r = lin - static_cast<uint32_t>(t.b) * at.per_inst.d;
  t.y = static_cast<int>(at.per_row.div(r));
  t.tx0 = static_cast<int>(r - static_cast<uint32_t>(t.y) * at.per_row.d) * kTW;
  t.ym = t.y == 0 ? g.ny - 1 : t.y - 1;
  t.yp = t.y == g.ny - 1 ? 0 : t.y + 1;
  return t;
}

template <class T>
struct FwdArgs {
  const T* R;              // state t of instance 0
  T* Rn;                   // state t + 1 of instance 0, or null (objective only)
  const T* alpha;          // alpha field of instance 0, or null (zero field)
  const uint32_t* mask;    // bit-packed, periodic ghost bits
  AdjGeom g;
  AdjTiles at;
  CollideConsts<T> k;      // the collision's constants (cf_* unused: the force is per cell)
  double* obj;             // per-warp slots [instance][block][warp] accumulating sum u_x, or null
  int reverse;             // walk the tiles from the last (alternate steps)
};

template <class T>
struct BwdArgs {
  const T* R;              // state t (linearisation point y_t = P R_t)
  const T* Z;              // adjoint ybar_{t+1}, or null (no later step)
  T* Yb;                   // adjoint ybar_t
  const T* alpha;          // or null
  T* aseg;                 // per-segment alpha_bar, or null (alpha gradient not requested)
  double* abar;            // alpha_bar, flushed into by the segment's last step (flush != 0)
  const uint32_t* mask;
  AdjGeom g;
  AdjTiles at;
  T omega, fp, fx, fy, hfx, hfy, obj_coef;
  int flush;
  double* grads;           // per-warp slots [instance][block][warp][omega_bar, fx_bar, fy_bar]
  int reverse;             // walk the tiles from the last (alternate steps)
};

// Row of plane j staged for the transpose gather: the source c + e_j lies in row y + c_y.
__device__ __forceinline__ int tr_row(int j, int y, int ym, int yp) {
  return dir_cy(j) == 1 ? yp : (dir_cy(j) == -1 ? ym : y);
}

// Extent of a tile's staged plane rows: cells tx0 - H .. tx0 + TW + H - 1 clipped to 0 .. pitch.
template <class S>
struct RowSpan {
  int xs, dst0;
  uint32_t bytes;
  __device__ __forceinline__ RowSpan(const AdjGeom& g, int tx0, int elem) {
    xs = tx0 - S::H > 0 ? tx0 - S::H : 0;
    const int xe = tx0 + S::TW + S::H < g.pitch ? tx0 + S::TW + S::H : g.pitch;
    bytes = static_cast<uint32_t>((xe - xs) * elem);
    dst0 = xs - (tx0 - S::H);
  }
};

// Bytes of a tile's per-cell field row (cells tx0 .. tx0 + TW - 1 clipped to the pitch).
template <class S>
__device__ __forceinline__ uint32_t field_bytes(const AdjGeom& g, int tx0, int elem) {
  const int xe = tx0 + S::TW < g.pitch ? tx0 + S::TW : g.pitch;
  return static_cast<uint32_t>((xe - tx0) * elem);
}

template <class S>
__device__ __forceinline__ void issue_mask_rows(unsigned char* dst, const uint32_t* mask, const AdjGeom& g,
                                                const TilePos& t, uint64_t* full) {
  uint32_t* sm = reinterpret_cast<uint32_t*>(dst);
  const int r3[3] = {t.ym, t.y, t.yp};
#pragma unroll
  for (int r = 0; r < 3; ++r)
    bulk_copy_g2s(sm + r * S::MW, mask + static_cast<size_t>(r3[r]) * g.mask_words + (t.tx0 >> 5), S::MW * 4,
                  full);
}

// Warp vote: does any cell of warp cw's strip (32 kC cells), or a neighbour of one, lie in a
// solid? Mask words w0 .. w0 + kC of the 3 staged rows, w0 = cw kC.
template <class S>
__device__ __forceinline__ bool strip_has_solid(const uint32_t* sm, int cw, int lane) {
  constexpr int kWords = S::WPS + 1;
  uint32_t mine = 0;
  if (lane < 3 * kWords) mine = sm[(lane / kWords) * S::MW + cw * S::WPS + lane % kWords];
  return __any_sync(0xffffffffu, mine != 0u);
}

// Neighbour bits of the lane's cell (staged mask word `word`, bit offset lane): bits 0, 1, 2 =
// cells x - 1, x, x + 1 of rows y - 1 (nm), y (n0), y + 1 (np).
struct Nbits {
  uint32_t nm, n0, np;
};
template <class S>
__device__ __forceinline__ Nbits cell_bits(const uint32_t* sm, int word, int lane) {
  Nbits b;
  b.nm = __funnelshift_r(sm[word], sm[word + 1], lane) & 7u;
  b.n0 = __funnelshift_r(sm[S::MW + word], sm[S::MW + word + 1], lane) & 7u;
  b.np = __funnelshift_r(sm[2 * S::MW + word], sm[2 * S::MW + word + 1], lane) & 7u;
  return b;
}
// Pull source c - e_i solid?
__device__ __forceinline__ bool pull_solid(const Nbits& b, int i) {
  const uint32_t w = dir_cy(i) == 1 ? b.nm : (dir_cy(i) == -1 ? b.np : b.n0);
  return (w >> (1 - dir_cx(i))) & 1u;
}
// Transpose source c + e_j solid?
__device__ __forceinline__ bool push_solid(const Nbits& b, int j) {
  const uint32_t w = dir_cy(j) == 1 ? b.np : (dir_cy(j) == -1 ? b.nm : b.n0);
  return (w >> (1 + dir_cx(j))) & 1u;
}

// Pull-gathered state of cell x of a tile from the staged rows: st plane rows (rows y - c_y),
// wr the wrap blocks (planes 1, 5, 8 at column nx - 1, planes 3, 6, 7 at column 0).
template <class T, class S>
__device__ __forceinline__ void staged_pull(const T* st, const T* wr, int nx, int x, int lx, T (&v)[kQ]) {
#pragma unroll
  for (int i = 0; i < kQ; ++i) v[i] = st[i * S::SROW + lx - dir_cx(i)];
  if (x == 0) {
    const int k = (nx - 1) & (S::H - 1);
    v[1] = wr[0 * S::H + k];
    v[5] = wr[1 * S::H + k];
    v[8] = wr[2 * S::H + k];
  }
  if (x == nx - 1) {
    v[3] = wr[3 * S::H];
    v[6] = wr[4 * S::H];
    v[7] = wr[5 * S::H];
  }
}

// Producer copies shared by both sweeps: the 9 pull rows of state R and their wrap blocks.
template <class T, class S>
__device__ __forceinline__ void issue_pull(unsigned char* st, unsigned char* wrap, const T* R, const AdjGeom& g,
                                           const TilePos& t, const RowSpan<S>& rs, bool lo, bool hi,
                                           uint64_t* full) {
  T* rows = reinterpret_cast<T*>(st);
#pragma unroll
  for (int i = 0; i < kQ; ++i)
    bulk_copy_g2s(rows + i * S::SROW + rs.dst0,
                  R + i * g.plane + static_cast<long long>(src_row(i, t.y, t.ym, t.yp)) * g.pitch + rs.xs, rs.bytes,
                  full);
  T* wr = reinterpret_cast<T*>(wrap);
  if (lo) {
    const int xb = (g.nx - 1) & ~(S::H - 1);
    for (int j = 0; j < 3; ++j) {
      const int i = wrap_dir(j);
      bulk_copy_g2s(wr + j * S::H, R + i * g.plane + static_cast<long long>(src_row(i, t.y, t.ym, t.yp)) * g.pitch + xb,
                    16, full);
    }
  }
  if (hi) {
    for (int j = 3; j < 6; ++j) {
      const int i = wrap_dir(j);
      bulk_copy_g2s(wr + j * S::H, R + i * g.plane + static_cast<long long>(src_row(i, t.y, t.ym, t.yp)) * g.pitch,
                    16, full);
    }
  }
}

// Warp sum (fixed shuffle tree) of one value per lane, added by lane 0 to *slot.
__device__ __forceinline__ void warp_add_to(double v, double* slot, int lane) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) *slot += v;
}

// Slot of (instance b, this block, consumer warp cw).
__device__ __forceinline__ long long warp_slot(int b, int cw) {
  return (static_cast<long long>(b) * gridDim.x + blockIdx.x) * kAdjW + cw;
}

// ---------------------------------------------------------------------------------------------
// Forward sweep
// ---------------------------------------------------------------------------------------------

template <class A, int kC>
struct AdjForward {
  using T = typename A::T;
  using S = AdjRing<T, kC>;
  using L = FwdStage<T, kC>;
  static constexpr bool kFinish = true;
  const FwdArgs<T>& p;
  int cur_b = -1;  // instance of the lane sums
  T usum = T(0);   // this lane's sum of u_x over the instance's cells it collided

  __device__ __forceinline__ void issue(int tile, unsigned char* base, uint64_t* full) const {
    const AdjGeom& g = p.g;
    const TilePos t = tile_pos<S::TW>(g, p.at, tile, p.reverse);
    const RowSpan<S> rs(g, t.tx0, sizeof(T));
    const bool lo = t.tx0 == 0, hi = t.tx0 + S::TW >= g.nx;
    const uint32_t fb = p.alpha ? field_bytes<S>(g, t.tx0, sizeof(T)) : 0u;
    mbar_arrive_expect_tx(full, kQ * rs.bytes + S::kMaskBytes + (lo ? 48u : 0u) + (hi ? 48u : 0u) + fb);
    issue_pull<T, S>(base, base + L::kWrap, p.R + t.b * g.inst, g, t, rs, lo, hi, full);
    issue_mask_rows<S>(base + L::kMask, p.mask, g, t, full);
    if (fb)
      bulk_copy_g2s(base + L::kAlpha, p.alpha + t.b * g.plane + static_cast<long long>(t.y) * g.pitch + t.tx0, fb,
                    full);
  }

  __device__ __forceinline__ void flush(int cw, int lane) {
    if (cur_b >= 0 && p.obj) warp_add_to(static_cast<double>(usum), p.obj + warp_slot(cur_b, cw), lane);
    usum = T(0);
  }

  __device__ __forceinline__ void cell(const TilePos& t, const unsigned char* base, int x, int word, int lane,
                                       bool solids) {
    const AdjGeom& g = p.g;
    const int lx = x - t.tx0 + S::H;
    T v[kQ];
    staged_pull<T, S>(reinterpret_cast<const T*>(base), reinterpret_cast<const T*>(base + L::kWrap), g.nx, x, lx, v);
    const long long c = static_cast<long long>(t.y) * g.pitch + x;
    T* d = p.Rn ? p.Rn + t.b * g.inst + c : nullptr;
    if (solids) {
      const Nbits nb = cell_bits<S>(reinterpret_cast<const uint32_t*>(base + L::kMask), word, lane);
      if (nb.n0 & 2u) {
        if (d) {
#pragma unroll
          for (int i = 0; i < kQ; ++i) d[i * g.plane] = T(0);
        }
        return;
      }
      if ((nb.nm | nb.n0 | nb.np) != 0u) {
        const T* R = p.R + t.b * g.inst + c;
#pragma unroll
        for (int i = 1; i < kQ; ++i)
          if (pull_solid(nb, i)) v[i] = __ldg(R + dir_opp(i) * g.plane);
      }
    }
    const T alpha = p.alpha ? reinterpret_cast<const T*>(base + L::kAlpha)[lx - S::H] : T(0);
    T out[kQ];
    const T ux = collide_exact_drag<A>(v, p.k, alpha, out);
    if (d) {
#pragma unroll
      for (int i = 0; i < kQ; ++i) d[i * g.plane] = out[i];
    }
    usum += ux;
  }

  __device__ __forceinline__ void consume(int tile, const unsigned char* base, int cw, int lane) {
    const AdjGeom& g = p.g;
    const TilePos t = tile_pos<S::TW>(g, p.at, tile, p.reverse);
    if (t.b != cur_b) {
      flush(cw, lane);
      cur_b = t.b;
    }
    const int xw = t.tx0 + cw * S::SW;
    if (xw >= g.nx) return;
    const bool solids = strip_has_solid<S>(reinterpret_cast<const uint32_t*>(base + L::kMask), cw, lane);
#pragma unroll 1
    for (int c = 0; c < kC; ++c) {
      const int x = xw + 32 * c + lane;
      if (x < g.nx) cell(t, base, x, cw * S::WPS + c, lane, solids);
    }
  }

  __device__ __forceinline__ void finish(int cw, int lane) { flush(cw, lane); }
};

template <class A, int kC, int kStages, int kMinBlocks>
__global__ void __launch_bounds__(kAdjThreads, kMinBlocks)
    adj_forward_kernel(const FwdArgs<typename A::T> p, int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dependency_wait();
  AdjForward<A, kC> pol{p};
  tile_pipeline<kAdjW, kStages, FwdStage<typename A::T, kC>::kBytes, kAdjProd>(smem, pol, p.at.total, err);
}

// ---------------------------------------------------------------------------------------------
// Backward sweep
// ---------------------------------------------------------------------------------------------

// Reciprocal of the backward sweep's linearisation (rounding-level accuracy suffices there):
// FP32 uses the hardware approximation, which keeps the IEEE division's out-of-line slow path
// (and the register spills its call forces) out of the kernel.
__device__ __forceinline__ float adj_rcp(float d) { return __fdividef(1.0f, d); }
__device__ __forceinline__ double adj_rcp(double d) { return 1.0 / d; }

// Adjoint of one fluid cell: out = J_C(yv)^T v + obj_coef du_x/dyv, where yv is the cell's
// pull-gathered state and v its transpose-gathered next adjoint. Returns the cell's alpha_bar
// term and adds its omega / fx / fy terms to go / gx / gy. The linearisation point comes from
// the exact forward states; the intermediates and the adjoint arithmetic use FMA (this file is
// compiled with contraction allowed), which changes the gradient only at rounding level.
template <class T>
__device__ __forceinline__ T adj_cell(const BwdArgs<T>& p, const T (&yv)[kQ], const T (&v)[kQ], T alpha,
                                      T (&out)[kQ], T& go, T& gx, T& gy) {
  // Forward intermediates (zero-coefficient terms dropped at compile time).
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
  const T sA = T(3) * uV + T(4.5) * Q - T(1.5) * usq * V0;        // sum w v A_i
  const T cxu = ux * Vxx + uy * Vxy, cyu = ux * Vxy + uy * Vyy;   // sum w v cu c_x, c_y
  const T cxF = Fx * Vxx + Fy * Vxy, cyF = Fx * Vxy + Fy * Vyy;   // sum w v cf c_x, c_y
  const T sgeq = drho * V0 + rho * sA;                             // sum v geq
  const T sguo = T(3) * (Fx * Vx + Fy * Vy - (ux * Fx + uy * Fy) * V0) +
                 T(9) * (ux * cxF + uy * cyF);                      // sum v guo
  const T om = sgeq - vy - T(0.5) * sguo;
  const T orho = p.omega * rho;
  T d_drho = p.omega * V0;
  T d_rho = p.omega * sA;
  const T d_usq = T(-1.5) * orho * V0;
  T d_ux = p.obj_coef + orho * (T(3) * Vx + T(9) * cxu) + T(9) * p.fp * cxF - T(3) * p.fp * Fx * V0 +
           T(2) * ux * d_usq;
  T d_uy = orho * (T(3) * Vy + T(9) * cyu) + T(9) * p.fp * cyF - T(3) * p.fp * Fy * V0 + T(2) * uy * d_usq;
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
    out[i] = o;
  }
  go += om;
  gx += d_Fx + T(0.5) * mxb;
  gy += d_Fy + T(0.5) * myb;
  return a_b;
}

// One adjoint step: Ybar = J_C(y_t)^T (P^T Z) + obj_coef du_x/dy_t, with y_t = P R_t. alpha_bar
// accumulates per segment in `aseg` (precision T; zero at the start of the sweep and after every
// flush) and is flushed into the double-precision `abar` by the segment's last adjoint step, so
// that the per-step update is a T add, not a double one.
template <class T, int kC>
struct AdjBackward {
  using S = AdjRing<T, kC>;
  using L = BwdStage<T, kC>;
  static constexpr bool kFinish = true;
  const BwdArgs<T>& p;
  int cur_b = -1;
  T go = T(0), gx = T(0), gy = T(0);

  __device__ __forceinline__ void issue(int tile, unsigned char* base, uint64_t* full) const {
    const AdjGeom& g = p.g;
    const TilePos t = tile_pos<S::TW>(g, p.at, tile, p.reverse);
    const RowSpan<S> rs(g, t.tx0, sizeof(T));
    const bool lo = t.tx0 == 0, hi = t.tx0 + S::TW >= g.nx;
    const bool z = p.Z != nullptr;
    const uint32_t fa = p.alpha ? field_bytes<S>(g, t.tx0, sizeof(T)) : 0u;
    const uint32_t fs = p.aseg ? field_bytes<S>(g, t.tx0, sizeof(T)) : 0u;
    const uint32_t wraps = (lo ? 48u : 0u) + (hi ? 48u : 0u);
    mbar_arrive_expect_tx(full, (z ? 2u : 1u) * (kQ * rs.bytes + wraps) + S::kMaskBytes + fa + fs);
    issue_pull<T, S>(base, base + L::kWrapR, p.R + t.b * g.inst, g, t, rs, lo, hi, full);
    issue_mask_rows<S>(base + L::kMask, p.mask, g, t, full);
    if (z) {
      const T* Z = p.Z + t.b * g.inst;
      T* rows = reinterpret_cast<T*>(base + L::kZ);
#pragma unroll
      for (int j = 0; j < kQ; ++j)
        bulk_copy_g2s(rows + j * S::SROW + rs.dst0,
                      Z + j * g.plane + static_cast<long long>(tr_row(j, t.y, t.ym, t.yp)) * g.pitch + rs.xs,
                      rs.bytes, full);
      // Wrap blocks of the transpose: planes 1, 5, 8 (c_x = +1) at x = nx - 1 read column 0;
      // planes 3, 6, 7 (c_x = -1) at x = 0 read column nx - 1.
      T* wz = reinterpret_cast<T*>(base + L::kWrapZ);
      if (hi) {
        for (int j = 0; j < 3; ++j) {
          const int i = wrap_dir(j);
          bulk_copy_g2s(wz + j * S::H, Z + i * g.plane + static_cast<long long>(tr_row(i, t.y, t.ym, t.yp)) * g.pitch,
                        16, full);
        }
      }
      if (lo) {
        const int xb = (g.nx - 1) & ~(S::H - 1);
        for (int j = 3; j < 6; ++j) {
          const int i = wrap_dir(j);
          bulk_copy_g2s(wz + j * S::H,
                        Z + i * g.plane + static_cast<long long>(tr_row(i, t.y, t.ym, t.yp)) * g.pitch + xb, 16, full);
        }
      }
    }
    const long long f0 = t.b * g.plane + static_cast<long long>(t.y) * g.pitch + t.tx0;
    if (fa) bulk_copy_g2s(base + L::kAlpha, p.alpha + f0, fa, full);
    if (fs) bulk_copy_g2s(base + L::kAseg, p.aseg + f0, fs, full);
  }

  __device__ __forceinline__ void flush(int cw, int lane) {
    if (cur_b >= 0) {
      double* slot = p.grads + 3 * warp_slot(cur_b, cw);
      warp_add_to(static_cast<double>(go), slot + 0, lane);
      warp_add_to(static_cast<double>(gx), slot + 1, lane);
      warp_add_to(static_cast<double>(gy), slot + 2, lane);
    }
    go = gx = gy = T(0);
  }

  __device__ __forceinline__ void cell(const TilePos& t, const unsigned char* base, int x, int word, int lane,
                                       bool solids) {
    const AdjGeom& g = p.g;
    const int lx = x - t.tx0 + S::H;
    const long long c = static_cast<long long>(t.y) * g.pitch + x;
    T* Yb = p.Yb + t.b * g.inst + c;
    T yv[kQ], v[kQ];
    staged_pull<T, S>(reinterpret_cast<const T*>(base), reinterpret_cast<const T*>(base + L::kWrapR), g.nx, x, lx,
                      yv);
    if (p.Z) {
      const T* sz = reinterpret_cast<const T*>(base + L::kZ);
#pragma unroll
      for (int j = 0; j < kQ; ++j) v[j] = sz[j * S::SROW + lx + dir_cx(j)];
      const T* wz = reinterpret_cast<const T*>(base + L::kWrapZ);
      if (x == g.nx - 1) {
        v[1] = wz[0 * S::H];
        v[5] = wz[1 * S::H];
        v[8] = wz[2 * S::H];
      }
      if (x == 0) {
        const int k = (g.nx - 1) & (S::H - 1);
        v[3] = wz[3 * S::H + k];
        v[6] = wz[4 * S::H + k];
        v[7] = wz[5 * S::H + k];
      }
    } else {
#pragma unroll
      for (int j = 0; j < kQ; ++j) v[j] = T(0);
    }
    if (solids) {
      const Nbits nb = cell_bits<S>(reinterpret_cast<const uint32_t*>(base + L::kMask), word, lane);
      if (nb.n0 & 2u) {
#pragma unroll
        for (int i = 0; i < kQ; ++i) Yb[i * g.plane] = T(0);
        return;
      }
      if ((nb.nm | nb.n0 | nb.np) != 0u) {
        const T* R = p.R + t.b * g.inst + c;
        const T* Z = p.Z ? p.Z + t.b * g.inst + c : nullptr;
#pragma unroll
        for (int i = 1; i < kQ; ++i) {
          if (pull_solid(nb, i)) yv[i] = __ldg(R + dir_opp(i) * g.plane);
          if (push_solid(nb, i)) v[i] = Z ? __ldg(Z + dir_opp(i) * g.plane) : T(0);
        }
      }
    }
    const T alpha = p.alpha ? reinterpret_cast<const T*>(base + L::kAlpha)[lx - S::H] : T(0);
    T out[kQ];
    const T a_b = adj_cell<T>(p, yv, v, alpha, out, go, gx, gy);
#pragma unroll
    for (int i = 0; i < kQ; ++i) Yb[i * g.plane] = out[i];
    if (p.aseg) {
      const long long ia = t.b * g.plane + c;
      const T acc = reinterpret_cast<const T*>(base + L::kAseg)[lx - S::H] + a_b;
      if (p.flush) {
        p.abar[ia] += static_cast<double>(acc);
        p.aseg[ia] = T(0);
      } else {
        p.aseg[ia] = acc;
      }
    }
  }

  __device__ __forceinline__ void consume(int tile, const unsigned char* base, int cw, int lane) {
    const AdjGeom& g = p.g;
    const TilePos t = tile_pos<S::TW>(g, p.at, tile, p.reverse);
    if (t.b != cur_b) {
      flush(cw, lane);
      cur_b = t.b;
    }
    const int xw = t.tx0 + cw * S::SW;
    if (xw >= g.nx) return;
    const bool solids = strip_has_solid<S>(reinterpret_cast<const uint32_t*>(base + L::kMask), cw, lane);
#pragma unroll 1
    for (int c = 0; c < kC; ++c) {
      const int x = xw + 32 * c + lane;
      if (x < g.nx) cell(t, base, x, cw * S::WPS + c, lane, solids);
    }
  }

  __device__ __forceinline__ void finish(int cw, int lane) { flush(cw, lane); }
};

template <class T, int kC, int kStages, int kMinBlocks>
__global__ void __launch_bounds__(kAdjThreads, kMinBlocks)
    adj_backward_kernel(const BwdArgs<T> p, int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dependency_wait();
  AdjBackward<T, kC> pol{p};
  tile_pipeline<kAdjW, kStages, BwdStage<T, kC>::kBytes, kAdjProd>(smem, pol, p.at.total, err);
}

// Per-instance sums of the per-warp slots (nval values each): block b adds its instance's
// slots in a fixed order (thread-strided, then a fixed tree), so the result is deterministic.
__global__ void __launch_bounds__(kAuxThreads) slot_sum_kernel(const double* __restrict__ slots, int per_inst,
                                                               int nval, double* __restrict__ out) {
  __shared__ double sh[kAuxThreads];
  const int b = blockIdx.x;
  for (int v = 0; v < nval; ++v) {
    double s = 0.0;
    for (int k = threadIdx.x; k < per_inst; k += kAuxThreads)
      s += slots[(static_cast<long long>(b) * per_inst + k) * nval + v];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = kAuxThreads / 2; o > 0; o >>= 1) {
      if (static_cast<int>(threadIdx.x) < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[static_cast<long long>(b) * nval + v] = sh[0];
    __syncthreads();
  }
}

// Kernel configurations: cells per lane kC, ring depth and residency target. FP32: forward 3
// stages at 3 blocks per SM (kC = 1: 32 KB, kC = 2: 63 KB of shared memory per block);
// backward kC = 1 3 stages (64 KB) at 3 blocks per SM, kC = 2 2 stages (84 KB) at 2 blocks.
// FP64 (kC = 1 only): forward 3 stages (63 KB), backward 2 stages (84 KB), 2 blocks per SM.
template <class T, int kC>
struct AdjLaunch {
  static constexpr int kFwdStages = 3;
  static constexpr int kFwdMin = sizeof(T) == 8 ? 2 : 3;
  static constexpr int kBwdStages = (sizeof(T) == 8 || kC == 2) ? 2 : 3;
  static constexpr int kBwdMin = (sizeof(T) == 8 || kC == 2) ? 2 : 3;
  static constexpr size_t fwd_smem() { return adj_smem_bytes(FwdStage<T, kC>::kBytes, kFwdStages); }
  static constexpr size_t bwd_smem() { return adj_smem_bytes(BwdStage<T, kC>::kBytes, kBwdStages); }
};

// Pull state of every instance from v0-layout post-streaming states (closed domain).
template <class T>
__global__ void adj_set_state_kernel(T* __restrict__ R, const uint32_t* __restrict__ mask,
                                     const AdjGeom g, const T* __restrict__ aos) {
  const int b = blockIdx.y;
  const long long n = static_cast<long long>(g.nx) * g.ny;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    const bool solid = mask_solid(mask, g.mask_words, x, y);
    const T* s = aos + b * kQ * n;
#pragma unroll
    for (int i = 0; i < kQ; ++i) {
      T v = T(0);
      if (!solid) {
        int xn = x + dir_cx(i), yn = y + dir_cy(i);
        xn = xn < 0 ? g.nx - 1 : (xn >= g.nx ? 0 : xn);
        yn = yn < 0 ? g.ny - 1 : (yn >= g.ny ? 0 : yn);
        const long long cn = static_cast<long long>(yn) * g.nx + xn;
        v = mask_solid(mask, g.mask_words, xn, yn) ? s[c * kQ + dir_opp(i)] : s[cn * kQ + i];
      }
      R[b * g.inst + i * g.plane + static_cast<long long>(y) * g.pitch + x] = v;
    }
  }
}

// v0-layout post-streaming state of instance b (pull gather of its pitched state).
template <class T>
__global__ void adj_get_state_kernel(const T* __restrict__ R, const uint32_t* __restrict__ mask,
                                     const AdjGeom g, int b, T* __restrict__ aos) {
  const long long n = static_cast<long long>(g.nx) * g.ny;
  const T* Rb = R + b * g.inst;
  for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
       c += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    const long long own = static_cast<long long>(y) * g.pitch + x;
    const bool solid = mask_solid(mask, g.mask_words, x, y);
#pragma unroll
    for (int i = 0; i < kQ; ++i) {
      T s = T(0);
      if (!solid) {
        int xs = x - dir_cx(i), ys = y - dir_cy(i);
        xs = xs < 0 ? g.nx - 1 : (xs >= g.nx ? 0 : xs);
        ys = ys < 0 ? g.ny - 1 : (ys >= g.ny ? 0 : ys);
        s = mask_solid(mask, g.mask_words, xs, ys)
                ? Rb[dir_opp(i) * g.plane + own]
                : Rb[i * g.plane + static_cast<long long>(ys) * g.pitch + xs];
      }
      aos[c * kQ + i] = s;
    }
  }
}

// Unpadded FP64 per-cell fields of every instance -> pitched fields of type T.
template <class T>
__global__ void to_pitched_kernel(const double* __restrict__ in, T* __restrict__ out, const AdjGeom g) {
  const long long n = static_cast<long long>(g.nx) * g.ny;
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < g.batch * n;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long b = k / n, c = k - b * n;
    const int y = static_cast<int>(c / g.nx), x = static_cast<int>(c - static_cast<long long>(y) * g.nx);
    out[b * g.plane + static_cast<long long>(y) * g.pitch + x] = static_cast<T>(in[k]);
  }
}


}  // namespace

struct lbm_adjoint {
  int precision = LBM_FP32, elem = 4, batch = 1, K = 100;
  AdjGeom g{};
  long long fluid = 0;
  double tau = 0, fx = 0, fy = 0;
  uint32_t* mask_d = nullptr;
  void* alpha = nullptr;         // batch pitched planes (T), null = zero field
  void* state[2] = {nullptr, nullptr};
  void* ckpt = nullptr;          // checkpoints: (T/K + 1) states
  size_t ckpt_count = 0;
  void* seg = nullptr;           // K recomputed states (a segment's first state is its checkpoint)
  void* ybar[2] = {nullptr, nullptr};
  double* abar = nullptr;        // batch pitched planes
  void* aseg = nullptr;          // batch pitched planes, per-segment alpha_bar in the state precision
  int fwd_req = 0, bwd_req = 0;  // requested cells per lane (0: automatic)
  int fwd_c = 1, bwd_c = 1;      // cells per lane in use
  int fwd_grid = 1, bwd_grid = 1;  // blocks of the two sweeps
  double* obj_part = nullptr;    // batch * fwd_grid * kAdjW objective slots
  double* grad_part = nullptr;   // batch * bwd_grid * kAdjW * 3 gradient slots
  size_t obj_slots = 0, grad_slots = 0;
  double* sums = nullptr;        // batch * 3 per-instance sums of the slots
  int* err_d = nullptr;          // bounded-wait error flag of the ring kernels
  void* stage = nullptr;
  size_t stage_bytes = 0;
  int steps = 0, window = 0;     // of the last forward
  const void* fin = nullptr;     // R_T after the forward (a state buffer or a checkpoint slot)
  bool have_forward = false;
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;  // the second half of the batch (forward sweep)
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaEvent_t join = nullptr;      // orders the two halves' streams
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
size_t field_bytes_all(const lbm_adjoint* a, int elem) {
  return static_cast<size_t>(a->batch) * a->g.plane * elem;
}

// Runs f(std::integral_constant<int, kC>) for cells per lane c (2 exists for FP32 only).
template <class T, class F>
int with_shape(int c, F&& f) {
  if constexpr (sizeof(T) == 4) {
    if (c == 2) return f(std::integral_constant<int, 2>{});
  }
  return f(std::integral_constant<int, 1>{});
}

template <class A, int kC>
struct AdjKernels {
  using T = typename A::T;
  using LC = AdjLaunch<T, kC>;
  static constexpr auto fwd = adj_forward_kernel<A, kC, LC::kFwdStages, LC::kFwdMin>;
  static constexpr auto bwd = adj_backward_kernel<T, kC, LC::kBwdStages, LC::kBwdMin>;
};

// Automatic cells per lane. Forward (FP32): the tile width (256 or 512 cells) that leaves fewer
// idle lanes in a row, the wider one on a tie (half the per-tile work per cell). Backward and
// FP64: one cell per lane (a 512-cell backward stage needs 42 KB, which leaves two blocks of 16
// consumer warps per SM instead of three of 24).
int auto_cells(const lbm_adjoint* a, bool backward) {
  if (a->precision == LBM_FP64 || backward) return 1;
  const int nx = a->g.nx;
  const int w1 = (nx + 255) / 256 * 256 - nx, w2 = (nx + 511) / 512 * 512 - nx;
  return w2 <= w1 ? 2 : 1;
}

// Tiles of a sweep with `cells` cells per lane, launched on `grid` blocks (0: grid not known yet).
AdjTiles make_tiles(const AdjGeom& g, int cells, int grid) {
  const int tw = 32 * kAdjW * cells;
  const int tpr = (g.nx + tw - 1) / tw;
  AdjTiles at;
  at.per_row = FastDiv(static_cast<uint32_t>(tpr));
  at.per_inst = FastDiv(static_cast<uint32_t>(tpr * g.ny));
  at.total = tpr * g.ny * g.batch;
  const int G = std::max(grid, 1);
  at.grid = FastDiv(static_cast<uint32_t>(G));
  at.q = at.total / G;
  at.r = at.total - at.q * G;
  return at;
}

// Grid of a sweep: every resident block slot of the GPU (at most one block per tile), so that all
// blocks run at once and stride over the tiles of all instances.
template <class K>
int sweep_grid(lbm_adjoint* a, K kernel, size_t smem, int cells, int* grid) {
  ADJ_CUDA(a, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  ADJ_CUDA(a, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kAdjThreads, smem));
  const long long total = make_tiles(a->g, cells, 0).total;
  *grid = static_cast<int>(std::max<long long>(1, std::min<long long>(total, static_cast<long long>(std::max(per_sm, 1)) * a->sm_count)));
  return LBM_OK;
}

// Chooses the tile shapes, sizes the grids and the slot buffers.
template <class A>
int configure(lbm_adjoint* a) {
  using T = typename A::T;
  const int fc = a->fwd_req ? a->fwd_req : auto_cells(a, false);
  const int bc = a->bwd_req ? a->bwd_req : auto_cells(a, true);
  int rc = with_shape<T>(fc, [&](auto kc) {
    using LC = AdjLaunch<T, decltype(kc)::value>;
    return sweep_grid(a, AdjKernels<A, decltype(kc)::value>::fwd, LC::fwd_smem(), decltype(kc)::value, &a->fwd_grid);
  });
  if (rc) return rc;
  rc = with_shape<T>(bc, [&](auto kc) {
    using LC = AdjLaunch<T, decltype(kc)::value>;
    return sweep_grid(a, AdjKernels<A, decltype(kc)::value>::bwd, LC::bwd_smem(), decltype(kc)::value, &a->bwd_grid);
  });
  if (rc) return rc;
  a->fwd_c = (sizeof(T) == 4 && fc == 2) ? 2 : 1;
  a->bwd_c = (sizeof(T) == 4 && bc == 2) ? 2 : 1;
  const size_t os = static_cast<size_t>(a->batch) * a->fwd_grid * kAdjW;
  const size_t gs = static_cast<size_t>(a->batch) * a->bwd_grid * kAdjW * 3;
  if (os > a->obj_slots) {
    cudaFree(a->obj_part);
    a->obj_part = nullptr;
    a->obj_slots = 0;
    ADJ_CUDA(a, cudaMalloc(&a->obj_part, os * sizeof(double)));
    a->obj_slots = os;
  }
  if (gs > a->grad_slots) {
    cudaFree(a->grad_part);
    a->grad_part = nullptr;
    a->grad_slots = 0;
    ADJ_CUDA(a, cudaMalloc(&a->grad_part, gs * sizeof(double)));
    a->grad_slots = gs;
  }
  return LBM_OK;
}

template <class A>
FwdArgs<typename A::T> fwd_args(const lbm_adjoint* a) {
  using T = typename A::T;
  FwdArgs<T> p{};
  const T tau = T(a->tau);
  p.k.omega = T(1) / tau;
  p.k.force_prefactor = T(1) - T(0.5) * p.k.omega;
  p.k.fx = T(a->fx);
  p.k.fy = T(a->fy);
  p.k.hfx = T(0.5) * p.k.fx;
  p.k.hfy = T(0.5) * p.k.fy;
  p.alpha = static_cast<const T*>(a->alpha);
  p.mask = a->mask_d;
  p.g = a->g;
  p.at = make_tiles(a->g, a->fwd_c, a->fwd_grid);
  return p;
}

template <class K, class Args>
int launch_ring(lbm_adjoint* a, K kernel, int grid, size_t smem, const Args& p, cudaStream_t stream) {
  ADJ_CUDA(a, launch_dependent(kernel, dim3(grid), dim3(kAdjThreads), smem, stream, p, a->err_d));
  return LBM_OK;
}

// One half of the batch for the forward sweep: its instances' arguments and where they start in
// the batch's state, field and slot arrays. The two halves run on two streams, so that one
// half's launch fills the SMs while the other's drains (a sweep step is a short kernel, and
// its fill and drain cost a sixth of it when one launch holds the whole batch).
template <class T>
struct FwdHalf {
  FwdArgs<T> p;
  long long state_off = 0, slot_off = 0;
  cudaStream_t stream = nullptr;
};

template <class A>
FwdHalf<typename A::T> fwd_half(const lbm_adjoint* a, const FwdArgs<typename A::T>& p, int k);

template <class A>
int launch_forward(lbm_adjoint* a, const FwdHalf<typename A::T>& h, const void* R, void* Rn, double* obj,
                   int reverse) {
  using T = typename A::T;
  FwdArgs<T> p = h.p;
  p.R = static_cast<const T*>(R) + h.state_off;
  p.Rn = Rn ? static_cast<T*>(Rn) + h.state_off : nullptr;
  p.obj = obj ? obj + h.slot_off : nullptr;
  p.reverse = reverse;
  return with_shape<T>(a->fwd_c, [&](auto kc) {
    constexpr int kC = decltype(kc)::value;
    return launch_ring(a, AdjKernels<A, kC>::fwd, a->fwd_grid, AdjLaunch<T, kC>::fwd_smem(), p, h.stream);
  });
}

template <class A>
int launch_backward(lbm_adjoint* a, const BwdArgs<typename A::T>& p, cudaStream_t stream) {
  using T = typename A::T;
  return with_shape<T>(a->bwd_c, [&](auto kc) {
    constexpr int kC = decltype(kc)::value;
    return launch_ring(a, AdjKernels<A, kC>::bwd, a->bwd_grid, AdjLaunch<T, kC>::bwd_smem(), p, stream);
  });
}

// Number of halves the batch runs as (two when it has at least two instances) and the first
// instance of half k.
inline int adj_halves(const lbm_adjoint* a) { return a->batch >= 2 ? 2 : 1; }
inline int adj_half_first(const lbm_adjoint* a, int k) { return k == 0 ? 0 : a->batch / 2; }
inline int adj_half_count(const lbm_adjoint* a, int k) {
  return adj_halves(a) == 1 ? a->batch : (k == 0 ? a->batch / 2 : a->batch - a->batch / 2);
}

// Makes stream `to` wait for the work enqueued so far on stream `from`.
inline cudaError_t adj_join(lbm_adjoint* a, cudaStream_t from, cudaStream_t to) {
  cudaError_t e = cudaEventRecord(a->join, from);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(to, a->join, 0);
  return e;
}

// Per-instance sums of nval-valued slots into host memory (synchronises the stream), then the
// bounded-wait error flag.
int read_sums(lbm_adjoint* a, const double* slots, int grid, int nval, std::vector<double>& out) {
  slot_sum_kernel<<<a->batch, kAuxThreads, 0, a->stream>>>(slots, grid * kAdjW, nval, a->sums);
  ADJ_CUDA(a, cudaGetLastError());
  out.assign(static_cast<size_t>(a->batch) * nval, 0.0);
  ADJ_CUDA(a, cudaMemcpyAsync(out.data(), a->sums, out.size() * sizeof(double), cudaMemcpyDeviceToHost, a->stream));
  int flag = 0;
  ADJ_CUDA(a, cudaMemcpyAsync(&flag, a->err_d, sizeof(int), cudaMemcpyDeviceToHost, a->stream));
  ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  if (flag) {
    ADJ_CUDA(a, cudaMemsetAsync(a->err_d, 0, sizeof(int), a->stream));
    return adj_fail(a, LBM_ERR_TIMEOUT, "an adjoint kernel gave up waiting for its shared-memory ring");
  }
  return LBM_OK;
}

// Half k of the batch for the forward sweep (the whole batch when it runs undivided).
template <class A>
FwdHalf<typename A::T> fwd_half(const lbm_adjoint* a, const FwdArgs<typename A::T>& p, int k) {
  FwdHalf<typename A::T> h;
  const long long b0 = adj_half_first(a, k);
  h.p = p;
  h.p.g.batch = adj_half_count(a, k);
  h.p.at = make_tiles(h.p.g, a->fwd_c, a->fwd_grid);
  h.state_off = b0 * a->g.inst;
  h.slot_off = b0 * a->fwd_grid * kAdjW;
  if (p.alpha) h.p.alpha = p.alpha + b0 * a->g.plane;
  h.stream = k == 0 ? a->stream : a->stream2;
  return h;
}

template <class A>
int forward_t(lbm_adjoint* a, const void* s0_host, int steps, int window, double* J) {
  using T = typename A::T;
  if (const int rc = configure<A>(a)) return rc;
  const size_t sb = state_bytes(a);
  const size_t nckpt = static_cast<size_t>(steps / a->K) + 1;
  if (a->ckpt_count < nckpt) {
    cudaFree(a->ckpt);
    a->ckpt = nullptr;
    a->ckpt_count = 0;
    ADJ_CUDA(a, cudaMalloc(&a->ckpt, nckpt * sb));
    a->ckpt_count = nckpt;
  }
  // Checkpoint slot k holds R_{kK}; the forward writes checkpoint steps straight into their slot
  // and the other steps into the two state buffers alternately.
  char* ckpt = static_cast<char*>(a->ckpt);
  if (s0_host) {
    const size_t hb = static_cast<size_t>(a->batch) * kQ * a->g.nx * a->g.ny * sizeof(T);
    if (a->stage_bytes < hb) {
      cudaFree(a->stage);
      a->stage = nullptr;
      ADJ_CUDA(a, cudaMalloc(&a->stage, hb));
      a->stage_bytes = hb;
    }
    ADJ_CUDA(a, cudaMemcpyAsync(a->stage, s0_host, hb, cudaMemcpyHostToDevice, a->stream));
    adj_set_state_kernel<T><<<dim3(2 * a->sm_count, a->batch), kAuxThreads, 0, a->stream>>>(
        reinterpret_cast<T*>(ckpt), a->mask_d, a->g, static_cast<const T*>(a->stage));
  } else {
    ADJ_CUDA(a, cudaMemsetAsync(ckpt, 0, sb, a->stream));  // rest: f_i - w_i = 0
  }
  ADJ_CUDA(a, cudaMemsetAsync(a->obj_part, 0, a->obj_slots * sizeof(double), a->stream));
  // The batch as two halves on two streams (one launch per half and step), or whole.
  const FwdArgs<T> p = fwd_args<A>(a);
  const int nhalf = adj_halves(a);
  FwdHalf<T> half[2];
  for (int k = 0; k < nhalf; ++k) half[k] = fwd_half<A>(a, p, k);
  const void* cur = ckpt;
  int spare = 0;
  ADJ_CUDA(a, cudaEventRecord(a->ev[0], a->stream));
  if (nhalf == 2) ADJ_CUDA(a, adj_join(a, a->stream, a->stream2));
  for (int t = 0; t < steps; ++t) {
    const bool in_window = t >= steps - window + 1;
    const bool is_ckpt = (t + 1) % a->K == 0;
    void* out = is_ckpt ? ckpt + static_cast<size_t>((t + 1) / a->K) * sb : a->state[spare];
    for (int k = 0; k < nhalf; ++k)
      if (const int rc = launch_forward<A>(a, half[k], cur, out, in_window ? a->obj_part : nullptr, t & 1)) return rc;
    if (!is_ckpt) spare ^= 1;
    cur = out;
  }
  if (nhalf == 2) ADJ_CUDA(a, adj_join(a, a->stream2, a->stream));
  ADJ_CUDA(a, cudaEventRecord(a->ev[1], a->stream));
  // the final state's objective
  if (nhalf == 2) ADJ_CUDA(a, adj_join(a, a->stream, a->stream2));
  for (int k = 0; k < nhalf; ++k)
    if (const int rc = launch_forward<A>(a, half[k], cur, nullptr, a->obj_part, steps & 1)) return rc;
  if (nhalf == 2) ADJ_CUDA(a, adj_join(a, a->stream2, a->stream));
  ADJ_CUDA(a, cudaGetLastError());
  std::vector<double> sums;
  if (const int rc = read_sums(a, a->obj_part, a->fwd_grid, 1, sums)) return rc;
  float ms = 0.f;
  ADJ_CUDA(a, cudaEventElapsedTime(&ms, a->ev[0], a->ev[1]));
  a->fwd_step_s = steps > 0 ? ms * 1e-3 / steps : 0.0;
  for (int b = 0; b < a->batch; ++b) J[b] = sums[b] / (static_cast<double>(window) * a->fluid);
  a->steps = steps;
  a->window = window;
  a->have_forward = true;
  a->fin = cur;
  return LBM_OK;
}

template <class A>
int backward_t(lbm_adjoint* a, double* dtau, double* dfx, double* dfy, double* dalpha) {
  using T = typename A::T;
  if (const int rc = configure<A>(a)) return rc;
  const size_t sb = state_bytes(a);
  const int T_steps = a->steps, W = a->window, K = a->K;
  if (!a->seg) {
    ADJ_CUDA(a, cudaMalloc(&a->seg, static_cast<size_t>(K) * sb));
    ADJ_CUDA(a, cudaMemsetAsync(a->seg, 0, static_cast<size_t>(K) * sb, a->stream));
  }
  for (int k = 0; k < 2; ++k)
    if (!a->ybar[k]) {
      ADJ_CUDA(a, cudaMalloc(&a->ybar[k], sb));
      ADJ_CUDA(a, cudaMemsetAsync(a->ybar[k], 0, sb, a->stream));
    }
  ADJ_CUDA(a, cudaMemsetAsync(a->grad_part, 0, a->grad_slots * sizeof(double), a->stream));
  if (dalpha) {
    if (!a->aseg) ADJ_CUDA(a, cudaMalloc(&a->aseg, field_bytes_all(a, a->elem)));
    ADJ_CUDA(a, cudaMemsetAsync(a->aseg, 0, field_bytes_all(a, a->elem), a->stream));
    ADJ_CUDA(a, cudaMemsetAsync(a->abar, 0, field_bytes_all(a, sizeof(double)), a->stream));
  }
  const FwdArgs<T> pf = fwd_args<A>(a);
  BwdArgs<T> pb{};
  pb.alpha = pf.alpha;
  pb.aseg = dalpha ? static_cast<T*>(a->aseg) : nullptr;
  pb.abar = a->abar;
  pb.mask = a->mask_d;
  pb.g = a->g;
  pb.at = make_tiles(a->g, a->bwd_c, a->bwd_grid);
  pb.omega = pf.k.omega;
  pb.fp = pf.k.force_prefactor;
  pb.fx = pf.k.fx;
  pb.fy = pf.k.fy;
  pb.hfx = pf.k.hfx;
  pb.hfy = pf.k.hfy;
  pb.grads = a->grad_part;
  const T coef = T(1.0 / (static_cast<double>(W) * a->fluid));
  char* seg = static_cast<char*>(a->seg);
  // The batch as two halves on two streams, as in the forward sweep: per half its instances'
  // recomputation and adjoint arguments, offset into the batch's arrays.
  const int nhalf = adj_halves(a);
  FwdHalf<T> fh[2];
  BwdArgs<T> bh[2];
  long long st_off[2] = {0, 0};
  cudaStream_t hs[2] = {a->stream, a->stream2};
  for (int k = 0; k < nhalf; ++k) {
    fh[k] = fwd_half<A>(a, pf, k);
    const long long b0 = adj_half_first(a, k);
    st_off[k] = b0 * a->g.inst;
    bh[k] = pb;
    bh[k].g.batch = adj_half_count(a, k);
    bh[k].at = make_tiles(bh[k].g, a->bwd_c, a->bwd_grid);
    if (pb.alpha) bh[k].alpha = pb.alpha + b0 * a->g.plane;
    if (pb.aseg) bh[k].aseg = pb.aseg + b0 * a->g.plane;
    bh[k].abar = pb.abar + b0 * a->g.plane;
    bh[k].grads = pb.grads + 3 * b0 * a->bwd_grid * kAdjW;
  }
  int yb = 0;
  bool first = true;
  ADJ_CUDA(a, cudaEventRecord(a->ev[0], a->stream));
  if (nhalf == 2) ADJ_CUDA(a, adj_join(a, a->stream, a->stream2));
  const int nseg = (T_steps + K - 1) / K;
  for (int s = nseg - 1; s >= 0; --s) {
    const int t0 = s * K, t1 = std::min(T_steps, t0 + K);
    // R_{t0} is checkpoint s; recompute R_{t0 + 1 .. t1} into seg[0 .. t1 - t0 - 1].
    const char* base = static_cast<const char*>(a->ckpt) + static_cast<size_t>(s) * sb;
    auto state_at = [&](int t) -> const void* { return t == t0 ? base : seg + static_cast<size_t>(t - t0 - 1) * sb; };
    for (int t = t0; t < t1; ++t)
      for (int k = 0; k < nhalf; ++k)
        if (const int rc = launch_forward<A>(a, fh[k], state_at(t), seg + static_cast<size_t>(t - t0) * sb, nullptr, t & 1))
          return rc;
    // Adjoint steps t1 (only for the last segment: the final state) .. t0.
    const int top = (s == nseg - 1) ? t1 : t1 - 1;
    for (int t = top; t >= t0; --t) {
      const bool in_window = t >= T_steps - W + 1;
      for (int k = 0; k < nhalf; ++k) {
        BwdArgs<T>& q = bh[k];
        q.R = static_cast<const T*>(state_at(t)) + st_off[k];
        q.Z = first ? nullptr : static_cast<const T*>(a->ybar[yb ^ 1]) + st_off[k];
        q.Yb = static_cast<T*>(a->ybar[yb]) + st_off[k];
        q.obj_coef = in_window ? coef : T(0);
        q.flush = t == t0 ? 1 : 0;
        q.reverse = t & 1;
        if (const int rc = launch_backward<A>(a, q, hs[k])) return rc;
      }
      first = false;
      yb ^= 1;
    }
  }
  if (nhalf == 2) ADJ_CUDA(a, adj_join(a, a->stream2, a->stream));
  ADJ_CUDA(a, cudaEventRecord(a->ev[1], a->stream));
  ADJ_CUDA(a, cudaGetLastError());
  if (dalpha)
    ADJ_CUDA(a, cudaMemcpy2DAsync(dalpha, a->g.nx * sizeof(double), a->abar, a->g.pitch * sizeof(double),
                                  a->g.nx * sizeof(double), static_cast<size_t>(a->batch) * a->g.ny,
                                  cudaMemcpyDeviceToHost, a->stream));
  std::vector<double> g3;
  if (const int rc = read_sums(a, a->grad_part, a->bwd_grid, 3, g3)) return rc;
  float ms = 0.f;
  ADJ_CUDA(a, cudaEventElapsedTime(&ms, a->ev[0], a->ev[1]));
  a->bwd_step_s = T_steps > 0 ? ms * 1e-3 / (T_steps + 1) : 0.0;
  const double omega = 1.0 / static_cast<double>(T(a->tau));
  for (int b = 0; b < a->batch; ++b) {
    if (dtau) dtau[b] = g3[3 * b] * (-omega * omega);  // d omega / d tau = -1/tau^2
    if (dfx) dfx[b] = g3[3 * b + 1];
    if (dfy) dfy[b] = g3[3 * b + 2];
  }
  return LBM_OK;
}

template <class T>
int get_state_t(lbm_adjoint* a, int b, void* host) {
  const size_t bytes = static_cast<size_t>(kQ) * a->g.nx * a->g.ny * sizeof(T);
  if (a->stage_bytes < bytes) {
    cudaFree(a->stage);
    a->stage = nullptr;
    ADJ_CUDA(a, cudaMalloc(&a->stage, bytes));
    a->stage_bytes = bytes;
  }
  adj_get_state_kernel<T><<<2 * a->sm_count, kAuxThreads, 0, a->stream>>>(
      static_cast<const T*>(a->fin), a->mask_d, a->g, b, static_cast<T*>(a->stage));
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
      (precision != LBM_FP32 && precision != LBM_FP64))
    return LBM_ERR_INVALID_ARG;
  const int elem = precision == LBM_FP64 ? 8 : 4;
  const long long pitch = (static_cast<long long>(nx) * elem + 127) / 128 * 128 / elem;
  // Tile indices of all instances are 32-bit: (ny * tiles per row) * batch < 2^31.
  if (pitch * ny > static_cast<long long>(INT_MAX) ||
      static_cast<long long>((nx + 255) / 256) * ny * batch > static_cast<long long>(INT_MAX))
    return LBM_ERR_INVALID_ARG;
  lbm_adjoint* a = new (std::nothrow) lbm_adjoint();
  if (!a) return LBM_ERR_OUT_OF_MEMORY;
  a->precision = precision;
  a->elem = elem;
  a->batch = batch;
  a->K = checkpoint_every;
  a->tau = tau;
  a->fx = fx;
  a->fy = fy;
  a->g.nx = nx;
  a->g.ny = ny;
  a->g.pitch = static_cast<int>(pitch);
  a->g.batch = batch;
  a->g.plane = pitch * ny;
  a->g.inst = kQ * a->g.plane;
  a->g.mask_words = mask_row_words(nx);
  for (long long c = 0; c < static_cast<long long>(nx) * ny; ++c) a->fluid += solid[c] ? 0 : 1;
  auto fail = [&](int code) {
    lbm_adj_destroy(a);
    return code;
  };
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&a->sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&a->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&a->ev[0]) != cudaSuccess || cudaEventCreate(&a->ev[1]) != cudaSuccess)
    return fail(LBM_ERR_CUDA);
  if (const int rc = precision == LBM_FP64 ? configure<ExactF64>(a) : configure<ExactF32>(a)) return fail(rc);
  std::vector<uint32_t> words;
  pack_mask(solid, nx, ny, a->g.mask_words, words);
  const size_t sb = state_bytes(a);
  cudaError_t e = cudaMalloc(&a->mask_d, words.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpy(a->mask_d, words.data(), words.size() * 4, cudaMemcpyHostToDevice);
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    e = cudaMalloc(&a->state[k], sb);
    if (e == cudaSuccess) e = cudaMemset(a->state[k], 0, sb);
  }
  if (e == cudaSuccess) e = cudaMalloc(&a->abar, field_bytes_all(a, sizeof(double)));
  if (e == cudaSuccess) e = cudaMalloc(&a->sums, static_cast<size_t>(batch) * 3 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&a->err_d, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(a->err_d, 0, sizeof(int));
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA);
  *out = a;
  return LBM_OK;
}

int lbm_adj_destroy(lbm_adjoint* a) {
  if (!a) return LBM_OK;
  if (a->stream) cudaStreamSynchronize(a->stream);
  for (void* p : {static_cast<void*>(a->mask_d), a->alpha, a->state[0], a->state[1], a->ckpt, a->seg, a->ybar[0],
                  a->ybar[1], static_cast<void*>(a->abar), a->aseg, static_cast<void*>(a->obj_part),
                  static_cast<void*>(a->grad_part), static_cast<void*>(a->sums), static_cast<void*>(a->err_d),
                  a->stage})
    cudaFree(p);
  for (cudaEvent_t ev : a->ev)
    if (ev) cudaEventDestroy(ev);
  if (a->join) cudaEventDestroy(a->join);
  if (a->stream) cudaStreamDestroy(a->stream);
  if (a->stream2) cudaStreamDestroy(a->stream2);
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

int lbm_adj_set_tiles(lbm_adjoint* a, int forward_cells, int backward_cells) {
  if (!a) return LBM_ERR_INVALID_ARG;
  const int maxc = a->precision == LBM_FP64 ? 1 : 2;
  if (forward_cells < 0 || forward_cells > maxc || backward_cells < 0 || backward_cells > maxc)
    return adj_fail(a, LBM_ERR_INVALID_ARG, "cells per lane: 0 (automatic), 1, or 2 (FP32 only)");
  a->fwd_req = forward_cells;
  a->bwd_req = backward_cells;
  return a->precision == LBM_FP64 ? configure<ExactF64>(a) : configure<ExactF32>(a);
}

int lbm_adj_get_tiles(const lbm_adjoint* a, int* forward_cells, int* backward_cells) {
  if (!a) return LBM_ERR_INVALID_ARG;
  if (forward_cells) *forward_cells = a->fwd_c;
  if (backward_cells) *backward_cells = a->bwd_c;
  return LBM_OK;
}

int lbm_adj_set_alpha(lbm_adjoint* a, const double* alpha) {
  if (!a) return LBM_ERR_INVALID_ARG;
  if (!alpha) {
    cudaFree(a->alpha);
    a->alpha = nullptr;
    return LBM_OK;
  }
  const size_t n = static_cast<size_t>(a->batch) * a->g.nx * a->g.ny;
  double* tmp = nullptr;
  if (!a->alpha) {
    ADJ_CUDA(a, cudaMalloc(&a->alpha, field_bytes_all(a, a->elem)));
    ADJ_CUDA(a, cudaMemsetAsync(a->alpha, 0, field_bytes_all(a, a->elem), a->stream));  // row padding
  }
  ADJ_CUDA(a, cudaMalloc(&tmp, n * sizeof(double)));
  ADJ_CUDA(a, cudaMemcpyAsync(tmp, alpha, n * sizeof(double), cudaMemcpyHostToDevice, a->stream));
  if (a->precision == LBM_FP64)
    to_pitched_kernel<double><<<2 * a->sm_count, kAuxThreads, 0, a->stream>>>(tmp, static_cast<double*>(a->alpha), a->g);
  else
    to_pitched_kernel<float><<<2 * a->sm_count, kAuxThreads, 0, a->stream>>>(tmp, static_cast<float*>(a->alpha), a->g);
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
