// Warp-specialised pull stream-collide step, one cell (plain FP32 / FP64 storage) or one pair of
// cells (16-bit storage) per lane.
// Same results as pull_step_kernel (step_kernel.cuh); same producer as tma_step_kernel
// (step_tma.cuh), different consumers:
//
//   * a tile is TW = kW * 32 * kC consecutive cells of one row; the producer warp (one lane)
//     streams, per tile, the 9 source plane rows (plus a 16-byte halo each side), the 3 mask rows
//     and, on a periodic row's first and last tile, the 16-byte blocks holding the wrapped
//     neighbours (cell nx - 1 of the 3 planes moving right, cell 0 of the 3 moving left) into a
//     shared ring stage with cp.async.bulk, completing on the stage's "full" mbarrier;
//   * consumer warp w owns a strip of 32 * kC * LC cells (LC = 1, or 2 for 16-bit storage), and
//     lane l the cells strip + 32 LC c + LC l .. + LC - 1 (c = 0 .. kC - 1): consecutive lanes
//     hold consecutive cells, so each plane value is one conflict-free 4- or 8-byte shared load
//     at offset -c_x (16-bit pairs: two aligned 4-byte loads and a byte permute for the shifted
//     planes), and each of the 9 results is one fully coalesced warp store of 128 bytes (FP64:
//     256 bytes);
//   * a lane keeps one cell live at a time (9 inputs, 9 outputs, the collision's temporaries),
//     which leaves registers for many resident warps: the exact collision is a long chain of
//     dependent IEEE operations, and warps are what hides its latency;
//   * one vote per strip tells whether any of its cells or their neighbours is solid; only then
//     are per-cell neighbour bits formed and bounce-back values read (opposite population of the
//     cell itself, from global memory);
//   * waits are bounded as in the bulk-copy kernel (error flag, LBM_ERR_TIMEOUT on the host);
//   * tiles cover rows row0 .. row0 + tiles / tiles_per_row - 1 (the strip engine steps the owned
//     rows of a strip between its two ghost rows).
#pragma once

#include <type_traits>
#include <utility>

#include "step_tma.cuh"

namespace lbm_b200 {

template <class ST, int kW, int kC>
struct RingShape {
  static constexpr int H = 16 / static_cast<int>(sizeof(ST));  // halo elements (16 bytes)
  static constexpr int LC = sizeof(ST) == 2 ? 2 : 1;            // cells per lane per pass
  static constexpr int SW = 32 * kC * LC;                       // strip width (cells per warp)
  static constexpr int WPS = SW / 32;                            // mask words per strip
  static constexpr int TW = kW * SW;                            // tile width
  static constexpr int SROW = TW + 2 * H;
  static constexpr int MW = TW / 32 + 4;  // staged mask words per row
  static constexpr int kPlaneBytes = kQ * SROW * static_cast<int>(sizeof(ST));
  static constexpr int kMaskBytes = 3 * MW * 4;
  static constexpr int kWrapBytes = 6 * 16;
  static constexpr int kStageBytes = kPlaneBytes + kMaskBytes + kWrapBytes;
  static constexpr int kThreads = 32 * (kW + 1);
  static_assert((TW / 32) % 4 == 0, "mask rows must stay 16-byte aligned");
  static_assert(kStageBytes % 16 == 0, "stages must stay 16-byte aligned");
};

template <class S>
__host__ __device__ constexpr size_t ring_smem_bytes(int stages) {
  return static_cast<size_t>(stages) * S::kStageBytes + 2 * stages * sizeof(uint64_t);
}

// Directions whose wrapped source lies at the other end of the row: c_x = +1 (1, 5, 8) read
// cell nx - 1 at x = 0, c_x = -1 (3, 6, 7) read cell 0 at x = nx - 1.
__device__ __forceinline__ int wrap_dir(int j) {
  return j == 0 ? 1 : j == 1 ? 5 : j == 2 ? 8 : j == 3 ? 3 : j == 4 ? 6 : 7;
}

// One cell of a strip. st: stage planes (plane i row at st + i * SROW, local column lx = cell x);
// sm: 3 staged mask rows (y - 1, y, y + 1) whose word 0 is word tx0 / 32; wr: wrap blocks.
// kWrapInRow: the stage holds the cell's whole row (columns 0 .. nx - 1 at lx - x ..), and the
// periodic neighbours of x = 0 and x = nx - 1 are read from it instead of from wrap blocks.
// kHalo: the strip engine's fused halo (StepArgs::halo_top / halo_bot).
template <class ST, class A, bool kOpen, class S, bool kWrapInRow = false, bool kHalo = false>
__device__ __forceinline__ void ring_cell(const StepArgs<ST, ExactPhys<A>>& p, const ST* st,
                                          const uint32_t* sm, const ST* wr, int y, int ym, int yp,
                                          int x, int lx, int word, int lane, bool solids) {
  using T = typename A::T;
  const int nx = p.g.nx;
  const long long plane = p.g.plane;
  T v[kQ];
#pragma unroll
  for (int i = 0; i < kQ; ++i) v[i] = st[i * S::SROW + lx - dir_cx(i)];
  if (!kOpen && kWrapInRow) {
    const int r0 = lx - x;  // column 0 of the staged row
    if (x == 0) {
      v[1] = st[1 * S::SROW + r0 + nx - 1];
      v[5] = st[5 * S::SROW + r0 + nx - 1];
      v[8] = st[8 * S::SROW + r0 + nx - 1];
    }
    if (x == nx - 1) {
      v[3] = st[3 * S::SROW + r0];
      v[6] = st[6 * S::SROW + r0];
      v[7] = st[7 * S::SROW + r0];
    }
  } else if (!kOpen) {
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
  uint32_t nm = 0, n0 = 0, np = 0;  // bits 0, 1, 2: cells x - 1, x, x + 1 of rows y - 1, y, y + 1
  if (solids) {
    nm = __funnelshift_r(sm[word], sm[word + 1], lane) & 7u;
    n0 = __funnelshift_r(sm[S::MW + word], sm[S::MW + word + 1], lane) & 7u;
    np = __funnelshift_r(sm[2 * S::MW + word], sm[2 * S::MW + word + 1], lane) & 7u;
    if (!(n0 & 2u) && (nm | n0 | np) != 0u) {
#pragma unroll
      for (int i = 1; i < kQ; ++i) {
        const uint32_t w = dir_cy(i) == 1 ? nm : (dir_cy(i) == -1 ? np : n0);
        if ((w >> (1 - dir_cx(i))) & 1u)
          v[i] = __ldg(p.src + dir_opp(i) * plane + static_cast<long long>(y) * p.g.pitch + x);
      }
    }
  }
  if (kOpen) {
    if (x == 0) {
      v[1] = p.eq_in[1];
      v[5] = p.eq_in[5];
      v[8] = p.eq_in[8];
    }
    if (x == nx - 1) {
#pragma unroll
      for (int i = 1; i < kQ; ++i) {
        if (dir_cx(i) != -1) continue;
        // Zero-gradient outflow: the source is cell nx - 1 of row y - c_y; bounce-back from cell
        // nx - 2 of row y when that source is solid.
        const uint32_t w = dir_cy(i) == 1 ? nm : (dir_cy(i) == -1 ? np : n0);
        v[i] = ((w >> 1) & 1u)
                   ? __ldg(p.src + dir_opp(i) * plane + static_cast<long long>(y) * p.g.pitch + (nx - 2))
                   : st[i * S::SROW + lx];
      }
    }
  }
  (void)ym;
  (void)yp;
  T out[kQ];
  collide_exact<A>(v, p.k, out);
  ST* d = p.dst + static_cast<long long>(y) * p.g.pitch + x;
#pragma unroll
  for (int i = 0; i < kQ; ++i) d[i * plane] = out[i];
  if constexpr (kHalo) {
    if (y == p.g.ny - 2) {
      const long long pl = p.halo[1];
      ST* h = p.dst + p.halo[0] + x;
      h[2 * pl] = out[2];
      h[5 * pl] = out[5];
      h[6 * pl] = out[6];
    }
    if (y == 1) {
      const long long pl = p.halo[3];
      ST* h = p.dst + p.halo[2] + x;
      h[4 * pl] = out[4];
      h[7 * pl] = out[7];
      h[8 * pl] = out[8];
    }
  }
}

// 16-bit storage: widen a packed pair of stored (scaled) values to FP32, element 0 in the low
// half (the compute representation of the step kernels).
template <class ST>
__device__ __forceinline__ float2 widen_pair(uint32_t raw);
template <>
__device__ __forceinline__ float2 widen_pair<__half>(uint32_t raw) {
  __half2 h;
  memcpy(&h, &raw, 4);
  return __half22float2(h);
}
template <>
__device__ __forceinline__ float2 widen_pair<__nv_bfloat16>(uint32_t raw) {
  __nv_bfloat162 h;
  memcpy(&h, &raw, 4);
  return __bfloat1622float2(h);
}

// One pair of cells x, x + 1 (x even) of a strip, 16-bit storage, FP32 fast collision. Same
// stage layout (and kWrapInRow, kHalo) as ring_cell; word / lane locate the pair's mask bits
// (cells x - 1 .. x + 2); rkey is the step's stochastic-rounding key (step_rkey).
template <class ST, bool kOpen, class S, bool kWrapInRow = false, bool kHalo = false>
__device__ __forceinline__ void ring_pair(const StepArgs<ST, FastPhys>& p, const ST* st,
                                          const uint32_t* sm, const ST* wr, int y, int x, int lx,
                                          int word, int lane, bool solids, uint32_t rkey) {
  const int nx = p.g.nx;
  const long long plane = p.g.plane;
  const long long row = static_cast<long long>(y) * p.g.pitch;
  float2 v[kQ];
#pragma unroll
  for (int i = 0; i < kQ; ++i) {
    const uint32_t* r = reinterpret_cast<const uint32_t*>(st + i * S::SROW + lx);
    const uint32_t own = r[0];
    uint32_t raw = own;
    if (dir_cx(i) == 1) raw = __byte_perm(r[-1], own, 0x5432);   // cells x - 1, x
    if (dir_cx(i) == -1) raw = __byte_perm(own, r[1], 0x5432);   // cells x + 1, x + 2
    v[i] = widen_pair<ST>(raw);
  }
  if (!kOpen && kWrapInRow) {
    const int r0 = lx - x;  // column 0 of the staged row
    if (x == 0) {
      v[1].x = widen<ST>(st[1 * S::SROW + r0 + nx - 1]);
      v[5].x = widen<ST>(st[5 * S::SROW + r0 + nx - 1]);
      v[8].x = widen<ST>(st[8 * S::SROW + r0 + nx - 1]);
    }
    if (x == nx - 1) {
      v[3].x = widen<ST>(st[3 * S::SROW + r0]);
      v[6].x = widen<ST>(st[6 * S::SROW + r0]);
      v[7].x = widen<ST>(st[7 * S::SROW + r0]);
    }
    if (x + 1 == nx - 1) {
      v[3].y = widen<ST>(st[3 * S::SROW + r0]);
      v[6].y = widen<ST>(st[6 * S::SROW + r0]);
      v[7].y = widen<ST>(st[7 * S::SROW + r0]);
    }
  } else if (!kOpen) {
    if (x == 0) {
      const int k = (nx - 1) & (S::H - 1);
      v[1].x = widen<ST>(wr[0 * S::H + k]);
      v[5].x = widen<ST>(wr[1 * S::H + k]);
      v[8].x = widen<ST>(wr[2 * S::H + k]);
    }
    if (x == nx - 1) {
      v[3].x = widen<ST>(wr[3 * S::H]);
      v[6].x = widen<ST>(wr[4 * S::H]);
      v[7].x = widen<ST>(wr[5 * S::H]);
    }
    if (x + 1 == nx - 1) {
      v[3].y = widen<ST>(wr[3 * S::H]);
      v[6].y = widen<ST>(wr[4 * S::H]);
      v[7].y = widen<ST>(wr[5 * S::H]);
    }
  }
  uint32_t nm = 0, n0 = 0, np = 0;  // bits 0..3: cells x - 1 .. x + 2 of rows y - 1, y, y + 1
  if (solids) {
    const int q = word + (lane >> 4), sh = (2 * lane) & 31;
    nm = __funnelshift_r(sm[q], sm[q + 1], sh) & 15u;
    n0 = __funnelshift_r(sm[S::MW + q], sm[S::MW + q + 1], sh) & 15u;
    np = __funnelshift_r(sm[2 * S::MW + q], sm[2 * S::MW + q + 1], sh) & 15u;
    if ((nm | n0 | np) != 0u) {
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        if ((n0 >> (1 + k)) & 1u) continue;  // solid cell: its slots are never read
#pragma unroll
        for (int i = 1; i < kQ; ++i) {
          const uint32_t w = dir_cy(i) == 1 ? nm : (dir_cy(i) == -1 ? np : n0);
          if ((w >> (1 + k - dir_cx(i))) & 1u) {
            const float b = load_step<ST>(p.src + dir_opp(i) * plane + row + x + k);
            if (k == 0) v[i].x = b; else v[i].y = b;
          }
        }
      }
    }
  }
  if (kOpen) {
    if (x == 0) {
      v[1].x = p.eq_in[1];
      v[5].x = p.eq_in[5];
      v[8].x = p.eq_in[8];
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (x + k != nx - 1) continue;
#pragma unroll
      for (int i = 1; i < kQ; ++i) {
        if (dir_cx(i) != -1) continue;
        const uint32_t w = dir_cy(i) == 1 ? nm : (dir_cy(i) == -1 ? np : n0);
        const float val = ((w >> (1 + k)) & 1u)
                              ? load_step<ST>(p.src + dir_opp(i) * plane + row + (nx - 2))
                              : widen<ST>(st[i * S::SROW + lx + k]);
        if (k == 0) v[i].x = val; else v[i].y = val;
      }
    }
  }
  float2 out[kQ];
  collide_fast_t<FastF32x2>(v, p.k, out);
  const uint32_t ph = sr_pair_hash(p.key_base + row + x, rkey);
  uint32_t* d = reinterpret_cast<uint32_t*>(p.dst + row + x);
  uint32_t w[kQ];
#pragma unroll
  for (int i = 0; i < kQ; ++i) {
    w[i] = encode_pair_sr<ST>(out[i].x, out[i].y, i, ph);
    d[i * (plane / 2)] = w[i];
  }
  if constexpr (kHalo) {
    if (y == p.g.ny - 2) {
      const long long pl = p.halo[1] / 2;
      uint32_t* h = reinterpret_cast<uint32_t*>(p.dst + p.halo[0] + x);
      h[2 * pl] = w[2];
      h[5 * pl] = w[5];
      h[6 * pl] = w[6];
    }
    if (y == 1) {
      const long long pl = p.halo[3] / 2;
      uint32_t* h = reinterpret_cast<uint32_t*>(p.dst + p.halo[2] + x);
      h[4 * pl] = w[4];
      h[7 * pl] = w[7];
      h[8 * pl] = w[8];
    }
  }
}

// Producer work of one tile (row y, first cell tx0) of grid p into the stage at `base`: arms the
// stage's full barrier with the byte count, then issues the bulk copies of the 9 plane rows, the
// 3 mask rows and, on a periodic row's first / last tile, the wrap blocks.
template <class ST, class Phys, bool kOpen, class S>
__device__ __forceinline__ void ring_issue_tile(const StepArgs<ST, Phys>& p, unsigned char* base,
                                                uint64_t* full, int y, int tx0) {
  const int nx = p.g.nx, ny = p.g.ny;
  const int ym = y == 0 ? ny - 1 : y - 1;
  const int yp = y == ny - 1 ? 0 : y + 1;
  const int xs = tx0 - S::H > 0 ? tx0 - S::H : 0;
  const int xe = tx0 + S::TW + S::H < p.g.pitch ? tx0 + S::TW + S::H : p.g.pitch;
  const uint32_t bytes = static_cast<uint32_t>((xe - xs) * sizeof(ST));
  const bool wrap_lo = !kOpen && tx0 == 0;
  const bool wrap_hi = !kOpen && tx0 + S::TW >= nx;
  mbar_arrive_expect_tx(full, kQ * bytes + S::kMaskBytes + (wrap_lo ? 48u : 0u) + (wrap_hi ? 48u : 0u));
  ST* stage = reinterpret_cast<ST*>(base);
#pragma unroll
  for (int i = 0; i < kQ; ++i) {
    const ST* src = p.src + i * p.g.plane + static_cast<long long>(src_row(i, y, ym, yp)) * p.g.pitch + xs;
    bulk_copy_g2s(stage + i * S::SROW + (xs - (tx0 - S::H)), src, bytes, full);
  }
  uint32_t* smask = reinterpret_cast<uint32_t*>(base + S::kPlaneBytes);
  const int r3[3] = {ym, y, yp};
#pragma unroll
  for (int r = 0; r < 3; ++r)
    bulk_copy_g2s(smask + r * S::MW, p.mask + static_cast<size_t>(r3[r]) * p.g.mask_words + (tx0 >> 5),
                  S::MW * 4, full);
  ST* wr = reinterpret_cast<ST*>(base + S::kPlaneBytes + S::kMaskBytes);
  if (wrap_lo) {
    const int xb = (nx - 1) & ~(S::H - 1);
    for (int j = 0; j < 3; ++j) {
      const int i = wrap_dir(j);
      bulk_copy_g2s(wr + j * S::H,
                    p.src + i * p.g.plane + static_cast<long long>(src_row(i, y, ym, yp)) * p.g.pitch + xb, 16, full);
    }
  }
  if (wrap_hi) {
    for (int j = 3; j < 6; ++j) {
      const int i = wrap_dir(j);
      bulk_copy_g2s(wr + j * S::H, p.src + i * p.g.plane + static_cast<long long>(src_row(i, y, ym, yp)) * p.g.pitch,
                    16, full);
    }
  }
}

// Consumer work of one tile: warp cw's strip of the stage at `base`.
template <class ST, class Phys, bool kOpen, class S, int kC, bool kHalo = false>
__device__ __forceinline__ void ring_consume_tile(const StepArgs<ST, Phys>& p, const unsigned char* base,
                                                  int y, int tx0, int cw, int lane) {
  const int nx = p.g.nx, ny = p.g.ny;
  const int xw = tx0 + cw * S::SW;
  if (xw >= nx) return;
  const ST* st = reinterpret_cast<const ST*>(base);
  const uint32_t* sm = reinterpret_cast<const uint32_t*>(base + S::kPlaneBytes);
  const ST* wr = reinterpret_cast<const ST*>(base + S::kPlaneBytes + S::kMaskBytes);
  const int ym = y == 0 ? ny - 1 : y - 1;
  const int yp = y == ny - 1 ? 0 : y + 1;
  const int w0 = cw * S::WPS;  // first staged mask word of the strip
  // Any solid among the strip's cells and their neighbours (words w0 .. w0 + WPS of 3 rows).
  uint32_t mine = 0;
  if (lane < 3 * (S::WPS + 1)) mine = sm[(lane / (S::WPS + 1)) * S::MW + w0 + lane % (S::WPS + 1)];
  const bool solids = __any_sync(0xffffffffu, mine != 0u);
#pragma unroll 1
  for (int c = 0; c < kC; ++c) {
    const int x = xw + 32 * S::LC * c + S::LC * lane;
    if (x < nx) {
      if constexpr (S::LC == 2)
        ring_pair<ST, kOpen, S, false, kHalo>(p, st, sm, wr, y, x, x - tx0 + S::H, w0 + 2 * c, lane, solids,
                                              step_rkey(p));
      else
        ring_cell<ST, typename Phys::Arith, kOpen, S, false, kHalo>(p, st, sm, wr, y, ym, yp, x, x - tx0 + S::H, w0 + c,
                                                     lane, solids);
    }
  }
}

// Policies whose producer issues its copies from all 32 lanes set kWarpIssue (pol.issue then
// also gets the lane and must arm the barrier from one lane before any lane issues a copy).
template <class P, class = void>
struct warp_issue : std::false_type {};
template <class P>
struct warp_issue<P, std::void_t<decltype(P::kWarpIssue)>> : std::bool_constant<P::kWarpIssue> {};

// Warp-specialised pipeline over tiles 0 .. tiles - 1 (grid-stride) with a ring of kStages
// stages of kStageBytes: the block's j-th tile goes to stage j % kStages (use j / kStages of it)
// and is issued by producer warp j % kProd (one lane, or all lanes for kWarpIssue policies),
// which calls pol.issue(tile, stage, full_barrier) to arm the barrier with its byte count and
// issue the bulk copies. Several producers overlap the issue of consecutive tiles when a
// policy's issue is long (many short copies per tile); each issues its tiles in increasing j
// and waits for the release of tile j - kStages. That parity wait is exact only while the
// stage's `empty` barrier is at most one phase behind, i.e. tile j - 2 kStages already
// released: the producer's previous wait (for tile j - kProd - kStages) and the consumers'
// in-order releases guarantee it when kProd <= kStages, which is therefore required (a model
// of the schedule under random interleavings: tests/test_pipeline_schedule.py).
// Consumer warps kProd .. kProd + kW - 1 wait
// for the stage, call pol.consume(tile, stage, consumer_warp, lane) and release it. Waits are
// bounded (error flag; a consumer whose first wait ran out under the test limit drains, see
// consumer_wait_full). Afterwards every consumer warp (not the producers) calls
// pol.finish(cw, lane), also after a wait ran out (the host then reports the timeout), e.g. to
// write the warp's partial sums. Warps never synchronise with one another after the start, so
// a wait that ran out in one warp cannot leave another waiting at a barrier.
template <int kW, int kStages, int kStageBytes, int kProd = 1, class Pol>
__device__ __forceinline__ void tile_pipeline(unsigned char* smem, Pol& pol, int tiles, int* err) {
  static_assert(kProd >= 1 && kStages >= 1, "at least one producer warp and one stage");
  static_assert(kProd <= kStages, "a stage's barrier may run two phases behind a producer otherwise");
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(kStages) * kStageBytes);
  uint64_t* empty = full + kStages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kW);
    }
    mbar_fence_init();
  }
  __syncthreads();

  if (warp < kProd) {
    constexpr bool kWarp = warp_issue<Pol>::value;
    if (!kWarp && lane != 0) return;
    if constexpr (kProd == 1) {
      // The single producer: stage and phase advanced incrementally (this form of the loop is
      // what the producer-bound adjoint kernels were tuned with; the general form below made
      // them 4-7 % slower).
      int s = 0, issued = 0;
      uint32_t phase = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++issued) {
        if (issued >= kStages) {
          const bool got = kWarp ? mbar_wait_bounded_warp(&empty[s], phase ^ 1u, err)
                                 : mbar_wait_bounded(&empty[s], phase ^ 1u, err);
          if (!got) {
            ok = false;
            break;
          }
        }
        if constexpr (kWarp)
          pol.issue(tile, smem + static_cast<size_t>(s) * kStageBytes, &full[s], lane);
        else
          pol.issue(tile, smem + static_cast<size_t>(s) * kStageBytes, &full[s]);
        if (++s == kStages) {
          s = 0;
          phase ^= 1u;
        }
      }
      if (!ok && lane == 0) {
        for (int k = 0; k < kStages && k < issued; ++k) {
          const int st = (s + kStages - 1 - k) % kStages;
          const int use = (issued - 1 - k) / kStages;
          mbar_wait_bounded(&full[st], static_cast<uint32_t>(use & 1), err);
        }
      }
      return;
    }
    // Producer `warp` of several.
    bool ok = true;
    int last = -1;
    for (int j = warp;; j += kProd) {
      const int tile = blockIdx.x + j * gridDim.x;
      if (tile >= tiles) break;
      const int s = j % kStages;
      if (j >= kStages) {
        const uint32_t parity = static_cast<uint32_t>((j / kStages - 1) & 1);
        const bool got = kWarp ? mbar_wait_bounded_warp(&empty[s], parity, err)
                               : mbar_wait_bounded(&empty[s], parity, err);
        if (!got) {
          ok = false;
          break;
        }
      }
      if constexpr (kWarp)
        pol.issue(tile, smem + static_cast<size_t>(s) * kStageBytes, &full[s], lane);
      else
        pol.issue(tile, smem + static_cast<size_t>(s) * kStageBytes, &full[s]);
      last = j;
    }
    if (!ok && lane == 0) {
      // Let this producer's copies still in flight land before the block exits.
      for (int j = last; j >= 0 && j > last - kStages; j -= kProd)
        mbar_wait_bounded(&full[j % kStages], static_cast<uint32_t>((j / kStages) & 1), err);
    }
    return;
  }

  // Consumers. A warp whose wait ran out under the test limit drains (consumer_wait_full).
  const int cw = warp - kProd;
  int s = 0;
  uint32_t phase = 0;
  bool drain = false;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int got = drain ? (mbar_wait_bounded_warp(&full[s], phase, err) ? 2 : 0)
                          : consumer_wait_full(&full[s], phase, err);
    if (!got) break;
    drain = got == 2;
    if (!drain) pol.consume(tile, smem + static_cast<size_t>(s) * kStageBytes, cw, lane);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    if (++s == kStages) {
      s = 0;
      phase ^= 1u;
    }
  }
  if (Pol::kFinish) pol.finish(cw, lane);
}

// The step pipeline of one tile visitor (`tiles_of.visit(tile, f)` calls f(p, y, tx0) with the
// grid, row and first cell of a tile; GridTiles below for the solver and the strip engine).
// The batched ensemble and the adjoint use tile_pipeline with their own stage policies
// (batch.cu, adjoint.cu).
template <class ST, class Phys, bool kOpen, int kW, int kC, class Tiles, bool kHalo = false>
struct StepPolicy {
  using S = RingShape<ST, kW, kC>;
  static constexpr bool kFinish = false;
  const Tiles& tiles_of;
  __device__ __forceinline__ void issue(int tile, unsigned char* base, uint64_t* full) const {
    tiles_of.visit(tile, [&](const StepArgs<ST, Phys>& p, int y, int tx0) {
      ring_issue_tile<ST, Phys, kOpen, S>(p, base, full, y, tx0);
    });
  }
  __device__ __forceinline__ void consume(int tile, const unsigned char* base, int cw, int lane) const {
    tiles_of.visit(tile, [&](const StepArgs<ST, Phys>& p, int y, int tx0) {
      ring_consume_tile<ST, Phys, kOpen, S, kC, kHalo>(p, base, y, tx0, cw, lane);
    });
  }
  __device__ __forceinline__ void finish(int, int) const {}
};

template <class ST, class Phys, bool kOpen, int kW, int kC, int kStages, class Tiles, bool kHalo = false>
__device__ __forceinline__ void ring_pipeline(unsigned char* smem, const Tiles& tiles_of, int tiles, int* err) {
  using S = RingShape<ST, kW, kC>;
  StepPolicy<ST, Phys, kOpen, kW, kC, Tiles, kHalo> pol{tiles_of};
  tile_pipeline<kW, kStages, S::kStageBytes>(smem, pol, tiles, err);
}

// Tiles of one grid: tiles_per_row tiles per row, rows row0, row0 + 1, ...; with `reverse` the
// blocks walk them from the last one, so that a step started right after one that walked
// forward first reads the rows that step wrote last, which are still in L2 (the launches
// alternate: on a 4096^2 FP32 grid the 129 MB L2 holds about a sixth of a 604 MB state).
// Each consumer warp decodes the tile itself: a multiply-high division by the invariant
// tiles_per_row made the FP32 step 3 % slower (88.3k against 91.0k MLUPS at 4096^2), and the
// producer decoding once and handing the row to the consumers through the stage, as the strip
// engine does with its heavier decoding, 1.4 % slower (89.4k against 90.7k).
template <class ST, class Phys, int kTW>
struct GridTiles {
  const StepArgs<ST, Phys>& p;
  int tiles_per_row, row0, tiles, reverse;
  template <class F>
  __device__ __forceinline__ void visit(int tile, F&& f) const {
    if (reverse) tile = tiles - 1 - tile;
    const int tr = tile / tiles_per_row;
    f(p, row0 + tr, (tile - tr * tiles_per_row) * kTW);
  }
};

template <class ST, class Phys, bool kOpen, int kW, int kC, int kStages, int kMinBlocks>
__global__ void __launch_bounds__(32 * (kW + 1), kMinBlocks)
    ring_step_kernel(const StepArgs<ST, Phys> p, int tiles_per_row, int tiles, int row0, int reverse, int* err) {
  using S = RingShape<ST, kW, kC>;
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dependency_wait();
  const GridTiles<ST, Phys, S::TW> grid_tiles{p, tiles_per_row, row0, tiles, reverse};
  ring_pipeline<ST, Phys, kOpen, kW, kC, kStages>(smem, grid_tiles, tiles, err);
}

}  // namespace lbm_b200
