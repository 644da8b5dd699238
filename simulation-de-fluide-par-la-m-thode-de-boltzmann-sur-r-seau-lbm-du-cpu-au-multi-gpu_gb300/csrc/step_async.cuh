// Pull stream-collide step with a per-warp asynchronous-copy pipeline. Same results as
// pull_step_kernel (step_kernel.cuh) and tma_step_kernel (step_tma.cuh); different data path:
//
//   * a warp owns chunks of 32 * G consecutive cells of one row (G cells per lane), taken
//     grid-stride like the direct kernel;
//   * each warp keeps kDepth chunks in a private shared-memory ring: while it collides chunk k,
//     the 16-byte cp.async copies of chunks k + 1 .. k + kDepth - 1 are in flight (the 9 source
//     plane rows of the chunk plus a 16-byte halo on each side, and its 3 mask rows), so the bytes
//     in flight per SM are set by the ring, not by registers;
//   * warps never wait on one another: completion is the warp's own cp.async.wait_group (a
//     hardware wait, no polling) followed by __syncwarp, which orders the lanes' copies before the
//     other lanes read them;
//   * the collision reads the stage exactly like the bulk-copy kernel's consumers
//     (consume_cells).
#pragma once

#include "step_tma.cuh"

namespace lbm_b200 {

template <class ST>
struct AsyncShape {
  static constexpr int G = StoreTraits<ST>::kVec;
  static constexpr int H = G;                   // halo elements (16 bytes) on each side
  static constexpr int CW = 32 * G;             // chunk width in cells
  static constexpr int SROW = CW + 2 * H;       // staged row length in elements (544 bytes)
  static constexpr int MW = 12;                 // mask words staged per row (3 x 16 bytes)
  static constexpr int kPlaneBytes = kQ * SROW * static_cast<int>(sizeof(ST));
  static constexpr int kStageBytes = kPlaneBytes + 3 * MW * 4;
  static_assert(kStageBytes % 16 == 0, "stages must keep 16-byte alignment");
};

template <class ST>
constexpr size_t async_smem_bytes(int depth, int warps) {
  return static_cast<size_t>(depth) * warps * AsyncShape<ST>::kStageBytes;
}

__device__ __forceinline__ void cp_async16(void* dst_smem, const void* src_gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst_smem)), "l"(src_gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// First staged mask word of a chunk starting at cell x0c: word x0c / 32 rounded down to a
// multiple of 4 (16-byte aligned). The staged 12 words cover every window of the chunk.
__device__ __forceinline__ int chunk_mask_base(int x0c) { return (x0c >> 5) & ~3; }

// Issues this lane's copies of chunk `item` into stage `st`:
//   lanes with cells in the row: their 16-byte vector of each plane;
//   lanes 0..8: left halo of plane `lane` (16 bytes before the chunk) when the chunk is not the
//   first of its row; lanes 9..17: right halo of plane lane - 9 when it lies inside the row pitch;
//   lanes 18..26: 16 bytes (4 words) each of the 3 staged mask rows.
template <class ST, class Phys>
__device__ __forceinline__ void issue_chunk(const StepArgs<ST, Phys>& p, unsigned char* st, int item,
                                            int lane) {
  using S = AsyncShape<ST>;
  constexpr int G = S::G;
  const int y = item / p.cpr;
  const int x0c = (item - y * p.cpr) * S::CW;
  const int ym = y == 0 ? p.g.ny - 1 : y - 1;
  const int yp = y == p.g.ny - 1 ? 0 : y + 1;
  ST* stage = reinterpret_cast<ST*>(st);
  const int x0 = x0c + lane * G;
  if (x0 < p.g.nx) {
#pragma unroll
    for (int i = 0; i < kQ; ++i)
      cp_async16(stage + i * S::SROW + S::H + lane * G,
                 p.src + i * p.g.plane + static_cast<long long>(src_row(i, y, ym, yp)) * p.g.pitch + x0);
  }
  if (lane < kQ) {
    if (x0c > 0)
      cp_async16(stage + lane * S::SROW,
                 p.src + lane * p.g.plane + static_cast<long long>(src_row(lane, y, ym, yp)) * p.g.pitch +
                     (x0c - G));
  } else if (lane < 2 * kQ) {
    const int i = lane - kQ;
    if (x0c + S::CW < p.g.pitch)
      cp_async16(stage + i * S::SROW + S::H + S::CW,
                 p.src + i * p.g.plane + static_cast<long long>(src_row(i, y, ym, yp)) * p.g.pitch +
                     (x0c + S::CW));
  } else if (lane < 2 * kQ + 9) {
    const int k = lane - 2 * kQ;  // 0..8: row k / 3 (y - 1, y, y + 1), part k % 3
    const int r = k / 3, part = k - 3 * r;
    const int row = r == 0 ? ym : (r == 1 ? y : yp);
    uint32_t* smask = reinterpret_cast<uint32_t*>(st + S::kPlaneBytes);
    cp_async16(smask + r * S::MW + 4 * part,
               p.mask + static_cast<size_t>(row) * p.g.mask_words + chunk_mask_base(x0c) + 4 * part);
  }
}

template <class ST, class Phys, bool kOpen, int kDepth>
__global__ void __launch_bounds__(128) async_step_kernel(const StepArgs<ST, Phys> p) {
  using S = AsyncShape<ST>;
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dependency_wait();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  unsigned char* ring = smem + static_cast<size_t>(warp) * kDepth * S::kStageBytes;
  const int first = blockIdx.x * wpb + warp;
  const int stride = gridDim.x * wpb;

#pragma unroll
  for (int d = 0; d < kDepth - 1; ++d) {
    const int it = first + d * stride;
    if (it < p.items) issue_chunk<ST, Phys>(p, ring + d * S::kStageBytes, it, lane);
    cp_async_commit();
  }
  int s = 0;
  for (int item = first; item < p.items; item += stride) {
    const int ahead = item + (kDepth - 1) * stride;
    const int sa = s == 0 ? kDepth - 1 : s - 1;  // stage of chunk k + kDepth - 1 = (k - 1) mod kDepth
    if (ahead < p.items) issue_chunk<ST, Phys>(p, ring + sa * S::kStageBytes, ahead, lane);
    cp_async_commit();
    cp_async_wait<kDepth - 1>();
    __syncwarp();
    const unsigned char* st = ring + s * S::kStageBytes;
    const int y = item / p.cpr;
    const int x0c = (item - y * p.cpr) * S::CW;
    consume_cells<ST, Phys, kOpen, S::SROW, S::MW>(
        p, reinterpret_cast<const ST*>(st), reinterpret_cast<const uint32_t*>(st + S::kPlaneBytes),
        chunk_mask_base(x0c), y, x0c + lane * S::G, S::H + lane * S::G);
    __syncwarp();
    if (++s == kDepth) s = 0;
  }
  cp_async_wait<0>();
}

}  // namespace lbm_b200
