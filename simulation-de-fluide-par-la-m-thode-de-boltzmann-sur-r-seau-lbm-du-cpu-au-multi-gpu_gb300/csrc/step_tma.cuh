// Warp-specialised pull stream-collide step with bulk asynchronous copies (TMA) into a
// shared-memory ring. Same results as pull_step_kernel (step_kernel.cuh), different data path:
//
//   * a tile is TW = kConsumers * 32 * G consecutive cells of one row;
//   * warp 0 (producer, one lane) streams, for each tile of the block, the 9 source plane rows
//     (plane i, row y - cy_i, columns tx0 - G .. tx0 + TW + G, clamped to the row) and the three
//     mask rows y - 1, y, y + 1 of the tile into ring stage s with 12 cp.async.bulk copies
//     completing on the stage's "full" mbarrier;
//   * warps 1..kConsumers (consumers) wait for the stage, read their G cells of every plane
//     with one aligned 16-byte shared load plus one element for the x shift, apply bounce-back
//     and the collision, store straight to global memory, and release the stage on its "empty"
//     mbarrier;
//   * bytes in flight per SM are set by the ring depth (kStages stages of ~37 KB), not by
//     registers, so the consumers compute while the next tiles stream in.
// Waits are bounded: a wait that exceeds kSpinLimit polls sets *err and the block stops issuing
// and consuming (the host reports LBM_ERR_TIMEOUT); the producer first waits, again bounded,
// for the copies it has in flight.
#pragma once

#include "step_kernel.cuh"

namespace lbm_b200 {

constexpr int kConsumers = 8;
constexpr int kTmaThreads = 32 * (1 + kConsumers);
constexpr unsigned kSpinLimit = 1u << 26;

template <class ST>
struct TmaShape {
  static constexpr int G = StoreTraits<ST>::kVec;
  static constexpr int H = G;                    // halo elements (16 bytes) on each side
  static constexpr int TW = kConsumers * 32 * G; // tile width in cells
  static constexpr int SROW = TW + 2 * H;        // shared row length in elements
  static constexpr int MW = TW / 32 + 4;         // mask words staged per row (16-byte multiple)
  static constexpr int kPlaneBytes = kQ * SROW * static_cast<int>(sizeof(ST));
  static constexpr int kStageBytes = kPlaneBytes + 3 * MW * 4;
};

template <class ST>
constexpr size_t tma_smem_bytes(int stages) {
  return static_cast<size_t>(stages) * TmaShape<ST>::kStageBytes + 2 * stages * sizeof(uint64_t);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait by one thread; returns false (after setting *err) when the limit is reached.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err) {
  for (unsigned it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  atomicExch(err, 1);
  return false;
}

// Bounded wait by a whole warp, with a warp-uniform result: every lane observes the phase
// completion itself (acquire for its own shared-memory reads), the warp leaves together.
__device__ __forceinline__ bool mbar_wait_bounded_warp(uint64_t* bar, uint32_t parity, int* err) {
  for (unsigned it = 0; it < kSpinLimit; ++it)
    if (__all_sync(0xffffffffu, mbar_try_wait(bar, parity))) return true;
  if ((threadIdx.x & 31) == 0) atomicExch(err, 1);
  return false;
}

// Non-blocking test of a phase's completion (one poll, no suspension).
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Limit of a ring consumer's first wait for a full stage (tile_pipeline, step_ring.cuh), in
// non-blocking polls. kSpinLimit, the default, selects the ordinary bounded wait. A smaller
// value is a test setting (lbm_test_set_consumer_wait_limit, solver.cu) that makes the wait run
// out on purpose: the consumer warp then sets the error flag and drains, i.e. waits (bounded,
// blocking) for that stage and every later stage of its block and releases them without
// computing, so the producer is never left waiting and no copy is still in flight into a block
// that has exited. Each translation unit holds its own copy; only the solver's is settable.
static __constant__ unsigned c_consumer_wait_limit = kSpinLimit;

// A consumer warp's wait for a full stage: 1 = data ready, 2 = the test limit ran out (error
// flag set) and the stage's copies have landed (drain from here on), 0 = a bounded wait ran
// out (error flag set).
__device__ __forceinline__ int consumer_wait_full(uint64_t* bar, uint32_t parity, int* err) {
  const unsigned limit = c_consumer_wait_limit;
  if (limit < kSpinLimit) {
    for (unsigned it = 0; it < limit; ++it)
      if (__all_sync(0xffffffffu, mbar_test_wait(bar, parity))) return 1;
    if ((threadIdx.x & 31) == 0) atomicExch(err, 1);
    return mbar_wait_bounded_warp(bar, parity, err) ? 2 : 0;
  }
  return mbar_wait_bounded_warp(bar, parity, err) ? 1 : 0;
}

// One-dimensional bulk copy global -> shared, completing `bytes` on the mbarrier.
__device__ __forceinline__ void bulk_copy_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Shared-memory vector load of G elements (16 bytes, aligned), decoded.
template <class ST>
__device__ __forceinline__ void lds_vec(const ST* p, typename StoreTraits<ST>::T (&v)[StoreTraits<ST>::kVec],
                                        int i, const PlaneScales& sc);
template <>
__device__ __forceinline__ void lds_vec<float>(const float* p, float (&v)[4], int, const PlaneScales&) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x;
  v[1] = t.y;
  v[2] = t.z;
  v[3] = t.w;
}
template <>
__device__ __forceinline__ void lds_vec<double>(const double* p, double (&v)[2], int, const PlaneScales&) {
  const double2 t = *reinterpret_cast<const double2*>(p);
  v[0] = t.x;
  v[1] = t.y;
}
template <class H>
__device__ __forceinline__ void lds_vec16(const H* p, float (&v)[8], int, const PlaneScales&) {
  const uint4 t = *reinterpret_cast<const uint4*>(p);
  const uint32_t w[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    H lo, hi;
    const uint16_t a = static_cast<uint16_t>(w[k] & 0xffffu), b = static_cast<uint16_t>(w[k] >> 16);
    memcpy(&lo, &a, 2);
    memcpy(&hi, &b, 2);
    v[2 * k] = to_float(lo);  // scaled values (compute representation of the step kernels)
    v[2 * k + 1] = to_float(hi);
  }
}
template <>
__device__ __forceinline__ void lds_vec<__half>(const __half* p, float (&v)[8], int i, const PlaneScales& s) {
  lds_vec16(p, v, i, s);
}
template <>
__device__ __forceinline__ void lds_vec<__nv_bfloat16>(const __nv_bfloat16* p, float (&v)[8], int i,
                                                       const PlaneScales& s) {
  lds_vec16(p, v, i, s);
}

template <class ST>
__device__ __forceinline__ typename StoreTraits<ST>::T lds_one(const ST* p, int, const PlaneScales&) {
  return widen<ST>(*p);
}

// Mask window of cells x0 - 1 .. x0 + 30 from a staged mask row whose word 0 is word wb of the
// row.
__device__ __forceinline__ uint32_t smem_mask_window(const uint32_t* row, int x0, int wb) {
  const int w = (x0 >> 5) - wb;
  return __funnelshift_r(row[w], row[w + 1], x0 & 31);
}

// Collides one lane's G cells x0 .. x0 + G - 1 of row y, reading the source planes from shared
// memory (plane i row at st + i * kSrow, cell x0 at local column lx; the elements at lx - 1 and
// lx + G hold cells x0 - 1 and x0 + G wherever those lie inside the row) and the mask rows
// y - 1, y, y + 1 from `sm` (3 rows of kMw words, word 0 = word wb of the row). Every lane of the
// warp calls it (warp-uniform skip of all-solid groups).
template <class ST, class Phys, bool kOpen, int kSrow, int kMw>
__device__ __forceinline__ void consume_cells(const StepArgs<ST, Phys>& p, const ST* st,
                                              const uint32_t* sm, int wb, int y, int x0, int lx) {
  using T = typename StoreTraits<ST>::T;
  constexpr int G = StoreTraits<ST>::kVec;
  constexpr uint32_t kFull = (1u << G) - 1u;
  const int nx = p.g.nx, ny = p.g.ny, pitch = p.g.pitch;
  const long long plane = p.g.plane;
  const bool active = x0 < nx;
  const int ym = y == 0 ? ny - 1 : y - 1;
  const int yp = y == ny - 1 ? 0 : y + 1;

  const uint32_t wm = smem_mask_window(sm, x0, wb);
  const uint32_t w0 = smem_mask_window(sm + kMw, x0, wb);
  const uint32_t wp = smem_mask_window(sm + 2 * kMw, x0, wb);
  const int valid = nx - x0;
  uint32_t own = (w0 >> 1) & kFull;
  if (valid < G) own |= valid <= 0 ? kFull : (kFull & ~((1u << valid) - 1u));
  if (__all_sync(0xffffffffu, own == kFull)) return;
  if (!active) return;

  T v[kQ][G];
#pragma unroll
  for (int i = 0; i < kQ; ++i) {
    const ST* row = st + i * kSrow;
    lds_vec<ST>(row + lx, v[i], i, p.sc);
    if (dir_cx(i) == 1) {
      // cell x0 + k reads x0 + k - 1
      T left;
      if (x0 > 0) {
        left = lds_one<ST>(row + lx - 1, i, p.sc);
      } else {
        const ST* g = p.src + i * plane + static_cast<long long>(src_row(i, y, ym, yp)) * pitch;
        left = kOpen ? T(0) : load_step<ST>(g + (nx - 1));
      }
#pragma unroll
      for (int k = G - 1; k > 0; --k) v[i][k] = v[i][k - 1];
      v[i][0] = left;
    } else if (dir_cx(i) == -1) {
      // cell x0 + k reads x0 + k + 1
      const T right = lds_one<ST>(row + lx + G, i, p.sc);
#pragma unroll
      for (int k = 0; k < G - 1; ++k) v[i][k] = v[i][k + 1];
      v[i][G - 1] = right;
      if (!kOpen) {
        const int kl = nx - 1 - x0;  // periodic wrap: cell nx - 1 reads x = 0
        if (kl >= 0 && kl < G) {
          const ST* g = p.src + i * plane + static_cast<long long>(src_row(i, y, ym, yp)) * pitch;
          const T w = load_step<ST>(g);
#pragma unroll
          for (int k = 0; k < G; ++k)
            if (k == kl) v[i][k] = w;
        }
      }
    }
  }

  constexpr uint32_t kWin = (1u << (G + 2)) - 1u;
  if (((wm | w0 | wp) & kWin) != 0u) {
#pragma unroll
    for (int i = 1; i < kQ; ++i) {
      const uint32_t w = dir_cy(i) == 1 ? wm : (dir_cy(i) == -1 ? wp : w0);
      const uint32_t bounce = (w >> (1 - dir_cx(i))) & kFull & ~own;
      if (bounce) {
        T b[G];
        load_vec<ST>(p.src + dir_opp(i) * plane + static_cast<long long>(y) * pitch + x0, b,
                     dir_opp(i), p.sc);  // step representation
#pragma unroll
        for (int k = 0; k < G; ++k)
          if ((bounce >> k) & 1u) v[i][k] = b[k];
      }
    }
  }

  if (kOpen) {
    if (x0 == 0) {
      v[1][0] = p.eq_in[1];
      v[5][0] = p.eq_in[5];
      v[8][0] = p.eq_in[8];
    }
    const int kl = nx - 1 - x0;
    if (kl >= 0 && kl < G) {
#pragma unroll
      for (int i = 1; i < kQ; ++i) {
        if (dir_cx(i) != -1) continue;
        const int r = src_row(i, y, ym, yp);
        const uint32_t w = dir_cy(i) == 1 ? wm : (dir_cy(i) == -1 ? wp : w0);
        const bool solid_src = (w >> (kl + 1)) & 1u;
        const T val = solid_src
                          ? load_step<ST>(p.src + dir_opp(i) * plane + static_cast<long long>(y) * pitch + (nx - 2))
                          : load_step<ST>(p.src + i * plane + static_cast<long long>(r) * pitch + (nx - 1));
#pragma unroll
        for (int k = 0; k < G; ++k)
          if (k == kl) v[i][k] = val;
      }
    }
  }

  T out[kQ][G];
  Phys::template collide_all<G>(v, p.k, out);
  using SS = StepStore<ST, G>;
  uint32_t ph[SS::kPairs];
  if constexpr (SS::kSr) SS::hashes(p.key_base + static_cast<long long>(y) * pitch + x0, step_rkey(p), ph);
#pragma unroll
  for (int i = 0; i < kQ; ++i)
    SS::store(p.dst + i * plane + static_cast<long long>(y) * pitch + x0, out[i], i, p.sc, ph);
}

template <class ST, class Phys, bool kOpen, int kStages>
__global__ void __launch_bounds__(kTmaThreads, kStages <= 3 ? 2 : 1)
    tma_step_kernel(const StepArgs<ST, Phys> p, int tiles_per_row, int tiles, int* err) {
  using S = TmaShape<ST>;
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dependency_wait();
  // Stage s: 9 plane rows (kPlaneBytes) then 3 mask rows (3 * MW words).
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(kStages) * S::kStageBytes);
  uint64_t* empty = full + kStages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumers);
    }
    mbar_fence_init();
  }
  __syncthreads();

  if (warp == 0) {
    if (lane != 0) return;
    // Producer.
    int s = 0, issued = 0;
    uint32_t phase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++issued) {
      if (issued >= kStages && !mbar_wait_bounded(&empty[s], phase ^ 1u, err)) {
        ok = false;
        break;
      }
      const int y = tile / tiles_per_row;
      const int tx0 = (tile - y * tiles_per_row) * S::TW;
      const int ym = y == 0 ? p.g.ny - 1 : y - 1;
      const int yp = y == p.g.ny - 1 ? 0 : y + 1;
      const int xs = tx0 - S::H > 0 ? tx0 - S::H : 0;
      const int xe = tx0 + S::TW + S::H < p.g.pitch ? tx0 + S::TW + S::H : p.g.pitch;
      const uint32_t bytes = static_cast<uint32_t>((xe - xs) * sizeof(ST));
      mbar_arrive_expect_tx(&full[s], kQ * bytes + 3 * S::MW * 4);
      unsigned char* base = smem + static_cast<size_t>(s) * S::kStageBytes;
      ST* stage = reinterpret_cast<ST*>(base);
#pragma unroll
      for (int i = 0; i < kQ; ++i) {
        const ST* src = p.src + i * p.g.plane + static_cast<long long>(src_row(i, y, ym, yp)) * p.g.pitch + xs;
        bulk_copy_g2s(stage + i * S::SROW + (xs - (tx0 - S::H)), src, bytes, &full[s]);
      }
      uint32_t* smask = reinterpret_cast<uint32_t*>(base + S::kPlaneBytes);
      const int r3[3] = {ym, y, yp};
#pragma unroll
      for (int r = 0; r < 3; ++r)
        bulk_copy_g2s(smask + r * S::MW,
                      p.mask + static_cast<size_t>(r3[r]) * p.g.mask_words + (tx0 >> 5),
                      S::MW * 4, &full[s]);
      if (++s == kStages) {
        s = 0;
        phase ^= 1u;
      }
    }
    if (!ok) {
      // Stop: wait (bounded) for the copies still in flight into the ring.
      for (int k = 0; k < kStages && k < issued; ++k) {
        const int st = (s + kStages - 1 - k) % kStages;
        const int use = (issued - 1 - k) / kStages;
        mbar_wait_bounded(&full[st], static_cast<uint32_t>(use & 1), err);
      }
    }
    return;
  }

  // Consumers.
  const int cw = warp - 1;
  int s = 0;
  uint32_t phase = 0;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    if (!mbar_wait_bounded_warp(&full[s], phase, err)) return;
    const int y = tile / tiles_per_row;
    const int tx0 = (tile - y * tiles_per_row) * S::TW;
    const unsigned char* base = smem + static_cast<size_t>(s) * S::kStageBytes;
    const int x0 = tx0 + cw * 32 * S::G + lane * S::G;
    consume_cells<ST, Phys, kOpen, S::SROW, S::MW>(
        p, reinterpret_cast<const ST*>(base), reinterpret_cast<const uint32_t*>(base + S::kPlaneBytes),
        tx0 >> 5, y, x0, x0 - tx0 + S::H);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    if (++s == kStages) {
      s = 0;
      phase ^= 1u;
    }
  }
}

}  // namespace lbm_b200
