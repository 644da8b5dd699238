// Single-grid solver: device memory, launches and the C ABI of include/lbm_b200.h.
//
// Host code of this file is compiled with -ffp-contract=off: the per-launch constants (omega,
// the force prefactor, the inlet and initial equilibria) are computed here in the solver
// precision with the reference's expressions, and must round exactly as the reference's host
// code does (src/v3_cuda_opt/solver_v3.cu:194-226,252-253).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "aux_kernels.cuh"
#include "lbm_b200.h"
#include "solver_internal.h"
#include "step_kernel.cuh"
#include "step_async.cuh"
#include "step_ring.cuh"
#include "step_tma.cuh"
#include "forms.cuh"

using namespace lbm_b200;

namespace {

int set_error(lbm_solver* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}

int cuda_fail(lbm_solver* s, cudaError_t e, const char* what) {
  cudaGetLastError();  // clear a sticky launch error so that later calls can report their own
  const int code = e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA;
  return set_error(s, code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define LBM_CUDA(s, call)                                   \
  do {                                                      \
    const cudaError_t lbm_e_ = (call);                      \
    if (lbm_e_ != cudaSuccess) return cuda_fail(s, lbm_e_, #call); \
  } while (0)

int grid_for_cells(const lbm_solver* s, long long n, int block) {
  const long long want = (n + block - 1) / block;
  return static_cast<int>(std::max<long long>(1, std::min<long long>(want, 32LL * s->sm_count)));
}

template <class ST>
Eq9<typename StoreTraits<ST>::T> inlet_eq(const lbm_solver* s) {
  using T = typename StoreTraits<ST>::T;
  if (!s->open_x) return Eq9<T>{};
  return host_equilibrium<T>(T(1), T(s->u_in), T(0));
}

// The inlet equilibrium in the step kernels' compute representation (16-bit forms: scaled).
template <class ST>
Eq9<typename StoreTraits<ST>::T> step_inlet_eq(const lbm_solver* s) {
  Eq9<typename StoreTraits<ST>::T> e = inlet_eq<ST>(s);
  if (sizeof(ST) == 2)
    for (int i = 0; i < kQ; ++i) e.v[i] *= s->sc.enc[i];
  return e;
}

// Physics of a launch: the scalar form, or (kPacked) its two-cells-per-instruction twin.
template <class ST, bool kPacked>
using PhysOf = std::conditional_t<kPacked, typename Form<ST>::PackedPhys, typename Form<ST>::Phys>;

template <class ST, bool kOpen, int kVariant, bool kPacked = false>
int launch_steps_t(lbm_solver* s, int steps) {
  using Phys = PhysOf<ST, kPacked>;
  using T = typename StoreTraits<ST>::T;
  constexpr int G = StoreTraits<ST>::kVec;
  StepArgs<ST, Phys> a{};
  a.mask = s->mask_d;
  a.g = s->g;
  a.cpr = (s->nx + 32 * G - 1) / (32 * G);
  a.items = s->ny * a.cpr;
  a.k = Form<ST>::consts(s->tau, s->fx, s->fy);
  const Eq9<T> e = step_inlet_eq<ST>(s);
  for (int i = 0; i < kQ; ++i) a.eq_in[i] = e.v[i];
  a.sc = s->sc;
  const auto kernel = pull_step_kernel<ST, Phys, kOpen, kVariant>;
  int grid = s->grid;
  if (grid <= 0) {
    int per_sm = 0;
    LBM_CUDA(s, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, s->block, 0));
    const int warps_per_block = s->block / 32;
    const int need = (a.items + warps_per_block - 1) / warps_per_block;
    grid = std::max(1, std::min(need, std::max(1, per_sm) * s->sm_count));
  }
  s->last_grid = grid;
  for (int k = 0; k < steps; ++k) {
    a.src = static_cast<const ST*>(s->buf[s->cur]);
    a.dst = static_cast<ST*>(s->buf[s->cur ^ 1]);
    a.step_ctr = s->step_ctr;
    a.step_off = static_cast<uint32_t>(k);
    LBM_CUDA(s, launch_dependent(kernel, dim3(grid), dim3(s->block), 0, s->stream, a));
    s->cur ^= 1;
  }
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

// Warp-specialised bulk-copy step (step_tma.cuh) with kStages ring stages.
template <class ST, bool kOpen, int kStages, bool kPacked = false>
int launch_tma_t(lbm_solver* s, int steps) {
  using Phys = PhysOf<ST, kPacked>;
  using T = typename StoreTraits<ST>::T;
  using S = TmaShape<ST>;
  StepArgs<ST, Phys> a{};
  a.mask = s->mask_d;
  a.g = s->g;
  a.cpr = (s->nx + 32 * S::G - 1) / (32 * S::G);
  a.items = s->ny * a.cpr;
  a.k = Form<ST>::consts(s->tau, s->fx, s->fy);
  const Eq9<T> e = step_inlet_eq<ST>(s);
  for (int i = 0; i < kQ; ++i) a.eq_in[i] = e.v[i];
  a.sc = s->sc;
  const int tpr = (s->nx + S::TW - 1) / S::TW;
  const int tiles = tpr * s->ny;
  const auto kernel = tma_step_kernel<ST, Phys, kOpen, kStages>;
  const size_t smem = tma_smem_bytes<ST>(kStages);
  LBM_CUDA(s, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
  int grid = s->grid;
  if (grid <= 0) {
    int per_sm = 0;
    LBM_CUDA(s, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTmaThreads, smem));
    grid = std::max(1, std::min(tiles, std::max(1, per_sm) * s->sm_count));
  }
  s->last_grid = grid;
  for (int k = 0; k < steps; ++k) {
    a.src = static_cast<const ST*>(s->buf[s->cur]);
    a.dst = static_cast<ST*>(s->buf[s->cur ^ 1]);
    a.step_ctr = s->step_ctr;
    a.step_off = static_cast<uint32_t>(k);
    LBM_CUDA(s, launch_dependent(kernel, dim3(grid), dim3(kTmaThreads), smem, s->stream, a, tpr, tiles,
                                 s->err_flag));
    s->cur ^= 1;
  }
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

// Per-warp asynchronous-copy pipeline (step_async.cuh), kDepth chunks per warp, 4 warps per block.
template <class ST, bool kOpen, int kDepth, bool kPacked = true>
int launch_async_t(lbm_solver* s, int steps) {
  using Phys = PhysOf<ST, kPacked>;
  using T = typename StoreTraits<ST>::T;
  constexpr int G = StoreTraits<ST>::kVec;
  constexpr int kBlock = 128;
  StepArgs<ST, Phys> a{};
  a.mask = s->mask_d;
  a.g = s->g;
  a.cpr = (s->nx + 32 * G - 1) / (32 * G);
  a.items = s->ny * a.cpr;
  a.k = Form<ST>::consts(s->tau, s->fx, s->fy);
  const Eq9<T> e = step_inlet_eq<ST>(s);
  for (int i = 0; i < kQ; ++i) a.eq_in[i] = e.v[i];
  a.sc = s->sc;
  const auto kernel = async_step_kernel<ST, Phys, kOpen, kDepth>;
  const size_t smem = async_smem_bytes<ST>(kDepth, kBlock / 32);
  LBM_CUDA(s, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
  int grid = s->grid;
  if (grid <= 0) {
    int per_sm = 0;
    LBM_CUDA(s, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem));
    const int need = (a.items + kBlock / 32 - 1) / (kBlock / 32);
    grid = std::max(1, std::min(need, std::max(1, per_sm) * s->sm_count));
  }
  s->last_grid = grid;
  for (int k = 0; k < steps; ++k) {
    a.src = static_cast<const ST*>(s->buf[s->cur]);
    a.dst = static_cast<ST*>(s->buf[s->cur ^ 1]);
    a.step_ctr = s->step_ctr;
    a.step_off = static_cast<uint32_t>(k);
    LBM_CUDA(s, launch_dependent(kernel, dim3(grid), dim3(kBlock), smem, s->stream, a));
    s->cur ^= 1;
  }
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

// Warp-specialised ring with one cell (plain FP32 / FP64) or one pair of cells (16-bit storage)
// per lane (step_ring.cuh).
template <class ST, bool kOpen, int kW, int kC, int kStages, int kMinBlocks>
int launch_ring_t(lbm_solver* s, int steps) {
  {
    using Phys = typename Form<ST>::Phys;
    using T = typename StoreTraits<ST>::T;
    using S = RingShape<ST, kW, kC>;
    StepArgs<ST, Phys> a{};
    a.mask = s->mask_d;
    a.g = s->g;
    a.k = Form<ST>::consts(s->tau, s->fx, s->fy);
    const Eq9<T> e = step_inlet_eq<ST>(s);
    for (int i = 0; i < kQ; ++i) a.eq_in[i] = e.v[i];
    a.sc = s->sc;
    const int tpr = (s->nx + S::TW - 1) / S::TW;
    const int tiles = tpr * s->ny;
    const auto kernel = ring_step_kernel<ST, Phys, kOpen, kW, kC, kStages, kMinBlocks>;
    const size_t smem = ring_smem_bytes<S>(kStages);
    LBM_CUDA(s, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
    int grid = s->grid;
    if (grid <= 0) {
      int per_sm = 0;
      LBM_CUDA(s, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, S::kThreads, smem));
      grid = std::max(1, std::min(tiles, std::max(1, per_sm) * s->sm_count));
    }
    s->last_grid = grid;
    for (int k = 0; k < steps; ++k) {
      a.src = static_cast<const ST*>(s->buf[s->cur]);
      a.dst = static_cast<ST*>(s->buf[s->cur ^ 1]);
      a.step_ctr = s->step_ctr;
      a.step_off = static_cast<uint32_t>(k);
      // Odd steps (by buffer parity) walk the tiles backwards: they start on the rows the
      // previous step wrote last.
      LBM_CUDA(s, launch_dependent(kernel, dim3(grid), dim3(S::kThreads), smem, s->stream, a, tpr, tiles, 0,
                                   s->cur, s->err_flag));
      s->cur ^= 1;
    }
    LBM_CUDA(s, cudaGetLastError());
    return LBM_OK;
  }
}

// Automatic kernel choice (variant < 0), from a sweep of every variant on one GB300 (channel,
// best of 3 runs, MLUPS): plain FP32: 256^2 v19 20.8k (v0 19.8k), 512^2 / 1024x256 v17 51.9k /
// 51.7k (v12 47.4k / 46.2k), 1024^2 v17 83.9k (v12 81.7k), 2048^2 v12 86.2k, 4096^2 v12 90.6k;
// 16-bit storage: 256^2 v19 20.2k (v0 13.5k), 512^2 v19 61.2k, 1024^2 v19 114.5k (v17 108.6k,
// v20 91.1k: its 2048-cell tiles are half empty on 1024-cell rows), 2048^2 v20 157.1k (v17
// 143.0k), 4096^2 v20 168.7k (v17 159.3k). With the one-instruction stochastic conversion
// (fewer instructions per cell) the 16-bit sweep moved on the largest grids (walled channel,
// seeded state, best of 3): 2048^2 v20 170.6k (v17 149.7k), 4096^2 v20 169.5k (v17 169.0k,
// v22 170.3k), 8192^2 v17 175.7k (v20 168.9k), so grids of at least 2^25 cells take v17.
// Rows narrower than 256 cells take the
// direct kernel (0), whose 128-cell chunks leave fewer lanes idle than the rings' wide tiles
// (FP64 on 100 x 2000: the ring 12 reached 1.0k MLUPS with a fifth of its lanes busy); otherwise
// FP64 (FP64-ALU-bound) takes the ring 12 with at least two of its tiles per SM, else 0.
template <class ST>
int auto_variant(const lbm_solver* s) {
  using S = RingShape<ST, 8, 2>;
  const long long cells = static_cast<long long>(s->nx) * s->ny;
  if (s->nx < 256) return 0;
  if (sizeof(ST) == 8) {
    const long long tiles = static_cast<long long>((s->nx + S::TW - 1) / S::TW) * s->ny;
    return tiles < 2LL * s->sm_count ? 0 : 12;
  }
  if (sizeof(ST) == 2) {
    if (cells < (2LL << 20)) return 19;
    if (cells >= (32LL << 20)) return 17;
    return (s->nx >= 2048 && cells >= (4LL << 20)) ? 20 : 17;  // 2048-cell tiles need wide rows
  }
  return cells < (1LL << 17) ? 19 : (cells < (2LL << 20) ? 17 : 12);
}

template <class ST, bool kOpen>
int launch_steps_o(lbm_solver* s, int steps) {
  s->last_variant = s->variant >= 0 ? s->variant : auto_variant<ST>(s);
  switch (s->last_variant) {
    case 1: return launch_steps_t<ST, kOpen, 1>(s, steps);
    case 2: return launch_steps_t<ST, kOpen, 2>(s, steps);
    case 3: return launch_steps_t<ST, kOpen, 3>(s, steps);
    case 4: return launch_tma_t<ST, kOpen, 2>(s, steps);
    case 5: return launch_tma_t<ST, kOpen, 3>(s, steps);
    case 6: return launch_tma_t<ST, kOpen, 4>(s, steps);
    case 7: return launch_tma_t<ST, kOpen, 2, true>(s, steps);
    case 8: return launch_steps_t<ST, kOpen, 0, true>(s, steps);
    case 9: return launch_async_t<ST, kOpen, 2>(s, steps);
    case 10: return launch_async_t<ST, kOpen, 3>(s, steps);
    case 11: return launch_async_t<ST, kOpen, 4>(s, steps);
    case 12: return launch_ring_t<ST, kOpen, 8, 2, 2, 1>(s, steps);
    case 13: return launch_ring_t<ST, kOpen, 8, 2, 3, 1>(s, steps);
    case 14: return launch_ring_t<ST, kOpen, 8, 2, 2, 4>(s, steps);
    case 15: return launch_ring_t<ST, kOpen, 4, 2, 3, 1>(s, steps);
    case 16: return launch_ring_t<ST, kOpen, 4, 2, 3, 7>(s, steps);
    case 17: return launch_ring_t<ST, kOpen, 8, 2, 2, 3>(s, steps);
    case 18: return launch_ring_t<ST, kOpen, 8, 2, 3, 3>(s, steps);
    case 19: return launch_ring_t<ST, kOpen, 8, 1, 4, 3>(s, steps);
    case 20: return launch_ring_t<ST, kOpen, 8, 4, 2, 2>(s, steps);
    case 21: return launch_ring_t<ST, kOpen, 4, 4, 2, 5>(s, steps);
    case 22: return launch_ring_t<ST, kOpen, 8, 4, 3, 2>(s, steps);
    default: return launch_steps_t<ST, kOpen, 0>(s, steps);
  }
}

template <class ST>
int launch_steps(lbm_solver* s, int steps) {
  const int rc = s->open_x ? launch_steps_o<ST, true>(s, steps) : launch_steps_o<ST, false>(s, steps);
  if (rc) return rc;
  LBM_CUDA(s, launch_dependent(counter_add_dep_kernel, dim3(1), dim3(1), 0, s->stream, s->step_ctr,
                               static_cast<uint32_t>(steps)));
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int set_state_t(lbm_solver* s, const void* aos_dev, Eq9<typename StoreTraits<ST>::T> eq) {
  using T = typename StoreTraits<ST>::T;
  const long long n = static_cast<long long>(s->nx) * s->ny;
  const int grid = grid_for_cells(s, n, 256);
  // Both buffers: the step never writes solid cells of an all-solid chunk, so they must hold 0
  // in the buffer it writes too (cudaMemset at creation); the current one gets the state.
  set_state_kernel<ST><<<grid, 256, 0, s->stream>>>(static_cast<ST*>(s->buf[s->cur]), s->mask_d,
                                                    s->g, static_cast<const T*>(aos_dev), eq,
                                                    s->sc);
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int get_state_t(lbm_solver* s, void* aos_dev) {
  using T = typename StoreTraits<ST>::T;
  const long long n = static_cast<long long>(s->nx) * s->ny;
  get_state_kernel<ST><<<grid_for_cells(s, n, 256), 256, 0, s->stream>>>(
      static_cast<const ST*>(s->buf[s->cur]), s->mask_d, s->g, inlet_eq<ST>(s), s->sc,
      static_cast<T*>(aos_dev));
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int moments_t(lbm_solver* s, void* rho, void* ux, void* uy) {
  using A = typename Form<ST>::A;
  using T = typename A::T;
  const long long n = static_cast<long long>(s->nx) * s->ny;
  const T hfx = T(0.5) * T(s->fx), hfy = T(0.5) * T(s->fy);
  moments_kernel<ST, A><<<grid_for_cells(s, n, 256), 256, 0, s->stream>>>(
      static_cast<const ST*>(s->buf[s->cur]), s->mask_d, s->g, inlet_eq<ST>(s), s->sc, hfx, hfy,
      static_cast<T*>(rho), static_cast<T*>(ux), static_cast<T*>(uy));
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int mass_t(lbm_solver* s, const void* state, double* partials, int blocks, double* out) {
  mass_partial_kernel<ST><<<blocks, kReduceThreads, 0, s->stream>>>(
      static_cast<const ST*>(state), s->mask_d, s->g, inlet_eq<ST>(s), s->sc, partials);
  mass_final_kernel<<<1, kReduceThreads, 0, s->stream>>>(partials, blocks,
                                                         static_cast<double>(s->fluid), out);
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int finite_t(lbm_solver* s, int* flag) {
  const long long n = static_cast<long long>(s->nx) * s->ny;
  finite_kernel<ST><<<grid_for_cells(s, n, 256), 256, 0, s->stream>>>(
      static_cast<const ST*>(s->buf[s->cur]), s->mask_d, s->g, s->sc, flag);
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int body_force_t(lbm_solver* s, double* out) {
  const long long n = static_cast<long long>(s->nx) * s->ny;
  const uint32_t* body = s->body_d ? s->body_d : s->mask_d;
  body_force_partial_kernel<ST><<<s->red_blocks, kReduceThreads, 0, s->stream>>>(
      static_cast<const ST*>(s->buf[s->cur]), s->mask_d, body, s->g, s->sc, s->force_red);
  pair_final_kernel<<<1, kReduceThreads, 0, s->stream>>>(s->force_red, s->red_blocks, out);
  (void)n;
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int probe_t(lbm_solver* s, int x, int y, void* out) {
  using T = typename StoreTraits<ST>::T;
  probe_kernel<ST><<<1, 32, 0, s->stream>>>(static_cast<const ST*>(s->buf[s->cur]), s->mask_d,
                                            s->g, inlet_eq<ST>(s), s->sc, x, y,
                                            static_cast<T*>(out));
  LBM_CUDA(s, cudaGetLastError());
  return LBM_OK;
}

// Dispatch on the storage form (one code path per form, no fallback).
#define LBM_DISPATCH(s, fn, ...)                                       \
  switch ((s)->precision) {                                           \
    case LBM_FP32: return fn<float>(__VA_ARGS__);                     \
    case LBM_FP64: return fn<double>(__VA_ARGS__);                    \
    case LBM_FP16_STORE: return fn<__half>(__VA_ARGS__);              \
    case LBM_BF16_STORE: return fn<__nv_bfloat16>(__VA_ARGS__);       \
    default: return set_error(s, LBM_ERR_INVALID_ARG, "bad precision"); \
  }

template <class ST>
int init_eq_t(lbm_solver* s, double rho0, double ux0, double uy0) {
  using T = typename StoreTraits<ST>::T;
  return set_state_t<ST>(s, nullptr, host_equilibrium<T>(T(rho0), T(ux0), T(uy0)));
}

int ensure_stage(lbm_solver* s, size_t bytes) {
  if (s->stage_bytes >= bytes) return LBM_OK;
  if (s->stage) {
    LBM_CUDA(s, cudaStreamSynchronize(s->stream));
    cudaFree(s->stage);
    s->stage = nullptr;
    s->stage_bytes = 0;
  }
  LBM_CUDA(s, cudaMalloc(&s->stage, bytes));
  s->stage_bytes = bytes;
  return LBM_OK;
}

int check(const lbm_solver* s) { return s ? LBM_OK : LBM_ERR_INVALID_ARG; }

// Storage scales: 1 for the plain forms, kStoreScale16 (2^15) on every plane of the 16-bit forms
// (the largest stored magnitude 65504 / 2^15 ~ 2 bounds |g_i| = |f_i - w_i| of any state with
// 0 <= f_i <= 1, and values down to 2^-29 stay normal).
PlaneScales default_scales(int precision) {
  PlaneScales p{};
  const bool s16 = precision == LBM_FP16_STORE || precision == LBM_BF16_STORE;
  for (int i = 0; i < kQ; ++i) {
    p.enc[i] = s16 ? kStoreScale16 : 1.0f;
    p.dec[i] = s16 ? 1.0f / kStoreScale16 : 1.0f;
  }
  return p;
}

}  // namespace

// ----------------------------------------------------------------------------------------------
// Internal helpers shared with the other translation units
// ----------------------------------------------------------------------------------------------
namespace lbm_b200 {

int solver_launch(lbm_solver* s, int steps) { LBM_DISPATCH(s, launch_steps, s, steps); }

void drop_step_graph(lbm_solver* s) {
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  s->graph_cur = -1;
}

// Captures kGraphSteps step launches (and the step-counter update) from the current buffer
// parity into a CUDA graph. kGraphSteps is even, so a replay leaves the parity unchanged. A
// capture that fails turns graphs off for this solver (direct launches give the same results).
int ensure_step_graph(lbm_solver* s) {
  if (s->graph && s->graph_cur == s->cur) return LBM_OK;
  drop_step_graph(s);
  const int cur0 = s->cur;
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGetLastError();
    s->graphs = false;
    return LBM_OK;
  }
  const int rc = solver_launch(s, kGraphSteps);
  const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  s->cur = cur0;
  if (rc || e != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    s->graphs = false;
    return LBM_OK;
  }
  const cudaError_t ei = cudaGraphInstantiate(&s->graph, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    cudaGetLastError();
    s->graph = nullptr;
    s->graphs = false;
    return LBM_OK;
  }
  s->graph_cur = cur0;
  return LBM_OK;
}

// Steps: whole CUDA graphs of kGraphSteps launches for long runs on a non-default stream (no
// per-launch host overhead, which dominates small grids), direct launches for the remainder.
int solver_step_raw(lbm_solver* s, int steps) {
  if (s->graphs && s->stream != nullptr && steps >= kGraphSteps) {
    if (int rc = ensure_step_graph(s)) return rc;
    while (s->graph && steps >= kGraphSteps) {
      LBM_CUDA(s, cudaGraphLaunch(s->graph, s->stream));
      s->kernels += kGraphSteps + 1;  // the graph's step launches and its step-counter update
      steps -= kGraphSteps;
    }
  }
  if (steps <= 0) return LBM_OK;
  const int rc = solver_launch(s, steps);
  if (!rc) s->kernels += steps + 1;
  return rc;
}

int solver_mass_into(lbm_solver* s, const void* state, double* partials, int blocks,
                     double* out) {
  LBM_DISPATCH(s, mass_t, s, state, partials, blocks, out);
}

void pack_mask(const uint8_t* solid, int nx, int ny, int mask_words, std::vector<uint32_t>& out) {
  out.assign(static_cast<size_t>(mask_words) * ny, 0xffffffffu);
  for (int y = 0; y < ny; ++y) {
    uint32_t* row = out.data() + static_cast<size_t>(y) * mask_words;
    const uint8_t* src = solid + static_cast<size_t>(y) * nx;
    auto set = [&](int bit, bool v) {
      if (v)
        row[bit >> 5] |= 1u << (bit & 31);
      else
        row[bit >> 5] &= ~(1u << (bit & 31));
    };
    set(0, src[nx - 1] != 0);
    for (int x = 0; x < nx; ++x) set(x + 1, src[x] != 0);
    set(nx + 1, src[0] != 0);
  }
}

int element_bytes(int precision) {
  switch (precision) {
    case LBM_FP32: return 4;
    case LBM_FP64: return 8;
    case LBM_FP16_STORE:
    case LBM_BF16_STORE: return 2;
    default: return 0;
  }
}

}  // namespace lbm_b200

// ----------------------------------------------------------------------------------------------
// C ABI
// ----------------------------------------------------------------------------------------------
extern "C" {

const char* lbm_version(void) { return "lbm_b200 1.0 (sm_103a)"; }

int lbm_create(int nx, int ny, const uint8_t* solid, double tau, double fx, double fy,
               int precision, lbm_solver** out) {
  if (!out) return LBM_ERR_INVALID_ARG;
  *out = nullptr;
  const int elem = element_bytes(precision);
  if (nx < 1 || ny < 1 || !solid || elem == 0) return LBM_ERR_INVALID_ARG;
  // The reference compares tau in its own precision (solver_v3.cu:169-170).
  const bool tau_ok = precision == LBM_FP64 ? tau > 0.5 : static_cast<float>(tau) > 0.5f;
  if (!tau_ok || !std::isfinite(tau) || !std::isfinite(fx) || !std::isfinite(fy))
    return LBM_ERR_INVALID_ARG;
  if (static_cast<long long>(nx) * ny > (1LL << 31) - 1) return LBM_ERR_INVALID_ARG;

  lbm_solver* s = new (std::nothrow) lbm_solver();
  if (!s) return LBM_ERR_OUT_OF_MEMORY;
  s->nx = nx;
  s->ny = ny;
  s->precision = precision;
  s->elem = elem;
  s->vec = 16 / elem;
  s->host_elem = precision == LBM_FP64 ? 8 : 4;
  s->tau = tau;
  s->fx = fx;
  s->fy = fy;
  s->solid.assign(solid, solid + static_cast<size_t>(nx) * ny);
  for (uint8_t v : s->solid) s->fluid += v ? 0 : 1;
  s->sc = default_scales(precision);

  const int per_line = 128 / elem;
  const int pitch = (nx + per_line - 1) / per_line * per_line;
  s->g.nx = nx;
  s->g.ny = ny;
  s->g.pitch = pitch;
  s->g.mask_words = mask_row_words(nx);
  s->g.plane = static_cast<long long>(pitch) * ny;
  s->g.open_x = 0;

  auto fail = [&](int code) {
    lbm_destroy(s);
    return code;
  };
  cudaError_t e = cudaGetDevice(&s->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA);
  e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA);
  s->own_stream = true;
  e = cudaEventCreate(&s->ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev[1]);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA);

  const size_t state_bytes = static_cast<size_t>(kQ) * s->g.plane * elem + 256;
  for (int b = 0; b < 2; ++b) {
    e = cudaMalloc(&s->buf[b], state_bytes);
    if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA);
    e = cudaMemsetAsync(s->buf[b], 0, state_bytes, s->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA);
  }
  s->state_bytes = state_bytes;
  std::vector<uint32_t> words;
  pack_mask(solid, nx, ny, s->g.mask_words, words);
  e = cudaMalloc(&s->mask_d, words.size() * sizeof(uint32_t));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->mask_d, words.data(), words.size() * sizeof(uint32_t),
                        cudaMemcpyHostToDevice, s->stream);
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA);
  s->red_blocks = 4 * s->sm_count;
  e = cudaMalloc(&s->red, (s->red_blocks + 2) * sizeof(double) + 4 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(s->red, 0, (s->red_blocks + 2) * sizeof(double) + 4 * sizeof(int), s->stream);
  s->err_flag = reinterpret_cast<int*>(s->red + s->red_blocks + 2) + 1;
  s->step_ctr = reinterpret_cast<uint32_t*>(s->red + s->red_blocks + 2) + 2;
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA);
  e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA);
  *out = s;
  return LBM_OK;
}

int lbm_destroy(lbm_solver* s) {
  if (!s) return LBM_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (void* p : s->buf) cudaFree(p);
  cudaFree(s->mask_d);
  lbm_b200::drop_step_graph(s);
  cudaFree(s->red);
  cudaFree(s->body_d);
  cudaFree(s->force_red);
  cudaFree(s->stage);
  for (cudaEvent_t ev : s->ev)
    if (ev) cudaEventDestroy(ev);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return LBM_OK;
}

const char* lbm_last_error(const lbm_solver* s) { return s ? s->err.c_str() : "null solver"; }

int lbm_set_stream(lbm_solver* s, void* stream) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  if (s->own_stream) cudaStreamDestroy(s->stream);
  s->own_stream = false;
  s->stream = static_cast<cudaStream_t>(stream);
  return LBM_OK;
}

int lbm_set_inflow_outflow(lbm_solver* s, double u_in) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  if (s->nx < 3 || !std::isfinite(u_in))
    return set_error(s, LBM_ERR_INVALID_ARG, "open boundaries need nx >= 3 and a finite u_in");
  s->open_x = true;
  s->u_in = u_in;
  s->g.open_x = 1;
  lbm_b200::drop_step_graph(s);
  return LBM_OK;
}

int lbm_init_equilibrium(lbm_solver* s, double rho0, double ux0, double uy0) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  LBM_DISPATCH(s, init_eq_t, s, rho0, ux0, uy0);
}

// Device address of a host buffer that kernels may access directly (pinned or registered host
// memory, e.g. over NVLink-C2C), or null: pageable memory is staged through device memory.
static const void* mapped_view(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int lbm_set_populations(lbm_solver* s, const void* s_host) {
  if (check(s) || !s_host) return set_error(s, LBM_ERR_INVALID_ARG, "null state");
  const size_t bytes = static_cast<size_t>(s->nx) * s->ny * kQ * s->host_elem;
  // One copy into device memory, then the conversion kernel (whose neighbour gathers would be
  // slow over the host link): from pinned host memory with coalesced 16-byte kernel loads
  // (size and address permitting), else with a copy engine.
  if (int rc = ensure_stage(s, bytes)) return rc;
  const void* mapped = mapped_view(s_host);
  if (mapped && bytes % 16 == 0 && reinterpret_cast<uintptr_t>(mapped) % 16 == 0) {
    const long long n16 = static_cast<long long>(bytes / 16);
    copy16_kernel<<<grid_for_cells(s, n16, 256), 256, 0, s->stream>>>(static_cast<const uint4*>(mapped),
                                                                      static_cast<uint4*>(s->stage), n16);
    LBM_CUDA(s, cudaGetLastError());
  } else {
    LBM_CUDA(s, cudaMemcpyAsync(s->stage, s_host, bytes, cudaMemcpyHostToDevice, s->stream));
  }
  const void* src = s->stage;
  int rc;
  switch (s->precision) {
    case LBM_FP32: rc = set_state_t<float>(s, src, Eq9<float>{}); break;
    case LBM_FP64: rc = set_state_t<double>(s, src, Eq9<double>{}); break;
    case LBM_FP16_STORE: rc = set_state_t<__half>(s, src, Eq9<float>{}); break;
    case LBM_BF16_STORE: rc = set_state_t<__nv_bfloat16>(s, src, Eq9<float>{}); break;
    default: rc = LBM_ERR_INVALID_ARG;
  }
  if (rc) return rc;
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));  // the host buffer may be reused on return
  return LBM_OK;
}

int lbm_step(lbm_solver* s, int steps) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  if (steps < 0) return set_error(s, LBM_ERR_INVALID_ARG, "steps must be >= 0");
  if (steps == 0) return LBM_OK;
  return lbm_b200::solver_step_raw(s, steps);
}

// Reads and clears the device error flag of the step kernels (a bounded wait that ran out).
static int check_step_flag(lbm_solver* s) {
  int flag = 0;
  LBM_CUDA(s, cudaMemcpyAsync(&flag, s->err_flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  if (flag) {
    LBM_CUDA(s, cudaMemsetAsync(s->err_flag, 0, sizeof(int), s->stream));
    LBM_CUDA(s, cudaStreamSynchronize(s->stream));
    return set_error(s, LBM_ERR_TIMEOUT, "a step kernel gave up waiting for its shared-memory ring");
  }
  return LBM_OK;
}

int lbm_synchronize(lbm_solver* s) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  return check_step_flag(s);
}

int lbm_run(lbm_solver* s, int steps) {
  if (int rc = lbm_step(s, steps)) return rc;
  return lbm_synchronize(s);
}

int lbm_kernel_launches(const lbm_solver* s, long long* count) {
  if (!s || !count) return LBM_ERR_INVALID_ARG;
  *count = s->kernels;
  return LBM_OK;
}

int lbm_timed_run(lbm_solver* s, int steps, double* seconds) {
  if (check(s) || !seconds) return set_error(s, LBM_ERR_INVALID_ARG, "null argument");
  LBM_CUDA(s, cudaEventRecord(s->ev[0], s->stream));
  if (int rc = lbm_step(s, steps)) return rc;
  LBM_CUDA(s, cudaEventRecord(s->ev[1], s->stream));
  LBM_CUDA(s, cudaEventSynchronize(s->ev[1]));
  float ms = 0.f;
  LBM_CUDA(s, cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]));
  *seconds = static_cast<double>(ms) * 1e-3;
  return check_step_flag(s);
}

int lbm_get_populations(lbm_solver* s, void* s_host) {
  if (check(s) || !s_host) return set_error(s, LBM_ERR_INVALID_ARG, "null output");
  const size_t bytes = static_cast<size_t>(s->nx) * s->ny * kQ * s->host_elem;
  // Pinned host output: the gather kernel writes it in place; else through device memory.
  void* dst = const_cast<void*>(mapped_view(s_host));
  if (!dst) {
    if (int rc = ensure_stage(s, bytes)) return rc;
    dst = s->stage;
  }
  int rc;
  switch (s->precision) {
    case LBM_FP32: rc = get_state_t<float>(s, dst); break;
    case LBM_FP64: rc = get_state_t<double>(s, dst); break;
    case LBM_FP16_STORE: rc = get_state_t<__half>(s, dst); break;
    case LBM_BF16_STORE: rc = get_state_t<__nv_bfloat16>(s, dst); break;
    default: rc = LBM_ERR_INVALID_ARG;
  }
  if (rc) return rc;
  if (dst == s->stage)
    LBM_CUDA(s, cudaMemcpyAsync(s_host, s->stage, bytes, cudaMemcpyDeviceToHost, s->stream));
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_macroscopic(lbm_solver* s, void* rho, void* ux, void* uy) {
  if (check(s) || !rho || !ux || !uy) return set_error(s, LBM_ERR_INVALID_ARG, "null output");
  const size_t n = static_cast<size_t>(s->nx) * s->ny;
  const size_t plane = n * s->host_elem;
  // Pinned host outputs (all three): the moment kernel writes them in place; else through
  // device memory.
  void* mr = const_cast<void*>(mapped_view(rho));
  void* mu = const_cast<void*>(mapped_view(ux));
  void* mv = const_cast<void*>(mapped_view(uy));
  const bool direct = mr && mu && mv;
  char* d = nullptr;
  if (!direct) {
    if (int rc = ensure_stage(s, std::max(3 * plane, n * kQ * s->host_elem))) return rc;
    d = static_cast<char*>(s->stage);
    mr = d;
    mu = d + plane;
    mv = d + 2 * plane;
  }
  int rc;
  switch (s->precision) {
    case LBM_FP32: rc = moments_t<float>(s, mr, mu, mv); break;
    case LBM_FP64: rc = moments_t<double>(s, mr, mu, mv); break;
    case LBM_FP16_STORE: rc = moments_t<__half>(s, mr, mu, mv); break;
    case LBM_BF16_STORE: rc = moments_t<__nv_bfloat16>(s, mr, mu, mv); break;
    default: rc = LBM_ERR_INVALID_ARG;
  }
  if (rc) return rc;
  if (!direct) {
    LBM_CUDA(s, cudaMemcpyAsync(rho, d, plane, cudaMemcpyDeviceToHost, s->stream));
    LBM_CUDA(s, cudaMemcpyAsync(ux, d + plane, plane, cudaMemcpyDeviceToHost, s->stream));
    LBM_CUDA(s, cudaMemcpyAsync(uy, d + 2 * plane, plane, cudaMemcpyDeviceToHost, s->stream));
  }
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_total_mass(lbm_solver* s, double* mass) {
  if (check(s) || !mass) return set_error(s, LBM_ERR_INVALID_ARG, "null output");
  double* out = s->red + s->red_blocks;
  if (int rc = lbm_b200::solver_mass_into(s, s->buf[s->cur], s->red, s->red_blocks, out)) return rc;
  LBM_CUDA(s, cudaMemcpyAsync(mass, out, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_populations_at(lbm_solver* s, int x, int y, void* out9) {
  if (check(s) || !out9) return set_error(s, LBM_ERR_INVALID_ARG, "null output");
  if (x < 0 || x >= s->nx || y < 0 || y >= s->ny)
    return set_error(s, LBM_ERR_INVALID_ARG, "cell outside the grid");
  if (int rc = ensure_stage(s, kQ * 8)) return rc;
  int rc;
  switch (s->precision) {
    case LBM_FP32: rc = probe_t<float>(s, x, y, s->stage); break;
    case LBM_FP64: rc = probe_t<double>(s, x, y, s->stage); break;
    case LBM_FP16_STORE: rc = probe_t<__half>(s, x, y, s->stage); break;
    case LBM_BF16_STORE: rc = probe_t<__nv_bfloat16>(s, x, y, s->stage); break;
    default: rc = LBM_ERR_INVALID_ARG;
  }
  if (rc) return rc;
  LBM_CUDA(s, cudaMemcpyAsync(out9, s->stage, kQ * s->host_elem, cudaMemcpyDeviceToHost, s->stream));
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_set_body(lbm_solver* s, const uint8_t* body) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  if (!body) {
    cudaFree(s->body_d);
    s->body_d = nullptr;
    return LBM_OK;
  }
  const size_t n = static_cast<size_t>(s->nx) * s->ny;
  for (size_t c = 0; c < n; ++c)
    if (body[c] && !s->solid[c]) return set_error(s, LBM_ERR_INVALID_ARG, "body cells must be solid");
  std::vector<uint32_t> words;
  pack_mask(body, s->nx, s->ny, s->g.mask_words, words);
  const size_t bytes = words.size() * sizeof(uint32_t);
  if (!s->body_d) LBM_CUDA(s, cudaMalloc(&s->body_d, bytes));
  LBM_CUDA(s, cudaMemcpyAsync(s->body_d, words.data(), bytes, cudaMemcpyHostToDevice, s->stream));
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_body_force(lbm_solver* s, double* fx, double* fy) {
  if (check(s) || !fx || !fy) return set_error(s, LBM_ERR_INVALID_ARG, "null output");
  if (!s->force_red) LBM_CUDA(s, cudaMalloc(&s->force_red, (2 * s->red_blocks + 2) * sizeof(double)));
  double* out = s->force_red + 2 * s->red_blocks;
  int rc;
  switch (s->precision) {
    case LBM_FP32: rc = body_force_t<float>(s, out); break;
    case LBM_FP64: rc = body_force_t<double>(s, out); break;
    case LBM_FP16_STORE: rc = body_force_t<__half>(s, out); break;
    case LBM_BF16_STORE: rc = body_force_t<__nv_bfloat16>(s, out); break;
    default: rc = LBM_ERR_INVALID_ARG;
  }
  if (rc) return rc;
  double f[2];
  LBM_CUDA(s, cudaMemcpyAsync(f, out, sizeof(f), cudaMemcpyDeviceToHost, s->stream));
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  *fx = f[0];
  *fy = f[1];
  return LBM_OK;
}

int lbm_check_finite(lbm_solver* s, int* finite) {
  if (check(s) || !finite) return set_error(s, LBM_ERR_INVALID_ARG, "null output");
  int* flag = reinterpret_cast<int*>(s->red + s->red_blocks + 2);
  LBM_CUDA(s, cudaMemsetAsync(flag, 0, sizeof(int), s->stream));
  int rc;
  switch (s->precision) {
    case LBM_FP32: rc = finite_t<float>(s, flag); break;
    case LBM_FP64: rc = finite_t<double>(s, flag); break;
    case LBM_FP16_STORE: rc = finite_t<__half>(s, flag); break;
    case LBM_BF16_STORE: rc = finite_t<__nv_bfloat16>(s, flag); break;
    default: rc = LBM_ERR_INVALID_ARG;
  }
  if (rc) return rc;
  int bad = 0;
  LBM_CUDA(s, cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  LBM_CUDA(s, cudaStreamSynchronize(s->stream));
  *finite = bad ? 0 : 1;
  return LBM_OK;
}

int lbm_device_info(lbm_solver* s, char* buf, size_t size) {
  if (check(s) || !buf || size == 0) return set_error(s, LBM_ERR_INVALID_ARG, "null buffer");
  cudaDeviceProp prop{};
  int driver = 0, runtime = 0;
  LBM_CUDA(s, cudaGetDeviceProperties(&prop, s->device));
  LBM_CUDA(s, cudaDriverGetVersion(&driver));
  LBM_CUDA(s, cudaRuntimeGetVersion(&runtime));
  auto ver = [](int v) { return std::to_string(v / 1000) + "." + std::to_string((v % 1000) / 10); };
  static const char* names[] = {"fp32", "fp64", "fp16_store", "bf16_store"};
  const std::string info =
      "\"gpu\": \"" + std::string(prop.name) + "\", \"gpu_driver_cuda\": \"" + ver(driver) +
      "\", \"cuda_runtime\": \"" + ver(runtime) + "\", \"cuda_compiled\": \"" +
      ver(CUDART_VERSION) + "\", \"ecc\": " + std::to_string(prop.ECCEnabled) +
      ", \"sm_count\": " + std::to_string(s->sm_count) + ", \"block\": \"" +
      std::to_string(s->block) + "x1\", \"grid\": " + std::to_string(s->last_grid) +
      ", \"variant\": \"b200_pull_vec" + std::to_string(s->vec) +
      "_v" + std::to_string(s->last_variant) + (s->variant < 0 ? "_auto" : "") + "\", \"precision\": \"" +
      names[s->precision] + "\"";
  std::snprintf(buf, size, "%s", info.c_str());
  return LBM_OK;
}

int lbm_get_shape(const lbm_solver* s, int* nx, int* ny, int* precision) {
  if (!s) return LBM_ERR_INVALID_ARG;
  if (nx) *nx = s->nx;
  if (ny) *ny = s->ny;
  if (precision) *precision = s->precision;
  return LBM_OK;
}

int lbm_set_launch(lbm_solver* s, int block_threads, int grid_blocks) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  if (block_threads <= 0) block_threads = kStepThreads;
  if (block_threads % 32 != 0 || block_threads > kStepThreads || grid_blocks < 0)
    return set_error(s, LBM_ERR_INVALID_ARG, "block must be a multiple of 32 and <= 256");
  s->block = block_threads;
  s->grid = grid_blocks;
  lbm_b200::drop_step_graph(s);
  return LBM_OK;
}

int lbm_set_variant(lbm_solver* s, int variant) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  if (variant < -1 || variant > 22)
    return set_error(s, LBM_ERR_INVALID_ARG, "variant must be in [-1, 22]");
  s->variant = variant;
  lbm_b200::drop_step_graph(s);
  return LBM_OK;
}

int lbm_state_view(lbm_solver* s, void** current, long long* plane_stride, int* row_pitch) {
  if (check(s)) return LBM_ERR_INVALID_ARG;
  if (current) *current = s->buf[s->cur];
  if (plane_stride) *plane_stride = s->g.plane;
  if (row_pitch) *row_pitch = s->g.pitch;
  return LBM_OK;
}

int lbm_test_set_consumer_wait_limit(unsigned polls) {
  const unsigned v = polls == 0 || polls >= lbm_b200::kSpinLimit ? lbm_b200::kSpinLimit : polls;
  const cudaError_t e = cudaMemcpyToSymbol(lbm_b200::c_consumer_wait_limit, &v, sizeof v);
  return e == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}

}  // extern "C"
