// Strip engine: the lattice decomposed into horizontal strips with one ghost row on each side,
// stepped strip by strip with a device halo exchange between the steps. Counterpart of the
// reference's multi-rank solver (src/v4_mpi_cuda: SolverV4 over the StripEngine interface,
// engine.hpp:34-62; decomposition.hpp:19-33), with the ranks' strips held by one GPU and the
// halo packed, moved and unpacked on the device instead of through host buffers and MPI:
//
//   * decomposition as the reference's make_strip: strip k owns ny / S rows, the first ny % S
//     strips one more (at least 2 rows each); its buffers hold local rows 0 .. n_k + 1, row 0 and
//     row n_k + 1 being the ghost copies of global rows y0 - 1 and y0 + n_k (periodic ring);
//   * one step = one launch of the ring step kernel over the owned rows of every strip (rows
//     1 .. n_k, whose y-neighbours are all local; a tile finds its strip from its row by the
//     decomposition's arithmetic), with the halo exchange fused into it: the ghost row below
//     strip k receives the populations moving up (c_y = +1: 2, 5, 6) of the top owned row of the
//     strip below, the ghost row above receives those moving down (c_y = -1: 4, 7, 8) of the
//     bottom owned row of the strip above: 3 * nx values per message, the reference's halo
//     content (engine.hpp:14-20), written by the step kernel as it stores those rows (one
//     device, so a neighbour's ghost row is plain memory); other ghost-row values are never
//     read. A separate halo kernel fills the ghost rows after a state upload;
//   * every cell update is the solver's, so the result is bit-for-bit that of the undivided
//     solver (and of the reference's v0) for any number of strips, and the 16-bit forms draw the
//     same rounding bits (the strip's rows carry their global cell offsets in the hash);
//   * long runs replay CUDA graphs of kStripGraphSteps steps, as the solver does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "aux_kernels.cuh"
#include "fastdiv.h"
#include "forms.cuh"
#include "lbm_b200.h"
#include "solver_internal.h"
#include "step_ring.cuh"

using namespace lbm_b200;

namespace {

constexpr int kStripGraphSteps = 16;  // steps per captured graph (even)
// Halo planes: j = 0..2 -> 2, 5, 6 (c_y = +1, into the ghost row below the next strip up);
// j = 3..5 -> 4, 7, 8 (c_y = -1, into the ghost row above the next strip down).
__host__ __device__ constexpr int halo_plane(int j) {
  return j == 0 ? 2 : j == 1 ? 5 : j == 2 ? 6 : j == 3 ? 4 : j == 4 ? 7 : 8;
}

struct StripView {
  long long off;    // element offset of the strip's planes in a state buffer
  long long plane;  // elements per plane (pitch * (n + 2))
  int n;            // owned rows
};

// A strip as the step kernel sees it: offsets of its planes and mask rows, its rounding-key
// base (cell offset of global row y0 - 1), owned rows,
// and the fused halo's targets (StepArgs::halo): ghost row 0 of the strip above and ghost row
// n + 1 of the strip below, as offsets from this strip's planes, with their plane strides.
struct StripTile {
  long long off, plane, key_base, moff;
  long long halo[4];
  int n;
};
constexpr int kStripTableSmem = 256;  // strip tables up to this size are staged in shared memory

// How the owned rows split into strips (the reference's make_strip): the first `extra` strips own
// base + 1 rows, the others base; a global owned row's strip and local row follow from two
// divisions by invariant divisors.
struct StripSplit {
  int base, extra;
  FastDiv by_long, by_short;  // by base + 1, by base
  __device__ __forceinline__ void locate(int row, int& k, int& local) const {
    const int split = extra * (base + 1);
    if (row < split) {
      k = static_cast<int>(by_long.div(static_cast<uint32_t>(row)));
      local = row - k * (base + 1);
    } else {
      const int q = static_cast<int>(by_short.div(static_cast<uint32_t>(row - split)));
      k = extra + q;
      local = row - split - q * base;
    }
  }
};

// Stage policy of the strips' tiles for the ring pipeline: tpr tiles per row, the owned rows of
// strip 0, then of strip 1, ... (the lattice's rows in order); the grid of a tile is the strip's
// (base arguments with the strip's offsets). The producer decodes each tile once and hands its
// strip, local row and first cell to the consumer warps in 16 bytes after the ring stage
// (written before it arms the stage, read after the wait), so that eight consumer warps do not
// repeat the divisions.
template <class ST, class Phys, bool kOpen, int kC>
struct StripPolicy {
  using S = RingShape<ST, 8, kC>;
  static constexpr bool kFinish = false;
  static constexpr int kStageBytes = S::kStageBytes + 16;
  const StepArgs<ST, Phys>& base;  // src / dst / mask: buffer bases; g: nx, pitch, mask words
  const StripTile* tab;
  const StripSplit& split;
  FastDiv tpr;
  int tiles, reverse;  // reverse: walk the tiles from the last (alternate steps)

  __device__ __forceinline__ StepArgs<ST, Phys> strip_args(int k) const {
    const StripTile& t = tab[k];
    StepArgs<ST, Phys> p = base;
    p.src = base.src + t.off;
    p.dst = base.dst + t.off;
    p.mask = base.mask + t.moff;
    p.g.ny = t.n + 2;
    p.g.plane = t.plane;
    p.key_base = t.key_base;
    p.halo = t.halo;
    return p;
  }

  __device__ __forceinline__ void issue(int tile, unsigned char* stage, uint64_t* full) const {
    if (reverse) tile = tiles - 1 - tile;
    const int row = static_cast<int>(tpr.div(static_cast<uint32_t>(tile)));
    int k, r;
    split.locate(row, k, r);
    const int tx0 = (tile - row * static_cast<int>(tpr.d)) * S::TW;
    *reinterpret_cast<int4*>(stage + S::kStageBytes) = make_int4(k, r + 1, tx0, 0);
    ring_issue_tile<ST, Phys, kOpen, S>(strip_args(k), stage, full, r + 1, tx0);
  }

  __device__ __forceinline__ void consume(int, const unsigned char* stage, int cw, int lane) const {
    const int4 d = *reinterpret_cast<const int4*>(stage + S::kStageBytes);
    ring_consume_tile<ST, Phys, kOpen, S, kC, true>(strip_args(d.x), stage, d.y, d.z, cw, lane);
  }

  __device__ __forceinline__ void finish(int, int) const {}
};

// Shared memory of a strip ring block: 2 stages of the policy, their barriers, then the strip
// table when it is staged.
template <class ST, class Phys, int kC>
__host__ __device__ constexpr size_t strip_ring_smem() {
  return 2 * static_cast<size_t>(StripPolicy<ST, Phys, false, kC>::kStageBytes) + 4 * sizeof(uint64_t);
}

// One step of every strip: the solver's ring kernel (8 consumer warps x kC passes, 2 stages)
// over the strips' tiles, with the halo exchange fused into the stores of each strip's top and
// bottom owned rows (the ghost rows of the destination buffer are complete when it ends).
template <class ST, class Phys, bool kOpen, int kC, int kMinBlocks>
__global__ void __launch_bounds__(32 * 9, kMinBlocks)
    strip_ring_kernel(const StepArgs<ST, Phys> base, const StripTile* __restrict__ tab, int strips,
                      const StripSplit split, FastDiv tpr, int tiles, int reverse, int* err) {
  using Pol = StripPolicy<ST, Phys, kOpen, kC>;
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dependency_wait();
  const StripTile* t = tab;
  if (strips <= kStripTableSmem) {
    StripTile* s_tab = reinterpret_cast<StripTile*>(smem + strip_ring_smem<ST, Phys, kC>());
    for (int k = threadIdx.x; k < strips; k += blockDim.x) s_tab[k] = tab[k];
    __syncthreads();
    t = s_tab;
  }
  const Pol pol{base, t, split, tpr, tiles, reverse};
  tile_pipeline<8, 2, Pol::kStageBytes>(smem, pol, tiles, err);
}

// Device halo exchange of all strips (raw elements E, the storage bits): thread per
// (strip, one of 6 (direction, plane) pairs, column).
template <class E>
__global__ void strip_halo_kernel(E* __restrict__ buf, const StripView* __restrict__ v, int strips,
                                  int nx, int pitch) {
  grid_dependency_wait();
  const long long total = static_cast<long long>(strips) * 6 * nx;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(t % nx);
    const int j = static_cast<int>((t / nx) % 6);
    const int k = static_cast<int>(t / (6LL * nx));
    const StripView me = v[k];
    if (j < 3) {  // ghost row 0 of k <- top owned row of the strip below
      const StripView src = v[k == 0 ? strips - 1 : k - 1];
      const int i = halo_plane(j);
      buf[me.off + i * me.plane + x] = buf[src.off + i * src.plane + static_cast<long long>(src.n) * pitch + x];
    } else {  // ghost row n + 1 of k <- bottom owned row of the strip above
      const StripView src = v[k == strips - 1 ? 0 : k + 1];
      const int i = halo_plane(j);
      buf[me.off + i * me.plane + static_cast<long long>(me.n + 1) * pitch + x] =
          buf[src.off + i * src.plane + static_cast<long long>(pitch) + x];
    }
  }
}

}  // namespace

struct lbm_strips {
  int precision = LBM_FP32, elem = 4, host_elem = 4;
  int nx = 0, ny = 0, strips = 0, pitch = 0, mask_words = 0;
  double tau = 0, fx = 0, fy = 0, u_in = 0;
  bool open_x = false;
  std::vector<uint8_t> solid;
  long long fluid = 0;
  std::vector<int> y0, n;            // first global row and owned rows of each strip
  std::vector<long long> off, moff;  // element / mask-word offsets of each strip
  long long total_elems = 0;
  void* buf[2] = {nullptr, nullptr};
  int cur = 0;
  uint32_t* mask_d = nullptr;
  StripView* views_d = nullptr;
  StripTile* tiles_d = nullptr;  // the step kernel's strip table
  uint32_t* ctr = nullptr;  // [0]: step counter, [1]: error flag of the bounded waits
  void* stage = nullptr;
  size_t stage_bytes = 0;
  PlaneScales sc{};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaGraphExec_t graph = nullptr;
  int graph_cur = -1;
  bool graphs = true;
  int passes = 2;  // ring passes per strip: 4 (2048-cell tiles) for 16-bit storage on rows >= 2048
  int sm_count = 0;
  std::string err;
};

namespace {

int sfail(lbm_strips* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define S_CUDA(h, call)                                                                          \
  do {                                                                                           \
    const cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                                     \
      cudaGetLastError();                                                                        \
      return sfail(h, e_ == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA,    \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    }                                                                                            \
  } while (0)

Grid2D strip_grid(const lbm_strips* h, int k) {
  Grid2D g{};
  g.nx = h->nx;
  g.ny = h->n[k] + 2;
  g.pitch = h->pitch;
  g.mask_words = h->mask_words;
  g.plane = static_cast<long long>(h->pitch) * g.ny;
  g.open_x = h->open_x ? 1 : 0;
  return g;
}

// Global row of local row r of strip k (periodic).
int global_row(const lbm_strips* h, int k, int r) { return (h->y0[k] + r - 1 + h->ny) % h->ny; }

int grid_cells(const lbm_strips* h, long long n) {
  return static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 16LL * h->sm_count)));
}

template <class ST>
Eq9<typename StoreTraits<ST>::T> strip_inlet(const lbm_strips* h, bool scaled) {
  using T = typename StoreTraits<ST>::T;
  Eq9<T> e{};
  if (!h->open_x) return e;
  e = host_equilibrium<T>(T(1), T(h->u_in), T(0));
  if (scaled && sizeof(ST) == 2)
    for (int i = 0; i < kQ; ++i) e.v[i] *= h->sc.enc[i];
  return e;
}

template <class ST>
int halo_t(lbm_strips* h, int b) {
  using E = std::conditional_t<sizeof(ST) == 2, uint16_t, std::conditional_t<sizeof(ST) == 4, uint32_t, uint64_t>>;
  const long long total = static_cast<long long>(h->strips) * 6 * h->nx;
  S_CUDA(h, launch_dependent(strip_halo_kernel<E>, dim3(grid_cells(h, total)), dim3(256), 0, h->stream,
                             static_cast<E*>(h->buf[b]), static_cast<const StripView*>(h->views_d), h->strips,
                             h->nx, h->pitch));
  return LBM_OK;
}

// `steps` steps: one ring launch per step over every strip's owned rows (halo fused); then the
// step counter advances. kC: ring passes per strip (the solver's variant 12 / 17 shape, or
// variant 20's for 16-bit storage on wide rows).
template <class ST, bool kOpen, int kC>
int steps_tc(lbm_strips* h, int steps) {
  using Phys = typename Form<ST>::Phys;
  using T = typename StoreTraits<ST>::T;
  // Register caps: 3 resident blocks (72 registers); 2 for the four-pass shape with open x
  // boundaries (it would spill at 72); none in FP64.
  constexpr int kMin = sizeof(ST) == 8 ? 1 : ((kC == 4 && kOpen) ? 2 : 3);
  using S = RingShape<ST, 8, kC>;
  const auto kernel = strip_ring_kernel<ST, Phys, kOpen, kC, kMin>;
  const size_t smem = strip_ring_smem<ST, Phys, kC>() +
                      (h->strips <= kStripTableSmem ? h->strips * sizeof(StripTile) : 0);
  S_CUDA(h, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  S_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, S::kThreads, smem));
  const int tpr = (h->nx + S::TW - 1) / S::TW;
  const int tiles = tpr * h->ny;  // the strips' owned rows cover the lattice once
  const int grid = std::max(1, std::min(tiles, std::max(1, per_sm) * h->sm_count));
  const Eq9<T> e = strip_inlet<ST>(h, true);
  StepArgs<ST, Phys> a{};
  a.mask = h->mask_d;
  a.g = strip_grid(h, 0);
  a.k = Form<ST>::consts(h->tau, h->fx, h->fy);
  for (int i = 0; i < kQ; ++i) a.eq_in[i] = e.v[i];
  a.sc = h->sc;
  a.step_ctr = h->ctr;
  int* err = reinterpret_cast<int*>(h->ctr + 1);
  StripSplit split{};
  split.base = h->ny / h->strips;
  split.extra = h->ny % h->strips;
  split.by_long = FastDiv(static_cast<uint32_t>(split.base + 1));
  split.by_short = FastDiv(static_cast<uint32_t>(split.base));
  for (int s = 0; s < steps; ++s) {
    a.src = static_cast<const ST*>(h->buf[h->cur]);
    a.dst = static_cast<ST*>(h->buf[h->cur ^ 1]);
    a.step_off = static_cast<uint32_t>(s);
    S_CUDA(h, launch_dependent(kernel, dim3(grid), dim3(S::kThreads), smem, h->stream, a,
                               static_cast<const StripTile*>(h->tiles_d), h->strips, split,
                               FastDiv(static_cast<uint32_t>(tpr)), tiles, h->cur, err));
    h->cur ^= 1;
  }
  counter_add_kernel<<<1, 1, 0, h->stream>>>(h->ctr, static_cast<uint32_t>(steps));
  S_CUDA(h, cudaGetLastError());
  return LBM_OK;
}

template <class ST, bool kOpen>
int steps_t(lbm_strips* h, int steps) {
  if constexpr (sizeof(ST) == 2) {
    if (h->passes == 4) return steps_tc<ST, kOpen, 4>(h, steps);
  }
  return steps_tc<ST, kOpen, 2>(h, steps);
}

template <class ST>
int launch_t(lbm_strips* h, int steps) {
  return h->open_x ? steps_t<ST, true>(h, steps) : steps_t<ST, false>(h, steps);
}

int launch(lbm_strips* h, int steps) {
  switch (h->precision) {
    case LBM_FP32: return launch_t<float>(h, steps);
    case LBM_FP64: return launch_t<double>(h, steps);
    case LBM_FP16_STORE: return launch_t<__half>(h, steps);
    case LBM_BF16_STORE: return launch_t<__nv_bfloat16>(h, steps);
    default: return LBM_ERR_INVALID_ARG;
  }
}

void drop_graph(lbm_strips* h) {
  if (h->graph) cudaGraphExecDestroy(h->graph);
  h->graph = nullptr;
  h->graph_cur = -1;
}

int run_steps(lbm_strips* h, int steps) {
  if (h->graphs && steps >= kStripGraphSteps) {
    if (!h->graph || h->graph_cur != h->cur) {
      drop_graph(h);
      const int cur0 = h->cur;
      cudaGraph_t g = nullptr;
      bool ok = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed) == cudaSuccess;
      const int rc = ok ? launch(h, kStripGraphSteps) : LBM_OK;
      if (ok) ok = cudaStreamEndCapture(h->stream, &g) == cudaSuccess && g && rc == LBM_OK;
      h->cur = cur0;
      if (ok) ok = cudaGraphInstantiate(&h->graph, g, 0) == cudaSuccess;
      if (g) cudaGraphDestroy(g);
      if (!ok) {
        cudaGetLastError();
        h->graph = nullptr;
        h->graphs = false;
      } else {
        h->graph_cur = cur0;
      }
    }
    while (h->graph && steps >= kStripGraphSteps) {
      S_CUDA(h, cudaGraphLaunch(h->graph, h->stream));
      steps -= kStripGraphSteps;
    }
  }
  return steps > 0 ? launch(h, steps) : LBM_OK;
}

int ensure_stage(lbm_strips* h, size_t bytes) {
  if (h->stage_bytes >= bytes) return LBM_OK;
  cudaFree(h->stage);
  h->stage = nullptr;
  h->stage_bytes = 0;
  S_CUDA(h, cudaMalloc(&h->stage, bytes));
  h->stage_bytes = bytes;
  return LBM_OK;
}

// Uploads the state (v0 layout, global) or the uniform equilibrium into the current buffer of
// every strip (the pull preimage, ghost rows included), then exchanges the halos.
template <class ST>
int set_t(lbm_strips* h, const void* s_host, Eq9<typename StoreTraits<ST>::T> eq) {
  using T = typename StoreTraits<ST>::T;
  const int nx = h->nx;
  std::vector<T> local;
  for (int k = 0; k < h->strips; ++k) {
    const Grid2D g = strip_grid(h, k);
    const size_t cells = static_cast<size_t>(nx) * g.ny;
    const T* aos_dev = nullptr;
    if (s_host) {
      local.resize(cells * kQ);
      for (int r = 0; r < g.ny; ++r)
        std::memcpy(local.data() + static_cast<size_t>(r) * nx * kQ,
                    static_cast<const T*>(s_host) + static_cast<size_t>(global_row(h, k, r)) * nx * kQ,
                    static_cast<size_t>(nx) * kQ * sizeof(T));
      if (int rc = ensure_stage(h, cells * kQ * sizeof(T))) return rc;
      S_CUDA(h, cudaMemcpyAsync(h->stage, local.data(), cells * kQ * sizeof(T), cudaMemcpyHostToDevice, h->stream));
      aos_dev = static_cast<const T*>(h->stage);
    }
    set_state_kernel<ST><<<grid_cells(h, static_cast<long long>(cells)), 256, 0, h->stream>>>(
        static_cast<ST*>(h->buf[h->cur]) + h->off[k], h->mask_d + h->moff[k], g, aos_dev, eq, h->sc);
    S_CUDA(h, cudaGetLastError());
    if (s_host) S_CUDA(h, cudaStreamSynchronize(h->stream));  // the staging buffer is reused
  }
  if (int rc = halo_t<ST>(h, h->cur)) return rc;
  S_CUDA(h, cudaStreamSynchronize(h->stream));
  return LBM_OK;
}

// Owned rows of every strip: v0-layout populations (what = 0) or rho/ux/uy (what = 1).
template <class ST>
int get_t(lbm_strips* h, int what, void* out0, void* out1, void* out2) {
  using T = typename StoreTraits<ST>::T;
  using A = typename Form<ST>::A;
  const int nx = h->nx;
  const Eq9<T> eq_in = strip_inlet<ST>(h, false);
  std::vector<T> local;
  for (int k = 0; k < h->strips; ++k) {
    const Grid2D g = strip_grid(h, k);
    const size_t cells = static_cast<size_t>(nx) * g.ny;
    const size_t per_cell = what == 0 ? kQ : 3;
    if (int rc = ensure_stage(h, cells * per_cell * sizeof(T))) return rc;
    T* st = static_cast<T*>(h->stage);
    const ST* R = static_cast<const ST*>(h->buf[h->cur]) + h->off[k];
    const int grid = grid_cells(h, static_cast<long long>(cells));
    if (what == 0) {
      get_state_kernel<ST><<<grid, 256, 0, h->stream>>>(R, h->mask_d + h->moff[k], g, eq_in, h->sc, st);
    } else {
      moments_kernel<ST, A><<<grid, 256, 0, h->stream>>>(R, h->mask_d + h->moff[k], g, eq_in, h->sc,
                                                         T(T(0.5) * T(h->fx)), T(T(0.5) * T(h->fy)), st,
                                                         st + cells, st + 2 * cells);
    }
    S_CUDA(h, cudaGetLastError());
    local.resize(cells * per_cell);
    S_CUDA(h, cudaMemcpyAsync(local.data(), st, cells * per_cell * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
    S_CUDA(h, cudaStreamSynchronize(h->stream));
    const size_t row0 = static_cast<size_t>(h->y0[k]) * nx;
    const size_t owned = static_cast<size_t>(h->n[k]) * nx;
    if (what == 0) {
      std::memcpy(static_cast<T*>(out0) + row0 * kQ, local.data() + static_cast<size_t>(nx) * kQ,
                  owned * kQ * sizeof(T));
    } else {
      void* outs[3] = {out0, out1, out2};
      for (int f = 0; f < 3; ++f)
        std::memcpy(static_cast<T*>(outs[f]) + row0, local.data() + f * cells + nx, owned * sizeof(T));
    }
  }
  return LBM_OK;
}

#define S_DISPATCH(h, fn, ...)                                            \
  switch ((h)->precision) {                                               \
    case LBM_FP32: return fn<float>(__VA_ARGS__);                         \
    case LBM_FP64: return fn<double>(__VA_ARGS__);                        \
    case LBM_FP16_STORE: return fn<__half>(__VA_ARGS__);                  \
    case LBM_BF16_STORE: return fn<__nv_bfloat16>(__VA_ARGS__);           \
    default: return LBM_ERR_INVALID_ARG;                                  \
  }

template <class ST>
int init_eq_t(lbm_strips* h, double rho0, double ux0, double uy0) {
  using T = typename StoreTraits<ST>::T;
  return set_t<ST>(h, nullptr, host_equilibrium<T>(T(rho0), T(ux0), T(uy0)));
}

template <class ST>
int set_pops_t(lbm_strips* h, const void* s_host) {
  return set_t<ST>(h, s_host, Eq9<typename StoreTraits<ST>::T>{});
}

template <class ST>
int get_pops_t(lbm_strips* h, void* s_host) {
  return get_t<ST>(h, 0, s_host, nullptr, nullptr);
}

template <class ST>
int moments_t(lbm_strips* h, void* rho, void* ux, void* uy) {
  return get_t<ST>(h, 1, rho, ux, uy);
}

int check_flag(lbm_strips* h) {
  uint32_t flag = 0;
  S_CUDA(h, cudaMemcpyAsync(&flag, h->ctr + 1, sizeof(flag), cudaMemcpyDeviceToHost, h->stream));
  S_CUDA(h, cudaStreamSynchronize(h->stream));
  if (flag) {
    S_CUDA(h, cudaMemsetAsync(h->ctr + 1, 0, sizeof(flag), h->stream));
    return sfail(h, LBM_ERR_TIMEOUT, "a step kernel gave up waiting for its shared-memory ring");
  }
  return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_strips_create(int nx, int ny, const uint8_t* solid, double tau, double fx, double fy,
                      int precision, int strips, lbm_strips** out) {
  if (!out) return LBM_ERR_INVALID_ARG;
  *out = nullptr;
  const int elem = element_bytes(precision);
  if (nx < 1 || ny < 1 || !solid || !elem || strips < 1 || ny / strips < 2) return LBM_ERR_INVALID_ARG;
  const bool tau_ok = precision == LBM_FP64 ? tau > 0.5 : static_cast<float>(tau) > 0.5f;
  if (!tau_ok) return LBM_ERR_INVALID_ARG;
  lbm_strips* h = new (std::nothrow) lbm_strips();
  if (!h) return LBM_ERR_OUT_OF_MEMORY;
  auto fail = [&](int code) {
    lbm_strips_destroy(h);
    return code;
  };
  h->precision = precision;
  h->elem = elem;
  h->host_elem = precision == LBM_FP64 ? 8 : 4;
  h->nx = nx;
  h->ny = ny;
  h->strips = strips;
  h->tau = tau;
  h->fx = fx;
  h->fy = fy;
  h->solid.assign(solid, solid + static_cast<size_t>(nx) * ny);
  for (uint8_t v : h->solid) h->fluid += v ? 0 : 1;
  const bool s16 = precision == LBM_FP16_STORE || precision == LBM_BF16_STORE;
  for (int i = 0; i < kQ; ++i) {
    h->sc.enc[i] = s16 ? kStoreScale16 : 1.0f;
    h->sc.dec[i] = s16 ? 1.0f / kStoreScale16 : 1.0f;
  }
  const int per_line = 128 / elem;
  h->pitch = (nx + per_line - 1) / per_line * per_line;
  h->mask_words = mask_row_words(nx);
  // Decomposition of the reference's make_strip (decomposition.hpp:19-33).
  const int base = ny / strips, extra = ny % strips;
  std::vector<uint32_t> all_words, words;
  std::vector<uint8_t> local;
  std::vector<StripView> views(strips);
  long long off = 0, moff = 0;
  for (int k = 0; k < strips; ++k) {
    h->n.push_back(base + (k < extra ? 1 : 0));
    h->y0.push_back(k * base + (k < extra ? k : extra));
    const int rows = h->n[k] + 2;
    local.resize(static_cast<size_t>(nx) * rows);
    for (int r = 0; r < rows; ++r)
      std::memcpy(local.data() + static_cast<size_t>(r) * nx,
                  solid + static_cast<size_t>(global_row(h, k, r)) * nx, nx);
    pack_mask(local.data(), nx, rows, h->mask_words, words);
    all_words.insert(all_words.end(), words.begin(), words.end());
    h->off.push_back(off);
    h->moff.push_back(moff);
    views[k] = StripView{off, static_cast<long long>(h->pitch) * rows, h->n[k]};
    off += kQ * static_cast<long long>(h->pitch) * rows;
    moff += static_cast<long long>(h->mask_words) * rows;
  }
  h->total_elems = off;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess ||
      cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev[0]) != cudaSuccess || cudaEventCreate(&h->ev[1]) != cudaSuccess)
    return fail(LBM_ERR_CUDA);
  const size_t bytes = static_cast<size_t>(off) * elem + 256;
  cudaError_t e = cudaSuccess;
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaMalloc(&h->buf[b], bytes);
    if (e == cudaSuccess) e = cudaMemset(h->buf[b], 0, bytes);
  }
  if (e == cudaSuccess) e = cudaMalloc(&h->mask_d, all_words.size() * sizeof(uint32_t));
  if (e == cudaSuccess)
    e = cudaMemcpy(h->mask_d, all_words.data(), all_words.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&h->views_d, strips * sizeof(StripView));
  if (e == cudaSuccess) e = cudaMemcpy(h->views_d, views.data(), strips * sizeof(StripView), cudaMemcpyHostToDevice);
  // The step kernel's strip table (its tiles: the ring shape of 8 consumer warps x 2 passes, 512
  // cells per tile, 1024 with 16-bit storage, or 4 passes for 16-bit storage on rows of at
  // least 2048 cells, over the owned rows, strip after strip).
  {
    h->passes = (elem == 2 && nx >= 2048) ? 4 : 2;
    std::vector<StripTile> tt(strips);
    for (int k = 0; k < strips; ++k) {
      const int up = k == strips - 1 ? 0 : k + 1, dn = k == 0 ? strips - 1 : k - 1;
      StripTile& t = tt[k];
      t.off = h->off[k];
      t.plane = views[k].plane;
      t.key_base = static_cast<long long>(h->y0[k] - 1) * h->pitch;
      t.moff = h->moff[k];
      t.halo[0] = h->off[up] - h->off[k];  // ghost row 0 of the strip above
      t.halo[1] = views[up].plane;
      t.halo[2] = h->off[dn] + static_cast<long long>(h->n[dn] + 1) * h->pitch - h->off[k];  // row n + 1 below
      t.halo[3] = views[dn].plane;
      t.n = h->n[k];
    }
    if (e == cudaSuccess) e = cudaMalloc(&h->tiles_d, strips * sizeof(StripTile));
    if (e == cudaSuccess) e = cudaMemcpy(h->tiles_d, tt.data(), strips * sizeof(StripTile), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMalloc(&h->ctr, 4 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(h->ctr, 0, 4 * sizeof(uint32_t));
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA);
  *out = h;
  return LBM_OK;
}

int lbm_strips_destroy(lbm_strips* h) {
  if (!h) return LBM_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graph(h);
  for (void* p : {h->buf[0], h->buf[1], static_cast<void*>(h->mask_d), static_cast<void*>(h->views_d),
                  static_cast<void*>(h->tiles_d), static_cast<void*>(h->ctr), h->stage})
    cudaFree(p);
  for (cudaEvent_t ev : h->ev)
    if (ev) cudaEventDestroy(ev);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return LBM_OK;
}

const char* lbm_strips_last_error(const lbm_strips* h) { return h ? h->err.c_str() : "null"; }

int lbm_strips_layout(const lbm_strips* h, int* first_row, int* rows) {
  if (!h || !first_row || !rows) return LBM_ERR_INVALID_ARG;
  for (int k = 0; k < h->strips; ++k) {
    first_row[k] = h->y0[k];
    rows[k] = h->n[k];
  }
  return LBM_OK;
}

int lbm_strips_set_inflow_outflow(lbm_strips* h, double u_in) {
  if (!h) return LBM_ERR_INVALID_ARG;
  if (h->nx < 3 || !std::isfinite(u_in))
    return sfail(h, LBM_ERR_INVALID_ARG, "open boundaries need nx >= 3 and a finite u_in");
  h->open_x = true;
  h->u_in = u_in;
  drop_graph(h);
  return LBM_OK;
}

int lbm_strips_init_equilibrium(lbm_strips* h, double rho0, double ux0, double uy0) {
  if (!h) return LBM_ERR_INVALID_ARG;
  S_DISPATCH(h, init_eq_t, h, rho0, ux0, uy0);
}

int lbm_strips_set_populations(lbm_strips* h, const void* s_host) {
  if (!h || !s_host) return LBM_ERR_INVALID_ARG;
  S_DISPATCH(h, set_pops_t, h, s_host);
}

int lbm_strips_get_populations(lbm_strips* h, void* s_host) {
  if (!h || !s_host) return LBM_ERR_INVALID_ARG;
  S_DISPATCH(h, get_pops_t, h, s_host);
}

int lbm_strips_macroscopic(lbm_strips* h, void* rho, void* ux, void* uy) {
  if (!h || !rho || !ux || !uy) return LBM_ERR_INVALID_ARG;
  S_DISPATCH(h, moments_t, h, rho, ux, uy);
}

int lbm_strips_step(lbm_strips* h, int steps) {
  if (!h || steps < 0) return LBM_ERR_INVALID_ARG;
  if (int rc = run_steps(h, steps)) return rc;
  return check_flag(h);
}

int lbm_strips_timed_run(lbm_strips* h, int steps, double* seconds) {
  if (!h || !seconds || steps < 0) return LBM_ERR_INVALID_ARG;
  S_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
  if (int rc = run_steps(h, steps)) return rc;
  S_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
  S_CUDA(h, cudaEventSynchronize(h->ev[1]));
  float ms = 0.f;
  S_CUDA(h, cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
  *seconds = static_cast<double>(ms) * 1e-3;
  return check_flag(h);
}

}  // extern "C"
