// Batched ensemble: many independent channels of uneven sizes stepped by one persistent launch.
//
// All instances live in one allocation per state buffer (each instance's 9 planes at a
// 128-byte-aligned offset) and one mask allocation. A device table describes every instance
// (offsets, geometry, collision constants, first global chunk index). The step kernel's warps
// walk the global chunk list (chunks of 32 * G cells of one row of one instance), find their
// instance by binary search over the first-chunk indices staged in shared memory, and run the
// same chunk code as the single-grid kernel (step_kernel.cuh). The default kernel is instead the
// warp-specialised ring of the single-grid solver (step_ring.cuh) over the ensemble's tiles of
// consecutive row strips (a tile may cover several short rows): a tile's instance and place come
// from a per-tile header built on the host (TileHead). Steps are replayed from a CUDA graph of
// kGraphSteps launches. lbm_batch_run_separate() runs the same instances one launch per
// instance per step (the comparison point). lbm_batch_autotune() times the candidate launch
// shapes (cells per thread G, i.e. the chunk width 32 G, threads per block, blocks per SM) on the
// actual ensemble and keeps the fastest, caching the choice per GPU, form and ensemble size.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include "aux_kernels.cuh"
#include "lbm_b200.h"
#include "solver_internal.h"
#include "forms.cuh"
#include "fastdiv.h"
#include "step_kernel.cuh"
#include "step_ring.cuh"

using namespace lbm_b200;

namespace {

constexpr int kBatchThreads = 256;
constexpr int kBatchMaxInstances = 4096;  // first-chunk indices staged in shared memory
constexpr int kGraphSteps = 64;

// One instance of the table (16-byte aligned and sized: the ring kernel's producer copies a tile's
// entry into the tile's stage).
template <class Consts>
struct alignas(16) BatchInst {
  long long off;       // element offset of the instance's planes in a state buffer
  long long mask_off;  // word offset of its mask rows
  Grid2D g;
  int cpr;     // chunks per row for the launch's G
  int item0;   // first global chunk index
  int spr;     // ring strips per row (strips of the tile shape's strip width)
  FastDiv spr_div;
  int rpt;     // ring tiles of whole rows: rows per tile (0: tiles of consecutive strips)
  int tile0;   // first global ring tile index
  Consts k;
};

// The step arguments of one instance for one buffer parity (source buffer 0 or 1), built on the
// host with the table; 16-byte aligned and sized so that the ring kernel's producer can copy a
// tile's entry into the tile's stage.
template <class ST, class Phys>
struct alignas(16) StagedArgs {
  StepArgs<ST, Phys> p;
};

// The copy plan of the ring tiles, built on the host for the current tile shape (build_plan):
// the producer warps read where a tile lies and which bulk copies fill its stage instead of
// deriving them, so that their instructions, which compete with the consumers' for issue
// slots, stay few.
//
// Per tile (TilePlan):
//   inst_nseg  instance index | (row segments of a strip tile << 16) (0 segments: whole rows);
//   ya         the tile's first row;
//   a, b       whole-row tiles: rows in the tile, 0; strip tiles: first strip and one past the
//              last (strips numbered row by row within the instance);
//   first, ncopy, bytes  its copies in the copy array and their total size.
// Per copy (CopyOp, 8 bytes): source offset in 16-byte units from the state buffer being read,
// or from the mask buffer (bit 15 of len16), destination offset and length in 16-byte units
// within the stage.
struct alignas(16) TilePlan {
  int inst_nseg, ya, a, b;
  int first, ncopy, bytes, pad;
};
struct CopyOp {
  uint32_t src16;
  uint16_t dst16;
  uint16_t len16;
};
static_assert(sizeof(CopyOp) == 8, "copy descriptors are 8 bytes");
constexpr uint16_t kCopyFromMask = 0x8000u;

template <class ST, class Phys>
struct BatchArgs {
  const ST* src;
  ST* dst;
  const uint32_t* mask;
  const BatchInst<typename Phys::Consts>* inst;
  int count;
  int items;
  PlaneScales sc;
  const uint32_t* step;  // lattice steps taken (device counter; stochastic-rounding key)
  const StagedArgs<ST, Phys>* args;  // [instance][parity]
  int parity;                        // src == buffer `parity`; odd parity walks the tiles backwards
  int tiles;                         // ring tiles of the ensemble
  const TilePlan* plans;             // [tiles]
  const CopyOp* ops;                 // the tiles' copies
};

// Device step counter of a batch: read by every step launch, advanced by one after it (inside a
// captured graph as well, so every replay of the graph rounds with fresh keys). Behind a ring
// step it is a dependent launch (it waits for the step to complete), as is the next step.
__global__ void step_counter_add(uint32_t* c) {
  grid_dependency_wait();
  *c += 1u;
}
__global__ void step_counter_set(uint32_t* c, uint32_t v) { *c = v; }

template <class ST, class Phys, int G>
__global__ void __launch_bounds__(kBatchThreads)
    batch_step_kernel(const BatchArgs<ST, Phys> a) {
  using T = typename StoreTraits<ST>::T;
  __shared__ int s_item0[kBatchMaxInstances];
  for (int k = threadIdx.x; k < a.count; k += blockDim.x) s_item0[k] = a.inst[k].item0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; item < a.items; item += nwarps) {
    int lo = 0, hi = a.count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_item0[mid] <= item)
        lo = mid;
      else
        hi = mid - 1;
    }
    const BatchInst<typename Phys::Consts>& d = a.inst[lo];
    StepArgs<ST, Phys> p;
    p.src = a.src + d.off;
    p.dst = a.dst + d.off;
    p.mask = a.mask + d.mask_off;
    p.g = d.g;
    p.cpr = d.cpr;
    p.items = d.cpr * d.g.ny;
    p.k = d.k;
    p.sc = a.sc;
    p.step_ctr = a.step;
    p.step_off = 0;
    p.key_base = d.off / kQ;
    const Chunk c = chunk_at<G>(item - d.item0, d.cpr, d.g.nx, d.g.ny, lane);
    T v[kQ][G];
    load_planes<ST, Phys, G>(p, c, v);
    process_chunk<ST, Phys, false, G>(p, c, v, lane);
  }
}

// Ring tiles of the ensemble. An instance's rows are cut into strips of SW = 32 kC LC cells (one
// consumer warp's share of a tile, LC = 2 for the 16-bit pairs); its strips are numbered row by
// row. An instance whose rows fit in a tile (at most kW strips per row) is cut into tiles of
// whole rows (kW / spr rows each): 9 plane copies (a second one where the rows wrap past the
// last row) and one per mask row, whatever the row count, at the price of idle lanes and warps.
// A wider instance is cut into tiles of kW consecutive strips, which straddle two rows (18 copies
// per row segment). The producer's copy issue is what limits the ensemble, so fewer copies beat
// fuller lanes: whole-row tiles for every row that fits raised the 256-channel benchmark
// ensemble (row widths 65..1020) from 99.8k to 106.3k MLUPS with 16-bit storage (8 x 2 shape),
// against whole-row tiles only for rows of at most half a tile.
//
// Stage layout: the tile's rows are segments g = 0 .. nseg - 1 (nseg <= kW). Plane i holds, for
// each segment, its cells plus a 16-byte halo on each side, segments one after the other: the
// strip of consumer warp w, in segment g, starts at element w SW + (2 g + 1) H of the plane's
// SROW elements. Per segment the stage also holds the 3 mask rows around it (MW words each, from
// the 16-byte-aligned word below the segment's first cell) and its 6 wrap blocks.
template <class ST, int kW, int kC>
struct FlatShape {
  using R = RingShape<ST, kW, kC>;
  static constexpr int H = R::H, LC = R::LC, SW = R::SW, WPS = R::WPS, TW = R::TW;
  static constexpr int SROW = TW + 2 * H * kW;
  static constexpr int MW = TW / 32 + 4;
  static constexpr int kPlaneBytes = kQ * SROW * static_cast<int>(sizeof(ST));
  static constexpr int kMaskBytes = kW * 3 * MW * 4;
  static constexpr int kWrapBytes = kW * 6 * 16;
  static constexpr int kStageBytes = kPlaneBytes + kMaskBytes + kWrapBytes;
  // Producer warps of a ring block: two for FP32 and the 16-bit forms, whose many short copies
  // per tile make one producer the limit on uneven ensembles (measured on the 256-channel
  // benchmark ensemble: FP32 59.0k -> 65.6k MLUPS at the same launch; FP16 106.5k -> 113.2k
  // autotuned, at fewer resident blocks so that the collision keeps its registers); one for
  // FP64 (FP64-ALU-bound).
  static constexpr int kProd = sizeof(ST) <= 4 ? 2 : 1;
  static constexpr int kThreads = 32 * (kW + kProd);
  static_assert(SW % 32 == 0 && (SROW * static_cast<int>(sizeof(ST))) % 16 == 0 && kStageBytes % 16 == 0,
                "stage parts must stay 16-byte aligned");
};

// Segment g of a tile whose strips are s0 .. s1 - 1 (row ya = s0 / spr first): its row and its
// first and last strip in that row.
struct Segment {
  int y, j_lo, j_hi, w_first;
};
inline Segment tile_segment(int g, int s0, int s1, int ya, int spr) {
  Segment sg;
  sg.y = ya + g;
  const int row_s = sg.y * spr;
  sg.j_lo = s0 > row_s ? s0 - row_s : 0;
  sg.j_hi = (s1 - 1 < row_s + spr - 1 ? s1 - 1 : row_s + spr - 1) - row_s;
  sg.w_first = row_s + sg.j_lo - s0;
  return sg;
}

// Where consumer warp w's strip lies: its row (and the rows above and below), first cell, first
// stage element, first staged mask word, offsets of its 3 staged mask rows (words) and of its
// wrap blocks (elements), flags (kStripValid: the warp has a strip; kStripRows: the stage holds
// whole rows, periodic neighbours come from the row itself).
constexpr int kStripValid = 1, kStripRows = 2;
struct alignas(16) StripDesc {
  int y, ym, yp, x0, lx0, w0, sm_off, wr_off, flags;
};

// Stage of the batch ring: the tile's rows, masks and wrap blocks (FlatShape), then the step
// arguments of the tile's instance (copied by the producer with the rest) and the kW strip
// descriptors (written by the producer's lanes before it arms the barrier), so that the
// consumers neither search the table, nor hold the instance's constants in registers, nor repeat
// the strip arithmetic in every warp.
template <class ST, class Phys, int kW, int kC>
struct BatchFlatPolicy {
  using S = FlatShape<ST, kW, kC>;
  using Inst = BatchInst<typename Phys::Consts>;
  static constexpr bool kFinish = false;
  static constexpr bool kWarpIssue = true;
  static constexpr int kArgsBytes = static_cast<int>(sizeof(StagedArgs<ST, Phys>));
  static constexpr int kDescOff = S::kStageBytes + kArgsBytes;
  static constexpr int kStageBytes = kDescOff + kW * static_cast<int>(sizeof(StripDesc));
  static_assert(kArgsBytes % 16 == 0, "step arguments are copied in 16-byte units");
  const BatchArgs<ST, Phys>& a;
  // The step's stochastic-rounding key (16-bit storage), read from the step counter once per
  // launch instead of once per strip pass (a global load on the consumers' path: +3 % on the
  // 256-channel benchmark ensemble in FP16). The single-grid ring keeps the load per pass, which
  // there measured 2 to 3 % faster than one per tile or one per launch.
  uint32_t rkey;

  // Producer (all 32 lanes): the lanes describe the consumer warps' strips, lane 0 copies the
  // step arguments, the lanes issue the tile's planned copies between them, and lane 0 then
  // arrives on the stage's barrier with their byte count. A copy may land before that arrive:
  // its complete-tx takes the barrier's transaction count below zero, which the barrier allows,
  // and the phase cannot complete before the arrive (one expected arrival).
  __device__ __forceinline__ void issue(int tile, unsigned char* base, uint64_t* full, int lane) const {
    // Odd steps walk the tiles from the last: they start on the rows the previous step wrote
    // last, still in L2 (the consumers only read what the producer staged).
    if (a.parity) tile = a.tiles - 1 - tile;
    const TilePlan h = a.plans[tile];
    const int k = h.inst_nseg & 0xffff;
    const Inst& d = a.inst[k];
    const int ny = d.g.ny;
    StripDesc sd;
    if (d.rpt) {
      const int ya = h.ya, rn = h.a;
      const int r = static_cast<int>(d.spr_div.div(static_cast<uint32_t>(lane)));
      const int j = lane - r * d.spr;
      sd.flags = (r < rn ? kStripValid : 0) | kStripRows;
      sd.y = r < rn ? ya + r : ya;
      sd.x0 = j * S::SW;
      sd.lx0 = r * d.g.pitch + sd.x0;
      sd.w0 = sd.x0 >> 5;
      sd.sm_off = r * S::MW;
      sd.wr_off = 0;
    } else {
      // Lane w describes consumer warp w's strip.
      const int s0 = h.a, s1 = h.b, ya = h.ya;
      const int st = s0 + lane;
      const bool valid = st < s1;
      sd.flags = valid ? kStripValid : 0;
      sd.y = static_cast<int>(d.spr_div.div(static_cast<uint32_t>(valid ? st : s0)));
      const int j = (valid ? st : s0) - sd.y * d.spr;
      const int g = sd.y - ya;
      const int j_lo = g == 0 ? s0 - ya * d.spr : 0;
      sd.x0 = j * S::SW;
      sd.lx0 = lane * S::SW + (2 * g + 1) * S::H;
      sd.w0 = (sd.x0 >> 5) - (((j_lo * S::SW) >> 5) & ~3);
      sd.sm_off = g * 3 * S::MW;
      sd.wr_off = g * 6 * S::H;
    }
    if (lane < kW) {
      // Ordered before lane 0's arrive by __syncwarp; the consumers acquire it with the phase.
      sd.ym = sd.y == 0 ? ny - 1 : sd.y - 1;
      sd.yp = sd.y == ny - 1 ? 0 : sd.y + 1;
      reinterpret_cast<StripDesc*>(base + kDescOff)[lane] = sd;
    }
    __syncwarp();
    if (lane == 0) bulk_copy_g2s(base + S::kStageBytes, a.args + 2 * k + a.parity, kArgsBytes, full);
    const CopyOp* ops = a.ops + h.first;
    for (int c = lane; c < h.ncopy; c += 32) {
      const CopyOp op = ops[c];
      const unsigned char* src = (op.len16 & kCopyFromMask) ? reinterpret_cast<const unsigned char*>(a.mask)
                                                             : reinterpret_cast<const unsigned char*>(a.src);
      bulk_copy_g2s(base + 16u * op.dst16, src + 16ull * op.src16, 16u * (op.len16 & ~kCopyFromMask), full);
    }
    if (lane == 0) mbar_arrive_expect_tx(full, static_cast<uint32_t>(h.bytes) + kArgsBytes);
  }

  template <bool kRows>
  __device__ __forceinline__ void strip(const StepArgs<ST, Phys>& p, const StripDesc& sd, const unsigned char* base,
                                        int lane) const {
    const ST* st = reinterpret_cast<const ST*>(base);
    const uint32_t* sm = reinterpret_cast<const uint32_t*>(base + S::kPlaneBytes) + sd.sm_off;
    const ST* wr = reinterpret_cast<const ST*>(base + S::kPlaneBytes + S::kMaskBytes) + sd.wr_off;
    uint32_t mine = 0;
    if (lane < 3 * (S::WPS + 1)) mine = sm[(lane / (S::WPS + 1)) * S::MW + sd.w0 + lane % (S::WPS + 1)];
    const bool solids = __any_sync(0xffffffffu, mine != 0u);
#pragma unroll 1
    for (int c = 0; c < kC; ++c) {
      const int x = sd.x0 + 32 * S::LC * c + S::LC * lane;
      if (x < p.g.nx) {
        const int lx = sd.lx0 + 32 * S::LC * c + S::LC * lane;
        if constexpr (S::LC == 2)
          ring_pair<ST, false, S, kRows>(p, st, sm, wr, sd.y, x, lx, sd.w0 + 2 * c, lane, solids, rkey);
        else
          ring_cell<ST, typename Phys::Arith, false, S, kRows>(p, st, sm, wr, sd.y, sd.ym, sd.yp, x, lx,
                                                               sd.w0 + c, lane, solids);
      }
    }
  }

  __device__ __forceinline__ void consume(int, const unsigned char* base, int cw, int lane) const {
    const StripDesc sd = reinterpret_cast<const StripDesc*>(base + kDescOff)[cw];
    if (!(sd.flags & kStripValid)) return;
    const StagedArgs<ST, Phys>* sa = reinterpret_cast<const StagedArgs<ST, Phys>*>(base + S::kStageBytes);
    if constexpr (std::is_same_v<ST, float>) {
      // FP32: the step arguments as a local copy, which lets the compiler keep the fields the
      // collision uses in registers across the strip instead of reading them from the stage at
      // every use (+1.8 % on the benchmark ensemble; the 16-bit collision has no registers to
      // spare and lost 10 % with it).
      const StepArgs<ST, Phys> p = sa->p;
      if (sd.flags & kStripRows)
        strip<true>(p, sd, base, lane);
      else
        strip<false>(p, sd, base, lane);
    } else {
      if (sd.flags & kStripRows)
        strip<true>(sa->p, sd, base, lane);
      else
        strip<false>(sa->p, sd, base, lane);
    }
  }

  __device__ __forceinline__ void finish(int, int) const {}
};

// Shared memory of a batch ring block: the stages and the ring's barriers.
template <class Pol>
__host__ __device__ constexpr size_t batch_ring_smem(int stages) {
  return static_cast<size_t>(stages) * Pol::kStageBytes + 2 * stages * sizeof(uint64_t);
}

// Resident blocks per SM the register budget of a ring shape is capped for (blocks of kW
// consumer and two producer warps): 24 to 32 warps per SM for the FP32 collision (4 blocks of
// the 4x2 shape, which its 4-stage ring's shared memory allows anyway, leave it the registers
// to hold the step arguments), 20 to 28 warps at 73 to 80 registers for the 16-bit one (which
// spills under 72), none for FP64 (FP64-ALU-bound: its kernels are compiled without a register
// cap).
__host__ __device__ constexpr int batch_ring_blocks(int elem, int kW) {
  return elem == 8 ? 1 : elem == 2 ? (kW == 8 ? 2 : (kW == 4 ? 4 : 7)) : (kW == 8 ? 3 : (kW == 4 ? 4 : 8));
}
// Most resident blocks per SM the autotuner tries for a ring shape: the register cap above,
// and for FP64 what its uncapped registers let reside (blocks of kW consumer warps and one
// producer, 82 to 90 registers: 2 / 4 / 6 blocks of 8 / 4 / 2 consumer warps; checked against
// ptxas by tests/test_register_budget.py).
__host__ __device__ constexpr int batch_ring_tune_blocks(int elem, int kW) {
  return elem == 8 ? (kW == 8 ? 2 : (kW == 4 ? 4 : 6)) : batch_ring_blocks(elem, kW);
}
template <class ST, int kW>
constexpr int batch_ring_min_blocks() {
  return batch_ring_blocks(static_cast<int>(sizeof(ST)), kW);
}

template <class ST, class Phys, int kW, int kC, int kStages>
__global__ void __launch_bounds__(FlatShape<ST, kW, kC>::kThreads, (batch_ring_min_blocks<ST, kW>()))
    batch_ring_kernel(const BatchArgs<ST, Phys> a, int tiles, int* err) {
  using Pol = BatchFlatPolicy<ST, Phys, kW, kC>;
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dependency_wait();
  Pol pol{a, sizeof(ST) == 2 ? sr_step_key(__ldg(a.step)) : 0u};
  tile_pipeline<kW, kStages, Pol::kStageBytes, FlatShape<ST, kW, kC>::kProd>(smem, pol, tiles, err);
}

template <class ST>
struct BForm;
template <>
struct BForm<float> {
  using Phys = ExactPhys<ExactF32>;
  static Phys::Consts consts(double tau, double fx, double fy) {
    return make_collide_consts<float>(float(tau), float(fx), float(fy));
  }
};
template <>
struct BForm<double> {
  using Phys = ExactPhys<ExactF64>;
  static Phys::Consts consts(double tau, double fx, double fy) {
    return make_collide_consts<double>(tau, fx, fy);
  }
};
template <>
struct BForm<__half> {
  using Phys = FastPhys;
  static Phys::Consts consts(double tau, double fx, double fy) {
    return make_fast_consts(float(tau), float(fx), float(fy), kStoreScale16);
  }
};
template <>
struct BForm<__nv_bfloat16> {
  using Phys = FastPhys;
  static Phys::Consts consts(double tau, double fx, double fy) {
    return make_fast_consts(float(tau), float(fx), float(fy), kStoreScale16);
  }
};

}  // namespace

struct lbm_batch {
  int precision = LBM_FP32, elem = 4, vec = 4, host_elem = 4, count = 0;
  struct Inst {
    int nx, ny;
    double tau, fx, fy;
    long long off, mask_off, fluid;
    Grid2D g;
  };
  std::vector<Inst> inst;
  long long total_elems = 0, total_cells = 0;
  void* buf[2] = {nullptr, nullptr};
  int cur = 0;
  uint32_t* mask_d = nullptr;
  void* table_d = nullptr;  // BatchInst<Consts>[count] for the current G
  void* args_d = nullptr;   // StagedArgs[count][2] (step arguments per instance and parity)
  void* plans_d = nullptr;  // TilePlan[plans_cap]: the ring tiles of the current tile shape
  void* ops_d = nullptr;    // CopyOp[ops_cap]: their copies
  long long plans_cap = 0, ops_cap = 0;
  int plan_sw = 0, plan_kw = 0, plan_kc = 0;  // tile shape of the current plan
  long long mask_words_total = 0;
  int table_G = 0;
  void* stage = nullptr;
  size_t stage_bytes = 0;
  double* red = nullptr;
  int red_blocks = 0;
  PlaneScales sc{};
  // launch configuration (autotuned)
  // G: cells per thread of the chunk kernel (V or V / 2), or 1 (also 0, the default) for the
  // ring kernel; tiles: the ring kernel's tile count
  int G = 0, block = kBatchThreads, grid = 0, items = 0, tiles = 0, grid_eff = 1;
  int ring_w = 8, ring_c = 2, ring_s = 2;  // ring tile shape: consumer warps, passes; stages
  int table_sw = 0, table_kw = 0;  // ring strip width and strips per tile of the table's tiles
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaGraphExec_t graph = nullptr;
  int graph_cur = -1;  // buffer parity the graph was captured from
  uint32_t t = 0;             // lattice steps taken (host copy of *step_d)
  uint32_t* step_d = nullptr;  // device: [0] step counter, [1] error flag of the bounded waits
  int sm_count = 0, device = 0;
  std::string err, tune_report;
};

namespace {

int bfail(lbm_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

#define B_CUDA(b, call)                                                                          \
  do {                                                                                           \
    const cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                                     \
      cudaGetLastError();                                                                        \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA,    \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    }                                                                                            \
  } while (0)

void drop_graph(lbm_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_cur = -1;
}

// Builds the device instance table for cells-per-thread G.
template <class ST>
int build_table(lbm_batch* b, int G) {
  using Consts = typename BForm<ST>::Phys::Consts;
  std::vector<BatchInst<Consts>> tab(b->count);
  int item = 0, tile = 0;
  for (int k = 0; k < b->count; ++k) {
    const auto& in = b->inst[k];
    BatchInst<Consts>& d = tab[k];
    d.off = in.off;
    d.mask_off = in.mask_off;
    d.g = in.g;
    d.cpr = (in.nx + 32 * G - 1) / (32 * G);
    d.item0 = item;
    d.spr = (in.nx + b->table_sw - 1) / b->table_sw;
    d.spr_div = FastDiv(static_cast<uint32_t>(d.spr));
    // Whole-row tiles for instances whose rows fit in a tile (few copies per tile); tiles of
    // consecutive strips otherwise.
    d.rpt = d.spr <= b->table_kw ? b->table_kw / d.spr : 0;
    d.tile0 = tile;
    d.k = BForm<ST>::consts(in.tau, in.fx, in.fy);
    item += d.cpr * in.ny;
    tile += d.rpt ? (in.ny + d.rpt - 1) / d.rpt
                  : static_cast<int>((static_cast<long long>(d.spr) * in.ny + b->table_kw - 1) / b->table_kw);
  }
  b->tiles = tile;
  using Phys = typename BForm<ST>::Phys;
  std::vector<StagedArgs<ST, Phys>> args(2 * static_cast<size_t>(b->count));
  for (int k = 0; k < b->count; ++k) {
    for (int par = 0; par < 2; ++par) {
      StepArgs<ST, Phys>& p = args[2 * k + par].p;
      p = StepArgs<ST, Phys>{};
      p.src = static_cast<const ST*>(b->buf[par]) + tab[k].off;
      p.dst = static_cast<ST*>(b->buf[par ^ 1]) + tab[k].off;
      p.mask = b->mask_d + tab[k].mask_off;
      p.g = tab[k].g;
      p.k = tab[k].k;
      p.sc = b->sc;
      p.step_ctr = b->step_d;
      p.step_off = 0;
      p.key_base = tab[k].off / kQ;
    }
  }
  if (!b->args_d) B_CUDA(b, cudaMalloc(&b->args_d, args.size() * sizeof(args[0])));
  B_CUDA(b, cudaMemcpy(b->args_d, args.data(), args.size() * sizeof(args[0]), cudaMemcpyHostToDevice));
  if (!b->table_d) B_CUDA(b, cudaMalloc(&b->table_d, b->count * sizeof(BatchInst<Consts>)));
  B_CUDA(b, cudaMemcpy(b->table_d, tab.data(), b->count * sizeof(BatchInst<Consts>), cudaMemcpyHostToDevice));
  b->items = item;
  b->table_G = G;
  return LBM_OK;
}

// Source row of plane i for destination row y (the host's copy of src_row) and the plane of wrap
// block j (of wrap_dir).
inline int plan_src_row(int i, int y, int ym, int yp) { return dir_cy(i) == 1 ? ym : (dir_cy(i) == -1 ? yp : y); }
inline int plan_wrap_dir(int j) { return j == 0 ? 1 : j == 1 ? 5 : j == 2 ? 8 : j == 3 ? 3 : j == 4 ? 6 : 7; }

// Builds the copy plan of the ring tiles for tile shape kW x kC (the table's tiling: whole rows
// where a row holds at most kW strips, kW consecutive strips otherwise). The copies are those
// the stage layout of FlatShape needs, 16-byte aligned:
//   whole-row tiles (rows ya .. ya + rn - 1): per plane i the rows ya - c_y .. as one copy, two
//     where they wrap past row ny - 1, into plane i's stage rows at pitch stride; the mask rows
//     ya - 1 .. ya + rn, one copy each;
//   strip tiles: per row segment g (row y, strips j_lo .. j_hi of the row), the 9 plane rows
//     y - c_y over the segment's cells plus a 16-byte halo each side (clipped to the row), the
//     mask rows y - 1, y, y + 1 from the aligned word below the segment's first cell, and where
//     the segment starts at x = 0 (ends at x = nx - 1) the 16-byte blocks holding column nx - 1
//     of planes 1, 5, 8 (column 0 of planes 3, 6, 7).
// Every copy is checked against its source buffer and its stage region before upload; a plan
// that would leave them is an internal error, reported instead of launched.
template <class ST, int kW, int kC>
int build_plan(lbm_batch* b) {
  using S = FlatShape<ST, kW, kC>;
  constexpr long long es = static_cast<long long>(sizeof(ST));
  std::vector<TilePlan> plans;
  std::vector<CopyOp> ops;
  plans.reserve(static_cast<size_t>(b->tiles));
  const long long state_bytes = b->total_elems * es, mask_bytes = b->mask_words_total * 4;
  bool ok = true;
  // One copy: source byte offset (state or mask buffer), stage byte offset, bytes.
  auto add = [&](long long src, bool from_mask, long long dst, long long bytes, long long dst_lo,
                 long long dst_hi) {
    if (bytes <= 0) return 0LL;
    ok = ok && src % 16 == 0 && dst % 16 == 0 && bytes % 16 == 0 && src >= 0 && dst >= dst_lo &&
         dst + bytes <= dst_hi && src + bytes <= (from_mask ? mask_bytes : state_bytes) &&
         src / 16 <= 0xffffffffLL && dst / 16 < 0x10000 && bytes / 16 < kCopyFromMask;
    if (ok)
      ops.push_back(CopyOp{static_cast<uint32_t>(src / 16), static_cast<uint16_t>(dst / 16),
                           static_cast<uint16_t>(bytes / 16 | (from_mask ? kCopyFromMask : 0))});
    return bytes;
  };
  for (int k = 0; k < b->count && ok; ++k) {
    const auto& in = b->inst[k];
    const Grid2D& g = in.g;
    const int nx = g.nx, ny = g.ny, pitch = g.pitch;
    const int spr = (nx + S::SW - 1) / S::SW;
    const int rpt = spr <= kW ? kW / spr : 0;
    const int ntiles = rpt ? (ny + rpt - 1) / rpt
                           : static_cast<int>((static_cast<long long>(spr) * ny + kW - 1) / kW);
    for (int j = 0; j < ntiles; ++j) {
      TilePlan h{};
      h.first = static_cast<int>(ops.size());
      long long bytes = 0;
      if (rpt) {
        const int ya = j * rpt, rn = std::min(rpt, ny - ya);
        h.inst_nseg = k;
        h.ya = ya;
        h.a = rn;
        for (int i = 0; i < kQ; ++i) {
          int r0 = ya - dir_cy(i);
          r0 = r0 < 0 ? r0 + ny : (r0 >= ny ? r0 - ny : r0);
          const int len0 = std::min(rn, ny - r0);
          const long long plane0 = in.off + i * g.plane;
          const long long lo = i * S::SROW * es, hi = (i + 1) * S::SROW * es;
          bytes += add((plane0 + static_cast<long long>(r0) * pitch) * es, false, lo, len0 * pitch * es, lo, hi);
          bytes += add(plane0 * es, false, lo + len0 * pitch * es, (rn - len0) * pitch * es, lo, hi);
        }
        for (int r = 0; r < rn + 2; ++r) {
          int m = ya - 1 + r;
          m = m < 0 ? m + ny : (m >= ny ? m - ny : m);
          bytes += add((in.mask_off + static_cast<long long>(m) * g.mask_words) * 4, true,
                       S::kPlaneBytes + r * S::MW * 4, S::MW * 4, S::kPlaneBytes,
                       S::kPlaneBytes + S::kMaskBytes);
        }
      } else {
        const int s0 = j * kW, s1 = std::min(s0 + kW, spr * ny);
        const int ya = s0 / spr, nseg = (s1 - 1) / spr - ya + 1;
        h.inst_nseg = k | (nseg << 16);
        h.ya = ya;
        h.a = s0;
        h.b = s1;
        for (int sgi = 0; sgi < nseg; ++sgi) {
          const Segment sg = tile_segment(sgi, s0, s1, ya, spr);
          const int y = sg.y, ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
          const int x0 = sg.j_lo * S::SW;
          const int xs = std::max(x0 - S::H, 0);
          const int xe = std::min((sg.j_hi + 1) * S::SW + S::H, pitch);
          for (int q = 0; q < kQ; ++q) {
            const long long lo = q * S::SROW * es, hi = (q + 1) * S::SROW * es;
            const long long dst = (q * S::SROW + sg.w_first * S::SW + 2 * sgi * S::H + (xs - (x0 - S::H))) * es;
            bytes += add((in.off + q * g.plane + static_cast<long long>(plan_src_row(q, y, ym, yp)) * pitch + xs) * es,
                         false, dst, (xe - xs) * es, lo, hi);
          }
          const int rows3[3] = {ym, y, yp};
          for (int r = 0; r < 3; ++r)
            bytes += add((in.mask_off + static_cast<long long>(rows3[r]) * g.mask_words + (((sg.j_lo * S::SW) >> 5) & ~3)) * 4,
                         true, S::kPlaneBytes + (sgi * 3 + r) * S::MW * 4, S::MW * 4, S::kPlaneBytes,
                         S::kPlaneBytes + S::kMaskBytes);
          for (int wj = 0; wj < 6; ++wj) {
            const bool lo_end = wj < 3;
            if (lo_end ? sg.j_lo != 0 : sg.j_hi != spr - 1) continue;
            const int i = plan_wrap_dir(wj);
            const int xb = lo_end ? ((nx - 1) & ~(S::H - 1)) : 0;
            const long long wlo = S::kPlaneBytes + S::kMaskBytes;
            bytes += add((in.off + i * g.plane + static_cast<long long>(plan_src_row(i, y, ym, yp)) * pitch + xb) * es,
                         false, wlo + (sgi * 6 + wj) * S::H * es, 16, wlo, wlo + S::kWrapBytes);
          }
        }
      }
      h.ncopy = static_cast<int>(ops.size()) - h.first;
      h.bytes = static_cast<int>(bytes);
      plans.push_back(h);
    }
  }
  if (!ok || static_cast<long long>(plans.size()) != b->tiles)
    return bfail(b, LBM_ERR_CUDA, "internal error: a ring tile's copy plan leaves its buffers");
  if (ops.empty()) ops.push_back(CopyOp{0, 0, 0});
  if (b->plans_cap < static_cast<long long>(plans.size())) {
    cudaFree(b->plans_d);
    b->plans_d = nullptr;
    b->plans_cap = 0;
    B_CUDA(b, cudaMalloc(&b->plans_d, plans.size() * sizeof(TilePlan)));
    b->plans_cap = static_cast<long long>(plans.size());
  }
  if (b->ops_cap < static_cast<long long>(ops.size())) {
    cudaFree(b->ops_d);
    b->ops_d = nullptr;
    b->ops_cap = 0;
    B_CUDA(b, cudaMalloc(&b->ops_d, ops.size() * sizeof(CopyOp)));
    b->ops_cap = static_cast<long long>(ops.size());
  }
  B_CUDA(b, cudaMemcpy(b->plans_d, plans.data(), plans.size() * sizeof(TilePlan), cudaMemcpyHostToDevice));
  B_CUDA(b, cudaMemcpy(b->ops_d, ops.data(), ops.size() * sizeof(CopyOp), cudaMemcpyHostToDevice));
  b->plan_sw = S::SW;
  b->plan_kw = kW;
  b->plan_kc = kC;
  return LBM_OK;
}

template <class ST, int G>
int launch_batch_t(lbm_batch* b, int steps, bool prepare_only) {
  using Phys = typename BForm<ST>::Phys;
  const auto kernel = batch_step_kernel<ST, Phys, G>;
  if (prepare_only) {
    // Everything that is not a stream operation happens here, outside any graph capture.
    if (b->table_G != G) {
      if (b->table_sw == 0) {
        b->table_sw = RingShape<ST, 8, 2>::SW;
        b->table_kw = 8;
      }
      if (int rc = build_table<ST>(b, G)) return rc;
    }
    int grid = b->grid;
    if (grid <= 0) {
      int per_sm = 0;
      B_CUDA(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, b->block, 0));
      grid = std::max(1, per_sm) * b->sm_count;
    }
    b->grid_eff = std::max(1, std::min(grid, (b->items + b->block / 32 - 1) / (b->block / 32)));
    return LBM_OK;
  }
  BatchArgs<ST, Phys> a{};
  a.mask = b->mask_d;
  a.inst = static_cast<const BatchInst<typename Phys::Consts>*>(b->table_d);
  a.count = b->count;
  a.items = b->items;
  a.sc = b->sc;
  a.step = b->step_d;
  for (int s = 0; s < steps; ++s) {
    a.src = static_cast<const ST*>(b->buf[b->cur]);
    a.dst = static_cast<ST*>(b->buf[b->cur ^ 1]);
    kernel<<<b->grid_eff, b->block, 0, b->stream>>>(a);
    step_counter_add<<<1, 1, 0, b->stream>>>(b->step_d);
    ++b->t;
    b->cur ^= 1;
  }
  const cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) return bfail(b, LBM_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
  return LBM_OK;
}

// The ring kernel over the ensemble's tiles (one cell, or a pair with 16-bit storage, per lane),
// tile shape kW consumer warps x kC passes, kStages ring stages per block.
template <class ST, int kW, int kC, int kStages>
int launch_batch_ring_t(lbm_batch* b, int steps, bool prepare_only) {
  using Phys = typename BForm<ST>::Phys;
  using S = FlatShape<ST, kW, kC>;
  const auto kernel = batch_ring_kernel<ST, Phys, kW, kC, kStages>;
  const size_t smem = batch_ring_smem<BatchFlatPolicy<ST, Phys, kW, kC>>(kStages);
  if (prepare_only) {
    if (b->table_G == 0 || b->table_sw != S::SW || b->table_kw != kW) {
      b->table_sw = S::SW;
      b->table_kw = kW;
      if (int rc = build_table<ST>(b, b->table_G ? b->table_G : StoreTraits<ST>::kVec)) return rc;
    }
    if (b->plan_sw != S::SW || b->plan_kw != kW || b->plan_kc != kC)
      if (int rc = build_plan<ST, kW, kC>(b)) return rc;
    B_CUDA(b, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int grid = b->grid;
    if (grid <= 0) {
      int per_sm = 0;
      B_CUDA(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, S::kThreads, smem));
      grid = std::max(1, per_sm) * b->sm_count;
    }
    b->grid_eff = std::max(1, std::min(grid, b->tiles));
    return LBM_OK;
  }
  BatchArgs<ST, Phys> a{};
  a.mask = b->mask_d;
  a.inst = static_cast<const BatchInst<typename Phys::Consts>*>(b->table_d);
  a.count = b->count;
  a.items = b->items;
  a.sc = b->sc;
  a.step = b->step_d;
  a.args = static_cast<const StagedArgs<ST, Phys>*>(b->args_d);
  a.tiles = b->tiles;
  a.plans = static_cast<const TilePlan*>(b->plans_d);
  a.ops = static_cast<const CopyOp*>(b->ops_d);
  int* err = reinterpret_cast<int*>(b->step_d + 1);
  for (int s = 0; s < steps; ++s) {
    a.src = static_cast<const ST*>(b->buf[b->cur]);
    a.dst = static_cast<ST*>(b->buf[b->cur ^ 1]);
    a.parity = b->cur;
    // Dependent launches (programmatic stream serialisation): the next launch is scheduled while
    // this one drains (+0.1-0.2 % on the benchmark ensemble).
    B_CUDA(b, launch_dependent(kernel, dim3(b->grid_eff), dim3(S::kThreads), smem, b->stream, a, b->tiles, err));
    B_CUDA(b, launch_dependent(step_counter_add, dim3(1), dim3(1), 0, b->stream, b->step_d));
    ++b->t;
    b->cur ^= 1;
  }
  const cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) return bfail(b, LBM_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
  return LBM_OK;
}

template <class ST>
int launch_batch_ring(lbm_batch* b, int steps, bool prepare_only) {
  const bool deep = b->ring_s == 4;
  if (b->ring_w == 4 && b->ring_c == 2)
    return deep ? launch_batch_ring_t<ST, 4, 2, 4>(b, steps, prepare_only) : launch_batch_ring_t<ST, 4, 2, 2>(b, steps, prepare_only);
  if (b->ring_w == 4 && b->ring_c == 1)
    return deep ? launch_batch_ring_t<ST, 4, 1, 4>(b, steps, prepare_only) : launch_batch_ring_t<ST, 4, 1, 2>(b, steps, prepare_only);
  if (b->ring_w == 2 && b->ring_c == 2)
    return deep ? launch_batch_ring_t<ST, 2, 2, 4>(b, steps, prepare_only) : launch_batch_ring_t<ST, 2, 2, 2>(b, steps, prepare_only);
  return deep ? launch_batch_ring_t<ST, 8, 2, 4>(b, steps, prepare_only) : launch_batch_ring_t<ST, 8, 2, 2>(b, steps, prepare_only);
}

template <class ST>
int launch_batch(lbm_batch* b, int steps, bool prepare_only) {
  constexpr int V = StoreTraits<ST>::kVec;
  constexpr int H = V / 2 >= 2 ? V / 2 : V;  // the narrower vector (8 bytes), FP64 keeps 16
  if (b->G <= 1) return launch_batch_ring<ST>(b, steps, prepare_only);
  if (b->G == H && H != V) return launch_batch_t<ST, H>(b, steps, prepare_only);
  return launch_batch_t<ST, V>(b, steps, prepare_only);
}

int batch_dispatch(lbm_batch* b, int steps, bool prepare_only) {
  switch (b->precision) {
    case LBM_FP32: return launch_batch<float>(b, steps, prepare_only);
    case LBM_FP64: return launch_batch<double>(b, steps, prepare_only);
    case LBM_FP16_STORE: return launch_batch<__half>(b, steps, prepare_only);
    case LBM_BF16_STORE: return launch_batch<__nv_bfloat16>(b, steps, prepare_only);
    default: return LBM_ERR_INVALID_ARG;
  }
}

int batch_steps(lbm_batch* b, int steps) {
  if (int rc = batch_dispatch(b, 0, true)) return rc;
  return batch_dispatch(b, steps, false);
}

// Runs `steps` steps: whole graphs of kGraphSteps launches, then the remainder directly.
int batch_run(lbm_batch* b, int steps) {
  if (steps >= kGraphSteps && (b->graph == nullptr || b->graph_cur != b->cur)) {
    drop_graph(b);
    if (int rc = batch_dispatch(b, 0, true)) return rc;  // table and grid, outside the capture
    const int cur0 = b->cur;
    cudaGraph_t g = nullptr;
    B_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = batch_dispatch(b, kGraphSteps, false);
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();  // the failed capture must not leak into later calls
      b->cur = cur0;
      return rc ? rc : bfail(b, LBM_ERR_CUDA, cudaGetErrorString(e));
    }
    const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return bfail(b, LBM_ERR_CUDA, cudaGetErrorString(ei));
    b->cur = cur0;  // capture recorded the launches without running them
    b->graph_cur = cur0;
  }
  while (steps >= kGraphSteps && b->graph) {
    B_CUDA(b, cudaGraphLaunch(b->graph, b->stream));
    steps -= kGraphSteps;  // kGraphSteps is even: the current buffer is unchanged
  }
  return steps > 0 ? batch_steps(b, steps) : LBM_OK;
}

template <class ST>
int separate_t(lbm_batch* b, int steps) {
  using Phys = typename BForm<ST>::Phys;
  constexpr int G = StoreTraits<ST>::kVec;
  std::vector<StepArgs<ST, Phys>> args(b->count);
  std::vector<int> grids(b->count);
  const auto kernel = pull_step_kernel<ST, Phys, false, 0>;
  int per_sm = 0;
  B_CUDA(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kStepThreads, 0));
  for (int k = 0; k < b->count; ++k) {
    const auto& in = b->inst[k];
    StepArgs<ST, Phys>& a = args[k];
    a = StepArgs<ST, Phys>{};
    a.mask = b->mask_d + in.mask_off;
    a.g = in.g;
    a.cpr = (in.nx + 32 * G - 1) / (32 * G);
    a.items = a.cpr * in.ny;
    a.k = BForm<ST>::consts(in.tau, in.fx, in.fy);
    a.sc = b->sc;
    a.key_base = in.off / kQ;
    a.step_ctr = b->step_d;
    a.step_off = 0;
    grids[k] = std::max(1, std::min((a.items + kStepThreads / 32 - 1) / (kStepThreads / 32),
                                    std::max(1, per_sm) * b->sm_count));
  }
  for (int s = 0; s < steps; ++s) {
    const ST* src = static_cast<const ST*>(b->buf[b->cur]);
    ST* dst = static_cast<ST*>(b->buf[b->cur ^ 1]);
    for (int k = 0; k < b->count; ++k) {
      args[k].src = src + b->inst[k].off;
      args[k].dst = dst + b->inst[k].off;
      kernel<<<grids[k], kStepThreads, 0, b->stream>>>(args[k]);
    }
    step_counter_add<<<1, 1, 0, b->stream>>>(b->step_d);
    ++b->t;
    b->cur ^= 1;
  }
  B_CUDA(b, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int set_inst_t(lbm_batch* b, int k, const void* aos_dev, Eq9<typename StoreTraits<ST>::T> eq) {
  using T = typename StoreTraits<ST>::T;
  const auto& in = b->inst[k];
  const long long n = static_cast<long long>(in.nx) * in.ny;
  const int grid = static_cast<int>(std::min<long long>((n + 255) / 256, 16LL * b->sm_count));
  for (int buf = 0; buf < 2; ++buf)
    set_state_kernel<ST><<<grid, 256, 0, b->stream>>>(static_cast<ST*>(b->buf[buf]) + in.off,
                                                      b->mask_d + in.mask_off, in.g,
                                                      static_cast<const T*>(aos_dev), eq, b->sc);
  B_CUDA(b, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int get_inst_t(lbm_batch* b, int k, void* aos_dev) {
  using T = typename StoreTraits<ST>::T;
  const auto& in = b->inst[k];
  const long long n = static_cast<long long>(in.nx) * in.ny;
  const int grid = static_cast<int>(std::min<long long>((n + 255) / 256, 16LL * b->sm_count));
  get_state_kernel<ST><<<grid, 256, 0, b->stream>>>(static_cast<const ST*>(b->buf[b->cur]) + in.off,
                                                    b->mask_d + in.mask_off, in.g, Eq9<T>{}, b->sc,
                                                    static_cast<T*>(aos_dev));
  B_CUDA(b, cudaGetLastError());
  return LBM_OK;
}

template <class ST>
int mass_inst_t(lbm_batch* b, int k, double* out_dev) {
  using T = typename StoreTraits<ST>::T;
  const auto& in = b->inst[k];
  mass_partial_kernel<ST><<<b->red_blocks, kReduceThreads, 0, b->stream>>>(
      static_cast<const ST*>(b->buf[b->cur]) + in.off, b->mask_d + in.mask_off, in.g, Eq9<T>{}, b->sc,
      b->red);
  mass_final_kernel<<<1, kReduceThreads, 0, b->stream>>>(b->red, b->red_blocks,
                                                         static_cast<double>(in.fluid), out_dev);
  B_CUDA(b, cudaGetLastError());
  return LBM_OK;
}

int ensure_stage(lbm_batch* b, size_t bytes) {
  if (b->stage_bytes >= bytes) return LBM_OK;
  B_CUDA(b, cudaStreamSynchronize(b->stream));
  cudaFree(b->stage);
  b->stage = nullptr;
  b->stage_bytes = 0;
  B_CUDA(b, cudaMalloc(&b->stage, bytes));
  b->stage_bytes = bytes;
  return LBM_OK;
}

#define B_DISPATCH(b, fn, ...)                                      \
  switch ((b)->precision) {                                         \
    case LBM_FP32: return fn<float>(__VA_ARGS__);                   \
    case LBM_FP64: return fn<double>(__VA_ARGS__);                  \
    case LBM_FP16_STORE: return fn<__half>(__VA_ARGS__);            \
    case LBM_BF16_STORE: return fn<__nv_bfloat16>(__VA_ARGS__);     \
    default: return bfail(b, LBM_ERR_INVALID_ARG, "bad precision"); \
  }

template <class ST>
int init_eq_t(lbm_batch* b, double rho0, double ux0, double uy0) {
  using T = typename StoreTraits<ST>::T;
  Eq9<T> e{};
  const T r = T(rho0), u = T(ux0), v = T(uy0);
  const T usq = u * u + v * v, drho0 = r - T(1);
  static const int cx[kQ] = {0, 1, 0, -1, 0, 1, -1, -1, 1}, cy[kQ] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
  for (int i = 0; i < kQ; ++i) {
    const T cu = cx[i] * u + cy[i] * v;
    e.v[i] = weight<T>(i) * (drho0 + r * (T(3) * cu + T(4.5) * cu * cu - T(1.5) * usq));
  }
  for (int k = 0; k < b->count; ++k)
    if (int rc = set_inst_t<ST>(b, k, nullptr, e)) return rc;
  return LBM_OK;
}

template <class ST>
int set_pop_t(lbm_batch* b, int k, const void* host) {
  using T = typename StoreTraits<ST>::T;
  const auto& in = b->inst[k];
  const size_t bytes = static_cast<size_t>(in.nx) * in.ny * kQ * sizeof(T);
  if (int rc = ensure_stage(b, bytes)) return rc;
  B_CUDA(b, cudaMemcpyAsync(b->stage, host, bytes, cudaMemcpyHostToDevice, b->stream));
  if (int rc = set_inst_t<ST>(b, k, b->stage, Eq9<T>{})) return rc;
  B_CUDA(b, cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

template <class ST>
int get_pop_t(lbm_batch* b, int k, void* host) {
  using T = typename StoreTraits<ST>::T;
  const auto& in = b->inst[k];
  const size_t bytes = static_cast<size_t>(in.nx) * in.ny * kQ * sizeof(T);
  if (int rc = ensure_stage(b, bytes)) return rc;
  if (int rc = get_inst_t<ST>(b, k, b->stage)) return rc;
  B_CUDA(b, cudaMemcpyAsync(host, b->stage, bytes, cudaMemcpyDeviceToHost, b->stream));
  B_CUDA(b, cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

// Reads and clears the error flag of the ring kernel's bounded waits (after a synchronisation).
int check_batch_flag(lbm_batch* b) {
  uint32_t flag = 0;
  B_CUDA(b, cudaMemcpyAsync(&flag, b->step_d + 1, sizeof(flag), cudaMemcpyDeviceToHost, b->stream));
  B_CUDA(b, cudaStreamSynchronize(b->stream));
  if (flag) {
    B_CUDA(b, cudaMemsetAsync(b->step_d + 1, 0, sizeof(flag), b->stream));
    return bfail(b, LBM_ERR_TIMEOUT, "a step kernel gave up waiting for its shared-memory ring");
  }
  return LBM_OK;
}

int time_steps(lbm_batch* b, int steps, double* seconds) {
  B_CUDA(b, cudaEventRecord(b->ev[0], b->stream));
  if (int rc = batch_run(b, steps)) return rc;
  B_CUDA(b, cudaEventRecord(b->ev[1], b->stream));
  B_CUDA(b, cudaEventSynchronize(b->ev[1]));
  float ms = 0.f;
  B_CUDA(b, cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
  *seconds = ms * 1e-3;
  return check_batch_flag(b);
}

// Revision of the batch kernels in autotuner cache keys: raised whenever a change can reorder
// the candidates or change what a cached launch means (2: two producer warps per ring block and
// the resident-block caps that come with them; 3: the host-built copy plan), so that older
// cached choices are timed again.
constexpr int kBatchKernelRev = 3;

std::string tune_key(const lbm_batch* b) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, b->device);
  std::ostringstream k;
  k << prop.name << "|p" << b->precision << "|n" << b->count << "|c" << b->total_cells << "|r" << kBatchKernelRev;
  return k.str();
}

}  // namespace

extern "C" {

int lbm_batch_create(int count, const int* nx, const int* ny, const uint8_t* const* solid,
                     const double* tau, const double* fx, const double* fy, int precision,
                     lbm_batch** out) {
  if (!out) return LBM_ERR_INVALID_ARG;
  *out = nullptr;
  const int elem = element_bytes(precision);
  if (count < 1 || count > kBatchMaxInstances || !nx || !ny || !solid || !tau || !fx || !fy || !elem)
    return LBM_ERR_INVALID_ARG;
  for (int k = 0; k < count; ++k) {
    const bool tau_ok = precision == LBM_FP64 ? tau[k] > 0.5 : static_cast<float>(tau[k]) > 0.5f;
    if (nx[k] < 1 || ny[k] < 1 || !solid[k] || !tau_ok) return LBM_ERR_INVALID_ARG;
  }
  lbm_batch* b = new (std::nothrow) lbm_batch();
  if (!b) return LBM_ERR_OUT_OF_MEMORY;
  b->precision = precision;
  b->elem = elem;
  b->vec = 16 / elem;
  if (elem != 8) {  // the untuned ring: 4 x 2 tiles, 4 stages (the benchmark ensemble's tuned choice)
    b->ring_w = 4;
    b->ring_s = 4;
  }
  b->host_elem = precision == LBM_FP64 ? 8 : 4;
  b->count = count;
  b->inst.resize(count);
  const bool s16 = precision == LBM_FP16_STORE || precision == LBM_BF16_STORE;
  for (int i = 0; i < kQ; ++i) {
    b->sc.enc[i] = s16 ? kStoreScale16 : 1.0f;
    b->sc.dec[i] = s16 ? 1.0f / kStoreScale16 : 1.0f;
  }
  auto fail = [&](int code) {
    lbm_batch_destroy(b);
    return code;
  };
  long long off = 0, moff = 0;
  std::vector<uint32_t> words;
  std::vector<uint32_t> all_words;
  const int per_line = 128 / elem;
  for (int k = 0; k < count; ++k) {
    auto& in = b->inst[k];
    in.nx = nx[k];
    in.ny = ny[k];
    in.tau = tau[k];
    in.fx = fx[k];
    in.fy = fy[k];
    in.g.nx = nx[k];
    in.g.ny = ny[k];
    in.g.pitch = (nx[k] + per_line - 1) / per_line * per_line;
    in.g.mask_words = mask_row_words(nx[k]);
    in.g.plane = static_cast<long long>(in.g.pitch) * ny[k];
    in.g.open_x = 0;
    in.off = off;
    in.mask_off = moff;
    in.fluid = 0;
    const size_t n = static_cast<size_t>(nx[k]) * ny[k];
    for (size_t c = 0; c < n; ++c) in.fluid += solid[k][c] ? 0 : 1;
    pack_mask(solid[k], nx[k], ny[k], in.g.mask_words, words);
    all_words.insert(all_words.end(), words.begin(), words.end());
    off += kQ * in.g.plane;
    moff += static_cast<long long>(in.g.mask_words) * ny[k];
    b->total_cells += static_cast<long long>(nx[k]) * ny[k];
  }
  b->total_elems = off;
  b->mask_words_total = moff;
  if (cudaGetDevice(&b->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev[0]) != cudaSuccess || cudaEventCreate(&b->ev[1]) != cudaSuccess)
    return fail(LBM_ERR_CUDA);
  const size_t bytes = static_cast<size_t>(off) * elem + 256;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    e = cudaMalloc(&b->buf[k], bytes);
    if (e == cudaSuccess) e = cudaMemset(b->buf[k], 0, bytes);
  }
  if (e == cudaSuccess) e = cudaMalloc(&b->mask_d, all_words.size() * sizeof(uint32_t));
  if (e == cudaSuccess)
    e = cudaMemcpy(b->mask_d, all_words.data(), all_words.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  b->red_blocks = 4 * b->sm_count;
  if (e == cudaSuccess) e = cudaMalloc(&b->red, (b->red_blocks + 2) * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&b->step_d, 4 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(b->step_d, 0, 4 * sizeof(uint32_t));
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA);
  *out = b;
  return LBM_OK;
}

int lbm_batch_destroy(lbm_batch* b) {
  if (!b) return LBM_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  for (void* p : {b->buf[0], b->buf[1], static_cast<void*>(b->mask_d), b->table_d, b->args_d, b->plans_d, b->ops_d, b->stage,
                  static_cast<void*>(b->red), static_cast<void*>(b->step_d)})
    cudaFree(p);
  for (cudaEvent_t ev : b->ev)
    if (ev) cudaEventDestroy(ev);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return LBM_OK;
}

const char* lbm_batch_last_error(const lbm_batch* b) { return b ? b->err.c_str() : "null"; }

int lbm_batch_init_equilibrium(lbm_batch* b, double rho0, double ux0, double uy0) {
  if (!b) return LBM_ERR_INVALID_ARG;
  B_DISPATCH(b, init_eq_t, b, rho0, ux0, uy0);
}

int lbm_batch_set_populations(lbm_batch* b, int instance, const void* s_host) {
  if (!b || !s_host || instance < 0 || instance >= b->count)
    return bfail(b, LBM_ERR_INVALID_ARG, "bad instance or null state");
  B_DISPATCH(b, set_pop_t, b, instance, s_host);
}

int lbm_batch_get_populations(lbm_batch* b, int instance, void* s_host) {
  if (!b || !s_host || instance < 0 || instance >= b->count)
    return bfail(b, LBM_ERR_INVALID_ARG, "bad instance or null output");
  B_DISPATCH(b, get_pop_t, b, instance, s_host);
}

int lbm_batch_total_mass(lbm_batch* b, int instance, double* mass) {
  if (!b || !mass || instance < 0 || instance >= b->count)
    return bfail(b, LBM_ERR_INVALID_ARG, "bad instance or null output");
  int rc;
  double* out = b->red + b->red_blocks;
  switch (b->precision) {
    case LBM_FP32: rc = mass_inst_t<float>(b, instance, out); break;
    case LBM_FP64: rc = mass_inst_t<double>(b, instance, out); break;
    case LBM_FP16_STORE: rc = mass_inst_t<__half>(b, instance, out); break;
    default: rc = mass_inst_t<__nv_bfloat16>(b, instance, out); break;
  }
  if (rc) return rc;
  B_CUDA(b, cudaMemcpyAsync(mass, out, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  B_CUDA(b, cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

int lbm_batch_run(lbm_batch* b, int steps) {
  if (!b || steps < 0) return bfail(b, LBM_ERR_INVALID_ARG, "steps must be >= 0");
  if (int rc = batch_run(b, steps)) return rc;
  return check_batch_flag(b);
}

int lbm_batch_timed_run(lbm_batch* b, int steps, double* seconds) {
  if (!b || !seconds || steps < 0) return bfail(b, LBM_ERR_INVALID_ARG, "bad arguments");
  return time_steps(b, steps, seconds);
}

int lbm_batch_run_separate(lbm_batch* b, int steps, double* seconds) {
  if (!b || steps < 0) return bfail(b, LBM_ERR_INVALID_ARG, "steps must be >= 0");
  B_CUDA(b, cudaEventRecord(b->ev[0], b->stream));
  int rc;
  switch (b->precision) {
    case LBM_FP32: rc = separate_t<float>(b, steps); break;
    case LBM_FP64: rc = separate_t<double>(b, steps); break;
    case LBM_FP16_STORE: rc = separate_t<__half>(b, steps); break;
    default: rc = separate_t<__nv_bfloat16>(b, steps); break;
  }
  if (rc) return rc;
  B_CUDA(b, cudaEventRecord(b->ev[1], b->stream));
  B_CUDA(b, cudaEventSynchronize(b->ev[1]));
  float ms = 0.f;
  B_CUDA(b, cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
  if (seconds) *seconds = ms * 1e-3;
  drop_graph(b);  // the current buffer may have changed parity
  return LBM_OK;
}

int lbm_batch_set_launch(lbm_batch* b, int cells_per_thread, int block_threads, int grid_blocks) {
  if (!b) return LBM_ERR_INVALID_ARG;
  const int V = b->vec, H = V / 2 >= 2 ? V / 2 : V;
  if ((cells_per_thread > 1 && cells_per_thread != V && cells_per_thread != H) || cells_per_thread < 0 ||
      block_threads % 32 != 0 || block_threads <= 0 || block_threads > kBatchThreads || grid_blocks < 0)
    return bfail(b, LBM_ERR_INVALID_ARG, "bad launch configuration");
  b->G = cells_per_thread;
  b->block = block_threads;
  b->grid = grid_blocks;
  drop_graph(b);
  return LBM_OK;
}

int lbm_batch_set_tiles(lbm_batch* b, int consumer_warps, int passes, int stages) {
  if (!b) return LBM_ERR_INVALID_ARG;
  const bool ok = ((consumer_warps == 8 && passes == 2) || (consumer_warps == 4 && passes == 2) ||
                   (consumer_warps == 4 && passes == 1) || (consumer_warps == 2 && passes == 2)) &&
                  (stages == 2 || stages == 4);
  if (!ok) return bfail(b, LBM_ERR_INVALID_ARG, "tile shape must be 8x2, 4x2, 4x1 or 2x2, with 2 or 4 stages");
  b->ring_w = consumer_warps;
  b->ring_c = passes;
  b->ring_s = stages;
  b->G = 0;
  drop_graph(b);
  return LBM_OK;
}

int lbm_batch_autotune(lbm_batch* b, const char* cache_path, char* report, size_t report_size) {
  if (!b) return LBM_ERR_INVALID_ARG;
  const std::string key = tune_key(b);
  struct Cand {
    int G, blk, per_sm, w, c, s;  // G <= 1: ring kernel of tile shape w x c, s stages
    double t;
  };
  auto apply = [&](const Cand& c) {
    if (c.G <= 1)
      if (int rc = lbm_batch_set_tiles(b, c.w, c.c, c.s)) return rc;
    return lbm_batch_set_launch(b, c.G, c.blk, c.per_sm * b->sm_count);
  };
  auto describe = [&](const Cand& c) {
    std::ostringstream d;
    if (c.G <= 1)
      d << "ring " << c.w << "x" << c.c << " stages=" << c.s << " grid=" << c.per_sm * b->sm_count;
    else
      d << "G=" << c.G << " block=" << c.blk << " grid=" << c.per_sm * b->sm_count;
    return d.str();
  };
  // Cached choice? Lines: key \t G block grid [warps passes].
  if (cache_path) {
    std::ifstream in(cache_path);
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::string k;
      int G, blk, grd, w = 8, c = 2, s = 2;
      if (std::getline(ls, k, '\t') && k == key && (ls >> G >> blk >> grd)) {
        ls >> w >> c >> s;
        const Cand cand{G, blk, grd / std::max(1, b->sm_count), w, c, s, 0.0};
        if (apply(cand) == LBM_OK) {
          b->grid = grd;
          b->tune_report = "cached: " + describe(cand);
          if (report && report_size) std::snprintf(report, report_size, "%s", b->tune_report.c_str());
          return LBM_OK;
        }
      }
    }
  }
  // Time every candidate on the current state; the state and the step counter advance, which
  // is harmless for timing, and both are put back from a saved copy afterwards, on success and
  // on every error exit, together with the launch shape the ensemble had on entry.
  const uint32_t t_saved = b->t;
  const int entry_G = b->G, entry_block = b->block, entry_grid = b->grid;
  const int entry_w = b->ring_w, entry_c = b->ring_c, entry_s = b->ring_s;
  const size_t bytes = static_cast<size_t>(b->total_elems) * b->elem + 256;
  void* saved = nullptr;
  B_CUDA(b, cudaMalloc(&saved, bytes));
  B_CUDA(b, cudaMemcpyAsync(saved, b->buf[b->cur], bytes, cudaMemcpyDeviceToDevice, b->stream));
  auto restore = [&](bool entry_shape) {
    const cudaError_t e1 =
        cudaMemcpyAsync(b->buf[b->cur], saved, bytes, cudaMemcpyDeviceToDevice, b->stream);
    step_counter_set<<<1, 1, 0, b->stream>>>(b->step_d, t_saved);
    b->t = t_saved;
    const cudaError_t e2 = cudaStreamSynchronize(b->stream);
    cudaFree(saved);
    if (entry_shape) {
      b->G = entry_G;
      b->block = entry_block;
      b->grid = entry_grid;
      b->ring_w = entry_w;
      b->ring_c = entry_c;
      b->ring_s = entry_s;
      drop_graph(b);
    }
    return e1 != cudaSuccess ? e1 : e2;
  };
  // An error exit: state, step counter and launch shape back as on entry, the first error kept.
  auto fail_restored = [&](int rc) {
    const std::string msg = b->err;
    restore(true);
    b->err = msg;
    return rc;
  };
  const int V = b->vec, H = V / 2 >= 2 ? V / 2 : V;
  std::vector<Cand> cands;
  // Ring kernel: tile shape x stages x resident blocks per SM (up to what the register and
  // shared-memory budgets let reside).
  const int shapes[6][3] = {{8, 2, 2}, {4, 2, 2}, {4, 2, 4}, {4, 1, 4}, {2, 2, 2}, {2, 2, 4}};
  for (const auto& sh : shapes)
    for (int per_sm : {1, 2, 3, 4, 5, 6, 7, 8})
      if (per_sm <= batch_ring_tune_blocks(b->elem, sh[0]))
        cands.push_back({1, kBatchThreads, per_sm, sh[0], sh[1], sh[2], 0.0});
  for (int G : {V, H}) {  // chunk kernel: cells per thread x block x blocks per SM
    if (G == H && H == V) continue;
    for (int blk : {128, 256})
      for (int per_sm : {1, 2, 4, 8}) cands.push_back({G, blk, per_sm, 8, 2, 2, 0.0});
  }
  if (H == V)
    for (int blk : {128, 256})
      for (int per_sm : {1, 2, 4, 8}) cands.push_back({V, blk, per_sm, 8, 2, 2, 0.0});
  double best = 1e30;
  Cand pick = cands.front();
  std::ostringstream rep;
  for (Cand& c : cands) {
    if (int rc = apply(c)) return fail_restored(rc);
    double t = 0.0;
    if (int rc = time_steps(b, 4, &t)) return fail_restored(rc);  // warm-up
    if (int rc = time_steps(b, 16, &t)) return fail_restored(rc);
    c.t = t;
    rep << (c.G <= 1 ? "R" + std::to_string(c.w) + "x" + std::to_string(c.c) + "s" + std::to_string(c.s)
                     : "G" + std::to_string(c.G) + "/b" + std::to_string(c.blk))
        << "/x" << c.per_sm << ":" << static_cast<long long>(b->total_cells * 16 / t / 1e6) << " ";
    if (t < best) {
      best = t;
      pick = c;
    }
  }
  B_CUDA(b, restore(false));
  if (int rc = apply(pick)) return rc;
  b->tune_report = "tuned: " + describe(pick) + " | " + rep.str();
  if (cache_path) {
    std::ofstream outf(cache_path, std::ios::app);
    outf << key << '\t' << pick.G << ' ' << pick.blk << ' ' << pick.per_sm * b->sm_count << ' ' << pick.w << ' '
         << pick.c << ' ' << pick.s << '\n';
  }
  if (report && report_size) std::snprintf(report, report_size, "%s", b->tune_report.c_str());
  return LBM_OK;
}

int lbm_batch_info(const lbm_batch* b, int* count, long long* total_cells, int* items) {
  if (!b) return LBM_ERR_INVALID_ARG;
  if (count) *count = b->count;
  if (total_cells) *total_cells = b->total_cells;
  if (items) *items = b->items;
  return LBM_OK;
}

}  // extern "C"
