// Internal state of a single-grid solver (the opaque lbm_solver of include/lbm_b200.h).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "lbm_device.cuh"

struct lbm_solver {
  int nx = 0, ny = 0, precision = 0;
  lbm_b200::Grid2D g{};
  int elem = 4;       // bytes per stored population
  int vec = 4;        // cells per 16-byte vector (G)
  int host_elem = 4;  // bytes per host value (float, or double for FP64)
  void* buf[2] = {nullptr, nullptr};  // pull states; buf[cur] is the current one
  int cur = 0;
  uint32_t* step_ctr = nullptr;  // device: lattice steps taken (stochastic-rounding key)
  cudaGraphExec_t graph = nullptr;  // kGraphSteps step launches (see solver_step_raw)
  int graph_cur = -1;               // buffer parity the graph was captured from
  bool graphs = true;               // false after a failed capture
  long long kernels = 0;            // kernels enqueued by steps (step launches and counter updates)
  size_t state_bytes = 0;
  uint32_t* mask_d = nullptr;  // bit-packed mask with periodic ghost bits
  uint32_t* body_d = nullptr;  // bit-packed body of lbm_body_force (null: every solid cell)
  double* force_red = nullptr;  // body-force partials [2 red_blocks], then the result pair
  std::vector<uint8_t> solid;  // host copy (the reference's solid())
  long long fluid = 0;
  double tau = 0, fx = 0, fy = 0;
  bool open_x = false;
  double u_in = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  double* red = nullptr;  // mass partials [red_blocks], result, spare, then an int flag
  int red_blocks = 0;
  void* stage = nullptr;  // device staging for host input / output
  size_t stage_bytes = 0;
  int block = 256, grid = 0, last_grid = 0;  // step launch shape (grid 0: persistent, automatic)
  int* err_flag = nullptr;  // set by a step kernel whose bounded wait ran out
  int variant = -1;      // step kernel variant (lbm_set_variant); -1: chosen from the grid shape
  int last_variant = 0;  // variant of the last launch
  int device = 0, sm_count = 0;
  lbm_b200::PlaneScales sc{};
  std::string err;
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

namespace lbm_b200 {

constexpr int kGraphSteps = 32;  // step launches per captured graph (even)
void drop_step_graph(lbm_solver* s);
// Enqueues `steps` steps without argument checks (graph replays plus single launches).
int solver_step_raw(lbm_solver* s, int steps);
// Two-pass FP64 mass reduction of the pull state `state` into *out (device), using `partials`
// (device, `blocks` doubles) as scratch.
int solver_mass_into(lbm_solver* s, const void* state, double* partials, int blocks, double* out);
// Bit-packed mask rows with the periodic ghost bits (see lbm_device.cuh).
void pack_mask(const uint8_t* solid, int nx, int ny, int mask_words, std::vector<uint32_t>& out);
int element_bytes(int precision);
// Words per bit-packed mask row: the row's bits, the ghost bits, and kMaskPadWords words (all
// solid) past the row, so that a staged copy of a tile's mask words (at most tile width / 32 + 4
// words from the tile's first word, 68 for the widest tile) stays inside; a multiple of 4 so
// that every row starts on a 16-byte boundary (asynchronous-copy alignment).
constexpr int kMaskPadWords = 80;
inline int mask_row_words(int nx) { return ((nx + 31) / 32 + kMaskPadWords + 3) / 4 * 4; }

}  // namespace lbm_b200
