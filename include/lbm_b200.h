/*
 * lbm_b200.h - C ABI of the GB300 (sm_103a) D2Q9 lattice-Boltzmann library.
 *
 * The library runs the hot path of the reference solver (H-HABCHANE "Simulation de fluide par
 * la methode de Boltzmann sur reseau", reference paths below are relative to that project):
 * the fused pull-scheme stream-collide step on structure-of-arrays planes of shifted populations
 * g_i = f_i - w_i (D2Q9, BGK, Guo body force, halfway bounce-back on a solid mask, periodic in
 * x and y, optional open inflow/outflow in x) and the rho/u moment pass.
 *
 * The reference has no C ABI: its solvers are C++ classes used through templates
 * (src/common/driver.hpp:5-16). Each entry point below replaces one member of the reference's
 * GPU solver class lbm::SolverV3 (src/v3_cuda_opt/solver_v3.hpp:27-57); the header-only C++
 * wrapper lbm_b200.hpp maps them back onto that member set.
 *
 * Conventions
 *   - Every function returns an int status (LBM_OK = 0). No C++ exception crosses this ABI.
 *     lbm_last_error() describes the last failure of a solver.
 *   - Host arrays use the reference's v0 layout: populations s[(y*nx + x)*9 + i] (post-streaming,
 *     shifted), fields f[y*nx + x]. The element type is the solver's host type: float for
 *     LBM_FP32 / LBM_FP16_STORE / LBM_BF16_STORE, double for LBM_FP64.
 *   - Direction order 0: rest, 1: +x, 2: +y, 3: -x, 4: -y, 5: (+,+), 6: (-,+), 7: (-,-),
 *     8: (+,-) (src/common/d2q9.hpp:14-25).
 *   - All work of a solver is issued on its stream (lbm_set_stream); functions returning host
 *     data synchronise that stream.
 *   - Host buffers that kernels can address (pinned / registered memory) are read and written by
 *     the library's kernels (state upload, moments, populations); other host buffers are staged
 *     through device memory with copies. Results are the same either way.
 */
#ifndef LBM_B200_H
#define LBM_B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum {
  LBM_OK = 0,
  LBM_ERR_INVALID_ARG = 1, /* the reference throws std::invalid_argument (solver_v3.cu:169-170) */
  LBM_ERR_CUDA = 2,        /* a CUDA runtime error (the reference aborts, cuda_check.hpp:17-27) */
  LBM_ERR_OUT_OF_MEMORY = 3,
  LBM_ERR_DIVERGED = 4, /* non-finite density (the reference's driver throws, driver.hpp:217-218) */
  LBM_ERR_UNSUPPORTED = 5,
  LBM_ERR_TIMEOUT = 6 /* a kernel's bounded wait ran out (reported by the next synchronising call) */
};

/* Storage / arithmetic forms. FP32 and FP64 are bit-exact with the reference's v0 in float and
 * double. FP16_STORE / BF16_STORE keep g_i * scale_i in 16 bits (scale_i a power of two per
 * plane) and compute in FP32. The step kernels round each stored value stochastically (unbiased:
 * the expected stored value is the FP32 result), with random bits that are a fixed function of
 * (cell, plane, lattice step), so a run is reproducible; round-to-nearest would drop the sub-ulp
 * per-step increments of low-Mach flows. Uploads (lbm_set_populations, lbm_init_equilibrium)
 * round to nearest. A value beyond the format's range saturates, and lbm_check_finite reports a
 * saturated value as non-finite. */
typedef enum {
  LBM_FP32 = 0,
  LBM_FP64 = 1,
  LBM_FP16_STORE = 2,
  LBM_BF16_STORE = 3
} lbm_precision;

typedef struct lbm_solver lbm_solver;

/* Library version string. */
const char* lbm_version(void);

/* Replaces SolverV3::SolverV3(nx, ny, tau, fx, fy, Mask) (src/v3_cuda_opt/solver_v3.cu:166-186).
 * solid: nx*ny bytes, row-major, non-zero = solid. tau, fx, fy are rounded to the solver
 * precision first (the reference receives them as `real`). Errors: LBM_ERR_INVALID_ARG for
 * nx < 1, ny < 1, a null mask or tau <= 0.5 (solver_v3.cu:169-170); LBM_ERR_OUT_OF_MEMORY. */
int lbm_create(int nx, int ny, const uint8_t* solid, double tau, double fx, double fy,
               int precision, lbm_solver** out);

/* Replaces SolverV3::~SolverV3 (solver_v3.cu:188-192). Null is accepted. */
int lbm_destroy(lbm_solver* s);

/* Message of the last failed call on s ("" if none). Valid until the next call on s. */
const char* lbm_last_error(const lbm_solver* s);

/* Uses `stream` (a cudaStream_t, 0 = legacy default stream) for all later work of s. The
 * reference runs on the legacy default stream (solver_v3.cu:259-264). */
int lbm_set_stream(lbm_solver* s, void* stream);

/* Replaces SolverV3::set_inflow_outflow(u_in) (solver_v3.cu:228-232): open domain in x, inlet
 * velocity (u_in, 0) at x = 0, zero-gradient outlet at x = nx - 1. Call before the initial
 * state is set. Requires nx >= 3. */
int lbm_set_inflow_outflow(lbm_solver* s, double u_in);

/* Replaces SolverV3::init_equilibrium(rho0, ux0, uy0) (solver_v3.cu:194-226): every fluid cell
 * at the equilibrium of (rho0, ux0, uy0), solid cells 0. Built on the device. */
int lbm_init_equilibrium(lbm_solver* s, double rho0, double ux0, double uy0);

/* Sets the post-streaming state from a host array in v0 layout (nx*ny*9 values of the host
 * type); solid cells are ignored. The reference can only set a state through
 * init_equilibrium(); this generalises it to any state (converted to the pull state on the
 * device, by the preimage of streaming). */
int lbm_set_populations(lbm_solver* s, const void* s_host);

/* Enqueues `steps` time steps (asynchronous). Replaces `steps` calls of SolverV3::step()
 * (solver_v3.cu:251-278); steps >= 0. */
int lbm_step(lbm_solver* s, int steps);

/* Replaces SolverV3::run(steps) (solver_v3.cu:280-283): steps, then waits for them. */
int lbm_run(lbm_solver* s, int steps);

/* Replaces SolverV3::timed_run(steps) (solver_v3.cu:285-298): runs `steps` steps and returns
 * their elapsed GPU time in seconds, measured with CUDA events on the solver's stream. */
int lbm_timed_run(lbm_solver* s, int steps, double* seconds);

/* Waits for all work of s. */
int lbm_synchronize(lbm_solver* s);

/* Number of kernels s has enqueued for time steps so far: one per step plus one step-counter
 * update per launch sequence (a replayed step graph counts the kernels it holds). For
 * benchmarks that report how many of the library's kernels ran in a timed region. */
int lbm_kernel_launches(const lbm_solver* s, long long* count);

/* Replaces SolverV3::populations() (solver_v3.cu:300-320): post-streaming populations in v0
 * layout into s_host (nx*ny*9 values of the host type), solid cells 0. The gather runs on the
 * device. */
int lbm_get_populations(lbm_solver* s, void* s_host);

/* Replaces SolverV3::macroscopic(rho, ux, uy) (solver_v3.cu:322-343): rho, ux, uy (nx*ny values
 * each of the host type, row-major) with the Guo half-force velocity; solid cells 0. Computed by
 * a device moment pass, bit-exact with v0 in the FP32 / FP64 forms. */
int lbm_macroscopic(lbm_solver* s, void* rho, void* ux, void* uy);

/* Replaces SolverV3::total_mass() (solver_v3.cu:345-355): fluid-cell count + sum of all fluid
 * populations, accumulated in double on the device (fixed-order two-pass reduction; the
 * summation order differs from v0 in the last bits, as the reference's v1 notes,
 * src/v1_omp/solver_v1.cpp:221-222). */
int lbm_total_mass(lbm_solver* s, double* mass);

/* Replaces SolverV3::populations_at(x, y, out) (solver_v3.cu:234-249): the 9 post-streaming
 * populations of cell (x, y) into out9 (host type). */
int lbm_populations_at(lbm_solver* s, int x, int y, void* out9);

/* Body force by momentum exchange (no counterpart in the reference, which computes no lift;
 * its cylinder case probes u_y behind the disc, src/common/driver.hpp:167-184). For halfway
 * bounce-back on stationary walls, every link from a fluid cell x to a body cell x + c_i carries
 * 2 c_i f*_i(x), f*_i the post-collision population of x leaving along c_i; lbm_body_force sums
 * them over the current state in FP64 (lattice units: force per unit depth). The body is a
 * subset of the solid cells (nx*ny bytes, row-major, nonzero = body) set with lbm_set_body;
 * a null body (the default) means every solid cell. Links leaving an open x boundary carry
 * nothing. */
int lbm_set_body(lbm_solver* s, const uint8_t* body);
int lbm_body_force(lbm_solver* s, double* fx, double* fy);

/* Writes 1 to *finite if every population is finite, else 0 (device check). */
int lbm_check_finite(lbm_solver* s, int* finite);

/* Replaces SolverV3::bench_info() (solver_v3.cu:357-370): JSON fields (no braces) describing
 * the device and the kernel configuration, written into buf (always NUL-terminated). */
int lbm_device_info(lbm_solver* s, char* buf, size_t size);

/* Geometry and precision of s (any pointer may be null). */
int lbm_get_shape(const lbm_solver* s, int* nx, int* ny, int* precision);

/* Kernel configuration of the step: threads per block and blocks (0 = automatic: a persistent
 * grid of resident blocks). Used by the autotuner. */
int lbm_set_launch(lbm_solver* s, int block_threads, int grid_blocks);

/* Step kernel variant (results are identical; used by the autotuner): 0 and 2 load a chunk's
 * plane vectors when the warp reaches it, 1 and 3 also load the warp's next chunk while the
 * current one is computed (more bytes in flight, more registers); 2 and 3 cap the registers for
 * 4 and 3 resident blocks per SM. 4, 5, 6: warp-specialised kernel, a producer warp streams
 * tiles into a shared-memory ring of 2, 3, 4 stages with bulk asynchronous copies (TMA) and
 * eight consumer warps collide from shared memory. 7 and 8: variants 4 and 0 with the FP32
 * collision computed for two cells per packed instruction (other precisions: same as 4 and 0).
 * 9, 10, 11: per-warp pipeline, each warp keeps 2, 3, 4 chunks in flight in its own
 * shared-memory ring with 16-byte asynchronous copies (packed FP32 collision). 12..17: producer
 * warp and bulk-copy ring as in 4, consumers with one cell (FP32 / FP64) or one pair of cells
 * (16-bit storage) per lane, consecutive lanes on consecutive cells: 12 = 8 consumer warps,
 * 2 passes per strip, 2 stages; 13 = the same with 3 stages; 14 = 12 capped at 56 registers for
 * 4 resident blocks; 15 = 4 consumer warps, 3 stages; 16 = 15 capped for 7 resident blocks;
 * 17 = 12 capped for 3 resident blocks; 18 = 17 with 3 stages; 19 = 17 with 1 pass per strip
 * (half-width tiles) and 4 stages; 20 = 8 consumer warps, 4 passes per strip (double-width
 * tiles), 2 stages, 2 resident blocks; 21 = 4 consumer warps, 4 passes, 2 stages, 5 blocks;
 * 22 = 20 with 3 stages. The ring variants are launched with programmatic stream
 * serialisation (the next step's blocks are scheduled while the previous step drains).
 * -1 (the default), by grid size from a sweep on GB300: rows narrower than 256 cells: 0; plain
 * FP32: 19 below 2^17 cells, 17 below 2^21, 12 above; 16-bit storage: 19 below 2^21 cells, 20
 * with rows of at least 2048 cells and 2^22 to 2^25 cells, 17 otherwise; FP64: 12 with at least
 * two 512-cell tiles per SM, 0 otherwise.
 * The 16-bit forms round stored populations stochastically (see lbm_create); every variant
 * derives the same random bits, so the variants give the same results. */
int lbm_set_variant(lbm_solver* s, int variant);

/* Device memory of the two population buffers (for zero-copy consumers): plane stride and row
 * pitch in elements, and the current read buffer. */
int lbm_state_view(lbm_solver* s, void** current, long long* plane_stride, int* row_pitch);

/* Test setting, no counterpart in the reference: the limit, in non-blocking polls, of a ring
 * step kernel's first wait for a staged tile (variants 12-22 of lbm_step / lbm_run, on the
 * current device, for every solver). 0 restores the default (the ordinary bounded wait). A
 * small limit makes that wait run out on purpose, so that the failure path can be tested
 * without a wait that never ends: the kernel sets its error flag, lets every copy it issued
 * land and finishes without computing the rest of its tiles, and the next synchronising call
 * (lbm_run, lbm_synchronize, ...) returns LBM_ERR_TIMEOUT and clears the flag. The state is
 * then invalid until it is set again. */
int lbm_test_set_consumer_wait_limit(unsigned polls);

/* ---------------------------------------------------------------------------------------------
 * Adjoint (no counterpart in the reference): gradients of a flow objective with respect to the
 * body force, tau and a per-cell Brinkman drag field alpha, as a forward/backward pair.
 *   Forward model: the reference's step with a drag force F_tot = F - alpha rho u, the Guo
 *   velocity u = (m + F/2) / (rho (1 + alpha/2)); alpha = 0 is the plain method, bit for bit.
 *   Objective: J = mean over the last `window` states (t = steps - window + 1 .. steps) of the
 *   mean u_x over fluid cells.
 *   The forward run stores the state every `checkpoint_every` steps; the backward run recomputes
 *   each segment from its checkpoint and runs the adjoint step (transposed pull gather with
 *   transposed bounce-back, collision Jacobian transposed) backwards through it. Parameter
 *   gradients are accumulated in double. Closed (periodic in x and y) domains only.
 *   A batch of instances shares geometry, tau and force; each has its own alpha field.
 * ------------------------------------------------------------------------------------------- */
typedef struct lbm_adjoint lbm_adjoint;

/* precision: LBM_FP32 or LBM_FP64; batch >= 1 instances; checkpoint_every >= 1. */
int lbm_adj_create(int nx, int ny, const uint8_t* solid, double tau, double fx, double fy,
                   int precision, int batch, int checkpoint_every, lbm_adjoint** out);
int lbm_adj_destroy(lbm_adjoint* a);
const char* lbm_adj_last_error(const lbm_adjoint* a);
/* New tau / force for all instances (e.g. for finite differences). */
int lbm_adj_set_params(lbm_adjoint* a, double tau, double fx, double fy);
/* alpha: batch * nx * ny doubles (instance-major, row-major), or null for alpha = 0. */
int lbm_adj_set_alpha(lbm_adjoint* a, const double* alpha);
/* Runs `steps` steps from s0 (batch * nx * ny * 9 values of the host type in v0 layout, or null
 * for the rest state f_i - w_i = 0), storing checkpoints; J receives `batch` objectives. */
int lbm_adj_forward(lbm_adjoint* a, const void* s0, int steps, int window, double* J);
/* Gradients of J for every instance (arrays of `batch` values; dalpha: batch * nx * ny, any
 * pointer may be null). Needs a preceding lbm_adj_forward. */
int lbm_adj_backward(lbm_adjoint* a, double* dtau, double* dfx, double* dfy, double* dalpha);
/* Post-streaming populations (v0 layout) of one instance after the forward run. */
int lbm_adj_get_populations(lbm_adjoint* a, int instance, void* s_host);
/* Average device time of one forward step and of one backward step (recomputation included)
 * of the last runs, in seconds. */
int lbm_adj_step_times(lbm_adjoint* a, double* forward_step_s, double* backward_step_s);
/* Tile shape of the forward and backward kernels: cells per consumer lane, 1 (tiles of 256
 * cells of a row) or 2 (512 cells, FP32 only), or 0 for the automatic choice (FP32 forward: the
 * width leaving fewer idle lanes per row, the wider one on a tie; backward and FP64: 1). Results
 * do not depend on it
 * (forward bit for bit; gradients up to the order of their final FP64 sums). */
int lbm_adj_set_tiles(lbm_adjoint* a, int forward_cells, int backward_cells);
int lbm_adj_get_tiles(const lbm_adjoint* a, int* forward_cells, int* backward_cells);

/* ---------------------------------------------------------------------------------------------
 * Batched ensemble (no counterpart in the reference): `count` independent closed channels of
 * uneven sizes, each with its own mask, tau and force, stepped together by one persistent kernel
 * launch per time step, replayed from a CUDA graph. Same arithmetic as the single-grid solver
 * (FP32 / FP64 bit-exact with the reference's v0 per instance).
 * ------------------------------------------------------------------------------------------- */
typedef struct lbm_batch lbm_batch;

/* solid[k]: nx[k]*ny[k] bytes; count <= 4096. */
int lbm_batch_create(int count, const int* nx, const int* ny, const uint8_t* const* solid,
                     const double* tau, const double* fx, const double* fy, int precision,
                     lbm_batch** out);
int lbm_batch_destroy(lbm_batch* b);
const char* lbm_batch_last_error(const lbm_batch* b);
/* Every instance at the equilibrium of (rho0, ux0, uy0). */
int lbm_batch_init_equilibrium(lbm_batch* b, double rho0, double ux0, double uy0);
/* Post-streaming state of one instance, v0 layout, host type (as lbm_set_populations). */
int lbm_batch_set_populations(lbm_batch* b, int instance, const void* s_host);
int lbm_batch_get_populations(lbm_batch* b, int instance, void* s_host);
int lbm_batch_total_mass(lbm_batch* b, int instance, double* mass);
/* `steps` steps of every instance (one launch per step, graph-replayed), then waits. */
int lbm_batch_run(lbm_batch* b, int steps);
/* Same, timed with CUDA events on the batch's stream (seconds). */
int lbm_batch_timed_run(lbm_batch* b, int steps, double* seconds);
/* The comparison point: the same steps with one launch per instance per step. */
int lbm_batch_run_separate(lbm_batch* b, int steps, double* seconds);
/* Launch shape. cells_per_thread 0 or 1: the warp-specialised ring kernel (one cell, or one
 * pair with 16-bit storage, per lane; the default) with the tile shape of lbm_batch_set_tiles;
 * the form's two vector widths (FP32: 4, 2; FP64: 2; 16-bit: 8, 4): the chunk kernel with that
 * many cells per thread and block_threads threads per block (multiple of 32, <= 256).
 * grid_blocks: blocks (0 = all resident blocks). */
int lbm_batch_set_launch(lbm_batch* b, int cells_per_thread, int block_threads, int grid_blocks);
/* Tile shape of the ring kernel (selects it): consumer warps x passes per tile, one of 8x2
 * (the FP64 default), 4x2 (the FP32 / 16-bit default, with 4 stages), 4x1, 2x2, and the ring
 * depth (2 or 4 stages); a tile spans
 * warps * passes * 32 cells of a row (twice that with 16-bit storage), so narrow instances waste
 * fewer lanes with smaller shapes, and deeper rings keep more bytes in flight per block. */
int lbm_batch_set_tiles(lbm_batch* b, int consumer_warps, int passes, int stages);
/* Times the candidate launch shapes on the current ensemble and keeps the fastest; with a cache
 * path the choice is read from / appended to that file (one line per GPU, form, size and kernel
 * revision). The state is restored afterwards. report (may be null) receives a one-line
 * summary. */
int lbm_batch_autotune(lbm_batch* b, const char* cache_path, char* report, size_t report_size);
int lbm_batch_info(const lbm_batch* b, int* count, long long* total_cells, int* items);

/* Largest ny accepted by lbm_total_mass_noalloc (rows of its static scratch). */
#define LBM_NOALLOC_MAX_ROWS 16384

/* ------------------------------------------------------------------------------------------
 * Strip engine: the reference's multi-rank solver (src/v4_mpi_cuda, SolverV4 over StripEngine,
 * engine.hpp:34-62) with the ranks' strips held by one GPU. The lattice is cut into `strips`
 * horizontal strips as the reference's make_strip does (decomposition.hpp:19-33: ny / strips
 * rows each, the first ny % strips one more, at least 2), each with a ghost row below and
 * above; a step runs the step kernel on every strip's owned rows, then one device launch
 * exchanges the halos (populations 2, 5, 6 of each strip's top row into the ghost row below
 * the strip above, 4, 7, 8 of its bottom row into the ghost row above the strip below: the
 * reference's 3 * nx-value messages, engine.hpp:14-20), with no host staging. Results are
 * bit-for-bit those of lbm_create / lbm_step on the whole lattice (and of the reference's v0
 * in FP32 / FP64) for any number of strips. Host arrays as for the solver (v0 layout).
 * ------------------------------------------------------------------------------------------ */
typedef struct lbm_strips lbm_strips;
int lbm_strips_create(int nx, int ny, const uint8_t* solid, double tau, double fx, double fy,
                      int precision, int strips, lbm_strips** out);
int lbm_strips_destroy(lbm_strips* h);
const char* lbm_strips_last_error(const lbm_strips* h);
/* First global row and owned rows of each strip (arrays of `strips` ints). */
int lbm_strips_layout(const lbm_strips* h, int* first_row, int* rows);
int lbm_strips_set_inflow_outflow(lbm_strips* h, double u_in);
int lbm_strips_init_equilibrium(lbm_strips* h, double rho0, double ux0, double uy0);
int lbm_strips_set_populations(lbm_strips* h, const void* s_host);
int lbm_strips_get_populations(lbm_strips* h, void* s_host);
int lbm_strips_macroscopic(lbm_strips* h, void* rho, void* ux, void* uy);
int lbm_strips_step(lbm_strips* h, int steps);
int lbm_strips_timed_run(lbm_strips* h, int steps, double* seconds);

/* Total mass of a pull state held in caller memory, without allocating any device memory.
 * No counterpart in the reference: it is an extra entry point for callers that cannot let a
 * library call cudaMalloc/cudaFree, such as hosts that own all device memory through their own
 * pool or arena, or loops that cannot afford the device synchronisation those calls may cause.
 * The reduction's scratch lives in static device arrays of the library (one FP64 partial and
 * one count per row, 256 KiB, held by every GPU that loads the library until the process
 * exits); nothing else is used.
 *   planes        device pointer to a pull state: 9 planes, plane i row y column x at
 *                 planes[i*plane_stride + y*row_pitch + x] (e.g. lbm_state_view's pointer);
 *   precision     LBM_FP32 (float elements) or LBM_FP64 (double);
 *   solid         device pointer to nx*ny bytes, row-major, non-zero = solid cell;
 *   mass          device pointer to one double that receives fluid-cell count + the sum of the
 *                 stored populations of the fluid cells (the total mass of a periodic domain:
 *                 streaming only permutes the fluid slots);
 *   stream        cudaStream_t the two kernels are enqueued on (asynchronous; 0 = legacy);
 *   err, err_size optional buffer for a message (may be null).
 * Returns LBM_ERR_INVALID_ARG for null pointers, bad sizes, or ny > LBM_NOALLOC_MAX_ROWS;
 * LBM_ERR_UNSUPPORTED for the 16-bit forms. The first call in each CUDA context (the first call
 * on a device, and again after cudaDeviceReset or in a context the caller creates and makes
 * current) looks up the device address of the scratch in that context (cudaGetSymbolAddress)
 * and caches it under the context's id, so make that first call before any stream capture.
 * All calls share the same scratch and every call rewrites the rows it reads: calls that
 * overlap on the GPU (e.g. on two streams) race and must be serialised by the caller. */
int lbm_total_mass_noalloc(const void* planes, int precision, int nx, int ny, int row_pitch,
                           long long plane_stride, const uint8_t* solid, double* mass,
                           void* stream, char* err, size_t err_size);

#ifdef __cplusplus
}
#endif

#endif /* LBM_B200_H */
