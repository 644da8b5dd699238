// Mass reduction that allocates no device memory: lbm_total_mass_noalloc (include/lbm_b200.h).
//
// Some callers cannot let a library call cudaMalloc: hosts that hand out all device memory from
// their own pool or arena (a stray allocation fragments it, or fails once the pool has taken the
// memory), long-running loops that cannot afford the implicit device-wide synchronisation that
// cudaMalloc and cudaFree may cause, and embedders that pre-reserve a fixed device-memory budget.
// For them this file keeps the reduction's scratch in file-scope __device__ arrays: they are
// part of the loaded module, so every GPU that loads the library holds them (256 KiB) until the
// process exits, and the call itself allocates nothing.
//
// The scratch holds one FP64 partial sum and one fluid-cell count per grid row, hence the row
// limit kNoAllocMaxRows. Every call rewrites all the rows it uses before reading them, so nothing
// needs clearing, but all calls share the same arrays: two calls that overlap on the GPU (for
// example on two streams) race on them.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "lbm_b200.h"

namespace {

constexpr int kNoAllocMaxRows = 16384;  // LBM_NOALLOC_MAX_ROWS in the header
static_assert(kNoAllocMaxRows == LBM_NOALLOC_MAX_ROWS, "header and library disagree");

static __device__ __align__(256) double g_row_sum[kNoAllocMaxRows];
static __device__ __align__(256) unsigned long long g_row_fluid[kNoAllocMaxRows];

// Device addresses of the scratch arrays. In host code the names above are host-side
// stand-ins, not device addresses, so they must never be passed to a kernel. The addresses
// belong to the copy of this module loaded in one CUDA context: every device's primary context
// has its own, a context that the caller creates and makes current (driver API) loads another,
// and cudaDeviceReset discards them. They are therefore looked up once per context and cached
// under the context's process-unique id (cuCtxGetId, which is never reused, unlike a context
// handle), so that a stale address is never handed to a kernel.
struct ScratchAddr {
  unsigned long long ctx_id = 0;
  double* row_sum = nullptr;
  unsigned long long* row_fluid = nullptr;
  bool ready = false;
};
constexpr int kMaxContexts = 64;
std::mutex g_mu;
ScratchAddr g_addr[kMaxContexts];
int g_next_slot = 0;

// The two driver calls that identify the current context, reached through the runtime's
// entry-point query so that the library does not link against libcuda.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
std::once_flag g_driver_once;
bool g_driver_ok = false;

// Pass 1: one warp per row. Per fluid cell the 9 stored populations are added in order
// i = 0..8 in double; lanes take the columns x = lane, lane + 32, ...; the warp then combines
// its 32 partial sums in a fixed shuffle tree.
template <class T>
__global__ void row_sums_kernel(const T* __restrict__ planes, long long plane_stride, int pitch,
                                const uint8_t* __restrict__ solid, int nx, int ny,
                                double* __restrict__ row_sum,
                                unsigned long long* __restrict__ row_fluid) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int y = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; y < ny; y += warps) {
    double acc = 0.0;
    unsigned long long fluid = 0;
    for (int x = lane; x < nx; x += 32) {
      if (solid[static_cast<long long>(y) * nx + x]) continue;
      const T* p = planes + static_cast<long long>(y) * pitch + x;
      double cell = 0.0;
#pragma unroll
      for (int i = 0; i < 9; ++i) cell += static_cast<double>(p[i * plane_stride]);
      acc += cell;
      ++fluid;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc += __shfl_down_sync(0xffffffffu, acc, o);
      fluid += __shfl_down_sync(0xffffffffu, fluid, o);
    }
    if (lane == 0) {
      row_sum[y] = acc;
      row_fluid[y] = fluid;
    }
  }
}

// Pass 2: one block adds the row partials in a fixed order and writes count + sum to *out.
__global__ void rows_total_kernel(const double* __restrict__ row_sum,
                                  const unsigned long long* __restrict__ row_fluid, int ny,
                                  double* __restrict__ out) {
  __shared__ double s_sum[32];
  __shared__ unsigned long long s_cnt[32];
  double acc = 0.0;
  unsigned long long cnt = 0;
  for (int y = threadIdx.x; y < ny; y += blockDim.x) {
    acc += row_sum[y];
    cnt += row_fluid[y];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_down_sync(0xffffffffu, acc, o);
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_sum[warp] = acc;
    s_cnt[warp] = cnt;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    acc = lane < nw ? s_sum[lane] : 0.0;
    cnt = lane < nw ? s_cnt[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc += __shfl_down_sync(0xffffffffu, acc, o);
      cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
      *out = static_cast<double>(cnt) + acc;
    }
  }
}

int report(char* err, size_t err_size, int code, const char* msg) {
  if (err && err_size) std::snprintf(err, err_size, "%s", msg);
  return code;
}

// Process-unique id of the context current on this thread; false if there is none yet or the
// driver cannot tell.
bool current_context_id(unsigned long long* id) {
  std::call_once(g_driver_once, [] {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    const cudaError_t e1 = cudaGetDriverEntryPointByVersion(
        "cuCtxGetCurrent", reinterpret_cast<void**>(&g_ctx_get_current), 12000,
        cudaEnableDefault, &q1);
    const cudaError_t e2 = cudaGetDriverEntryPointByVersion(
        "cuCtxGetId", reinterpret_cast<void**>(&g_ctx_get_id), 12000, cudaEnableDefault, &q2);
    g_driver_ok = e1 == cudaSuccess && e2 == cudaSuccess && q1 == cudaDriverEntryPointSuccess &&
                  q2 == cudaDriverEntryPointSuccess && g_ctx_get_current && g_ctx_get_id;
  });
  if (!g_driver_ok) return false;
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
  return g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}

// Device addresses of the scratch arrays in the current context: from the cache, or looked up
// with cudaGetSymbolAddress (the first call in each context; it also makes the runtime bind
// its context if none is current yet) and cached under the context's id.
int scratch_for_current_context(ScratchAddr* out, char* err, size_t err_size) {
  unsigned long long id = 0;
  if (current_context_id(&id)) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (const ScratchAddr& a : g_addr)
      if (a.ready && a.ctx_id == id) {
        *out = a;
        return LBM_OK;
      }
  }
  ScratchAddr a;
  cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&a.row_sum), g_row_sum);
  if (e == cudaSuccess) e = cudaGetSymbolAddress(reinterpret_cast<void**>(&a.row_fluid), g_row_fluid);
  if (e != cudaSuccess) return report(err, err_size, LBM_ERR_CUDA, cudaGetErrorString(e));
  if (current_context_id(&a.ctx_id)) {
    a.ready = true;
    std::lock_guard<std::mutex> lock(g_mu);
    g_addr[g_next_slot] = a;  // the oldest entry goes first once the table is full
    g_next_slot = (g_next_slot + 1) % kMaxContexts;
  }
  *out = a;
  return LBM_OK;
}

}  // namespace

extern "C" int lbm_total_mass_noalloc(const void* planes, int precision, int nx, int ny,
                                      int row_pitch, long long plane_stride,
                                      const uint8_t* solid, double* mass, void* stream,
                                      char* err, size_t err_size) {
  if (!planes || !solid || !mass)
    return report(err, err_size, LBM_ERR_INVALID_ARG, "null pointer argument");
  if (nx < 1 || ny < 1 || row_pitch < nx || plane_stride < static_cast<long long>(row_pitch) * ny)
    return report(err, err_size, LBM_ERR_INVALID_ARG,
                  "need nx >= 1, ny >= 1, row_pitch >= nx, plane_stride >= row_pitch * ny");
  if (ny > kNoAllocMaxRows)
    return report(err, err_size, LBM_ERR_INVALID_ARG,
                  "ny exceeds LBM_NOALLOC_MAX_ROWS (16384 rows of static scratch)");
  if (precision != LBM_FP32 && precision != LBM_FP64)
    return report(err, err_size, LBM_ERR_UNSUPPORTED, "only LBM_FP32 and LBM_FP64 states");
  ScratchAddr a;
  if (int rc = scratch_for_current_context(&a, err, err_size)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int threads = 256;
  const int blocks = (ny + (threads / 32) - 1) / (threads / 32);
  if (precision == LBM_FP32)
    row_sums_kernel<float><<<blocks, threads, 0, s>>>(static_cast<const float*>(planes),
                                                      plane_stride, row_pitch, solid, nx, ny,
                                                      a.row_sum, a.row_fluid);
  else
    row_sums_kernel<double><<<blocks, threads, 0, s>>>(static_cast<const double*>(planes),
                                                       plane_stride, row_pitch, solid, nx, ny,
                                                       a.row_sum, a.row_fluid);
  rows_total_kernel<<<1, 1024, 0, s>>>(a.row_sum, a.row_fluid, ny, mass);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return report(err, err_size, LBM_ERR_CUDA, cudaGetErrorString(e));
  return report(err, err_size, LBM_OK, "");
}
