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
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "lbm_b200.h"

namespace {

constexpr int kNoAllocMaxRows = 16384;  // LBM_NOALLOC_MAX_ROWS in the header
constexpr int kMaxDevices = 64;
static_assert(kNoAllocMaxRows == LBM_NOALLOC_MAX_ROWS, "header and library disagree");

static __device__ __align__(256) double g_row_sum[kNoAllocMaxRows];
static __device__ __align__(256) unsigned long long g_row_fluid[kNoAllocMaxRows];

// Device addresses of the scratch arrays, looked up once per device. In host code the names
// above are host-side stand-ins, not device addresses, so they must never be passed to a kernel.
struct ScratchAddr {
  double* row_sum = nullptr;
  unsigned long long* row_fluid = nullptr;
  bool ready = false;
};
std::mutex g_mu;
ScratchAddr g_addr[kMaxDevices];

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

// Looks up the device addresses of the scratch arrays on the current device (first call on
// each device only).
int scratch_for_current_device(ScratchAddr* out, char* err, size_t err_size) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return report(err, err_size, LBM_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return report(err, err_size, LBM_ERR_UNSUPPORTED, "device index beyond the supported range");
  std::lock_guard<std::mutex> lock(g_mu);
  ScratchAddr& a = g_addr[dev];
  if (!a.ready) {
    e = cudaGetSymbolAddress(reinterpret_cast<void**>(&a.row_sum), g_row_sum);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(reinterpret_cast<void**>(&a.row_fluid), g_row_fluid);
    if (e != cudaSuccess) {
      a = ScratchAddr{};
      return report(err, err_size, LBM_ERR_CUDA, cudaGetErrorString(e));
    }
    a.ready = true;
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
  if (int rc = scratch_for_current_device(&a, err, err_size)) return rc;
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
