// Device-side building blocks shared by the kernels of the library: arithmetic policies, the
// storage codecs of the populations, 16-byte vector loads/stores, the bit-packed solid mask and
// the kernel argument blocks.
//
// Data layout in HBM (one instance):
//   populations  R[i][y][x] at  base + i * plane + y * pitch + x   (structure of arrays: 9 planes
//                of shifted post-collision populations g_i = f_i - w_i, pull scheme). pitch is nx
//                rounded up so that every row starts on a 128-byte boundary; plane = pitch * ny.
//                Two such buffers (read / write), swapped every step.
//   mask         uint32 words, mask_words per row, bit (x + 1) of row y = solid(x, y); bit 0 holds
//                solid(nx - 1, y) and bit nx + 1 holds solid(0, y) (the periodic neighbours of the
//                edge columns), bits beyond nx + 1 are 1. A thread that owns cells x0 .. x0+G-1
//                extracts the G + 2 bits of cells x0 - 1 .. x0 + G with one funnel shift.
#pragma once

#include <utility>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "collide.h"

namespace lbm_b200 {

// ---------------------------------------------------------------------------------------------
// Arithmetic policies
// ---------------------------------------------------------------------------------------------
// IEEE round-to-nearest operations that the compiler never contracts into FMA (CUDA's __f*_rn /
// __d*_rn intrinsics). Used by the plain FP32/FP64 forms, which must match the reference bit for
// bit. Host fallbacks keep the templates instantiable on the host side of the translation unit.
struct ExactF32 {
  using T = float;
  using S = float;
  static __host__ __device__ __forceinline__ float k(float v) { return v; }
  static __host__ __device__ __forceinline__ float neg(float a) { return -a; }
  static __host__ __device__ __forceinline__ float add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
  }
  static __host__ __device__ __forceinline__ float sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
  }
  static __host__ __device__ __forceinline__ float mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
  }
  static __host__ __device__ __forceinline__ float div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
  }
};

struct ExactF64 {
  using T = double;
  using S = double;
  static __host__ __device__ __forceinline__ double k(double v) { return v; }
  static __host__ __device__ __forceinline__ double neg(double a) { return -a; }
  static __host__ __device__ __forceinline__ double add(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
  }
  static __host__ __device__ __forceinline__ double sub(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
  }
  static __host__ __device__ __forceinline__ double mul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
  }
  static __host__ __device__ __forceinline__ double div(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
  }
};

// Exact FP32 arithmetic on two cells per instruction (packed add.rn.f32x2 / fma.rn.f32x2).
// Each packed operation is correctly rounded per lane, like the scalar one, but the compiler
// contracts a packed multiply feeding a packed add into one fused multiply-add even when both
// carry an explicit rounding mode (measured: 3a + 4.5aa differs from the two-rounding result in
// 25% of random pairs, the rate of contraction). So the multiply is written as a fused
// multiply-add with a -0 addend, round(a*b + -0) = round(a*b) for every a, b (a zero product
// keeps its sign), and the -0 comes from constant memory, a value the compiler cannot see
// through: nothing is left to contract. Division stays per lane (__fdiv_rn).
static __constant__ float2 kNegZero2 = {-0.0f, -0.0f};

struct ExactF32x2 {
  using T = float2;
  using S = float;
  static __device__ __forceinline__ float2 k(float v) { return make_float2(v, v); }
  static __device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
  static __device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
  static __device__ __forceinline__ float2 sub(float2 a, float2 b) { return __fadd2_rn(a, neg(b)); }
  static __device__ __forceinline__ float2 mul(float2 a, float2 b) { return __ffma2_rn(a, b, kNegZero2); }
  static __device__ __forceinline__ float2 div(float2 a, float2 b) {
    return make_float2(__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y));
  }
};

// Packed arithmetic of the fast collision (two cells per instruction). The reciprocal of the
// density is the hardware approximation (rcp.approx.ftz.f32: at most 1 ulp from the correctly
// rounded value, one instruction; the correctly rounded one is a sequence with a slow path):
// rho stays near 1, far from the subnormal range, and the 16-bit storage that follows rounds
// 2^13 (FP16) to 2^16 (BF16) times coarser. The issue-bound batched ensemble ran 4.6 % faster
// with it in FP16.
__device__ __forceinline__ float rcp_approx(float a) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}
struct FastF32x2 {
  using T = float2;
  static __device__ __forceinline__ float2 k(float v) { return make_float2(v, v); }
  static __device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
  static __device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
  static __device__ __forceinline__ float2 sub(float2 a, float2 b) { return __fadd2_rn(a, neg(b)); }
  static __device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
  static __device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
  static __device__ __forceinline__ float2 rcp(float2 a) { return make_float2(rcp_approx(a.x), rcp_approx(a.y)); }
};

// ---------------------------------------------------------------------------------------------
// Storage codecs: stored type ST <-> compute type T. Plain forms store T itself; the 16-bit
// forms store g_i * scale_i rounded to half / bfloat16, scale_i a power of two per plane.
// ---------------------------------------------------------------------------------------------
template <class ST>
struct StoreTraits;
template <>
struct StoreTraits<float> {
  using T = float;
  static constexpr int kVec = 4;  // cells per 16-byte vector
};
template <>
struct StoreTraits<double> {
  using T = double;
  static constexpr int kVec = 2;
};
template <>
struct StoreTraits<__half> {
  using T = float;
  static constexpr int kVec = 8;
};
template <>
struct StoreTraits<__nv_bfloat16> {
  using T = float;
  static constexpr int kVec = 8;
};

struct PlaneScales {
  float enc[kQ];  // stored = g * enc[i]
  float dec[kQ];  // g = stored * dec[i]
};

// Storage scale of the 16-bit forms, the same power of two for every plane (the step kernels
// fold it into the collision constants): |g_i| <= 2 fits FP16 (g_i = f_i - w_i of a state with
// 0 <= f_i <= 1 lies in [-w_i, 1 - w_i]), and values down to 2^-29 stay normal.
constexpr float kStoreScale16 = 32768.0f;

__device__ __forceinline__ float to_float(__half h) { return __half2float(h); }
__device__ __forceinline__ float to_float(__nv_bfloat16 h) { return __bfloat162float(h); }
template <class ST>
__device__ __forceinline__ ST from_float(float v);
template <>
__device__ __forceinline__ __half from_float<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_float<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}

// Scalar decode / encode of plane i.
template <class ST>
__device__ __forceinline__ typename StoreTraits<ST>::T decode(ST v, int, const PlaneScales&) {
  return v;
}
template <>
__device__ __forceinline__ float decode<__half>(__half v, int i, const PlaneScales& s) {
  return to_float(v) * s.dec[i];
}
template <>
__device__ __forceinline__ float decode<__nv_bfloat16>(__nv_bfloat16 v, int i,
                                                       const PlaneScales& s) {
  return to_float(v) * s.dec[i];
}
template <class ST>
__device__ __forceinline__ ST encode(typename StoreTraits<ST>::T v, int, const PlaneScales&) {
  return v;
}
template <>
__device__ __forceinline__ __half encode<__half>(float v, int i, const PlaneScales& s) {
  return from_float<__half>(v * s.enc[i]);
}
template <>
__device__ __forceinline__ __nv_bfloat16 encode<__nv_bfloat16>(float v, int i,
                                                               const PlaneScales& s) {
  return from_float<__nv_bfloat16>(v * s.enc[i]);
}

// 16-byte vector load (read-only path) / store of kVec consecutive cells in the step kernels'
// compute representation (plain forms: the values; 16-bit forms: the scaled values widened to
// FP32, see load_vec16).
template <class ST>
__device__ __forceinline__ void load_vec(const ST* p, typename StoreTraits<ST>::T (&v)[StoreTraits<ST>::kVec],
                                         int plane_index, const PlaneScales& s);
template <>
__device__ __forceinline__ void load_vec<float>(const float* p, float (&v)[4], int,
                                                const PlaneScales&) {
  const float4 t = __ldg(reinterpret_cast<const float4*>(p));
  v[0] = t.x;
  v[1] = t.y;
  v[2] = t.z;
  v[3] = t.w;
}
template <>
__device__ __forceinline__ void load_vec<double>(const double* p, double (&v)[2], int,
                                                 const PlaneScales&) {
  const double2 t = __ldg(reinterpret_cast<const double2*>(p));
  v[0] = t.x;
  v[1] = t.y;
}
// 16-bit forms: the step kernels compute on the scaled values (FastConsts carries the scale), so
// their loads only widen to FP32.
template <class H>
__device__ __forceinline__ void load_vec16(const H* p, float (&v)[8], int, const PlaneScales&) {
  const uint4 t = __ldg(reinterpret_cast<const uint4*>(p));
  const uint32_t w[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    H lo, hi;
    const uint16_t a = static_cast<uint16_t>(w[k] & 0xffffu), b = static_cast<uint16_t>(w[k] >> 16);
    memcpy(&lo, &a, 2);
    memcpy(&hi, &b, 2);
    v[2 * k] = to_float(lo);
    v[2 * k + 1] = to_float(hi);
  }
}
template <>
__device__ __forceinline__ void load_vec<__half>(const __half* p, float (&v)[8], int i,
                                                 const PlaneScales& s) {
  load_vec16(p, v, i, s);
}
template <>
__device__ __forceinline__ void load_vec<__nv_bfloat16>(const __nv_bfloat16* p, float (&v)[8],
                                                        int i, const PlaneScales& s) {
  load_vec16(p, v, i, s);
}

template <class ST>
__device__ __forceinline__ void store_vec(ST* p, const typename StoreTraits<ST>::T (&v)[StoreTraits<ST>::kVec],
                                          int plane_index, const PlaneScales& s);
template <>
__device__ __forceinline__ void store_vec<float>(float* p, const float (&v)[4], int,
                                                 const PlaneScales&) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <>
__device__ __forceinline__ void store_vec<double>(double* p, const double (&v)[2], int,
                                                  const PlaneScales&) {
  *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
}
template <class H>
__device__ __forceinline__ void store_vec16(H* p, const float (&v)[8], int i, const PlaneScales& s) {
  uint32_t w[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const H lo = from_float<H>(v[2 * k] * s.enc[i]);
    const H hi = from_float<H>(v[2 * k + 1] * s.enc[i]);
    uint16_t a, b;
    memcpy(&a, &lo, 2);
    memcpy(&b, &hi, 2);
    w[k] = static_cast<uint32_t>(a) | (static_cast<uint32_t>(b) << 16);
  }
  *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
}
template <>
__device__ __forceinline__ void store_vec<__half>(__half* p, const float (&v)[8], int i,
                                                  const PlaneScales& s) {
  store_vec16(p, v, i, s);
}
template <>
__device__ __forceinline__ void store_vec<__nv_bfloat16>(__nv_bfloat16* p, const float (&v)[8],
                                                         int i, const PlaneScales& s) {
  store_vec16(p, v, i, s);
}

// ---------------------------------------------------------------------------------------------
// Stochastic rounding of the 16-bit storage forms.
//
// Round-to-nearest storage loses every per-step change smaller than half a unit in the last
// place of the stored value: at low Mach numbers the body-force and viscous increments of g_i
// (~1e-6) are below half an FP16 ulp of g_i (~4e-6), so the flow stagnates (measured: 10 %
// velocity error on a developing Poiseuille channel). The step kernels therefore round the
// encoded FP32 value v to the 16-bit format stochastically: with D the number of significand
// bits the format drops (FP16 13, BF16 16) and r uniform in [0, 2^D), the magnitude bits of v
// plus r are truncated (round toward zero), which rounds up with probability equal to the
// dropped fraction, so E[stored] = v and sub-ulp increments survive on average.
//
// Blackwell does this in one instruction per pair of values: cvt.rs.satfinite.{f16x2,bf16x2}.f32
// takes 32 random bits and adds D of them below the kept significand of each value before
// truncating. An in-bounds probe on a GB300 (single set bits, and the mean over 10^6 random
// words) showed which bits each half uses and that the result is unbiased: FP16 takes bits
// [0, 13) for the low half and [16, 29) for the high half, BF16 bits [0, 16) and [16, 32); all
// random bits zero is plain truncation. .satfinite clamps a value past the format's largest
// finite value to it (the finite check treats a saturated value as diverged). Against adding
// the bits with integer instructions and converting with cvt.rz (six instructions per pair),
// it made the issue-bound batched ensemble 4.7 % faster in FP16.
//
// The random bits of each value are a deterministic function of (cell pair, plane, step): a
// 32-bit hash H of the pair's cell offset (y * pitch + x) / 2 xor the step key, rotated left by
// 7 i bits for plane i, gives the conversion's 32 random bits; the two halves read disjoint
// fields, each uniform because H is. Fields of different planes overlap, so their rounding
// errors are correlated, which leaves every stored value unbiased. Every kernel variant derives
// them identically, so results do not depend on the variant, and a run is reproducible from its
// step counter. The hash is the "lowbias32" integer mixer (C. Wellons, hash-prospector, 2018).
// ---------------------------------------------------------------------------------------------
__host__ __device__ constexpr uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
__host__ __device__ constexpr int sr_plane_rot(int i) { return (7 * i) & 31; }
// Key of lattice step t (computed on the host for each launch, or on the device from a step
// counter in device memory for graph-captured launches).
__host__ __device__ constexpr uint32_t sr_step_key(uint32_t t) { return mix32(t * 0x9e3779b9u + 0x7f4a7c15u); }
// Hash of the cell pair whose even cell sits at cell offset `cell` (y * pitch + x + base).
__device__ __forceinline__ uint32_t sr_pair_hash(long long cell, uint32_t rkey) {
  return mix32(static_cast<uint32_t>(cell >> 1) ^ rkey);
}

// Stochastically rounded, saturating conversion of a pair (lo = even cell, in the low half).
template <class ST>
__device__ __forceinline__ uint32_t cvt_rs_pair(float lo, float hi, uint32_t rbits);
template <>
__device__ __forceinline__ uint32_t cvt_rs_pair<__half>(float lo, float hi, uint32_t rbits) {
  uint32_t d;
  asm("cvt.rs.satfinite.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
  return d;
}
template <>
__device__ __forceinline__ uint32_t cvt_rs_pair<__nv_bfloat16>(float lo, float hi, uint32_t rbits) {
  uint32_t d;
  asm("cvt.rs.satfinite.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
  return d;
}

// Stochastically rounded pair of plane-i values, already scaled (lo = even cell, in the low
// half).
template <class ST>
__device__ __forceinline__ uint32_t encode_pair_sr(float lo, float hi, int i, uint32_t pair_hash) {
  return cvt_rs_pair<ST>(lo, hi, __funnelshift_l(pair_hash, pair_hash, sr_plane_rot(i)));
}

// True for a stored 16-bit value at the format's largest finite magnitude (saturated).
template <class ST>
__device__ __forceinline__ bool stored_saturated(ST) {
  return false;
}
template <>
__device__ __forceinline__ bool stored_saturated<__half>(__half v) {
  uint16_t b;
  memcpy(&b, &v, 2);
  return (b & 0x7fffu) == 0x7bffu;
}
template <>
__device__ __forceinline__ bool stored_saturated<__nv_bfloat16>(__nv_bfloat16 v) {
  uint16_t b;
  memcpy(&b, &v, 2);
  return (b & 0x7fffu) == 0x7f7fu;
}

// G consecutive cells as one aligned vector of G * sizeof(ST) bytes (8 or 16), decoded /
// encoded; generalises load_vec / store_vec to the narrower vectors of the cells-per-thread
// tuning dimension.
template <class ST, int G>
struct VecIO;
template <class ST>
struct VecIO<ST, StoreTraits<ST>::kVec> {
  using T = typename StoreTraits<ST>::T;
  static constexpr int G = StoreTraits<ST>::kVec;
  static __device__ __forceinline__ void load(const ST* p, T (&v)[G], int i, const PlaneScales& s) {
    load_vec<ST>(p, v, i, s);
  }
  static __device__ __forceinline__ void store(ST* p, const T (&v)[G], int i, const PlaneScales& s) {
    store_vec<ST>(p, v, i, s);
  }
};
template <>
struct VecIO<float, 2> {
  static __device__ __forceinline__ void load(const float* p, float (&v)[2], int, const PlaneScales&) {
    const float2 t = __ldg(reinterpret_cast<const float2*>(p));
    v[0] = t.x;
    v[1] = t.y;
  }
  static __device__ __forceinline__ void store(float* p, const float (&v)[2], int, const PlaneScales&) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  }
};
template <class H>
struct VecIO16x4 {
  static __device__ __forceinline__ void load(const H* p, float (&v)[4], int, const PlaneScales&) {
    const uint2 t = __ldg(reinterpret_cast<const uint2*>(p));
    const uint32_t w[2] = {t.x, t.y};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      H lo, hi;
      const uint16_t a = static_cast<uint16_t>(w[k] & 0xffffu), b = static_cast<uint16_t>(w[k] >> 16);
      memcpy(&lo, &a, 2);
      memcpy(&hi, &b, 2);
      v[2 * k] = to_float(lo);
      v[2 * k + 1] = to_float(hi);
    }
  }
  static __device__ __forceinline__ void store(H* p, const float (&v)[4], int i, const PlaneScales& s) {
    uint32_t w[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const H lo = from_float<H>(v[2 * k] * s.enc[i]);
      const H hi = from_float<H>(v[2 * k + 1] * s.enc[i]);
      uint16_t a, b;
      memcpy(&a, &lo, 2);
      memcpy(&b, &hi, 2);
      w[k] = static_cast<uint32_t>(a) | (static_cast<uint32_t>(b) << 16);
    }
    *reinterpret_cast<uint2*>(p) = make_uint2(w[0], w[1]);
  }
};
template <>
struct VecIO<__half, 4> : VecIO16x4<__half> {};
template <>
struct VecIO<__nv_bfloat16, 4> : VecIO16x4<__nv_bfloat16> {};

template <class ST>
__device__ __forceinline__ typename StoreTraits<ST>::T load_one(const ST* p, int i,
                                                                const PlaneScales& s) {
  return decode<ST>(__ldg(p), i, s);
}
// One value in the step kernels' compute representation (16-bit forms: scaled, widened).
template <class ST>
__device__ __forceinline__ typename StoreTraits<ST>::T widen(ST v) {
  if constexpr (sizeof(ST) == 2)
    return to_float(v);
  else
    return v;
}
template <class ST>
__device__ __forceinline__ typename StoreTraits<ST>::T load_step(const ST* p) {
  return widen<ST>(__ldg(p));
}

// ---------------------------------------------------------------------------------------------
// Bit-packed mask
// ---------------------------------------------------------------------------------------------
// Bits x0 .. x0+31 of a mask row (cells x0 - 1 .. x0 + 30).
__device__ __forceinline__ uint32_t mask_window(const uint32_t* __restrict__ row, int x0) {
  const int w = x0 >> 5;
  return __funnelshift_r(__ldg(row + w), __ldg(row + w + 1), x0 & 31);
}
__device__ __forceinline__ bool mask_solid(const uint32_t* __restrict__ mask, int mask_words,
                                           int x, int y) {
  const uint32_t word = __ldg(mask + static_cast<size_t>(y) * mask_words + ((x + 1) >> 5));
  return (word >> ((x + 1) & 31)) & 1u;
}

// ---------------------------------------------------------------------------------------------
// Geometry of one instance on the device
// ---------------------------------------------------------------------------------------------
// Step-kernel store of G consecutive cells x0 .. x0 + G - 1 of plane i (x0 even): plain forms
// store the values, 16-bit forms round each pair k of scaled values stochastically with pair
// hash ph[k].
template <class ST, int G>
struct StepStore {
  static constexpr bool kSr = sizeof(ST) == 2;
  static constexpr int kPairs = kSr ? G / 2 : 1;
  static __device__ __forceinline__ void hashes(long long cell0, uint32_t rkey, uint32_t (&ph)[kPairs]) {
#pragma unroll
    for (int k = 0; k < kPairs; ++k) ph[k] = sr_pair_hash(cell0 + 2 * k, rkey);
  }
  static __device__ __forceinline__ void store(ST* p, const typename StoreTraits<ST>::T (&v)[G], int i,
                                               const PlaneScales& s, const uint32_t (&ph)[kPairs]) {
    if constexpr (kSr) {
      static_assert(G == 4 || G == 8, "16-bit stores are 8 or 16 bytes");
      uint32_t w[G / 2];
#pragma unroll
      for (int k = 0; k < G / 2; ++k) w[k] = encode_pair_sr<ST>(v[2 * k], v[2 * k + 1], i, ph[k]);
      if constexpr (G == 8)
        *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
      else
        *reinterpret_cast<uint2*>(p) = make_uint2(w[0], w[1]);
    } else {
      (void)ph;
      VecIO<ST, G>::store(p, v, i, s);
    }
  }
};

struct Grid2D {
  int nx, ny, pitch;
  int mask_words;
  long long plane;  // elements per population plane (pitch * ny)
  int open_x;
};

// Nine values passed by value as a kernel parameter (inlet or initial equilibrium).
template <class T>
struct Eq9 {
  T v[kQ];
};

// ---------------------------------------------------------------------------------------------
// Programmatic dependent launch, device side: wait until the previous kernel on the stream has
// completed and its writes are visible (a no-op for a kernel launched without the attribute),
// then let the next kernel's blocks be scheduled as this one's exit.
__device__ __forceinline__ void grid_dependency_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Host side: a launch with programmatic stream serialisation, so that its blocks may be
// scheduled while the previous kernel on the stream drains (they start with
// grid_dependency_wait before touching memory).
template <class... Params, class... Args>
cudaError_t launch_dependent(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                             Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace lbm_b200
