// tx_numeric.cuh -- small device helpers shared by the assembly kernels:
// 4-vector shared-memory access, FP64 reductions, and exact FP32 <-> FP64
// conversions done with integer operations (GB300's FP64 pipe, which runs the
// hardware conversions, is a small fraction of the FP32 rate).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace tx {
namespace {

template <typename R>
struct R4 {
  R x, y, z, w;
};
__device__ __forceinline__ R4<float> ld4(const float* p) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ R4<double> ld4(const double* p) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  return {a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void st4(double* p, double a, double b, double c, double d) {
  reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
  reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
}

// FP64 reduction at an address known to be global memory (red.global: no
// return value, no generic-address resolution), for addresses the compiler
// cannot trace to a global pointer, e.g. ones read from shared memory.  No
// memory clobber: the reduction depends only on its operands and nothing in
// the kernels reads the reduced arrays back, so later shared-memory loads may
// be scheduled ahead of it (CTA barriers still order everything).
__device__ __forceinline__ void red_global(double* p, double v) {
  asm volatile("red.global.add.f64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "d"(v));
}

template <bool ATOMIC>
__device__ __forceinline__ void accumulate(double* p, double v) {
  if constexpr (ATOMIC) atomicAdd(p, v);  // red.global.add.f64
  else *p += v;
}

// Exact IEEE-754 binary32 -> binary64 widening with integer operations:
// exponent rebiased by 1023 - 127 = 896, 23-bit fraction moved to the top of
// the 52-bit fraction.  Keeps the mixed kernel's output conversions off the
// FP64 pipe (a small fraction of the FP32 rate on this part): |v| >> 3 puts
// exponent and fraction in place and adding 896 << 20 rebiases.  Zeros,
// subnormals, infinities and NaNs (one unsigned compare of |v| - 2^-126
// against the normal range) call the ordinary conversion out of line, so the
// compiler cannot if-convert it into every conversion.
__device__ __noinline__ double widen_rare(float v) { return (double)v; }
__device__ __forceinline__ double widen(float v) {
  const uint32_t b = __float_as_uint(v);
  const uint32_t a = b & 0x7fffffffu;
  if (a - 0x00800000u >= 0x7f000000u) return widen_rare(v);
  const uint32_t hi = (b & 0x80000000u) | ((a >> 3) + 0x38000000u);
  return __hiloint2double((int)hi, (int)(b << 29));
}
__device__ __forceinline__ double widen(double v) { return v; }

// Exact IEEE-754 binary64 -> binary32 rounding to nearest, ties to even, with
// integer operations: the 29 dropped fraction bits decide the round-up, whose
// carry runs into the exponent.  Zero is exact; results that would be
// subnormal, overflow, infinities and NaNs call the ordinary conversion out
// of line (kept off the common path, as in widen).
__device__ __noinline__ float narrow_rare(double v) { return (float)v; }
__device__ __forceinline__ float narrow(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const uint32_t hi = (uint32_t)(b >> 32);
  if ((b << 1) == 0ull) return __uint_as_float(hi & 0x80000000u);
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;  // rebias 1023 -> 127
  if (e <= 0 || e >= 255) return narrow_rare(v);
  uint32_t m = (uint32_t)((b & 0xFFFFFFFFFFFFFull) >> 29);
  const uint32_t rest = (uint32_t)(b & 0x1FFFFFFFull);
  m += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
  return __uint_as_float((hi & 0x80000000u) | (((uint32_t)e << 23) + m));
}
template <typename Real>
__device__ __forceinline__ Real to_real(double v) {
  if constexpr (sizeof(Real) == 4) return narrow(v);
  else return v;
}

}  // namespace
}  // namespace tx
