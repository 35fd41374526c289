// Double <-> float conversions on the integer pipe.
//
// GB300's FP64 pipe issues one warp instruction every ~64 cycles per SM
// sub-partition, and the conversion instructions between double and float
// run on it.  The per-node update and mirror kernels convert a dozen values
// per node, which made them FP64-pipe bound.  These helpers give the same
// bits from integer operations (IEEE 754 round-to-nearest-even, from the
// definition of the formats): a double whose float result is a normal
// number is converted by bit arithmetic, and only zero, subnormal results,
// overflow, infinities and NaN take the conversion instruction.
//
// Host-compilable (the CPU tests check them against the C++ casts).
#pragma once

#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif

namespace sph {

__host__ __device__ __forceinline__ uint64_t bitsOfDouble(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}
__host__ __device__ __forceinline__ double doubleOfBits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}
__host__ __device__ __forceinline__ float floatOfBits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}
__host__ __device__ __forceinline__ uint32_t bitsOfFloat(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

// The conversion instructions, kept out of line so that the compiler
// branches around them instead of predicating them into every call.
#ifdef __CUDA_ARCH__
__device__ __noinline__ inline float castToFloat(double x) { return (float)x; }
__device__ __noinline__ inline double castToDouble(float x) { return (double)x; }
__device__ __noinline__ inline double castIntToDouble(int x) { return (double)x; }
#else
inline float castToFloat(double x) { return (float)x; }
inline double castToDouble(float x) { return (double)x; }
inline double castIntToDouble(int x) { return (double)x; }
#endif

// double -> float, round to nearest even.  Exponent field e of the double:
// the float is normal before rounding when 897 <= e <= 1150 (float exponent
// e - 896 in 1..254).  Dropping the 29 low mantissa bits with a rounding
// bias of 2^28 - 1 plus the kept lowest bit rounds to nearest, ties to even;
// a carry out of the mantissa moves into the exponent, up to the infinity
// pattern for results at or above FLT_MAX + half an ulp.
__host__ __device__ __forceinline__ float toFloatRN(double x) {
  const uint64_t b = bitsOfDouble(x);
  const uint64_t mag = b & 0x7fffffffffffffffULL;
  if (mag - (897ULL << 52) >= ((1151ULL - 897ULL) << 52)) return castToFloat(x);
  const uint64_t r = (mag + 0x0fffffffULL + ((mag >> 29) & 1ULL)) >> 29;
  const uint32_t f = (uint32_t)(r - (896ULL << 23));
  return floatOfBits(f | ((uint32_t)(b >> 32) & 0x80000000u));
}

// float -> double (exact).  A normal float (exponent field 1..254) moves its
// exponent up by 1023 - 127 = 896 and its mantissa up by 29 bits.
__host__ __device__ __forceinline__ double toDouble(float x) {
  const uint32_t b = bitsOfFloat(x);
  const uint32_t mag = b & 0x7fffffffu;
  if (mag - 0x00800000u >= 0x7f000000u) return castToDouble(x);
  const uint64_t d = ((uint64_t)mag << 29) + (896ULL << 52);
  return doubleOfBits(d | ((uint64_t)(b & 0x80000000u) << 32));
}

// Non-negative int -> double (exact): the top set bit gives the exponent,
// the bits below it the mantissa.
__host__ __device__ __forceinline__ double smallIntToDouble(int c) {
  if (c <= 0) return c == 0 ? 0.0 : castIntToDouble(c);
#ifdef __CUDA_ARCH__
  const int e = 31 - __clz(c);
#else
  const int e = 31 - __builtin_clz((unsigned)c);
#endif
  const uint64_t m = ((uint64_t)c << (52 - e)) & ((1ULL << 52) - 1ULL);
  return doubleOfBits(((uint64_t)(1023 + e) << 52) | m);
}

}  // namespace sph
