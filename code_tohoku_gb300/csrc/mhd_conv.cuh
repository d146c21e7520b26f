// mhd_conv.cuh — FP64 <-> FP32 conversions built from integer instructions.
//
// GB300 issues the hardware conversions (F2F.F32.F64 / F2F.F64.F32) on its
// FP64 pipe, whose rate is about 1/64 of the FP32 pipe, so in the chosen
// form a kernel that loads FP64 state and computes in FP32 would spend most
// of its FP64 issue slots converting.  These helpers do the same conversions
// on the integer ALUs (about ten instructions each):
//
//   d2f: round to nearest (ties away from zero); |d| < 2^-126 flushes to a
//        signed zero, |d| >= 2^128 gives +-Inf, NaN stays NaN.
//   f2d: exact for normal floats; FP32 subnormals flush to a signed zero.
//
// The chosen form runs with FP32 denormals flushed (-ftz=true), so the
// flushes match what the FP32 arithmetic around them does anyway.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace mhd {

__host__ __device__ __forceinline__ uint32_t conv_hi(double d) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2hiint(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return (uint32_t)(u >> 32);
#endif
}
__host__ __device__ __forceinline__ uint32_t conv_lo(double d) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2loint(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return (uint32_t)u;
#endif
}

// Two forms of each conversion, the same results: BR = false evaluates
// every case and selects; BR = true tests the normal range with one
// unsigned compare and branches to the rare cases (zero and flushed values,
// overflow, Inf, NaN), so its common path is a funnel shift, the rounding
// bit and one three-input add (d2f) or a shift and an add (f2d).  Measured
// at 256^3 (ms, selects -> branch): x sweep 1.73 -> 1.69, y 2.01 -> 1.95,
// but z sweep 2.30 -> 2.33, time step 0.34 -> 0.37, SOURCE 0.64 -> 0.70;
// the x and y sweeps take the branching form.
template <bool BR>
__host__ __device__ __forceinline__ float d2f_t(double d) {
  uint32_t hi = conv_hi(d), lo = conv_lo(d);
  uint32_t ah = hi & 0x7fffffffu;
  uint32_t r;
  if constexpr (!BR) {
    // (hi:lo) << 3 keeps the low 9 exponent bits and the 23 mantissa bits
    // the float keeps; +128 in the exponent field re-biases 1023 -> 127
    // modulo 512, which is exact for every exponent of the float range.  The
    // first dropped bit rounds; a carry out of the mantissa moves the
    // exponent up.
    uint32_t t = (hi << 3) | (lo >> 29);
    r = t + (128u << 23) + ((lo >> 28) & 1u);
    if (ah >= 0x47f00000u) r = (ah >= 0x7ff00000u && ((ah & 0xfffffu) | lo)) ? 0x7fc00000u : 0x7f800000u;
    if (ah < 0x38100000u) r = 0u;
  } else if (ah - 0x38100000u < 0x0fe00000u) {   // 2^-126 <= |d| < 2^128
    // the same re-biasing shift and rounding; the result's top bit is 0 in
    // this range (float exponents 1..255 after a rounding carry)
    r = ((hi << 3) | (lo >> 29)) + (128u << 23) + ((lo >> 28) & 1u);
  } else {
    r = ah < 0x38100000u ? 0u : ((ah >= 0x7ff00000u && ((ah & 0xfffffu) | lo)) ? 0x7fc00000u : 0x7f800000u);
  }
  r |= hi & 0x80000000u;
#ifdef __CUDA_ARCH__
  return __uint_as_float(r);
#else
  float f;
  memcpy(&f, &r, 4);
  return f;
#endif
}

template <bool BR>
__host__ __device__ __forceinline__ double f2d_t(float f) {
#ifdef __CUDA_ARCH__
  uint32_t b = __float_as_uint(f);
#else
  uint32_t b;
  memcpy(&b, &f, 4);
#endif
  uint32_t a = b & 0x7fffffffu;
  uint32_t hi, lo;
  if constexpr (!BR) {
    hi = (a >> 3) + (896u << 20);
    lo = a << 29;
    if (a >= 0x7f800000u) hi = 0x7ff00000u | (a >> 3);
    if (a < 0x00800000u) { hi = 0u; lo = 0u; }
  } else if (a - 0x00800000u < 0x7f000000u) {   // normal float
    hi = (a >> 3) + (896u << 20);
    lo = a << 29;
  } else if (a >= 0x7f800000u) {   // Inf, NaN (payload kept)
    hi = 0x7ff00000u | (a >> 3);
    lo = a << 29;
  } else {   // zero and subnormals: signed zero
    hi = 0u;
    lo = 0u;
  }
  hi |= b & 0x80000000u;
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  uint64_t u = ((uint64_t)hi << 32) | lo;
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}

__host__ __device__ __forceinline__ float d2f(double d) { return d2f_t<false>(d); }
__host__ __device__ __forceinline__ double f2d(float f) { return f2d_t<false>(f); }

}  // namespace mhd
