// detmath.h — deterministic double-precision exp / log / log10 / 10^x.
//
// The KI cooling function and the implicit cooling bisection evaluate
// dexp, dlog10 and 10.d0**x (KIcool/1DMHDwCC3.f90:1131,1170-1172;
// 3DMHD-CfCA/MCF3DSGincfca3.f90:2913).  The host C library and the CUDA
// device library round those functions differently in the last bit, and
// the bisection turns a one-ulp difference into a different branch.  To
// make the GPU FP64 path and the CPU restatement produce identical bits,
// both call the functions below.  They use only IEEE +,-,*,/ and exact
// power-of-two scaling, so the result is the same on x86-64, aarch64 and
// the GPU as long as floating-point contraction is disabled
// (-ffp-contract=off on the host, --fmad=false on the device).
//
// Methods (all public textbook material):
//  * exp: Cody & Waite additive range reduction x = k*ln2 + r with a split
//    ln2 = LN2_HI + LN2_LO (LN2_HI has 42 significant bits so k*LN2_HI is
//    exact for |k| < 2^11), then the Taylor series of e^r to degree 13 by
//    Horner's rule; |r| <= ln2/2 makes the truncation term < 5e-18.
//  * log: x = m*2^e with m in [sqrt(1/2), sqrt(2)); log m = 2*atanh(s),
//    s = (m-1)/(m+1), summed as the odd series s + s^3/3 + ... + s^23/23.
//  * 10^y: exp of y*ln10 where the product is formed exactly with Dekker's
//    splitting (no fused multiply-add) and the low part is fed into the
//    reduced argument.
// Accuracy is about one ulp; the tests compare against the C library.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DM_HD __host__ __device__ __forceinline__
#else
#define DM_HD inline
#endif

namespace detmath {

static constexpr double LN2_HI = 0x1.62e42fefa3800p-1;
static constexpr double LN2_LO = 0x1.ef35793c76730p-45;
static constexpr double INV_LN2 = 0x1.71547652b82fep+0;
static constexpr double LN10 = 0x1.26bb1bbb55516p+1;
static constexpr double LN10_LO = -0x1.f48ad494ea3e9p-53;
static constexpr double INV_LN10 = 0x1.bcb7b1526e50ep-2;
static constexpr double SQRT2 = 0x1.6a09e667f3bcdp+0;

DM_HD double bits_to_double(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, sizeof d);
  return d;
#endif
}

DM_HD uint64_t double_to_bits(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, sizeof u);
  return u;
#endif
}

// 2^k for -1022 <= k <= 1023, built from the exponent field.
DM_HD double pow2i(int k) { return bits_to_double((uint64_t)(k + 1023) << 52); }

// e^(hi+lo) where |lo| is tiny compared with |hi|.
DM_HD double exp_hl(double hi, double lo) {
  if (hi != hi) return hi;                         // NaN
  if (hi > 709.782712893384) return bits_to_double(0x7ff0000000000000ull);
  if (hi < -745.2) return 0.0;
  double kd = hi * INV_LN2;
  // round to nearest integer without calling rint (ties away from zero)
  kd = (kd >= 0.0) ? (double)(long long)(kd + 0.5) : (double)(long long)(kd - 0.5);
  int k = (int)kd;
  double r = (hi - kd * LN2_HI) - kd * LN2_LO;
  r = r + lo;
  // Taylor coefficients 1/n!, n = 2..13
  double p = 0x1.6124613a86d09p-33;
  p = p * r + 0x1.1eed8eff8d898p-29;
  p = p * r + 0x1.ae64567f544e4p-26;
  p = p * r + 0x1.27e4fb7789f5cp-22;
  p = p * r + 0x1.71de3a556c734p-19;
  p = p * r + 0x1.a01a01a01a01ap-16;
  p = p * r + 0x1.a01a01a01a01ap-13;
  p = p * r + 0x1.6c16c16c16c17p-10;
  p = p * r + 0x1.1111111111111p-7;
  p = p * r + 0x1.5555555555555p-5;
  p = p * r + 0x1.5555555555555p-3;
  p = p * r + 0x1.0000000000000p-1;
  p = p * r + 1.0;
  p = p * r + 1.0;
  // scale in two steps so results in the subnormal range stay exact-ish
  if (k < -1021) {
    return (p * pow2i(k + 600)) * pow2i(-600);
  }
  if (k > 1023) {
    return (p * pow2i(k - 1)) * 2.0;
  }
  return p * pow2i(k);
}

DM_HD double exp(double x) { return exp_hl(x, 0.0); }

// Natural logarithm for finite x > 0 (returns NaN for x <= 0, inf for inf).
DM_HD double log(double x) {
  if (!(x > 0.0)) {
    if (x == 0.0) return -bits_to_double(0x7ff0000000000000ull);
    return bits_to_double(0x7ff8000000000000ull);
  }
  uint64_t u = double_to_bits(x);
  int e = (int)((u >> 52) & 0x7ff);
  if (e == 0x7ff) return x;                         // inf
  double m;
  if (e == 0) {                                     // subnormal: normalise
    x = x * 0x1p54;
    u = double_to_bits(x);
    e = (int)((u >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  m = bits_to_double((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  if (m > SQRT2) {
    m = m * 0.5;
    e += 1;
  }
  double s = (m - 1.0) / (m + 1.0);
  double z = s * s;
  double q = 0x1.642c8590b2164p-5;  // 1/23
  q = q * z + 0x1.8618618618618p-5; // 1/21
  q = q * z + 0x1.af286bca1af28p-5; // 1/19
  q = q * z + 0x1.e1e1e1e1e1e1ep-5; // 1/17
  q = q * z + 0x1.1111111111111p-4; // 1/15
  q = q * z + 0x1.3b13b13b13b14p-4; // 1/13
  q = q * z + 0x1.745d1745d1746p-4; // 1/11
  q = q * z + 0x1.c71c71c71c71cp-4; // 1/9
  q = q * z + 0x1.2492492492492p-3; // 1/7
  q = q * z + 0x1.999999999999ap-3; // 1/5
  q = q * z + 0x1.5555555555555p-2; // 1/3
  double lm = 2.0 * s + (2.0 * s) * (z * q);
  double ed = (double)e;
  return ed * LN2_HI + (ed * LN2_LO + lm);
}

DM_HD double log10(double x) { return detmath::log(x) * INV_LN10; }

// Exact product a*b = p + e (Dekker / Veltkamp splitting, no FMA).
DM_HD void two_prod(double a, double b, double &p, double &e) {
  const double split = 134217729.0;  // 2^27 + 1
  p = a * b;
  double ca = split * a;
  double ah = ca - (ca - a);
  double al = a - ah;
  double cb = split * b;
  double bh = cb - (cb - b);
  double bl = b - bh;
  e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
}

// 10^y.
DM_HD double exp10(double y) {
  if (y != y) return y;
  if (y > 308.3) return bits_to_double(0x7ff0000000000000ull);
  if (y < -323.7) return 0.0;
  double p, e;
  two_prod(y, LN10, p, e);
  return exp_hl(p, e + y * LN10_LO);
}

// x**y for x >= 0 as exp(y log x) with the functions above: the real powers
// the reference takes of positive quantities (temperatures, rates, column
// terms); 0**y is 0 for y > 0 and +inf for y < 0, as libm gives.
DM_HD double pow(double x, double y) {
  if (x == 0.0) return y > 0.0 ? 0.0 : (y < 0.0 ? bits_to_double(0x7ff0000000000000ull) : 1.0);
  double p, e;
  two_prod(y, detmath::log(x), p, e);
  return exp_hl(p, e);
}

// Fortran intrinsic semantics used by the reference, written once so the
// CPU restatement and the GPU kernels agree on signed zeros:
//   SIGN(a,b) = |a| with the sign bit of b (gfortran follows copysign),
//   MAX(a,b)  = b if b > a else a,  MIN(a,b) = b if b < a else a.
DM_HD double fsign(double a, double b) {
  uint64_t ua = double_to_bits(a) & 0x7fffffffffffffffull;
  uint64_t sb = double_to_bits(b) & 0x8000000000000000ull;
  return bits_to_double(ua | sb);
}
DM_HD double fmax2(double a, double b) { return (b > a) ? b : a; }
DM_HD double fmin2(double a, double b) { return (b < a) ? b : a; }

}  // namespace detmath
