// Checks the FP64 <-> FP32 integer conversions of mhd_conv.cuh (host path of
// the same code the kernels run) against an independent statement of their
// semantics: round to nearest with ties away from zero, |d| < 2^-126 to a
// signed zero, |d| >= 2^128 to a signed infinity, NaN to a quiet NaN with
// its sign; f2d exact for normal floats, subnormals to a signed zero, Inf
// and NaN payloads kept.  Every exponent with random and boundary mantissas
// (the rounding bit and carries), both signs; f2d over a stride of all
// float patterns and the special values.  Exit status 0 when all agree.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
#include "mhd_conv.cuh"
// reference semantics of the conversions, written independently
static uint32_t ref_d2f(uint64_t b) {
  uint32_t sign = (uint32_t)(b >> 63) << 31;
  uint32_t ex = (uint32_t)(b >> 52) & 0x7ff;
  uint64_t m = b & ((1ull << 52) - 1);
  if (ex == 0x7ff && m) return 0x7fc00000u | sign;
  if (ex >= 1023 + 128) return 0x7f800000u | sign;
  if (ex < 1023 - 126) return sign;
  uint32_t r = ((ex - 896) << 23) + (uint32_t)(m >> 29) + (uint32_t)((m >> 28) & 1);
  return r | sign;
}
static uint64_t ref_f2d(uint32_t b) {
  uint64_t sign = (uint64_t)(b >> 31) << 63;
  uint32_t ex = (b >> 23) & 0xff, m = b & 0x7fffff;
  if (ex == 0) return sign;
  if (ex == 0xff) return sign | (0x7ffull << 52) | ((uint64_t)m << 29);
  return sign | ((uint64_t)(ex + 896) << 52) | ((uint64_t)m << 29);
}
int main() {
  std::mt19937_64 rng(12345);
  long bad = 0, n = 0;
  auto chk = [&](uint64_t b) {
    double d; memcpy(&d, &b, 8);
    float f = mhd::d2f_t<MHD_CONV_BRANCH != 0>(d); uint32_t fb; memcpy(&fb, &f, 4);
    if (fb != ref_d2f(b)) { if (bad < 5) printf("d2f %016llx -> %08x ref %08x\n", (unsigned long long)b, fb, ref_d2f(b)); bad++; }
    n++;
  };
  for (int e = 0; e < 2048; e++)
    for (int k = 0; k < 2000; k++) {
      uint64_t m = rng() & ((1ull << 52) - 1);
      if (k < 8) m = (k & 1 ? 0 : (1ull << 52) - 1) ^ ((uint64_t)k << 27);
      if (k == 8) m = 1ull << 28; if (k == 9) m = (1ull << 28) - 1; if (k == 10) m = (1ull << 29) | (1ull << 28);
      chk(((uint64_t)e << 52) | m);
      chk((1ull << 63) | ((uint64_t)e << 52) | m);
    }
  for (uint64_t i = 0; i < (1ull << 32); i += 40009) {   // f2d over a stride of every float pattern
    uint32_t b = (uint32_t)i;
    float f; memcpy(&f, &b, 4);
    double d = mhd::f2d_t<MHD_CONV_BRANCH != 0>(f); uint64_t db; memcpy(&db, &d, 8);
    if (db != ref_f2d(b)) { if (bad < 10) printf("f2d %08x\n", b); bad++; }
    n++;
  }
  for (uint32_t b : {0u, 0x80000000u, 0x00800000u, 0x007fffffu, 0x7f7fffffu, 0x7f800000u, 0xff800000u, 0x7fc00001u, 0x80000001u}) {
    float f; memcpy(&f, &b, 4);
    double d = mhd::f2d_t<MHD_CONV_BRANCH != 0>(f); uint64_t db; memcpy(&db, &d, 8);
    if (db != ref_f2d(b)) { printf("f2d special %08x\n", b); bad++; }
  }
  printf("%ld checked, %ld mismatches\n", n, bad);
  return bad != 0;
}
