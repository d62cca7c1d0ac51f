// rg_math.cuh — deterministic FP64 exp and log for the parity path (host and device).
//
// The Dupire calibration amplifies last-ulp differences between elementary-function libraries
// by about 1e6, so the FP64 parity kernel, the FP64 calibration kernel and the host-built
// discount tables all use these two functions instead of the platform's.  They are built only
// from IEEE-754 +, -, *, / and exact power-of-two scaling, evaluated in a fixed order; compiled
// without FMA contraction they return the same bits on the CPU and on the GPU.
//
// exp: Cody–Waite additive reduction x = k·ln2 + r with ln2 split into a 29-bit head (k·head is
//      exact) and a tail, |r| <= ln2/2, then the degree-13 Taylor polynomial of e^r by Horner's
//      rule (truncation error below 0.05 ulp) and exact scaling by 2^k.
// log: x = 2^e·m with m in (sqrt(1/2), sqrt(2)], log m = 2·artanh(s), s = (m-1)/(m+1), using the
//      artanh series through s^23 (|s| <= 0.1716), then e·ln2 added in head/tail form.
// Coefficients are the correctly rounded values of 1/n! and 1/(2k+1), written as hex literals.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define RG_HD __host__ __device__ __forceinline__
#else
#define RG_HD static inline
#endif

RG_HD uint64_t rg_bits64(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

RG_HD double rg_from_bits64(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

// Round-to-nearest multiply and add that are never fused, whatever the compile flags.
#if defined(__CUDA_ARCH__)
#define RG_MUL(a, b) __dmul_rn((a), (b))
#define RG_ADD(a, b) __dadd_rn((a), (b))
#else
#define RG_MUL(a, b) ((a) * (b))
#define RG_ADD(a, b) ((a) + (b))
#endif

// 2^k for -1022 <= k <= 1023, exact.
RG_HD double rg_pow2(int k) { return rg_from_bits64((uint64_t)(k + 1023) << 52); }

RG_HD double rg_exp64(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return INFINITY;
  if (x < -745.1332191019412) return 0.0;
  const double ln2_hi = 0x1.62e42ffp-1, ln2_lo = -0x1.718432a1b0e26p-35;
  const double inv_ln2 = 0x1.71547652b82fep+0;
  const double k = floor(RG_ADD(RG_MUL(x, inv_ln2), 0.5));
  const double r = RG_ADD(RG_ADD(x, -RG_MUL(k, ln2_hi)), -RG_MUL(k, ln2_lo));
  double p = 0x1.6124613a86d09p-33;             // 1/13!
  p = RG_ADD(RG_MUL(p, r), 0x1.1eed8eff8d898p-29);            // 1/12!
  p = RG_ADD(RG_MUL(p, r), 0x1.ae64567f544e4p-26);            // 1/11!
  p = RG_ADD(RG_MUL(p, r), 0x1.27e4fb7789f5cp-22);            // 1/10!
  p = RG_ADD(RG_MUL(p, r), 0x1.71de3a556c734p-19);            // 1/9!
  p = RG_ADD(RG_MUL(p, r), 0x1.a01a01a01a01ap-16);            // 1/8!
  p = RG_ADD(RG_MUL(p, r), 0x1.a01a01a01a01ap-13);            // 1/7!
  p = RG_ADD(RG_MUL(p, r), 0x1.6c16c16c16c17p-10);            // 1/6!
  p = RG_ADD(RG_MUL(p, r), 0x1.1111111111111p-7);             // 1/5!
  p = RG_ADD(RG_MUL(p, r), 0x1.5555555555555p-5);             // 1/4!
  p = RG_ADD(RG_MUL(p, r), 0x1.5555555555555p-3);             // 1/3!
  p = RG_ADD(RG_MUL(p, r), 0.5);
  p = RG_ADD(RG_MUL(p, r), 1.0);
  p = RG_ADD(RG_MUL(p, r), 1.0);
  const int ki = (int)k;
  if (ki >= -1022) {
    if (ki <= 1023) return p * rg_pow2(ki);
    return (p * rg_pow2(1023)) * rg_pow2(ki - 1023);
  }
  return (p * rg_pow2(ki + 54)) * rg_pow2(-54);
}

RG_HD double rg_log64(double x) {
  if (x != x) return x;
  if (x < 0.0) return NAN;
  if (x == 0.0) return -INFINITY;
  if (x == INFINITY) return x;
  int e = 0;
  if (x < 0x1p-1022) {  // subnormal: scale into the normal range
    x = x * 0x1p54;
    e = -54;
  }
  const uint64_t b = rg_bits64(x);
  e += (int)((b >> 52) & 0x7ff) - 1023;
  double m = rg_from_bits64((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
  if (m > 0x1.6a09e667f3bcdp+0) {  // sqrt(2)
    m = m * 0.5;
    e += 1;
  }
  const double f = m - 1.0;
  const double s = f / RG_ADD(2.0, f);
  const double z = RG_MUL(s, s);
  double R = 0x1.642c8590b2164p-5;              // 1/23
  R = RG_ADD(RG_MUL(R, z), 0x1.8618618618618p-5);             // 1/21
  R = RG_ADD(RG_MUL(R, z), 0x1.af286bca1af28p-5);             // 1/19
  R = RG_ADD(RG_MUL(R, z), 0x1.e1e1e1e1e1e1ep-5);             // 1/17
  R = RG_ADD(RG_MUL(R, z), 0x1.1111111111111p-4);             // 1/15
  R = RG_ADD(RG_MUL(R, z), 0x1.3b13b13b13b14p-4);             // 1/13
  R = RG_ADD(RG_MUL(R, z), 0x1.745d1745d1746p-4);             // 1/11
  R = RG_ADD(RG_MUL(R, z), 0x1.c71c71c71c71cp-4);             // 1/9
  R = RG_ADD(RG_MUL(R, z), 0x1.2492492492492p-3);             // 1/7
  R = RG_ADD(RG_MUL(R, z), 0x1.999999999999ap-3);             // 1/5
  R = RG_ADD(RG_MUL(R, z), 0x1.5555555555555p-2);             // 1/3
  R = RG_MUL(R, z);
  const double lm = RG_MUL(2.0, RG_ADD(s, RG_MUL(s, R)));
  const double ed = (double)e;
  return RG_ADD(RG_MUL(ed, 0x1.62e42ffp-1), RG_ADD(lm, RG_MUL(ed, -0x1.718432a1b0e26p-35)));
}
