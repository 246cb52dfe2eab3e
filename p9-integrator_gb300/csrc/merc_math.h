// merc_math.h - deterministic binary64 elementary functions for host and device.
//
// The element-based Kepler drift of the reference (cartesian -> elements ->
// cartesian every step) amplifies any 1-ulp change of sin, cos, acos, atan2,
// rsqrt or a norm by ~1e6 within 100 steps on near-circular orbits.  To make
// the GPU integrator and its CPU check agree bit for bit, both evaluate these
// functions with the code below: only IEEE +, -, *, /, sqrt and fma (all
// correctly rounded on both CUDA and the host when a*b+c is not contracted:
// nvcc -fmad=false, gcc -ffp-contract=off) plus exact bit manipulation.
//
// Methods (accuracy ~1 ulp, not correctly rounded; see tests for measured
// bounds against a 64-bit-mantissa reference):
//  sincos  Cody & Waite three-constant reduction by pi/2 with fma, Taylor
//          polynomials of degree 17 (sin) and 18 (cos) on [-pi/4, pi/4].
//  atan2   reduction to t = min/max in [0,1], t = c + d with c = k/16 from a
//          double-double table of atan(k/16), atan((t-c)/(1+tc)) by Taylor
//          series to degree 11, then octant and sign fix-up (C99 semantics
//          for zeros and infinities).
//  acos    atan2(sqrt((1-x)(1+x)), x).
//  exp     Cody & Waite reduction by ln 2 (double-double), Taylor degree 13,
//          exponent scaling by bit manipulation; sinh (Taylor for |x|<0.5) and
//          cosh from it.
//  log     exponent split to m in [sqrt(1/2), sqrt(2)), 2 atanh((m-1)/(m+1))
//          by Taylor series to degree 21, plus k ln 2 (double-double).
//  cbrt    exponent split x = 2^(3q) w, w in [1, 8), quadratic seed, three
//          Halley steps y <- y (y^3 + 2w) / (2y^3 + w).
// Constants come from merc_math_tables.h, generated with mpmath.
#pragma once
#include <stdint.h>
#include <string.h>

#include "merc_math_tables.h"

#if defined(__CUDACC__)
#define MERC_HD __host__ __device__ __forceinline__
#else
#define MERC_HD static inline
#include <math.h>
#endif

namespace mm {

#if defined(__CUDACC__)
__constant__ double kAtanHi[17] = MERC_ATAN_TABLE_HI;
__constant__ double kAtanLo[17] = MERC_ATAN_TABLE_LO;
#endif
static const double kAtanHiHost[17] = MERC_ATAN_TABLE_HI;
static const double kAtanLoHost[17] = MERC_ATAN_TABLE_LO;

MERC_HD uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
MERC_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}
MERC_HD double fma_(double a, double b, double c) { return fma(a, b, c); }
MERC_HD double sqrt_(double x) { return sqrt(x); }
MERC_HD double abs_(double x) { return from_bits(bits(x) & 0x7fffffffffffffffull); }
MERC_HD double copysign_(double x, double s) {
  return from_bits((bits(x) & 0x7fffffffffffffffull) | (bits(s) & 0x8000000000000000ull));
}
MERC_HD bool isnan_(double x) { return (bits(x) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull; }
MERC_HD bool isinf_(double x) { return (bits(x) & 0x7fffffffffffffffull) == 0x7ff0000000000000ull; }
MERC_HD bool isfinite_(double x) { return (bits(x) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull; }
// round to nearest integer value for |x| < 2^51
MERC_HD double rint_(double x) {
  const double big = 6755399441055744.0;  // 1.5 * 2^52
  double t = x + big;
  return t - big;
}
// x * 2^k for the exponent range used here (result normal or inf/zero)
MERC_HD double ldexp_(double x, int k) {
  // split the scale in two factors so each is a normal power of two
  int k1 = k / 2, k2 = k - k1;
  double s1 = from_bits((uint64_t)(k1 + 1023) << 52);
  double s2 = from_bits((uint64_t)(k2 + 1023) << 52);
  return (x * s1) * s2;
}

// ---- sin, cos ----------------------------------------------------------
MERC_HD void sincos(double x, double* s, double* c) {
  if (!isfinite_(x)) {
    *s = x - x;
    *c = x - x;
    return;
  }
  double k = rint_(x * MERC_2_OVER_PI);
  double r = fma_(-k, MERC_PIO2_1, x);
  r = fma_(-k, MERC_PIO2_2, r);
  r = fma_(-k, MERC_PIO2_3, r);
  int q = (int)((int64_t)k & 3);
  double z = r * r;
  // sin r = r + r z (-1/3! + z (1/5! - ...)), degree 17
  double ps = fma_(z, 1.0 / 355687428096000.0, -1.0 / 1307674368000.0);
  ps = fma_(z, ps, 1.0 / 6227020800.0);
  ps = fma_(z, ps, -1.0 / 39916800.0);
  ps = fma_(z, ps, 1.0 / 362880.0);
  ps = fma_(z, ps, -1.0 / 5040.0);
  ps = fma_(z, ps, 1.0 / 120.0);
  ps = fma_(z, ps, -1.0 / 6.0);
  double sn = fma_(r * z, ps, r);
  // cos r = 1 + z (-1/2 + z (1/4! - ...)), degree 18
  double pc = fma_(z, -1.0 / 6402373705728000.0, 1.0 / 20922789888000.0);
  pc = fma_(z, pc, -1.0 / 87178291200.0);
  pc = fma_(z, pc, 1.0 / 479001600.0);
  pc = fma_(z, pc, -1.0 / 3628800.0);
  pc = fma_(z, pc, 1.0 / 40320.0);
  pc = fma_(z, pc, -1.0 / 720.0);
  pc = fma_(z, pc, 1.0 / 24.0);
  pc = fma_(z, pc, -0.5);
  double cs = fma_(z, pc, 1.0);
  double so, co;
  switch (q) {
    case 0: so = sn; co = cs; break;
    case 1: so = cs; co = -sn; break;
    case 2: so = -sn; co = -cs; break;
    default: so = -cs; co = sn; break;
  }
  *s = so;
  *c = co;
}
MERC_HD double sin(double x) {
  double s, c;
  sincos(x, &s, &c);
  return s;
}
MERC_HD double cos(double x) {
  double s, c;
  sincos(x, &s, &c);
  return c;
}

// ---- atan2 ---------------------------------------------------------------
// atan(t) for 0 <= t <= 1 as hi + lo (lo small)
MERC_HD double atan01(double t, double* lo) {
#if defined(__CUDA_ARCH__)
  const double* thi = kAtanHi;
  const double* tlo = kAtanLo;
#else
  const double* thi = kAtanHiHost;
  const double* tlo = kAtanLoHost;
#endif
  int k = (int)rint_(t * 16.0);
  double c = (double)k * 0.0625;
  double u = (t - c) / fma_(t, c, 1.0);
  double z = u * u;
  double p = fma_(z, -1.0 / 11.0, 1.0 / 9.0);
  p = fma_(z, p, -1.0 / 7.0);
  p = fma_(z, p, 1.0 / 5.0);
  p = fma_(z, p, -1.0 / 3.0);
  *lo = tlo[k] + fma_(u * z, p, u);
  return thi[k];
}

MERC_HD double atan2(double y, double x) {
  if (isnan_(x) || isnan_(y)) return x + y;
  double ax = abs_(x), ay = abs_(y);
  bool xneg = (bits(x) >> 63) != 0;
  double res;
  if (isinf_(ax) || isinf_(ay)) {
    if (isinf_(ax) && isinf_(ay))
      res = xneg ? 3.0 * MERC_PIO2_HI * 0.5 : MERC_PIO2_HI * 0.5;  // 3pi/4 or pi/4
    else if (isinf_(ax))
      res = xneg ? MERC_PI_HI : 0.0;
    else
      res = MERC_PIO2_HI;
    return copysign_(res, y);
  }
  if (ay == 0.0) {
    res = xneg ? MERC_PI_HI : 0.0;
    return copysign_(res, y);
  }
  if (ax == 0.0) return copysign_(MERC_PIO2_HI, y);
  bool swap = ay > ax;
  double t = swap ? ax / ay : ay / ax;
  double lo;
  double hi = atan01(t, &lo);
  double a;
  if (swap) {  // pi/2 - atan(t)
    a = (MERC_PIO2_HI - hi) + (MERC_PIO2_LO - lo);
  } else {
    a = hi + lo;
  }
  if (xneg) a = (MERC_PI_HI - a) + MERC_PI_LO;
  return copysign_(a, y);
}

MERC_HD double acos(double x) {
  if (isnan_(x)) return x;
  if (abs_(x) > 1.0) return (x - x) / (x - x);  // NaN
  double s = sqrt_((1.0 - x) * (1.0 + x));
  return atan2(s, x);
}

// ---- exp, sinh, cosh -------------------------------------------------------
MERC_HD double exp(double x) {
  if (isnan_(x)) return x;
  if (x > 709.78) return from_bits(0x7ff0000000000000ull);
  if (x < -745.2) return 0.0;
  double k = rint_(x * MERC_INV_LN2);
  double r = fma_(-k, MERC_LN2_HI, x);
  r = fma_(-k, MERC_LN2_LO, r);
  double p = fma_(r, 1.0 / 6227020800.0, 1.0 / 479001600.0);
  p = fma_(r, p, 1.0 / 39916800.0);
  p = fma_(r, p, 1.0 / 3628800.0);
  p = fma_(r, p, 1.0 / 362880.0);
  p = fma_(r, p, 1.0 / 40320.0);
  p = fma_(r, p, 1.0 / 5040.0);
  p = fma_(r, p, 1.0 / 720.0);
  p = fma_(r, p, 1.0 / 120.0);
  p = fma_(r, p, 1.0 / 24.0);
  p = fma_(r, p, 1.0 / 6.0);
  p = fma_(r, p, 0.5);
  p = fma_(r * r, p, r);
  double er = 1.0 + p;
  return ldexp_(er, (int)k);
}

MERC_HD double sinh(double x) {
  double ax = abs_(x);
  if (ax < 0.5) {
    double z = x * x;
    double p = fma_(z, 1.0 / 121645100408832000.0, 1.0 / 355687428096000.0);
    p = fma_(z, p, 1.0 / 1307674368000.0);
    p = fma_(z, p, 1.0 / 6227020800.0);
    p = fma_(z, p, 1.0 / 39916800.0);
    p = fma_(z, p, 1.0 / 362880.0);
    p = fma_(z, p, 1.0 / 5040.0);
    p = fma_(z, p, 1.0 / 120.0);
    p = fma_(z, p, 1.0 / 6.0);
    return fma_(x * z, p, x);
  }
  if (!isfinite_(x)) return x;
  if (ax > 710.0) return copysign_(from_bits(0x7ff0000000000000ull), x);
  double e = exp(ax);
  double r = 0.5 * (e - 1.0 / e);
  return copysign_(r, x);
}

MERC_HD double cosh(double x) {
  double ax = abs_(x);
  if (isnan_(x)) return x;
  if (ax > 710.0) return from_bits(0x7ff0000000000000ull);
  double e = exp(ax);
  return 0.5 * (e + 1.0 / e);
}

// ---- log -------------------------------------------------------------------
MERC_HD double log(double x) {
  if (isnan_(x)) return x;
  if (x < 0.0) return (x - x) / (x - x);
  if (x == 0.0) return -from_bits(0x7ff0000000000000ull);
  if (isinf_(x)) return x;
  int k = 0;
  if (x < 2.2250738585072014e-308) {  // subnormal
    x *= 18014398509481984.0;       // 2^54
    k = -54;
  }
  uint64_t u = bits(x);
  int e = (int)((u >> 52) & 0x7ff) - 1023;
  double m = from_bits((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull);  // [1, 2)
  if (m > 1.4142135623730951) {
    m *= 0.5;
    e += 1;
  }
  k += e;
  double f = (m - 1.0) / (m + 1.0);
  double z = f * f;
  double p = fma_(z, 1.0 / 21.0, 1.0 / 19.0);
  p = fma_(z, p, 1.0 / 17.0);
  p = fma_(z, p, 1.0 / 15.0);
  p = fma_(z, p, 1.0 / 13.0);
  p = fma_(z, p, 1.0 / 11.0);
  p = fma_(z, p, 1.0 / 9.0);
  p = fma_(z, p, 1.0 / 7.0);
  p = fma_(z, p, 1.0 / 5.0);
  p = fma_(z, p, 1.0 / 3.0);
  double lm = fma_(2.0 * f * z, p, 2.0 * f);
  double dk = (double)k;
  return fma_(dk, MERC_LN2_HI, fma_(dk, MERC_LN2_LO, lm));
}

// ---- cbrt ------------------------------------------------------------------
MERC_HD double cbrt(double x) {
  if (x == 0.0 || !isfinite_(x)) return x;
  double ax = abs_(x);
  int k = 0;
  if (ax < 2.2250738585072014e-308) {
    ax *= 18014398509481984.0;  // 2^54
    k = -54;
  }
  uint64_t u = bits(ax);
  int e = (int)((u >> 52) & 0x7ff) - 1023 + k;
  double m = from_bits((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull);  // [1, 2)
  int q = e >= 0 ? e / 3 : -((-e + 2) / 3);
  int rr = e - 3 * q;  // 0, 1, 2
  double w = m * (double)(1 << rr);  // [1, 8)
  // seed: least-squares quadratic of w^(1/3) on [1, 8] (relative error < 3.9e-02)
  double y = fma_(w, fma_(w, -0.0127267, 0.24779181), 0.80167772);
  for (int it = 0; it < 3; it++) {
    double y3 = y * y * y;
    y = y * (fma_(2.0, w, y3) / fma_(2.0, y3, w));
  }
  return copysign_(ldexp_(y, q), x);
}

}  // namespace mm
