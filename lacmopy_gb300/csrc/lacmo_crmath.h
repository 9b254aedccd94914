/*
 * Correctly-rounded double-precision log and pow for the bit-exact collision
 * path, usable from host and device code.
 *
 * Why: the collision step's outcome bits depend on the droplet radius
 * R = (3/(4 pi) m / rho)^(1/3) and on the kernel bin int((log R - a)/b + 0.5).
 * CUDA's pow/log are faithfully but not correctly rounded, so they disagree
 * with any CPU libm in the last bit on a sizeable fraction of inputs.  A
 * correctly-rounded result is platform independent: the GPU kernels and the
 * CPU oracle compile this same header and agree bit for bit.
 *
 * Method (written for this project from textbook techniques):
 *   log: x = 2^E m with m in [sqrt(1/2), sqrt(2)); a 512-entry table gives
 *        r ~ 1/m with 9 significant bits, so t = m r - 1 is exact (one fma)
 *        and |t| < 2^-7.9; log x = E ln2 - log r + log1p(t), log1p by its
 *        Taylor series to degree 13, the terms up to t^6 in double-double.
 *   exp: k = round(P 256/ln2), r = P - k ln2/256 in double-double
 *        (|r| <= ln2/512), exp(r) by its Taylor series to degree 9 (terms up
 *        to r^4 in double-double), times 2^(k/256) from a double-double table.
 *   pow: exp(y * log x) with log x kept in double-double.
 * The double-double result (relative error below about 2^-97) is rounded to
 * the nearest double.  This is the correctly-rounded value unless the exact
 * value lies within 2^-90 (relative) of a rounding midpoint; the *_checked
 * variants report such hard cases, which are vanishingly rare.
 * Constants and tables come from gen_crmath_tables.py (mpmath).
 *
 * Translation units that use this header must not contract a*b+c into fma
 * (nvcc -fmad=false, gcc -ffp-contract=off): the explicit fma() calls are the
 * only fused operations, so host and device round identically.
 */
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "lacmo_crmath_tables.h"

#if defined(__CUDACC__)
#define LACMO_HD __host__ __device__ __forceinline__
#else
#define LACMO_HD static inline
#endif

static const double lacmo_cr_log_r_h[512] = {LACMO_CR_LOG_R_VALUES};
static const double lacmo_cr_log_mlr_hi_h[512] = {LACMO_CR_LOG_MLR_HI_VALUES};
static const double lacmo_cr_log_mlr_lo_h[512] = {LACMO_CR_LOG_MLR_LO_VALUES};
static const double lacmo_cr_exp_hi_h[256] = {LACMO_CR_EXP_HI_VALUES};
static const double lacmo_cr_exp_lo_h[256] = {LACMO_CR_EXP_LO_VALUES};
#if defined(__CUDACC__)
static __device__ const double lacmo_cr_log_r_d[512] = {LACMO_CR_LOG_R_VALUES};
static __device__ const double lacmo_cr_log_mlr_hi_d[512] = {LACMO_CR_LOG_MLR_HI_VALUES};
static __device__ const double lacmo_cr_log_mlr_lo_d[512] = {LACMO_CR_LOG_MLR_LO_VALUES};
static __device__ const double lacmo_cr_exp_hi_d[256] = {LACMO_CR_EXP_HI_VALUES};
static __device__ const double lacmo_cr_exp_lo_d[256] = {LACMO_CR_EXP_LO_VALUES};
#endif
#if defined(__CUDA_ARCH__)
#define LACMO_CRT(name) (name##_d)
#define LACMO_FMA(a, b, c) __fma_rn((a), (b), (c))
#else
#define LACMO_CRT(name) (name##_h)
#define LACMO_FMA(a, b, c) fma((a), (b), (c))
#endif

typedef struct { double hi, lo; } lacmo_dd;

LACMO_HD uint64_t lacmo_as_u64(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u; memcpy(&u, &x, 8); return u;
#endif
}
LACMO_HD double lacmo_as_f64(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x; memcpy(&x, &u, 8); return x;
#endif
}
LACMO_HD lacmo_dd lacmo_dd_make(double h, double l) { lacmo_dd r; r.hi = h; r.lo = l; return r; }
LACMO_HD lacmo_dd lacmo_two_sum(double a, double b) {
  double s = a + b; double bb = s - a;
  return lacmo_dd_make(s, (a - (s - bb)) + (b - bb));
}
LACMO_HD lacmo_dd lacmo_fast_two_sum(double a, double b) {
  double s = a + b;
  return lacmo_dd_make(s, b - (s - a));
}
LACMO_HD lacmo_dd lacmo_two_prod(double a, double b) {
  double p = a * b;
  return lacmo_dd_make(p, LACMO_FMA(a, b, -p));
}
LACMO_HD lacmo_dd lacmo_dd_add(lacmo_dd a, lacmo_dd b) {
  lacmo_dd s = lacmo_two_sum(a.hi, b.hi);
  lacmo_dd t = lacmo_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = lacmo_fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return lacmo_fast_two_sum(s.hi, s.lo);
}
LACMO_HD lacmo_dd lacmo_dd_add_d(lacmo_dd a, double b) {
  lacmo_dd s = lacmo_two_sum(a.hi, b);
  s.lo += a.lo;
  return lacmo_fast_two_sum(s.hi, s.lo);
}
LACMO_HD lacmo_dd lacmo_dd_mul(lacmo_dd a, lacmo_dd b) {
  lacmo_dd p = lacmo_two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return lacmo_fast_two_sum(p.hi, p.lo);
}
LACMO_HD lacmo_dd lacmo_dd_mul_d(lacmo_dd a, double b) {
  lacmo_dd p = lacmo_two_prod(a.hi, b);
  p.lo += a.lo * b;
  return lacmo_fast_two_sum(p.hi, p.lo);
}
LACMO_HD lacmo_dd lacmo_dd_scale(lacmo_dd a, double s) { return lacmo_dd_make(a.hi * s, a.lo * s); }

/* log(x) as a double-double for positive finite x */
LACMO_HD lacmo_dd lacmo_cr_log_dd(double x) {
  uint64_t bits = lacmo_as_u64(x);
  int64_t E = (int64_t)((bits >> 52) & 0x7ff);
  if (E == 0) {                                  /* subnormal: scale up */
    x *= 0x1p54;
    bits = lacmo_as_u64(x);
    E = (int64_t)((bits >> 52) & 0x7ff) - 54;
  }
  E -= 1023;
  double m = lacmo_as_f64((bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
  if (m >= 0x1.6a09e667f3bcdp+0) { m *= 0.5; E += 1; }
  int idx = (int)((lacmo_as_u64(m) >> 44) & 0x1ff);
  double r = LACMO_CRT(lacmo_cr_log_r)[idx];
  double t = LACMO_FMA(m, r, -1.0);              /* exact */
  /* log1p(t): terms t^7..t^13 in double, t^1..t^6 in double-double */
  double q = LACMO_CR_INV13_HI;
  q = q * -t + LACMO_CR_INV12_HI;
  q = q * -t + LACMO_CR_INV11_HI;
  q = q * -t + LACMO_CR_INV10_HI;
  q = q * -t + LACMO_CR_INV9_HI;
  q = q * -t + LACMO_CR_INV8_HI;
  q = q * -t + LACMO_CR_INV7_HI;
  lacmo_dd t2 = lacmo_two_prod(t, t);
  lacmo_dd t3 = lacmo_dd_mul_d(t2, t);
  lacmo_dd t4 = lacmo_dd_mul(t2, t2);
  lacmo_dd t5 = lacmo_dd_mul_d(t4, t);
  lacmo_dd t6 = lacmo_dd_mul(t3, t3);
  double t7q = (t6.hi * t) * q;
  lacmo_dd acc = lacmo_dd_mul(t6, lacmo_dd_make(-LACMO_CR_INV6_HI, -LACMO_CR_INV6_LO));
  acc = lacmo_dd_add_d(acc, t7q);
  acc = lacmo_dd_add(acc, lacmo_dd_mul(t5, lacmo_dd_make(LACMO_CR_INV5_HI, LACMO_CR_INV5_LO)));
  acc = lacmo_dd_add(acc, lacmo_dd_scale(t4, -0.25));
  acc = lacmo_dd_add(acc, lacmo_dd_mul(t3, lacmo_dd_make(LACMO_CR_INV3_HI, LACMO_CR_INV3_LO)));
  acc = lacmo_dd_add(acc, lacmo_dd_scale(t2, -0.5));
  acc = lacmo_dd_add_d(acc, t);
  lacmo_dd lm = lacmo_dd_add(lacmo_dd_make(LACMO_CRT(lacmo_cr_log_mlr_hi)[idx],
                                           LACMO_CRT(lacmo_cr_log_mlr_lo)[idx]), acc);
  if (E == 0) return lm;
  double Ed = (double)E;
  lacmo_dd em = lacmo_two_prod(Ed, LACMO_CR_LN2_MID);
  lacmo_dd el = lacmo_fast_two_sum(Ed * LACMO_CR_LN2_HI, em.hi);   /* E*HI exact */
  el.lo += em.lo + Ed * LACMO_CR_LN2_LO;
  el = lacmo_fast_two_sum(el.hi, el.lo);
  return lacmo_dd_add(el, lm);
}

/* exp(p) as a double-double for |p.hi| < 708 */
LACMO_HD lacmo_dd lacmo_cr_exp_dd(lacmo_dd p) {
  double kf = rint(p.hi * LACMO_CR_INV_LN2_256);
  int64_t k = (int64_t)kf;
  double a = p.hi - kf * LACMO_CR_LN2_256_HI;              /* exact */
  lacmo_dd km = lacmo_two_prod(kf, LACMO_CR_LN2_256_MID);
  lacmo_dd r = lacmo_dd_add(lacmo_dd_make(a, 0.0), lacmo_dd_make(-km.hi, -km.lo));
  r = lacmo_dd_add_d(r, -kf * LACMO_CR_LN2_256_LO);
  r = lacmo_dd_add_d(r, p.lo);
  lacmo_dd r2 = lacmo_dd_mul(r, r);
  lacmo_dd r3 = lacmo_dd_mul(r2, r);
  lacmo_dd r4 = lacmo_dd_mul(r2, r2);
  double rh = r.hi;
  double tail = LACMO_CR_INVF9_HI;
  tail = tail * rh + LACMO_CR_INVF8_HI;
  tail = tail * rh + LACMO_CR_INVF7_HI;
  tail = tail * rh + LACMO_CR_INVF6_HI;
  tail = tail * rh + LACMO_CR_INVF5_HI;
  tail = (r4.hi * rh) * tail;
  lacmo_dd s = lacmo_dd_mul(r4, lacmo_dd_make(LACMO_CR_INVF4_HI, LACMO_CR_INVF4_LO));
  s = lacmo_dd_add_d(s, tail);
  s = lacmo_dd_add(s, lacmo_dd_mul(r3, lacmo_dd_make(LACMO_CR_INVF3_HI, LACMO_CR_INVF3_LO)));
  s = lacmo_dd_add(s, lacmo_dd_scale(r2, 0.5));
  s = lacmo_dd_add(s, r);
  s = lacmo_dd_add_d(s, 1.0);
  int64_t j = k & 255;
  int64_t qe = (k - j) / 256;
  lacmo_dd res = lacmo_dd_mul(lacmo_dd_make(LACMO_CRT(lacmo_cr_exp_hi)[j],
                                            LACMO_CRT(lacmo_cr_exp_lo)[j]), s);
  double sc = lacmo_as_f64((uint64_t)(qe + 1023) << 52);   /* |qe| < 1022 */
  return lacmo_dd_scale(res, sc);
}

/* Round a double-double to double; *hard = 1 when the value is so close to a
   rounding midpoint that a 2^-90 relative error could change the result. */
LACMO_HD double lacmo_cr_round(lacmo_dd v, int* hard) {
  lacmo_dd s = lacmo_fast_two_sum(v.hi, v.lo);
  double h = s.hi, l = s.lo;
  if (hard) {
    *hard = 0;
    if (l != 0.0 && h != 0.0) {
      double ah = fabs(h);
      uint64_t b = lacmo_as_u64(ah);
      int64_t ex = (int64_t)((b >> 52) & 0x7ff);
      if (ex > 53) {
        double ulp = lacmo_as_f64((uint64_t)(ex - 52) << 52);
        int toward_smaller = ((l < 0) != (h < 0));
        if (toward_smaller && (b & 0x000fffffffffffffULL) == 0) ulp *= 0.5;
        if (fabs(fabs(l) - 0.5 * ulp) <= 0x1p-90 * ah) *hard = 1;
      }
    }
  }
  return h;
}

LACMO_HD double lacmo_cr_log_checked(double x, int* hard) {
  if (hard) *hard = 0;
  if (isnan(x)) return x + x;
  if (x < 0.0) return NAN;
  if (x == 0.0) return -INFINITY;
  if (isinf(x)) return x;
  if (x == 1.0) return 0.0;
  return lacmo_cr_round(lacmo_cr_log_dd(x), hard);
}
LACMO_HD double lacmo_cr_log(double x) { return lacmo_cr_log_checked(x, 0); }

/* x^y for x >= 0 (x < 0 gives NaN, as for a non-integer exponent) */
LACMO_HD double lacmo_cr_pow_checked(double x, double y, int* hard) {
  if (hard) *hard = 0;
  if (y == 0.0 || x == 1.0) return 1.0;
  if (isnan(x) || isnan(y)) return x + y;
  if (x < 0.0) return NAN;
  if (x == 0.0) return y > 0.0 ? 0.0 : INFINITY;
  if (isinf(x)) return y > 0.0 ? INFINITY : 0.0;
  lacmo_dd L = lacmo_cr_log_dd(x);
  lacmo_dd P = lacmo_two_prod(y, L.hi);
  P.lo += y * L.lo;
  P = lacmo_fast_two_sum(P.hi, P.lo);
  if (P.hi > 709.0) return INFINITY;
  if (P.hi < -708.0) return 0.0;
  return lacmo_cr_round(lacmo_cr_exp_dd(P), hard);
}
LACMO_HD double lacmo_cr_pow(double x, double y) { return lacmo_cr_pow_checked(x, y, 0); }
