// FP64 exp, log and division with fewer FP64-pipe instructions than the CUDA library forms, for
// the FP64 cell-model steps. GB300 issues FP64 arithmetic (and FP64 conversions) at 2 per clock
// per SM, so the plain ten Tusscher and Courtemanche steps are bound by the count of those
// instructions, most of which sit in their exponentials, logarithms and divisions. Measured on a
// GB300 in units of one DFMA's issue cost: exp 14.9 -> exp64 11.7, log 28.7 -> log64 13.8,
// a / b 8.3 -> div64 6.5; the TT2 FP64 step went from 1.03e9 to 1.36e9 cell-steps/s with them
// (and its quotients over shared denominators), Courtemanche's from 1.20e9 to 1.46e9. (The
// O'Hara-Rudy and Tomek FP64 steps, with ~50 exponentials and ~60-95 divisions each, measured 2 %
// slower with all three and 3 % slower with the division and log alone, and keep the library
// forms.)
// Accuracy: exp64 and log64 within 1 ulp of the CUDA functions and of the correctly rounded
// value (equal to it for over 99 % of arguments), div64 equal to the IEEE quotient on every
// sampled operand pair (tests/test_gpu_fp64_math.py checks all three against extended-precision
// host values). Arguments outside the ranges stated below take the library form.
#pragma once

#include <cmath>
#include <cstdint>

#include "cm_common.cuh"
#ifdef __CUDACC__
#include "cm_fp64_tables.h"
#endif

namespace cm {
namespace fp64 {

#ifdef __CUDACC__

// e^x, |x| < 700 (else exp). Tang's table-driven method (P. T. P. Tang, ACM TOMS 15(2), 1989):
// x = (64 m + j) ln2/64 + r with |r| <= ln2/128, e^x = 2^m * 2^(j/64) * e^r, e^r - 1 from its
// Taylor series to r^6 (truncation below 2^-64), 2^(j/64) as a head + tail pair, 2^m applied to
// the exponent field.
__device__ __forceinline__ double exp64(double x) {
  if ((__double2hiint(x) & 0x7fffffff) >= 0x4085e000) return exp(x);  // |x| >= 700, inf, nan
  constexpr double kShift = 0x1.8p52;  // adding it rounds to an integer held in the low word
  const double t = fma(x, k64ByLn2, kShift);
  const int k = __double2loint(t);
  const double kd = t - kShift;
  double r = fma(-kd, kLn2By64Hi, x);  // exact: kd * kLn2By64Hi has at most 53 bits
  r = fma(-kd, kLn2By64Lo, r);
  const int j = k & 63, m = k >> 6;
  double q = fma(r, 1.0 / 720, 1.0 / 120);
  q = fma(q, r, 1.0 / 24);
  q = fma(q, r, 1.0 / 6);
  q = fma(q, r, 0.5);
  const double p = fma(q, r * r, r);  // e^r - 1
  const double th = __ldg(kExp2Hi + j);
  const double y = th + fma(th, p, __ldg(kExp2Lo + j));  // in [0.99, 2.02): 2^m keeps it normal
  return __hiloint2double(__double2hiint(y) + (int)((unsigned int)m << 20), __double2loint(y));
}

// ln x for positive normal finite x (else log). Tang's table-driven method (P. T. P. Tang, ACM
// TOMS 16(4), 1990): x = 2^m y with y in [1, 2), F_j = 1 + j/128 the nearest such point to y,
// ln x = m ln2 + ln F_j + ln(1 + u), u = (y - F_j)/F_j with |u| <= 2^-8 (y - F_j is exact), ln(1+u)
// from its Taylor series to u^7 (truncation below 2^-59 relative).
__device__ __forceinline__ double log64(double x) {
  const int hx = __double2hiint(x);
  if (hx < 0x00100000 || hx >= 0x7ff00000) return log(x);  // zero, negative, subnormal, inf, nan
  const int m = (hx >> 20) - 1023;
  const int fr = hx & 0x000fffff;
  const int j = ((fr >> 12) + 1) >> 1;  // leading 8 fraction bits, rounded to 7: j in [0, 128]
  const double y = __hiloint2double(fr | 0x3ff00000, __double2loint(x));
  const double F = __hiloint2double(0x3ff00000 + (j << 13), 0);  // j = 128 carries into F = 2
  const double u = (y - F) * __ldg(kLogInvF + j);
  double q = fma(u, 1.0 / 7, -1.0 / 6);
  q = fma(q, u, 0.2);
  q = fma(q, u, -0.25);
  q = fma(q, u, 1.0 / 3);
  q = fma(q, u, -0.5);
  const double p = fma(q, u * u, u);  // ln(1 + u)
  const double md = (double)m;
  // exact: both heads are multiples of 2^-42 and |m| <= 1023, so one rounding (the last) remains
  const double a = fma(md, kLn2Hi, __ldg(kLogFHi + j));
  const double b = fma(md, kLn2Lo, __ldg(kLogFLo + j)) + p;
  return a + b;
}

// a / b. Newton-Raphson from the approximate reciprocal instruction (relative error about
// 2^-20): one cubic step r1 = r0 + r0 (e + e^2), e = 1 - b r0 (error below 2^-60 before
// rounding), q1 = a r1, then one residual correction q = q1 + r1 (a - b q1) (Markstein's
// correction, as in P. Markstein, IA-64 and Elementary Functions, 2000). Operands with b zero,
// subnormal, huge, inf or nan, a zero, subnormal, inf or nan, or a quotient near the overflow or
// underflow range take the IEEE division.
__device__ __forceinline__ double div64(double a, double b) {
  const int ea = (__double2hiint(a) >> 20) & 0x7ff, eb = (__double2hiint(b) >> 20) & 0x7ff;
  const int d = ea - eb;
  if (ea == 0 || ea == 0x7ff || eb < 2 || eb > 2044 || d > 1000 || d < -1000) return a / b;
  double r0;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(b));
  const double e = fma(-b, r0, 1.0);
  const double r1 = fma(fma(e, e, e), r0, r0);
  const double q1 = a * r1;
  return fma(fma(-b, q1, a), r1, q1);
}

#endif  // __CUDACC__

// The entry points for code compiled for host and device: the forms above on the device, the
// library forms on the host.
CM_HD double dexp(double x) {
#ifdef __CUDA_ARCH__
  return exp64(x);
#else
  return std::exp(x);
#endif
}

CM_HD double dlog(double x) {
#ifdef __CUDA_ARCH__
  return log64(x);
#else
  return std::log(x);
#endif
}

CM_HD double ddiv(double a, double b) {
#ifdef __CUDA_ARCH__
  return div64(a, b);
#else
  return a / b;
#endif
}

}  // namespace fp64
}  // namespace cm
