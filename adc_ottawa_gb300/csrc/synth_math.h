// Deterministic exp and log for the synthetic-system generator.
//
// Both are written from their series expansions with IEEE basic operations
// only, so that x86-64 and aarch64 hosts produce the same bits (the compiler
// must not contract a*b+c into an FMA: build with -ffp-contract=off).
// Accuracy is a few ulp, ample for a random-number generator.
#pragma once
#include <cmath>

namespace adcsynth {

inline double sqrt_rn(double x) { return std::sqrt(x); }  // IEEE correctly rounded

// ln 2 split so that k*LN2_HI is exact for |k| < 2^20.
constexpr double LN2_HI = 6.93147180369123816490e-01;
constexpr double LN2_LO = 1.90821492927058770002e-10;

// exp(x) = 2^k exp(r), r = x - k ln2 in [-ln2/2, ln2/2]; Taylor series of
// exp(r) summed from the smallest term upwards.
inline double exp_series(double x) {
  if (x < -700.0) return 0.0;
  if (x > 700.0) return HUGE_VAL;
  double kf = std::floor(x / 0.69314718055994530942 + 0.5);
  int k = (int)kf;
  double r = (x - kf * LN2_HI) - kf * LN2_LO;
  // terms r^n / n!, n = 0..20
  double term[21];
  term[0] = 1.0;
  for (int n = 1; n <= 20; ++n) term[n] = term[n - 1] * r / (double)n;
  double s = 0.0;
  for (int n = 20; n >= 0; --n) s = s + term[n];
  return std::ldexp(s, k);
}

// log(x), x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
// log(m) = 2 atanh(f), f = (m-1)/(m+1), atanh(f) = sum f^(2n+1)/(2n+1).
inline double log_series(double x) {
  int e;
  double m = std::frexp(x, &e);           // m in [0.5, 1)
  if (m < 0.70710678118654752440) { m = m * 2.0; e = e - 1; }
  double f = (m - 1.0) / (m + 1.0);
  double f2 = f * f;
  double pw[16];
  pw[0] = f;
  for (int n = 1; n < 16; ++n) pw[n] = pw[n - 1] * f2;
  double s = 0.0;
  for (int n = 15; n >= 0; --n) s = s + pw[n] / (double)(2 * n + 1);
  double ef = (double)e;
  return (ef * LN2_HI + (ef * LN2_LO + 2.0 * s));
}

}  // namespace adcsynth
