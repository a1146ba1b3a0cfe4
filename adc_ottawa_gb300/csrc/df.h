// Double-float ("DF") arithmetic: FP64-accurate products and sums on the
// FP32 pipe.  A double x is held as hi + lo with hi = fl32(x),
// lo = fl32(x - hi) (48 significant bits).  A product of two such pairs is
// formed exactly in its leading part with an FMA (Dekker's two-product) plus
// the two cross terms; sums use Knuth's two-sum.  A 32-term step sum carries
// ~1e-14 relative error (against sum |a_i b_i|) before it is added to an
// FP64 accumulator.  On GB300 the FP32 pipe issues 64 FMAs for every FP64
// FMA, and one DF multiply-add costs about 12 FP32 instructions.
#pragma once
#include <cuda_runtime.h>

namespace adcgpu {

struct df { float hi, lo; };

// Split without FP64 arithmetic (GB300's FP64 pipe, which also converts
// between double and float, is 64x slower than the FP32 pipe): hi takes the
// sign, exponent and leading 24 significant bits of x, lo the next bits
// (together 47-48 bits; the split truncates).  |x| below 2^-126 gives 0
// (values of that size do not occur in these products).
__device__ __forceinline__ df df_split(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned sgn = (unsigned)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7ff);
  const int eh = e - 1023 + 127;
  if (eh <= 0) return df{0.f, 0.f};
  if (eh >= 255) return df{(float)x, 0.f};   // out of float range (and inf/nan)
  const float hi = __int_as_float((int)(sgn | ((unsigned)eh << 23) | ((unsigned)(u >> 29) & 0x7fffffu)));
  const unsigned r = (unsigned)(u & 0x1fffffffull);   // the 29 mantissa bits below hi
  if (r == 0u) return df{hi, 0.f};
  const int msb = 31 - __clz((int)r);
  const int el = e - 1075 + msb + 127;
  if (el <= 0) return df{hi, 0.f};
  const unsigned ml = (msb >= 23 ? (r >> (msb - 23)) : (r << (23 - msb))) & 0x7fffffu;
  return df{hi, __int_as_float((int)(sgn | ((unsigned)el << 23) | ml))};
}

// s += a * b
__device__ __forceinline__ void df_fma(df& s, df a, df b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float t = s.hi + p;
  const float v = t - s.hi;
  const float err = (s.hi - (t - v)) + (p - v);
  s.lo += err + e;
  s.hi = t;
}

// a + b
__device__ __forceinline__ df df_add(df a, df b) {
  const float t = a.hi + b.hi;
  const float v = t - a.hi;
  const float err = (a.hi - (t - v)) + (b.hi - v);
  return df{t, a.lo + b.lo + err};
}

__device__ __forceinline__ double df_value(df s) { return (double)s.hi + (double)s.lo; }

}  // namespace adcgpu
