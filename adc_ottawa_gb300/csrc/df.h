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

__device__ __forceinline__ df df_split(double x) {
  const float h = (float)x;
  return df{h, (float)(x - (double)h)};
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
