// Double-float ("float-float") arithmetic: a value held as an unevaluated
// sum hi + lo of two floats, |lo| <= ulp(hi) / 2, about 48 significant bits.
// The operations are the published error-free transformations: Knuth's
// two-sum (The Art of Computer Programming, vol. 2, 4.2.2), the exact
// product error by a fused multiply-add (Dekker's product), and their
// renormalisation as in Hida, Li & Bailey's double-double library.  Each
// operation's relative error is a few 2^-48.
//
// GB300 runs FP32 64 times as fast as FP64, so a long chain of FP64
// multiplies and adds (the q_l recurrences) runs faster here even at about
// ten FP32 operations each.  On the device every operation is an explicit
// round-to-nearest intrinsic, so the compiler neither contracts nor
// reorders them; the host build (the library's CPU test) must be compiled
// without contraction.
#pragma once

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD static inline
#include <cmath>
#endif

namespace hsmc {

struct F2 {
  float hi, lo;
};

#if defined(__CUDA_ARCH__)
DF_HD float df_add(float a, float b) { return __fadd_rn(a, b); }
DF_HD float df_sub(float a, float b) { return __fsub_rn(a, b); }
DF_HD float df_mul(float a, float b) { return __fmul_rn(a, b); }
DF_HD float df_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
DF_HD float df_add(float a, float b) { return a + b; }
DF_HD float df_sub(float a, float b) { return a - b; }
DF_HD float df_mul(float a, float b) { return a * b; }
DF_HD float df_fma(float a, float b, float c) { return std::fmaf(a, b, c); }
#endif

// s + e = a + b exactly (any a, b)
DF_HD F2 two_sum(float a, float b) {
  const float s = df_add(a, b);
  const float bb = df_sub(s, a);
  const float e = df_add(df_sub(a, df_sub(s, bb)), df_sub(b, bb));
  return F2{s, e};
}

// s + e = a + b exactly, for |a| >= |b|
DF_HD F2 quick_two_sum(float a, float b) {
  const float s = df_add(a, b);
  return F2{s, df_sub(b, df_sub(s, a))};
}

DF_HD F2 f2_of(double x) {
  const float h = (float)x;
  return F2{h, (float)(x - (double)h)};
}

DF_HD double f2_value(F2 a) { return (double)a.hi + (double)a.lo; }

DF_HD F2 f2_neg(F2 a) { return F2{-a.hi, -a.lo}; }

DF_HD F2 f2_add(F2 a, F2 b) {
  F2 s = two_sum(a.hi, b.hi);
  const F2 t = two_sum(a.lo, b.lo);
  s.lo = df_add(s.lo, t.hi);
  s = quick_two_sum(s.hi, s.lo);
  s.lo = df_add(s.lo, t.lo);
  return quick_two_sum(s.hi, s.lo);
}

DF_HD F2 f2_sub(F2 a, F2 b) { return f2_add(a, f2_neg(b)); }

DF_HD F2 f2_mul(F2 a, F2 b) {
  const float p = df_mul(a.hi, b.hi);
  float e = df_fma(a.hi, b.hi, -p);  // the exact error of the leading product
  e = df_fma(a.hi, b.lo, e);
  e = df_fma(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}

}  // namespace hsmc
