// dfloat.cuh - double-float arithmetic (a value as an unevaluated FP32 pair s + c)
// for the mixed form's table and operand builders.
//
// GB300 runs FP64 at 1/64 of its FP32 rate, so values that need more than
// FP32's 24 bits but are only ever stored as FP32 slices are computed as FP32
// pairs: products keep their rounding error through an FMA, sums through
// TwoSum, which gives about 2^-44 of the terms.  The rounded operations are
// the _rn intrinsics so that no two of them are contracted into an FMA.
#pragma once

#include <math.h>

namespace gdft {
namespace df {

struct DF {
  float s, c;
};

__device__ __forceinline__ DF of(float s) { return DF{s, 0.0f}; }
// An FP64 value as s = fp32(x), c = fp32(x - s).
__device__ __forceinline__ DF of_double(double x) {
  const float s = (float)x;
  return DF{s, (float)(x - (double)s)};
}
// a + b exactly as s + e (Knuth's TwoSum).
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp))};
}
// a + b exactly, for |a| >= |b| (Fast2Sum).
__device__ __forceinline__ DF fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF add(DF a, DF b) {
  const DF t = two_sum(a.s, b.s);
  return two_sum(t.s, __fadd_rn(t.c, __fadd_rn(a.c, b.c)));
}
__device__ __forceinline__ DF neg(DF a) { return DF{-a.s, -a.c}; }
__device__ __forceinline__ DF sub(DF a, DF b) { return add(a, neg(b)); }
__device__ __forceinline__ DF mul(DF a, DF b) {
  const float p = __fmul_rn(a.s, b.s);
  const float e = fmaf(a.s, b.s, -p);
  return fast_two_sum(p, __fadd_rn(e, fmaf(a.s, b.c, __fmul_rn(a.c, b.s))));
}
__device__ __forceinline__ DF mul(DF a, float b) {
  const float p = __fmul_rn(a.s, b);
  const float e = fmaf(a.s, b, -p);
  return fast_two_sum(p, fmaf(a.c, b, e));
}
// The normalised sum s + c as one FP32 value is s; the remainder below it is c.
__device__ __forceinline__ DF norm(DF a) { return two_sum(a.s, a.c); }

// exp(x) to about 2^-47 relative for -70 < x < 88 (below, the pair's low part
// falls into FP32's subnormal range and the relative error grows towards
// 2^-24, for values under 1e-30): x = k ln2 + r with ln2 in three
// FP32 parts (the first with 16 significant bits, so k * ln2_0 is exact for
// |k| < 256), |r| <= ln2 / 2, exp(r) from its Taylor series to degree 12
// (truncation below 2^-52) by Horner in double-float, then scaled by 2^k.
// Results below FP32's normal range are returned as 0.
__device__ __forceinline__ DF exp_df(DF x) {
  if (x.s < -87.0f) return DF{0.0f, 0.0f};
  constexpr float kLn2_0 = 0.693145751953125f, kLn2_1 = 1.428606765330187e-06f, kLn2_2 = 5.497923148104107e-14f;
  constexpr float kLog2e = 1.4426950216293335f;
  // 1 / n!, n = 0..12, as FP32 pairs (hi = fp32(1/n!), lo = fp32(1/n! - hi)).
  constexpr float kInvFactHi[13] = {1.0f, 1.0f, 0.5f, 0.1666666716337204f, 0.0416666679084301f,
                                    0.008333333767950535f, 0.0013888889225199819f, 0.00019841270113829523f,
                                    2.4801587642286904e-05f, 2.7557318844628753e-06f, 2.755731998149713e-07f,
                                    2.5052107943679403e-08f, 2.0876755879584152e-09f};
  constexpr float kInvFactLo[13] = {0.0f, 0.0f, 0.0f, -4.967053879312289e-09f, -1.2417634698280722e-09f,
                                    -4.34617203337595e-10f, -3.3631094437103215e-11f, -2.725596874933456e-12f,
                                    -3.40699609366682e-13f, 3.793571224297229e-14f, -7.575112209051195e-15f,
                                    4.4176230446483665e-16f, 1.1082839147459852e-16f};
  const float k = rintf(__fmul_rn(x.s, kLog2e));
  DF r = two_sum(__fsub_rn(x.s, __fmul_rn(k, kLn2_0)), x.c);  // the first difference is exact
  const float p1 = __fmul_rn(k, kLn2_1);
  r = sub(r, DF{p1, fmaf(k, kLn2_1, -p1)});
  r = sub(r, of(__fmul_rn(k, kLn2_2)));
  DF e{kInvFactHi[12], kInvFactLo[12]};
#pragma unroll
  for (int n = 11; n >= 0; --n) e = add(mul(e, r), DF{kInvFactHi[n], kInvFactLo[n]});
  const int ki = (int)k;
  return DF{ldexpf(e.s, ki), ldexpf(e.c, ki)};
}

}  // namespace df
}  // namespace gdft
