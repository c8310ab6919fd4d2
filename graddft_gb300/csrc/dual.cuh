// dual.cuh - forward-mode dual numbers for the per-point energy densities.
//
// The reference obtains V_xc from jax.value_and_grad through every pointwise
// function of the energy densities (train.py:86).  Here each pointwise
// function is written once as a template over the scalar type; instantiating
// it with Dual<K> yields the value and the K partial derivatives with respect
// to the point's density variables in one pass.  Gradient conventions follow
// jax.numpy:
//   clip(x, a_min=c) == maximum(c, x): derivative 1 above c, 0 below, 1/2 at a tie;
//   where(p, a, b): derivative of the selected branch;
//   abs(x): derivative sign(x).
#pragma once

#include <math.h>

namespace gdft {

template <int K>
struct Dual {
  double v;
  double d[K];
};

__device__ __forceinline__ double val(double x) { return x; }
template <int K>
__device__ __forceinline__ double val(const Dual<K> &x) { return x.v; }

template <int K>
__device__ __forceinline__ Dual<K> dconst(double c) {
  Dual<K> r;
  r.v = c;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = 0.0;
  return r;
}

// Unary rule: value f, derivative factor df (r.d = df * x.d).
template <int K>
__device__ __forceinline__ Dual<K> chain(const Dual<K> &x, double f, double df) {
  Dual<K> r;
  r.v = f;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = df * x.d[i];
  return r;
}

template <int K>
__device__ __forceinline__ Dual<K> operator+(const Dual<K> &a, const Dual<K> &b) {
  Dual<K> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K> &a, const Dual<K> &b) {
  Dual<K> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K> &a) {
  Dual<K> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(const Dual<K> &a, const Dual<K> &b) {
  Dual<K> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(const Dual<K> &a, const Dual<K> &b) {
  Dual<K> r;
  r.v = a.v / b.v;
  const double inv = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
  return r;
}
// Mixed with constants.
template <int K>
__device__ __forceinline__ Dual<K> operator+(const Dual<K> &a, double c) {
  Dual<K> r = a;
  r.v = a.v + c;
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator+(double c, const Dual<K> &a) {
  Dual<K> r = a;
  r.v = c + a.v;
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K> &a, double c) {
  Dual<K> r = a;
  r.v = a.v - c;
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(double c, const Dual<K> &a) {
  Dual<K> r;
  r.v = c - a.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(const Dual<K> &a, double c) {
  Dual<K> r;
  r.v = a.v * c;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = a.d[i] * c;
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(double c, const Dual<K> &a) {
  Dual<K> r;
  r.v = c * a.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = c * a.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(const Dual<K> &a, double c) {
  Dual<K> r;
  r.v = a.v / c;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = a.d[i] / c;
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(double c, const Dual<K> &a) {
  Dual<K> r;
  r.v = c / a.v;
  const double f = -r.v / a.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = f * a.d[i];
  return r;
}

// ---- elementary functions (double and Dual overloads) ---------------------
__device__ __forceinline__ double xlog2(double x) { return log2(x); }
__device__ __forceinline__ double xexp2(double x) { return exp2(x); }
__device__ __forceinline__ double xlog(double x) { return log(x); }
__device__ __forceinline__ double xexp(double x) { return exp(x); }
__device__ __forceinline__ double xsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ double xasinh(double x) { return asinh(x); }
__device__ __forceinline__ double xatan(double x) { return atan(x); }
__device__ __forceinline__ double xpow(double x, double p) { return pow(x, p); }
__device__ __forceinline__ double xpow3(double x, int n) {
  if (!(x >= 0.0)) return pow(x, n / 3.0);  // NaN for negative or NaN x, as pow
  if (n == -1) return rcbrt(x);
  if (n == -5) {
    const double r = rcbrt(x);
    return (r * r) / x;
  }
  if (n == 4) return x * cbrt(x);
  if (n == 8) {
    const double c = cbrt(x);
    return (x * x) * (c * c);
  }
  return pow(x, n / 3.0);
}
__device__ __forceinline__ double xsq(double x) { return x * x; }
__device__ __forceinline__ double xclipmin(double x, double c) { return isnan(x) ? x : fmax(c, x); }
__device__ __forceinline__ double xabs(double x) { return fabs(x); }
__device__ __forceinline__ double xsign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }

constexpr double kLn2 = 0.69314718055994530942;

template <int K>
__device__ __forceinline__ Dual<K> xlog2(const Dual<K> &x) {
  return chain(x, log2(x.v), 1.0 / (x.v * kLn2));
}
template <int K>
__device__ __forceinline__ Dual<K> xexp2(const Dual<K> &x) {
  const double f = exp2(x.v);
  return chain(x, f, f * kLn2);
}
template <int K>
__device__ __forceinline__ Dual<K> xlog(const Dual<K> &x) {
  return chain(x, log(x.v), 1.0 / x.v);
}
template <int K>
__device__ __forceinline__ Dual<K> xexp(const Dual<K> &x) {
  const double f = exp(x.v);
  return chain(x, f, f);
}
template <int K>
__device__ __forceinline__ Dual<K> xsqrt(const Dual<K> &x) {
  const double f = sqrt(x.v);
  return chain(x, f, 0.5 / f);
}
template <int K>
__device__ __forceinline__ Dual<K> xasinh(const Dual<K> &x) {
  return chain(x, asinh(x.v), 1.0 / sqrt(1.0 + x.v * x.v));
}
template <int K>
__device__ __forceinline__ Dual<K> xatan(const Dual<K> &x) {
  return chain(x, atan(x.v), 1.0 / (1.0 + x.v * x.v));
}
// x ** p with a constant real exponent (jax pow JVP: p * x ** (p - 1)).
template <int K>
__device__ __forceinline__ Dual<K> xpow(const Dual<K> &x, double p) {
  return chain(x, pow(x.v, p), p * pow(x.v, p - 1.0));
}
// x ** (n/3) with an integer n from CUDA's cube roots (cbrt and rcbrt are
// within 1 ulp; pow evaluates a logarithm and an exponential): n = -1, -5, 4
// and 8, the powers of LYP and B88, to within a few ulp (pow for x < 0 or NaN);
// partial (n/3) f / x (elsewhere than at finite x > 0 the pow form, p x ** (p - 1)).
template <int K>
__device__ __forceinline__ Dual<K> xpow3(const Dual<K> &x, int n) {
  const double f = xpow3(x.v, n);
  const double df = x.v > 0.0 && isfinite(f) ? (n / 3.0) * f / x.v : (n / 3.0) * pow(x.v, n / 3.0 - 1.0);
  return chain(x, f, df);
}
// x ** 2 with an integer exponent (jax integer_pow JVP: 2 x).
template <int K>
__device__ __forceinline__ Dual<K> xsq(const Dual<K> &x) {
  return chain(x, x.v * x.v, 2.0 * x.v);
}
template <int K>
__device__ __forceinline__ Dual<K> xclipmin(const Dual<K> &x, double c) {
  const double f = isnan(x.v) ? x.v : fmax(c, x.v);
  const double df = x.v > c ? 1.0 : (x.v == c ? 0.5 : 0.0);
  return chain(x, f, df);
}
template <int K>
__device__ __forceinline__ Dual<K> xabs(const Dual<K> &x) {
  return chain(x, fabs(x.v), xsign(x.v));
}

template <class T>
__device__ __forceinline__ T xwhere(bool p, const T &a, const T &b) {
  return p ? a : b;
}

// A constant of the same scalar type as `like` (zero partials).
__device__ __forceinline__ double tconst(double, double c) { return c; }
template <int K>
__device__ __forceinline__ Dual<K> tconst(const Dual<K> &, double c) {
  return dconst<K>(c);
}

}  // namespace gdft
