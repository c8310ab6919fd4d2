// xc_functionals.cuh - pointwise energy densities of the reference functionals.
//
// Each function restates one reference function for a single grid point,
// keeping its evaluation order, clip and where semantics; it is a template
// over the scalar type (double for values, Dual<K> for values plus partials).
// Powers of a third come from cube roots (xpow3), within a few ulp of pow, and
// B88 is evaluated without its logarithms (see b88_x_e).
// Inputs per point: rho[2], s[2] = |grad rho_sigma|^2, st = |grad rho_a +
// grad rho_b|^2, lap[2], tau[2].
#pragma once

#include "dual.cuh"

namespace gdft {

constexpr double kPi = 3.14159265358979323846;

// exchange_polarization_correction, functional.py:950-979.
template <class T>
__device__ __forceinline__ T exch_pol(const T &e0, const T &e1, const T &r0, const T &r1) {
  const T zeta = (r0 - r1) / (r0 + r1);
  const double den = 2.0 * (pow(2.0, 1.0 / 3.0) - 1.0);
  const T fz = (xpow(1.0 - zeta, 4.0 / 3.0) + xpow(1.0 + zeta, 4.0 / 3.0) - 2.0) / den;
  return e0 + (e1 - e0) * fz;
}

// fzeta in log2 form, functional.py:1008-1011.
template <class T>
__device__ __forceinline__ T fzeta_log2(const T &z) {
  const T zm = xexp2(4.0 * xlog2(1.0 - z) / 3.0);
  const T zp = xexp2(4.0 * xlog2(1.0 + z) / 3.0);
  return (zm + zp - 2.0) / (2.0 * (pow(2.0, 1.0 / 3.0) - 1.0));
}

// grad(grad(fzeta))(0.0) of functional.py:1040: d^2/dz^2 of fzeta at 0
// = (4/3)(1/3) 2 / (2 (2^(1/3) - 1)) = 4 / (9 (2^(1/3) - 1)).
__device__ __forceinline__ double fzeta_pp0() { return 4.0 / (9.0 * (pow(2.0, 1.0 / 3.0) - 1.0)); }

// correlation_polarization_correction, functional.py:982-1045.
//
// `nan_path` is set when the reference's reverse-mode gradient is NaN: with
// rho_a + rho_b > clip and |zeta| >= 1 (zeta = +-1 exactly, or beyond when one
// spin density is negative, as the unconjugated k-point forms of a Solid
// allow), the backward of 2^(4/3 log2(1 -+ zeta)) in fzeta meets a division of
// a (possibly zero) cotangent by zero or a NaN forward value, and the NaN
// reaches rho_a and rho_b through the selected branch of the zeta `where`,
// whatever the masks further down (jax.grad at train.py:86).  Forward-mode
// partials would stay finite there, so the caller poisons those inputs.
template <class T>
__device__ __forceinline__ T corr_pol(const T &ep0, const T &ep1, const T &r0, const T &r1, double clip,
                                      bool *nan_path = nullptr) {
  const T rs = r0 + r1;
  const T log_rho = xlog2(xclipmin(rs, clip));
  const T log_rs = log2(pow(3.0 / (4.0 * kPi), 1.0 / 3.0)) - log_rho / 3.0;
  const T zeta = xwhere(val(rs) > clip, (r0 - r1) / rs, tconst(rs, 0.0));
  if (nan_path != nullptr) *nan_path = val(rs) > clip && !(1.0 - val(zeta) > 0.0 && 1.0 + val(zeta) > 0.0);
  const double A_ = 0.016887, alpha1 = 0.11125, beta1 = 10.357, beta2 = 3.6231, beta3 = 0.88026,
               beta4 = 0.49671;
  const T ars = xexp2(log2(alpha1) + log_rs);
  const T brs_1_2 = xexp2(log2(beta1) + log_rs / 2.0);
  const T brs = xexp2(log2(beta2) + log_rs);
  const T brs_3_2 = xexp2(log2(beta3) + 3.0 * log_rs / 2.0);
  const T brs2 = xexp2(log2(beta4) + 2.0 * log_rs);
  const T alphac = 2.0 * A_ * (1.0 + ars) * xlog(1.0 + (1.0 / (2.0 * A_)) / (brs_1_2 + brs + brs_3_2 + brs2));
  const T fz = fzeta_log2(zeta);
  const T z2 = xsq(zeta);
  const T z4 = xsq(z2);
  return ep0 + alphac * (fz / fzeta_pp0()) * (1.0 - z4) + (ep1 - ep0) * fz * z4;
}

// lsda_x_e, popular_functionals.py:29-50.
template <class T>
__device__ __forceinline__ T lsda_x_e(const T rho_in[2], double clip) {
  const T r0 = xclipmin(rho_in[0], clip);
  const T r1 = xclipmin(rho_in[1], clip);
  const T s43 = xpow(r0 + r1, 4.0 / 3.0);
  const T e0 = (-3.0 / 4.0 * pow(3.0 / kPi, 1.0 / 3.0)) * s43;
  const T e1 = (-3.0 / 4.0 * pow(6.0 / kPi, 1.0 / 3.0)) * s43;
  return exch_pol(e0, e1, r0, r1);
}

// b88_x_e, popular_functionals.py:52-103 (gradient correction, summed over spin).
// The reference works in base-2 logarithms: with g = |grad rho_s| (its squared
// norm clipped), log x = log2 g - 4/3 log2 rho and the term
// beta 2^(4/3 log2 rho + 2 log x - log2 D), D = 1 + 6 beta x asinh(x).  Since
// 4/3 log2 rho + 2 log x = log2(g x), the term is beta g x / D with
// x = g / rho^(4/3): the same function (and the same clips) without the four
// logarithms and exponentials per spin.
template <class T>
__device__ __forceinline__ T b88_x_e(const T rho_in[2], const T s[2], double clip) {
  const double beta = 0.0042;
  T out;
#pragma unroll
  for (int sp = 0; sp < 2; ++sp) {
    const T rho = xclipmin(rho_in[sp], clip);
    const T g = xsqrt(xclipmin(s[sp], clip));
    const T x = g / xpow3(xclipmin(rho, clip), 4);
    const T term = beta * (g * x) / (1.0 + 6.0 * beta * x * xasinh(x));
    out = sp == 0 ? term : out + term;
  }
  return -out;
}

// pw92_c_e, popular_functionals.py:105-139.
template <class T>
__device__ __forceinline__ T pw92_c_e(const T rho[2], double clip, unsigned *poison = nullptr) {
  const double A_[2] = {0.031091, 0.015545}, alpha1[2] = {0.21370, 0.20548}, beta1[2] = {7.5957, 14.1189},
               beta2[2] = {3.5876, 6.1977}, beta3[2] = {1.6382, 3.3662}, beta4[2] = {0.49294, 0.62517};
  const T rs_sum = rho[0] + rho[1];
  const T log_rho = xlog2(xclipmin(rs_sum, clip));
  const T log_rs = log2(pow(3.0 / (4.0 * kPi), 1.0 / 3.0)) - log_rho / 3.0;
  T ep[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const T brs_1_2 = xexp2(log_rs / 2.0 + log2(beta1[k]));
    const T ars = xexp2(log_rs + log2(alpha1[k]));
    const T brs = xexp2(log_rs + log2(beta2[k]));
    const T brs_3_2 = xexp2(3.0 * log_rs / 2.0 + log2(beta3[k]));
    const T brs2 = xexp2(2.0 * log_rs + log2(beta4[k]));
    ep[k] = -2.0 * A_[k] * (1.0 + ars) * xlog(1.0 + (1.0 / (2.0 * A_[k])) / (brs_1_2 + brs + brs_3_2 + brs2));
  }
  bool np = false;
  const T et = corr_pol(ep[0], ep[1], rho[0], rho[1], clip, &np);
  if (poison != nullptr && np) *poison |= 3u;  // both spins reach zeta unmasked
  return et * rs_sum;
}

// vwn_c_e, popular_functionals.py:141-195.
template <class T>
__device__ __forceinline__ T vwn_c_e(const T rho_in[2], double clip, unsigned *poison = nullptr) {
  const double A[2] = {0.0621814, 0.0621814 / 2.0}, b[2] = {3.72744, 7.06042}, c[2] = {12.9352, 18.0578},
               x0[2] = {-0.10498, -0.325};
  const T r0 = xwhere(val(rho_in[0]) > clip, rho_in[0], tconst(rho_in[0], 0.0));
  const T r1 = xwhere(val(rho_in[1]) > clip, rho_in[1], tconst(rho_in[1], 0.0));
  const T rs_sum = r0 + r1;
  const T log_rho = xlog2(xclipmin(rs_sum, clip));
  const T log_rs = log2(pow(3.0 / (4.0 * kPi), 1.0 / 3.0)) - log_rho / 3.0;
  const T log_x = log_rs / 2.0;
  const T x = xexp2(log_x);
  T ep[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const T X = xexp2(2.0 * log_x) + xexp2(log_x + log2(b[k])) + c[k];
    const double X0 = x0[k] * x0[k] + b[k] * x0[k] + c[k];
    const double Q = sqrt(4.0 * c[k] - b[k] * b[k]);
    const T at = xatan(Q / (2.0 * x + b[k]));
    ep[k] = A[k] / 2.0 *
            (2.0 * xlog(x) - xlog(X) + 2.0 * b[k] / Q * at -
             b[k] * x0[k] / X0 * (xlog(xsq(x - x0[k]) / X) + 2.0 * (2.0 * x0[k] + b[k]) / Q * at));
  }
  bool np = false;
  const T et = corr_pol(ep[0], ep[1], r0, r1, clip, &np);
  // where(rho > clip, rho, 0) routes the NaN only to the spins above the clip.
  if (poison != nullptr && np) *poison |= (val(rho_in[0]) > clip ? 1u : 0u) | (val(rho_in[1]) > clip ? 2u : 0u);
  return et * rs_sum;
}

// lyp_c_e, popular_functionals.py:197-269 (original LYP with the Laplacian).
template <class T>
__device__ __forceinline__ T lyp_c_e(const T rho_in[2], const T s[2], const T lap[2], double clip) {
  const double a = 0.04918, b = 0.132, c = 0.2533, d = 0.349;
  const double CF = (3.0 / 10.0) * pow(3.0 * kPi * kPi, 2.0 / 3.0);
  const T r0 = xclipmin(rho_in[0], clip);
  const T r1 = xclipmin(rho_in[1], clip);
  const T zero = tconst(r0, 0.0);
  const T t0 = (xwhere(val(r0) > clip, s[0] / r0, zero) - lap[0]) / 8.0;
  const T t1 = (xwhere(val(r1) > clip, s[1] / r1, zero) - lap[1]) / 8.0;
  const T rsum = r0 + r1;
  const bool big = val(rsum) > clip;
  const T frac = xwhere(big, (xsq(r0) + xsq(r1)) / xsq(rsum), tconst(r0, 1.0));
  const T gamma = 2.0 * (1.0 - frac);
  const T rhos_ts = rsum * (t0 + t1);
  const T rho_t = r0 * t0 + r1 * t1;
  const T rho_grad2rho = r0 * lap[0] + r1 * lap[1];
  const T rhom1_3 = xpow3(rsum, -1);
  const T rho8_3 = xpow3(r0, 8) + xpow3(r1, 8);
  const T rhom5_3 = xpow3(rsum, -5);
  const T exp_factor = xwhere(val(rsum) > 0.0, xexp(-c * rhom1_3), zero);
  const T parenthesis = pow(2.0, 2.0 / 3.0) * CF * rho8_3 - rhos_ts + rho_t / 9.0 + rho_grad2rho / 18.0;
  const T braket = xwhere(big, 2.0 * b * rhom5_3 * parenthesis * exp_factor, zero);
  return -a * xwhere(big, gamma / (1.0 + d * rhom1_3) * (rsum + braket), zero);
}

// One spin's u^i w^j feature term, 2^(4/3 log rho + i log u + j log w), of
// dm21_densities (functional.py:588-624) and of densities() (:1104-1134):
//   log rho = log2(clip(rho)),  log x = log2(clip(|grad rho|^2))/2 - 4/3 log rho,
//   log u   = where(log rho > log2 clip, log x - log2(1 + beta 2^log x) + log2 beta, 0),
//   log 1/t = -(5/3 log rho - log tau + 2/3 log2(6 pi^2) + log2(3/5))   (dm21_densities, :601-603)
//           = log tau - 5/3 log rho                                      (densities(), :1119),
//   log w   = where(log rho > log2 clip, log 1/t - log2(1 + beta 2^log 1/t) + log2 beta, 0),
// with clip(v) = clip(v, a_min=clip_cte) and beta = 1/1024.  A zero power
// adds 0 * (a finite log u or log w) to the exponent in the reference, so the
// term is skipped (2^(e + 0) = 2^e).
template <class T>
__device__ __forceinline__ T uw_term(const T &rho, const T &sig, const T &tau, int i, int j, bool dm21_form,
                                     double clip) {
  const double beta = 1.0 / 1024.0;
  const double lbeta = log2(beta);
  const T log_rho = xlog2(xclipmin(rho, clip));
  const bool above = val(log_rho) > log2(clip);
  T ex = 4.0 / 3.0 * log_rho;
  if (i != 0) {
    const T log_x = xlog2(xclipmin(sig, clip)) / 2.0 - 4.0 / 3.0 * log_rho;
    const T log_u = above ? (log_x - xlog2(1.0 + beta * xexp2(log_x))) + lbeta : tconst(rho, 0.0);
    ex = ex + (double)i * log_u;
  }
  if (j != 0) {
    const T log_tau = xlog2(xclipmin(tau, clip));
    const T log_1t = dm21_form ? -(((5.0 / 3.0 * log_rho - log_tau) + 2.0 / 3.0 * log2(6.0 * (kPi * kPi))) +
                                   log2(3.0 / 5.0))
                               : log_tau - 5.0 / 3.0 * log_rho;
    const T log_w = above ? (log_1t - xlog2(1.0 + beta * xexp2(log_1t))) + lbeta : tconst(rho, 0.0);
    ex = ex + (double)j * log_w;
  }
  return xexp2(ex);
}

// dm21_densities' column for (i, j): the spin sum of uw_term, times the
// Dirac exchange constant -2 pi (3/(4 pi))^(4/3) for i = j = 0 (functional.py:616-624).
template <class T>
__device__ __forceinline__ T dm21_uw(const T rho[2], const T sig[2], const T tau[2], int i, int j, double clip) {
  const T s = uw_term(rho[0], sig[0], tau[0], i, j, true, clip) + uw_term(rho[1], sig[1], tau[1], i, j, true, clip);
  return (i == 0 && j == 0) ? s * (-2.0 * kPi * pow(3.0 / (4.0 * kPi), 4.0 / 3.0)) : s;
}

// dm21_densities(functional_type="LDA"), functional.py:534-626: one column.
template <class T>
__device__ __forceinline__ T dm21_lda(const T rho[2], double clip) {
  const double scale = -2.0 * kPi * pow(3.0 / (4.0 * kPi), 4.0 / 3.0);
  const T a = xexp2(4.0 / 3.0 * xlog2(xclipmin(rho[0], clip)));
  const T b = xexp2(4.0 / 3.0 * xlog2(xclipmin(rho[1], clip)));
  return (a + b) * scale;
}

}  // namespace gdft
