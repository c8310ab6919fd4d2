// shells.cuh - contracted Gaussian shells evaluated at one grid point (the
// device half of numint.eval_ao, interface/pyscf.py:849-852, and ao_grads,
// interface/pyscf.py:677-705).
//
//   phi(r) = E0(r2) * A(d),  d = r - R_shell,  r2 = |d|^2,
//   E0 = sum_p C_p exp(-alpha_p r2),  E1 = sum_p -2 alpha_p C_p exp(..),  E2 = sum_p 4 alpha_p^2 C_p exp(..),
//   A(d) = sum_(i,j,k) t_ijk x^i y^j z^k  (the AO's row of cartesian coefficients, degree l),
// so that d_x phi = A_x E0 + A x E1 and d_xx phi = A_xx E0 + 2 A_x x E1 + A (E1 + x^2 E2).
#pragma once

#include "common.cuh"

namespace gdft {

constexpr int kMaxShellL = 6;

struct ShellView {
  const int32_t *shell;  // (n_shell, 4): l, nprim, exponent offset, coefficient offset
  const double *centre;  // (n_shell, 3)
  const double *exps;
  const double *coef;    // contraction-major per shell
  const int32_t *ao;     // (n_ao, 4): shell, contraction, row offset in trans, 0
  const double *trans;
  int n_shell, n_ao;
  int64_t n_prim, n_coef, n_trans;
};

namespace shells_detail {

// The angular polynomial and its first and diagonal second derivatives.
template <int L>
__device__ __forceinline__ void poly(const double *__restrict__ t, double x, double y, double z, double P[7]) {
  double xp[L + 1], yp[L + 1], zp[L + 1];
  xp[0] = yp[0] = zp[0] = 1.0;
#pragma unroll
  for (int i = 1; i <= L; ++i) {
    xp[i] = xp[i - 1] * x;
    yp[i] = yp[i - 1] * y;
    zp[i] = zp[i - 1] * z;
  }
#pragma unroll
  for (int q = 0; q < 7; ++q) P[q] = 0.0;
  int idx = 0;
#pragma unroll
  for (int lx = L; lx >= 0; --lx) {
#pragma unroll
    for (int ly = L - lx; ly >= 0; --ly) {
      const int lz = L - lx - ly;
      const double c = t[idx++];
      const double X0 = xp[lx], Y0 = yp[ly], Z0 = zp[lz];
      const double X1 = lx > 0 ? lx * xp[lx > 0 ? lx - 1 : 0] : 0.0;
      const double Y1 = ly > 0 ? ly * yp[ly > 0 ? ly - 1 : 0] : 0.0;
      const double Z1 = lz > 0 ? lz * zp[lz > 0 ? lz - 1 : 0] : 0.0;
      const double X2 = lx > 1 ? lx * (lx - 1) * xp[lx > 1 ? lx - 2 : 0] : 0.0;
      const double Y2 = ly > 1 ? ly * (ly - 1) * yp[ly > 1 ? ly - 2 : 0] : 0.0;
      const double Z2 = lz > 1 ? lz * (lz - 1) * zp[lz > 1 ? lz - 2 : 0] : 0.0;
      const double YZ = Y0 * Z0;
      P[0] = fma(c, X0 * YZ, P[0]);
      P[1] = fma(c, X1 * YZ, P[1]);
      P[2] = fma(c, X0 * Y1 * Z0, P[2]);
      P[3] = fma(c, X0 * Y0 * Z1, P[3]);
      P[4] = fma(c, X2 * YZ, P[4]);
      P[5] = fma(c, X0 * Y2 * Z0, P[5]);
      P[6] = fma(c, X0 * Y0 * Z2, P[6]);
    }
  }
}

}  // namespace shells_detail

// Values of AO a at point (px, py, pz): v = phi, d_x, d_y, d_z, d_xx, d_yy, d_zz.
// Returns false, without reading outside the tables, when the AO's entries
// are out of range.
__device__ __forceinline__ bool shell_ao_eval(const ShellView &B, double px, double py, double pz, int a,
                                              double v[7]) {
  if (a < 0 || a >= B.n_ao) return false;
  const int s = B.ao[4 * a], c = B.ao[4 * a + 1];
  const int64_t toff = B.ao[4 * a + 2];
  if (s < 0 || s >= B.n_shell) return false;
  const int l = B.shell[4 * s], np = B.shell[4 * s + 1];
  const int64_t poff = B.shell[4 * s + 2], coff = B.shell[4 * s + 3];
  if (l < 0 || l > kMaxShellL || np <= 0 || c < 0 || poff < 0 || poff + np > B.n_prim || coff < 0 ||
      coff + (int64_t)(c + 1) * np > B.n_coef)
    return false;
  if (toff < 0 || toff + (l + 1) * (l + 2) / 2 > B.n_trans) return false;
  const double x = px - B.centre[3 * s + 0];
  const double y = py - B.centre[3 * s + 1];
  const double z = pz - B.centre[3 * s + 2];
  const double r2 = x * x + y * y + z * z;
  double E0 = 0.0, E1 = 0.0, E2 = 0.0;
  const double *ex = B.exps + poff;
  const double *cf = B.coef + coff + (int64_t)c * np;
  for (int q = 0; q < np; ++q) {
    const double al = ex[q];
    const double e = cf[q] * exp(-al * r2);
    const double t1 = -2.0 * al * e;
    E0 += e;
    E1 += t1;
    E2 = fma(-2.0 * al, t1, E2);
  }
  double P[7];
  const double *t = B.trans + toff;
  switch (l) {
    case 0: shells_detail::poly<0>(t, x, y, z, P); break;
    case 1: shells_detail::poly<1>(t, x, y, z, P); break;
    case 2: shells_detail::poly<2>(t, x, y, z, P); break;
    case 3: shells_detail::poly<3>(t, x, y, z, P); break;
    case 4: shells_detail::poly<4>(t, x, y, z, P); break;
    case 5: shells_detail::poly<5>(t, x, y, z, P); break;
    default: shells_detail::poly<6>(t, x, y, z, P); break;
  }
  const double d[3] = {x, y, z};
  v[0] = P[0] * E0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    v[1 + i] = fma(P[0] * d[i], E1, P[1 + i] * E0);
    v[4 + i] = P[4 + i] * E0 + 2.0 * P[1 + i] * d[i] * E1 + P[0] * fma(d[i] * d[i], E2, E1);
  }
  return true;
}

}  // namespace gdft
