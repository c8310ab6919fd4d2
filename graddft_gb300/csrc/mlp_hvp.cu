// mlp_hvp.cu - second-order adjoint of the DM21-style network energy (FP64 form).
//
// The differentiable SCF loop (evaluate.py:314-344) builds every iteration's
// Fock matrix from V_xc = dE_xc/dD (train.py:86) and jax.grad then
// differentiates through it.  Its vector-Jacobian product, for a cotangent G
// on V_xc, is the gradient of L = <G, V_xc(D, theta)> with respect to D and
// theta - a Hessian-vector product of E_xc.  Per grid point
//   L_r = d/de E_r(F + e F~)|_{e=0},  F = features of D, F~ = features of G
// (density, gradient, tau are linear in the density matrix), so L is the
// energy's tangent along F~.  This file evaluates it as one tangent-augmented
// pass through the network (primal and tangent activations stacked as
// [2][np][width], so each layer is one GEMM over 2 np rows) followed by the
// reverse pass of that augmented graph, which carries the second-order terms
// of tanh, LayerNorm, ELU, the sigmoid head, the log squash and the DM21 LDA
// density.  The result is dL/dtheta and per-point coefficients dL/dF whose V
// contraction (vxc_*.cu) is dL/dD.
#include "common.cuh"
#include "dual.cuh"
#include "kernels.cuh"
#include "mlp.cuh"
#include "mlp_gemm.cuh"
#include "xc_functionals.cuh"

namespace gdft {

namespace {

constexpr int kIn = kDm21In, kInPad = kDm21InPad;

// d|x|/dx as jax's abs JVP takes it: +1 for x >= 0, -1 below.
__device__ __forceinline__ double abs_slope(double x) { return x >= 0.0 ? 1.0 : -1.0; }

// Primal and tangent network inputs, squashed inputs and energy densities.
__global__ void features_tan_kernel(const double *__restrict__ featp, const double *__restrict__ featt,
                                    const double *__restrict__ ehf, int64_t n_grid, int64_t np, double clip,
                                    double off, double *__restrict__ x, double *__restrict__ xt,
                                    double *__restrict__ u, double *__restrict__ e, double *__restrict__ et) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double xv[kIn], xd[kIn];
  double ev[3] = {0.0, 0.0, 0.0}, ed0 = 0.0;
#pragma unroll
  for (int k = 0; k < kIn; ++k) xv[k] = xd[k] = 0.0;
  if (p < n_grid) {
    double rho[2], g[2][3], tau[2], rt[2], gt[2][3], tt[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const double *f = featp + (size_t)s * kFeat * np;
      const double *ft = featt + (size_t)s * kFeat * np;
      rho[s] = f[F_RHO * np + p];
      rt[s] = ft[F_RHO * np + p];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        g[s][j] = f[(F_GX + j) * np + p];
        gt[s][j] = ft[(F_GX + j) * np + p];
      }
      tau[s] = f[F_TAU * np + p];
      tt[s] = ft[F_TAU * np + p];
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const double a = fabs(rho[s]);
      xv[s] = fmax(a, clip) * xsign(rho[s]);
      xd[s] = (a > clip ? 1.0 : (a == clip ? 0.5 : 0.0)) * rt[s];
    }
    double sg[3], sgt[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      sg[j] = g[0][j] + g[1][j];
      sgt[j] = gt[0][j] + gt[1][j];
    }
    xv[2] = (sg[0] * sg[0] + sg[1] * sg[1]) + sg[2] * sg[2];
    xd[2] = 2.0 * ((sg[0] * sgt[0] + sg[1] * sgt[1]) + sg[2] * sgt[2]);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      xv[3 + s] = (g[s][0] * g[s][0] + g[s][1] * g[s][1]) + g[s][2] * g[s][2];
      xd[3 + s] = 2.0 * ((g[s][0] * gt[s][0] + g[s][1] * gt[s][1]) + g[s][2] * gt[s][2]);
      xv[5 + s] = tau[s];
      xd[5 + s] = tt[s];
    }
    const double e00 = ehf[(0 * 2 + 0) * n_grid + p], e10 = ehf[(1 * 2 + 0) * n_grid + p];
    const double e01 = ehf[(0 * 2 + 1) * n_grid + p], e11 = ehf[(1 * 2 + 1) * n_grid + p];
    xv[7] = e00;
    xv[8] = e10;
    xv[9] = e01;
    xv[10] = e11;
    Dual<2> r2[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      r2[s] = dconst<2>(rho[s]);
      r2[s].d[s] = 1.0;
    }
    const Dual<2> e0 = dm21_lda(r2, clip);
    ev[0] = e0.v;
    ev[1] = e00 + e01;
    ev[2] = e10 + e11;
    ed0 = e0.d[0] * rt[0] + e0.d[1] * rt[1];
  }
  double *u0 = u + (size_t)p * kInPad, *u1 = u + ((size_t)np + p) * kInPad;
#pragma unroll
  for (int k = 0; k < kIn; ++k) {
    x[(size_t)p * kIn + k] = xv[k];
    xt[(size_t)p * kIn + k] = xd[k];
    u0[k] = log(fabs(xv[k]) + off);
    u1[k] = xd[k] * abs_slope(xv[k]) / (fabs(xv[k]) + off);
  }
#pragma unroll
  for (int k = kIn; k < kInPad; ++k) u0[k] = u1[k] = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) e[(size_t)p * 3 + k] = ev[k];
  et[p] = ed0;
}

// Layer 0: h = tanh(z + b), h~ = (1 - h^2) z~.  Z = [z; z~] (z gets the bias
// added in place), H = [h; h~].
__global__ void tanh_tan_kernel(double *__restrict__ Z, const double *__restrict__ b, size_t act, int width,
                                double *__restrict__ H) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= act) return;
  const double z = Z[i] + b[i % width];
  Z[i] = z;
  const double h = tanh(z);
  H[i] = h;
  H[act + i] = (1.0 - h * h) * Z[act + i];
}

// Residual layer, primal and tangent: z = zW + b + h_prev, z~ = z~W + h~_prev
// (both stored back into Z); a = LayerNorm(z), a~ = gamma * xhat~;
// h = elu(a), h~ = elu'(a) a~.  One warp per row.
template <int PL>
__global__ void res_ln_elu_tan_fwd_kernel(double *__restrict__ Z, const double *__restrict__ b,
                                          const double *__restrict__ Hp, const double *__restrict__ gam,
                                          const double *__restrict__ bet, double eps, int64_t rows,
                                          double *__restrict__ H) {
  constexpr int W = 32 * PL;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  const size_t act = (size_t)rows * W;
  double *z = Z + (size_t)r * W, *zt = Z + act + (size_t)r * W;
  const double *hp = Hp + (size_t)r * W, *hpt = Hp + act + (size_t)r * W;
  double v[PL], vt[PL], s1 = 0.0, s2 = 0.0;
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    const int c = lane + 32 * k;
    v[k] = (z[c] + b[c]) + hp[c];
    vt[k] = zt[c] + hpt[c];
    z[c] = v[k];
    zt[c] = vt[k];
    s1 += v[k];
    s2 += v[k] * v[k];
  }
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  const double mean = s1 / W;
  const double var = fmax(0.0, s2 / W - mean * mean);
  const double rs = 1.0 / sqrt(var + eps);
  double m1 = 0.0, m2 = 0.0, xh[PL];
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    xh[k] = (v[k] - mean) * rs;
    m1 += vt[k];
    m2 += xh[k] * vt[k];
  }
  m1 = warp_sum(m1) / W;
  m2 = warp_sum(m2) / W;
  double *h = H + (size_t)r * W, *ht = H + act + (size_t)r * W;
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    const int c = lane + 32 * k;
    const double a = (v[k] - mean) * (rs * gam[c]) + bet[c];
    const double at = gam[c] * (rs * (vt[k] - m1 - xh[k] * m2));
    const double e1 = a > 0.0 ? 1.0 : exp(a);
    h[c] = a > 0.0 ? a : expm1(a);
    ht[c] = e1 * at;
  }
}

// Head: L_r = m w sum_f (c~_f ec_f + c_f e~'_f) with c = s sigmoid(y/s),
// c~ = sigmoid' y~; writes G = [dL/dy; dL/dy~], dL/de_0 and dL/de~_0, and
// block partial sums of L.
__global__ void __launch_bounds__(256) head_tan_kernel(const double *__restrict__ Y, const double *__restrict__ bout,
                                                       const double *__restrict__ e, const double *__restrict__ et,
                                                       const double *__restrict__ w, int64_t n_grid, int64_t np,
                                                       double clip, double sscale, double *__restrict__ GY,
                                                       double *__restrict__ ge, double *__restrict__ lpart) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double l_r = 0.0;
  if (p < np) {
    double gy[3] = {0.0, 0.0, 0.0}, gyt[3] = {0.0, 0.0, 0.0}, ge0 = 0.0, get0 = 0.0;
    if (p < n_grid) {
      double sg[3], c[3], ct[3], ec[3], ed[3];
      double exc = 0.0;
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const double yv = Y[(size_t)p * 3 + f] + bout[f];
        sg[f] = 1.0 / (1.0 + exp(-(yv / sscale)));
        c[f] = sscale * sg[f];
        ct[f] = sg[f] * (1.0 - sg[f]) * Y[((size_t)np + p) * 3 + f];
        const double ev = e[(size_t)p * 3 + f];
        const bool keep = fabs(ev) > clip;
        ec[f] = keep ? ev : 0.0;
        ed[f] = (f == 0 && keep) ? et[p] : 0.0;
        exc = f == 0 ? c[f] * ec[f] : exc + c[f] * ec[f];
      }
      const bool m = fabs(exc) > clip;
      const double W = fabs(w[p]) > clip ? w[p] : 0.0;
      if (m) {
        double lr = 0.0;
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          lr += ct[f] * ec[f] + c[f] * ed[f];
          const double dct = W * ec[f], dc = W * ed[f];
          const double s1 = sg[f] * (1.0 - sg[f]);
          gyt[f] = dct * s1;
          gy[f] = dct * Y[((size_t)np + p) * 3 + f] * s1 * (1.0 - 2.0 * sg[f]) / sscale + dc * s1;
        }
        l_r = W * lr;
        const bool keep0 = fabs(e[(size_t)p * 3]) > clip;
        ge0 = keep0 ? W * ct[0] : 0.0;
        get0 = keep0 ? W * c[0] : 0.0;
      }
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      GY[(size_t)p * 3 + f] = gy[f];
      GY[((size_t)np + p) * 3 + f] = gyt[f];
    }
    ge[2 * (size_t)p] = ge0;
    ge[2 * (size_t)p + 1] = get0;
  }
  __shared__ double red[8];
  double v = warp_sum(l_r);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) lpart[blockIdx.x] = v;
  }
}

// Reverse of the residual layer: D = [dL/dh; dL/dh~] in, [dL/dz; dL/dz~] out
// (in place); LayerNorm parameter partials per block:
// part[block][0][W] = dL/dgamma, part[block][1][W] = dL/dbeta.
template <int PL>
__global__ void __launch_bounds__(256) res_ln_elu_tan_bwd_kernel(double *__restrict__ D, const double *__restrict__ Z,
                                                                 const double *__restrict__ gam,
                                                                 const double *__restrict__ bet, double eps,
                                                                 int64_t rows, double *__restrict__ part) {
  constexpr int W = 32 * PL;
  __shared__ double sacc[8][2][W];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t act = (size_t)rows * W;
  double pg[PL], pb[PL];
#pragma unroll
  for (int k = 0; k < PL; ++k) pg[k] = pb[k] = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * 8 + wid; r < rows; r += (int64_t)gridDim.x * 8) {
    const double *z = Z + (size_t)r * W, *zt = Z + act + (size_t)r * W;
    double *dh = D + (size_t)r * W, *dht = D + act + (size_t)r * W;
    double v[PL], vt[PL], s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int k = 0; k < PL; ++k) {
      v[k] = z[lane + 32 * k];
      vt[k] = zt[lane + 32 * k];
      s1 += v[k];
      s2 += v[k] * v[k];
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    const double mean = s1 / W;
    const double var = fmax(0.0, s2 / W - mean * mean);
    const double rs = 1.0 / sqrt(var + eps);
    double xh[PL], m1 = 0.0, m2 = 0.0;
#pragma unroll
    for (int k = 0; k < PL; ++k) {
      xh[k] = (v[k] - mean) * rs;
      m1 += vt[k];
      m2 += xh[k] * vt[k];
    }
    m1 = warp_sum(m1) / W;
    m2 = warp_sum(m2) / W;
    // g_a, g_a~ -> gp = g_a gamma (primal LN input), gt = g_a~ gamma (tangent).
    double gp[PL], gt[PL], xht[PL];
    double sgp = 0.0, sgpx = 0.0, sgt = 0.0, sgtx = 0.0, sgtz = 0.0;
#pragma unroll
    for (int k = 0; k < PL; ++k) {
      const int c = lane + 32 * k;
      xht[k] = rs * (vt[k] - m1 - xh[k] * m2);
      const double a = gam[c] * xh[k] + bet[c];
      const double at = gam[c] * xht[k];
      const double e1 = a > 0.0 ? 1.0 : exp(a);
      const double e2 = a > 0.0 ? 0.0 : exp(a);
      const double gat = dht[c] * e1;
      const double ga = dh[c] * e1 + dht[c] * at * e2;
      pg[k] += ga * xh[k] + gat * xht[k];
      pb[k] += ga;
      gp[k] = ga * gam[c];
      gt[k] = gat * gam[c];
      sgp += gp[k];
      sgpx += gp[k] * xh[k];
      sgt += gt[k];
      sgtx += gt[k] * xh[k];
      sgtz += gt[k] * vt[k];
    }
    const double mgp = warp_sum(sgp) / W, mgpx = warp_sum(sgpx) / W;
    const double mgt = warp_sum(sgt) / W, mgtx = warp_sum(sgtx) / W, mgtz = warp_sum(sgtz) / W;
    const double r2 = rs * rs;
#pragma unroll
    for (int k = 0; k < PL; ++k) {
      const int c = lane + 32 * k;
      const double second =
          -r2 * (xh[k] * (mgtz - mgt * m1 - 3.0 * m2 * mgtx) + mgtx * (vt[k] - m1) + m2 * (gt[k] - mgt));
      dh[c] = rs * (gp[k] - mgp - xh[k] * mgpx) + second;
      dht[c] = rs * (gt[k] - mgt - xh[k] * mgtx);
    }
  }
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    sacc[wid][0][lane + 32 * k] = pg[k];
    sacc[wid][1][lane + 32 * k] = pb[k];
  }
  __syncthreads();
  double *out = part + (size_t)blockIdx.x * 2 * W;
  for (int c = threadIdx.x; c < 2 * W; c += blockDim.x) {
    const int q = c / W, cc = c % W;
    double s = 0.0;
    for (int w8 = 0; w8 < 8; ++w8) s += sacc[w8][q][cc];
    out[c] = s;
  }
}

// Reverse of layer 0: D = [dL/dh0; dL/dh0~] -> [dL/dz0; dL/dz0~] in place.
__global__ void tanh_tan_bwd_kernel(double *__restrict__ D, const double *__restrict__ H,
                                    const double *__restrict__ Z, size_t act) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= act) return;
  const double h = H[i], s = 1.0 - h * h;
  const double gh = D[i], ght = D[act + i];
  D[act + i] = ght * s;
  D[i] = gh * s - 2.0 * h * s * Z[act + i] * ght;
}

// dL/dF per point -> V-contraction coefficients (as dm21_potentials_kernel).
__global__ void hvp_potentials_kernel(const double *__restrict__ featp, const double *__restrict__ featt,
                                      const double *__restrict__ x, const double *__restrict__ xt,
                                      const double *__restrict__ GU, const double *__restrict__ ge, int64_t n_grid,
                                      int64_t np, double clip, double off, double *__restrict__ coef) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double c[2][kFeat];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int k = 0; k < kFeat; ++k) c[s][k] = 0.0;
  if (p < n_grid) {
    double gx[7], gxt[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const double xv = x[(size_t)p * kIn + k], xd = xt[(size_t)p * kIn + k];
      const double den = fabs(xv) + off;
      const double gu = GU[(size_t)p * kInPad + k], gut = GU[((size_t)np + p) * kInPad + k];
      gx[k] = gu * abs_slope(xv) / den - gut * xd / (den * den);
      gxt[k] = gut * abs_slope(xv) / den;
    }
    double rho[2], rt[2], g[2][3], gt[2][3];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const double *f = featp + (size_t)s * kFeat * np;
      const double *ft = featt + (size_t)s * kFeat * np;
      rho[s] = f[F_RHO * np + p];
      rt[s] = ft[F_RHO * np + p];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        g[s][j] = f[(F_GX + j) * np + p];
        gt[s][j] = ft[(F_GX + j) * np + p];
      }
    }
    Dual<2> r2[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      r2[s] = dconst<2>(rho[s]);
      r2[s].d[s] = 1.0;
    }
    const Dual<2> e0 = dm21_lda(r2, clip);
    const double scale = -2.0 * kPi * pow(3.0 / (4.0 * kPi), 4.0 / 3.0);
    const double ge0 = ge[2 * (size_t)p], get0 = ge[2 * (size_t)p + 1];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const double a = fabs(rho[s]);
      const double dclip = a > clip ? 1.0 : (a == clip ? 0.5 : 0.0);
      // e_LDA = scale sum_s max(rho_s, clip)^(4/3): second derivative (4/9) scale rho^(-2/3) above the clip.
      const double d2 = rho[s] > clip ? scale * (4.0 / 9.0) / cbrt(rho[s] * rho[s]) : 0.0;
      c[s][C_RHO] = gx[s] * dclip + ge0 * e0.d[s] + get0 * d2 * rt[s];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double dg = 2.0 * (gx[2] * (g[0][j] + g[1][j]) + gx[3 + s] * g[s][j] +
                                 gxt[2] * (gt[0][j] + gt[1][j]) + gxt[3 + s] * gt[s][j]);
        c[s][C_GX + j] = 2.0 * dg;
      }
      c[s][C_LAP] = 0.0;
      c[s][C_KIN] = 0.5 * gx[5 + s];
    }
  }
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int k = 0; k < kFeat; ++k) coef[((size_t)s * kFeat + k) * np + p] = c[s][k];
}

cudaError_t launch_tan_fwd(int width, double *Z, const double *b, const double *Hp, const double *gam,
                           const double *bet, double eps, int64_t rows, double *H, cudaStream_t st) {
  const unsigned blocks = (unsigned)((rows * 32 + 255) / 256);
  switch (width) {
    case 32: res_ln_elu_tan_fwd_kernel<1><<<blocks, 256, 0, st>>>(Z, b, Hp, gam, bet, eps, rows, H); break;
    case 64: res_ln_elu_tan_fwd_kernel<2><<<blocks, 256, 0, st>>>(Z, b, Hp, gam, bet, eps, rows, H); break;
    case 128: res_ln_elu_tan_fwd_kernel<4><<<blocks, 256, 0, st>>>(Z, b, Hp, gam, bet, eps, rows, H); break;
    case 256: res_ln_elu_tan_fwd_kernel<8><<<blocks, 256, 0, st>>>(Z, b, Hp, gam, bet, eps, rows, H); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_tan_bwd(int width, double *D, const double *Z, const double *gam, const double *bet, double eps,
                           int64_t rows, double *part, cudaStream_t st) {
  switch (width) {
    case 32: res_ln_elu_tan_bwd_kernel<1><<<kLnBlocks, 256, 0, st>>>(D, Z, gam, bet, eps, rows, part); break;
    case 64: res_ln_elu_tan_bwd_kernel<2><<<kLnBlocks, 256, 0, st>>>(D, Z, gam, bet, eps, rows, part); break;
    case 128: res_ln_elu_tan_bwd_kernel<4><<<kLnBlocks, 256, 0, st>>>(D, Z, gam, bet, eps, rows, part); break;
    case 256: res_ln_elu_tan_bwd_kernel<8><<<kLnBlocks, 256, 0, st>>>(D, Z, gam, bet, eps, rows, part); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

size_t hvp_layer_offset(const MlpShape &S, int i) {
  return (size_t)S.n_in * S.width + S.width + (size_t)i * ((size_t)S.width * S.width + 3 * (size_t)S.width);
}

}  // namespace

cudaError_t launch_features_tan(const double *featp, const double *featt, const double *ehf, int64_t n_grid,
                                int64_t np, double clip, double off, double *x, double *xt, double *u, double *e,
                                double *et, cudaStream_t st) {
  features_tan_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(featp, featt, ehf, n_grid, np, clip, off, x, xt,
                                                                   u, e, et);
  return cudaGetLastError();
}

cudaError_t launch_hvp_potentials(const double *featp, const double *featt, const double *x, const double *xt,
                                  const double *GU, const double *ge, int64_t n_grid, int64_t np, double clip,
                                  double off, double *coef, cudaStream_t st) {
  hvp_potentials_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(featp, featt, x, xt, GU, ge, n_grid, np, clip,
                                                                     off, coef);
  return cudaGetLastError();
}

MlpHvpLayout mlp_hvp_layout(const MlpShape &s, int64_t np) {
  MlpHvpLayout L;
  const size_t act2 = 2 * (size_t)np * s.width;
  size_t off = 0;
  auto take = [&](size_t doubles) {
    const size_t o = off;
    off += (doubles + 31) / 32 * 32;
    return o;
  };
  L.nsplit = (int)((2 * np + 65535) / 65536);
  if (L.nsplit < 1) L.nsplit = 1;
  L.eblocks = (int)((np + 255) / 256);
  L.featp = take((size_t)2 * kFeat * np);
  L.x = take((size_t)np * kIn);
  L.xt = take((size_t)np * kIn);
  L.u = take(2 * (size_t)np * kInPad);
  L.e = take((size_t)np * 3);
  L.et = take((size_t)np);
  L.h = take(act2 * (s.n_layers + 1));  // [h_i; h~_i], i = 0..L
  L.z = take(act2 * (s.n_layers + 1));  // [z_i; z~_i], i = 0..L
  L.y = take(2 * (size_t)np * 3);
  L.gy = take(2 * (size_t)np * 3);
  L.ge = take(2 * (size_t)np);
  L.d0 = take(act2);
  L.d1 = take(act2);
  L.gu = take(2 * (size_t)np * kInPad);
  L.kpart = take((size_t)L.nsplit * s.width * s.width);
  L.lnpart = take((size_t)kLnBlocks * 2 * s.width);
  L.colpart = take((size_t)kColBlocks * 2 * s.width);
  L.lpart = take((size_t)L.eblocks);
  L.doubles = off;
  return L;
}

int mlp_hvp_f64(const MlpShape &S, const double *params, double *dparams, const double *featp, const double *featt,
                const double *ehf, const double *w, int64_t n_grid, int64_t np, double clip, double *ws,
                double *lval, double *coef, cudaStream_t st) {
  const MlpHvpLayout L = mlp_hvp_layout(S, np);
  const int Wd = S.width;
  const size_t act = (size_t)np * Wd, act2 = 2 * act;
  double *x = ws + L.x, *xt = ws + L.xt, *U = ws + L.u, *e = ws + L.e, *et = ws + L.et;
  double *H = ws + L.h, *Z = ws + L.z, *Y = ws + L.y, *GY = ws + L.gy, *GE = ws + L.ge;
  double *D0 = ws + L.d0, *D1 = ws + L.d1, *GU = ws + L.gu;
  double *kpart = ws + L.kpart, *lnpart = ws + L.lnpart, *colpart = ws + L.colpart, *lpart = ws + L.lpart;
  const double *W0 = params, *b0 = W0 + (size_t)S.n_in * Wd;
  const size_t head_off = hvp_layer_offset(S, S.n_layers);
  const double *Wout = params + head_off, *bout = Wout + (size_t)Wd * S.n_out;
  const int64_t rows2 = 2 * np;
  const unsigned pb = (unsigned)L.eblocks;
  int rc;
#define GDFT_CK(expr, what)                                    \
  do {                                                         \
    if ((rc = check_cuda((expr), what)) != GDFT_OK) return rc; \
  } while (0)

  // ---- tangent-augmented forward ----
  features_tan_kernel<<<pb, 256, 0, st>>>(featp, featt, ehf, n_grid, np, clip, S.squash_offset, x, xt, U, e, et);
  GDFT_CK(cudaGetLastError(), "hvp features");
  GDFT_CK(gemm<kNN>((int)rows2, Wd, S.n_in, U, kInPad, W0, Wd, Z, Wd, 0.0, st), "hvp dense_0");
  tanh_tan_kernel<<<(unsigned)((act + 255) / 256), 256, 0, st>>>(Z, b0, act, Wd, H);
  GDFT_CK(cudaGetLastError(), "hvp tanh");
  for (int i = 1; i <= S.n_layers; ++i) {
    const double *Wi = params + hvp_layer_offset(S, i - 1), *bi = Wi + (size_t)Wd * Wd, *gi = bi + Wd,
                 *bei = gi + Wd;
    double *Hp = H + (size_t)(i - 1) * act2, *Hi = H + (size_t)i * act2, *Zi = Z + (size_t)i * act2;
    GDFT_CK(gemm<kNN>((int)rows2, Wd, Wd, Hp, Wd, Wi, Wd, Zi, Wd, 0.0, st), "hvp dense_i");
    GDFT_CK(launch_tan_fwd(Wd, Zi, bi, Hp, gi, bei, S.ln_eps, np, Hi, st), "hvp layernorm");
  }
  double *HL = H + (size_t)S.n_layers * act2;
  GDFT_CK(gemm<kNN>((int)rows2, S.n_out, Wd, HL, Wd, Wout, S.n_out, Y, S.n_out, 0.0, st), "hvp head");
  head_tan_kernel<<<pb, 256, 0, st>>>(Y, bout, e, et, w, n_grid, np, clip, S.sigmoid_scale, GY, GE, lpart);
  GDFT_CK(cudaGetLastError(), "hvp head_tan");
  if (lval) GDFT_CK(launch_energy_reduce(lpart, (int)pb, lval, st), "hvp value");

  // ---- reverse of the augmented graph ----
  auto wgrad = [&](int M, int N, const double *A, int lda, const double *B, int ldb, double *C) {
    return gemm_tn_split(M, N, rows2, A, lda, B, ldb, C, L.nsplit, kpart, st);
  };
  auto csum = [&](const double *X, int64_t rows, int ncols, int ld, double *out) {
    return col_sums(X, rows, ncols, ld, out, colpart, kColBlocks, st);
  };
  if (dparams) {
    GDFT_CK(wgrad(Wd, S.n_out, HL, Wd, GY, S.n_out, dparams + head_off), "hvp dW_out");
    GDFT_CK(csum(GY, np, S.n_out, S.n_out, dparams + head_off + (size_t)Wd * S.n_out), "hvp db_out");
  }
  GDFT_CK(gemm<kNT>((int)rows2, Wd, S.n_out, GY, S.n_out, Wout, S.n_out, D0, Wd, 0.0, st), "hvp dh_L");
  double *dcur = D0, *dnext = D1;
  for (int i = S.n_layers; i >= 1; --i) {
    const double *Wi = params + hvp_layer_offset(S, i - 1), *gi = Wi + (size_t)Wd * Wd + Wd, *bei = gi + Wd;
    const double *Hp = H + (size_t)(i - 1) * act2, *Zi = Z + (size_t)i * act2;
    GDFT_CK(launch_tan_bwd(Wd, dcur, Zi, gi, bei, S.ln_eps, np, lnpart, st), "hvp layernorm bwd");
    if (dparams) {
      double *dWi = dparams + hvp_layer_offset(S, i - 1);
      GDFT_CK(wgrad(Wd, Wd, Hp, Wd, dcur, Wd, dWi), "hvp dW_i");
      GDFT_CK(csum(dcur, np, Wd, Wd, dWi + (size_t)Wd * Wd), "hvp db_i");
      GDFT_CK(csum(lnpart, kLnBlocks, 2 * Wd, 2 * Wd, dWi + (size_t)Wd * Wd + Wd), "hvp dLN_i");
    }
    GDFT_CK(cudaMemcpyAsync(dnext, dcur, act2 * sizeof(double), cudaMemcpyDeviceToDevice, st), "hvp residual");
    GDFT_CK(gemm<kNT>((int)rows2, Wd, Wd, dcur, Wd, Wi, Wd, dnext, Wd, 1.0, st), "hvp dh_i");
    double *t = dcur;
    dcur = dnext;
    dnext = t;
  }
  tanh_tan_bwd_kernel<<<(unsigned)((act + 255) / 256), 256, 0, st>>>(dcur, H, Z, act);
  GDFT_CK(cudaGetLastError(), "hvp tanh bwd");
  if (dparams) {
    GDFT_CK(wgrad(S.n_in, Wd, U, kInPad, dcur, Wd, dparams), "hvp dW_0");
    GDFT_CK(csum(dcur, np, Wd, Wd, dparams + (size_t)S.n_in * Wd), "hvp db_0");
  }
  if (coef) {
    GDFT_CK(gemm<kNT>((int)rows2, S.n_in, Wd, dcur, Wd, W0, Wd, GU, kInPad, 0.0, st), "hvp du");
    hvp_potentials_kernel<<<pb, 256, 0, st>>>(featp, featt, x, xt, GU, GE, n_grid, np, clip, S.squash_offset, coef);
    GDFT_CK(cudaGetLastError(), "hvp potentials");
  }
#undef GDFT_CK
  return GDFT_OK;
}

}  // namespace gdft
