// mlp.cu - the DM21-style coefficient network c_theta and its adjoint (FP64 form).
//
// Restates DM21.default_nn + NeuralFunctional.head (functional.py:797-822,
// 407-419) with the features of dm21_coefficient_inputs / dm21_combine_cinputs
// (functional.py:504-531, 628-649), the energy densities of dm21_densities
// ('LDA') / dm21_combine_densities (functional.py:534-626, 652-675), the energy
// of xc_energy (functional.py:219-253) and the reverse-mode pass that
// jax.value_and_grad builds at train.py:86: dE/dtheta, and the per-point
// potentials dE/d(rho, grad rho, tau) that the V_xc contraction consumes.
//
//   x  = [rho_a', rho_b', |grad rho_a + grad rho_b|^2, |grad rho_a|^2,
//         |grad rho_b|^2, tau_a, tau_b, ehf(w0,a), ehf(w1,a), ehf(w0,b), ehf(w1,b)]
//   u  = log(|x| + squash_offset)
//   h0 = tanh(u W0 + b0)
//   h_i = elu(LayerNorm_i(h_{i-1} W_i + b_i + h_{i-1}))      i = 1..L
//   c  = s * sigmoid((h_L W_out + b_out) / s)                 s = sigmoid_scale
//
// The HF inputs ehf are constants of the energy (stop-gradient), as the
// nograd_* plugin slots make them in the reference (functional.py:176, 203-205).
//
// Data layout: activations row-major [np][width] FP64 per layer; every layer's
// output h_i and pre-normalisation sum z_i stay resident for the backward.
// GEMMs are plain tiled FP64; a row of the hidden width is one warp's work.
#include <string.h>

#include "common.cuh"
#include "kernels.cuh"
#include "mlp.cuh"
#include "mlp_gemm.cuh"
#include "xc_functionals.cuh"

namespace gdft {

namespace {

// ------------------------------------------------------------- features ---
// Per point: x (11), u = log(|x| + off) (row stride kDm21InPad), energy densities e (3).
__global__ void dm21_features_kernel(const double *__restrict__ feat, const double *__restrict__ ehf,
                                     int64_t n_grid, int64_t np, double clip, double off, double *__restrict__ x,
                                     double *__restrict__ u, double *__restrict__ e) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double xv[kDm21In];
  double ev[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < kDm21In; ++k) xv[k] = 0.0;
  if (p < n_grid) {
    double rho[2], g[2][3], tau[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const double *f = feat + (size_t)s * kFeat * np;
      rho[s] = f[F_RHO * np + p];
      g[s][0] = f[F_GX * np + p];
      g[s][1] = f[F_GY * np + p];
      g[s][2] = f[F_GZ * np + p];
      tau[s] = f[F_TAU * np + p];
    }
    // dm21_coefficient_inputs (functional.py:504-531): sign-preserving clip of rho.
#pragma unroll
    for (int s = 0; s < 2; ++s) xv[s] = fmax(fabs(rho[s]), clip) * xsign(rho[s]);
    const double t0 = g[0][0] + g[1][0], t1 = g[0][1] + g[1][1], t2 = g[0][2] + g[1][2];
    xv[2] = (t0 * t0 + t1 * t1) + t2 * t2;
#pragma unroll
    for (int s = 0; s < 2; ++s) xv[3 + s] = (g[s][0] * g[s][0] + g[s][1] * g[s][1]) + g[s][2] * g[s][2];
    xv[5] = tau[0];
    xv[6] = tau[1];
    // dm21_combine_cinputs (functional.py:628-649): ehf[:, 0].T then ehf[:, 1].T,
    // ehf laid out [omega][spin][n_grid].
    const double e00 = ehf[(0 * 2 + 0) * n_grid + p], e10 = ehf[(1 * 2 + 0) * n_grid + p];
    const double e01 = ehf[(0 * 2 + 1) * n_grid + p], e11 = ehf[(1 * 2 + 1) * n_grid + p];
    xv[7] = e00;
    xv[8] = e10;
    xv[9] = e01;
    xv[10] = e11;
    // dm21_densities 'LDA' + dm21_combine_densities: [e_LDA, sum_s ehf(w0), sum_s ehf(w1)].
    ev[0] = dm21_lda(rho, clip);
    ev[1] = e00 + e01;
    ev[2] = e10 + e11;
  }
#pragma unroll
  for (int k = 0; k < kDm21In; ++k) {
    x[(size_t)p * kDm21In + k] = xv[k];
    u[(size_t)p * kDm21InPad + k] = log(fabs(xv[k]) + off);
  }
#pragma unroll
  for (int k = kDm21In; k < kDm21InPad; ++k) u[(size_t)p * kDm21InPad + k] = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) e[(size_t)p * 3 + k] = ev[k];
}

// ------------------------------------------------------------ row kernels -

// h0 = tanh(z + b0) in place.
__global__ void tanh_bias_kernel(double *__restrict__ z, const double *__restrict__ b, size_t total, int width) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  z[i] = tanh(z[i] + b[i % width]);
}

// z = zW + b + h_prev (stored back into z); a = LayerNorm(z) as flax computes it
// (var = max(0, E[z^2] - E[z]^2), a = (z - mean) * (rsqrt(var + eps) * scale) + bias);
// h = elu(a).  One warp per row, PL = width / 32 values per lane.
template <int PL>
__global__ void res_ln_elu_fwd_kernel(double *__restrict__ z, const double *__restrict__ b,
                                      const double *__restrict__ hprev, const double *__restrict__ scale,
                                      const double *__restrict__ bias, double eps, int64_t rows,
                                      double *__restrict__ h) {
  constexpr int W = 32 * PL;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  double *zr = z + (size_t)r * W;
  const double *hp = hprev + (size_t)r * W;
  double v[PL], s1 = 0.0, s2 = 0.0;
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    const int c = lane + 32 * k;
    v[k] = (zr[c] + b[c]) + hp[c];
    zr[c] = v[k];
    s1 += v[k];
    s2 += v[k] * v[k];
  }
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  const double mean = s1 / W;
  const double var = fmax(0.0, s2 / W - mean * mean);
  const double rstd = 1.0 / sqrt(var + eps);
  double *hr = h + (size_t)r * W;
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    const int c = lane + 32 * k;
    const double a = (v[k] - mean) * (rstd * scale[c]) + bias[c];
    hr[c] = a > 0.0 ? a : expm1(a);
  }
}

// Backward of res_ln_elu: dh (row) -> dz in place; the LayerNorm parameter
// gradients accumulate per lane over the rows a warp visits and are summed over
// the block's warps in warp order into part[block][2][W] (dscale, dbias).
template <int PL>
__global__ void __launch_bounds__(256) res_ln_elu_bwd_kernel(double *__restrict__ dh, const double *__restrict__ z,
                                                             const double *__restrict__ scale,
                                                             const double *__restrict__ bias, double eps,
                                                             int64_t rows, double *__restrict__ part) {
  constexpr int W = 32 * PL;
  __shared__ double sacc[8][2][W];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double gs[PL], gb[PL];
#pragma unroll
  for (int k = 0; k < PL; ++k) gs[k] = gb[k] = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * 8 + wid; r < rows; r += (int64_t)gridDim.x * 8) {
    const double *zr = z + (size_t)r * W;
    double *dr = dh + (size_t)r * W;
    double zv[PL], s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int k = 0; k < PL; ++k) {
      zv[k] = zr[lane + 32 * k];
      s1 += zv[k];
      s2 += zv[k] * zv[k];
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    const double mean = s1 / W;
    const double var = fmax(0.0, s2 / W - mean * mean);
    const double rstd = 1.0 / sqrt(var + eps);
    double g[PL], xh[PL], m1 = 0.0, m2 = 0.0;
#pragma unroll
    for (int k = 0; k < PL; ++k) {
      const int c = lane + 32 * k;
      xh[k] = (zv[k] - mean) * rstd;
      const double a = (zv[k] - mean) * (rstd * scale[c]) + bias[c];
      const double da = dr[c] * (a > 0.0 ? 1.0 : exp(a));  // elu'(a)
      gs[k] += da * xh[k];
      gb[k] += da;
      g[k] = da * scale[c];
      m1 += g[k];
      m2 += g[k] * xh[k];
    }
    m1 = warp_sum(m1) / W;
    m2 = warp_sum(m2) / W;
#pragma unroll
    for (int k = 0; k < PL; ++k) dr[lane + 32 * k] = rstd * (g[k] - m1 - xh[k] * m2);
  }
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    sacc[wid][0][lane + 32 * k] = gs[k];
    sacc[wid][1][lane + 32 * k] = gb[k];
  }
  __syncthreads();
  double *pb = part + (size_t)blockIdx.x * 2 * W;
  for (int c = threadIdx.x; c < 2 * W; c += blockDim.x) {
    const int q = c / W, cc = c % W;
    double s = 0.0;
    for (int w8 = 0; w8 < 8; ++w8) s += sacc[w8][q][cc];
    pb[c] = s;
  }
}

// dp0 = dh0 * (1 - h0^2) in place.
__global__ void tanh_bwd_kernel(double *__restrict__ dh, const double *__restrict__ h, size_t total) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total) dh[i] *= 1.0 - h[i] * h[i];
}

// Head and energy: c = s * sigmoid((y + b) / s); block partial sums of
// E = sum_r abs_clip(w_r) abs_clip(sum_f c_rf abs_clip(e_rf)); dE/dy; dE/de.
__global__ void __launch_bounds__(256) head_energy_kernel(const double *__restrict__ y,
                                                          const double *__restrict__ bout,
                                                          const double *__restrict__ e,
                                                          const double *__restrict__ w, int64_t n_grid, int64_t np,
                                                          double clip, double sscale, double *__restrict__ dy,
                                                          double *__restrict__ de, double *__restrict__ epart) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double e_r = 0.0;
  if (p < np) {
    double dyv[3] = {0.0, 0.0, 0.0}, dev[3] = {0.0, 0.0, 0.0};
    if (p < n_grid) {
      double c[3], ec[3], sg[3];
      double exc = 0.0;
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const double yv = y[(size_t)p * 3 + f] + bout[f];
        sg[f] = 1.0 / (1.0 + exp(-(yv / sscale)));
        c[f] = sscale * sg[f];
        const double ev = e[(size_t)p * 3 + f];
        ec[f] = fabs(ev) > clip ? ev : 0.0;  // abs_clip of the densities, functional.py:184
        exc = f == 0 ? c[f] * ec[f] : exc + c[f] * ec[f];
      }
      const bool m = fabs(exc) > clip;  // abs_clip of the energy density, functional.py:252, 342
      const double W = fabs(w[p]) > clip ? w[p] : 0.0;
      e_r = m ? W * exc : 0.0;
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const double dc = m ? W * ec[f] : 0.0;
        dyv[f] = dc * (sg[f] * (1.0 - sg[f]));  // d(s sigmoid(y/s))/dy = sigmoid'(y/s)
        dev[f] = (m && fabs(e[(size_t)p * 3 + f]) > clip) ? W * c[f] : 0.0;
      }
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      dy[(size_t)p * 3 + f] = dyv[f];
      de[(size_t)p * 3 + f] = dev[f];
    }
  }
  __shared__ double red[8];
  double v = warp_sum(e_r);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) epart[blockIdx.x] = v;
  }
}

// Per-point adjoint coefficients for the V_xc contraction from dE/du (network
// input) and dE/de_LDA.  d|x|/dx follows jax (+1 at x = 0).  d rho'/d rho is
// the derivative of maximum(|rho|, clip) * sign(rho): 1 above the clip, 1/2 at
// the tie (jax splits the gradient of maximum evenly), 0 below.
__global__ void dm21_potentials_kernel(const double *__restrict__ feat, const double *__restrict__ x,
                                       const double *__restrict__ du, const double *__restrict__ de, int64_t n_grid,
                                       int64_t np, double clip, double off, double *__restrict__ coef) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double c[2][kFeat];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int k = 0; k < kFeat; ++k) c[s][k] = 0.0;
  if (p < n_grid) {
    double dx[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const double xv = x[(size_t)p * kDm21In + k];
      dx[k] = du[(size_t)p * kDm21InPad + k] * (xv >= 0.0 ? 1.0 : -1.0) / (fabs(xv) + off);
    }
    double rho[2], g[2][3];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const double *f = feat + (size_t)s * kFeat * np;
      rho[s] = f[F_RHO * np + p];
      g[s][0] = f[F_GX * np + p];
      g[s][1] = f[F_GY * np + p];
      g[s][2] = f[F_GZ * np + p];
    }
    Dual<2> r2[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      r2[s] = dconst<2>(rho[s]);
      r2[s].d[s] = 1.0;
    }
    const Dual<2> e0 = dm21_lda(r2, clip);
    const double de0 = de[(size_t)p * 3 + 0];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const double a = fabs(rho[s]);
      const double drho_clip = a > clip ? 1.0 : (a == clip ? 0.5 : 0.0);
      c[s][C_RHO] = dx[s] * drho_clip + de0 * e0.d[s];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        // dE/d(grad rho_s)_j; grad rho = 2 sum D phi d_j phi puts a factor 2 on phi_a d_j phi_b.
        const double dg = dx[2] * 2.0 * (g[0][j] + g[1][j]) + dx[3 + s] * 2.0 * g[s][j];
        c[s][C_GX + j] = 2.0 * dg;
      }
      c[s][C_LAP] = 0.0;
      c[s][C_KIN] = 0.5 * dx[5 + s];  // tau = 1/2 sum_j D d_j phi d_j phi
    }
  }
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int k = 0; k < kFeat; ++k) coef[((size_t)s * kFeat + k) * np + p] = c[s][k];
}


cudaError_t launch_res_ln_elu_fwd(int width, double *z, const double *b, const double *hprev, const double *scale,
                                  const double *bias, double eps, int64_t rows, double *h, cudaStream_t st) {
  const unsigned blocks = (unsigned)((rows * 32 + 255) / 256);
  switch (width) {
    case 32: res_ln_elu_fwd_kernel<1><<<blocks, 256, 0, st>>>(z, b, hprev, scale, bias, eps, rows, h); break;
    case 64: res_ln_elu_fwd_kernel<2><<<blocks, 256, 0, st>>>(z, b, hprev, scale, bias, eps, rows, h); break;
    case 128: res_ln_elu_fwd_kernel<4><<<blocks, 256, 0, st>>>(z, b, hprev, scale, bias, eps, rows, h); break;
    case 256: res_ln_elu_fwd_kernel<8><<<blocks, 256, 0, st>>>(z, b, hprev, scale, bias, eps, rows, h); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_res_ln_elu_bwd(int width, double *dh, const double *z, const double *scale, const double *bias,
                                  double eps, int64_t rows, double *part, cudaStream_t st) {
  switch (width) {
    case 32: res_ln_elu_bwd_kernel<1><<<kLnBlocks, 256, 0, st>>>(dh, z, scale, bias, eps, rows, part); break;
    case 64: res_ln_elu_bwd_kernel<2><<<kLnBlocks, 256, 0, st>>>(dh, z, scale, bias, eps, rows, part); break;
    case 128: res_ln_elu_bwd_kernel<4><<<kLnBlocks, 256, 0, st>>>(dh, z, scale, bias, eps, rows, part); break;
    case 256: res_ln_elu_bwd_kernel<8><<<kLnBlocks, 256, 0, st>>>(dh, z, scale, bias, eps, rows, part); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_dm21_features(const double *feat, const double *ehf, int64_t n_grid, int64_t np, double clip,
                                 double off, double *x, double *u, double *e, cudaStream_t st) {
  dm21_features_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(feat, ehf, n_grid, np, clip, off, x, u, e);
  return cudaGetLastError();
}

// dE/d ehf[w][s][r] of the DM21 network (for the HF Fock terms, molecule.py:545-685):
//   through the densities: the HF energy-density column of omega w is the spin
//   sum of ehf[w] (dm21_combine_densities, functional.py:652-675), so the
//   gradient is dE/de_{1+w} for both spins;
//   through the inputs: ehf[w][s] is input 7 + 2 s + w (dm21_combine_cinputs,
//   functional.py:628-649), entering as log(|x| + offset).
__global__ void dm21_hf_grads_kernel(const double *__restrict__ x, const double *__restrict__ du,
                                     const double *__restrict__ de, int64_t n_grid, double off,
                                     double *__restrict__ g_dens, double *__restrict__ g_cin) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_grid) return;
#pragma unroll
  for (int w = 0; w < 2; ++w)
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const size_t o = ((size_t)w * 2 + s) * n_grid + p;
      if (g_dens) g_dens[o] = de[(size_t)p * 3 + 1 + w];
      if (g_cin) {
        const int k = 7 + 2 * s + w;
        const double xv = x[(size_t)p * kDm21In + k];
        g_cin[o] = du[(size_t)p * kDm21InPad + k] * (xv >= 0.0 ? 1.0 : -1.0) / (fabs(xv) + off);
      }
    }
}

cudaError_t launch_dm21_hf_grads(const MlpShape &S, int64_t n_grid, int64_t np, const double *ws, double *g_dens,
                                 double *g_cin, cudaStream_t st) {
  const MlpLayout L = mlp_layout(S, np);
  return launch_dm21_hf_grads_from(ws + L.x, ws + L.du, ws + L.de, n_grid, S.squash_offset, g_dens, g_cin, st);
}

cudaError_t launch_dm21_hf_grads_from(const double *x, const double *du, const double *de, int64_t n_grid,
                                      double squash_offset, double *g_dens, double *g_cin, cudaStream_t st) {
  dm21_hf_grads_kernel<<<(unsigned)((n_grid + 255) / 256), 256, 0, st>>>(x, du, de, n_grid, squash_offset, g_dens,
                                                                          g_cin);
  return cudaGetLastError();
}

cudaError_t launch_dm21_potentials(const double *feat, const double *x, const double *du, const double *de,
                                   int64_t n_grid, int64_t np, double clip, double off, double *coef,
                                   cudaStream_t st) {
  dm21_potentials_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(feat, x, du, de, n_grid, np, clip, off,
                                                                      coef);
  return cudaGetLastError();
}

bool mlp_width_supported(int width) { return width == 32 || width == 64 || width == 128 || width == 256; }

size_t mlp_param_count(const MlpShape &s) {
  size_t n = (size_t)s.n_in * s.width + s.width;
  n += (size_t)s.n_layers * ((size_t)s.width * s.width + 3 * (size_t)s.width);
  n += (size_t)s.width * s.n_out + s.n_out;
  return n;
}

MlpLayout mlp_layout(const MlpShape &s, int64_t np) {
  MlpLayout L;
  const size_t act = (size_t)np * s.width;
  size_t off = 0;
  auto take = [&](size_t doubles) {
    const size_t o = off;
    off += (doubles + 31) / 32 * 32;  // 256-byte granules
    return o;
  };
  L.nsplit = (int)((np + 65535) / 65536);
  if (L.nsplit < 1) L.nsplit = 1;
  L.eblocks = (int)((np + 255) / 256);
  L.x = take((size_t)np * kDm21In);
  L.u = take((size_t)np * kDm21InPad);
  L.e = take((size_t)np * 3);
  L.h = take(act * (s.n_layers + 1));  // h_0 .. h_L
  L.z = take(act * s.n_layers);        // z_1 .. z_L
  L.y = take((size_t)np * 3);
  L.dy = take((size_t)np * 3);
  L.de = take((size_t)np * 3);
  L.d0 = take(act);
  L.d1 = take(act);
  L.du = take((size_t)np * kDm21InPad);
  L.kpart = take((size_t)L.nsplit * s.width * s.width);
  L.lnpart = take((size_t)kLnBlocks * 2 * s.width);
  L.colpart = take((size_t)kColBlocks * 2 * s.width);
  L.epart = take((size_t)L.eblocks);
  L.doubles = off;
  return L;
}

namespace {

size_t layer_offset(const MlpShape &S, int i) {
  return (size_t)S.n_in * S.width + S.width + (size_t)i * ((size_t)S.width * S.width + 3 * (size_t)S.width);
}

// u (np x kDm21InPad) -> h_0 .. h_L, z_1 .. z_L and y = h_L W_out (head bias not added).
int net_forward(const MlpShape &S, const double *params, const MlpLayout &L, double *ws, int64_t np,
                cudaStream_t st) {
  const int Wd = S.width;
  const size_t act = (size_t)np * Wd;
  double *u = ws + L.u, *h = ws + L.h, *z = ws + L.z, *y = ws + L.y;
  const double *W0 = params, *b0 = W0 + (size_t)S.n_in * Wd;
  const double *Wout = params + layer_offset(S, S.n_layers);
  int rc;
  if ((rc = check_cuda(gemm<kNN>((int)np, Wd, S.n_in, u, kDm21InPad, W0, Wd, h, Wd, 0.0, st), "mlp dense_0")))
    return rc;
  tanh_bias_kernel<<<(unsigned)((act + 255) / 256), 256, 0, st>>>(h, b0, act, Wd);
  if ((rc = check_cuda(cudaGetLastError(), "mlp tanh"))) return rc;
  for (int i = 1; i <= S.n_layers; ++i) {
    const double *Wi = params + layer_offset(S, i - 1), *bi = Wi + (size_t)Wd * Wd, *gi = bi + Wd, *bei = gi + Wd;
    const double *hprev = h + (size_t)(i - 1) * act;
    double *hi = h + (size_t)i * act, *zi = z + (size_t)(i - 1) * act;
    if ((rc = check_cuda(gemm<kNN>((int)np, Wd, Wd, hprev, Wd, Wi, Wd, zi, Wd, 0.0, st), "mlp dense_i"))) return rc;
    if ((rc = check_cuda(launch_res_ln_elu_fwd(Wd, zi, bi, hprev, gi, bei, S.ln_eps, np, hi, st), "mlp layernorm")))
      return rc;
  }
  const double *hL = h + (size_t)S.n_layers * act;
  return check_cuda(gemm<kNN>((int)np, S.n_out, Wd, hL, Wd, Wout, S.n_out, y, S.n_out, 0.0, st), "mlp head");
}

// u = log(|x| + off) for given network inputs x (rows x n_in).
__global__ void squash_kernel(const double *__restrict__ x, int64_t rows, int n_in, double off,
                              double *__restrict__ u) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= rows) return;
  for (int k = 0; k < kDm21InPad; ++k) u[(size_t)p * kDm21InPad + k] = k < n_in ? log(fabs(x[(size_t)p * n_in + k]) + off) : 0.0;
}

// c = s * sigmoid((y + b) / s), written (rows x n_out).
__global__ void head_coeff_kernel(const double *__restrict__ y, const double *__restrict__ bout, int64_t rows,
                                  int n_out, double sscale, double *__restrict__ c) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * n_out) return;
  const double yv = y[i] + bout[i % n_out];
  c[i] = sscale * (1.0 / (1.0 + exp(-(yv / sscale))));
}

}  // namespace

int mlp_inputs_f64(const MlpShape &S, const double *feat, const double *ehf, int64_t n_grid, int64_t np,
                   double clip, double *ws, double *x_out, double *e_out, cudaStream_t st) {
  const MlpLayout L = mlp_layout(S, np);
  dm21_features_kernel<<<(unsigned)L.eblocks, 256, 0, st>>>(feat, ehf, n_grid, np, clip, S.squash_offset, ws + L.x,
                                                            ws + L.u, ws + L.e);
  int rc = check_cuda(cudaGetLastError(), "dm21_features");
  if (rc) return rc;
  if (x_out &&
      (rc = check_cuda(cudaMemcpyAsync(x_out, ws + L.x, (size_t)n_grid * kDm21In * sizeof(double),
                                       cudaMemcpyDeviceToDevice, st),
                       "dm21 inputs copy")))
    return rc;
  if (e_out)
    rc = check_cuda(cudaMemcpyAsync(e_out, ws + L.e, (size_t)n_grid * 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                                    st),
                    "dm21 densities copy");
  return rc;
}

int mlp_apply_f64(const MlpShape &S, const double *params, const double *x, int64_t rows, double *ws, double *c,
                  cudaStream_t st) {
  const MlpLayout L = mlp_layout(S, rows);
  squash_kernel<<<(unsigned)((rows + 255) / 256), 256, 0, st>>>(x, rows, S.n_in, S.squash_offset, ws + L.u);
  int rc = check_cuda(cudaGetLastError(), "mlp squash");
  if (rc) return rc;
  if ((rc = net_forward(S, params, L, ws, rows, st))) return rc;
  const double *bout = params + layer_offset(S, S.n_layers) + (size_t)S.width * S.n_out;
  head_coeff_kernel<<<(unsigned)((rows * S.n_out + 255) / 256), 256, 0, st>>>(ws + L.y, bout, rows, S.n_out,
                                                                             S.sigmoid_scale, c);
  return check_cuda(cudaGetLastError(), "mlp head_coeff");
}

// Flat parameter order: Dense_0 (kernel n_in x W, bias W); for layer i = 1..L:
// Dense_i (kernel W x W, bias W), LayerNorm_{i-1} (scale W, bias W); head
// Dense_{L+1} (kernel W x n_out, bias n_out).  dparams uses the same order.
int mlp_run_f64(const MlpShape &S, const double *params, double *dparams, const double *feat, const double *ehf,
                const double *w, int64_t n_grid, int64_t np, double clip, double *ws, double *exc, double *coef,
                cudaStream_t st) {
  const MlpLayout L = mlp_layout(S, np);
  const int Wd = S.width;
  double *x = ws + L.x, *u = ws + L.u, *e = ws + L.e, *h = ws + L.h, *z = ws + L.z, *y = ws + L.y;
  double *dy = ws + L.dy, *de = ws + L.de, *d0 = ws + L.d0, *d1 = ws + L.d1, *du = ws + L.du;
  double *kpart = ws + L.kpart, *lnpart = ws + L.lnpart, *colpart = ws + L.colpart, *epart = ws + L.epart;
  const size_t act = (size_t)np * Wd;
  auto layer_off = [&](int i) { return layer_offset(S, i); };
  const size_t head_off = layer_off(S.n_layers);
  const double *W0 = params;
  const double *Wout = params + head_off, *bout = Wout + (size_t)Wd * S.n_out;
  double *hL = h + (size_t)S.n_layers * act;
  const unsigned pb = (unsigned)L.eblocks;
  int rc;
#define GDFT_CK(expr, what)                                    \
  do {                                                         \
    if ((rc = check_cuda((expr), what)) != GDFT_OK) return rc; \
  } while (0)

  // ---- forward ----
  dm21_features_kernel<<<pb, 256, 0, st>>>(feat, ehf, n_grid, np, clip, S.squash_offset, x, u, e);
  GDFT_CK(cudaGetLastError(), "dm21_features");
  if ((rc = net_forward(S, params, L, ws, np, st)) != GDFT_OK) return rc;
  head_energy_kernel<<<pb, 256, 0, st>>>(y, bout, e, w, n_grid, np, clip, S.sigmoid_scale, dy, de, epart);
  GDFT_CK(cudaGetLastError(), "mlp head_energy");
  GDFT_CK(launch_energy_reduce(epart, (int)pb, exc, st), "mlp energy_reduce");
  if (coef == nullptr && dparams == nullptr) return GDFT_OK;

  // ---- backward ----
  const int ns = L.nsplit;
  auto weight_grad = [&](int M, int N, const double *A, int lda, const double *B, int ldb, double *C) {
    return gemm_tn_split(M, N, np, A, lda, B, ldb, C, ns, kpart, st);
  };
  auto col_sum = [&](const double *X, int64_t rows, int ncols, int ld, double *out) {
    return col_sums(X, rows, ncols, ld, out, colpart, kColBlocks, st);
  };
  // Head: dW_out = h_L^T dy, db_out = sum_r dy, dh_L = dy W_out^T.
  if (dparams) {
    GDFT_CK(weight_grad(Wd, S.n_out, hL, Wd, dy, S.n_out, dparams + head_off), "mlp dW_out");
    GDFT_CK(col_sum(dy, np, S.n_out, S.n_out, dparams + head_off + (size_t)Wd * S.n_out), "mlp db_out");
  }
  GDFT_CK(gemm<kNT>((int)np, Wd, S.n_out, dy, S.n_out, Wout, S.n_out, d0, Wd, 0.0, st), "mlp dh_L");
  double *dcur = d0, *dnext = d1;
  for (int i = S.n_layers; i >= 1; --i) {
    const double *Wi = params + layer_off(i - 1), *gi = Wi + (size_t)Wd * Wd + Wd, *bei = gi + Wd;
    const double *hprev = h + (size_t)(i - 1) * act, *zi = z + (size_t)(i - 1) * act;
    GDFT_CK(launch_res_ln_elu_bwd(Wd, dcur, zi, gi, bei, S.ln_eps, np, lnpart, st), "mlp layernorm bwd");
    if (dparams) {
      double *dWi = dparams + layer_off(i - 1);
      GDFT_CK(weight_grad(Wd, Wd, hprev, Wd, dcur, Wd, dWi), "mlp dW_i");
      GDFT_CK(col_sum(dcur, np, Wd, Wd, dWi + (size_t)Wd * Wd), "mlp db_i");
      GDFT_CK(col_sum(lnpart, kLnBlocks, 2 * Wd, 2 * Wd, dWi + (size_t)Wd * Wd + Wd), "mlp dLN_i");
    }
    // dh_{i-1} = dz (residual) + dz W_i^T.
    GDFT_CK(cudaMemcpyAsync(dnext, dcur, act * sizeof(double), cudaMemcpyDeviceToDevice, st), "mlp residual");
    GDFT_CK(gemm<kNT>((int)np, Wd, Wd, dcur, Wd, Wi, Wd, dnext, Wd, 1.0, st), "mlp dh_i");
    double *t = dcur;
    dcur = dnext;
    dnext = t;
  }
  // Layer 0: dp0 = dh0 (1 - h0^2); dW0 = u^T dp0; db0 = sum_r dp0; du = dp0 W0^T.
  tanh_bwd_kernel<<<(unsigned)((act + 255) / 256), 256, 0, st>>>(dcur, h, act);
  GDFT_CK(cudaGetLastError(), "mlp tanh bwd");
  if (dparams) {
    GDFT_CK(weight_grad(S.n_in, Wd, u, kDm21InPad, dcur, Wd, dparams), "mlp dW_0");
    GDFT_CK(col_sum(dcur, np, Wd, Wd, dparams + (size_t)S.n_in * Wd), "mlp db_0");
  }
  if (coef != nullptr) {
    GDFT_CK(gemm<kNT>((int)np, S.n_in, Wd, dcur, Wd, W0, Wd, du, kDm21InPad, 0.0, st), "mlp du");
    dm21_potentials_kernel<<<pb, 256, 0, st>>>(feat, x, du, de, n_grid, np, clip, S.squash_offset, coef);
    GDFT_CK(cudaGetLastError(), "dm21_potentials");
  }
#undef GDFT_CK
  return GDFT_OK;
}

}  // namespace gdft
