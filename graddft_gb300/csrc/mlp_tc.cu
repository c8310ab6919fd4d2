// mlp_tc.cu - mixed form of the DM21-style network: hidden-layer GEMMs on the
// tensor cores (TF32x3, tc_gemm.cu), FP32 activations, FP64 row statistics.
//
// Same computation and adjoint as mlp.cu (DM21.default_nn + head,
// functional.py:797-822, 407-419; jax.value_and_grad at train.py:86):
//   forward  z_i = h_{i-1} W_i            tcgen05, A = row-tile pack of h, B = column-tile pack of W_i
//   backward dh_{i-1} = dz_i W_i^T       tcgen05, A = row-tile pack of dz, B = row-tile pack of W_i
//            dW_i = h_{i-1}^T dz_i       tcgen05 split-K over grid points, FP64 partials,
//                                        A / B = column-tile packs of h_{i-1} / dz_i
// The 11-wide input layer's gradient, the 3-wide head and the bias / LayerNorm
// parameter sums run on the CUDA cores in FP64 from FP32 activations.  Row
// kernels: one warp per row of the hidden width, FP64 statistics.
#include "common.cuh"
#include "kernels.cuh"
#include "mlp.cuh"
#include "mlp_gemm.cuh"
#include "mlp_rows.cuh"
#include "tc_gemm.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr size_t kBlk = 2 * (umma::kBlockBytes / 4);  // floats in one packed hi|lo block pair

// Per-element arithmetic and per-row statistics of these row kernels are FP32
// (GB300's FP64 rate is a small fraction of its FP32 rate, and the activations
// are FP32); long accumulations over grid points and the energy stay FP64.

// Forward row pass fused with the packing of its output h:
//   L0:    z = zW + b (stored back), h = tanh(z)
//   else:  z = zW + b + h_prev (stored back), h = elu(LayerNorm(z)) (in place of h_prev)
// h is written to H and, where the pointers are given, packed as the rt
// operand of the next dense layer and the ct operand of its weight gradient.
// rows is a multiple of 32.
template <int PL, bool L0>
__global__ void __launch_bounds__(256) layer_fwd_pack_kernel(float *__restrict__ Z, const float *__restrict__ b,
                                                             float *__restrict__ H, const float *__restrict__ gam,
                                                             const float *__restrict__ bet, double eps, int64_t rows,
                                                             float *__restrict__ rt_out, float *__restrict__ ct_out) {
  constexpr int W = 32 * PL, LD = W + 4;
  __shared__ __align__(16) float tile[kRowTile * LD];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float bf[PL], gf[PL], ef[PL];
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    const int c = lane + 32 * k;
    bf[k] = b[c];
    gf[k] = L0 ? 0.0f : gam[c];
    ef[k] = L0 ? 0.0f : bet[c];
  }
  for (int64_t r0 = (int64_t)blockIdx.x * kRowTile; r0 < rows; r0 += (int64_t)gridDim.x * kRowTile) {
    // All four rows' loads first (Z and H are written below).
    float v[4][PL];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const size_t base = (size_t)(r0 + wid * 4 + i) * W;
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const int c = lane + 32 * k;
        v[i][k] = L0 ? Z[base + c] + bf[k] : (Z[base + c] + bf[k]) + H[base + c];
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int rr = wid * 4 + i;
      const size_t base = (size_t)(r0 + rr) * W;
      float mean = 0.0f, rs = 1.0f;
      if (!L0) {
        float s1 = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) s1 += v[i][k];
        mean = warp_sumf(s1) * (1.0f / W);
        float s2 = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          const float d = v[i][k] - mean;
          s2 += d * d;
        }
        rs = 1.0f / sqrtf(warp_sumf(s2) * (1.0f / W) + (float)eps);
      }
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const int c = lane + 32 * k;
        const float h = L0 ? tanhf(v[i][k]) : eluf((v[i][k] - mean) * (rs * gf[k]) + ef[k]);
        Z[base + c] = v[i][k];
        H[base + c] = h;
        tile[rr * LD + c] = h;
      }
    }
    __syncthreads();
    store_tile_packs<PL>(tile, r0, rt_out, ct_out, rows / 32);
    __syncthreads();
  }
}

// Reverse of a residual layer fused with the packing of dE/dz as the rt
// operand of dh = dz W^T and the ct operand of dW = h^T dz.  The incoming
// dE/dh is dy W_out^T (last layer: dy != null) or dhp + gres (the GEMM output
// plus the residual branch of the layer above).  Writes dE/dz (FP32) and
// per-block partial sums [block][3][W] of dE/dgamma, dE/dbeta and dE/db
// (= sum dz): FP32 over 16 rows of a warp at a time, then Kahan-compensated
// FP32 per warp, FP64 across the block's warps.
// rows is a multiple of 32; part has gridDim.x blocks of [3][W].
template <int PL>
__global__ void __launch_bounds__(256, 2) layer_bwd_pack_kernel(
    const float *__restrict__ dhp, const float *__restrict__ gres, const double *__restrict__ dy,
    const float *__restrict__ Wo, const float *__restrict__ Z, const float *__restrict__ gam,
    const float *__restrict__ bet, double eps, int64_t rows, float *__restrict__ gz, double *__restrict__ part,
    float *__restrict__ rt_out, float *__restrict__ ct_out) {
  constexpr int W = 32 * PL, LD = W + 4;
  // Dynamic shared memory (bwd_pack_smem<PL>() bytes): per-warp Kahan sums
  // (total, compensation) of dgamma, dbeta, db in FP32 (GB300's FP64 rate is a
  // small fraction of its FP32 rate), then the row tile.
  extern __shared__ __align__(16) unsigned char bwd_smem[];
  float2(*sacc)[3][W] = reinterpret_cast<float2(*)[3][W]>(bwd_smem);
  float *tile = reinterpret_cast<float *>(bwd_smem + sizeof(float2) * 8 * 3 * W);
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float gmf[PL], btf[PL];
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    const int c = lane + 32 * k;
    gmf[k] = gam[c];
    btf[k] = bet[c];
    sacc[wid][0][c] = sacc[wid][1][c] = sacc[wid][2][c] = make_float2(0.0f, 0.0f);
  }
  float fg[PL], fb[PL], fd[PL];
#pragma unroll
  for (int k = 0; k < PL; ++k) fg[k] = fb[k] = fd[k] = 0.0f;
  int ntile = 0;
  for (int64_t r0 = (int64_t)blockIdx.x * kRowTile; r0 < rows; r0 += (int64_t)gridDim.x * kRowTile) {
#pragma unroll 1
    for (int i2 = 0; i2 < 4; i2 += 2) {
      float zv[2][PL], gh[2][PL];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int64_t r = r0 + wid * 4 + i2 + i;
        const size_t base = (size_t)r * W;
        float dy0 = 0.0f, dy1 = 0.0f, dy2 = 0.0f;
        if (dy) {
          dy0 = (float)dy[r * 3 + 0];
          dy1 = (float)dy[r * 3 + 1];
          dy2 = (float)dy[r * 3 + 2];
        }
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          const int c = lane + 32 * k;
          zv[i][k] = Z[base + c];
          gh[i][k] = dy ? fmaf(dy0, __ldg(Wo + c * 3), fmaf(dy1, __ldg(Wo + c * 3 + 1), dy2 * __ldg(Wo + c * 3 + 2)))
                        : dhp[base + c] + gres[base + c];
        }
      }
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int rr = wid * 4 + i2 + i;
        const size_t base = (size_t)(r0 + rr) * W;
        float s1 = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) s1 += zv[i][k];
        const float mean = warp_sumf(s1) * (1.0f / W);
        float s2 = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          const float d = zv[i][k] - mean;
          s2 += d * d;
        }
        const float rs = 1.0f / sqrtf(warp_sumf(s2) * (1.0f / W) + (float)eps);
        float g[PL], xh[PL], m1 = 0.0f, m2 = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          xh[k] = (zv[i][k] - mean) * rs;
          const float a = xh[k] * gmf[k] + btf[k];
          const float da = gh[i][k] * (a > 0.0f ? 1.0f : expf(a));
          fg[k] = fmaf(da, xh[k], fg[k]);
          fb[k] += da;
          g[k] = da * gmf[k];
          m1 += g[k];
          m2 += g[k] * xh[k];
        }
        const float mm1 = warp_sumf(m1) * (1.0f / W), mm2 = warp_sumf(m2) * (1.0f / W);
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          const int c = lane + 32 * k;
          const float d = rs * (g[k] - mm1 - xh[k] * mm2);
          fd[k] += d;
          gz[base + c] = d;
          tile[rr * LD + c] = d;
        }
      }
    }
    if (++ntile == 4) {  // 16 rows per warp: FP32 partials into the Kahan sums
      ntile = 0;
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const int c = lane + 32 * k;
        kahan_add(sacc[wid][0][c], fg[k]);
        kahan_add(sacc[wid][1][c], fb[k]);
        kahan_add(sacc[wid][2][c], fd[k]);
        fg[k] = fb[k] = fd[k] = 0.0f;
      }
    }
    __syncthreads();
    store_tile_packs<PL>(tile, r0, rt_out, ct_out, rows / 32);
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    const int c = lane + 32 * k;
    kahan_add(sacc[wid][0][c], fg[k]);
    kahan_add(sacc[wid][1][c], fb[k]);
    kahan_add(sacc[wid][2][c], fd[k]);
  }
  __syncthreads();
  double *out = part + (size_t)blockIdx.x * 3 * W;
  for (int c = threadIdx.x; c < 3 * W; c += blockDim.x) {
    const int q = c / W, cc = c % W;
    double sum = 0.0;
    for (int w8 = 0; w8 < 8; ++w8) sum += (double)sacc[w8][q][cc].x - (double)sacc[w8][q][cc].y;
    out[c] = sum;
  }
}

// Head and energy: each warp takes 32 rows; y = h W_out (FP32 row sums) for
// row i lands in lane i, which then evaluates c = s sigmoid((y + b_out) / s),
// its energy term, dE/dy and dE/de in FP64 (as head_energy_kernel).  E
// partials per block of 256 rows.
template <int PL>
__global__ void __launch_bounds__(256) head_kernel(const float *__restrict__ H, const float *__restrict__ Wo,
                                                   const double *__restrict__ bo, const double *__restrict__ e,
                                                   const double *__restrict__ w, int64_t n_grid, int64_t rows,
                                                   double clip, double sscale, double *__restrict__ dy,
                                                   float *__restrict__ dyf, double *__restrict__ de,
                                                   double *__restrict__ epart) {
  constexpr int W = 32 * PL;
  __shared__ double red[8];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t base = ((int64_t)blockIdx.x * 8 + wid) * 32;
  float wo[PL][3];
#pragma unroll
  for (int k = 0; k < PL; ++k)
#pragma unroll
    for (int f = 0; f < 3; ++f) wo[k][f] = Wo[(lane + 32 * k) * 3 + f];
  float my[3] = {0.0f, 0.0f, 0.0f};
  for (int i0 = 0; i0 < 32; i0 += 4) {  // four rows' loads in flight at a time
    float hv[4][PL];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t r = base + i0 + i;
#pragma unroll
      for (int k = 0; k < PL; ++k) hv[i][k] = r < rows ? H[(size_t)r * W + lane + 32 * k] : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float yf[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int k = 0; k < PL; ++k)
#pragma unroll
        for (int f = 0; f < 3; ++f) yf[f] = fmaf(hv[i][k], wo[k][f], yf[f]);
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const float t = warp_sumf(yf[f]);
        if (lane == i0 + i) my[f] = t;
      }
    }
  }
  const int64_t r = base + lane;
  double e_r = 0.0;
  if (r < rows) {
    double dyv[3] = {0.0, 0.0, 0.0}, dev[3] = {0.0, 0.0, 0.0};
    if (r < n_grid) {
      double c[3], ec[3], sg[3], exc = 0.0;
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        sg[f] = 1.0 / (1.0 + exp(-(((double)my[f] + bo[f]) / sscale)));
        c[f] = sscale * sg[f];
        const double ev = e[(size_t)r * 3 + f];
        ec[f] = fabs(ev) > clip ? ev : 0.0;
        exc = f == 0 ? c[f] * ec[f] : exc + c[f] * ec[f];
      }
      const bool m = fabs(exc) > clip;
      const double Wt = fabs(w[r]) > clip ? w[r] : 0.0;
      e_r = m ? Wt * exc : 0.0;
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        dyv[f] = (m ? Wt * ec[f] : 0.0) * (sg[f] * (1.0 - sg[f]));
        dev[f] = (m && fabs(e[(size_t)r * 3 + f]) > clip) ? Wt * c[f] : 0.0;
      }
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      dy[(size_t)r * 3 + f] = dyv[f];
      dyf[(size_t)r * 3 + f] = (float)dyv[f];
      de[(size_t)r * 3 + f] = dev[f];
    }
  }
  const double ws = warp_sum(e_r);
  if (lane == 0) red[wid] = ws;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < 8; ++i) t += red[i];
    epart[blockIdx.x] = t;
  }
}

// Layer 0 reverse fused with everything that consumes it.  dz0 = (dhp + gres)
// (1 - tanh(z0)^2) (FP32; the residual layer above passes dhp = dz_1 W_1^T and
// gres = dz_1) is formed per 32-row tile and not stored; from it
//   du[r][j] = sum_c dz0[r][c] W0[j][c]            (du != null; FP32 lane
//                                                   products, FP64 warp sums)
//   part[block][j][c] = sum_r u[r][j] dz0[r][c]    (j < n_in: dW0)
//   part[block][n_in][c] = sum_r dz0[r][c]         (db0)
// with the parameter sums in FP32 over 16 rows, then Kahan-compensated FP32
// per block (FP64 partials out), one thread per column.  Dynamic shared
// memory: l0_bwd_smem<PL>() bytes.
template <int PL>
constexpr size_t l0_bwd_smem() {
  return sizeof(float) * (kRowTile * (32 * PL + 4) + kRowTile * kDm21InPad + kDm21InPad * 32 * PL);
}

template <int PL>
__global__ void __launch_bounds__(256, 2) l0_bwd_fused_kernel(const float *__restrict__ dhp,
                                                           const float *__restrict__ gres,
                                                           const float *__restrict__ Z0, const double *__restrict__ u,
                                                           const float *__restrict__ W0, int n_in, int64_t rows,
                                                           double *__restrict__ du, double *__restrict__ part) {
  constexpr int W = 32 * PL, LD = W + 4, NJ = kDm21InPad + 1;
  extern __shared__ __align__(16) unsigned char l0_smem[];
  float *tile = reinterpret_cast<float *>(l0_smem);  // [32][LD] dz0
  float *uf = tile + kRowTile * LD;                   // [32][kDm21InPad] u (FP32)
  float *w0s = uf + kRowTile * kDm21InPad;            // [kDm21InPad][W] W0, zero rows past n_in
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < kDm21InPad * W; i += blockDim.x) w0s[i] = i / W < n_in ? W0[i] : 0.0f;
  const int c = threadIdx.x;  // column of the parameter sums (c < W)
  // FP32 sums over 16 rows (fac) folded into Kahan-compensated FP32 totals
  // (acc, comp): GB300's FP64 rate is a small fraction of its FP32 rate.
  float acc[NJ], comp[NJ], fac[NJ];
#pragma unroll
  for (int j = 0; j < NJ; ++j) acc[j] = comp[j] = fac[j] = 0.0f;
  __syncthreads();
  for (int64_t r0 = (int64_t)blockIdx.x * kRowTile; r0 < rows; r0 += (int64_t)gridDim.x * kRowTile) {
    float g[4][PL], z[4][PL];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const size_t base = (size_t)(r0 + wid * 4 + i) * W;
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const int cc = lane + 32 * k;
        g[i][k] = dhp[base + cc] + gres[base + cc];
        z[i][k] = Z0[base + cc];
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int rr = wid * 4 + i;
      const int64_t r = r0 + rr;
      float d[PL];
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const float h = tanhf(z[i][k]);
        d[k] = g[i][k] * (1.0f - h * h);
        tile[rr * LD + lane + 32 * k] = d[k];
      }
      if (lane < kDm21InPad) uf[rr * kDm21InPad + lane] = lane < n_in ? (float)u[r * kDm21InPad + lane] : 0.0f;
      if (du) {
#pragma unroll
        for (int j = 0; j < kDm21InPad; ++j) {  // independent warp sums: unrolled so they overlap
          float sj = 0.0f;
          if (j < n_in) {
            float sf = 0.0f;
#pragma unroll
            for (int k = 0; k < PL; ++k) sf = fmaf(d[k], w0s[j * W + lane + 32 * k], sf);
            sj = warp_sumf(sf);
          }
          if (lane == 0) du[(size_t)r * kDm21InPad + j] = (double)sj;
        }
      }
    }
    __syncthreads();
    if (part && c < W) {
#pragma unroll 4
      for (int rr = 0; rr < kRowTile; ++rr) {
        const float gv = tile[rr * LD + c];
#pragma unroll
        for (int j = 0; j < kDm21InPad; ++j) fac[j] = fmaf(uf[rr * kDm21InPad + j], gv, fac[j]);
        fac[kDm21InPad] += gv;
        if ((rr & 15) == 15) {
#pragma unroll
          for (int j = 0; j < NJ; ++j) {  // Kahan: acc + (fac - comp)
            const float y = fac[j] - comp[j];
            const float t = acc[j] + y;
            comp[j] = (t - acc[j]) - y;
            acc[j] = t;
            fac[j] = 0.0f;
          }
        }
      }
    }
    __syncthreads();
  }
  if (part && c < W) {
    double *out = part + (size_t)blockIdx.x * (n_in + 1) * W;
#pragma unroll
    for (int j = 0; j < kDm21InPad; ++j)
      if (j < n_in) out[(size_t)j * W + c] = (double)acc[j] - (double)comp[j];
    out[(size_t)n_in * W + c] = (double)acc[kDm21InPad] - (double)comp[kDm21InPad];
  }
}

// Per-segment energies from the 256-row energy partials (Kahan), the loss and
// its cotangents dloss/dE_m.  One thread per segment; thread 0 sums the loss.
__global__ void segment_loss_kernel(const double *__restrict__ epart, const int64_t *__restrict__ seg_off, int n_seg,
                                    const double *__restrict__ eref, double *__restrict__ energies,
                                    double *__restrict__ cot, double *__restrict__ loss) {
  for (int m = threadIdx.x; m < n_seg; m += blockDim.x) {
    Kahan k{0.0, 0.0};
    for (int64_t b = seg_off[m] / 256; b < seg_off[m + 1] / 256; ++b) k.add(epart[b]);
    energies[m] = k.s;
    cot[m] = eref ? 2.0 * (k.s - eref[m]) : 1.0;
  }
  __syncthreads();
  if (loss && threadIdx.x == 0) {
    double t = 0.0;
    for (int m = 0; m < n_seg; ++m) t += eref ? (energies[m] - eref[m]) * (energies[m] - eref[m]) : energies[m];
    *loss = t;
  }
}

// Seeds the backward with each row's segment cotangent: dy, dyf, de *= dloss/dE_m.
__global__ void scale_rows_kernel(const int64_t *__restrict__ seg_off, int n_seg, const double *__restrict__ cot,
                                  int64_t rows, double *__restrict__ dy, float *__restrict__ dyf,
                                  double *__restrict__ de) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  int lo = 0, hi = n_seg;  // seg_off[lo] <= r < seg_off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (seg_off[mid] <= r) lo = mid; else hi = mid;
  }
  const double g = cot[lo];
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    dy[r * 3 + f] *= g;
    dyf[r * 3 + f] = (float)dy[r * 3 + f];
    de[r * 3 + f] *= g;
  }
}

size_t tc_layer_offset(const MlpShape &S, int i) {
  return (size_t)S.n_in * S.width + S.width + (size_t)i * ((size_t)S.width * S.width + 3 * (size_t)S.width);
}

template <int PL>
int run_tc(const MlpShape &S, const double *params, double *dparams, const double *feat, const double *ehf,
           const double *w, int64_t n_grid, int64_t np, double clip, char *ws, double *exc, double *coef, int *err,
           cudaStream_t st, const MlpSegments *seg) {
  constexpr int Wd = 32 * PL;
  const MlpTcLayout L = mlp_tc_layout(S, np);
  auto d64 = [&](size_t off) { return (double *)(ws + off); };
  auto f32 = [&](size_t off) { return (float *)(ws + off); };
  double *x = d64(L.x), *u = d64(L.u), *e = d64(L.e), *dy = d64(L.dy), *de = d64(L.de), *du = d64(L.du);
  double *epart = d64(L.epart), *kpart = d64(L.kpart), *lnpart = d64(L.lnpart), *colpart = d64(L.colpart);
  double *colpart2 = d64(L.colpart2);
  float *PU = f32(L.pu), *WT = f32(L.wt), *WR = f32(L.wr), *ZF = f32(L.zf), *HF = f32(L.hf);
  float *PH = f32(L.ph), *CH = f32(L.ch), *GZ = f32(L.gz), *DHP = f32(L.dhp), *PG = f32(L.pg), *CG = f32(L.cg);
  const size_t act = (size_t)np * Wd;
  const int64_t rt = np / kPointTile, rc = np / 32;  // row tiles, row chunks
  constexpr int ft = Wd / 128, kcw = Wd / 32;         // feature tiles, K chunks of the width
  const size_t wt0 = (size_t)ft * kBlk, wti = (size_t)ft * kcw * kBlk;  // packed W0^T, W_i^T sizes
  auto WTi = [&](int i) { return WT + (i == 0 ? 0 : wt0 + (size_t)(i - 1) * wti); };
  auto WRi = [&](int i) { return WR + (size_t)(i - 1) * wti; };
  auto CHi = [&](int i) { return CH + (size_t)i * ft * rc * kBlk; };
  const size_t head_off = tc_layer_offset(S, S.n_layers);
  const double *W0 = params;
  const double *Wo = params + head_off, *bo = Wo + (size_t)Wd * S.n_out;
  // FP32 copy of the parameters for the row kernels (FP64 -> FP32 conversions
  // run at the FP64 rate, so they are done once per call, not per element).
  float *pf = f32(L.pf);
  const float *W0f = pf, *b0f = pf + (size_t)S.n_in * Wd, *Wof = pf + head_off;
  int rc_;
#define GDFT_CK(expr, what)                                      \
  do {                                                           \
    if ((rc_ = check_cuda((expr), what)) != GDFT_OK) return rc_; \
  } while (0)
  auto gemm_act = [&](const float *A, int64_t a_chunks, const float *B, int64_t b_chunks, int64_t kch, float *out) {
    TcgArgs a{};
    a.a = A;
    a.b = B;
    a.m_tiles = (int)rt;
    a.n_tiles = ft;
    a.a_chunks = a_chunks;
    a.b_chunks = b_chunks;
    a.k_chunks = kch;
    a.chunks_per_split = kch;
    a.out32 = out;
    a.ldo = Wd;
    a.m_valid = (int)np;
    a.n_valid = Wd;
    a.err = err;
    return launch_tcg(a, 1, st);
  };
  auto gemm_wgrad = [&](const float *A, int m_tiles, int m_valid, const float *B, double *out) -> cudaError_t {
    TcgArgs a{};
    a.a = A;
    a.b = B;
    a.m_tiles = m_tiles;
    a.n_tiles = ft;
    a.a_chunks = a.b_chunks = a.k_chunks = rc;
    // L.nsplit CTAs in all: the output tiles of one K range run side by side
    // and share its operand chunks through L2.
    const int ns = L.nsplit / (m_tiles * ft) > 1 ? L.nsplit / (m_tiles * ft) : 1;
    a.chunks_per_split = (rc + ns - 1) / ns;
    a.out64 = kpart;
    a.m_valid = m_valid;
    a.n_valid = Wd;
    a.err = err;
    cudaError_t r = launch_tcg(a, ns, st);
    if (r != cudaSuccess) return r;
    const size_t total = (size_t)m_valid * Wd;
    sum_splits_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(kpart, ns, total, out);
    return cudaGetLastError();
  };

  // ---- weights: packed once per call ----
  {
    const size_t n = mlp_param_count(S);
    to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(params, n, pf);
    GDFT_CK(cudaGetLastError(), "mlp_tc params f32");
  }
  GDFT_CK(launch_pack_ct<double>(W0, S.n_in, Wd, Wd, ft, 1, WTi(0), st), "mlp_tc pack W0");
  for (int i = 1; i <= S.n_layers; ++i) {
    const double *Wi = params + tc_layer_offset(S, i - 1);
    GDFT_CK(launch_pack_ct<double>(Wi, Wd, Wd, Wd, ft, kcw, WTi(i), st), "mlp_tc pack W^T");
    GDFT_CK(launch_pack_rt<double>(Wi, Wd, Wd, Wd, ft, kcw, WRi(i), st), "mlp_tc pack W");
  }

  // ---- forward ----
  GDFT_CK(launch_dm21_features(feat, ehf, n_grid, np, clip, S.squash_offset, x, u, e, st), "mlp_tc features");
  GDFT_CK(launch_pack_rt<double>(u, np, S.n_in, kDm21InPad, rt, 1, PU, st), "mlp_tc pack u");
  // Each row pass also packs its h for the next dense layer (rt) and, with
  // dparams, for that layer's weight gradient (ct).
  GDFT_CK(gemm_act(PU, 1, WTi(0), 1, 1, ZF), "mlp_tc dense_0");
  layer_fwd_pack_kernel<PL, true><<<kLnBlocks, 256, 0, st>>>(ZF, b0f, HF, nullptr, nullptr, 0.0, np,
                                                             S.n_layers > 0 ? PH : nullptr,
                                                             (dparams && S.n_layers > 0) ? CHi(0) : nullptr);
  GDFT_CK(cudaGetLastError(), "mlp_tc tanh");
  for (int i = 1; i <= S.n_layers; ++i) {
    const float *Wif = pf + tc_layer_offset(S, i - 1), *bi = Wif + (size_t)Wd * Wd, *gi = bi + Wd, *bei = gi + Wd;
    float *Zi = ZF + (size_t)i * act;
    GDFT_CK(gemm_act(PH, kcw, WTi(i), kcw, kcw, Zi), "mlp_tc dense_i");
    const bool more = i < S.n_layers;
    layer_fwd_pack_kernel<PL, false><<<kLnBlocks, 256, 0, st>>>(Zi, bi, HF, gi, bei, S.ln_eps, np,
                                                                more ? PH : nullptr,
                                                                (dparams && more) ? CHi(i) : nullptr);
    GDFT_CK(cudaGetLastError(), "mlp_tc layernorm");
  }
  const unsigned hblocks = (unsigned)((np + 255) / 256);
  float *dyf = f32(L.dyf);
  head_kernel<PL><<<hblocks, 256, 0, st>>>(HF, Wof, bo, e, w, n_grid, np, clip, S.sigmoid_scale, dy, dyf, de,
                                           epart);
  GDFT_CK(cudaGetLastError(), "mlp_tc head");
  if (exc) GDFT_CK(launch_energy_reduce(epart, (int)hblocks, exc, st), "mlp_tc energy_reduce");
  if (seg) {
    segment_loss_kernel<<<1, 256, 0, st>>>(epart, seg->d_seg_off, seg->n_seg, seg->d_eref, seg->d_energies,
                                           seg->d_cot, seg->d_loss);
    GDFT_CK(cudaGetLastError(), "mlp_tc segment loss");
    scale_rows_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(seg->d_seg_off, seg->n_seg, seg->d_cot, np, dy,
                                                                     dyf, de);
    GDFT_CK(cudaGetLastError(), "mlp_tc segment seed");
  }
  if (coef == nullptr && dparams == nullptr) return GDFT_OK;

  // ---- backward ----
  if (dparams) {
    head_wgrad_part_kernel<<<kHeadBlocks, 256, 0, st>>>(HF, dyf, dy, np, np, Wd, colpart);
    launch_colsum_final(colpart, kHeadBlocks, 3 * Wd + 3, dparams + head_off, st);
    GDFT_CK(cudaGetLastError(), "mlp_tc head wgrad");
  }
  float *gz_cur = GZ, *gz_prev = GZ + act;
  GDFT_CK(cudaFuncSetAttribute(layer_bwd_pack_kernel<PL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)bwd_pack_smem<PL>()),
          "mlp_tc layernorm bwd smem");
  for (int i = S.n_layers; i >= 1; --i) {
    const float *Wif = pf + tc_layer_offset(S, i - 1), *gi = Wif + (size_t)Wd * Wd + Wd, *bei = gi + Wd;
    const float *Zi = ZF + (size_t)i * act;
    const bool last = i == S.n_layers;
    layer_bwd_pack_kernel<PL><<<kLnBlocks, 256, bwd_pack_smem<PL>(), st>>>(last ? nullptr : DHP, last ? nullptr : gz_prev,
                                                         last ? dy : nullptr, Wof, Zi, gi, bei, S.ln_eps, np,
                                                         gz_cur, lnpart, PG, dparams ? CG : nullptr);
    GDFT_CK(cudaGetLastError(), "mlp_tc layernorm bwd");
    if (dparams) {
      double *dWi = dparams + tc_layer_offset(S, i - 1);
      GDFT_CK(gemm_wgrad(CHi(i - 1), ft, Wd, CG, dWi), "mlp_tc dW_i");
      // [dgamma | dbeta | db] partials -> db, then (dgamma, dbeta) in the flat order (db, gamma, beta).
      launch_colsum_final(lnpart, kLnBlocks, 3 * Wd, colpart2, st);
      GDFT_CK(cudaGetLastError(), "mlp_tc ln sums");
      GDFT_CK(cudaMemcpyAsync(dWi + (size_t)Wd * Wd, colpart2 + 2 * Wd, Wd * sizeof(double),
                              cudaMemcpyDeviceToDevice, st),
              "mlp_tc db");
      GDFT_CK(cudaMemcpyAsync(dWi + (size_t)Wd * Wd + Wd, colpart2, 2 * Wd * sizeof(double),
                              cudaMemcpyDeviceToDevice, st),
              "mlp_tc dln");
    }
    GDFT_CK(gemm_act(PG, kcw, WRi(i), kcw, kcw, DHP), "mlp_tc dh");
    float *t = gz_cur;
    gz_cur = gz_prev;
    gz_prev = t;
  }
  // Layer 0: gz_prev holds dE/dz_1, DHP its product with W_1^T.  One pass
  // gives du and the FP64 partials of [dW0 | db0] (kpart is free by now and
  // holds kLnBlocks x (n_in + 1) x W doubles: 4 (n_in + 1) <= W).
  GDFT_CK(cudaFuncSetAttribute(l0_bwd_fused_kernel<PL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)l0_bwd_smem<PL>()),
          "mlp_tc tanh bwd smem");
  l0_bwd_fused_kernel<PL><<<kLnBlocks, 256, l0_bwd_smem<PL>(), st>>>(DHP, gz_prev, ZF, u, W0f, S.n_in, np,
                                                                    coef ? du : nullptr, dparams ? kpart : nullptr);
  GDFT_CK(cudaGetLastError(), "mlp_tc tanh bwd");
  if (dparams) {
    launch_colsum_final(kpart, kLnBlocks, (S.n_in + 1) * Wd, dparams, st);
    GDFT_CK(cudaGetLastError(), "mlp_tc dW_0");
  }
  if (coef)
    GDFT_CK(launch_dm21_potentials(feat, x, du, de, n_grid, np, clip, S.squash_offset, coef, st),
            "mlp_tc potentials");
#undef GDFT_CK
  return GDFT_OK;
}

}  // namespace

bool mlp_tc_width_supported(int width) { return width == 128 || width == 256; }

MlpTcLayout mlp_tc_layout(const MlpShape &s, int64_t np) {
  MlpTcLayout L;
  const int W = s.width;
  const size_t act = (size_t)np * W;
  const int64_t rt = np / kPointTile, rc = np / 32;
  const int ft = W / 128, kcw = W / 32;
  L.nsplit = 148;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  L.x = take((size_t)np * kDm21In * 8);
  L.u = take((size_t)np * kDm21InPad * 8);
  L.e = take((size_t)np * 3 * 8);
  L.dy = take((size_t)np * 3 * 8);
  L.de = take((size_t)np * 3 * 8);
  L.du = take((size_t)np * kDm21InPad * 8);
  L.epart = take((size_t)((np + 255) / 256) * 8);
  L.kpart = take((size_t)L.nsplit * W * W * 8);
  L.lnpart = take((size_t)kLnBlocks * 3 * W * 8);
  L.colpart = take((size_t)kHeadBlocks * (3 * W + 3) * 8);
  L.colpart2 = take((size_t)3 * W * 8);
  L.pf = take(mlp_param_count(s) * 4);
  L.dyf = take((size_t)np * 3 * 4);
  L.pu = take((size_t)rt * kBlk * 4);
  L.wt = take(((size_t)ft * kBlk + (size_t)s.n_layers * ft * kcw * kBlk) * 4);
  L.wr = take((size_t)(s.n_layers > 0 ? s.n_layers : 1) * ft * kcw * kBlk * 4);
  L.zf = take(act * (s.n_layers + 1) * 4);
  L.hf = take(act * 4);
  L.ph = take((size_t)rt * kcw * kBlk * 4);
  L.ch = take((size_t)(s.n_layers > 0 ? s.n_layers : 1) * ft * rc * kBlk * 4);
  L.gz = take(2 * act * 4);
  L.dhp = take(act * 4);
  L.pg = take((size_t)rt * kcw * kBlk * 4);
  L.cg = take((size_t)ft * rc * kBlk * 4);
  L.bytes = off;
  return L;
}

int mlp_run_tc(const MlpShape &S, const double *params, double *dparams, const double *feat, const double *ehf,
               const double *w, int64_t n_grid, int64_t np, double clip, char *ws, double *exc, double *coef, int *err,
               cudaStream_t st, const MlpSegments *seg) {
  if (np % kPointTile != 0 || S.n_in > 128 || (seg && (seg->n_seg < 1 || np % 256 != 0))) {
    set_error("mlp_tc: grid padding or input width not supported");
    return GDFT_ERR_INVALID;
  }
  switch (S.width) {
    case 128: return run_tc<4>(S, params, dparams, feat, ehf, w, n_grid, np, clip, ws, exc, coef, err, st, seg);
    case 256: return run_tc<8>(S, params, dparams, feat, ehf, w, n_grid, np, clip, ws, exc, coef, err, st, seg);
    default:
      set_error("mlp_tc: width %d not built for the mixed form (128 or 256)", S.width);
      return GDFT_ERR_UNSUPPORTED;
  }
}

}  // namespace gdft
