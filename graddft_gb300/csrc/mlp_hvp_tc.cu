// mlp_hvp_tc.cu - mixed form of the second-order adjoint (mlp_hvp.cu): the
// tangent-augmented network pass and its reverse with the hidden-layer GEMMs on
// the tensor cores (tc_gemm.cu) over the stacked [primal; tangent] rows.
//
// Same graph as the FP64 form: features x(F), x~ = J_x F~; u, u~; layer 0
// tanh; L residual LayerNorm/ELU layers with tangents; sigmoid head; L_r =
// m w sum_f (c~_f ec_f + c_f e~'_f); then the reverse of that graph, carrying
// the second-order terms of tanh, LayerNorm and ELU.  Activations [2][np][W]
// FP32, one GEMM per layer over 2 np rows; the weight gradients contract over
// all 2 np rows (primal and tangent contributions in one split-K GEMM); per-row
// statistics FP32, sums over grid points FP64; per-point head and potentials
// FP64 (mlp_hvp.cu).
#include "common.cuh"
#include "kernels.cuh"
#include "mlp.cuh"
#include "mlp_gemm.cuh"
#include "mlp_rows.cuh"
#include "tc_gemm.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr size_t kBlk = 2 * (umma::kBlockBytes / 4);

// Head with tangents: each warp takes 32 rows; y, y~ (FP32 row sums) of row i
// land in lane i, which evaluates the FP64 head of head_tan_kernel (mlp_hvp.cu):
// GY = [dL/dy; dL/dy~] (FP64 and FP32 copies), ge = (dL/de_0, dL/de~_0), and
// partial sums of L per block of 256 rows.
template <int PL>
__global__ void __launch_bounds__(256) head_tan_tc_kernel(const float *__restrict__ H, const float *__restrict__ Wo,
                                                          const double *__restrict__ bo, const double *__restrict__ e,
                                                          const double *__restrict__ et, const double *__restrict__ w,
                                                          int64_t n_grid, int64_t np, double clip, double sscale,
                                                          double *__restrict__ GY, float *__restrict__ GYf,
                                                          double *__restrict__ ge, double *__restrict__ lpart) {
  constexpr int W = 32 * PL;
  __shared__ double red[8];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t base = ((int64_t)blockIdx.x * 8 + wid) * 32;
  const size_t act = (size_t)np * W;
  float wo[PL][3];
#pragma unroll
  for (int k = 0; k < PL; ++k)
#pragma unroll
    for (int f = 0; f < 3; ++f) wo[k][f] = Wo[(lane + 32 * k) * 3 + f];
  float my[3] = {0.0f, 0.0f, 0.0f}, myt[3] = {0.0f, 0.0f, 0.0f};
  for (int i = 0; i < 32; ++i) {
    const int64_t r = base + i;
    if (r >= np) break;
    float yf[3] = {0.0f, 0.0f, 0.0f}, ytf[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < PL; ++k) {
      const float hv = H[(size_t)r * W + lane + 32 * k];
      const float htv = H[act + (size_t)r * W + lane + 32 * k];
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        yf[f] = fmaf(hv, wo[k][f], yf[f]);
        ytf[f] = fmaf(htv, wo[k][f], ytf[f]);
      }
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const float a = warp_sumf(yf[f]), b = warp_sumf(ytf[f]);
      if (lane == i) {
        my[f] = a;
        myt[f] = b;
      }
    }
  }
  const int64_t p = base + lane;
  double l_r = 0.0;
  if (p < np) {
    double gy[3] = {0.0, 0.0, 0.0}, gyt[3] = {0.0, 0.0, 0.0}, ge0 = 0.0, get0 = 0.0;
    if (p < n_grid) {
      double sg[3], c[3], ct[3], ec[3], ed[3], exc = 0.0;
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        sg[f] = 1.0 / (1.0 + exp(-(((double)my[f] + bo[f]) / sscale)));
        c[f] = sscale * sg[f];
        ct[f] = sg[f] * (1.0 - sg[f]) * (double)myt[f];
        const double ev = e[(size_t)p * 3 + f];
        const bool keep = fabs(ev) > clip;
        ec[f] = keep ? ev : 0.0;
        ed[f] = (f == 0 && keep) ? et[p] : 0.0;
        exc = f == 0 ? c[f] * ec[f] : exc + c[f] * ec[f];
      }
      const bool m = fabs(exc) > clip;
      const double Wt = fabs(w[p]) > clip ? w[p] : 0.0;
      if (m) {
        double lr = 0.0;
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          lr += ct[f] * ec[f] + c[f] * ed[f];
          const double dct = Wt * ec[f], dc = Wt * ed[f];
          const double s1 = sg[f] * (1.0 - sg[f]);
          gyt[f] = dct * s1;
          gy[f] = dct * (double)myt[f] * s1 * (1.0 - 2.0 * sg[f]) / sscale + dc * s1;
        }
        l_r = Wt * lr;
        const bool keep0 = fabs(e[(size_t)p * 3]) > clip;
        ge0 = keep0 ? Wt * ct[0] : 0.0;
        get0 = keep0 ? Wt * c[0] : 0.0;
      }
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      GY[(size_t)p * 3 + f] = gy[f];
      GY[((size_t)np + p) * 3 + f] = gyt[f];
      GYf[(size_t)p * 3 + f] = (float)gy[f];
      GYf[((size_t)np + p) * 3 + f] = (float)gyt[f];
    }
    ge[2 * (size_t)p] = ge0;
    ge[2 * (size_t)p + 1] = get0;
  }
  const double s = warp_sum(l_r);
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < 8; ++i) t += red[i];
    lpart[blockIdx.x] = t;
  }
}

// ------------------------------------------------------- fused row passes
// Row passes with the operand packing folded in (as the network's first-order
// pass does, mlp_tc.cu): per 32-row tile of primal rows r0.. and its tangent
// rows np + r0.., each warp takes 4 row pairs, and the primal and then the
// tangent activations go through one shared-memory tile into the rt and ct
// packs over the stacked 2 np rows.

// Forward, stacked rows r (primal) and np + r (tangent):
//   L0:   z = zW + b (stored), h = tanh(z), h~ = (1 - h^2) z~
//   else: z = zW + b + h (stored), z~ = z~W + h~ (stored); h = elu(LN(z)),
//         h~ = elu'(a) gamma rs (z~ - mean(z~) - xh mean(xh z~)), a = LN(z)
// (h, h~ in place of the previous layer's).  np is a multiple of 32.
template <int PL, bool L0>
__global__ void __launch_bounds__(256) tan_fwd_pack_kernel(float *__restrict__ Z, const float *__restrict__ b,
                                                           float *__restrict__ H, const float *__restrict__ gam,
                                                           const float *__restrict__ bet, double eps, int64_t np,
                                                           float *__restrict__ rt_out, float *__restrict__ ct_out) {
  constexpr int W = 32 * PL, LD = W + 4;
  __shared__ __align__(16) float tile[kRowTile * LD];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t act = (size_t)np * W;
  const int64_t rchunks = 2 * np / 32;
  float bf[PL], gf[PL], ef[PL];
#pragma unroll
  for (int k = 0; k < PL; ++k) {
    const int c = lane + 32 * k;
    bf[k] = b[c];
    gf[k] = L0 ? 0.0f : gam[c];
    ef[k] = L0 ? 0.0f : bet[c];
  }
  for (int64_t r0 = (int64_t)blockIdx.x * kRowTile; r0 < np; r0 += (int64_t)gridDim.x * kRowTile) {
    float ht[4][PL];
#pragma unroll 1
    for (int i = 0; i < 4; ++i) {
      const int rr = wid * 4 + i;
      const size_t base = (size_t)(r0 + rr) * W;
      float v[PL], vt[PL];
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const int c = lane + 32 * k;
        if (L0) {
          v[k] = Z[base + c] + bf[k];
          vt[k] = Z[act + base + c];
        } else {
          v[k] = (Z[base + c] + bf[k]) + H[base + c];
          vt[k] = Z[act + base + c] + H[act + base + c];
        }
      }
      if (L0) {
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          const int c = lane + 32 * k;
          const float h = tanhf(v[k]);
          Z[base + c] = v[k];
          H[base + c] = h;
          ht[i][k] = (1.0f - h * h) * vt[k];
          H[act + base + c] = ht[i][k];
          tile[rr * LD + c] = h;
        }
      } else {
        float s1 = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) s1 += v[k];
        const float mean = warp_sumf(s1) * (1.0f / W);
        float s2 = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          const float d = v[k] - mean;
          s2 += d * d;
        }
        const float rs = 1.0f / sqrtf(warp_sumf(s2) * (1.0f / W) + (float)eps);
        float xh[PL], m1 = 0.0f, m2 = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          xh[k] = (v[k] - mean) * rs;
          m1 += vt[k];
          m2 += xh[k] * vt[k];
        }
        m1 = warp_sumf(m1) * (1.0f / W);
        m2 = warp_sumf(m2) * (1.0f / W);
#pragma unroll
        for (int k = 0; k < PL; ++k) {
          const int c = lane + 32 * k;
          Z[base + c] = v[k];
          Z[act + base + c] = vt[k];
          const float a = xh[k] * gf[k] + ef[k];
          const float at = gf[k] * (rs * (vt[k] - m1 - xh[k] * m2));
          const float h = eluf(a);
          H[base + c] = h;
          ht[i][k] = (a > 0.0f ? 1.0f : expf(a)) * at;
          H[act + base + c] = ht[i][k];
          tile[rr * LD + c] = h;
        }
      }
    }
    __syncthreads();
    store_tile_packs<PL>(tile, r0, rt_out, ct_out, rchunks);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = 0; k < PL; ++k) tile[(wid * 4 + i) * LD + lane + 32 * k] = ht[i][k];
    __syncthreads();
    store_tile_packs<PL>(tile, np + r0, rt_out, ct_out, rchunks);
    __syncthreads();
  }
}

// Reverse of a residual layer with tangents.  Incoming [dL/dh; dL/dh~] is
// GY W_out^T (last layer) or dhp + gres (stacked); writes [dL/dz; dL/dz~]
// (FP32), their rt and ct packs, and per-block partials [block][3][W] of
// dL/dgamma, dL/dbeta and dL/db (primal dz): FP32 per 16 rows of a warp, then
// Kahan-compensated FP32 per warp, FP64 across the block's warps.  The
// LayerNorm's second-order term follows mlp_hvp.cu.  Dynamic shared memory:
// bwd_pack_smem<PL>() bytes.
template <int PL>
__global__ void __launch_bounds__(256, 2) tan_bwd_pack_kernel(
    const float *__restrict__ dhp, const float *__restrict__ gres, const float *__restrict__ GYf,
    const float *__restrict__ Wo, const float *__restrict__ Z, const float *__restrict__ gam,
    const float *__restrict__ bet, double eps, int64_t rows, float *__restrict__ gz, double *__restrict__ part,
    float *__restrict__ rt_out, float *__restrict__ ct_out) {
  constexpr int W = 32 * PL, LD = W + 4;
  extern __shared__ __align__(16) unsigned char tbwd_smem[];
  float2(*sacc)[3][W] = reinterpret_cast<float2(*)[3][W]>(tbwd_smem);
  float *tile = reinterpret_cast<float *>(tbwd_smem + sizeof(float2) * 8 * 3 * W);
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t act = (size_t)rows * W;
  const int64_t rchunks = 2 * rows / 32;
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
    for (int i = 0; i < 4; ++i) {
      const int rr = wid * 4 + i;
      const int64_t r = r0 + rr;
      const size_t base = (size_t)r * W;
      float v[PL], vt[PL], gh[PL], ght[PL], s1 = 0.0f;
      float y0 = 0.0f, y1 = 0.0f, y2 = 0.0f, t0 = 0.0f, t1 = 0.0f, t2 = 0.0f;
      if (GYf) {
        y0 = GYf[r * 3 + 0];
        y1 = GYf[r * 3 + 1];
        y2 = GYf[r * 3 + 2];
        t0 = GYf[(rows + r) * 3 + 0];
        t1 = GYf[(rows + r) * 3 + 1];
        t2 = GYf[(rows + r) * 3 + 2];
      }
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const int c = lane + 32 * k;
        v[k] = Z[base + c];
        vt[k] = Z[act + base + c];
        s1 += v[k];
        if (GYf) {
          const float w0 = __ldg(Wo + c * 3), w1 = __ldg(Wo + c * 3 + 1), w2 = __ldg(Wo + c * 3 + 2);
          gh[k] = fmaf(y0, w0, fmaf(y1, w1, y2 * w2));
          ght[k] = fmaf(t0, w0, fmaf(t1, w1, t2 * w2));
        } else {
          gh[k] = dhp[base + c] + gres[base + c];
          ght[k] = dhp[act + base + c] + gres[act + base + c];
        }
      }
      const float mean = warp_sumf(s1) * (1.0f / W);
      float s2 = 0.0f;
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const float d = v[k] - mean;
        s2 += d * d;
      }
      const float rs = 1.0f / sqrtf(warp_sumf(s2) * (1.0f / W) + (float)eps);
      float xh[PL], m1 = 0.0f, m2 = 0.0f;
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        xh[k] = (v[k] - mean) * rs;
        m1 += vt[k];
        m2 += xh[k] * vt[k];
      }
      m1 = warp_sumf(m1) * (1.0f / W);
      m2 = warp_sumf(m2) * (1.0f / W);
      float gp[PL], gt[PL], xht[PL];
      float sgp = 0.0f, sgpx = 0.0f, sgt = 0.0f, sgtx = 0.0f, sgtz = 0.0f;
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        xht[k] = rs * (vt[k] - m1 - xh[k] * m2);
        const float a = gmf[k] * xh[k] + btf[k];
        const float at = gmf[k] * xht[k];
        const float ea = expf(a);
        const float e1 = a > 0.0f ? 1.0f : ea;
        const float e2 = a > 0.0f ? 0.0f : ea;
        const float gat = ght[k] * e1;
        const float ga = gh[k] * e1 + ght[k] * at * e2;
        fg[k] = fmaf(ga, xh[k], fmaf(gat, xht[k], fg[k]));
        fb[k] += ga;
        gp[k] = ga * gmf[k];
        gt[k] = gat * gmf[k];
        sgp += gp[k];
        sgpx += gp[k] * xh[k];
        sgt += gt[k];
        sgtx += gt[k] * xh[k];
        sgtz += gt[k] * vt[k];
      }
      const float mgp = warp_sumf(sgp) * (1.0f / W), mgpx = warp_sumf(sgpx) * (1.0f / W);
      const float mgt = warp_sumf(sgt) * (1.0f / W), mgtx = warp_sumf(sgtx) * (1.0f / W);
      const float mgtz = warp_sumf(sgtz) * (1.0f / W);
      const float r2 = rs * rs;
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const int c = lane + 32 * k;
        const float second =
            -r2 * (xh[k] * (mgtz - mgt * m1 - 3.0f * m2 * mgtx) + mgtx * (vt[k] - m1) + m2 * (gt[k] - mgt));
        const float d = rs * (gp[k] - mgp - xh[k] * mgpx) + second;
        fd[k] += d;
        gz[base + c] = d;
        gz[act + base + c] = rs * (gt[k] - mgt - xh[k] * mgtx);
        tile[rr * LD + c] = d;
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
    store_tile_packs<PL>(tile, r0, rt_out, ct_out, rchunks);
    __syncthreads();
    // The tangent rows this thread wrote above, back through the tile.
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const int rr = wid * 4 + i, c = lane + 32 * k;
        tile[rr * LD + c] = gz[act + (size_t)(r0 + rr) * W + c];
      }
    __syncthreads();
    store_tile_packs<PL>(tile, rows + r0, rt_out, ct_out, rchunks);
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

// Layer-0 reverse with tangents, g = dhp + gres (stacked), h = tanh(z0),
// s = 1 - h^2: dz0 = g s - 2 h s z0~ g~, dz0~ = g~ s; with everything that
// consumes [dz0; dz0~], per 32-row tile: GU[row][j] = sum_c dz0[row][c] W0[j][c]
// over the stacked rows, part[block][j][c] = sum over the stacked
// rows of U[row][j] dz0[row][c] (dW0), part[block][n_in][c] = sum over the
// primal rows of dz0 (db0); parameter sums FP32 per 16 rows, Kahan FP32 per
// block.  Dynamic shared memory: l0_tan_bwd_smem<PL>() bytes.
template <int PL>
constexpr size_t l0_tan_bwd_smem() {
  return sizeof(float) * (2 * kRowTile * (32 * PL + 4) + 2 * kRowTile * kDm21InPad + kDm21InPad * 32 * PL);
}

template <int PL>
__global__ void __launch_bounds__(256) tanh_tan_bwd_fused_kernel(
    const float *__restrict__ dhp, const float *__restrict__ gres, const float *__restrict__ Z0,
    const double *__restrict__ U, const float *__restrict__ W0, int n_in, int64_t np, double *__restrict__ GU,
    double *__restrict__ part) {
  constexpr int W = 32 * PL, LD = W + 4, NJ = kDm21InPad + 1;
  extern __shared__ __align__(16) unsigned char l0t_smem[];
  float *tp = reinterpret_cast<float *>(l0t_smem);  // [32][LD] dz0, primal rows
  float *tt = tp + kRowTile * LD;                    // [32][LD] dz0~, tangent rows
  float *up = tt + kRowTile * LD;                    // [32][kDm21InPad] u, primal rows
  float *ut = up + kRowTile * kDm21InPad;            // [32][kDm21InPad] u~, tangent rows
  float *w0s = ut + kRowTile * kDm21InPad;           // [kDm21InPad][W] W0, zero rows past n_in
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t act = (size_t)np * W;
  for (int i = threadIdx.x; i < kDm21InPad * W; i += blockDim.x) w0s[i] = i / W < n_in ? W0[i] : 0.0f;
  const int c = threadIdx.x;
  float acc[NJ], comp[NJ], fac[NJ];
#pragma unroll
  for (int j = 0; j < NJ; ++j) acc[j] = comp[j] = fac[j] = 0.0f;
  __syncthreads();
  auto du_row = [&](const float (&d)[PL], int64_t row) {
    if (GU == nullptr) return;
#pragma unroll
    for (int j = 0; j < kDm21InPad; ++j) {  // independent warp sums: unrolled so they overlap
      float sj = 0.0f;
      if (j < n_in) {
        float sf = 0.0f;
#pragma unroll
        for (int k = 0; k < PL; ++k) sf = fmaf(d[k], w0s[j * W + lane + 32 * k], sf);
        sj = warp_sumf(sf);
      }
      if (lane == 0) GU[(size_t)row * kDm21InPad + j] = (double)sj;
    }
  };
  for (int64_t r0 = (int64_t)blockIdx.x * kRowTile; r0 < np; r0 += (int64_t)gridDim.x * kRowTile) {
#pragma unroll 1
    for (int i = 0; i < 4; ++i) {
      const int rr = wid * 4 + i;
      const int64_t r = r0 + rr;
      const size_t base = (size_t)r * W;
      float d[PL], dt[PL];
#pragma unroll
      for (int k = 0; k < PL; ++k) {
        const size_t e = base + lane + 32 * k;
        const float h = tanhf(Z0[e]), sv = 1.0f - h * h;
        const float g = dhp[e] + gres[e], gt = dhp[act + e] + gres[act + e];
        dt[k] = gt * sv;
        d[k] = g * sv - 2.0f * h * sv * Z0[act + e] * gt;
        tp[rr * LD + lane + 32 * k] = d[k];
        tt[rr * LD + lane + 32 * k] = dt[k];
      }
      if (lane < kDm21InPad) {
        up[rr * kDm21InPad + lane] = lane < n_in ? (float)U[(size_t)r * kDm21InPad + lane] : 0.0f;
        ut[rr * kDm21InPad + lane] = lane < n_in ? (float)U[(size_t)(np + r) * kDm21InPad + lane] : 0.0f;
      }
      du_row(d, r);
      du_row(dt, np + r);
    }
    __syncthreads();
    if (part && c < W) {
#pragma unroll 2
      for (int rr = 0; rr < kRowTile; ++rr) {
        const float gp = tp[rr * LD + c], gt = tt[rr * LD + c];
#pragma unroll
        for (int j = 0; j < kDm21InPad; ++j)
          fac[j] = fmaf(ut[rr * kDm21InPad + j], gt, fmaf(up[rr * kDm21InPad + j], gp, fac[j]));
        fac[kDm21InPad] += gp;
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

size_t hvp_tc_layer_offset(const MlpShape &S, int i) {
  return (size_t)S.n_in * S.width + S.width + (size_t)i * ((size_t)S.width * S.width + 3 * (size_t)S.width);
}

template <int PL>
int run_hvp_tc(const MlpShape &S, const double *params, double *dparams, const double *featp, const double *featt,
               const double *ehf, const double *w, int64_t n_grid, int64_t np, double clip, char *ws, double *lval,
               double *coef, int *err, cudaStream_t st) {
  constexpr int Wd = 32 * PL;
  const MlpHvpTcLayout L = mlp_hvp_tc_layout(S, np);
  auto d64 = [&](size_t off) { return (double *)(ws + off); };
  auto f32 = [&](size_t off) { return (float *)(ws + off); };
  double *x = d64(L.x), *xt = d64(L.xt), *U = d64(L.u), *e = d64(L.e), *et = d64(L.et), *GY = d64(L.gy);
  double *GE = d64(L.ge), *GU = d64(L.gu), *lpart = d64(L.lpart), *kpart = d64(L.kpart);
  double *lnpart = d64(L.lnpart), *colpart = d64(L.colpart), *colpart2 = d64(L.colpart2);
  float *pf = f32(L.pf), *GYf = f32(L.gyf), *PU = f32(L.pu), *WT = f32(L.wt), *WR = f32(L.wr);
  float *Z = f32(L.z), *H = f32(L.h), *PH = f32(L.ph), *CH = f32(L.ch), *GZ = f32(L.gz), *DHP = f32(L.dhp);
  float *PG = f32(L.pg), *CG = f32(L.cg);
  const int64_t rows2 = 2 * np;
  const size_t act = (size_t)np * Wd, act2 = 2 * act;
  const int64_t rt2 = rows2 / kPointTile, rc2 = rows2 / 32;
  constexpr int ft = Wd / 128, kcw = Wd / 32;
  const size_t wt0 = (size_t)ft * kBlk, wti = (size_t)ft * kcw * kBlk;
  auto WTi = [&](int i) { return WT + (i == 0 ? 0 : wt0 + (size_t)(i - 1) * wti); };
  auto WRi = [&](int i) { return WR + (size_t)(i - 1) * wti; };
  auto CHi = [&](int i) { return CH + (size_t)i * ft * rc2 * kBlk; };
  const size_t head_off = hvp_tc_layer_offset(S, S.n_layers);
  const double *W0 = params;
  const double *bo = params + head_off + (size_t)Wd * S.n_out;
  const float *W0f = pf, *b0f = pf + (size_t)S.n_in * Wd, *Wof = pf + head_off;
  int rc_;
#define GDFT_CK(expr, what)                                      \
  do {                                                           \
    if ((rc_ = check_cuda((expr), what)) != GDFT_OK) return rc_; \
  } while (0)
  auto gemm_act = [&](const float *A, int64_t kch, const float *B, float *out) {
    TcgArgs a{};
    a.a = A;
    a.b = B;
    a.m_tiles = (int)rt2;
    a.n_tiles = ft;
    a.a_chunks = a.b_chunks = a.k_chunks = a.chunks_per_split = kch;
    a.out32 = out;
    a.ldo = Wd;
    a.m_valid = (int)rows2;
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
    a.a_chunks = a.b_chunks = a.k_chunks = rc2;
    // L.nsplit CTAs in all: the output tiles of one K range run side by side
    // and share its operand chunks through L2.
    const int ns = L.nsplit / (m_tiles * ft) > 1 ? L.nsplit / (m_tiles * ft) : 1;
    a.chunks_per_split = (rc2 + ns - 1) / ns;
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
  const unsigned pblocks = (unsigned)((np + 255) / 256);

  {
    const size_t n = mlp_param_count(S);
    to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(params, n, pf);
    GDFT_CK(cudaGetLastError(), "hvp_tc params f32");
  }
  GDFT_CK(launch_pack_ct<double>(W0, S.n_in, Wd, Wd, ft, 1, WTi(0), st), "hvp_tc pack W0");
  for (int i = 1; i <= S.n_layers; ++i) {
    const double *Wi = params + hvp_tc_layer_offset(S, i - 1);
    GDFT_CK(launch_pack_ct<double>(Wi, Wd, Wd, Wd, ft, kcw, WTi(i), st), "hvp_tc pack W^T");
    GDFT_CK(launch_pack_rt<double>(Wi, Wd, Wd, Wd, ft, kcw, WRi(i), st), "hvp_tc pack W");
  }

  // ---- tangent-augmented forward ----
  GDFT_CK(launch_features_tan(featp, featt, ehf, n_grid, np, clip, S.squash_offset, x, xt, U, e, et, st),
          "hvp_tc features");
  GDFT_CK(launch_pack_rt<double>(U, rows2, S.n_in, kDm21InPad, rt2, 1, PU, st), "hvp_tc pack u");
  // Each row pass also packs [h; h~] for the next dense layer (rt) and, with
  // dparams, for that layer's weight gradient (ct).
  GDFT_CK(gemm_act(PU, 1, WTi(0), Z), "hvp_tc dense_0");
  tan_fwd_pack_kernel<PL, true><<<kLnBlocks, 256, 0, st>>>(Z, b0f, H, nullptr, nullptr, 0.0, np,
                                                           S.n_layers > 0 ? PH : nullptr,
                                                           (dparams && S.n_layers > 0) ? CHi(0) : nullptr);
  GDFT_CK(cudaGetLastError(), "hvp_tc tanh");
  for (int i = 1; i <= S.n_layers; ++i) {
    const float *Wif = pf + hvp_tc_layer_offset(S, i - 1), *bi = Wif + (size_t)Wd * Wd, *gi = bi + Wd,
                *bei = gi + Wd;
    float *Zi = Z + (size_t)i * act2;
    GDFT_CK(gemm_act(PH, kcw, WTi(i), Zi), "hvp_tc dense_i");
    const bool more = i < S.n_layers;
    tan_fwd_pack_kernel<PL, false><<<kLnBlocks, 256, 0, st>>>(Zi, bi, H, gi, bei, S.ln_eps, np,
                                                              more ? PH : nullptr,
                                                              (dparams && more) ? CHi(i) : nullptr);
    GDFT_CK(cudaGetLastError(), "hvp_tc layernorm");
  }
  head_tan_tc_kernel<PL><<<pblocks, 256, 0, st>>>(H, Wof, bo, e, et, w, n_grid, np, clip, S.sigmoid_scale, GY, GYf,
                                                  GE, lpart);
  GDFT_CK(cudaGetLastError(), "hvp_tc head");
  if (lval) GDFT_CK(launch_energy_reduce(lpart, (int)pblocks, lval, st), "hvp_tc value");

  // ---- reverse of the augmented graph ----
  if (dparams) {
    head_wgrad_part_kernel<<<kHeadBlocks, 256, 0, st>>>(H, GYf, GY, rows2, np, Wd, colpart);
    launch_colsum_final(colpart, kHeadBlocks, 3 * Wd + 3, dparams + head_off, st);
    GDFT_CK(cudaGetLastError(), "hvp_tc head wgrad");
  }
  float *gz_cur = GZ, *gz_prev = GZ + act2;
  GDFT_CK(cudaFuncSetAttribute(tan_bwd_pack_kernel<PL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)bwd_pack_smem<PL>()),
          "hvp_tc layernorm bwd smem");
  for (int i = S.n_layers; i >= 1; --i) {
    const float *Wif = pf + hvp_tc_layer_offset(S, i - 1), *gi = Wif + (size_t)Wd * Wd + Wd, *bei = gi + Wd;
    const float *Zi = Z + (size_t)i * act2;
    const bool last = i == S.n_layers;
    tan_bwd_pack_kernel<PL><<<kLnBlocks, 256, bwd_pack_smem<PL>(), st>>>(
        last ? nullptr : DHP, last ? nullptr : gz_prev, last ? GYf : nullptr, Wof, Zi, gi, bei, S.ln_eps, np, gz_cur,
        lnpart, PG, dparams ? CG : nullptr);
    GDFT_CK(cudaGetLastError(), "hvp_tc layernorm bwd");
    if (dparams) {
      double *dWi = dparams + hvp_tc_layer_offset(S, i - 1);
      GDFT_CK(gemm_wgrad(CHi(i - 1), ft, Wd, CG, dWi), "hvp_tc dW_i");
      launch_colsum_final(lnpart, kLnBlocks, 3 * Wd, colpart2, st);
      GDFT_CK(cudaGetLastError(), "hvp_tc ln sums");
      GDFT_CK(cudaMemcpyAsync(dWi + (size_t)Wd * Wd, colpart2 + 2 * Wd, Wd * sizeof(double),
                              cudaMemcpyDeviceToDevice, st),
              "hvp_tc db");
      GDFT_CK(cudaMemcpyAsync(dWi + (size_t)Wd * Wd + Wd, colpart2, 2 * Wd * sizeof(double),
                              cudaMemcpyDeviceToDevice, st),
              "hvp_tc dln");
    }
    GDFT_CK(gemm_act(PG, kcw, WRi(i), DHP), "hvp_tc dh");
    float *t = gz_cur;
    gz_cur = gz_prev;
    gz_prev = t;
  }
  // Layer 0: gz_prev holds [dL/dz_1; dL/dz_1~], DHP its product with W_1^T.
  // One pass gives GU and the FP64 partials of [dW0 | db0] (kpart is free by
  // now and holds kLnBlocks x (n_in + 1) x W doubles: 4 (n_in + 1) <= W).
  GDFT_CK(cudaFuncSetAttribute(tanh_tan_bwd_fused_kernel<PL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)l0_tan_bwd_smem<PL>()),
          "hvp_tc tanh bwd smem");
  tanh_tan_bwd_fused_kernel<PL><<<kLnBlocks, 256, l0_tan_bwd_smem<PL>(), st>>>(
      DHP, gz_prev, Z, U, W0f, S.n_in, np, coef ? GU : nullptr, dparams ? kpart : nullptr);
  GDFT_CK(cudaGetLastError(), "hvp_tc tanh bwd");
  if (dparams) {
    launch_colsum_final(kpart, kLnBlocks, (S.n_in + 1) * Wd, dparams, st);
    GDFT_CK(cudaGetLastError(), "hvp_tc dW_0");
  }
  if (coef)
    GDFT_CK(launch_hvp_potentials(featp, featt, x, xt, GU, GE, n_grid, np, clip, S.squash_offset, coef, st),
            "hvp_tc potentials");
#undef GDFT_CK
  return GDFT_OK;
}

}  // namespace

MlpHvpTcLayout mlp_hvp_tc_layout(const MlpShape &s, int64_t np) {
  MlpHvpTcLayout L;
  const int W = s.width;
  const int64_t rows2 = 2 * np;
  const size_t act2 = (size_t)rows2 * W;
  const int64_t rt2 = rows2 / kPointTile, rc2 = rows2 / 32;
  const int ft = W / 128, kcw = W / 32;
  const int nl = s.n_layers > 0 ? s.n_layers : 1;
  L.nsplit = 148;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  L.featp = take((size_t)2 * kFeat * np * 8);
  L.x = take((size_t)np * kDm21In * 8);
  L.xt = take((size_t)np * kDm21In * 8);
  L.u = take((size_t)rows2 * kDm21InPad * 8);
  L.e = take((size_t)np * 3 * 8);
  L.et = take((size_t)np * 8);
  L.gy = take((size_t)rows2 * 3 * 8);
  L.ge = take((size_t)np * 2 * 8);
  L.gu = take((size_t)rows2 * kDm21InPad * 8);
  L.lpart = take((size_t)((np + 255) / 256) * 8);
  L.kpart = take((size_t)L.nsplit * W * W * 8);
  L.lnpart = take((size_t)kLnBlocks * 3 * W * 8);
  L.colpart = take((size_t)kHeadBlocks * (3 * W + 3) * 8);
  L.colpart2 = take((size_t)3 * W * 8);
  L.pf = take(mlp_param_count(s) * 4);
  L.gyf = take((size_t)rows2 * 3 * 4);
  L.pu = take((size_t)rt2 * kBlk * 4);
  L.wt = take(((size_t)ft * kBlk + (size_t)s.n_layers * ft * kcw * kBlk) * 4);
  L.wr = take((size_t)nl * ft * kcw * kBlk * 4);
  L.z = take(act2 * (s.n_layers + 1) * 4);
  L.h = take(act2 * 4);
  L.ph = take((size_t)rt2 * kcw * kBlk * 4);
  L.ch = take((size_t)nl * ft * rc2 * kBlk * 4);
  L.gz = take(2 * act2 * 4);
  L.dhp = take(act2 * 4);
  L.pg = take((size_t)rt2 * kcw * kBlk * 4);
  L.cg = take((size_t)ft * rc2 * kBlk * 4);
  L.bytes = off;
  return L;
}

int mlp_hvp_tc(const MlpShape &S, const double *params, double *dparams, const double *featp, const double *featt,
               const double *ehf, const double *w, int64_t n_grid, int64_t np, double clip, char *ws, double *lval,
               double *coef, int *err, cudaStream_t st) {
  if (np % kPointTile != 0 || S.n_layers < 1) {
    set_error("mlp_hvp_tc: grid padding or layer count not supported");
    return GDFT_ERR_INVALID;
  }
  switch (S.width) {
    case 128:
      return run_hvp_tc<4>(S, params, dparams, featp, featt, ehf, w, n_grid, np, clip, ws, lval, coef, err, st);
    case 256:
      return run_hvp_tc<8>(S, params, dparams, featp, featt, ehf, w, n_grid, np, clip, ws, lval, coef, err, st);
    default:
      set_error("mlp_hvp_tc: width %d not built for the mixed form (128 or 256)", S.width);
      return GDFT_ERR_UNSUPPORTED;
  }
}

}  // namespace gdft
