// vxc_q.cu - mixed form of the V_xc contraction as a packed tensor-core GEMM.
//
//   V_sigma[a][b] = sum_r sum_t P_t[r][a] Q_sigma,t[r][b]
//   Q_sigma,0 = c_rho phi + c_gx d_x phi + c_gy d_y phi + c_gz d_z phi + c_lap lap phi
//   Q_sigma,j = c_kin d_j phi                                    (j = x, y, z)
// with P_0 = phi, P_j = d_j phi and c the per-point adjoint coefficients (the
// transposed density contraction of jax.grad at train.py:86; the same sum as
// vxc_f64.cu).  A memory-bound pre-pass forms Q for both spins once per call,
// in double-float arithmetic from FP32 pairs of the planes and of the FP64
// coefficients (a Q formed in FP32, rounded at 2^-24 per element, left V_xc
// errors near 1e-7 of its largest entry at n_ao 512, 2^20 points), directly
// as block-scaled three-slice sets in the AO-major layout of the AO tables; the contraction is then tcg3_kernel with A = the
// AO-major phi planes (K = 4 planes x grid points), B = Q of both spins
// (N = 2 x n_ao), split-K over the grid, FP64 partials, and a reduction that
// also splits the spins.  Both operands' hi slices are quantised per row and
// 32-point chunk, so each chunk's hi*hi sum is exact in the tensor core's FP32
// accumulator and only the corrections (below 2^-10 of the terms) meet its
// truncation.
#include "common.cuh"
#include "kernels.cuh"
#include "tc_gemm.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr int kBlkF = umma::kBlockBytes / 4;  // floats in one 128 x 32 block

// Double-float values s + c (|c| below an ulp of s, up to rounding).
struct DF {
  float s, c;
};
// (ch + cl)(th + tl) to about 2^-44: the FP32 product, its exact rounding
// error (FMA) and the cross terms (the lo * lo term is below 2^-48).
__device__ __forceinline__ DF df_mul(float ch, float cl, float th, float tl) {
  const float p = __fmul_rn(ch, th);
  const float e = fmaf(ch, th, -p);
  return DF{p, e + fmaf(ch, tl, __fmul_rn(cl, th))};
}
// a + t with TwoSum on the leading parts.
__device__ __forceinline__ DF df_add(DF a, DF t) {
  const float s = __fadd_rn(a.s, t.s);
  const float bp = __fsub_rn(s, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bp)), __fsub_rn(t.s, bp));
  return DF{s, a.c + (t.c + err)};
}
// Renormalise (s, c) so that c is below an ulp of s (TwoSum).
__device__ __forceinline__ DF df_norm(DF a) {
  const float s = __fadd_rn(a.s, a.c);
  const float bp = __fsub_rn(s, a.s);
  return DF{s, __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bp)), __fsub_rn(a.c, bp))};
}
// Block-scaled three-slice split of s + c on the row quantum u: hi = s
// rounded to the quantum (exact), the remainder (s - hi) + c rounded once to
// FP32 (below 2^-34 of the row maximum), then its two TF32 slices.
__device__ __forceinline__ void df_split3(DF v, umma::Quant u, float &hi, float &lo, float &lo2) {
  hi = rintf(v.s * u.inv) * u.q;
  const float r = __fadd_rn(__fsub_rn(v.s, hi), v.c);
  lo = umma::tf32_rn(r);
  lo2 = umma::tf32_rn(__fsub_rn(r, lo));
}

// One CTA per (b tile, 32-point chunk): reads the five AO-major planes of
// that block as FP32 pairs (hi + lo, about 2^-48 of each value) and the
// chunk's FP64 coefficients (split into FP32 pairs), forms Q for 2 spins x 4
// planes in double-float arithmetic (each product with its FMA error, TwoSum
// accumulation: about 2^-44 of the terms) and writes hi|lo|lo2 sets whose
// representation error is below 2^-33 of each row's largest value.  A block
// is 1024 16-byte items in memory order c = 64 g + 8 k4 + r (AO row 8 g + r,
// points 4 k4 .. 4 k4 + 3); warp w takes row groups 2w and 2w + 1, lane l the
// items c = 64 g + l and 64 g + 32 + l of each, so every warp access is 512
// contiguous bytes and a thread holds half of its row's points.  A row's
// quantum needs only the exponent of its largest value: a spin's four plane
// exponents travel as the bytes of one word (byte max over the thread's two
// items, then over the four lanes l ^ 8, l ^ 16 that share the row).
__global__ void __launch_bounds__(256, 2) build_q_kernel(const float *__restrict__ af,
                                                         const double *__restrict__ coef, int64_t np, int nbt,
                                                         float *__restrict__ q) {
  __shared__ __align__(16) float sch[2][kFeat][32], scl[2][kFeat][32];  // [spin][coefficient][point] hi, lo
  const int64_t npc = np / 32;
  const int bt = (int)(blockIdx.x / npc);
  const int64_t pc = blockIdx.x % npc;
  for (int i = threadIdx.x; i < 2 * kFeat * 32; i += blockDim.x) {
    const double c = coef[(size_t)(i / 32) * np + pc * 32 + i % 32];
    const float ch = (float)c;
    (&sch[0][0][0])[i] = ch;
    (&scl[0][0][0])[i] = (float)(c - (double)ch);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float *src[kPlanes];
#pragma unroll
  for (int p = 0; p < kPlanes; ++p) src[p] = af + ((size_t)(bt * kPlanes + p) * npc + pc) * 2 * kBlkF;
#pragma unroll 1
  for (int gi = 0; gi < 2; ++gi) {
    const int g = 2 * warp + gi;
    uint32_t off[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) off[h] = (uint32_t)(64 * g + 32 * h + lane) * 4;  // floats
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
      DF qv[2][4][4];  // [item][plane t][point j]
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        // The item's plane values (the second spin re-reads them from L1).
        float4 vh[kPlanes], vl[kPlanes];
#pragma unroll
        for (int p = 0; p < kPlanes; ++p) {
          vh[p] = __ldg((const float4 *)(src[p] + off[h]));
          vl[p] = __ldg((const float4 *)(src[p] + kBlkF + off[h]));
        }
        const int p0 = 4 * (4 * h + (lane >> 3));  // first point of the item
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float *ch = &sch[s][0][p0 + j], *cl = &scl[s][0][p0 + j];
          float th[kPlanes], tl[kPlanes];
#pragma unroll
          for (int p = 0; p < kPlanes; ++p) {
            th[p] = (&vh[p].x)[j];
            tl[p] = (&vl[p].x)[j];
          }
          DF a = df_mul(ch[32 * C_RHO], cl[32 * C_RHO], th[T_PHI], tl[T_PHI]);
          a = df_add(a, df_mul(ch[32 * C_GX], cl[32 * C_GX], th[T_DX], tl[T_DX]));
          a = df_add(a, df_mul(ch[32 * C_GY], cl[32 * C_GY], th[T_DY], tl[T_DY]));
          a = df_add(a, df_mul(ch[32 * C_GZ], cl[32 * C_GZ], th[T_DZ], tl[T_DZ]));
          a = df_add(a, df_mul(ch[32 * C_LAP], cl[32 * C_LAP], th[T_LAP], tl[T_LAP]));
          qv[h][0][j] = df_norm(a);
#pragma unroll
          for (int d = 1; d < 4; ++d)
            qv[h][d][j] = df_norm(df_mul(ch[32 * C_KIN], cl[32 * C_KIN], th[T_PHI + d], tl[T_PHI + d]));
        }
      }
      uint32_t ebw = 0u;  // byte t: exponent field of the largest |Q_t| of the row
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        float m = 0.0f;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int j = 0; j < 4; ++j) m = fmaxf(m, fabsf(qv[h][t][j].s));
        ebw |= ((__float_as_uint(m) >> 23) & 0xFFu) << (8 * t);
      }
      ebw = __vmaxu4(ebw, __shfl_xor_sync(0xffffffffu, ebw, 8));
      ebw = __vmaxu4(ebw, __shfl_xor_sync(0xffffffffu, ebw, 16));
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const umma::Quant uq = umma::quant_eb((ebw >> (8 * t)) & 0xFFu);
        float *set = q + ((((size_t)s * nbt + bt) * 4 + t) * npc + pc) * 3 * kBlkF;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          float4 hi, lo, lo2;
          df_split3(qv[h][t][0], uq, hi.x, lo.x, lo2.x);
          df_split3(qv[h][t][1], uq, hi.y, lo.y, lo2.y);
          df_split3(qv[h][t][2], uq, hi.z, lo.z, lo2.z);
          df_split3(qv[h][t][3], uq, hi.w, lo.w, lo2.w);
          *(float4 *)(set + off[h]) = hi;
          *(float4 *)(set + kBlkF + off[h]) = lo;
          *(float4 *)(set + 2 * kBlkF + off[h]) = lo2;
        }
      }
    }
  }
}

// V[s][a][b] = sum over splits of part[split][a][s * ldk + b], a, b < n.
__global__ void vxc_q_reduce_kernel(const double *__restrict__ part, int nsplit, int n, int ldk,
                                    double *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)2 * n * n;
  if (i >= total) return;
  const int s = (int)(i / ((size_t)n * n)), a = (int)((i / n) % n), b = (int)(i % n);
  const size_t stride = (size_t)n * 2 * ldk;
  double acc = 0.0;
  for (int k = 0; k < nsplit; ++k) acc += part[(size_t)k * stride + (size_t)a * 2 * ldk + (size_t)s * ldk + b];
  out[i] = acc;
}

}  // namespace

// Split-K factor: about four waves of CTAs over the (a tile, b tile of both spins) grid.
int vxc_q_splits(int64_t np, int n_ao) {
  const int nbt = (int)(round_up(n_ao, 128) / 128);
  const int tiles = nbt * 2 * nbt;
  const int64_t kch = 4 * (np / 32);
  int s = (4 * 148 + tiles - 1) / tiles;
  if (s > kch) s = (int)kch;
  return s < 1 ? 1 : s;
}

size_t vxc_q_bytes(int64_t np, int n_ao) {
  const int ldk = (int)round_up(n_ao, 128);
  return (size_t)2 * 4 * np * ldk * 3 * sizeof(float);
}

cudaError_t launch_vxc_q_tc(const float *av, const float *af, const double *coef, int64_t np,
                            int ldk, int n_ao, float *q, int nsplit, double *vpart, double *vxc, int *err,
                            cudaStream_t st) {
  const int nbt = ldk / 128;
  const int64_t npc = np / 32;
  build_q_kernel<<<(unsigned)(nbt * npc), 256, 0, st>>>(af, coef, np, nbt, q);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  TcgArgs a{};
  a.a = av;
  a.b = q;
  a.m_tiles = nbt;
  a.n_tiles = 2 * nbt;
  a.a_chunks = a.b_chunks = a.k_chunks = 4 * npc;
  a.chunks_per_split = (a.k_chunks + nsplit - 1) / nsplit;
  a.out64 = vpart;
  a.m_valid = n_ao;
  a.n_valid = 2 * ldk;
  a.err = err;
  if ((e = launch_tcg3(a, nsplit, st)) != cudaSuccess) return e;
  const size_t total = (size_t)2 * n_ao * n_ao;
  vxc_q_reduce_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(vpart, nsplit, n_ao, ldk, vxc);
  return cudaGetLastError();
}

}  // namespace gdft
