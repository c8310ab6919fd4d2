// vxc_q.cu - mixed form of the V_xc contraction as a packed tensor-core GEMM.
//
//   V_sigma[a][b] = sum_r sum_t P_t[r][a] Q_sigma,t[r][b]
//   Q_sigma,0 = c_rho phi + c_gx d_x phi + c_gy d_y phi + c_gz d_z phi + c_lap lap phi
//   Q_sigma,j = c_kin d_j phi                                    (j = x, y, z)
// with P_0 = phi, P_j = d_j phi and c the per-point adjoint coefficients (the
// transposed density contraction of jax.grad at train.py:86; the same sum as
// vxc_f64.cu).  A memory-bound pre-pass forms Q for both spins once per call,
// directly as block-scaled three-slice sets (umma::split3) in the AO-major
// layout of the AO tables; the contraction is then tcg3_kernel with A = the
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

// One CTA per (b tile, 32-point chunk): reads the five AO-major FP32 planes of
// that block and the chunk's coefficients, writes Q for 2 spins x 4 planes as
// hi|lo|lo2 sets.  A block is 1024 16-byte items in memory order c = 64 g +
// 8 k4 + r (AO row 8 g + r, points 4 k4 .. 4 k4 + 3); warp w takes row groups
// 2w and 2w + 1, lane l the items c = 64 g + l and 64 g + 32 + l of each, so
// every warp access is 512 contiguous bytes and a thread holds half of its
// row's points.  A row's quantum needs only the exponent of its largest value:
// a spin's four plane exponents travel as the bytes of one word (byte max over
// the thread's two items, then over the four lanes l ^ 8, l ^ 16 that share
// the row).
__global__ void __launch_bounds__(256) build_q_kernel(const float *__restrict__ af, const double *__restrict__ coef,
                                                      int64_t np, int nbt, float *__restrict__ q) {
  __shared__ __align__(16) float sc[2][kFeat][32];  // [spin][coefficient][point]
  const int64_t npc = np / 32;
  const int bt = (int)(blockIdx.x / npc);
  const int64_t pc = blockIdx.x % npc;
  for (int i = threadIdx.x; i < 2 * kFeat * 32; i += blockDim.x)
    (&sc[0][0][0])[i] = (float)coef[(size_t)(i / 32) * np + pc * 32 + i % 32];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float *src[kPlanes];
#pragma unroll
  for (int p = 0; p < kPlanes; ++p) src[p] = af + ((size_t)(bt * kPlanes + p) * npc + pc) * kBlkF;
#pragma unroll 1
  for (int gi = 0; gi < 2; ++gi) {
    const int g = 2 * warp + gi;
    uint32_t off[2];
    float4 v[2][kPlanes];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      off[h] = (uint32_t)(64 * g + 32 * h + lane) * 4;  // floats
#pragma unroll
      for (int p = 0; p < kPlanes; ++p) v[h][p] = __ldg((const float4 *)(src[p] + off[h]));
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      float qv[2][4][4];  // [item][plane t][point j]
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int p0 = 4 * (4 * h + (lane >> 3));  // first point of the item
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float ph = (&v[h][T_PHI].x)[j], dx = (&v[h][T_DX].x)[j], dy = (&v[h][T_DY].x)[j],
                      dz = (&v[h][T_DZ].x)[j], lp = (&v[h][T_LAP].x)[j];
          const float *c = &sc[s][0][p0 + j];
          const float ck = c[32 * C_KIN];
          qv[h][0][j] = c[32 * C_RHO] * ph + c[32 * C_GX] * dx + c[32 * C_GY] * dy + c[32 * C_GZ] * dz +
                        c[32 * C_LAP] * lp;
          qv[h][1][j] = ck * dx;
          qv[h][2][j] = ck * dy;
          qv[h][3][j] = ck * dz;
        }
      }
      uint32_t ebw = 0u;  // byte t: exponent field of the largest |Q_t| of the row
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        float m = 0.0f;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int j = 0; j < 4; ++j) m = fmaxf(m, fabsf(qv[h][t][j]));
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
          umma::split3(qv[h][t][0], uq, hi.x, lo.x, lo2.x);
          umma::split3(qv[h][t][1], uq, hi.y, lo.y, lo2.y);
          umma::split3(qv[h][t][2], uq, hi.z, lo.z, lo2.z);
          umma::split3(qv[h][t][3], uq, hi.w, lo.w, lo2.w);
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
