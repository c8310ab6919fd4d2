// vxc_tc.cu - mixed (TF32x3) form of the V_xc contraction on tcgen05.
//
// V_sigma = sum_t P_t^T Q_sigma,t over the grid (operands as in vxc_f64.cu),
// computed per output tile a-block (128) x b-block (64) x both spins over a
// slice of the grid (split-K).  Per stage (32 grid points, one plane t):
//   A = P_t[points, a-block]^T : one 32 KB bulk copy (TMA) of the AO-major
//       hi/lo tables;
//   B = Q_sigma,t[points, b-block]^T for both spins: built in shared memory by
//       four warps from the AO-major FP32 planes and the per-point adjoint
//       coefficients, split into TF32 hi/lo.
// Three TF32 products per term (M = 128, N = 64).
//
// Accumulation: the tensor cores truncate each MMA's result to the
// accumulator's ulp grid, an error proportional to the accumulator's size at
// that instruction.  So each stage (32 grid points of one plane, 12 MMAs per
// accumulator) is accumulated in TMEM region W (double-buffered), with the
// small hi*lo and lo*hi correction products issued first (while the
// accumulator is still small) and the hi*hi products last; four drain warps
// fold every stage into a Kahan-compensated FP32 running sum (S, C) kept in
// TMEM, with round-to-nearest arithmetic on the CUDA cores.  The slice's sum
// S - C is written once, in FP64.
//
// Warp roles (320 threads): warp 0 = TMA producer of A, warp 1 = TMEM owner
// and MMA issuer, warps 2-5 = B builders, warps 6-9 = drainers.  All waits
// are bounded; on expiry the CTA records an error word and winds down.
#include "common.cuh"
#include "kernels.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr int kStages = 3;
constexpr uint32_t kHalfBlock = umma::kBlockBytes / 2;                   // 64 rows x 32 fp32
constexpr uint32_t kStageBytes = 2 * umma::kBlockBytes + 4 * kHalfBlock;  // A hi|lo, Q_a hi|lo, Q_b hi|lo
constexpr int kThreads = 320;
constexpr uint32_t kTmemCols = 512;  // W0 [0,128), W1 [128,256), S [256,384), C [384,512)
constexpr int kBN = 64;              // b-block
constexpr int kCoefBytes = 32 * 12 * 4;
constexpr int kSmemBytes = kStages * kStageBytes + 1024 + kCoefBytes;

struct VxcArgs {
  const float *am;     // AO-major hi/lo tables (4 planes)
  const float *af;     // AO-major FP32 tables (5 planes)
  const double *coef;  // [2][6][np]
  int64_t np;
  int ldk;
  int n;
  int64_t range;  // grid points per slice (multiple of 32)
  double *vpart;  // [nsplit][2][n][n]
  int *err;
};

__device__ __forceinline__ const float *am_blk(const VxcArgs &A, int atile, int plane, int64_t pc) {
  const int64_t npc = A.np / 32;
  return A.am + ((size_t)(atile * 4 + plane) * npc + pc) * 2 * (umma::kBlockBytes / 4);
}
__device__ __forceinline__ const float *af_blk(const VxcArgs &A, int atile, int plane, int64_t pc) {
  const int64_t npc = A.np / 32;
  return A.af + ((size_t)(atile * kPlanes + plane) * npc + pc) * (umma::kBlockBytes / 4);
}

__device__ __forceinline__ void flag(int *err, int code) { atomicCAS(err, 0, code); }
__device__ __forceinline__ void builders_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__device__ __forceinline__ void st_split(unsigned char *blk, uint32_t off, float4 q) {
  float4 h, l;
  umma::split_tf32f(q.x, h.x, l.x);
  umma::split_tf32f(q.y, h.y, l.y);
  umma::split_tf32f(q.z, h.z, l.z);
  umma::split_tf32f(q.w, h.w, l.w);
  *(float4 *)(blk + off) = h;
  *(float4 *)(blk + kHalfBlock + off) = l;
}

__global__ void __launch_bounds__(kThreads, 1) vxc_tc_kernel(const VxcArgs A) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float *scoef = (float *)(smem + kStages * kStageBytes);  // [32 points][2 spins][6]
  __shared__ __align__(8) uint64_t afull[kStages], bfull[kStages], empty[kStages], wfull[2], wempty[2], drain;
  __shared__ uint32_t tmem_base;
  __shared__ int s_ok;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_b = A.ldk / kBN;
  const int ta = blockIdx.x / tiles_b, tb = blockIdx.x % tiles_b;
  const int64_t r0 = (int64_t)blockIdx.y * A.range;
  const int64_t r1 = r0 + A.range < A.np ? r0 + A.range : A.np;
  const int64_t npcs = r1 > r0 ? (r1 - r0) / 32 : 0;  // point chunks (= windows) of this slice
  const int64_t nst = npcs * 4;                       // stages

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      umma::mbar_init(&afull[s], 1);
      umma::mbar_init(&bfull[s], 128);
      umma::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(&wfull[b], 1);
      umma::mbar_init(&wempty[b], 128);
    }
    umma::mbar_init(&drain, 1);
    umma::fence_barrier_init();
  }
  if (warp == 1) umma::tmem_alloc(&tmem_base, kTmemCols);
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tbase = tmem_base;

  if (warp == 0) {
    // ------------------------------------------------------------ A producer
    int64_t it = 0;
    for (; it < nst; ++it) {
      const int s = (int)(it % kStages);
      if (!umma::warp_wait(&empty[s], ((it / kStages) & 1) ^ 1)) {
        if (lane == 0) flag(A.err, 21);
        break;
      }
      if (lane == 0) {
        umma::mbar_arrive_expect_tx(&afull[s], 2 * umma::kBlockBytes);
        umma::bulk_g2s(smem + s * kStageBytes, am_blk(A, ta, (int)(it % 4), r0 / 32 + it / 4),
                       2 * umma::kBlockBytes, &afull[s]);
      }
      __syncwarp();
    }
    for (int64_t i = it > kStages ? it - kStages : 0; i < it; ++i)
      if (!umma::warp_wait(&afull[i % kStages], (i / kStages) & 1) && lane == 0) flag(A.err, 22);
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    const uint32_t idesc = umma::idesc_tf32(128, kBN);
    for (int64_t it = 0; it < nst; ++it) {
      const int s = (int)(it % kStages);
      const int buf = (int)(it & 1);
      if (!umma::warp_wait(&wempty[buf], ((it >> 1) & 1) ^ 1)) {
        if (lane == 0) flag(A.err, 23);
        break;
      }
      umma::tc_fence_after();
      const uint32_t ph = (it / kStages) & 1;
      if (!umma::warp_wait(&afull[s], ph) || !umma::warp_wait(&bfull[s], ph)) {
        if (lane == 0) flag(A.err, 24);
        break;
      }
      umma::tc_fence_after();
      if (lane == 0) {
        const uint32_t sb = umma::smem_u32(smem + s * kStageBytes);
#pragma unroll
        for (int sp = 0; sp < 2; ++sp) {
          const uint32_t d = tbase + buf * 128 + sp * kBN;
          // Corrections first (hi*lo, lo*hi), then the hi*hi products.
#pragma unroll
          for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint64_t ahi = umma::sdesc(sb + kk * 256, umma::kBlockLBO, umma::kBlockSBO);
              const uint64_t alo = umma::sdesc(sb + umma::kBlockBytes + kk * 256, umma::kBlockLBO, umma::kBlockSBO);
              const uint32_t bb = sb + 2 * umma::kBlockBytes + sp * 2 * kHalfBlock + kk * 256;
              const uint64_t bhi = umma::sdesc(bb, umma::kBlockLBO, umma::kBlockSBO);
              const uint64_t blo = umma::sdesc(bb + kHalfBlock, umma::kBlockLBO, umma::kBlockSBO);
              if (pass == 0) {
                umma::mma_tf32(d, ahi, blo, idesc, kk == 0 ? 0u : 1u);
                umma::mma_tf32(d, alo, bhi, idesc, 1u);
              } else {
                umma::mma_tf32(d, ahi, bhi, idesc, 1u);
              }
            }
          }
        }
        umma::mma_commit(&empty[s]);
        umma::mma_commit(&wfull[buf]);
      }
      __syncwarp();
    }
    if (lane == 0) umma::mma_commit(&drain);
    __syncwarp();
    if (!umma::warp_wait(&drain, 0) && lane == 0) flag(A.err, 25);
  } else if (warp < 6) {
    // ----------------------------------------------------------- B builders
    // The four builder warps decide every wait together (one thread polls,
    // a named barrier publishes the result), so they leave their loop at the
    // same iteration and never strand each other on bar.sync.
    const int bt = threadIdx.x - 64;  // 0..127
    const int row = bt & (kBN - 1);   // b row within the block
    const int gq = bt >> 6;           // which half of the 8 point groups
    const int btile = (tb * kBN) / 128, rsub = (tb * kBN) % 128;
    for (int64_t it = 0; it < nst; ++it) {
      const int s = (int)(it % kStages);
      const int64_t pcl = it / 4;
      const int64_t pc = r0 / 32 + pcl;
      const int t = (int)(it % 4);
      builders_sync();  // everyone is done with the previous stage and coefficients
      if (bt == 0) s_ok = umma::mbar_wait(&empty[s], ((it / kStages) & 1) ^ 1) ? 1 : 0;
      if (t == 0) {
        for (int i = bt; i < 32 * 12; i += 128) {
          const int pt = i / 12, k = i % 12;
          const int sp = k / 6, c = k % 6;
          scoef[i] = (float)A.coef[((size_t)sp * kFeat + c) * A.np + (pc * 32 + pt)];
        }
      }
      builders_sync();
      if (!s_ok) {
        if (bt == 0) flag(A.err, 26);
        break;
      }
      unsigned char *qa = smem + s * kStageBytes + 2 * umma::kBlockBytes;
      unsigned char *qb = qa + 2 * kHalfBlock;
      // All plane loads of the stage are issued before any use (memory-level parallelism).
      if (t == 0) {
        float4 ph[4], dx[4], dy[4], dz[4], lp[4];
#pragma unroll
        for (int gg = 0; gg < 4; ++gg) {
          const int g = gq * 4 + gg;
          const uint32_t src = (uint32_t)((((rsub + row) >> 3) * 8 + g) * 128 + (row & 7) * 16) / 4;
          ph[gg] = __ldg((const float4 *)(af_blk(A, btile, T_PHI, pc) + src));
          dx[gg] = __ldg((const float4 *)(af_blk(A, btile, T_DX, pc) + src));
          dy[gg] = __ldg((const float4 *)(af_blk(A, btile, T_DY, pc) + src));
          dz[gg] = __ldg((const float4 *)(af_blk(A, btile, T_DZ, pc) + src));
          lp[gg] = __ldg((const float4 *)(af_blk(A, btile, T_LAP, pc) + src));
        }
#pragma unroll
        for (int gg = 0; gg < 4; ++gg) {
          const int g = gq * 4 + gg;
          const uint32_t dst = (uint32_t)(((row >> 3) * 8 + g) * 128 + (row & 7) * 16);
          const float *cf = scoef + (4 * g) * 12;
          const float *c0 = cf, *c1 = cf + 12, *c2 = cf + 24, *c3 = cf + 36;
#define GDFT_Q0(SP, C, F)                                                                                   \
  (C[SP * 6 + C_RHO] * ph[gg].F + C[SP * 6 + C_GX] * dx[gg].F + C[SP * 6 + C_GY] * dy[gg].F +               \
   C[SP * 6 + C_GZ] * dz[gg].F + C[SP * 6 + C_LAP] * lp[gg].F)
          st_split(qa, dst, make_float4(GDFT_Q0(0, c0, x), GDFT_Q0(0, c1, y), GDFT_Q0(0, c2, z), GDFT_Q0(0, c3, w)));
          st_split(qb, dst, make_float4(GDFT_Q0(1, c0, x), GDFT_Q0(1, c1, y), GDFT_Q0(1, c2, z), GDFT_Q0(1, c3, w)));
#undef GDFT_Q0
        }
      } else {
        float4 dj[4];
#pragma unroll
        for (int gg = 0; gg < 4; ++gg) {
          const int g = gq * 4 + gg;
          const uint32_t src = (uint32_t)((((rsub + row) >> 3) * 8 + g) * 128 + (row & 7) * 16) / 4;
          dj[gg] = __ldg((const float4 *)(af_blk(A, btile, T_PHI + t, pc) + src));
        }
#pragma unroll
        for (int gg = 0; gg < 4; ++gg) {
          const int g = gq * 4 + gg;
          const uint32_t dst = (uint32_t)(((row >> 3) * 8 + g) * 128 + (row & 7) * 16);
          const float *cf = scoef + (4 * g) * 12;
          st_split(qa, dst, make_float4(cf[C_KIN] * dj[gg].x, cf[12 + C_KIN] * dj[gg].y, cf[24 + C_KIN] * dj[gg].z,
                                        cf[36 + C_KIN] * dj[gg].w));
          st_split(qb, dst, make_float4(cf[6 + C_KIN] * dj[gg].x, cf[18 + C_KIN] * dj[gg].y,
                                        cf[30 + C_KIN] * dj[gg].z, cf[42 + C_KIN] * dj[gg].w));
        }
      }
      umma::fence_proxy_async();
      umma::mbar_arrive(&bfull[s]);
    }
  } else {
    // --------------------------------------------------------------- drains
    const int q = warp & 3;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16);
    int64_t it = 0;
    for (; it < nst; ++it) {
      const int buf = (int)(it & 1);
      if (!umma::warp_wait(&wfull[buf], (it >> 1) & 1)) {
        if (lane == 0) flag(A.err, 27);
        break;
      }
      umma::tc_fence_after();
#pragma unroll 1
      for (int c = 0; c < 128; c += 32) {
        float w[32];
        umma::tmem_ld32(tl + buf * 128 + c, w);
        if (it == 0) {
          float z[32];
#pragma unroll
          for (int i = 0; i < 32; ++i) z[i] = 0.0f;
          umma::tmem_st32(tl + 256 + c, w);
          umma::tmem_st32(tl + 384 + c, z);
        } else {
          float sv[32], cv[32];
          umma::tmem_ld32(tl + 256 + c, sv);
          umma::tmem_ld32(tl + 384 + c, cv);
#pragma unroll
          for (int i = 0; i < 32; ++i) {  // Kahan: s + (w - c), c = rounding error
            const float y = w[i] - cv[i];
            const float tt = sv[i] + y;
            cv[i] = (tt - sv[i]) - y;
            sv[i] = tt;
          }
          umma::tmem_st32(tl + 256 + c, sv);
          umma::tmem_st32(tl + 384 + c, cv);
        }
      }
      umma::tmem_st_wait();
      umma::tc_fence_before();
      umma::mbar_arrive(&wempty[buf]);
    }
    // The slice's sums, once, in FP64 (zeros for a slice without points).
    const int a = ta * 128 + q * 32 + lane;
    double *vp = A.vpart + (size_t)blockIdx.y * 2 * A.n * A.n;
    const bool have = it == nst && nst > 0;
#pragma unroll 1
    for (int c = 0; c < 128; c += 32) {
      float sv[32], cv[32];
      if (have) {
        umma::tmem_ld32(tl + 256 + c, sv);
        umma::tmem_ld32(tl + 384 + c, cv);
      }
      const int sp = c / kBN;
      if (a < A.n) {
        double *row = vp + ((size_t)sp * A.n + a) * A.n;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int b = tb * kBN + (c % kBN) + i;
          if (b < A.n) row[b] = have ? (double)sv[i] - (double)cv[i] : 0.0;
        }
      }
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 1) umma::tmem_dealloc(tbase, kTmemCols);
}

}  // namespace

int vxc_tc_splits(int64_t np, int n_ao, int64_t *range) {
  const int ldk = (int)round_up(n_ao, 128);
  const int ntiles = (ldk / 128) * (ldk / kBN);
  // Whole waves of 148 CTAs where the tile count allows it.
  int want = 1;
  if (ntiles < 148) {
    int waves = 1;
    while ((148 * waves) % ntiles > ntiles / 4 && waves < 4) ++waves;
    want = (148 * waves) / ntiles;
    if (want < 1) want = 1;
  }
  int64_t r = round_up((np + want - 1) / want, 32);
  if (r < 32) r = 32;
  *range = r;
  return (int)((np + r - 1) / r);
}

cudaError_t launch_vxc_tc(const float *am, const float *af, const double *coef, int64_t np, int ldk, int n_ao,
                          int nsplit, int64_t range, double *vpart, int *err, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(vxc_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  VxcArgs a{am, af, coef, np, ldk, n_ao, range, vpart, err};
  dim3 grid((ldk / 128) * (ldk / kBN), nsplit);
  vxc_tc_kernel<<<grid, kThreads, kSmemBytes, st>>>(a);
  return cudaGetLastError();
}

}  // namespace gdft
