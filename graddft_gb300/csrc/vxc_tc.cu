// vxc_tc.cu - mixed (TF32x3) form of the V_xc contraction on tcgen05.
//
// V_sigma = sum_t P_t^T Q_sigma,t over the grid (see vxc_f64.cu for the
// operands), computed per output tile a-block (128) x b-block (128) x both
// spins (2 x 128 TMEM columns, M = 128, N = 128) over a slice of the grid
// (split-K).  Per stage (32 grid points, one plane t):
//   A = P_t[points, a-block]^T  : one 32 KB bulk copy of the AO-major tables;
//   B = Q_sigma,t[points, b-block]^T for both spins: built in shared memory by
//       four warps from the AO-major planes and the per-point adjoint
//       coefficients (FP32), split into TF32 hi/lo.
// Three TF32 products per term, FP32 accumulation in TMEM for at most
// kDrainPts grid points; then the accumulator is drained into the FP64
// partial sums of this slice (global memory), so long grids never accumulate
// in FP32 beyond one drain window.
//
// Warp roles (192 threads): warp 0 = TMA producer of A, warp 1 = TMEM owner
// and MMA issuer, warps 2-5 = B builders and drainers.  All waits bounded.
#include "common.cuh"
#include "kernels.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr int kStages = 2;
constexpr uint32_t kStageBytes = 6 * umma::kBlockBytes;  // A hi|lo, Q_a hi|lo, Q_b hi|lo
constexpr int kThreads = 192;
constexpr uint32_t kTmemCols = 256;
constexpr int kDrainPts = 1024;
constexpr int kCoefBytes = 32 * 12 * 4;
constexpr int kSmemBytes = kStages * kStageBytes + 1024 + kCoefBytes;

struct VxcArgs {
  const float *am;     // AO-major resident tables
  const double *coef;  // [2][6][np]
  int64_t np;
  int ldk;
  int n;
  int64_t range;  // grid points per slice (multiple of kDrainPts)
  double *vpart;  // [nsplit][2][n][n]
  int *err;
};

__device__ __forceinline__ const float *am_blk(const VxcArgs &A, int atile, int plane, int64_t pc) {
  const int64_t npc = A.np / 32;
  return A.am + ((size_t)(atile * kPlanes + plane) * npc + pc) * 2 * (umma::kBlockBytes / 4);
}

__device__ __forceinline__ void flag(int *err, int code) { atomicCAS(err, 0, code); }

__device__ __forceinline__ void builders_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__device__ __forceinline__ float4 ld_pair(const float *blk, uint32_t off) {
  const float4 h = __ldg((const float4 *)(blk + off / 4));
  const float4 l = __ldg((const float4 *)(blk + umma::kBlockBytes / 4 + off / 4));
  return make_float4(h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w);
}

__device__ __forceinline__ void st_split(unsigned char *blk, uint32_t off, float4 q) {
  float4 h, l;
  umma::split_tf32f(q.x, h.x, l.x);
  umma::split_tf32f(q.y, h.y, l.y);
  umma::split_tf32f(q.z, h.z, l.z);
  umma::split_tf32f(q.w, h.w, l.w);
  *(float4 *)(blk + off) = h;
  *(float4 *)(blk + umma::kBlockBytes + off) = l;
}

__global__ void __launch_bounds__(kThreads, 1) vxc_tc_kernel(const VxcArgs A) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float *scoef = (float *)(smem + kStages * kStageBytes);  // [32 points][2 spins][6]
  __shared__ __align__(8) uint64_t afull[kStages], bfull[kStages], empty[kStages], accf, acce, drain;
  __shared__ uint32_t tmem_base;
  __shared__ int s_ok;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_b = A.ldk / 128;
  const int ta = blockIdx.x / tiles_b, tb = blockIdx.x % tiles_b;
  const int64_t r0 = (int64_t)blockIdx.y * A.range;
  const int64_t r1 = r0 + A.range < A.np ? r0 + A.range : A.np;
  const int64_t npcs = r1 > r0 ? (r1 - r0) / 32 : 0;  // point chunks of this slice
  const int64_t nst = npcs * 4;                       // stages
  const int pcs_per_drain = kDrainPts / 32;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      umma::mbar_init(&afull[s], 1);
      umma::mbar_init(&bfull[s], 128);
      umma::mbar_init(&empty[s], 1);
    }
    umma::mbar_init(&accf, 1);
    umma::mbar_init(&acce, 128);
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
        const int64_t pc = r0 / 32 + it / 4;
        const int t = (int)(it % 4);
        umma::mbar_arrive_expect_tx(&afull[s], 2 * umma::kBlockBytes);
        umma::bulk_g2s(smem + s * kStageBytes, am_blk(A, ta, t, pc), 2 * umma::kBlockBytes, &afull[s]);
      }
      __syncwarp();
    }
    for (int64_t i = it > kStages ? it - kStages : 0; i < it; ++i)
      if (!umma::warp_wait(&afull[i % kStages], (i / kStages) & 1) && lane == 0) flag(A.err, 22);
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    const uint32_t idesc = umma::idesc_tf32(128, 128);
    int64_t drains = 0;
    for (int64_t it = 0; it < nst; ++it) {
      const int s = (int)(it % kStages);
      const uint32_t ph = (it / kStages) & 1;
      const int64_t pcl = it / 4;
      const bool window_first = (pcl % pcs_per_drain == 0) && (it % 4 == 0);
      const bool window_last = (((pcl + 1) % pcs_per_drain == 0) || pcl + 1 == npcs) && (it % 4 == 3);
      if (window_first) {
        if (!umma::warp_wait(&acce, (drains & 1) ^ 1)) {
          if (lane == 0) flag(A.err, 23);
          break;
        }
        umma::tc_fence_after();
      }
      if (!umma::warp_wait(&afull[s], ph) || !umma::warp_wait(&bfull[s], ph)) {
        if (lane == 0) flag(A.err, 24);
        break;
      }
      umma::tc_fence_after();
      if (lane == 0) {
        const uint32_t sb = umma::smem_u32(smem + s * kStageBytes);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint64_t ahi = umma::sdesc(sb + kk * 256, umma::kBlockLBO, umma::kBlockSBO);
          const uint64_t alo = umma::sdesc(sb + umma::kBlockBytes + kk * 256, umma::kBlockLBO, umma::kBlockSBO);
#pragma unroll
          for (int sp = 0; sp < 2; ++sp) {
            const uint32_t bb = sb + (2 + 2 * sp) * umma::kBlockBytes + kk * 256;
            const uint64_t bhi = umma::sdesc(bb, umma::kBlockLBO, umma::kBlockSBO);
            const uint64_t blo = umma::sdesc(bb + umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
            const uint32_t d = tbase + sp * 128;
            umma::mma_tf32(d, ahi, bhi, idesc, (window_first && kk == 0) ? 0u : 1u);
            umma::mma_tf32(d, ahi, blo, idesc, 1u);
            umma::mma_tf32(d, alo, bhi, idesc, 1u);
          }
        }
        umma::mma_commit(&empty[s]);
        if (window_last) umma::mma_commit(&accf);
      }
      __syncwarp();
      if (window_last) ++drains;
    }
    if (lane == 0) umma::mma_commit(&drain);
    __syncwarp();
    if (!umma::warp_wait(&drain, 0) && lane == 0) flag(A.err, 25);
  } else {
    // --------------------------------------------- B builders and drainers
    // The four builder warps decide every wait together (one thread polls,
    // a named barrier publishes the result), so they always leave their loop
    // at the same iteration and never strand each other on bar.sync.
    const int bt = threadIdx.x - 64;  // 0..127: row b of the block
    const int q = warp & 3;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16);
    int64_t drains = 0;
    for (int64_t it = 0; it < nst; ++it) {
      const int s = (int)(it % kStages);
      const int64_t pcl = it / 4;
      const int64_t pc = r0 / 32 + pcl;
      const int t = (int)(it % 4);
      builders_sync();  // everyone is done with the previous stage and coefficients
      if (bt == 0) s_ok = umma::mbar_wait(&empty[s], ((it / kStages) & 1) ^ 1) ? 1 : 0;
      if (t == 0) {
        // Coefficients of the chunk's 32 points (FP32), shared by its four stages.
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
      unsigned char *qb = qa + 2 * umma::kBlockBytes;
#pragma unroll 1
      for (int g = 0; g < 8; ++g) {
        const uint32_t off = (uint32_t)(((bt >> 3) * 8 + g) * 128 + (bt & 7) * 16);
        const float *cf = scoef + (4 * g) * 12;
        float4 q0, q1;
        if (t == 0) {
          const float4 ph = ld_pair(am_blk(A, tb, T_PHI, pc), off);
          const float4 dx = ld_pair(am_blk(A, tb, T_DX, pc), off);
          const float4 dy = ld_pair(am_blk(A, tb, T_DY, pc), off);
          const float4 dz = ld_pair(am_blk(A, tb, T_DZ, pc), off);
          const float4 lp = ld_pair(am_blk(A, tb, T_LAP, pc), off);
          const float *c0 = cf, *c1 = cf + 12, *c2 = cf + 24, *c3 = cf + 36;
#define GDFT_Q0(SP, C, F)                                                                                   \
  (C[SP * 6 + C_RHO] * ph.F + C[SP * 6 + C_GX] * dx.F + C[SP * 6 + C_GY] * dy.F + C[SP * 6 + C_GZ] * dz.F + \
   C[SP * 6 + C_LAP] * lp.F)
          q0 = make_float4(GDFT_Q0(0, c0, x), GDFT_Q0(0, c1, y), GDFT_Q0(0, c2, z), GDFT_Q0(0, c3, w));
          q1 = make_float4(GDFT_Q0(1, c0, x), GDFT_Q0(1, c1, y), GDFT_Q0(1, c2, z), GDFT_Q0(1, c3, w));
#undef GDFT_Q0
        } else {
          const float4 dj = ld_pair(am_blk(A, tb, T_PHI + t, pc), off);
          q0 = make_float4(cf[C_KIN] * dj.x, cf[12 + C_KIN] * dj.y, cf[24 + C_KIN] * dj.z, cf[36 + C_KIN] * dj.w);
          q1 = make_float4(cf[6 + C_KIN] * dj.x, cf[18 + C_KIN] * dj.y, cf[30 + C_KIN] * dj.z,
                           cf[42 + C_KIN] * dj.w);
        }
        st_split(qa, off, q0);
        st_split(qb, off, q1);
      }
      umma::fence_proxy_async();
      umma::mbar_arrive(&bfull[s]);
      const bool window_last = (((pcl + 1) % pcs_per_drain == 0) || pcl + 1 == npcs) && (t == 3);
      if (window_last) {
        // Drain the FP32 accumulator of this window into the slice's FP64 sums.
        builders_sync();
        if (bt == 0) s_ok = umma::mbar_wait(&accf, drains & 1) ? 1 : 0;
        builders_sync();
        if (!s_ok) {
          if (bt == 0) flag(A.err, 27);
          break;
        }
        umma::tc_fence_after();
        const int a = ta * 128 + q * 32 + lane;
        double *vp = A.vpart + (size_t)blockIdx.y * 2 * A.n * A.n;
#pragma unroll 1
        for (int sp = 0; sp < 2; ++sp) {
#pragma unroll 1
          for (int c0 = 0; c0 < 128; c0 += 32) {
            float v[32];
            umma::tmem_ld32(tl + sp * 128 + c0, v);
            if (a < A.n) {
              double *row = vp + ((size_t)sp * A.n + a) * A.n;
#pragma unroll
              for (int jj = 0; jj < 32; ++jj) {
                const int b = tb * 128 + c0 + jj;
                if (b < A.n) row[b] = (drains == 0 ? 0.0 : row[b]) + (double)v[jj];
              }
            }
          }
        }
        umma::tc_fence_before();
        umma::mbar_arrive(&acce);
        ++drains;
      }
    }
    // A slice without points still defines its partial sums.
    if (nst == 0) {
      const int a = ta * 128 + q * 32 + lane;
      if (a < A.n) {
        double *vp = A.vpart + (size_t)blockIdx.y * 2 * A.n * A.n;
        for (int sp = 0; sp < 2; ++sp)
          for (int b = tb * 128; b < tb * 128 + 128 && b < A.n; ++b) vp[((size_t)sp * A.n + a) * A.n + b] = 0.0;
      }
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 1) umma::tmem_dealloc(tbase, kTmemCols);
}

}  // namespace

int vxc_tc_splits(int64_t np, int n_ao, int64_t *range) {
  const int tiles = (int)(round_up(n_ao, 128) / 128);
  const int ntiles = tiles * tiles;
  // One wave of 148-152 CTAs where the tile count allows it.
  int want = ntiles >= 148 ? 1 : 148 / ntiles;
  int64_t r = round_up((np + want - 1) / want, kDrainPts);
  if (r < kDrainPts) r = kDrainPts;
  *range = r;
  return (int)((np + r - 1) / r);
}

cudaError_t launch_vxc_tc(const float *am, const double *coef, int64_t np, int ldk, int n_ao, int nsplit,
                          int64_t range, double *vpart, int *err, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(vxc_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  VxcArgs a{am, coef, np, ldk, n_ao, range, vpart, err};
  const int tiles = ldk / 128;
  dim3 grid(tiles * tiles, nsplit);
  vxc_tc_kernel<<<grid, kThreads, kSmemBytes, st>>>(a);
  return cudaGetLastError();
}

}  // namespace gdft
