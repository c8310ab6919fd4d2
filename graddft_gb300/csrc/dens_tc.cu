// dens_tc.cu - mixed (TF32x3) form of the density contraction on tcgen05.
//
// One CTA owns 128 grid points.  For every AO plane t (phi, d_x, d_y, d_z)
// and every 64-column block cb of the output it forms, for both spins,
//   X_t,sigma[:, cb] = T_t D_sigma[:, cb]          (M = 128, N = 64, K = n_ao)
// in TMEM with three TF32 products per term (hi*hi + hi*lo + lo*hi of the
// split operands, FP32 accumulation), then the epilogue warps reduce each row
// against the AO planes exactly as the FP64 form (dens_f64.cu) does:
//   t = phi : rho, grad rho (x2), and the phi*lap part of the Laplacian
//   t = d_j : the d_j phi . d_j phi part of the Laplacian and tau.
// Row reductions use FP32 FMA chains of 8 products summed in FP64.
//
// Accumulation: the tensor cores truncate every MMA's products to the
// accumulator's ulp grid, so long FP32 accumulation chains drift towards
// zero, by an amount proportional to the accumulator's size at each
// instruction.  Each job's K range is therefore split into sub-jobs of one
// 32-wide stage (12 MMAs per accumulator: the small hi*lo and lo*hi
// corrections first, the hi*hi products last) that accumulate in a TMEM buffer W
// (double-buffered); the epilogue folds W into a running sum S, also in
// TMEM, with round-to-nearest FP32 adds on the CUDA cores, then reduces S
// against the AO planes at the end of the job.
//
// Warp roles (320 threads): warp 0 = TMA producer (one thread issues bulk
// copies of pre-tiled operand images: A 32 KB, the two D halves 4 x 8 KB),
// warp 1 = TMEM owner and MMA issuer (one thread), warps 2-9 = epilogue, one
// per (TMEM lane quadrant = warp % 4, spin).  Three 64 KB smem stages.  Every wait is
// bounded (umma::mbar_wait); on expiry the CTA records an error word, waits
// for its own copies and MMAs to land and releases TMEM.
#include "common.cuh"
#include "kernels.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr int kStages = 3;
constexpr uint32_t kHalf = umma::kBlockBytes / 2;                     // 64 rows x 32 fp32
constexpr uint32_t kStageBytes = 2 * umma::kBlockBytes + 4 * kHalf;  // A hi|lo, B_a hi|lo, B_b hi|lo
constexpr int kThreads = 320;
constexpr uint32_t kTmemCols = 512;  // W0 [0,128), W1 [128,256), S [256,384) (2 spins x 64 columns each)
constexpr int kSubK = 32;             // K extent of one accumulation chain (one stage)
constexpr int kBN = 64;               // output columns per job
constexpr int kSmemBytes = kStages * kStageBytes + 1024;

struct DensArgs {
  const float *pm;   // point-major resident tables
  const float *dpk;  // packed rdm1
  int64_t np;
  int ldk;
  double *feat;  // [2][6][np]
  int *err;
};

__device__ __forceinline__ const float *pm_blk(const DensArgs &A, int64_t tile, int plane, int kc) {
  const int nkc = A.ldk / 32;
  return A.pm + ((size_t)(tile * kPlanes + plane) * nkc + kc) * 2 * (umma::kBlockBytes / 4);
}

__device__ __forceinline__ void flag(int *err, int code) { atomicCAS(err, 0, code); }

// The row's 32 values (hi + lo) of a point-major block.
__device__ __forceinline__ void load_row32(const float *blk, int row, float (&v)[32]) {
  const float4 *hi = (const float4 *)blk;
  const float4 *lo = (const float4 *)(blk + umma::kBlockBytes / 4);
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    const int o = (((row >> 3) * 8 + g) * 128 + (row & 7) * 16) / 16;
    const float4 h = __ldg(hi + o), l = __ldg(lo + o);
    v[4 * g + 0] = h.x + l.x;
    v[4 * g + 1] = h.y + l.y;
    v[4 * g + 2] = h.z + l.z;
    v[4 * g + 3] = h.w + l.w;
  }
}

__global__ void __launch_bounds__(kThreads, 1) dens_tc_kernel(const DensArgs A) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], wfull[2], wempty[2], drain;
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile = blockIdx.x;
  const int nkc = A.ldk / 32, ncb = A.ldk / kBN;
  const int njobs = 4 * ncb;
  const int nkq = A.ldk / kSubK, kc_per_sub = kSubK / 32;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(&wfull[b], 1);
      umma::mbar_init(&wempty[b], 256);
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
    // ------------------------------------------------------------ producer
    // One thread issues the copies; its waits are bounded and single-threaded.
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      const int ncb128 = A.ldk / 128;
      for (int j = 0; j < njobs && ok; ++j) {
        const int t = j / ncb, cb = j % ncb;
        for (int kc = 0; kc < nkc; ++kc) {
          const int s = it % kStages;
          if (!umma::mbar_wait(&empty[s], ((it / kStages) & 1) ^ 1)) {
            flag(A.err, 11);
            ok = false;
            break;
          }
          unsigned char *st = smem + s * kStageBytes;
          umma::mbar_arrive_expect_tx(&full[s], kStageBytes);
          umma::bulk_g2s(st, pm_blk(A, tile, t, kc), 2 * umma::kBlockBytes, &full[s]);
          // D blocks hold 128 columns; this job's 64 are a contiguous half of each.
          for (int sp = 0; sp < 2; ++sp) {
            const float *b = A.dpk + (((size_t)sp * ncb128 + cb / 2) * nkc + kc) * 2 * (umma::kBlockBytes / 4) +
                             (cb & 1) * (kHalf / 4);
            unsigned char *dst = st + 2 * umma::kBlockBytes + sp * 2 * kHalf;
            umma::bulk_g2s(dst, b, kHalf, &full[s]);
            umma::bulk_g2s(dst + kHalf, b + umma::kBlockBytes / 4, kHalf, &full[s]);
          }
          ++it;
        }
      }
      // Wait for the copies still in flight before the CTA can retire.
      for (uint32_t i = it > kStages ? it - kStages : 0; i < it; ++i)
        if (!umma::mbar_wait(&full[i % kStages], (i / kStages) & 1)) flag(A.err, 12);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    // One thread issues every MMA.  Operand descriptors are built once for
    // slot 0; a slot adds kStageBytes >> 4 and a K step of 8 (256 bytes) adds
    // 16 to the start-address field (address >> 4, bits 0-13).
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_tf32(128, kBN);
      const uint32_t s0 = umma::smem_u32(smem);
      const uint64_t dahi0 = umma::sdesc(s0, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dalo0 = umma::sdesc(s0 + umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
      uint64_t dbhi0[2], dblo0[2];
#pragma unroll
      for (int sp = 0; sp < 2; ++sp) {
        const uint32_t bb = s0 + 2 * umma::kBlockBytes + sp * 2 * kHalf;
        dbhi0[sp] = umma::sdesc(bb, umma::kBlockLBO, umma::kBlockSBO);
        dblo0[sp] = umma::sdesc(bb + kHalf, umma::kBlockLBO, umma::kBlockSBO);
      }
      uint32_t it = 0, sub = 0;
      bool ok = true;
      for (int j = 0; j < njobs && ok; ++j) {
        for (int kq = 0; kq < nkq && ok; ++kq, ++sub) {
          const int buf = sub & 1;
          if (!umma::mbar_wait(&wempty[buf], ((sub >> 1) & 1) ^ 1)) {
            flag(A.err, 13);
            ok = false;
            break;
          }
          umma::tc_fence_after();
          for (int kc = kq * kc_per_sub; kc < (kq + 1) * kc_per_sub; ++kc) {
            const int s = it % kStages;
            if (!umma::mbar_wait(&full[s], (it / kStages) & 1)) {
              flag(A.err, 14);
              ok = false;
              break;
            }
            umma::tc_fence_after();
            const uint64_t so = (uint64_t)s * (kStageBytes >> 4);
            const bool first = kc == kq * kc_per_sub;
#pragma unroll
            for (int sp = 0; sp < 2; ++sp) {
              const uint32_t d = tbase + buf * 128 + sp * kBN;
              const uint64_t ahi = dahi0 + so, alo = dalo0 + so, bhi = dbhi0[sp] + so, blo = dblo0[sp] + so;
              // Corrections first (hi*lo, lo*hi, small), then the hi*hi products.
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) {
                umma::mma_tf32(d, ahi + 16 * kk, blo + 16 * kk, idesc, (first && kk == 0) ? 0u : 1u);
                umma::mma_tf32(d, alo + 16 * kk, bhi + 16 * kk, idesc, 1u);
              }
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) umma::mma_tf32(d, ahi + 16 * kk, bhi + 16 * kk, idesc, 1u);
            }
            umma::mma_commit(&empty[s]);
            ++it;
          }
          if (!ok) break;
          umma::mma_commit(&wfull[buf]);
        }
      }
      // All issued MMAs complete before TMEM is released.
      umma::mma_commit(&drain);
      if (!umma::mbar_wait(&drain, 0)) flag(A.err, 15);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;
    const int sp = (warp - 2) >> 2;  // spin handled by this warp
    const int row = q * 32 + lane;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16) + sp * kBN;  // this spin's 64 columns
    double F[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) F[k] = 0.0;
    uint32_t sub = 0;
    bool ok = true;
    for (int j = 0; j < njobs && ok; ++j) {
      const int t = j / ncb, cb = j % ncb;
      for (int kq = 0; kq < nkq; ++kq, ++sub) {
        const int buf = sub & 1;
        if (!umma::warp_wait(&wfull[buf], (sub >> 1) & 1)) {
          if (lane == 0) flag(A.err, 16);
          ok = false;
          break;
        }
        umma::tc_fence_after();
        // S (+)= W for this spin's 64 columns (round-to-nearest FP32 adds).
#pragma unroll
        for (int c = 0; c < kBN; c += 32) {
          uint32_t w[32], sv[32];
          umma::tmem_ld32_nowait(tl + buf * 128 + c, w);
          if (kq > 0) umma::tmem_ld32_nowait(tl + 256 + c, sv);
          umma::tmem_ld_wait(w, sv);
          float o[32];
#pragma unroll
          for (int i = 0; i < 32; ++i)
            o[i] = kq > 0 ? __uint_as_float(w[i]) + __uint_as_float(sv[i]) : __uint_as_float(w[i]);
          umma::tmem_st32(tl + 256 + c, o);
        }
        umma::tmem_st_wait();
        umma::tc_fence_before();
        umma::mbar_arrive(&wempty[buf]);
      }
      if (!ok) break;
      // Row reductions of S: FP32 FMA chains of 8 products, summed in FP64.
      for (int c0 = 0; c0 < kBN; c0 += 32) {
        float x[32], pv[32];
        umma::tmem_ld32(tl + 256 + c0, x);
        const int kc = (cb * kBN + c0) / 32;
        const int k_lo = t == 0 ? 0 : t, k_hi = t == 0 ? kPlanes : t + 1;
#pragma unroll 1
        for (int k = k_lo; k < k_hi; ++k) {
          load_row32(pm_blk(A, tile, k, kc), row, pv);
          float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
          for (int i = 0; i < 32; ++i) a[i & 3] = fmaf(x[i], pv[i], a[i & 3]);
          const double d = ((double)a[0] + (double)a[1]) + ((double)a[2] + (double)a[3]);
          switch (t == 0 ? k : 5) {
            case 0: F[0] += d; break;
            case 1: F[1] += d; break;
            case 2: F[2] += d; break;
            case 3: F[3] += d; break;
            case 4: F[4] += d; break;
            default: F[5] += d; break;
          }
        }
      }
    }
    const int64_t p = tile * 128 + row;
    double *fs = A.feat + (size_t)sp * kFeat * A.np;
    fs[F_RHO * A.np + p] = F[T_PHI];
    fs[F_GX * A.np + p] = 2.0 * F[T_DX];
    fs[F_GY * A.np + p] = 2.0 * F[T_DY];
    fs[F_GZ * A.np + p] = 2.0 * F[T_DZ];
    fs[F_LAP * A.np + p] = 2.0 * F[5] + 2.0 * F[T_LAP];
    fs[F_TAU * A.np + p] = 0.5 * F[5];
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 1) umma::tmem_dealloc(tbase, kTmemCols);
}

}  // namespace

cudaError_t launch_dens_tc(const float *pm, const float *dpk, int64_t np, int ldk, double *feat, int *err,
                           cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(dens_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  DensArgs a{pm, dpk, np, ldk, feat, err};
  dens_tc_kernel<<<(unsigned)(np / 128), kThreads, kSmemBytes, st>>>(a);
  return cudaGetLastError();
}

}  // namespace gdft
