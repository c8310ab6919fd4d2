// dens_tc.cu - mixed (TF32x3) form of the density contraction on tcgen05.
//
// One CTA owns 128 grid points.  For every AO plane t (phi, d_x, d_y, d_z)
// and every 64-column block cb of the output it forms, for both spins,
//   X_t,sigma[:, cb] = T_t D_sigma[:, cb]          (M = 128, N = 64, K = n_ao)
// in TMEM with three TF32 products per term (hi*hi + hi*lo + lo*hi of the
// split operands, FP32 accumulation; both spins' 64 columns form one N = 128
// operand, so each MMA reads the A tile once for both), then the epilogue
// warps reduce each row
// against the AO planes exactly as the FP64 form (dens_f64.cu) does:
//   t = phi : rho, grad rho (x2), and the phi*lap part of the Laplacian
//   t = d_j : the d_j phi . d_j phi part of the Laplacian and tau.
// Row reductions use FP32 FMA chains of 8 products whose four chains per unit
// and the units of a feature are summed as FP32 pairs (TwoSum; about 2^-44 of
// the terms): GB300 runs FP64 conversions and adds at 1/64 of the FP32 rate.
//
// Accumulation: the tensor cores truncate every MMA's products to the
// accumulator's ulp grid, so long FP32 accumulation chains drift towards
// zero, by an amount proportional to the accumulator's size at each
// instruction.  Each job's K range is therefore split into sub-jobs of one
// 32-wide stage (12 MMAs: the small hi*lo and lo*hi corrections first, the
// hi*hi products last) that accumulate in a TMEM buffer W (double-buffered);
// the epilogue folds W into a running sum S, also in TMEM, with
// round-to-nearest FP32 adds on the CUDA cores.  S is double-buffered too: a
// job's row reductions against the AO planes run, unit by unit, between the
// folds of the next job's stages, so they never hold up the MMA pipeline.
//
// Warp roles (320 threads): warp 0 = TMA producer (one thread issues bulk
// copies of pre-tiled operand images: A 32 KB, the two spins' D halves 4 x 8 KB),
// warp 1 = TMEM owner and MMA issuer (one thread), warps 2-9 = epilogue, one
// per (TMEM lane quadrant = warp % 4, spin).  Three 64 KB smem stages.  Every wait is
// bounded (umma::mbar_wait); on expiry the CTA records an error word, waits
// for its own copies and MMAs to land and releases TMEM.
//
// Two launch forms: dens_tc_kernel, one CTA per 128-point tile of one
// molecule; dens_tc_ragged_kernel, a persistent grid over several molecules'
// tiles taken from a device work queue (launch_dens_tc_ragged: the batch of
// molecules in one launch, largest n_ao first).
#include "common.cuh"
#include "dfloat.cuh"
#include "kernels.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr int kStages = 3;
constexpr uint32_t kHalf = umma::kBlockBytes / 2;                     // 64 rows x 32 fp32
constexpr uint32_t kStageBytes = 2 * umma::kBlockBytes + 4 * kHalf;  // A hi|lo, B hi (both spins), B lo
constexpr int kThreads = 320;
constexpr uint32_t kTmemCols = 512;  // W0 [0,128), W1 [128,256), S0 [256,384), S1 [384,512) (2 spins x 64 columns)
constexpr uint32_t kScol = 256;
constexpr int kSubK = 32;             // K extent of one accumulation chain (one stage)
constexpr int kBN = 64;               // output columns per job
constexpr int kSmemBytes = kStages * kStageBytes + 1024;

struct DensArgs {
  const float *pm;   // point-major resident tables
  const float *dpk;  // packed rdm1
  int64_t np;
  int ldk;
  double *feat;  // [2][6][ldf]: this molecule's points at columns 0 .. np - 1
  int64_t ldf;
  int *err;
};

// Work queue of the ragged form: items are (molecule, 128-point tile) pairs,
// the molecules in the order of `mols` (largest n_ao first), molecule m's
// tiles at items first[m] .. first[m + 1] - 1; CTAs take items by atomicAdd
// on *counter (zero before the launch).
struct DensQueue {
  const DensArgs *mols;
  const int64_t *first;  // n_mol + 1 entries
  int n_mol;
  int64_t n_items;
  int *counter;
  int *err;
};

__device__ __forceinline__ const float *pm_blk(const DensArgs &A, int64_t tile, int plane, int kc) {
  const int nkc = A.ldk / 32;
  return A.pm + ((size_t)(tile * kPlanes + plane) * nkc + kc) * 2 * (umma::kBlockBytes / 4);
}

__device__ __forceinline__ void flag(int *err, int code) { atomicCAS(err, 0, code); }

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
            // B rows 0-63 = spin 0's columns, 64-127 = spin 1's: one N = 128 operand.
            unsigned char *dst = st + 2 * umma::kBlockBytes + sp * kHalf;
            umma::bulk_g2s(dst, b, kHalf, &full[s]);
            umma::bulk_g2s(dst + 2 * kHalf, b + umma::kBlockBytes / 4, kHalf, &full[s]);
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
      const uint32_t idesc = umma::idesc_tf32(128, 2 * kBN);  // both spins in one MMA
      const uint32_t s0 = umma::smem_u32(smem);
      const uint64_t dahi0 = umma::sdesc(s0, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dalo0 = umma::sdesc(s0 + umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dbhi0 = umma::sdesc(s0 + 2 * umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dblo0 = umma::sdesc(s0 + 2 * umma::kBlockBytes + 2 * kHalf, umma::kBlockLBO, umma::kBlockSBO);
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
            const uint32_t d = tbase + buf * 128;
            const uint64_t ahi = dahi0 + so, alo = dalo0 + so, bhi = dbhi0 + so, blo = dblo0 + so;
            // Corrections first (hi*lo, lo*hi, small), then the hi*hi products.
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              umma::mma_tf32(d, ahi + 16 * kk, blo + 16 * kk, idesc, (first && kk == 0) ? 0u : 1u);
              umma::mma_tf32(d, alo + 16 * kk, bhi + 16 * kk, idesc, 1u);
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) umma::mma_tf32(d, ahi + 16 * kk, bhi + 16 * kk, idesc, 1u);
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
    // Job j's stages fold into S[j & 1]; job j - 1's row reductions, split
    // into (plane, 32-column) units, run between those folds and are
    // software-pipelined: a unit's row values are loaded during one stage and
    // consumed in the next, so neither the loads' latency nor the reductions
    // hold up the MMA pipeline.
    const int q = warp & 3;
    const int sp = (warp - 2) >> 2;  // spin handled by this warp
    const int row = q * 32 + lane;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16) + sp * kBN;  // this spin's 64 columns
    df::DF F[6];  // per-feature sums as FP32 pairs
#pragma unroll
    for (int k = 0; k < 6; ++k) F[k] = df::of(0.0f);
    // Row-reduction unit u of job jr: plane k, columns 32 (u % 2) .. + 31 of the job's block.
    auto unit_plane = [&](int jr, int u) { return (jr / ncb == 0 ? 0 : jr / ncb) + (u >> 1); };
    auto unit_blk = [&](int jr, int u) {
      return pm_blk(A, tile, unit_plane(jr, u), ((jr % ncb) * kBN + (u & 1) * 32) / 32);
    };
    auto n_units = [&](int jr) { return jr / ncb == 0 ? 2 * kPlanes : 2; };
    float4 ph[8], pl[8];  // row values of the pending unit (hi, lo), in flight
    auto issue = [&](int jr, int u) {
      const float4 *hi = (const float4 *)unit_blk(jr, u);
      const float4 *lo = hi + umma::kBlockBytes / 16;
#pragma unroll
      for (int g = 0; g < 8; ++g) {
        const int o = (((row >> 3) * 8 + g) * 128 + (row & 7) * 16) / 16;
        ph[g] = __ldg(hi + o);
        pl[g] = __ldg(lo + o);
      }
    };
    auto consume = [&](int jr, int u) {
      float x[32];
      umma::tmem_ld32(tl + kScol + (jr & 1) * 128 + (u & 1) * 32, x);
      float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int g = 0; g < 8; ++g) {
        a[0] = fmaf(x[4 * g + 0], ph[g].x + pl[g].x, a[0]);
        a[1] = fmaf(x[4 * g + 1], ph[g].y + pl[g].y, a[1]);
        a[2] = fmaf(x[4 * g + 2], ph[g].z + pl[g].z, a[2]);
        a[3] = fmaf(x[4 * g + 3], ph[g].w + pl[g].w, a[3]);
      }
      const df::DF d = df::add(df::two_sum(a[0], a[1]), df::two_sum(a[2], a[3]));
      const int k = unit_plane(jr, u);
      switch (jr / ncb == 0 ? k : 5) {
        case 0: F[0] = df::add(F[0], d); break;
        case 1: F[1] = df::add(F[1], d); break;
        case 2: F[2] = df::add(F[2], d); break;
        case 3: F[3] = df::add(F[3], d); break;
        case 4: F[4] = df::add(F[4], d); break;
        default: F[5] = df::add(F[5], d); break;
      }
    };
    int pj = -1, pu = 0;  // pending unit (job, index), issued but not consumed
    uint32_t sub = 0;
    bool ok = true;
    for (int j = 0; j < njobs && ok; ++j) {
      const uint32_t sdst = tl + kScol + (j & 1) * 128;
      const int up = j > 0 ? n_units(j - 1) : 0;
      for (int kq = 0; kq < nkq; ++kq, ++sub) {
        const int buf = sub & 1;
        if (!umma::warp_wait(&wfull[buf], (sub >> 1) & 1)) {
          if (lane == 0) flag(A.err, 16);
          ok = false;
          break;
        }
        umma::tc_fence_after();
        // The unit loaded during the previous stage (its S buffer is about to
        // be reused when it belongs to job j - 2).
        if (pj >= 0) {
          consume(pj, pu);
          pj = -1;
        }
        // S[j & 1] (+)= W for this spin's 64 columns (round-to-nearest FP32 adds).
#pragma unroll
        for (int c = 0; c < kBN; c += 16) {
          uint32_t w[16], sv[16];
          umma::tmem_ld16_nowait(tl + buf * 128 + c, w);
          if (kq > 0) umma::tmem_ld16_nowait(sdst + c, sv);
          umma::tmem_ld_wait(w, sv);
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (kq > 0) w[i] = __float_as_uint(__uint_as_float(w[i]) + __uint_as_float(sv[i]));
          umma::tmem_st16(sdst + c, w);
        }
        umma::tmem_st_wait();
        umma::tc_fence_before();
        umma::mbar_arrive(&wempty[buf]);
        // This stage's share of job j - 1's units: the last one due is left
        // in flight for the next stage, any earlier ones run now.
        const int u0 = kq * up / nkq, u1 = (kq + 1) * up / nkq;
#pragma unroll 1
        for (int u = u0; u < u1; ++u) {
          issue(j - 1, u);
          if (u + 1 < u1) {
            consume(j - 1, u);
          } else {
            pj = j - 1;
            pu = u;
          }
        }
      }
    }
    if (ok) {
      if (pj >= 0) consume(pj, pu);
#pragma unroll 1
      for (int u = 0; u < n_units(njobs - 1); ++u) {
        issue(njobs - 1, u);
        consume(njobs - 1, u);
      }
    }
    const int64_t p = tile * 128 + row;
    double *fs = A.feat + (size_t)sp * kFeat * A.ldf;
    double Fd[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) Fd[k] = (double)F[k].s + (double)F[k].c;
    fs[F_RHO * A.ldf + p] = Fd[T_PHI];
    fs[F_GX * A.ldf + p] = 2.0 * Fd[T_DX];
    fs[F_GY * A.ldf + p] = 2.0 * Fd[T_DY];
    fs[F_GZ * A.ldf + p] = 2.0 * Fd[T_DZ];
    fs[F_LAP * A.ldf + p] = 2.0 * Fd[5] + 2.0 * Fd[T_LAP];
    fs[F_TAU * A.ldf + p] = 0.5 * Fd[5];
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 1) umma::tmem_dealloc(tbase, kTmemCols);
}

// Ragged form of dens_tc_kernel (same roles and arithmetic per tile): a
// persistent grid takes (molecule, tile) items from the queue; the operand
// pipeline, the barriers' phases and TMEM carry over from item to item, and
// the CTA's warps meet at each item boundary.  (The single-molecule case keeps
// dens_tc_kernel, one tile per CTA: this form, run that way, measured 9 %
// slower there.)
__global__ void __launch_bounds__(kThreads, 1) dens_tc_ragged_kernel(const DensQueue Q) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], wfull[2], wempty[2], drain;
  __shared__ uint32_t tmem_base;
  __shared__ int64_t s_item;
  __shared__ int s_mol;
  __shared__ volatile int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int *const err0 = Q.err;

  if (threadIdx.x == 0) {
    s_abort = 0;
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
  uint32_t p_it = 0;              // producer: stages issued
  uint32_t m_it = 0, m_sub = 0;   // MMA issuer: stages consumed, W buffers filled
  uint32_t e_sub = 0;             // epilogue: W buffers folded
  for (;;) {
    __syncthreads();  // every role is done with the previous item
    if (threadIdx.x == 0) {
      int64_t item = INT64_MAX;
      if (!s_abort) {
        item = atomicAdd(Q.counter, 1);
        if (item < Q.n_items) {
          int lo = 0, hi = Q.n_mol;  // first[lo] <= item < first[hi]
          while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (Q.first[mid] <= item) lo = mid; else hi = mid;
          }
          s_mol = lo;
        } else {
          item = INT64_MAX;
        }
      }
      s_item = item;
    }
    __syncthreads();
    if (s_item == INT64_MAX) break;
    const DensArgs A = Q.mols[s_mol];
    const int64_t tile = s_item - Q.first[s_mol];
    const int nkc = A.ldk / 32, ncb = A.ldk / kBN;
    const int njobs = 4 * ncb;
    const int nkq = A.ldk / kSubK, kc_per_sub = kSubK / 32;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    // One thread issues the copies; its waits are bounded and single-threaded.
    if (lane == 0) {
      uint32_t &it = p_it;
      bool ok = true;
      const int ncb128 = A.ldk / 128;
      for (int j = 0; j < njobs && ok; ++j) {
        const int t = j / ncb, cb = j % ncb;
        for (int kc = 0; kc < nkc; ++kc) {
          const int s = it % kStages;
          if (!umma::mbar_wait(&empty[s], ((it / kStages) & 1) ^ 1)) {
            flag(A.err, 11);
            s_abort = 1;
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
            // B rows 0-63 = spin 0's columns, 64-127 = spin 1's: one N = 128 operand.
            unsigned char *dst = st + 2 * umma::kBlockBytes + sp * kHalf;
            umma::bulk_g2s(dst, b, kHalf, &full[s]);
            umma::bulk_g2s(dst + 2 * kHalf, b + umma::kBlockBytes / 4, kHalf, &full[s]);
          }
          ++it;
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    // One thread issues every MMA.  Operand descriptors are built once for
    // slot 0; a slot adds kStageBytes >> 4 and a K step of 8 (256 bytes) adds
    // 16 to the start-address field (address >> 4, bits 0-13).
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_tf32(128, 2 * kBN);  // both spins in one MMA
      const uint32_t s0 = umma::smem_u32(smem);
      const uint64_t dahi0 = umma::sdesc(s0, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dalo0 = umma::sdesc(s0 + umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dbhi0 = umma::sdesc(s0 + 2 * umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dblo0 = umma::sdesc(s0 + 2 * umma::kBlockBytes + 2 * kHalf, umma::kBlockLBO, umma::kBlockSBO);
      uint32_t &it = m_it, &sub = m_sub;
      bool ok = true;
      for (int j = 0; j < njobs && ok; ++j) {
        for (int kq = 0; kq < nkq && ok; ++kq, ++sub) {
          const int buf = sub & 1;
          if (!umma::mbar_wait(&wempty[buf], ((sub >> 1) & 1) ^ 1)) {
            flag(A.err, 13);
            s_abort = 1;
            ok = false;
            break;
          }
          umma::tc_fence_after();
          for (int kc = kq * kc_per_sub; kc < (kq + 1) * kc_per_sub; ++kc) {
            const int s = it % kStages;
            if (!umma::mbar_wait(&full[s], (it / kStages) & 1)) {
              flag(A.err, 14);
              s_abort = 1;
              ok = false;
              break;
            }
            umma::tc_fence_after();
            const uint64_t so = (uint64_t)s * (kStageBytes >> 4);
            const bool first = kc == kq * kc_per_sub;
            const uint32_t d = tbase + buf * 128;
            const uint64_t ahi = dahi0 + so, alo = dalo0 + so, bhi = dbhi0 + so, blo = dblo0 + so;
            // Corrections first (hi*lo, lo*hi, small), then the hi*hi products.
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              umma::mma_tf32(d, ahi + 16 * kk, blo + 16 * kk, idesc, (first && kk == 0) ? 0u : 1u);
              umma::mma_tf32(d, alo + 16 * kk, bhi + 16 * kk, idesc, 1u);
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) umma::mma_tf32(d, ahi + 16 * kk, bhi + 16 * kk, idesc, 1u);
            umma::mma_commit(&empty[s]);
            ++it;
          }
          if (!ok) break;
          umma::mma_commit(&wfull[buf]);
        }
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    // Job j's stages fold into S[j & 1]; job j - 1's row reductions, split
    // into (plane, 32-column) units, run between those folds and are
    // software-pipelined: a unit's row values are loaded during one stage and
    // consumed in the next, so neither the loads' latency nor the reductions
    // hold up the MMA pipeline.
    const int q = warp & 3;
    const int sp = (warp - 2) >> 2;  // spin handled by this warp
    const int row = q * 32 + lane;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16) + sp * kBN;  // this spin's 64 columns
    df::DF F[6];  // per-feature sums as FP32 pairs
#pragma unroll
    for (int k = 0; k < 6; ++k) F[k] = df::of(0.0f);
    // Row-reduction unit u of job jr: plane k, columns 32 (u % 2) .. + 31 of the job's block.
    auto unit_plane = [&](int jr, int u) { return (jr / ncb == 0 ? 0 : jr / ncb) + (u >> 1); };
    auto unit_blk = [&](int jr, int u) {
      return pm_blk(A, tile, unit_plane(jr, u), ((jr % ncb) * kBN + (u & 1) * 32) / 32);
    };
    auto n_units = [&](int jr) { return jr / ncb == 0 ? 2 * kPlanes : 2; };
    float4 ph[8], pl[8];  // row values of the pending unit (hi, lo), in flight
    auto issue = [&](int jr, int u) {
      const float4 *hi = (const float4 *)unit_blk(jr, u);
      const float4 *lo = hi + umma::kBlockBytes / 16;
#pragma unroll
      for (int g = 0; g < 8; ++g) {
        const int o = (((row >> 3) * 8 + g) * 128 + (row & 7) * 16) / 16;
        ph[g] = __ldg(hi + o);
        pl[g] = __ldg(lo + o);
      }
    };
    auto consume = [&](int jr, int u) {
      float x[32];
      umma::tmem_ld32(tl + kScol + (jr & 1) * 128 + (u & 1) * 32, x);
      float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int g = 0; g < 8; ++g) {
        a[0] = fmaf(x[4 * g + 0], ph[g].x + pl[g].x, a[0]);
        a[1] = fmaf(x[4 * g + 1], ph[g].y + pl[g].y, a[1]);
        a[2] = fmaf(x[4 * g + 2], ph[g].z + pl[g].z, a[2]);
        a[3] = fmaf(x[4 * g + 3], ph[g].w + pl[g].w, a[3]);
      }
      const df::DF d = df::add(df::two_sum(a[0], a[1]), df::two_sum(a[2], a[3]));
      const int k = unit_plane(jr, u);
      switch (jr / ncb == 0 ? k : 5) {
        case 0: F[0] = df::add(F[0], d); break;
        case 1: F[1] = df::add(F[1], d); break;
        case 2: F[2] = df::add(F[2], d); break;
        case 3: F[3] = df::add(F[3], d); break;
        case 4: F[4] = df::add(F[4], d); break;
        default: F[5] = df::add(F[5], d); break;
      }
    };
    int pj = -1, pu = 0;  // pending unit (job, index), issued but not consumed
    uint32_t &sub = e_sub;
    bool ok = true;
    for (int j = 0; j < njobs && ok; ++j) {
      const uint32_t sdst = tl + kScol + (j & 1) * 128;
      const int up = j > 0 ? n_units(j - 1) : 0;
      for (int kq = 0; kq < nkq; ++kq, ++sub) {
        const int buf = sub & 1;
        if (!umma::warp_wait(&wfull[buf], (sub >> 1) & 1)) {
          if (lane == 0) {
            flag(A.err, 16);
            s_abort = 1;
          }
          ok = false;
          break;
        }
        umma::tc_fence_after();
        // The unit loaded during the previous stage (its S buffer is about to
        // be reused when it belongs to job j - 2).
        if (pj >= 0) {
          consume(pj, pu);
          pj = -1;
        }
        // S[j & 1] (+)= W for this spin's 64 columns (round-to-nearest FP32 adds).
#pragma unroll
        for (int c = 0; c < kBN; c += 16) {
          uint32_t w[16], sv[16];
          umma::tmem_ld16_nowait(tl + buf * 128 + c, w);
          if (kq > 0) umma::tmem_ld16_nowait(sdst + c, sv);
          umma::tmem_ld_wait(w, sv);
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (kq > 0) w[i] = __float_as_uint(__uint_as_float(w[i]) + __uint_as_float(sv[i]));
          umma::tmem_st16(sdst + c, w);
        }
        umma::tmem_st_wait();
        umma::tc_fence_before();
        umma::mbar_arrive(&wempty[buf]);
        // This stage's share of job j - 1's units: the last one due is left
        // in flight for the next stage, any earlier ones run now.
        const int u0 = kq * up / nkq, u1 = (kq + 1) * up / nkq;
#pragma unroll 1
        for (int u = u0; u < u1; ++u) {
          issue(j - 1, u);
          if (u + 1 < u1) {
            consume(j - 1, u);
          } else {
            pj = j - 1;
            pu = u;
          }
        }
      }
    }
    if (ok) {
      if (pj >= 0) consume(pj, pu);
#pragma unroll 1
      for (int u = 0; u < n_units(njobs - 1); ++u) {
        issue(njobs - 1, u);
        consume(njobs - 1, u);
      }
    }
    if (ok) {
      const int64_t p = tile * 128 + row;
      double *fs = A.feat + (size_t)sp * kFeat * A.ldf;
      double Fd[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) Fd[k] = (double)F[k].s + (double)F[k].c;
      fs[F_RHO * A.ldf + p] = Fd[T_PHI];
      fs[F_GX * A.ldf + p] = 2.0 * Fd[T_DX];
      fs[F_GY * A.ldf + p] = 2.0 * Fd[T_DY];
      fs[F_GZ * A.ldf + p] = 2.0 * Fd[T_DZ];
      fs[F_LAP * A.ldf + p] = 2.0 * Fd[5] + 2.0 * Fd[T_LAP];
      fs[F_TAU * A.ldf + p] = 0.5 * Fd[5];
    }
  }
  }  // items
  if (warp == 0 && lane == 0) {  // our own copies land before the CTA can retire
    for (uint32_t i = p_it > kStages ? p_it - kStages : 0; i < p_it; ++i)
      if (!umma::mbar_wait(&full[i % kStages], (i / kStages) & 1)) flag(err0, 12);
  }
  if (warp == 1 && lane == 0) {  // all issued MMAs complete before TMEM is released
    umma::mma_commit(&drain);
    if (!umma::mbar_wait(&drain, 0)) flag(err0, 15);
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 1) umma::tmem_dealloc(tbase, kTmemCols);
}

constexpr size_t align_up256(size_t b) { return (b + 255) / 256 * 256; }

// Queue table for up to 16 molecules per launch (kernel arguments by value,
// so that the whole setup can be captured in a CUDA graph).
struct DensTableChunk {
  int base, n;  // entries base .. base + n - 1 of first[] (n_mol + 1 in all)
  int n_mol;    // ... and of mols[] below n_mol only
  DensArgs a[16];
  int64_t first[16];
};
__global__ void dens_table_kernel(const DensTableChunk c, DensArgs *mols, int64_t *first) {
  const int i = threadIdx.x;
  if (i < c.n) {
    if (c.base + i < c.n_mol) mols[c.base + i] = c.a[i];
    first[c.base + i] = c.first[i];
  }
}

}  // namespace

size_t dens_ragged_scratch_bytes(int n_mol) {
  return align_up256((size_t)n_mol * sizeof(DensArgs)) + align_up256((size_t)(n_mol + 1) * sizeof(int64_t)) + 256;
}

cudaError_t launch_dens_tc_ragged(const DensMol *mols, int n_mol, void *d_scratch, int *err, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(dens_tc_ragged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (n_mol < 1 || mols == nullptr || d_scratch == nullptr) return cudaErrorInvalidValue;
  // Largest n_ao first: a tile's work grows as ldk^2, so the queue hands out the
  // longest items first.
  int order[1024];
  if (n_mol > 1024) return cudaErrorInvalidValue;
  for (int i = 0; i < n_mol; ++i) order[i] = i;
  for (int i = 1; i < n_mol; ++i)  // stable insertion sort by ldk, descending
    for (int k = i; k > 0 && mols[order[k]].ldk > mols[order[k - 1]].ldk; --k) {
      const int t = order[k];
      order[k] = order[k - 1];
      order[k - 1] = t;
    }
  char *base = (char *)d_scratch;
  DensArgs *d_mols = (DensArgs *)base;
  int64_t *d_first = (int64_t *)(base + align_up256((size_t)n_mol * sizeof(DensArgs)));
  int *d_counter = (int *)((char *)d_first + align_up256((size_t)(n_mol + 1) * sizeof(int64_t)));
  int64_t items = 0;
  for (int c0 = 0; c0 <= n_mol; c0 += 16) {  // n_mol + 1 first[] entries
    DensTableChunk c{};
    c.base = c0;
    c.n = n_mol + 1 - c0 < 16 ? n_mol + 1 - c0 : 16;
    c.n_mol = n_mol;
    for (int i = 0; i < c.n; ++i) {
      const int k = c0 + i;
      c.first[i] = items;
      if (k < n_mol) {
        const DensMol &m = mols[order[k]];
        if (m.np % 128 != 0 || m.ldk % 128 != 0) return cudaErrorInvalidValue;
        c.a[i] = DensArgs{m.pm, m.dpk, m.np, m.ldk, m.feat, m.ldf, err};
        items += m.np / 128;
      }
    }
    dens_table_kernel<<<1, 32, 0, st>>>(c, d_mols, d_first);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  static int n_sm = 0;
  if (n_sm == 0) {
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  const DensQueue q{d_mols, d_first, n_mol, items, d_counter, err};
  dens_tc_ragged_kernel<<<(unsigned)(items < n_sm ? items : n_sm), kThreads, kSmemBytes, st>>>(q);
  return cudaGetLastError();
}

cudaError_t launch_dens_tc(const float *pm, const float *dpk, int64_t np, int ldk, double *feat, int *err,
                           cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(dens_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  DensArgs a{pm, dpk, np, ldk, feat, np, err};
  dens_tc_kernel<<<(unsigned)(np / 128), kThreads, kSmemBytes, st>>>(a);
  return cudaGetLastError();
}

}  // namespace gdft
