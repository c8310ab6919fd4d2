// tc_gemm.cu - tensor-core GEMMs on pre-packed operand blocks (tcgen05, kind::tf32).
//
//   D[M x N] = sum_K A[M x K] B[N x K]^T      (both operands K-major)
//
// Operands arrive as 16 KB blocks of 128 rows x 32 K in the K-major
// no-swizzle shared-memory layout of umma::kblock_off, so that one stage is
// one bulk copy per operand.  M = 128 and N = 128 per CTA; the K range may be
// split across blockIdx.y, each split writing FP64 partials [split][M][N].
//
// tcg_kernel (TF32x3): blocks [tile][K chunk][hi|lo] of TF32 roundings, three
// products per term (hi*hi + hi*lo + lo*hi).  Each 32-wide K chunk is
// accumulated in one of three TMEM buffers W (the MMA runs up to two chunks
// ahead of the drains), correction products first, and the drains fold it into
// a Kahan-compensated FP32 running sum, the sum S and the compensation C both
// in registers (packed pairs), so a chunk's fold reads W once from TMEM.  A
// single split may write FP32 output instead.
//
// tcg3_kernel (block-scaled, six products): blocks [tile][K chunk][hi|lo|lo2]
// written by umma::store_row3, whose hi slices are quantised per row and K
// chunk so that a chunk's hi*hi sum is exact in FP32.  The tensor core
// truncates its FP32 accumulator toward zero; with plain TF32 slices that bias
// adds up over the chunks of a long contraction (about 2^-23 of the result
// where the chunk sums share a sign).  Here the hi*hi products go to an
// accumulator Y of their own, which stays exact, and the five correction
// products (hi*lo, lo*hi, lo*lo, hi*lo2, lo2*hi, all below 2^-10 of the terms)
// to a second accumulator X.  Two TMEM buffers of (Y, X) take all 512 columns.
// The drains fold Y and X into a running FP32 sum S held in registers (TwoSum
// for Y, Fast2Sum for the small X; packed f32x2 arithmetic, two columns per
// instruction) and store the rounding errors back into the X they just read:
// the MMA accumulates that buffer's next corrections on top of them (X is never
// reset), so the compensation travels in TMEM and the two pending ones are
// added at the end.
//
// Warp roles (320 threads): warp 0 = TMA producer, warp 1 = TMEM owner and
// MMA issuer, warps 2-9 = drains (TMEM lane quadrant warp % 4, column half
// (warp - 2) / 4; each drain thread owns one output row and 64 columns).  All
// waits are bounded; on expiry the CTA records an error word and winds down.
#include "common.cuh"
#include "kernels.cuh"
#include "tc_gemm.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr uint32_t kOpBytes = 2 * umma::kBlockBytes;    // hi | lo of one 128 x 32 block
constexpr uint32_t kStageBytes = 2 * kOpBytes;          // A hi|lo, B hi|lo
constexpr int kStages = 3;
constexpr int kSmemBytes = kStages * kStageBytes + 1024;
constexpr uint32_t kOp3Bytes = 3 * umma::kBlockBytes;   // hi | lo | lo2
constexpr uint32_t kStage3Bytes = 2 * kOp3Bytes;        // A, B
constexpr int kStages3 = 2;
constexpr int kSmem3Bytes = kStages3 * kStage3Bytes + 1024;
constexpr int kThreads = 320;
constexpr int kWBufs = 3;
constexpr uint32_t kTmemCols = 512;  // tcg: W0..W2 [0, 384); tcgw: 2 x 2 W buffers; tcg3: (Y, X) x 2

__device__ __forceinline__ void flag(int *err, int code) { atomicCAS(err, 0, code); }

// Persistent over output tiles: CTA x takes tiles x, x + gridDim.x, ... of its
// K split (blockIdx.y) with one continuous operand pipeline, so barrier and
// TMEM set-up, pipeline fill and the drain of a tile's result overlap the next
// tile's MMAs (the network's activation GEMMs have K = width, a few stages per
// tile).  Tile t is (m = t / n_tiles, n = t % n_tiles): the column tiles of one
// row tile run on neighbouring CTAs at about the same time and read its A
// chunks once from memory, the second time from L2.
__global__ void __launch_bounds__(kThreads, 1) tcg_kernel(const TcgArgs A) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], wfull[kWBufs], wempty[kWBufs], drain;
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = A.m_tiles * A.n_tiles;
  const int64_t c0 = (int64_t)blockIdx.y * A.chunks_per_split;
  const int64_t c1 = c0 + A.chunks_per_split < A.k_chunks ? c0 + A.chunks_per_split : A.k_chunks;
  const int64_t nst = c1 > c0 ? c1 - c0 : 0;  // K stages per tile

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < kWBufs; ++b) {
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
      int64_t it = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int mt = tile / A.n_tiles, nt = tile % A.n_tiles;
        const float *a_tile = A.a + (size_t)mt * A.a_chunks * (kOpBytes / 4);
        const float *b_tile = A.b + (size_t)nt * A.b_chunks * (kOpBytes / 4);
        for (int64_t k = 0; k < nst; ++k, ++it) {
          const int s = (int)(it % kStages);
          if (!umma::mbar_wait(&empty[s], ((it / kStages) & 1) ^ 1)) {
            flag(A.err, 41);
            ok = false;
            break;
          }
          const int64_t kc = c0 + k;
          umma::mbar_arrive_expect_tx(&full[s], kStageBytes);
          umma::bulk_g2s(smem + s * kStageBytes, a_tile + (size_t)kc * (kOpBytes / 4), kOpBytes, &full[s]);
          umma::bulk_g2s(smem + s * kStageBytes + kOpBytes, b_tile + (size_t)kc * (kOpBytes / 4), kOpBytes,
                         &full[s]);
        }
      }
      // Our own copies land before the CTA can release shared memory.
      for (int64_t i = it > kStages ? it - kStages : 0; i < it; ++i)
        if (!umma::mbar_wait(&full[i % kStages], (i / kStages) & 1)) flag(A.err, 42);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    // One thread issues every MMA.  The four operand descriptors are built once
    // for slot 0; a slot (64 KB) adds 4096 and a K step of 8 (256 bytes) adds
    // 16 to the start-address field (address >> 4, bits 0-13; shared memory
    // addresses stay below 2^18).
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_tf32(128, 128);
      const uint32_t sa0 = umma::smem_u32(smem);
      const uint64_t dahi0 = umma::sdesc(sa0, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dalo0 = umma::sdesc(sa0 + umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dbhi0 = umma::sdesc(sa0 + kOpBytes, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dblo0 = umma::sdesc(sa0 + kOpBytes + umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
      int64_t it = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        for (int64_t k = 0; k < nst; ++k, ++it) {
          const int s = (int)(it % kStages);
          const int buf = (int)(it % kWBufs);
          if (!umma::mbar_wait(&wempty[buf], ((it / kWBufs) & 1) ^ 1) ||
              !umma::mbar_wait(&full[s], (it / kStages) & 1)) {
            flag(A.err, 43);
            ok = false;
            break;
          }
          umma::tc_fence_after();
          const uint32_t d = tbase + buf * 128;
          const uint64_t so = (uint64_t)s * (kStageBytes >> 4);  // slot offset in the address field
          const uint64_t ahi = dahi0 + so, alo = dalo0 + so, bhi = dbhi0 + so, blo = dblo0 + so;
          // Products from the smallest up, the hi*hi ones last (the accumulator's
          // truncation is relative to its size at each instruction).
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma::mma_tf32(d, ahi + 16 * kk, blo + 16 * kk, idesc, kk == 0 ? 0u : 1u),
                umma::mma_tf32(d, alo + 16 * kk, bhi + 16 * kk, idesc, 1u);
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) umma::mma_tf32(d, ahi + 16 * kk, bhi + 16 * kk, idesc, 1u);
          umma::mma_commit(&empty[s]);
          umma::mma_commit(&wfull[buf]);
        }
      }
      umma::mma_commit(&drain);
      if (!umma::mbar_wait(&drain, 0)) flag(A.err, 45);
    }
    __syncwarp();
  } else {
    // -------------------------------------------------------------- drains
    // Per tile: every K stage's W is folded into the running sum S with Kahan
    // compensation C, both in registers (one TMEM read of W per stage); after
    // the tile's last stage S - C is written out and the next tile starts over.
    const int q = warp & 3, half = (warp - 2) >> 2;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16) + half * 64;
    int64_t it = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const int mt = tile / A.n_tiles, nt = tile % A.n_tiles;
      // Compensations of this thread's 64 columns as 32 packed FP32 pairs: the
      // fold runs on add/sub.rn.f32x2, two columns per instruction, each
      // rounded exactly like the scalar operation.
      uint64_t S2[32], C2[32];  // running sums and compensations, column pairs, in registers
#pragma unroll
      for (int i = 0; i < 32; ++i) C2[i] = 0ull;
      int64_t k = 0;
      for (; k < nst; ++k, ++it) {
        const int buf = (int)(it % kWBufs);
        if (!umma::warp_wait(&wfull[buf], (it / kWBufs) & 1)) {
          if (lane == 0) flag(A.err, 46);
          ok = false;
          break;
        }
        umma::tc_fence_after();
#pragma unroll
        for (int c = 0; c < 64; c += 16) {
          uint32_t wr[16];
          umma::tmem_ld16_nowait(tl + buf * 128 + c, wr);
          umma::tmem_ld_wait(wr);
#pragma unroll
          for (int i = 0; i < 16; i += 2) {
            const uint64_t w2 = umma::pk2(wr[i], wr[i + 1]);
            if (k > 0) {  // Kahan: S + (w - C)
              const uint64_t sp = S2[(c + i) / 2];
              const uint64_t y = umma::sub2(w2, C2[(c + i) / 2]);
              const uint64_t t = umma::add2(sp, y);
              C2[(c + i) / 2] = umma::sub2(umma::sub2(t, sp), y);
              S2[(c + i) / 2] = t;
            } else {
              S2[(c + i) / 2] = w2;
            }
          }
        }
        umma::tc_fence_before();
        umma::mbar_arrive(&wempty[buf]);
      }
      const bool have = ok && k == nst && nst > 0;
      const int m = mt * 128 + q * 32 + lane;
      const int n0 = nt * 128 + half * 64;
      // Output S - C, one column pair at a time from the packed registers.
      auto pair = [&](int i, float &x, float &y) {
        uint32_t s0, s1, c0, c1;
        umma::unpk2(S2[i], s0, s1);
        umma::unpk2(C2[i], c0, c1);
        x = __uint_as_float(s0) - __uint_as_float(c0);
        y = __uint_as_float(s1) - __uint_as_float(c1);
      };
      auto pair64 = [&](int i, double &x, double &y) {
        uint32_t s0, s1, c0, c1;
        umma::unpk2(S2[i], s0, s1);
        umma::unpk2(C2[i], c0, c1);
        x = (double)__uint_as_float(s0) - (double)__uint_as_float(c0);
        y = (double)__uint_as_float(s1) - (double)__uint_as_float(c1);
      };
      if (m < A.m_valid) {
        // Each lane owns one output row: whole 16-byte pieces where the row
        // segment is in range and aligned (a lane's 64 values are 256 bytes).
        if (A.out32) {
          float *row = A.out32 + (size_t)m * A.ldo + n0;
          if (n0 + 64 <= A.n_valid && (A.ldo & 3) == 0) {
#pragma unroll
            for (int i = 0; i < 64; i += 4) {
              float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
              if (have) {
                pair(i / 2, v.x, v.y);
                pair(i / 2 + 1, v.z, v.w);
              }
              *reinterpret_cast<float4 *>(row + i) = v;
            }
          } else {
#pragma unroll
            for (int i = 0; i < 64; i += 2) {
              float x = 0.0f, y = 0.0f;
              if (have) pair(i / 2, x, y);
              if (n0 + i < A.n_valid) row[i] = x;
              if (n0 + i + 1 < A.n_valid) row[i + 1] = y;
            }
          }
        } else {
          double *row = A.out64 + ((size_t)blockIdx.y * A.m_valid + m) * A.n_valid + n0;
          if (n0 + 64 <= A.n_valid && (A.n_valid & 1) == 0) {
#pragma unroll
            for (int i = 0; i < 64; i += 2) {
              double x = 0.0, y = 0.0;
              if (have) pair64(i / 2, x, y);
              *reinterpret_cast<double2 *>(row + i) = make_double2(x, y);
            }
          } else {
#pragma unroll
            for (int i = 0; i < 64; i += 2) {
              double x = 0.0, y = 0.0;
              if (have) pair64(i / 2, x, y);
              if (n0 + i < A.n_valid) row[i] = x;
              if (n0 + i + 1 < A.n_valid) row[i + 1] = y;
            }
          }
        }
      }
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 1) umma::tmem_dealloc(tbase, kTmemCols);
}

// ------------------------------------------------------------- tcgw_kernel
// Single-split FP32-output form for an even number of column tiles (the
// network's activation GEMMs, K = width): a CTA owns a 128 x 256 output tile
// (column tiles 2p, 2p + 1), so each stage copies the A chunk once for both
// halves (A hi|lo + two B hi|lo = 96 KB, two stages) and issues 24 MMAs.
// TMEM holds two W buffers per half (all 512 columns); the running sum of each
// drain thread's 128 columns stays in registers and takes each stage's W with
// a round-to-nearest FP32 add (unbiased; at K = width the few folds keep it
// within the FP32 rounding of the stored activations, while the tensor core's
// truncating accumulation still never spans more than one 32-wide K chunk).
// Drain warps 2-5 take half 0, warps 6-9 half 1 (TMEM lane quadrant warp % 4).
constexpr int kStagesW = 2;
constexpr uint32_t kStageWBytes = 3 * kOpBytes;  // A, B half 0, B half 1 (hi|lo each)
constexpr int kSmemWBytes = kStagesW * kStageWBytes + 1024;

__global__ void __launch_bounds__(kThreads, 1) tcgw_kernel(const TcgArgs A) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStagesW], empty[kStagesW], wfull[2][2], wempty[2][2], drain;
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int npairs = A.n_tiles / 2;
  const int ntiles = A.m_tiles * npairs;
  const int64_t nst = A.k_chunks;  // K stages per tile

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStagesW; ++s) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    for (int h = 0; h < 2; ++h)
      for (int b = 0; b < 2; ++b) {
        umma::mbar_init(&wfull[h][b], 1);
        umma::mbar_init(&wempty[h][b], 128);
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
    if (lane == 0) {
      int64_t it = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int mt = tile / npairs, np2 = tile % npairs;
        const float *a_tile = A.a + (size_t)mt * A.a_chunks * (kOpBytes / 4);
        const float *b_tile = A.b + (size_t)(2 * np2) * A.b_chunks * (kOpBytes / 4);
        for (int64_t k = 0; k < nst; ++k, ++it) {
          const int s = (int)(it % kStagesW);
          if (!umma::mbar_wait(&empty[s], ((it / kStagesW) & 1) ^ 1)) {
            flag(A.err, 51);
            ok = false;
            break;
          }
          unsigned char *slot = smem + s * kStageWBytes;
          umma::mbar_arrive_expect_tx(&full[s], kStageWBytes);
          umma::bulk_g2s(slot, a_tile + (size_t)k * (kOpBytes / 4), kOpBytes, &full[s]);
          umma::bulk_g2s(slot + kOpBytes, b_tile + (size_t)k * (kOpBytes / 4), kOpBytes, &full[s]);
          umma::bulk_g2s(slot + 2 * kOpBytes, b_tile + (size_t)(A.b_chunks + k) * (kOpBytes / 4), kOpBytes,
                         &full[s]);
        }
      }
      for (int64_t i = it > kStagesW ? it - kStagesW : 0; i < it; ++i)
        if (!umma::mbar_wait(&full[i % kStagesW], (i / kStagesW) & 1)) flag(A.err, 52);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_tf32(128, 128);
      const uint32_t sa0 = umma::smem_u32(smem);
      const uint64_t dahi0 = umma::sdesc(sa0, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t dalo0 = umma::sdesc(sa0 + umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
      int64_t it = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        for (int64_t k = 0; k < nst; ++k, ++it) {
          const int s = (int)(it % kStagesW), buf = (int)(it & 1);
          if (!umma::mbar_wait(&full[s], (it / kStagesW) & 1)) {
            flag(A.err, 53);
            ok = false;
            break;
          }
          const uint64_t so = (uint64_t)s * (kStageWBytes >> 4);  // slot offset in the address field
          const uint64_t ahi = dahi0 + so, alo = dalo0 + so;
          for (int h = 0; h < 2 && ok; ++h) {
            if (!umma::mbar_wait(&wempty[h][buf], ((it >> 1) & 1) ^ 1)) {
              flag(A.err, 54);
              ok = false;
              break;
            }
            umma::tc_fence_after();
            const uint32_t sb = sa0 + s * kStageWBytes + (1 + h) * kOpBytes;
            const uint64_t bhi = umma::sdesc(sb, umma::kBlockLBO, umma::kBlockSBO);
            const uint64_t blo = umma::sdesc(sb + umma::kBlockBytes, umma::kBlockLBO, umma::kBlockSBO);
            const uint32_t d = tbase + (2 * h + buf) * 128;
            // Products from the smallest up, the hi*hi ones last.
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              umma::mma_tf32(d, ahi + 16 * kk, blo + 16 * kk, idesc, kk == 0 ? 0u : 1u),
                  umma::mma_tf32(d, alo + 16 * kk, bhi + 16 * kk, idesc, 1u);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) umma::mma_tf32(d, ahi + 16 * kk, bhi + 16 * kk, idesc, 1u);
            umma::mma_commit(&wfull[h][buf]);
          }
          umma::mma_commit(&empty[s]);
        }
      }
      umma::mma_commit(&drain);
      if (!umma::mbar_wait(&drain, 0)) flag(A.err, 55);
    }
    __syncwarp();
  } else {
    // -------------------------------------------------------------- drains
    const int q = warp & 3, h = (warp - 2) >> 2;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16) + 2 * h * 128;
    int64_t it = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const int mt = tile / npairs, np2 = tile % npairs;
      float S[128];
      int64_t k = 0;
      for (; k < nst; ++k, ++it) {
        const int buf = (int)(it & 1);
        if (!umma::warp_wait(&wfull[h][buf], (it >> 1) & 1)) {
          if (lane == 0) flag(A.err, 56);
          ok = false;
          break;
        }
        umma::tc_fence_after();
#pragma unroll
        for (int c = 0; c < 128; c += 16) {
          uint32_t wr[16];
          umma::tmem_ld16_nowait(tl + buf * 128 + c, wr);
          umma::tmem_ld_wait(wr);
#pragma unroll
          for (int i = 0; i < 16; ++i) S[c + i] = k == 0 ? __uint_as_float(wr[i]) : S[c + i] + __uint_as_float(wr[i]);
        }
        umma::tc_fence_before();
        umma::mbar_arrive(&wempty[h][buf]);
      }
      if (!ok || k != nst) break;
      const int m = mt * 128 + q * 32 + lane;
      const int n0 = (2 * np2 + h) * 128;
      if (m < A.m_valid) {
        float *row = A.out32 + (size_t)m * A.ldo + n0;
        if (n0 + 128 <= A.n_valid && (A.ldo & 3) == 0) {
#pragma unroll
          for (int i = 0; i < 128; i += 4)
            *reinterpret_cast<float4 *>(row + i) = make_float4(S[i], S[i + 1], S[i + 2], S[i + 3]);
        } else {
#pragma unroll
          for (int i = 0; i < 128; ++i)
            if (n0 + i < A.n_valid) row[i] = S[i];
        }
      }
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 1) umma::tmem_dealloc(tbase, kTmemCols);
}

__global__ void __launch_bounds__(kThreads, 1) tcg3_kernel(const TcgArgs A) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStages3], empty[kStages3], wfull[2], wempty[2], drain;
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x % A.m_tiles, nt = blockIdx.x / A.m_tiles;
  const int64_t c0 = (int64_t)blockIdx.y * A.chunks_per_split;
  const int64_t c1 = c0 + A.chunks_per_split < A.k_chunks ? c0 + A.chunks_per_split : A.k_chunks;
  const int64_t nst = c1 > c0 ? c1 - c0 : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages3; ++s) {
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
  if (warp >= 2) {  // both X accumulators start at zero (the MMA only ever accumulates into them)
    const uint32_t tl = tbase + ((uint32_t)((warp & 3) * 32) << 16) + ((warp - 2) >> 2) * 64;
    uint32_t z[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) z[i] = 0u;
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 64; c += 16) umma::tmem_st16(tl + b * 256 + 128 + c, z);
    umma::tmem_st_wait();
  }
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const float *a_tile = A.a + (size_t)mt * A.a_chunks * (kOp3Bytes / 4);
  const float *b_tile = A.b + (size_t)nt * A.b_chunks * (kOp3Bytes / 4);

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      int64_t it = 0;
      for (; it < nst; ++it) {
        const int s = (int)(it % kStages3);
        if (!umma::mbar_wait(&empty[s], ((it / kStages3) & 1) ^ 1)) {
          flag(A.err, 51);
          break;
        }
        const int64_t kc = c0 + it;
        umma::mbar_arrive_expect_tx(&full[s], kStage3Bytes);
        umma::bulk_g2s(smem + s * kStage3Bytes, a_tile + (size_t)kc * (kOp3Bytes / 4), kOp3Bytes, &full[s]);
        umma::bulk_g2s(smem + s * kStage3Bytes + kOp3Bytes, b_tile + (size_t)kc * (kOp3Bytes / 4), kOp3Bytes,
                       &full[s]);
      }
      for (int64_t i = it > kStages3 ? it - kStages3 : 0; i < it; ++i)
        if (!umma::mbar_wait(&full[i % kStages3], (i / kStages3) & 1)) flag(A.err, 52);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    // Descriptors of slot 0's hi blocks; lo and lo2 add one and two blocks
    // (1024 and 2048 in the address field), a slot (96 KB) adds 6144, a K step
    // of 8 adds 16.
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_tf32(128, 128);
      const uint32_t sa0 = umma::smem_u32(smem);
      constexpr uint64_t kBlk = umma::kBlockBytes >> 4;
      const uint64_t da0 = umma::sdesc(sa0, umma::kBlockLBO, umma::kBlockSBO);
      const uint64_t db0 = umma::sdesc(sa0 + kOp3Bytes, umma::kBlockLBO, umma::kBlockSBO);
      for (int64_t it = 0; it < nst; ++it) {
        const int s = (int)(it % kStages3);
        const int buf = (int)(it & 1);
        if (!umma::mbar_wait(&wempty[buf], ((it >> 1) & 1) ^ 1) ||
            !umma::mbar_wait(&full[s], (it / kStages3) & 1)) {
          flag(A.err, 53);
          break;
        }
        umma::tc_fence_after();
        const uint32_t y = tbase + buf * 256, x = y + 128;
        const uint64_t so = (uint64_t)s * (kStage3Bytes >> 4);
        const uint64_t ahi = da0 + so, alo = ahi + kBlk, alo2 = ahi + 2 * kBlk;
        const uint64_t bhi = db0 + so, blo = bhi + kBlk, blo2 = bhi + 2 * kBlk;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          umma::mma_tf32(x, alo + 16 * kk, blo + 16 * kk, idesc, 1u),
              umma::mma_tf32(x, ahi + 16 * kk, blo2 + 16 * kk, idesc, 1u),
              umma::mma_tf32(x, alo2 + 16 * kk, bhi + 16 * kk, idesc, 1u);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          umma::mma_tf32(x, ahi + 16 * kk, blo + 16 * kk, idesc, 1u),
              umma::mma_tf32(x, alo + 16 * kk, bhi + 16 * kk, idesc, 1u);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) umma::mma_tf32(y, ahi + 16 * kk, bhi + 16 * kk, idesc, kk == 0 ? 0u : 1u);
        umma::mma_commit(&empty[s]);
        umma::mma_commit(&wfull[buf]);
      }
      umma::mma_commit(&drain);
      if (!umma::mbar_wait(&drain, 0)) flag(A.err, 55);
    }
    __syncwarp();
  } else {
    // -------------------------------------------------------------- drains
    const int q = warp & 3, half = (warp - 2) >> 2;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16) + half * 64;
    uint64_t S[32];  // column pairs (2i, 2i + 1), packed FP32
#pragma unroll
    for (int i = 0; i < 32; ++i) S[i] = 0ull;
    int64_t it = 0;
    for (; it < nst; ++it) {
      const int buf = (int)(it & 1);
      if (!umma::warp_wait(&wfull[buf], (it >> 1) & 1)) {
        if (lane == 0) flag(A.err, 56);
        break;
      }
      umma::tc_fence_after();
#pragma unroll
      for (int c = 0; c < 64; c += 16) {
        uint32_t yr[16], xr[16];
        umma::tmem_ld16_nowait(tl + buf * 256 + c, yr);
        umma::tmem_ld16_nowait(tl + buf * 256 + 128 + c, xr);
        umma::tmem_ld_wait(yr, xr);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          // S + Y = t + e1 exactly (TwoSum); t + X = u + e2 (Fast2Sum: X is
          // below 2^-10 of the chunk's terms, t holds the sum so far).  Two
          // columns per instruction.
          using namespace umma;
          const uint64_t yv = pk2(yr[2 * i], yr[2 * i + 1]), xv = pk2(xr[2 * i], xr[2 * i + 1]);
          const uint64_t sv = S[c / 2 + i];
          const uint64_t t = add2(sv, yv);
          const uint64_t bp = sub2(t, sv);
          const uint64_t e1 = add2(sub2(sv, sub2(t, bp)), sub2(yv, bp));
          const uint64_t u = add2(t, xv);
          const uint64_t e2 = sub2(xv, sub2(u, t));
          S[c / 2 + i] = u;
          unpk2(add2(e1, e2), xr[2 * i], xr[2 * i + 1]);
        }
        umma::tmem_st16(tl + buf * 256 + 128 + c, xr);
      }
      umma::tmem_st_wait();
      umma::tc_fence_before();
      umma::mbar_arrive(&wempty[buf]);
    }
    const bool have = it == nst;
    const int m = mt * 128 + q * 32 + lane;
    const int n0 = nt * 128 + half * 64;
    double *row = A.out64 + ((size_t)blockIdx.y * A.m_valid + (m < A.m_valid ? m : 0)) * A.n_valid + n0;
#pragma unroll
    for (int c = 0; c < 64; c += 16) {  // S plus the two compensations still pending in X
      uint32_t e0[16], e1[16];
      umma::tmem_ld16_nowait(tl + 128 + c, e0);
      umma::tmem_ld16_nowait(tl + 256 + 128 + c, e1);
      umma::tmem_ld_wait(e0, e1);
      if (m < A.m_valid) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          uint32_t sp[2];
          umma::unpk2(S[(c + i) / 2], sp[0], sp[1]);
          if (n0 + c + i < A.n_valid)
            row[c + i] = have ? ((double)__uint_as_float(sp[i & 1]) + (double)__uint_as_float(e0[i])) +
                                    (double)__uint_as_float(e1[i])
                              : 0.0;
        }
      }
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 1) umma::tmem_dealloc(tbase, kTmemCols);
}

}  // namespace

cudaError_t launch_tcg(const TcgArgs &a, int nsplit, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tcg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (a.m_tiles <= 0 || a.n_tiles <= 0 || nsplit <= 0 || (a.out32 == nullptr) == (a.out64 == nullptr) ||
      (a.out32 && nsplit != 1) || a.k_chunks > a.a_chunks || a.k_chunks > a.b_chunks)
    return cudaErrorInvalidValue;
  // One CTA per SM in all (each holds all 512 TMEM columns); the tiles of a split are shared out.
  static int n_sm = 0;
  if (n_sm == 0) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  if (a.out32 && a.n_tiles % 2 == 0 && a.k_chunks > 0) {  // 128 x 256 output tiles, sums in registers
    static bool attr_w = false;
    if (!attr_w) {
      cudaError_t e = cudaFuncSetAttribute(tcgw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemWBytes);
      if (e != cudaSuccess) return e;
      attr_w = true;
    }
    const int wtiles = a.m_tiles * (a.n_tiles / 2);
    tcgw_kernel<<<wtiles < n_sm ? wtiles : n_sm, kThreads, kSmemWBytes, st>>>(a);
    return cudaGetLastError();
  }
  const int tiles = a.m_tiles * a.n_tiles;
  int gx = n_sm / nsplit;
  gx = gx < 1 ? 1 : (gx > tiles ? tiles : gx);
  dim3 grid(gx, nsplit);
  tcg_kernel<<<grid, kThreads, kSmemBytes, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_tcg3(const TcgArgs &a, int nsplit, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tcg3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem3Bytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (a.m_tiles <= 0 || a.n_tiles <= 0 || nsplit <= 0 || a.out64 == nullptr || a.out32 != nullptr ||
      a.k_chunks > a.a_chunks || a.k_chunks > a.b_chunks)
    return cudaErrorInvalidValue;
  dim3 grid(a.m_tiles * a.n_tiles, nsplit);
  tcg3_kernel<<<grid, kThreads, kSmem3Bytes, st>>>(a);
  return cudaGetLastError();
}

}  // namespace gdft

namespace gdft {

namespace {

// TF32 hi/lo split: FP64 sources through FP64 (22 of their 53 bits kept),
// FP32 sources in FP32 arithmetic (exact: x - hi is representable).
__device__ __forceinline__ void split4(const double (&v)[4], float4 &h, float4 &l) {
  umma::split_tf32(v[0], h.x, l.x);
  umma::split_tf32(v[1], h.y, l.y);
  umma::split_tf32(v[2], h.z, l.z);
  umma::split_tf32(v[3], h.w, l.w);
}
__device__ __forceinline__ void split4(const float (&v)[4], float4 &h, float4 &l) {
  umma::split_tf32f(v[0], h.x, l.x);
  umma::split_tf32f(v[1], h.y, l.y);
  umma::split_tf32f(v[2], h.z, l.z);
  umma::split_tf32f(v[3], h.w, l.w);
}

// One CTA per block pair; 256 threads, each 4 (row, 4-wide k group) items.
template <class T>
__global__ void pack_rt_kernel(const T *__restrict__ X, int64_t rows, int cols, int ld, int kchunks,
                               float *__restrict__ out) {
  const int64_t t = blockIdx.x / kchunks;
  const int kc = blockIdx.x % kchunks;
  float *blk = out + (size_t)blockIdx.x * 2 * (umma::kBlockBytes / 4);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int item = threadIdx.x + i * 256;  // 0..1023
    const int row = item >> 3, k4 = item & 7;
    const int64_t r = t * 128 + row;
    T v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = kc * 32 + k4 * 4 + j;
      v[j] = (r < rows && c < cols) ? X[(size_t)r * ld + c] : (T)0;
    }
    float4 h, l;
    split4(v, h, l);
    const uint32_t off = umma::kblock_off(row, k4 * 4) / 4;
    *(float4 *)(blk + off) = h;
    *(float4 *)(blk + umma::kBlockBytes / 4 + off) = l;
  }
}

template <class T>
__global__ void pack_ct_kernel(const T *__restrict__ X, int64_t rows, int cols, int ld, int64_t rchunks,
                               float *__restrict__ out) {
  const int ft = (int)(blockIdx.x / rchunks);
  const int64_t rc = blockIdx.x % rchunks;
  float *blk = out + (size_t)blockIdx.x * 2 * (umma::kBlockBytes / 4);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int item = threadIdx.x + i * 256;
    const int m = item & 127, k4 = item >> 7;  // consecutive threads: consecutive columns of X
    const int c = ft * 128 + m;
    T v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t r = rc * 32 + k4 * 4 + j;
      v[j] = (r < rows && c < cols) ? X[(size_t)r * ld + c] : (T)0;
    }
    float4 h, l;
    split4(v, h, l);
    const uint32_t off = umma::kblock_off(m, k4 * 4) / 4;
    *(float4 *)(blk + off) = h;
    *(float4 *)(blk + umma::kBlockBytes / 4 + off) = l;
  }
}

// One CTA of 128 threads per block set, one row per thread.
__global__ void __launch_bounds__(128) pack_rt3_kernel(const double *__restrict__ X, int64_t rows, int cols, int ld,
                                                       int kchunks, float *__restrict__ out) {
  const int64_t t = blockIdx.x / kchunks;
  const int kc = blockIdx.x % kchunks;
  const int row = threadIdx.x;
  const int64_t r = t * 128 + row;
  double v[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const int c = kc * 32 + k;
    v[k] = (r < rows && c < cols) ? X[(size_t)r * ld + c] : 0.0;
  }
  umma::store_row3(out + (size_t)blockIdx.x * 3 * (umma::kBlockBytes / 4), row, v);
}

}  // namespace

cudaError_t launch_pack_rt3(const double *X, int64_t rows, int cols, int ld, int64_t tiles, int kchunks, float *out,
                            cudaStream_t st) {
  if (tiles <= 0 || kchunks <= 0) return cudaErrorInvalidValue;
  pack_rt3_kernel<<<(unsigned)(tiles * kchunks), 128, 0, st>>>(X, rows, cols, ld, kchunks, out);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_pack_rt(const T *X, int64_t rows, int cols, int ld, int64_t tiles, int kchunks, float *out,
                           cudaStream_t st) {
  if (tiles <= 0 || kchunks <= 0) return cudaErrorInvalidValue;
  pack_rt_kernel<T><<<(unsigned)(tiles * kchunks), 256, 0, st>>>(X, rows, cols, ld, kchunks, out);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_pack_ct(const T *X, int64_t rows, int cols, int ld, int ftiles, int64_t rchunks, float *out,
                           cudaStream_t st) {
  if (ftiles <= 0 || rchunks <= 0) return cudaErrorInvalidValue;
  pack_ct_kernel<T><<<(unsigned)(ftiles * rchunks), 256, 0, st>>>(X, rows, cols, ld, rchunks, out);
  return cudaGetLastError();
}

template cudaError_t launch_pack_rt<float>(const float *, int64_t, int, int, int64_t, int, float *, cudaStream_t);
template cudaError_t launch_pack_rt<double>(const double *, int64_t, int, int, int64_t, int, float *, cudaStream_t);
template cudaError_t launch_pack_ct<float>(const float *, int64_t, int, int, int, int64_t, float *, cudaStream_t);
template cudaError_t launch_pack_ct<double>(const double *, int64_t, int, int, int, int64_t, float *, cudaStream_t);

}  // namespace gdft

// Host-array probes of the packed GEMMs (synchronous; they allocate their own
// buffers): D (M x N, FP64) = A (M x K) B (N x K)^T through a row-tile packer
// and the kernel; FP32 output for a single split of the TF32x3 form, FP64
// split-K partials summed on the host otherwise.
static int tc_gemm_probe(bool three, int32_t M, int32_t N, int32_t K, int32_t nsplit, const double *h_a,
                         const double *h_b, double *h_d) {
  using namespace gdft;
  const char *name = three ? "gdft_tc_gemm3_probe" : "gdft_tc_gemm_probe";
  if (M <= 0 || N <= 0 || K <= 0 || nsplit <= 0 || !h_a || !h_b || !h_d || M > 4096 || N > 4096 ||
      K > (1 << 20)) {
    set_error("%s: invalid arguments", name);
    return GDFT_ERR_INVALID;
  }
  const int mt = (M + 127) / 128, ntl = (N + 127) / 128;
  const int64_t kch = (K + 31) / 32;
  const size_t blk = (three ? 3 : 2) * (umma::kBlockBytes / 4);
  const bool f32out = !three && nsplit == 1;
  double *dA = nullptr, *dB = nullptr, *d64 = nullptr;
  float *pA = nullptr, *pB = nullptr, *d32 = nullptr;
  int *err = nullptr;
  int rc = GDFT_OK;
  auto ck = [&](cudaError_t e, const char *w) {
    if (rc == GDFT_OK) rc = check_cuda(e, w);
    return rc == GDFT_OK;
  };
  const int64_t cps = (kch + nsplit - 1) / nsplit;
  if (ck(cudaMalloc(&dA, (size_t)M * K * 8), "probe alloc") && ck(cudaMalloc(&dB, (size_t)N * K * 8), "probe alloc") &&
      ck(cudaMalloc(&pA, (size_t)mt * kch * blk * 4), "probe alloc") &&
      ck(cudaMalloc(&pB, (size_t)ntl * kch * blk * 4), "probe alloc") &&
      ck(cudaMalloc(&d32, (size_t)M * N * 4), "probe alloc") &&
      ck(cudaMalloc(&d64, (size_t)nsplit * M * N * 8), "probe alloc") && ck(cudaMalloc(&err, 4), "probe alloc") &&
      ck(cudaMemset(err, 0, 4), "probe memset") &&
      ck(cudaMemcpy(dA, h_a, (size_t)M * K * 8, cudaMemcpyHostToDevice), "probe copy") &&
      ck(cudaMemcpy(dB, h_b, (size_t)N * K * 8, cudaMemcpyHostToDevice), "probe copy") &&
      ck(three ? launch_pack_rt3(dA, M, K, K, mt, (int)kch, pA, 0) : launch_pack_rt<double>(dA, M, K, K, mt, (int)kch, pA, 0),
         "probe pack A") &&
      ck(three ? launch_pack_rt3(dB, N, K, K, ntl, (int)kch, pB, 0) : launch_pack_rt<double>(dB, N, K, K, ntl, (int)kch, pB, 0),
         "probe pack B")) {
    TcgArgs a{};
    a.a = pA;
    a.b = pB;
    a.m_tiles = mt;
    a.n_tiles = ntl;
    a.a_chunks = a.b_chunks = a.k_chunks = kch;
    a.chunks_per_split = nsplit == 1 ? kch : cps;
    a.out32 = f32out ? d32 : nullptr;
    a.ldo = N;
    a.out64 = f32out ? nullptr : d64;
    a.m_valid = M;
    a.n_valid = N;
    a.err = err;
    if (ck(three ? launch_tcg3(a, nsplit, 0) : launch_tcg(a, nsplit, 0), "probe tcg") &&
        ck(cudaDeviceSynchronize(), "probe sync")) {
      int herr = 0;
      if (ck(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost), "probe err")) {
        if (herr) {
          set_error("%s: bounded wait expired (code %d)", name, herr);
          rc = GDFT_ERR_DEVICE;
        } else if (f32out) {
          float *tmp = new float[(size_t)M * N];
          if (ck(cudaMemcpy(tmp, d32, (size_t)M * N * 4, cudaMemcpyDeviceToHost), "probe out"))
            for (size_t i = 0; i < (size_t)M * N; ++i) h_d[i] = tmp[i];
          delete[] tmp;
        } else {
          double *tmp = new double[(size_t)nsplit * M * N];
          if (ck(cudaMemcpy(tmp, d64, (size_t)nsplit * M * N * 8, cudaMemcpyDeviceToHost), "probe out"))
            for (size_t i = 0; i < (size_t)M * N; ++i) {
              double s = 0.0;
              for (int z = 0; z < nsplit; ++z) s += tmp[(size_t)z * M * N + i];
              h_d[i] = s;
            }
          delete[] tmp;
        }
      }
    }
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(pA);
  cudaFree(pB);
  cudaFree(d32);
  cudaFree(d64);
  cudaFree(err);
  return rc;
}

extern "C" int gdft_tc_gemm_probe(int32_t M, int32_t N, int32_t K, int32_t nsplit, const double *h_a,
                                  const double *h_b, double *h_d) {
  return tc_gemm_probe(false, M, N, K, nsplit, h_a, h_b, h_d);
}

extern "C" int gdft_tc_gemm3_probe(int32_t M, int32_t N, int32_t K, int32_t nsplit, const double *h_a,
                                   const double *h_b, double *h_d) {
  return tc_gemm_probe(true, M, N, K, nsplit, h_a, h_b, h_d);
}
