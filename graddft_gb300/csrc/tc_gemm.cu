// tc_gemm.cu - TF32x3 tensor-core GEMM on pre-packed operand blocks (tcgen05).
//
//   D[M x N] = sum_K A[M x K] B[N x K]^T      (both operands K-major)
//
// Operands arrive as 16 KB blocks of 128 rows x 32 K (TF32 hi and lo images,
// the K-major no-swizzle shared-memory layout of umma::kblock_off), stored
// [row tile][K chunk][hi|lo]; one stage is one bulk copy of A (32 KB) and one
// of B (32 KB).  Three products per term (hi*hi + hi*lo + lo*hi), M = 128,
// N = 128 per CTA.  Accumulation: each 32-wide K chunk is accumulated in one
// of three TMEM buffers W (128 columns each; the MMA runs up to two chunks
// ahead of the drains), correction products first, and eight drain warps fold
// it into a Kahan-compensated FP32 running sum: S in TMEM (128 columns), the
// compensation C in registers (each drain thread owns one output row and 64
// columns).  The K range may be split
// across blockIdx.y (split-K); each split writes its S - C either as FP32 into
// a row-major output (single split) or as FP64 partials [split][M][N].
//
// Warp roles (320 threads): warp 0 = TMA producer, warp 1 = TMEM owner and
// MMA issuer, warps 2-9 = drains (TMEM lane quadrant warp % 4, column half
// (warp - 2) / 4).  All waits are bounded; on expiry the CTA records an error
// word and winds down.
#include "common.cuh"
#include "kernels.cuh"
#include "tc_gemm.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

constexpr uint32_t kOpBytes = 2 * umma::kBlockBytes;   // hi | lo of one 128 x 32 block
// Stage = A hi|lo, B hi|lo (and, with a third A slice, that block too).
template <bool kThree>
struct Cfg {
  static constexpr uint32_t kStageBytes = 2 * kOpBytes + (kThree ? umma::kBlockBytes : 0);
  static constexpr int kStages = kThree ? 2 : 3;
  static constexpr int kSmemBytes = kStages * kStageBytes + 1024;
};
constexpr int kThreads = 320;
constexpr int kWBufs = 3;
constexpr uint32_t kTmemCols = 512;  // W0..W2 [0, 384), S [384, 512)
constexpr uint32_t kScol = 384;

__device__ __forceinline__ void flag(int *err, int code) { atomicCAS(err, 0, code); }

template <bool kThree>
__global__ void __launch_bounds__(kThreads, 1) tcg_kernel(const TcgArgs A) {
  constexpr int kStages = Cfg<kThree>::kStages;
  constexpr uint32_t kStageBytes = Cfg<kThree>::kStageBytes;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], wfull[kWBufs], wempty[kWBufs], drain;
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x % A.m_tiles, nt = blockIdx.x / A.m_tiles;
  const int64_t c0 = (int64_t)blockIdx.y * A.chunks_per_split;
  const int64_t c1 = c0 + A.chunks_per_split < A.k_chunks ? c0 + A.chunks_per_split : A.k_chunks;
  const int64_t nst = c1 > c0 ? c1 - c0 : 0;

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
  const float *a_tile = A.a + (size_t)mt * A.a_chunks * (kOpBytes / 4);
  const float *a3_tile = kThree ? A.a3 + (size_t)mt * A.a_chunks * (umma::kBlockBytes / 4) : nullptr;
  const float *b_tile = A.b + (size_t)nt * A.b_chunks * (kOpBytes / 4);

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    // One thread issues the copies; its waits are bounded and single-threaded.
    if (lane == 0) {
      int64_t it = 0;
      for (; it < nst; ++it) {
        const int s = (int)(it % kStages);
        if (!umma::mbar_wait(&empty[s], ((it / kStages) & 1) ^ 1)) {
          flag(A.err, 41);
          break;
        }
        const int64_t kc = c0 + it;
        umma::mbar_arrive_expect_tx(&full[s], kStageBytes);
        umma::bulk_g2s(smem + s * kStageBytes, a_tile + (size_t)kc * (kOpBytes / 4), kOpBytes, &full[s]);
        umma::bulk_g2s(smem + s * kStageBytes + kOpBytes, b_tile + (size_t)kc * (kOpBytes / 4), kOpBytes, &full[s]);
        if (kThree)
          umma::bulk_g2s(smem + s * kStageBytes + 2 * kOpBytes, a3_tile + (size_t)kc * (umma::kBlockBytes / 4),
                         umma::kBlockBytes, &full[s]);
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
      const uint64_t da30 = umma::sdesc(sa0 + 2 * kOpBytes, umma::kBlockLBO, umma::kBlockSBO);
      for (int64_t it = 0; it < nst; ++it) {
        const int s = (int)(it % kStages);
        const int buf = (int)(it % kWBufs);
        if (!umma::mbar_wait(&wempty[buf], ((it / kWBufs) & 1) ^ 1) ||
            !umma::mbar_wait(&full[s], (it / kStages) & 1)) {
          flag(A.err, 43);
          break;
        }
        umma::tc_fence_after();
        const uint32_t d = tbase + buf * 128;
        const uint64_t so = (uint64_t)s * (kStageBytes >> 4);  // slot offset in the address field
        const uint64_t ahi = dahi0 + so, alo = dalo0 + so, bhi = dbhi0 + so, blo = dblo0 + so;
        // Products from the smallest up, the hi*hi ones last (the accumulator's
        // truncation is relative to its size at each instruction).
        if (kThree) {
          const uint64_t a3 = da30 + so;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma::mma_tf32(d, alo + 16 * kk, blo + 16 * kk, idesc, kk == 0 ? 0u : 1u),
                umma::mma_tf32(d, a3 + 16 * kk, bhi + 16 * kk, idesc, 1u);
        }
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          umma::mma_tf32(d, ahi + 16 * kk, blo + 16 * kk, idesc, (!kThree && kk == 0) ? 0u : 1u),
              umma::mma_tf32(d, alo + 16 * kk, bhi + 16 * kk, idesc, 1u);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) umma::mma_tf32(d, ahi + 16 * kk, bhi + 16 * kk, idesc, 1u);
        umma::mma_commit(&empty[s]);
        umma::mma_commit(&wfull[buf]);
      }
      umma::mma_commit(&drain);
      if (!umma::mbar_wait(&drain, 0)) flag(A.err, 45);
    }
    __syncwarp();
  } else {
    // -------------------------------------------------------------- drains
    const int q = warp & 3, half = (warp - 2) >> 2;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16) + half * 64;
    float C[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) C[i] = 0.0f;
    int64_t it = 0;
    for (; it < nst; ++it) {
      const int buf = (int)(it % kWBufs);
      if (!umma::warp_wait(&wfull[buf], (it / kWBufs) & 1)) {
        if (lane == 0) flag(A.err, 46);
        break;
      }
      umma::tc_fence_after();
#pragma unroll
      for (int c = 0; c < 64; c += 32) {
        uint32_t wr[32], sr[32];
        umma::tmem_ld32_nowait(tl + buf * 128 + c, wr);
        if (it > 0) umma::tmem_ld32_nowait(tl + kScol + c, sr);
        umma::tmem_ld_wait(wr, sr);
        float sv[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float w = __uint_as_float(wr[i]);
          if (it == 0) {
            sv[i] = w;
          } else {  // Kahan: S + (w - C)
            const float sp = __uint_as_float(sr[i]);
            const float y = w - C[c + i];
            const float t = sp + y;
            C[c + i] = (t - sp) - y;
            sv[i] = t;
          }
        }
        umma::tmem_st32(tl + kScol + c, sv);
      }
      umma::tmem_st_wait();
      umma::tc_fence_before();
      umma::mbar_arrive(&wempty[buf]);
    }
    const bool have = it == nst && nst > 0;
    const int m = mt * 128 + q * 32 + lane;
    const int n0 = nt * 128 + half * 64;
#pragma unroll
    for (int c = 0; c < 64; c += 32) {
      float sv[32];
      if (have) umma::tmem_ld32(tl + kScol + c, sv);
      if (m < A.m_valid) {
        if (A.out32) {
          float *row = A.out32 + (size_t)m * A.ldo + n0 + c;
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (n0 + c + i < A.n_valid) row[i] = have ? sv[i] - C[c + i] : 0.0f;
        } else {
          double *row = A.out64 + ((size_t)blockIdx.y * A.m_valid + m) * A.n_valid + n0 + c;
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (n0 + c + i < A.n_valid) row[i] = have ? (double)sv[i] - (double)C[c + i] : 0.0;
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
  static bool attr2 = false, attr3 = false;
  if (!attr2) {
    cudaError_t e = cudaFuncSetAttribute(tcg_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Cfg<false>::kSmemBytes);
    if (e != cudaSuccess) return e;
    attr2 = true;
  }
  if (!attr3) {
    cudaError_t e = cudaFuncSetAttribute(tcg_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Cfg<true>::kSmemBytes);
    if (e != cudaSuccess) return e;
    attr3 = true;
  }
  if (a.m_tiles <= 0 || a.n_tiles <= 0 || nsplit <= 0 || (a.out32 == nullptr) == (a.out64 == nullptr) ||
      (a.out32 && nsplit != 1) || a.k_chunks > a.a_chunks || a.k_chunks > a.b_chunks)
    return cudaErrorInvalidValue;
  dim3 grid(a.m_tiles * a.n_tiles, nsplit);
  if (a.a3)
    tcg_kernel<true><<<grid, kThreads, Cfg<true>::kSmemBytes, st>>>(a);
  else
    tcg_kernel<false><<<grid, kThreads, Cfg<false>::kSmemBytes, st>>>(a);
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

}  // namespace

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

// Host-array probe of the packed TF32x3 GEMM (synchronous; allocates its own
// buffers): D (M x N, FP64) = A (M x K) B (N x K)^T, through the row-tile packer
// and tcg_kernel, FP32 output for nsplit == 1, FP64 split-K partials summed on
// the host otherwise.
extern "C" int gdft_tc_gemm_probe(int32_t M, int32_t N, int32_t K, int32_t nsplit, const double *h_a,
                                  const double *h_b, double *h_d) {
  using namespace gdft;
  if (M <= 0 || N <= 0 || K <= 0 || nsplit <= 0 || !h_a || !h_b || !h_d || M > 4096 || N > 4096 ||
      K > (1 << 20)) {
    set_error("gdft_tc_gemm_probe: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  const int mt = (M + 127) / 128, ntl = (N + 127) / 128;
  const int64_t kch = (K + 31) / 32;
  const size_t blk = 2 * (umma::kBlockBytes / 4);
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
      ck(launch_pack_rt<double>(dA, M, K, K, mt, (int)kch, pA, 0), "probe pack A") &&
      ck(launch_pack_rt<double>(dB, N, K, K, ntl, (int)kch, pB, 0), "probe pack B")) {
    TcgArgs a{};
    a.a = pA;
    a.b = pB;
    a.m_tiles = mt;
    a.n_tiles = ntl;
    a.a_chunks = a.b_chunks = a.k_chunks = kch;
    a.chunks_per_split = nsplit == 1 ? kch : cps;
    a.out32 = nsplit == 1 ? d32 : nullptr;
    a.ldo = N;
    a.out64 = nsplit == 1 ? nullptr : d64;
    a.m_valid = M;
    a.n_valid = N;
    a.err = err;
    if (ck(launch_tcg(a, nsplit, 0), "probe tcg") && ck(cudaDeviceSynchronize(), "probe sync")) {
      int herr = 0;
      if (ck(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost), "probe err")) {
        if (herr) {
          set_error("gdft_tc_gemm_probe: bounded wait expired (code %d)", herr);
          rc = GDFT_ERR_DEVICE;
        } else if (nsplit == 1) {
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
