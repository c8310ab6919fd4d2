// tc_selftest.cu - device self-test of the tcgen05 building blocks.
//
// One CTA computes D (128 x 128) = A (128 x 32) * B (128 x 32)^T with kind::tf32
// from blocks in the K-major no-swizzle layout, loaded by the TMA engine
// (cp.async.bulk), accumulated in TMEM and read back with tcgen05.ld.  The
// inputs are small integers, so the product is exact and any layout or
// descriptor error shows up as a mismatch.
#include <math.h>
#include <stdlib.h>

#include "common.cuh"
#include "umma.cuh"

namespace gdft {
namespace {

__global__ void __launch_bounds__(128) umma_selftest_kernel(const float *__restrict__ a_blk,
                                                            const float *__restrict__ b_blk, float *__restrict__ d,
                                                            int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  float *sa = (float *)smem;
  float *sb = (float *)(smem + umma::kBlockBytes);
  __shared__ __align__(8) uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    umma::mbar_init(&bar_load, 1);
    umma::mbar_init(&bar_mma, 1);
    umma::fence_barrier_init();
  }
  if (warp == 0) umma::tmem_alloc(&tmem_base, 128);
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tbase = tmem_base;
  bool ok = true;
  if (threadIdx.x == 0) {
    umma::mbar_arrive_expect_tx(&bar_load, 2 * umma::kBlockBytes);
    umma::bulk_g2s(sa, a_blk, umma::kBlockBytes, &bar_load);
    umma::bulk_g2s(sb, b_blk, umma::kBlockBytes, &bar_load);
    ok = umma::mbar_wait(&bar_load, 0);
    if (ok) {
      umma::tc_fence_after();
      const uint32_t idesc = umma::idesc_tf32(128, 128);
      for (int kk = 0; kk < 4; ++kk) {
        const uint64_t ad = umma::sdesc(umma::smem_u32(sa) + kk * 256, umma::kBlockLBO, umma::kBlockSBO);
        const uint64_t bd = umma::sdesc(umma::smem_u32(sb) + kk * 256, umma::kBlockLBO, umma::kBlockSBO);
        umma::mma_tf32(tbase, ad, bd, idesc, kk > 0 ? 1u : 0u);
      }
      umma::mma_commit(&bar_mma);
    } else {
      atomicExch(err, 1);
    }
  }
  __syncthreads();
  // Every warp waits for the accumulator, then reads its 32 lanes.
  ok = umma::mbar_wait(&bar_mma, 0);
  if (!ok) atomicExch(err, 2);
  umma::tc_fence_after();
  if (ok) {
    const int row = warp * 32 + lane;
    for (int c0 = 0; c0 < 128; c0 += 32) {
      float v[32];
      umma::tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + c0, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) d[row * 128 + c0 + j] = v[j];
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tbase, 128);
}

// Waits on an mbarrier that nothing arrives on, with a short poll limit, so
// that the bounded wait every pipeline kernel uses runs out: the thread
// records `code` in the error word and the CTA returns.  Nothing else is in
// flight (no bulk copy, no MMA, no TMEM held), so the context stays usable.
__global__ void wait_expiry_probe_kernel(int *__restrict__ err, uint32_t limit, int code) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    umma::mbar_init(&bar, 1);
    umma::fence_barrier_init();
    if (!umma::mbar_wait_n(&bar, 0, limit)) atomicCAS(err, 0, code);
    umma::mbar_inval(&bar);
  }
}

}  // namespace

cudaError_t launch_wait_expiry_probe(int *err, uint32_t limit, int code, cudaStream_t st) {
  wait_expiry_probe_kernel<<<1, 32, 0, st>>>(err, limit, code);
  return cudaGetLastError();
}

}  // namespace gdft

using namespace gdft;

// D (128 x 128) = A (128 x 32) B (128 x 32)^T on the tensor cores for caller
// data (host arrays, row-major, values taken as TF32); used to characterise
// the accumulation rounding of kind::tf32 against exact products.
static int run_umma_128x128x32(const float *ha, const float *hb, float *hd) {
  const int M = 128, N = 128, K = 32;
  float *hpa = (float *)calloc(umma::kBlockBytes / 4, 4), *hpb = (float *)calloc(umma::kBlockBytes / 4, 4);
  for (int i = 0; i < M; ++i)
    for (int k = 0; k < K; ++k) hpa[umma::kblock_off(i, k) / 4] = ha[i * K + k];
  for (int j = 0; j < N; ++j)
    for (int k = 0; k < K; ++k) hpb[umma::kblock_off(j, k) / 4] = hb[j * K + k];
  float *da = nullptr, *db = nullptr, *dd = nullptr;
  int *derr = nullptr;
  int rc = GDFT_OK;
  cudaError_t e = cudaMalloc(&da, umma::kBlockBytes);
  if (e == cudaSuccess) e = cudaMalloc(&db, umma::kBlockBytes);
  if (e == cudaSuccess) e = cudaMalloc(&dd, sizeof(float) * M * N);
  if (e == cudaSuccess) e = cudaMalloc(&derr, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(da, hpa, umma::kBlockBytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, hpb, umma::kBlockBytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dd, 0, sizeof(float) * M * N);
  const int smem = 2 * umma::kBlockBytes + 1024;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(umma_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) {
    umma_selftest_kernel<<<1, 128, smem>>>(da, db, dd, derr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hd, dd, sizeof(float) * M * N, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    rc = check_cuda(e, "umma 128x128x32");
  } else if (herr != 0) {
    set_error("umma 128x128x32: bounded wait expired (stage %d)", herr);
    rc = GDFT_ERR_DEVICE;
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(dd);
  cudaFree(derr);
  free(hpa);
  free(hpb);
  return rc;
}

extern "C" int gdft_umma_probe(const float *h_a, const float *h_b, float *h_d) {
  if (h_a == nullptr || h_b == nullptr || h_d == nullptr) {
    set_error("gdft_umma_probe: null argument");
    return GDFT_ERR_INVALID;
  }
  return run_umma_128x128x32(h_a, h_b, h_d);
}

extern "C" int gdft_selftest_umma(double *max_abs_err) {
  if (max_abs_err == nullptr) {
    set_error("gdft_selftest_umma: null output");
    return GDFT_ERR_INVALID;
  }
  const int M = 128, N = 128, K = 32;
  float *ha = (float *)malloc(sizeof(float) * M * K), *hb = (float *)malloc(sizeof(float) * N * K);
  float *hd = (float *)malloc(sizeof(float) * M * N);
  for (int i = 0; i < M; ++i)
    for (int k = 0; k < K; ++k) ha[i * K + k] = (float)(((i * 7 + k * 3) % 11) - 5);
  for (int j = 0; j < N; ++j)
    for (int k = 0; k < K; ++k) hb[j * K + k] = (float)(((j * 5 + k * 13) % 9) - 4);
  const int rc = run_umma_128x128x32(ha, hb, hd);
  if (rc == GDFT_OK) {
    double mx = 0.0;
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < N; ++j) {
        double ref = 0.0;
        for (int k = 0; k < K; ++k) ref += (double)ha[i * K + k] * hb[j * K + k];
        mx = fmax(mx, fabs(ref - hd[i * N + j]));
      }
    *max_abs_err = mx;
  }
  free(ha);
  free(hb);
  free(hd);
  return rc;
}
