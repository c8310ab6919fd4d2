// mlp_gemm.cuh - FP64 GEMM and reduction kernels shared by the network passes
// (mlp.cu: forward and adjoint; mlp_hvp.cu: tangent and second-order adjoint).
#pragma once

#include "common.cuh"
#include "mlp.cuh"

namespace gdft {
namespace {

// ----------------------------------------------------------------- GEMM ---
// C[M x N] = op(A) op(B) (+ beta C); row-major operands with leading dimensions.
//   kNN: A (M x K), B (K x N)       kNT: A (M x K), B stored (N x K)
//   kTN: A stored (K x M), B (K x N); K is split over blockIdx.z, each split
//        writing its own partial C at C + z * split_stride.
enum { kNN = 0, kNT = 1, kTN = 2 };
constexpr int GT = 64, GK = 16, GTH = 256;

template <int MODE>
__global__ void __launch_bounds__(GTH) gemm_f64_kernel(int M, int N, int K, const double *__restrict__ A, int lda,
                                                      const double *__restrict__ B, int ldb, double *__restrict__ C,
                                                      int ldc, double beta, int kchunk, size_t split_stride) {
  __shared__ double As[GK][GT + 1];
  __shared__ double Bs[GK][GT + 1];
  const int tid = threadIdx.x, tr = tid >> 4, tc = tid & 15;
  const int m0 = blockIdx.x * GT, n0 = blockIdx.y * GT;
  const int kb = MODE == kTN ? blockIdx.z * kchunk : 0;
  const int ke = MODE == kTN ? min(K, kb + kchunk) : K;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = kb; k0 < ke; k0 += GK) {
#pragma unroll
    for (int i = 0; i < (GK * GT) / GTH; ++i) {
      const int idx = tid + i * GTH;
      // Index maps chosen so that consecutive threads read consecutive addresses.
      {
        int kk, mm;
        if (MODE == kTN) {
          kk = idx / GT, mm = idx % GT;  // A stored (K x M): m fastest
        } else {
          mm = idx / GK, kk = idx % GK;  // A (M x K): k fastest
        }
        const int m = m0 + mm, k = k0 + kk;
        double a = 0.0;
        if (m < M && k < ke) a = MODE == kTN ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
        As[kk][mm] = a;
      }
      {
        int kk, nn;
        if (MODE == kNT) {
          nn = idx / GK, kk = idx % GK;  // B stored (N x K): k fastest
        } else {
          kk = idx / GT, nn = idx % GT;  // B (K x N): n fastest
        }
        const int n = n0 + nn, k = k0 + kk;
        double b = 0.0;
        if (n < N && k < ke) b = MODE == kNT ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n];
        Bs[kk][nn] = b;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tr + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tc + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  double *Cz = C + (MODE == kTN ? (size_t)blockIdx.z * split_stride : 0);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + tr + 16 * i, n = n0 + tc + 16 * j;
      if (m < M && n < N) {
        double *c = Cz + (size_t)m * ldc + n;
        *c = beta != 0.0 ? beta * *c + acc[i][j] : acc[i][j];
      }
    }
}

// C[i] = sum over splits of part[split][i] (fixed order).
__global__ void sum_splits_kernel(const double *__restrict__ part, int nsplit, size_t total, double *__restrict__ C) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; ++k) s += part[(size_t)k * total + i];
  C[i] = s;
}

// Column sums of X [rows][ncols] (stride ld), first pass: block b sums its row
// range into part[b][ncols]; second pass sums the partials in block order.
__global__ void colsum_part_kernel(const double *__restrict__ X, int64_t rows, int ncols, int ld,
                                   double *__restrict__ part) {
  const int64_t chunk = (rows + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * chunk, r1 = r0 + chunk < rows ? r0 + chunk : rows;
  for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
    double s = 0.0;
    for (int64_t r = r0; r < r1; ++r) s += X[(size_t)r * ld + c];
    part[(size_t)blockIdx.x * ncols + c] = s;
  }
}

// out[c] = sum over b of part[b][c]: one block of 8 warps per 32 columns, each
// warp sums an interleaved slice of the parts, warp 0 adds the eight in order.
__global__ void __launch_bounds__(256) colsum_final_kernel(const double *__restrict__ part, int nparts, int ncols,
                                                           double *__restrict__ out) {
  __shared__ double ws[8][32];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (c < ncols)
    for (int b = wid; b < nparts; b += 8) s += part[(size_t)b * ncols + c];
  ws[wid][lane] = s;
  __syncthreads();
  if (wid == 0 && c < ncols) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += ws[w][lane];
    out[c] = t;
  }
}
inline void launch_colsum_final(const double *part, int nparts, int ncols, double *out, cudaStream_t st) {
  colsum_final_kernel<<<(ncols + 31) / 32, 256, 0, st>>>(part, nparts, ncols, out);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int MODE>
cudaError_t gemm(int M, int N, int K, const double *A, int lda, const double *B, int ldb, double *C, int ldc,
                 double beta, cudaStream_t st) {
  dim3 grid((M + GT - 1) / GT, (N + GT - 1) / GT, 1);
  gemm_f64_kernel<MODE><<<grid, GTH, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, beta, K, 0);
  return cudaGetLastError();
}

// Split-K TN GEMM C (M x N) = A^T B over K rows, in nsplit fixed slices whose
// partials (in part, nsplit x M x N) are summed in slice order.
inline cudaError_t gemm_tn_split(int M, int N, int64_t K, const double *A, int lda, const double *B, int ldb,
                                 double *C, int nsplit, double *part, cudaStream_t st) {
  const int kchunk = (int)(((K + nsplit - 1) / nsplit + GK - 1) / GK * GK);
  dim3 grid((M + GT - 1) / GT, (N + GT - 1) / GT, nsplit);
  gemm_f64_kernel<kTN><<<grid, GTH, 0, st>>>(M, N, (int)K, A, lda, B, ldb, part, N, 0.0, kchunk, (size_t)M * N);
  cudaError_t r = cudaGetLastError();
  if (r != cudaSuccess) return r;
  const size_t total = (size_t)M * N;
  sum_splits_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(part, nsplit, total, C);
  return cudaGetLastError();
}

// Column sums of X (rows x ncols, stride ld) into out, in a fixed order.
inline cudaError_t col_sums(const double *X, int64_t rows, int ncols, int ld, double *out, double *part, int nparts,
                            cudaStream_t st) {
  colsum_part_kernel<<<nparts, 256, 0, st>>>(X, rows, ncols, ld, part);
  launch_colsum_final(part, nparts, ncols, out, st);
  return cudaGetLastError();
}


// ---- FP32 helpers of the mixed (tensor-core) network passes ----
__device__ __forceinline__ float eluf(float a) { return a > 0.0f ? a : expm1f(a); }

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void to_f32_kernel(const double *__restrict__ x, size_t n, float *__restrict__ y) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}

// Head weight gradients: part[block][c][0..2] = sum_r h[r][c] dy[r][f] over the
// block's row range, part[block][W*3 + f] = sum of dy[r][f] over its rows below
// rows_bias (the bias sees only primal rows); one thread per column.
__global__ void head_wgrad_part_kernel(const float *__restrict__ H, const float *__restrict__ dyf,
                                       const double *__restrict__ dy, int64_t rows, int64_t rows_bias, int width,
                                       double *__restrict__ part) {
  const int64_t chunk = (rows + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * chunk, r1 = r0 + chunk < rows ? r0 + chunk : rows;
  double *pb = part + (size_t)blockIdx.x * (3 * width + 3);
  for (int c = threadIdx.x; c < width; c += blockDim.x) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int64_t rb = r0; rb < r1; rb += 16) {  // FP32 over 16 rows, FP64 across
      float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f;
      if (rb + 16 <= r1) {  // all 16 rows' loads issued together
        float hv[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) hv[j] = H[(size_t)(rb + j) * width + c];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int64_t r = rb + j;
          f0 = fmaf(hv[j], dyf[r * 3 + 0], f0);
          f1 = fmaf(hv[j], dyf[r * 3 + 1], f1);
          f2 = fmaf(hv[j], dyf[r * 3 + 2], f2);
        }
      } else {
        for (int64_t r = rb; r < r1; ++r) {
          const float hv = H[(size_t)r * width + c];
          f0 = fmaf(hv, dyf[r * 3 + 0], f0);
          f1 = fmaf(hv, dyf[r * 3 + 1], f1);
          f2 = fmaf(hv, dyf[r * 3 + 2], f2);
        }
      }
      a0 += f0;
      a1 += f1;
      a2 += f2;
    }
    pb[c * 3 + 0] = a0;
    pb[c * 3 + 1] = a1;
    pb[c * 3 + 2] = a2;
  }
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int64_t r = r0; r < (r1 < rows_bias ? r1 : rows_bias); ++r) s += dy[r * 3 + threadIdx.x];
    pb[3 * width + threadIdx.x] = s;
  }
}

}  // namespace
}  // namespace gdft
