// tc_pack.cu - operand layouts of the TF32x3 (mixed) form.
//
// The AO planes (phi, d_x phi, d_y phi, d_z phi, lap phi) are kept resident in
// pre-tiled layouts whose 16 KB blocks are exactly the shared-memory images the
// tensor cores read (K-major, no swizzle, see umma::kblock_off), so every
// operand stage is one contiguous bulk copy:
//   point-major  [point tile (128)][plane][AO chunk (32)][hi|lo] : 128 points x 32 AO,
//     TF32 pairs hi + lo ~= the FP64 value to about 22 bits
//     (A operand of the density contraction and its epilogue partners)
//   AO-major     [AO tile (128)][plane 0-3][point chunk (32)][hi|lo|lo2] : 128 AO x 32 points,
//     block-scaled three-slice sets (umma::store_row3: hi quantised per AO and
//     point chunk, hi + lo + lo2 ~= x to about 2^-33 of the chunk's largest value)
//     (A operand of the V_xc contraction, contracted over points)
//   AO-major FP32 pairs [AO tile (128)][plane][point chunk (32)][hi|lo] : the same
//     blocks as hi = fp32(x), lo = fp32(x - hi) (together about 2^-48 of x; the
//     inputs of the B operand that is built per call in double-float arithmetic)
// The density matrix is packed per call as the B operand of the density
// contraction: [spin][column tile (128)][k chunk (32)][hi|lo], element (c, k) = D[k][c].
#include "common.cuh"
#include "kernels.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

__device__ __forceinline__ size_t pm_block(int64_t tile, int plane, int kc, int nkc) {
  return ((size_t)(tile * kPlanes + plane) * nkc + kc) * 2;  // in units of 16 KB blocks (hi; lo = +1)
}
__device__ __forceinline__ size_t av_set(int atile, int plane, int64_t pc, int64_t npc) {
  return (size_t)(atile * 4 + plane) * npc + pc;  // in units of three-block sets (48 KB)
}
__device__ __forceinline__ size_t af_block(int atile, int plane, int64_t pc, int64_t npc) {
  return ((size_t)(atile * kPlanes + plane) * npc + pc) * 2;  // in units of 16 KB blocks (hi; lo = +1)
}

__device__ __forceinline__ void store_split(float *base, size_t blk, uint32_t off, double v) {
  float hi, lo;
  umma::split_tf32(v, hi, lo);
  float *b = (float *)((char *)base + blk * umma::kBlockBytes);
  b[off / 4] = hi;
  b[umma::kBlockBytes / 4 + off / 4] = lo;
}

// Sources of the plane values (contracted shells go through the tile sink below).
enum PackSrc { kFromTables = 0, kFromSynthetic = 1 };

// Scatter the five plane values of (point p, AO a) into the point-major pairs,
// the parked FP64 values of the AO-major sets and the AO-major FP32 pairs.
__device__ __forceinline__ void pack_store(float *__restrict__ pm, float *__restrict__ av, float *__restrict__ af,
                                           int64_t np, int ldk, int64_t p, int a, const double v[kPlanes]) {
  const int nkc = ldk / 32;
  const int64_t npc = np / 32;
  const int64_t tile = p / 128;
#pragma unroll
  for (int t = 0; t < kPlanes; ++t) {
    store_split(pm, pm_block(tile, t, a / 32, nkc), umma::kblock_off((int)(p % 128), a % 32), v[t]);
    if (t < 4)
      ((double *)(av + av_set(a / 128, t, p / 32, npc) * 3 * (umma::kBlockBytes / 4)))[(p % 32) * 128 + a % 128] =
          v[t];
    float *afb = af + af_block(a / 128, t, p / 32, npc) * (umma::kBlockBytes / 4) +
                 umma::kblock_off(a % 128, (int)(p % 32)) / 4;
    const float hi = (float)v[t];
    afb[0] = hi;
    afb[umma::kBlockBytes / 4] = (float)(v[t] - (double)hi);
  }
}

// One thread per (point, AO) of the padded tables: computes the five plane
// values (from reference layouts, the synthetic basis or contracted shells) and scatters
// them into the point-major and FP32 layouts.  The AO-major three-slice sets
// need each AO's maximum over a point chunk first: this pass parks the FP64
// values of a set, [point (32)][AO (128)], in the set's own first 32 KB and
// pack_av_kernel splits them in place.
template <int kSrc>
__global__ void pack_tables_kernel(const double *__restrict__ ao, const double *__restrict__ grad_ao,
                                   const double *__restrict__ grad2_ao, const double *__restrict__ basis,
                                   const double *__restrict__ coords, const double *__restrict__ w, int64_t n_grid,
                                   int n_ao, int64_t np, int ldk, float *__restrict__ pm, float *__restrict__ av,
                                   float *__restrict__ af, double *__restrict__ wout) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)np * ldk) return;
  const int64_t p = (int64_t)(idx / ldk);
  const int a = (int)(idx % ldk);
  double v[kPlanes] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (p < n_grid && a < n_ao) {
    if (kSrc == kFromTables) {
      const size_t r = (size_t)p * n_ao + a;
      v[T_PHI] = ao[r];
      v[T_DX] = grad_ao[3 * r + 0];
      v[T_DY] = grad_ao[3 * r + 1];
      v[T_DZ] = grad_ao[3 * r + 2];
      if (grad2_ao != nullptr) v[T_LAP] = (grad2_ao[3 * r + 0] + grad2_ao[3 * r + 1]) + grad2_ao[3 * r + 2];
    } else {
      const double *b = basis + 8 * (size_t)a;
      const double x = coords[3 * p + 0] - b[0];
      const double y = coords[3 * p + 1] - b[1];
      const double z = coords[3 * p + 2] - b[2];
      const double al = b[3];
      const double ex = b[4] * exp(-al * (x * x + y * y + z * z));
      const int kind = (int)b[5], comp = (int)b[6];
      double P = 1.0, dP[3] = {0.0, 0.0, 0.0}, d2P[3] = {0.0, 0.0, 0.0};
      const double xyz[3] = {x, y, z};
      if (kind == 1) {
        P = xyz[comp];
        dP[comp] = 1.0;
      } else if (kind == 2) {
        if (comp <= 2) {
          const int i0 = comp == 1 ? 1 : 0, i1 = comp == 0 ? 1 : 2;
          P = xyz[i0] * xyz[i1];
          dP[i0] = xyz[i1];
          dP[i1] = xyz[i0];
        } else if (comp == 3) {
          P = x * x - y * y;
          dP[0] = 2 * x;
          dP[1] = -2 * y;
          d2P[0] = 2.0;
          d2P[1] = -2.0;
        } else {
          P = 2 * z * z - x * x - y * y;
          dP[0] = -2 * x;
          dP[1] = -2 * y;
          dP[2] = 4 * z;
          d2P[0] = -2.0;
          d2P[1] = -2.0;
          d2P[2] = 4.0;
        }
      }
      v[T_PHI] = P * ex;
      double lp[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        v[T_DX + i] = (dP[i] - 2 * al * xyz[i] * P) * ex;
        lp[i] = (d2P[i] - 2 * al * P - 4 * al * xyz[i] * dP[i] + 4 * al * al * xyz[i] * xyz[i] * P) * ex;
      }
      v[T_LAP] = (lp[0] + lp[1]) + lp[2];
    }
  }
  pack_store(pm, av, af, np, ldk, p, a, v);
  if (a == 0) wout[p] = p < n_grid ? w[p] : 0.0;
}

// Sink of the shell tiles (shells.cuh) into the same three layouts.
struct PackSink {
  float *pm, *av, *af;
  const double *w;
  double *wout;
  int64_t n_grid, np;
  int n_ao, ldk;
  __device__ void operator()(const double *tile, int t, int ps, int64_t p, int a) const {
    if (a >= ldk) return;
    const bool live = p < n_grid && a < n_ao;
    double v[kPlanes];
#pragma unroll
    for (int q = 0; q < kPlanes; ++q) v[q] = live ? tile[q * ps + t] : 0.0;
    pack_store(pm, av, af, np, ldk, p, a, v);
    if (a == 0) wout[p] = p < n_grid ? w[p] : 0.0;
  }
};

// One CTA of 128 threads per AO-major set, one AO row per thread: reads the
// parked FP64 values, then (after the whole CTA has read) writes hi|lo|lo2 over them.
__global__ void __launch_bounds__(128) pack_av_kernel(float *__restrict__ av) {
  float *set = av + (size_t)blockIdx.x * 3 * (umma::kBlockBytes / 4);
  const double *parked = (const double *)set;
  const int row = threadIdx.x;
  double v[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = parked[k * 128 + row];
  __syncthreads();
  umma::store_row3(set, row, v);
}

// D (2, n, n) -> [spin][column tile][k chunk][hi|lo] blocks with (c, k) = D[k][c].
__global__ void pack_rdm1_kernel(const double *__restrict__ D, int n, int ldk, float *__restrict__ out) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per_spin = (size_t)ldk * ldk;
  if (idx >= 2 * per_spin) return;
  const int s = (int)(idx / per_spin);
  const int k = (int)((idx % per_spin) / ldk);
  const int c = (int)(idx % ldk);
  const double v = (k < n && c < n) ? D[((size_t)s * n + k) * n + c] : 0.0;
  const int nkc = ldk / 32, ncb = ldk / 128;
  const size_t blk = (((size_t)s * ncb + c / 128) * nkc + k / 32) * 2;
  store_split(out, blk, umma::kblock_off(c % 128, k % 32), v);
}

}  // namespace

cudaError_t launch_pack_tables(const double *ao, const double *grad_ao, const double *grad2_ao, const double *basis,
                               const double *coords, const double *w, int64_t n_grid, int n_ao, int64_t np, int ldk,
                               float *pm, float *av, float *af, double *wout, cudaStream_t st,
                               const ShellView *shells) {
  cudaError_t e;
  if (shells != nullptr) {
    e = launch_shell_tiles<kPlanes>(*shells, coords, n_grid, np, ldk,
                                    PackSink{pm, av, af, w, wout, n_grid, np, n_ao, ldk}, st);
  } else {
    const size_t total = (size_t)np * ldk;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    if (basis != nullptr)
      pack_tables_kernel<kFromSynthetic><<<blocks, 256, 0, st>>>(ao, grad_ao, grad2_ao, basis, coords, w, n_grid,
                                                                 n_ao, np, ldk, pm, av, af, wout);
    else
      pack_tables_kernel<kFromTables><<<blocks, 256, 0, st>>>(ao, grad_ao, grad2_ao, basis, coords, w, n_grid, n_ao,
                                                              np, ldk, pm, av, af, wout);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return e;
  pack_av_kernel<<<(unsigned)((size_t)(ldk / 128) * 4 * (np / 32)), 128, 0, st>>>(av);
  return cudaGetLastError();
}

cudaError_t launch_pack_rdm1(const double *D, int n, int ldk, float *out, cudaStream_t st) {
  const size_t total = (size_t)2 * ldk * ldk;
  pack_rdm1_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(D, n, ldk, out);
  return cudaGetLastError();
}

}  // namespace gdft
