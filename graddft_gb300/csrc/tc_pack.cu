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
#include "dfloat.cuh"
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

// Block-scaled three-slice split of a double-float value on the row quantum u
// (as umma::split3, with the remainder (s - hi) + c formed in FP32).
__device__ __forceinline__ void split3_df(df::DF v, umma::Quant u, float &hi, float &lo, float &lo2) {
  hi = rintf(v.s * u.inv) * u.q;
  const float r = __fadd_rn(__fsub_rn(v.s, hi), v.c);
  lo = umma::tf32_rn(r);
  lo2 = umma::tf32_rn(__fsub_rn(r, lo));
}
// TF32 hi + lo of a double-float value (hi + lo about 2^-22 of it).
__device__ __forceinline__ void split_tf32_df(df::DF v, float &hi, float &lo) {
  hi = umma::tf32_rn(v.s);
  lo = umma::tf32_rn(__fadd_rn(__fsub_rn(v.s, hi), v.c));
}

// Scatter the five plane values of (point p, AO a), given as double-float
// pairs, into the point-major pairs, the parked pairs of the AO-major sets and
// the AO-major FP32 pairs.
__device__ __forceinline__ void pack_store(float *__restrict__ pm, float *__restrict__ av, float *__restrict__ af,
                                           int64_t np, int ldk, int64_t p, int a, const df::DF v[kPlanes]) {
  const int nkc = ldk / 32;
  const int64_t npc = np / 32;
  const int64_t tile = p / 128;
#pragma unroll
  for (int t = 0; t < kPlanes; ++t) {
    const df::DF x = df::norm(v[t]);
    float hi, lo;
    split_tf32_df(x, hi, lo);
    float *b = (float *)((char *)pm + pm_block(tile, t, a / 32, nkc) * umma::kBlockBytes);
    const uint32_t off = umma::kblock_off((int)(p % 128), a % 32) / 4;
    b[off] = hi;
    b[umma::kBlockBytes / 4 + off] = lo;
    if (t < 4)
      ((float2 *)(av + av_set(a / 128, t, p / 32, npc) * 3 * (umma::kBlockBytes / 4)))[(p % 32) * 128 + a % 128] =
          make_float2(x.s, x.c);
    float *afb = af + af_block(a / 128, t, p / 32, npc) * (umma::kBlockBytes / 4) +
                 umma::kblock_off(a % 128, (int)(p % 32)) / 4;
    afb[0] = x.s;
    afb[umma::kBlockBytes / 4] = x.c;
  }
}

// One thread per (point, AO) of the padded tables: the five plane values from
// the reference layouts (ao, grad_ao, grad_n_ao[2]), scattered into the
// point-major and FP32-pair layouts.  The AO-major three-slice sets need each
// AO's maximum over a point chunk first: this pass parks the values of a set,
// [point (32)][AO (128)] as FP32 pairs, in the set's own first 32 KB and
// pack_av_kernel splits them in place.
__global__ void pack_tables_kernel(const double *__restrict__ ao, const double *__restrict__ grad_ao,
                                   const double *__restrict__ grad2_ao, const double *__restrict__ w,
                                   int64_t n_grid, int n_ao, int64_t np, int ldk, float *__restrict__ pm,
                                   float *__restrict__ av, float *__restrict__ af, double *__restrict__ wout) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)np * ldk) return;
  const int64_t p = (int64_t)(idx / ldk);
  const int a = (int)(idx % ldk);
  double v[kPlanes] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (p < n_grid && a < n_ao) {
    const size_t r = (size_t)p * n_ao + a;
    v[T_PHI] = ao[r];
    v[T_DX] = grad_ao[3 * r + 0];
    v[T_DY] = grad_ao[3 * r + 1];
    v[T_DZ] = grad_ao[3 * r + 2];
    if (grad2_ao != nullptr) v[T_LAP] = (grad2_ao[3 * r + 0] + grad2_ao[3 * r + 1]) + grad2_ao[3 * r + 2];
  }
  df::DF dv[kPlanes];
#pragma unroll
  for (int t = 0; t < kPlanes; ++t) dv[t] = df::of_double(v[t]);
  pack_store(pm, av, af, np, ldk, p, a, dv);
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
    df::DF v[kPlanes];
#pragma unroll
    for (int q = 0; q < kPlanes; ++q) v[q] = df::of_double(live ? tile[q * ps + t] : 0.0);
    pack_store(pm, av, af, np, ldk, p, a, v);
    if (a == 0) wout[p] = p < n_grid ? w[p] : 0.0;
  }
};

// Writes one AO row (32 points) of a three-slice set [hi | lo | lo2] from
// double-float values, quantised on the row's own maximum.
__device__ __forceinline__ void store_row3_df(float *blk3, int row, const df::DF (&v)[32]) {
  float m = 0.0f;
#pragma unroll
  for (int k = 0; k < 32; ++k) m = fmaxf(m, fabsf(v[k].s));
  const umma::Quant u = umma::quant(m);
#pragma unroll
  for (int k4 = 0; k4 < 8; ++k4) {
    float4 h, l, l2;
    split3_df(v[4 * k4 + 0], u, h.x, l.x, l2.x);
    split3_df(v[4 * k4 + 1], u, h.y, l.y, l2.y);
    split3_df(v[4 * k4 + 2], u, h.z, l.z, l2.z);
    split3_df(v[4 * k4 + 3], u, h.w, l.w, l2.w);
    const uint32_t off = umma::kblock_off(row, 4 * k4) / 4;
    *(float4 *)(blk3 + off) = h;
    *(float4 *)(blk3 + umma::kBlockBytes / 4 + off) = l;
    *(float4 *)(blk3 + umma::kBlockBytes / 2 + off) = l2;
  }
}

// One CTA of 128 threads per AO-major set, one AO row per thread: reads the
// parked double-float pairs, then (after the whole CTA has read) writes
// hi|lo|lo2 over them.
__global__ void __launch_bounds__(128) pack_av_kernel(float *__restrict__ av) {
  float *set = av + (size_t)blockIdx.x * 3 * (umma::kBlockBytes / 4);
  const float2 *parked = (const float2 *)set;
  const int row = threadIdx.x;
  df::DF v[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const float2 x = parked[k * 128 + row];
    v[k] = df::DF{x.x, x.y};
  }
  __syncthreads();
  store_row3_df(set, row, v);
}

// The mixed form's tables for the synthetic basis rows (n_ao, 8: centre,
// exponent, normalisation, kind, component), in double-float arithmetic: one
// CTA per (32-point chunk, 128-AO tile).  Phase 1 evaluates the tile's
// 32 x 128 x 5 values (phi, the gradient, the Laplacian) into shared memory;
// phase 2 writes the three layouts from there: the AO-major three-slice sets
// (quantised on each row's maximum over the chunk, so no parking pass), the
// AO-major FP32 pairs and the point-major TF32 pairs.  For an s/p/d function
// of degree l, with P its polynomial and e = N exp(-alpha r^2):
//   phi = P e,  d_i phi = (d_i P - 2 alpha x_i P) e,
//   lap phi = (4 alpha^2 r^2 - (6 + 4 l) alpha) P e   (these P are harmonic and
//   homogeneous: lap P = 0, x . grad P = l P).
constexpr int kBuildThreads = 256;
constexpr size_t kBuildSmem = (size_t)kPlanes * 32 * 128 * sizeof(float2);

__global__ void __launch_bounds__(kBuildThreads) build_tables_df_kernel(
    const double *__restrict__ basis, const double *__restrict__ coords, const double *__restrict__ w,
    int64_t n_grid, int n_ao, int64_t np, int ldk, float *__restrict__ pm, float *__restrict__ av,
    float *__restrict__ af, double *__restrict__ wout) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *S = (float2 *)smem_raw;  // [plane][point 32][AO 128]
  __shared__ float sx[32][6];       // point coordinates as pairs
  __shared__ float sb[128][10];     // AO centre (3 pairs), exponent pair, normalisation pair
  __shared__ int sk[128][2];        // kind, component
  const int64_t npc = np / 32;
  const int atile = (int)(blockIdx.x / npc);
  const int64_t pc = blockIdx.x % npc;
  const int tid = threadIdx.x;
  // Conversions to pairs once per point and per AO (the only FP64 work).
  if (tid < 32) {
    const int64_t p = pc * 32 + tid;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const df::DF c = df::of_double(p < n_grid ? coords[3 * p + i] : 0.0);
      sx[tid][2 * i] = c.s;
      sx[tid][2 * i + 1] = c.c;
    }
    if (atile == 0) wout[p] = p < n_grid ? w[p] : 0.0;
  }
  if (tid < 128) {
    const int a = atile * 128 + tid;
    const double *b = basis + 8 * (size_t)(a < n_ao ? a : 0);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const df::DF c = df::of_double(b[i]);
      sb[tid][2 * i] = c.s;
      sb[tid][2 * i + 1] = c.c;
    }
    sk[tid][0] = a < n_ao ? (int)b[5] : -1;  // -1: a padding AO (zero)
    sk[tid][1] = (int)b[6];
  }
  __syncthreads();
  // Phase 1: thread = (AO, half of the points).
  {
    const int al = tid & 127, ph = tid >> 7;
    const int kind = sk[al][0], comp = sk[al][1];
    const df::DF cen[3] = {{sb[al][0], sb[al][1]}, {sb[al][2], sb[al][3]}, {sb[al][4], sb[al][5]}};
    const df::DF alpha{sb[al][6], sb[al][7]}, nrm{sb[al][8], sb[al][9]};
    for (int j = 0; j < 16; ++j) {
      const int pl = ph * 16 + j;
      df::DF v[kPlanes] = {df::of(0.0f), df::of(0.0f), df::of(0.0f), df::of(0.0f), df::of(0.0f)};
      if (kind >= 0 && pc * 32 + pl < n_grid) {
        df::DF x[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) x[i] = df::sub(df::DF{sx[pl][2 * i], sx[pl][2 * i + 1]}, cen[i]);
        const df::DF r2 = df::add(df::add(df::mul(x[0], x[0]), df::mul(x[1], x[1])), df::mul(x[2], x[2]));
        const df::DF e = df::mul(nrm, df::exp_df(df::neg(df::mul(alpha, r2))));
        df::DF P = df::of(1.0f), dP[3] = {df::of(0.0f), df::of(0.0f), df::of(0.0f)};
        int l = 0;
        if (kind == 1) {
          l = 1;
          P = x[comp];
          dP[comp] = df::of(1.0f);
        } else if (kind == 2) {
          l = 2;
          if (comp <= 2) {
            const int i0 = comp == 1 ? 1 : 0, i1 = comp == 0 ? 1 : 2;
            P = df::mul(x[i0], x[i1]);
            dP[i0] = x[i1];
            dP[i1] = x[i0];
          } else if (comp == 3) {
            P = df::sub(df::mul(x[0], x[0]), df::mul(x[1], x[1]));
            dP[0] = df::mul(x[0], 2.0f);
            dP[1] = df::mul(x[1], -2.0f);
          } else {
            P = df::sub(df::mul(df::mul(x[2], x[2]), 2.0f), df::add(df::mul(x[0], x[0]), df::mul(x[1], x[1])));
            dP[0] = df::mul(x[0], -2.0f);
            dP[1] = df::mul(x[1], -2.0f);
            dP[2] = df::mul(x[2], 4.0f);
          }
        }
        const df::DF Pe = df::mul(P, e);
        const df::DF a2 = df::mul(alpha, 2.0f);
        v[T_PHI] = Pe;
#pragma unroll
        for (int i = 0; i < 3; ++i) v[T_DX + i] = df::sub(df::mul(dP[i], e), df::mul(df::mul(a2, x[i]), Pe));
        const df::DF lapf = df::sub(df::mul(df::mul(df::mul(alpha, alpha), r2), 4.0f),
                                    df::mul(alpha, (float)(6 + 4 * l)));
        v[T_LAP] = df::mul(lapf, Pe);
      }
#pragma unroll
      for (int t = 0; t < kPlanes; ++t) {
        const df::DF x = df::norm(v[t]);
        S[((size_t)t * 32 + pl) * 128 + al] = make_float2(x.s, x.c);
      }
    }
  }
  __syncthreads();
  // Phase 2a/b: AO-major rows (thread = AO row; the two halves of the CTA take alternate planes).
  {
    const int row = tid & 127;
    for (int t = tid >> 7; t < kPlanes; t += 2) {
      df::DF v[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const float2 x = S[((size_t)t * 32 + k) * 128 + row];
        v[k] = df::DF{x.x, x.y};
      }
      if (t < 4) store_row3_df(av + av_set(atile, t, pc, npc) * 3 * (umma::kBlockBytes / 4), row, v);
      float *afb = af + af_block(atile, t, pc, npc) * (umma::kBlockBytes / 4);
#pragma unroll
      for (int k4 = 0; k4 < 8; ++k4) {
        const uint32_t off = umma::kblock_off(row, 4 * k4) / 4;
        *(float4 *)(afb + off) = make_float4(v[4 * k4].s, v[4 * k4 + 1].s, v[4 * k4 + 2].s, v[4 * k4 + 3].s);
        *(float4 *)(afb + umma::kBlockBytes / 4 + off) =
            make_float4(v[4 * k4].c, v[4 * k4 + 1].c, v[4 * k4 + 2].c, v[4 * k4 + 3].c);
      }
    }
  }
  // Phase 2c: point-major TF32 pairs (warp = one point, plane and 32-AO chunk; lane = AO).
  {
    const int warp = tid >> 5, lane = tid & 31;
    const int nkc = ldk / 32;
    for (int u = warp; u < kPlanes * 32 * 4; u += kBuildThreads / 32) {
      const int t = u / 128, pl = (u / 4) % 32, kcl = u % 4;
      const float2 x = S[((size_t)t * 32 + pl) * 128 + kcl * 32 + lane];
      float hi, lo;
      split_tf32_df(df::DF{x.x, x.y}, hi, lo);
      const int64_t p = pc * 32 + pl;
      float *b = (float *)((char *)pm + pm_block(p / 128, t, atile * 4 + kcl, nkc) * umma::kBlockBytes);
      const uint32_t off = umma::kblock_off((int)(p % 128), lane) / 4;
      b[off] = hi;
      b[umma::kBlockBytes / 4 + off] = lo;
    }
  }
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
    if (basis != nullptr) {  // all three layouts in one pass, the sets split in place
      static bool attr = false;
      if (!attr) {
        e = cudaFuncSetAttribute(build_tables_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kBuildSmem);
        if (e != cudaSuccess) return e;
        attr = true;
      }
      build_tables_df_kernel<<<(unsigned)((size_t)(ldk / 128) * (np / 32)), kBuildThreads, kBuildSmem, st>>>(
          basis, coords, w, n_grid, n_ao, np, ldk, pm, av, af, wout);
      return cudaGetLastError();
    }
    const size_t total = (size_t)np * ldk;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    pack_tables_kernel<<<blocks, 256, 0, st>>>(ao, grad_ao, grad2_ao, w, n_grid, n_ao, np, ldk, pm, av, af, wout);
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
