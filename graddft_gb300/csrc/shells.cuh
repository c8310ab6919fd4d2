// shells.cuh - contracted Gaussian shells evaluated on the grid (the device
// half of numint.eval_ao, interface/pyscf.py:849-852, and ao_grads,
// interface/pyscf.py:677-705).
//
//   phi(r) = E0(r2) * A(d),  d = r - R_shell,  r2 = |d|^2,
//   E0 = sum_p C_p exp(-alpha_p r2),  E1 = sum_p -2 alpha_p C_p exp(..),  E2 = sum_p 4 alpha_p^2 C_p exp(..),
//   A(d) = sum_(i,j,k) t_ijk x^i y^j z^k  (the component's row of cartesian coefficients, degree l),
// so that d_x phi = A_x E0 + A x E1 and d_xx phi = A_xx E0 + 2 A_x x E1 + A (E1 + x^2 E2).
//
// Work layout: a CTA evaluates a tile of 32 grid points x 64 AOs into shared
// memory, then a sink writes the tile to its destination with the AO index
// fastest (coalesced).  In the evaluation phase the lanes of a warp are the 32
// points and each warp takes whole shells, so the angular momentum and the
// primitive count are uniform across the warp (no divergence) and each
// exponential is computed once per point and shell, shared by all of the
// shell's contractions and components.
#pragma once

#include "common.cuh"

namespace gdft {

constexpr int kMaxShellL = 6;
constexpr int kShellCols = 8;  // l, nprim, exp offset, coef offset, first AO, ncomp, nctr, row offset
constexpr int kTilePts = 32;
constexpr int kTileAo = 64;
constexpr int kTileLd = kTileAo + 1;  // padded row: lanes (points) land in different banks
constexpr int kTileThreads = 256;
constexpr int kCtrGroup = 4;  // contractions whose radial sums are carried together

struct ShellView {
  const int32_t *shell;  // (n_shell, 8)
  const double *centre;  // (n_shell, 3)
  const double *exps;
  const double *coef;    // shell s, contraction c, primitive p at coef offset + c * nprim + p
  const int32_t *ao;     // (n_ao, 4): shell, contraction, component, 0
  const double *trans;   // shell s, component k: ncart(l) values at row offset + k * ncart(l)
  int n_shell, n_ao;
  int64_t n_prim, n_coef, n_trans;
};

__device__ __forceinline__ double nan_value() { return __longlong_as_double(0x7ff8000000000000LL); }

namespace shells_detail {

// The angular polynomial and its first and diagonal second derivatives.
template <int L>
__device__ __forceinline__ void poly(const double *__restrict__ t, double x, double y, double z, double P[7]) {
  double xp[L + 1], yp[L + 1], zp[L + 1];
  xp[0] = yp[0] = zp[0] = 1.0;
#pragma unroll
  for (int i = 1; i <= L; ++i) {
    xp[i] = xp[i - 1] * x;
    yp[i] = yp[i - 1] * y;
    zp[i] = zp[i - 1] * z;
  }
#pragma unroll
  for (int q = 0; q < 7; ++q) P[q] = 0.0;
  int idx = 0;
#pragma unroll
  for (int lx = L; lx >= 0; --lx) {
#pragma unroll
    for (int ly = L - lx; ly >= 0; --ly) {
      const int lz = L - lx - ly;
      const double c = t[idx++];
      // the lanes of a warp evaluate the same AO row (warp-uniform branch): solid-harmonic
      // rows are mostly zero, and a zero term adds nothing
      if (c == 0.0) continue;
      const double X0 = xp[lx], Y0 = yp[ly], Z0 = zp[lz];
      const double X1 = lx > 0 ? lx * xp[lx > 0 ? lx - 1 : 0] : 0.0;
      const double Y1 = ly > 0 ? ly * yp[ly > 0 ? ly - 1 : 0] : 0.0;
      const double Z1 = lz > 0 ? lz * zp[lz > 0 ? lz - 1 : 0] : 0.0;
      const double X2 = lx > 1 ? lx * (lx - 1) * xp[lx > 1 ? lx - 2 : 0] : 0.0;
      const double Y2 = ly > 1 ? ly * (ly - 1) * yp[ly > 1 ? ly - 2 : 0] : 0.0;
      const double Z2 = lz > 1 ? lz * (lz - 1) * zp[lz > 1 ? lz - 2 : 0] : 0.0;
      const double YZ = Y0 * Z0;
      P[0] = fma(c, X0 * YZ, P[0]);
      P[1] = fma(c, X1 * YZ, P[1]);
      P[2] = fma(c, X0 * Y1 * Z0, P[2]);
      P[3] = fma(c, X0 * Y0 * Z1, P[3]);
      P[4] = fma(c, X2 * YZ, P[4]);
      P[5] = fma(c, X0 * Y2 * Z0, P[5]);
      P[6] = fma(c, X0 * Y0 * Z2, P[6]);
    }
  }
}

__device__ __forceinline__ void poly_l(int l, const double *t, double x, double y, double z, double P[7]) {
  switch (l) {
    case 0: poly<0>(t, x, y, z, P); break;
    case 1: poly<1>(t, x, y, z, P); break;
    case 2: poly<2>(t, x, y, z, P); break;
    case 3: poly<3>(t, x, y, z, P); break;
    case 4: poly<4>(t, x, y, z, P); break;
    case 5: poly<5>(t, x, y, z, P); break;
    default: poly<6>(t, x, y, z, P); break;
  }
}

// A shell's table entries, checked against the table sizes.
struct ShellRec {
  int l, np, aoff, ncomp, nctr, ncart;
  int64_t poff, coff, toff;
};

__device__ __forceinline__ bool load_shell(const ShellView &B, int s, ShellRec &r) {
  if (s < 0 || s >= B.n_shell) return false;
  const int32_t *e = B.shell + (size_t)kShellCols * s;
  r.l = e[0];
  r.np = e[1];
  r.poff = e[2];
  r.coff = e[3];
  r.aoff = e[4];
  r.ncomp = e[5];
  r.nctr = e[6];
  r.toff = e[7];
  if (r.l < 0 || r.l > kMaxShellL || r.np <= 0 || r.ncomp <= 0 || r.nctr <= 0) return false;
  r.ncart = (r.l + 1) * (r.l + 2) / 2;
  return r.poff >= 0 && r.poff + r.np <= B.n_prim && r.coff >= 0 && r.coff + (int64_t)r.nctr * r.np <= B.n_coef &&
         r.toff >= 0 && r.toff + (int64_t)r.ncomp * r.ncart <= B.n_trans && r.aoff >= 0 &&
         (int64_t)r.aoff + (int64_t)r.nctr * r.ncomp <= B.n_ao;
}

}  // namespace shells_detail

// Evaluation phase: the tile [kVals][kTilePts][kTileLd] of AOs [a0, a0 + kTileAo)
// at points [p0, p0 + 32).  kVals = 7 keeps the three diagonal second
// derivatives, kVals = 5 their sum (the Laplacian).  Entries no shell covers
// stay NaN; AOs at or beyond n_ao stay NaN too (sinks write zero padding there).
template <int kVals>
__device__ __forceinline__ void eval_tile(const ShellView &B, const double *__restrict__ coords, int64_t n_grid,
                                          int64_t p0, int a0, double *tile) {
  using namespace shells_detail;
  for (int i = threadIdx.x; i < kVals * kTilePts * kTileLd; i += blockDim.x) tile[i] = nan_value();
  __syncthreads();
  if (a0 >= B.n_ao) return;
  const int a1 = min(a0 + kTileAo, B.n_ao);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int64_t p = p0 + lane;
  double px = 0.0, py = 0.0, pz = 0.0;
  if (p < n_grid) {
    px = coords[3 * p + 0];
    py = coords[3 * p + 1];
    pz = coords[3 * p + 2];
  }
  const int s_lo = B.ao[4 * a0], s_hi = B.ao[4 * (a1 - 1)];
  if (s_lo < 0 || s_hi >= B.n_shell || s_hi < s_lo) return;
  for (int s = s_lo + warp; s <= s_hi; s += nwarps) {
    ShellRec r;
    if (!load_shell(B, s, r)) continue;
    const int lo = max(a0, r.aoff), hi = min(a1, r.aoff + r.nctr * r.ncomp);
    if (lo >= hi) continue;
    const double x = px - B.centre[3 * s + 0];
    const double y = py - B.centre[3 * s + 1];
    const double z = pz - B.centre[3 * s + 2];
    const double r2 = x * x + y * y + z * z;
    const double d[3] = {x, y, z};
    const int c_lo = (lo - r.aoff) / r.ncomp, c_hi = (hi - 1 - r.aoff) / r.ncomp;
    for (int cg = c_lo; cg <= c_hi; cg += kCtrGroup) {
      const int nc = min(kCtrGroup, c_hi - cg + 1);
      double E0[kCtrGroup], E1[kCtrGroup], E2[kCtrGroup];
#pragma unroll
      for (int j = 0; j < kCtrGroup; ++j) E0[j] = E1[j] = E2[j] = 0.0;
      for (int q = 0; q < r.np; ++q) {
        const double al = B.exps[r.poff + q];
        const double e = exp(-al * r2);
        const double m1 = -2.0 * al;
#pragma unroll
        for (int j = 0; j < kCtrGroup; ++j) {
          if (j < nc) {
            const double ce = B.coef[r.coff + (int64_t)(cg + j) * r.np + q] * e;
            E0[j] += ce;
            E1[j] = fma(m1, ce, E1[j]);
            E2[j] = fma(m1 * m1, ce, E2[j]);
          }
        }
      }
      for (int k = 0; k < r.ncomp; ++k) {
        double P[7];
        bool have = false;
#pragma unroll
        for (int j = 0; j < kCtrGroup; ++j) {
          const int a = r.aoff + (cg + j) * r.ncomp + k;
          if (j >= nc || a < lo || a >= hi) continue;
          if (!have) {
            poly_l(r.l, B.trans + r.toff + (int64_t)k * r.ncart, x, y, z, P);
            have = true;
          }
          double v[7];
          v[0] = P[0] * E0[j];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            v[1 + i] = fma(P[0] * d[i], E1[j], P[1 + i] * E0[j]);
            v[4 + i] = P[4 + i] * E0[j] + 2.0 * P[1 + i] * d[i] * E1[j] + P[0] * fma(d[i] * d[i], E2[j], E1[j]);
          }
          double *t = tile + (size_t)lane * kTileLd + (a - a0);
#pragma unroll
          for (int q = 0; q < 4; ++q) t[q * kTilePts * kTileLd] = v[q];
          if (kVals == 7) {
#pragma unroll
            for (int q = 4; q < 7; ++q) t[q * kTilePts * kTileLd] = v[q];
          } else {
            t[4 * kTilePts * kTileLd] = (v[4] + v[5]) + v[6];
          }
        }
      }
    }
  }
}

// One tile per CTA: blockIdx.x = 32-point group, blockIdx.y = 64-AO chunk of
// the sink's AO extent.  The sink is called after the whole tile is written.
template <int kVals, class Sink>
__global__ void __launch_bounds__(kTileThreads) eval_shells_tile_kernel(ShellView B, const double *__restrict__ coords,
                                                                        int64_t n_grid, Sink sink) {
  extern __shared__ double tile[];
  const int64_t p0 = (int64_t)blockIdx.x * kTilePts;
  const int a0 = blockIdx.y * kTileAo;
  eval_tile<kVals>(B, coords, n_grid, p0, a0, tile);
  __syncthreads();
  for (int i = threadIdx.x; i < kTilePts * kTileAo; i += blockDim.x) {
    const int pt = i / kTileAo, aa = i % kTileAo;
    sink(tile, pt * kTileLd + aa, kTilePts * kTileLd, p0 + pt, a0 + aa);
  }
}

constexpr size_t tile_smem_bytes(int vals) { return (size_t)vals * kTilePts * kTileLd * sizeof(double); }

// Launch over (points rounded to 32) x (AO extent rounded to 64).
template <int kVals, class Sink>
cudaError_t launch_shell_tiles(const ShellView &B, const double *coords, int64_t n_grid, int64_t n_points,
                               int ao_extent, const Sink &sink, cudaStream_t st) {
  const size_t smem = tile_smem_bytes(kVals);
  cudaError_t e = cudaFuncSetAttribute(eval_shells_tile_kernel<kVals, Sink>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const dim3 grid((unsigned)((n_points + kTilePts - 1) / kTilePts), (unsigned)((ao_extent + kTileAo - 1) / kTileAo));
  eval_shells_tile_kernel<kVals, Sink><<<grid, kTileThreads, smem, st>>>(B, coords, n_grid, sink);
  return cudaGetLastError();
}

}  // namespace gdft
