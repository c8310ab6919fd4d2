// dens_f64.cu - plain FP64 form of the density contraction.
//
// For a tile of 32 grid points and each spin it forms X_t = T_t D_sigma for the
// four AO planes T_t in {phi, d_x phi, d_y phi, d_z phi} (64 output columns at
// a time, K = n_ao) and reduces each row against the AO planes in the
// epilogue, so X never leaves the SM:
//   rho            = sum_b X_phi[b] phi_b                       (molecule.py:409)
//   grad_j rho     = 2 sum_b X_phi[b] d_j phi_b                 (molecule.py:440)
//   lapl rho       = 2 sum_j sum_b X_dj[b] d_j phi_b
//                    + 2 sum_b X_phi[b] lap phi_b               (molecule.py:472-474)
//   tau            = 1/2 sum_j sum_b X_dj[b] d_j phi_b          (molecule.py:502)
// Output feat[spin][6][np].
#include "common.cuh"
#include "kernels.cuh"

namespace gdft {

namespace {

constexpr int BP = 32;   // points per block
constexpr int BN = 64;   // output columns per chunk
constexpr int BK = 16;   // reduction step
constexpr int NT = 256;  // threads: 32 points x 8 column lanes

__global__ void __launch_bounds__(NT) dens_f64_kernel(const double *__restrict__ tab, int64_t np, int ld, int n,
                                                      const double *__restrict__ D, double *__restrict__ feat) {
  __shared__ double As[4][BP][BK + 1];
  __shared__ double Bs[BK][BN];
  const size_t pe = (size_t)np * ld;
  const int tid = threadIdx.x;
  const int pt = tid >> 3;  // point within the tile
  const int cg = tid & 7;   // column lane: columns c0 + j*8 + cg
  const int64_t p0 = (int64_t)blockIdx.x * BP;
  const int64_t p = p0 + pt;

  for (int s = 0; s < 2; ++s) {
    const double *Ds = D + (size_t)s * n * n;
    double f_rho = 0.0, f_g[3] = {0.0, 0.0, 0.0}, f_lp = 0.0, f_kin = 0.0;
    for (int c0 = 0; c0 < n; c0 += BN) {
      double acc[4][8];
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[t][j] = 0.0;
      for (int k0 = 0; k0 < n; k0 += BK) {
#pragma unroll
        for (int i = 0; i < (4 * BP * BK) / NT; ++i) {
          const int idx = tid + i * NT;
          const int t = idx / (BP * BK);
          const int rem = idx % (BP * BK);
          const int r = rem / BK, kk = rem % BK;
          As[t][r][kk] = tab[(size_t)t * pe + (size_t)(p0 + r) * ld + (k0 + kk)];
        }
#pragma unroll
        for (int i = 0; i < (BK * BN) / NT; ++i) {
          const int idx = tid + i * NT;
          const int kk = idx / BN, cc = idx % BN;
          const int k = k0 + kk, c = c0 + cc;
          Bs[kk][cc] = (k < n && c < n) ? Ds[(size_t)k * n + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
          double a[4], b[8];
#pragma unroll
          for (int t = 0; t < 4; ++t) a[t] = As[t][pt][kk];
#pragma unroll
          for (int j = 0; j < 8; ++j) b[j] = Bs[kk][j * 8 + cg];
#pragma unroll
          for (int t = 0; t < 4; ++t)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[t][j] = fma(a[t], b[j], acc[t][j]);
        }
        __syncthreads();
      }
      // Epilogue: row reductions against the AO planes.
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = c0 + j * 8 + cg;
        if (c < n) {
          const size_t o = (size_t)p * ld + c;
          const double phi = tab[o];
          const double dx = tab[pe + o], dy = tab[2 * pe + o], dz = tab[3 * pe + o];
          const double lp = tab[4 * pe + o];
          f_rho = fma(acc[0][j], phi, f_rho);
          f_g[0] = fma(acc[0][j], dx, f_g[0]);
          f_g[1] = fma(acc[0][j], dy, f_g[1]);
          f_g[2] = fma(acc[0][j], dz, f_g[2]);
          f_lp = fma(acc[0][j], lp, f_lp);
          f_kin = fma(acc[1][j], dx, f_kin);
          f_kin = fma(acc[2][j], dy, f_kin);
          f_kin = fma(acc[3][j], dz, f_kin);
        }
      }
    }
    // Reduce over the 8 column lanes of the point.
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      f_rho += __shfl_xor_sync(0xffffffffu, f_rho, o);
      f_g[0] += __shfl_xor_sync(0xffffffffu, f_g[0], o);
      f_g[1] += __shfl_xor_sync(0xffffffffu, f_g[1], o);
      f_g[2] += __shfl_xor_sync(0xffffffffu, f_g[2], o);
      f_lp += __shfl_xor_sync(0xffffffffu, f_lp, o);
      f_kin += __shfl_xor_sync(0xffffffffu, f_kin, o);
    }
    if (cg == 0) {
      double *fs = feat + (size_t)s * kFeat * np;
      fs[F_RHO * np + p] = f_rho;
      fs[F_GX * np + p] = 2.0 * f_g[0];
      fs[F_GY * np + p] = 2.0 * f_g[1];
      fs[F_GZ * np + p] = 2.0 * f_g[2];
      fs[F_LAP * np + p] = 2.0 * f_kin + 2.0 * f_lp;
      fs[F_TAU * np + p] = 0.5 * f_kin;
    }
  }
}

}  // namespace

cudaError_t launch_dens_f64(const double *tab, int64_t np, int ld, int n_ao, const double *rdm1, double *feat,
                            cudaStream_t st) {
  const int64_t blocks = np / BP;
  dens_f64_kernel<<<(unsigned)blocks, NT, 0, st>>>(tab, np, ld, n_ao, rdm1, feat);
  return cudaGetLastError();
}

}  // namespace gdft
