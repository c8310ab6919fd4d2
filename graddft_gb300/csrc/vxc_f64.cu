// vxc_f64.cu - plain FP64 form of the V_xc contraction.
//
// V_sigma[a][b] = sum_r phi_ra Qa_sigma[r][b] + sum_j sum_r d_j phi_ra Qk_sigma[r][b] d_j...
// written as one contraction over the stacked operand pairs
//   P_0 = phi,   Q_0 = C_RHO phi + sum_j C_GJ d_j phi + C_LAP lap phi
//   P_j = d_j phi, Q_j = C_KIN d_j phi                         (j = x, y, z)
// so V_sigma = sum_t P_t^T Q_t (the transpose of the density contraction that
// jax.value_and_grad builds at train.py:86).  The Q operands are formed in
// shared memory from the AO planes and the per-point adjoint coefficients.
// Each block computes a 64 x 64 tile of both spins over one slice of the grid
// (split-K); the slices are summed in a fixed order by reduce.cu.
#include "common.cuh"
#include "kernels.cuh"

namespace gdft {

namespace {

constexpr int BT = 64;   // tile edge (a and b)
constexpr int BK = 8;    // grid points per step
constexpr int NT = 256;

__global__ void __launch_bounds__(NT) vxc_f64_kernel(const double *__restrict__ tab, int64_t np, int ld, int n,
                                                     const double *__restrict__ coef, int64_t chunk,
                                                     double *__restrict__ vpart) {
  __shared__ double Ps[4][BK][BT];
  __shared__ double Qs[2][4][BK][BT];
  const size_t pe = (size_t)np * ld;
  const int tid = threadIdx.x;
  const int ta = tid >> 4, tb = tid & 15;
  const int tiles_b = (n + BT - 1) / BT;
  const int a0 = (blockIdx.x / tiles_b) * BT;
  const int b0 = (blockIdx.x % tiles_b) * BT;
  const int64_t r_begin = (int64_t)blockIdx.y * chunk;
  const int64_t r_end = r_begin + chunk < np ? r_begin + chunk : np;

  double acc[2][4][4];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[s][i][j] = 0.0;

  for (int64_t r0 = r_begin; r0 < r_end; r0 += BK) {
    // a-side operands.
#pragma unroll
    for (int i = 0; i < (4 * BK * BT) / NT; ++i) {
      const int idx = tid + i * NT;
      const int t = idx / (BK * BT);
      const int rem = idx % (BK * BT);
      const int r = rem / BT, aa = rem % BT;
      const int a = a0 + aa;
      Ps[t][r][aa] = (a < ld) ? tab[(size_t)t * pe + (size_t)(r0 + r) * ld + a] : 0.0;
    }
    // b-side operands, both spins.
#pragma unroll
    for (int i = 0; i < (BK * BT) / NT; ++i) {
      const int idx = tid + i * NT;
      const int r = idx / BT, bb = idx % BT;
      const int b = b0 + bb;
      const int64_t pr = r0 + r;
      double phi = 0.0, d[3] = {0.0, 0.0, 0.0}, lp = 0.0;
      if (b < ld) {
        const size_t o = (size_t)pr * ld + b;
        phi = tab[o];
        d[0] = tab[pe + o];
        d[1] = tab[2 * pe + o];
        d[2] = tab[3 * pe + o];
        lp = tab[4 * pe + o];
      }
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const double *cs = coef + (size_t)s * kFeat * np;
        const double cr = cs[C_RHO * np + pr], cgx = cs[C_GX * np + pr], cgy = cs[C_GY * np + pr],
                     cgz = cs[C_GZ * np + pr], cl = cs[C_LAP * np + pr], ck = cs[C_KIN * np + pr];
        Qs[s][0][r][bb] = cr * phi + cgx * d[0] + cgy * d[1] + cgz * d[2] + cl * lp;
        Qs[s][1][r][bb] = ck * d[0];
        Qs[s][2][r][bb] = ck * d[1];
        Qs[s][3][r][bb] = ck * d[2];
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < BK; ++r) {
      double pa[4][4];
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int i = 0; i < 4; ++i) pa[t][i] = Ps[t][r][ta + 16 * i];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          double qb[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) qb[j] = Qs[s][t][r][tb + 16 * j];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[s][i][j] = fma(pa[t][i], qb[j], acc[s][i][j]);
        }
      }
    }
    __syncthreads();
  }
  double *out = vpart + (size_t)blockIdx.y * 2 * n * n;
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int a = a0 + ta + 16 * i, b = b0 + tb + 16 * j;
        if (a < n && b < n) out[((size_t)s * n + a) * n + b] = acc[s][i][j];
      }
}

}  // namespace

int vxc_f64_splits(int64_t np, int n_ao) {
  const int tiles = ((n_ao + BT - 1) / BT) * ((n_ao + BT - 1) / BT);
  int64_t want = (4 * 152 + tiles - 1) / tiles;
  const int64_t max_split = np / 64 > 0 ? np / 64 : 1;
  if (want > max_split) want = max_split;
  if (want < 1) want = 1;
  return (int)want;
}

cudaError_t launch_vxc_f64(const double *tab, int64_t np, int ld, int n_ao, const double *coef, int nsplit,
                           double *vpart, cudaStream_t st) {
  const int tiles_a = (n_ao + BT - 1) / BT;
  int64_t chunk = (np + nsplit - 1) / nsplit;
  chunk = (chunk + BK - 1) / BK * BK;
  dim3 grid(tiles_a * tiles_a, nsplit);
  vxc_f64_kernel<<<grid, NT, 0, st>>>(tab, np, ld, n_ao, coef, chunk, vpart);
  return cudaGetLastError();
}

}  // namespace gdft
