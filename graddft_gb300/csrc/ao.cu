// ao.cu - filling the resident AO tables of a molecule.
//
// Resident layout: five FP64 planes of (np, ld) row-major: phi, d_x phi,
// d_y phi, d_z phi and the Laplacian sum_i d_i^2 phi (the only combination of
// grad_n_ao[2] that lapl_density uses, molecule.py:472-474), zero-padded to
// np rows (multiple of 128) and ld columns (multiple of 32).
#include "common.cuh"
#include "kernels.cuh"
#include "shells.cuh"

namespace gdft {

namespace {

// Reference layouts -> planes.  One thread per (point, ao).
__global__ void load_tables_kernel(const double *__restrict__ ao, const double *__restrict__ grad_ao,
                                   const double *__restrict__ grad2_ao, const double *__restrict__ w,
                                   int64_t n_grid, int n_ao, int64_t np, int ld, double *__restrict__ tab,
                                   double *__restrict__ wout) {
  const size_t pe = (size_t)np * ld;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= pe) return;
  const int64_t p = (int64_t)(idx / ld);
  const int a = (int)(idx % ld);
  double v[kPlanes] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (p < n_grid && a < n_ao) {
    const size_t r = (size_t)p * n_ao + a;
    v[T_PHI] = ao[r];
    v[T_DX] = grad_ao[3 * r + 0];
    v[T_DY] = grad_ao[3 * r + 1];
    v[T_DZ] = grad_ao[3 * r + 2];
    if (grad2_ao != nullptr) v[T_LAP] = (grad2_ao[3 * r + 0] + grad2_ao[3 * r + 1]) + grad2_ao[3 * r + 2];
  }
#pragma unroll
  for (int k = 0; k < kPlanes; ++k) tab[k * pe + idx] = v[k];
  if (a == 0) wout[p] = p < n_grid ? w[p] : 0.0;
}

// Synthetic Gaussian basis evaluated on the grid (phi = N P(x,y,z) exp(-alpha r^2)).
__global__ void eval_basis_kernel(const double *__restrict__ basis, const double *__restrict__ coords,
                                  const double *__restrict__ w, int64_t n_grid, int n_ao, int64_t np, int ld,
                                  double *__restrict__ tab, double *__restrict__ wout) {
  const size_t pe = (size_t)np * ld;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= pe) return;
  const int64_t p = (int64_t)(idx / ld);
  const int a = (int)(idx % ld);
  double v[kPlanes] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (p < n_grid && a < n_ao) {
    const double *b = basis + 8 * (size_t)a;
    const double x = coords[3 * p + 0] - b[0];
    const double y = coords[3 * p + 1] - b[1];
    const double z = coords[3 * p + 2] - b[2];
    const double al = b[3];
    const double ex = b[4] * exp(-al * (x * x + y * y + z * z));
    const int kind = (int)b[5];
    const int comp = (int)b[6];
    double P = 1.0, dP[3] = {0.0, 0.0, 0.0}, d2P[3] = {0.0, 0.0, 0.0};
    const double xyz[3] = {x, y, z};
    if (kind == 1) {
      P = xyz[comp];
      dP[comp] = 1.0;
    } else if (kind == 2) {
      if (comp <= 2) {
        const int i0 = comp == 1 ? 1 : 0;
        const int i1 = comp == 0 ? 1 : 2;
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
    double lap[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      v[T_DX + i] = (dP[i] - 2 * al * xyz[i] * P) * ex;
      lap[i] = (d2P[i] - 2 * al * P - 4 * al * xyz[i] * dP[i] + 4 * al * al * xyz[i] * xyz[i] * P) * ex;
    }
    v[T_LAP] = (lap[0] + lap[1]) + lap[2];
  }
#pragma unroll
  for (int k = 0; k < kPlanes; ++k) tab[k * pe + idx] = v[k];
  if (a == 0) wout[p] = p < n_grid ? w[p] : 0.0;
}

// Sinks of the shell tiles (shells.cuh).  Reference layouts: ao (grid, ao),
// grad (grid, ao, 3), grad2 (grid, ao, 3) diagonal second derivatives.
struct RefSink {
  double *ao, *g1, *g2;
  int64_t n_grid;
  int n_ao, deriv;
  __device__ void operator()(const double *tile, int t, int ps, int64_t p, int a) const {
    if (p >= n_grid || a >= n_ao) return;
    const size_t r = (size_t)p * n_ao + a;
    ao[r] = tile[t];
    if (deriv >= 1)
      for (int i = 0; i < 3; ++i) g1[3 * r + i] = tile[(1 + i) * ps + t];
    if (deriv >= 2)
      for (int i = 0; i < 3; ++i) g2[3 * r + i] = tile[(4 + i) * ps + t];
  }
};

// The FP64 form's resident planes (zero padding beyond n_grid and n_ao).
struct PlaneSink {
  double *tab;
  const double *w;
  double *wout;
  int64_t n_grid;
  size_t pe;
  int n_ao, ld;
  __device__ void operator()(const double *tile, int t, int ps, int64_t p, int a) const {
    if (a >= ld) return;
    const bool live = p < n_grid && a < n_ao;
    const size_t o = (size_t)p * ld + a;
#pragma unroll
    for (int q = 0; q < kPlanes; ++q) tab[q * pe + o] = live ? tile[q * ps + t] : 0.0;
    if (a == 0) wout[p] = p < n_grid ? w[p] : 0.0;
  }
};

}  // namespace

cudaError_t launch_eval_ao(const ShellView &B, const double *coords, int64_t n_grid, int deriv, double *ao,
                           double *g1, double *g2, cudaStream_t st) {
  return launch_shell_tiles<7>(B, coords, n_grid, n_grid, B.n_ao, RefSink{ao, g1, g2, n_grid, B.n_ao, deriv}, st);
}

cudaError_t launch_eval_shell_tables(const ShellView &B, const double *coords, const double *w, int64_t n_grid,
                                     int64_t np, int ld, double *tab, double *wout, cudaStream_t st) {
  return launch_shell_tiles<kPlanes>(B, coords, n_grid, np, ld,
                                     PlaneSink{tab, w, wout, n_grid, (size_t)np * ld, B.n_ao, ld}, st);
}

cudaError_t launch_load_tables(const double *ao, const double *grad_ao, const double *grad2_ao, const double *w,
                               int64_t n_grid, int n_ao, int64_t np, int ld, double *tab, double *wout,
                               cudaStream_t st) {
  const size_t total = (size_t)np * ld;
  const int bs = 256;
  load_tables_kernel<<<(unsigned)((total + bs - 1) / bs), bs, 0, st>>>(ao, grad_ao, grad2_ao, w, n_grid, n_ao, np,
                                                                       ld, tab, wout);
  return cudaGetLastError();
}

cudaError_t launch_eval_basis(const double *basis, const double *coords, const double *w, int64_t n_grid, int n_ao,
                              int64_t np, int ld, double *tab, double *wout, cudaStream_t st) {
  const size_t total = (size_t)np * ld;
  const int bs = 256;
  eval_basis_kernel<<<(unsigned)((total + bs - 1) / bs), bs, 0, st>>>(basis, coords, w, n_grid, n_ao, np, ld, tab,
                                                                      wout);
  return cudaGetLastError();
}

}  // namespace gdft
