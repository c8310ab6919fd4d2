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

// Contracted shells -> reference layouts: ao (grid, ao), grad (grid, ao, 3),
// grad2 (grid, ao, 3) diagonal second derivatives.  One thread per (point, AO),
// AO fastest, so a warp writes a contiguous run.  An AO whose table entries are
// out of range gets NaN.
__global__ void eval_ao_kernel(ShellView B, const double *__restrict__ coords, int64_t n_grid, int deriv,
                               double *__restrict__ ao, double *__restrict__ g1, double *__restrict__ g2) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n_grid * B.n_ao) return;
  const int64_t p = (int64_t)(idx / B.n_ao);
  const int a = (int)(idx % B.n_ao);
  double v[7];
  if (!shell_ao_eval(B, coords[3 * p], coords[3 * p + 1], coords[3 * p + 2], a, v))
    for (int q = 0; q < 7; ++q) v[q] = __longlong_as_double(0x7ff8000000000000LL);
  ao[idx] = v[0];
  if (deriv >= 1)
    for (int i = 0; i < 3; ++i) g1[3 * idx + i] = v[1 + i];
  if (deriv >= 2)
    for (int i = 0; i < 3; ++i) g2[3 * idx + i] = v[4 + i];
}

// Contracted shells -> the FP64 form's resident planes.
__global__ void eval_shell_tables_kernel(ShellView B, const double *__restrict__ coords,
                                         const double *__restrict__ w, int64_t n_grid, int64_t np, int ld,
                                         double *__restrict__ tab, double *__restrict__ wout) {
  const size_t pe = (size_t)np * ld;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= pe) return;
  const int64_t p = (int64_t)(idx / ld);
  const int a = (int)(idx % ld);
  double v[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (p < n_grid && a < B.n_ao &&
      !shell_ao_eval(B, coords[3 * p], coords[3 * p + 1], coords[3 * p + 2], a, v))
    for (int q = 0; q < 7; ++q) v[q] = __longlong_as_double(0x7ff8000000000000LL);
  tab[T_PHI * pe + idx] = v[0];
  tab[T_DX * pe + idx] = v[1];
  tab[T_DY * pe + idx] = v[2];
  tab[T_DZ * pe + idx] = v[3];
  tab[T_LAP * pe + idx] = (v[4] + v[5]) + v[6];
  if (a == 0) wout[p] = p < n_grid ? w[p] : 0.0;
}

}  // namespace

cudaError_t launch_eval_ao(const ShellView &B, const double *coords, int64_t n_grid, int deriv, double *ao,
                           double *g1, double *g2, cudaStream_t st) {
  const size_t total = (size_t)n_grid * B.n_ao;
  eval_ao_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(B, coords, n_grid, deriv, ao, g1, g2);
  return cudaGetLastError();
}

cudaError_t launch_eval_shell_tables(const ShellView &B, const double *coords, const double *w, int64_t n_grid,
                                     int64_t np, int ld, double *tab, double *wout, cudaStream_t st) {
  const size_t total = (size_t)np * ld;
  eval_shell_tables_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(B, coords, w, n_grid, np, ld, tab,
                                                                             wout);
  return cudaGetLastError();
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
