// reduce.cu - reductions and small assembly kernels of the XC path.
#include "common.cuh"
#include "kernels.cuh"

namespace gdft {

namespace {

__device__ __forceinline__ double abs_clip(double x, double t) { return fabs(x) > t ? x : 0.0; }

// Kahan-compensated FP64 sum of the per-block energy partials (functional.py:342).
__global__ void energy_reduce_kernel(const double *__restrict__ part, int n, double *__restrict__ out) {
  __shared__ double hs[256], hc[256];
  Kahan k{0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) k.add(part[i]);
  hs[threadIdx.x] = k.s;
  hc[threadIdx.x] = k.c;
  __syncthreads();
  if (threadIdx.x == 0) {
    Kahan t{0.0, 0.0};
    for (int i = 0; i < (int)blockDim.x; ++i) {
      t.add(hs[i]);
      t.add(-hc[i]);
    }
    out[0] = t.s;
  }
}

// Sum of the split-K partial V tiles in a fixed order (deterministic).
__global__ void vxc_reduce_kernel(const double *__restrict__ part, int nsplit, size_t total,
                                  double *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; ++k) s += part[(size_t)k * total + i];
  out[i] = s;
}

__global__ void feat_to_ref_kernel(const double *__restrict__ feat, int64_t n_grid, int64_t np, double *rho,
                                   double *grad_rho, double *lapl, double *tau) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_grid) return;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const double *f = feat + (size_t)s * kFeat * np;
    if (rho) rho[2 * p + s] = f[F_RHO * np + p];
    if (grad_rho) {
      grad_rho[6 * p + 3 * s + 0] = f[F_GX * np + p];
      grad_rho[6 * p + 3 * s + 1] = f[F_GY * np + p];
      grad_rho[6 * p + 3 * s + 2] = f[F_GZ * np + p];
    }
    if (lapl) lapl[2 * p + s] = f[F_LAP * np + p];
    if (tau) tau[2 * p + s] = f[F_TAU * np + p];
  }
}

// predict's Fock assembly (train.py:147-163).
__global__ void fock_kernel(int n, const double *__restrict__ h1e, const double *__restrict__ vj,
                            const double *__restrict__ vxc, double clip, double *__restrict__ fock) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nn = (size_t)n * n;
  if (i >= 2 * nn) return;
  const int s = (int)(i / nn);
  const int a = (int)((i % nn) / n), b = (int)(i % n);
  const double gab = abs_clip((h1e[(size_t)a * n + b] + vj[(size_t)a * n + b]) + vxc[i], clip);
  const double gba = abs_clip((h1e[(size_t)b * n + a] + vj[(size_t)b * n + a]) + vxc[s * nn + (size_t)b * n + a], clip);
  fock[i] = abs_clip(0.5 * (gab + gba), clip);
}

// J_pq = sum_rt (pq|rt) (D_a + D_b)_rt, one warp per (p, q) (molecule.py:783-811).
__global__ void coulomb_kernel(int n, const double *__restrict__ eri, const double *__restrict__ rdm1,
                               double *__restrict__ vj) {
  const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const size_t nn = (size_t)n * n;
  if (warp >= nn) return;
  const double *row = eri + warp * nn;
  double s = 0.0;
  for (size_t k = lane; k < nn; k += 32) s = fma(row[k], rdm1[k] + rdm1[nn + k], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) vj[warp] = s;
}

// E_nuc + tr(D h1e) + 1/2 tr(D J) (molecule.py:694-781).
__global__ void nonxc_kernel(int n, const double *__restrict__ rdm1, const double *__restrict__ h1e,
                             const double *__restrict__ vj, double enuc, double *__restrict__ out) {
  __shared__ double sh[256], sj[256];
  const size_t nn = (size_t)n * n;
  double a = 0.0, b = 0.0;
  for (size_t k = threadIdx.x; k < nn; k += blockDim.x) {
    const double d = rdm1[k] + rdm1[nn + k];
    a = fma(d, h1e[k], a);
    b = fma(d, vj[k], b);
  }
  sh[threadIdx.x] = a;
  sj[threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sh[threadIdx.x] += sh[threadIdx.x + o];
      sj[threadIdx.x] += sj[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = enuc + sh[0] + sj[0] / 2.0;
}

// Functional.xc_energy on given densities (functional.py:219-253, :316-342).
__global__ void integrate_kernel(int64_t n_grid, int n_cols, gdft_functional fn, const double *__restrict__ dens,
                                 const double *__restrict__ w, double *__restrict__ part) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double e_r = 0.0;
  if (p < n_grid) {
    double exc = 0.0;
    for (int f = 0; f < n_cols; ++f) {
      const double c = fn.n_coeffs == 1 ? fn.coeffs[0] : fn.coeffs[f];
      exc = f == 0 ? c * dens[(size_t)p * n_cols + f] : exc + c * dens[(size_t)p * n_cols + f];
    }
    exc = abs_clip(exc, fn.clip);
    e_r = abs_clip(w[p], fn.clip) * abs_clip(exc, fn.clip);
  }
  __shared__ double red[8];
  double v = e_r;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

// (2, 6, n_grid) -> [2][6][np] (padded points get zero potentials).
__global__ void pad_potentials_kernel(const double *__restrict__ pot, int64_t n_grid, int64_t np,
                                      double *__restrict__ coef) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
#pragma unroll
  for (int k = 0; k < 2 * kFeat; ++k) coef[(size_t)k * np + p] = p < n_grid ? pot[(size_t)k * n_grid + p] : 0.0;
}

}  // namespace

cudaError_t launch_pad_potentials(const double *pot, int64_t n_grid, int64_t np, double *coef, cudaStream_t st) {
  pad_potentials_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(pot, n_grid, np, coef);
  return cudaGetLastError();
}

int integrate_blocks(int64_t n_grid) { return (int)((n_grid + 255) / 256); }

cudaError_t launch_integrate(int64_t n_grid, int n_cols, const gdft_functional &fn, const double *dens,
                             const double *w, double *epart, cudaStream_t st) {
  integrate_kernel<<<integrate_blocks(n_grid), 256, 0, st>>>(n_grid, n_cols, fn, dens, w, epart);
  return cudaGetLastError();
}

// Move a per-call error word into a persistent one (the first code recorded wins) and clear it.
__global__ void err_fold_kernel(int *__restrict__ dst, int *__restrict__ src) {
  const int e = *src;
  if (e != 0) atomicCAS(dst, 0, e);
  *src = 0;
}

cudaError_t launch_err_fold(int *dst, int *src, cudaStream_t st) {
  err_fold_kernel<<<1, 1, 0, st>>>(dst, src);
  return cudaGetLastError();
}

cudaError_t launch_energy_reduce(const double *epart, int n, double *exc, cudaStream_t st) {
  energy_reduce_kernel<<<1, 256, 0, st>>>(epart, n, exc);
  return cudaGetLastError();
}

cudaError_t launch_vxc_reduce(const double *vpart, int nsplit, int n_ao, double *vxc, cudaStream_t st) {
  const size_t total = (size_t)2 * n_ao * n_ao;
  vxc_reduce_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(vpart, nsplit, total, vxc);
  return cudaGetLastError();
}

cudaError_t launch_feat_to_reference(const double *feat, int64_t n_grid, int64_t np, double *rho, double *grad_rho,
                                     double *lapl, double *tau, cudaStream_t st) {
  feat_to_ref_kernel<<<(unsigned)((n_grid + 255) / 256), 256, 0, st>>>(feat, n_grid, np, rho, grad_rho, lapl, tau);
  return cudaGetLastError();
}

cudaError_t launch_fock(int n_ao, const double *h1e, const double *vj, const double *vxc, double clip, double *fock,
                        cudaStream_t st) {
  const size_t total = (size_t)2 * n_ao * n_ao;
  fock_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(n_ao, h1e, vj, vxc, clip, fock);
  return cudaGetLastError();
}

cudaError_t launch_coulomb(int n_ao, const double *eri, const double *rdm1, const double *h1e, double enuc,
                           double *vj, double *enonxc, cudaStream_t st) {
  const size_t nn = (size_t)n_ao * n_ao;
  coulomb_kernel<<<(unsigned)((nn * 32 + 255) / 256), 256, 0, st>>>(n_ao, eri, rdm1, vj);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (enonxc != nullptr) nonxc_kernel<<<1, 256, 0, st>>>(n_ao, rdm1, h1e, vj, enuc, enonxc);
  return cudaGetLastError();
}

}  // namespace gdft
