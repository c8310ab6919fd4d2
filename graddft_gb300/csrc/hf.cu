// hf.cu - exact-exchange (Hartree-Fock) terms from a supplied chi tensor.
//
//   ehf[w][s][r] = -1/2 sum_c chi[r][w][s][c] (sum_a ao[r][a] D_s[a][c])      (molecule.py:507-541)
//   F_s[a][b]    = -1/2 sum_w sum_r ao[r][a] g[w][s][r] chi[r][w][s][b]       (molecule.py:545-613, the
//                  omega sum of b3lyp_hfgrads, popular_functionals.py:357-372, and dm21_hfgrads_*,
//                  functional.py:677-757)
// with g = dE_xc/d ehf.  chi keeps the reference's layout (grid, omega, spin,
// orbitals).  Both contractions run in FP64 on the tiled FP64 GEMM: X_s =
// ao D_s, then a warp per (point, spin) takes the row dot with chi; B_s =
// -1/2 sum_w g chi, then F_s = ao^T B_s with the grid split over CTAs and the
// partials summed in a fixed order.
#include "common.cuh"
#include "kernels.cuh"
#include "mlp_gemm.cuh"

namespace gdft {

namespace {

// One warp per (point, spin): ehf of every omega.
__global__ void hf_rowdot_kernel(const double *__restrict__ chi, const double *__restrict__ X, int64_t n_grid, int n,
                                 int n_omega, double *__restrict__ ehf) {
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= 2 * n_grid) return;  // whole warps leave together
  const int64_t r = gw >> 1;
  const int s = (int)(gw & 1);
  const double *x = X + ((size_t)s * n_grid + r) * n;
  for (int w = 0; w < n_omega; ++w) {
    const double *c = chi + (((size_t)r * n_omega + w) * 2 + s) * n;
    double acc = 0.0;
    for (int k = lane; k < n; k += 32) acc = fma(c[k], x[k], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) ehf[((size_t)w * 2 + s) * n_grid + r] = -0.5 * acc;
  }
}

// B[s][r][b] = -1/2 sum_w g[w][s][r] chi[r][w][s][b].
__global__ void hf_bmat_kernel(const double *__restrict__ chi, const double *__restrict__ g, int64_t n_grid, int n,
                               int n_omega, double *__restrict__ B) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per_spin = (size_t)n_grid * n;
  if (i >= 2 * per_spin) return;
  const int s = (int)(i / per_spin);
  const int64_t r = (int64_t)((i % per_spin) / n);
  const int b = (int)(i % n);
  double acc = 0.0;
  for (int w = 0; w < n_omega; ++w)
    acc = fma(g[((size_t)w * 2 + s) * n_grid + r], chi[(((size_t)r * n_omega + w) * 2 + s) * n + b], acc);
  B[i] = -0.5 * acc;
}

// fock[s] = abs_clip(fock[s] + F[s] + F[s]^T)  (train.py:200-210).
__global__ void fock_add_hf_kernel(double *__restrict__ fock, const double *__restrict__ F, int n, double clip) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nn = (size_t)n * n;
  if (i >= 2 * nn) return;
  const size_t s = i / nn;
  const int a = (int)((i % nn) / n), b = (int)(i % n);
  const double v = fock[i] + F[i] + F[s * nn + (size_t)b * n + a];
  fock[i] = fabs(v) > clip ? v : 0.0;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

int hf_splits(int64_t n_grid) {
  int64_t s = n_grid / 2048;
  if (s < 1) s = 1;
  if (s > 148) s = 148;
  return (int)s;
}

int check_hf_args(const char *who, const void *ao, const void *chi, int64_t n_grid, int n_ao, int n_omega,
                  const void *out, const void *ws, size_t ws_bytes) {
  if (ao == nullptr || chi == nullptr || out == nullptr || ws == nullptr) {
    set_error("%s: ao, chi, the output and the workspace are required", who);
    return GDFT_ERR_INVALID;
  }
  if (n_grid <= 0 || n_ao <= 0 || n_omega <= 0 || n_omega > 8 || n_grid > (int64_t)INT32_MAX) {
    set_error("%s: n_grid=%lld n_ao=%d n_omega=%d", who, (long long)n_grid, n_ao, n_omega);
    return GDFT_ERR_INVALID;
  }
  size_t need = 0;
  gdft_hf_workspace_bytes(n_grid, n_ao, n_omega, &need);
  if (ws_bytes < need) {
    set_error("%s: workspace of %zu bytes, %zu needed", who, ws_bytes, need);
    return GDFT_ERR_INVALID;
  }
  if (((uintptr_t)ao | (uintptr_t)chi | (uintptr_t)out | (uintptr_t)ws) & 7) {
    set_error("%s: device pointers must be 8-byte aligned", who);
    return GDFT_ERR_INVALID;
  }
  return GDFT_OK;
}

}  // namespace

}  // namespace gdft

using namespace gdft;

extern "C" {

int gdft_hf_workspace_bytes(int64_t n_grid, int32_t n_ao, int32_t n_omega, size_t *bytes) {
  (void)n_omega;
  if (bytes == nullptr || n_grid <= 0 || n_ao <= 0) {
    set_error("gdft_hf_workspace_bytes: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  // X or B: [2][n_grid][n_ao]; split partials of F: [nsplit][n_ao][n_ao].
  *bytes = align256((size_t)2 * n_grid * n_ao * sizeof(double)) +
           align256((size_t)hf_splits(n_grid) * n_ao * n_ao * sizeof(double));
  return GDFT_OK;
}

int gdft_hf_energy_density(const double *d_ao, const double *d_rdm1, const double *d_chi, int64_t n_grid,
                           int32_t n_ao, int32_t n_omega, double *d_ehf, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_hf_args("gdft_hf_energy_density", d_ao, d_chi, n_grid, n_ao, n_omega, d_ehf, d_ws, ws_bytes);
  if (rc) return rc;
  if (d_rdm1 == nullptr) {
    set_error("gdft_hf_energy_density: rdm1 is required");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  double *X = (double *)d_ws;
  for (int s = 0; s < 2; ++s)
    if ((rc = check_cuda(gemm<kNN>((int)n_grid, n_ao, n_ao, d_ao, n_ao, d_rdm1 + (size_t)s * n_ao * n_ao, n_ao,
                                   X + (size_t)s * n_grid * n_ao, n_ao, 0.0, st),
                         "hf ao.D")))
      return rc;
  const int64_t threads = 2 * n_grid * 32;
  hf_rowdot_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(d_chi, X, n_grid, n_ao, n_omega, d_ehf);
  return check_cuda(cudaGetLastError(), "hf rowdot");
}

int gdft_hf_fock(const double *d_ao, const double *d_chi, const double *d_g, int64_t n_grid, int32_t n_ao,
                 int32_t n_omega, double *d_fock_hf, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_hf_args("gdft_hf_fock", d_ao, d_chi, n_grid, n_ao, n_omega, d_fock_hf, d_ws, ws_bytes);
  if (rc) return rc;
  if (d_g == nullptr) {
    set_error("gdft_hf_fock: g = dE/d ehf is required");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  double *B = (double *)d_ws;
  double *part = (double *)((char *)d_ws + align256((size_t)2 * n_grid * n_ao * sizeof(double)));
  const size_t total = (size_t)2 * n_grid * n_ao;
  hf_bmat_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(d_chi, d_g, n_grid, n_ao, n_omega, B);
  if ((rc = check_cuda(cudaGetLastError(), "hf B"))) return rc;
  const int nsplit = hf_splits(n_grid);
  for (int s = 0; s < 2; ++s)
    if ((rc = check_cuda(gemm_tn_split(n_ao, n_ao, n_grid, d_ao, n_ao, B + (size_t)s * n_grid * n_ao, n_ao,
                                       d_fock_hf + (size_t)s * n_ao * n_ao, nsplit, part, st),
                         "hf ao^T B")))
      return rc;
  return GDFT_OK;
}

int gdft_fock_add_hf(double *d_fock, const double *d_fock_hf, int32_t n_ao, double clip, void *stream) {
  if (d_fock == nullptr || d_fock_hf == nullptr || n_ao <= 0) {
    set_error("gdft_fock_add_hf: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  const size_t total = (size_t)2 * n_ao * n_ao;
  fock_add_hf_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_fock, d_fock_hf, n_ao,
                                                                                       clip);
  return check_cuda(cudaGetLastError(), "fock_add_hf");
}

}  // extern "C"
