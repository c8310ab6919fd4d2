// hf.cu - exact-exchange (Hartree-Fock) terms from a supplied chi tensor.
//
//   ehf[w][s][r] = -1/2 sum_c chi[r][w][s][c] (sum_a ao[r][a] D_s[a][c])      (molecule.py:507-541)
//   F_s[a][b]    = -1/2 sum_w sum_r ao[r][a] g[w][s][r] chi[r][w][s][b]       (molecule.py:545-613, the
//                  omega sum of b3lyp_hfgrads, popular_functionals.py:357-372, and dm21_hfgrads_*,
//                  functional.py:677-757)
// with g = dE_xc/d ehf.  chi keeps the reference's layout (grid, omega, spin,
// orbitals).
//
// FP64 form: both contractions on the tiled FP64 GEMM: X_s = ao D_s, then a
// warp per (point, spin) takes the row dot with chi; B_s = -1/2 sum_w g chi,
// then F_s = ao^T B_s with the grid split over CTAs and the partials summed in
// a fixed order.
//
// Mixed (TF32x3) form: the same two contractions on the block-scaled
// three-slice tcgen05 GEMM (tcg3: exact hi*hi chunk sums, compensated FP32
// running sums, FP64 output).  Both spins share one GEMM each: X = ao [D_0 | D_1]
// (N = 2n, one split), then the FP64 row dot; F = ao^T [B_0 | B_1] with
// K = grid points split over CTAs, B formed inside its packer (never stored),
// partials summed in a fixed order.
#include "common.cuh"
#include "kernels.cuh"
#include "mlp_gemm.cuh"
#include "tc_gemm.cuh"
#include "umma.cuh"

namespace gdft {

namespace {

// One warp per (point, spin): ehf of every omega.  X_s[r][c] sits at
// X[s * spin_stride + r * ld + c].
__global__ void hf_rowdot_kernel(const double *__restrict__ chi, const double *__restrict__ X, int64_t n_grid, int n,
                                 int n_omega, int64_t ld, int64_t spin_stride, double *__restrict__ ehf) {
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= 2 * n_grid) return;  // whole warps leave together
  const int64_t r = gw >> 1;
  const int s = (int)(gw & 1);
  const double *x = X + (size_t)s * spin_stride + (size_t)r * ld;
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

// ---- mixed form: operands of the three-slice GEMM ----

// Operand element (row m, K index k) of each packed operand.  Callers keep
// m < rows and k < kdim, which bounds every index below.
struct FetchRows {  // X[m][k]: ao as the A operand of X = ao D (rows = points, K = orbitals)
  const double *x;
  int64_t ld;
  __device__ double operator()(int64_t m, int64_t k) const { return x[m * ld + k]; }
};
struct FetchCols {  // X[k][m]: ao^T as the A operand of F = ao^T B (rows = orbitals, K = points)
  const double *x;
  int64_t ld;
  __device__ double operator()(int64_t m, int64_t k) const { return x[k * ld + m]; }
};
struct FetchDensity {  // row j = s n + c, K = a: D_s[a][c]
  const double *d;
  int64_t n;
  __device__ double operator()(int64_t j, int64_t a) const {
    const int64_t s = j >= n ? 1 : 0, c = j - s * n;
    return d[(s * n + a) * n + c];
  }
};
struct FetchHfB {  // row j = s n + b, K = r: sum_w g[w][s][r] chi[r][w][s][b] (the packer scales by -1/2)
  const double *chi, *g;
  int64_t n_grid, n;
  int n_omega;
  __device__ double operator()(int64_t j, int64_t r) const {
    const int64_t s = j >= n ? 1 : 0, b = j - s * n;
    double acc = 0.0;
    for (int w = 0; w < n_omega; ++w)
      acc = fma(g[((size_t)w * 2 + s) * n_grid + r], chi[(((size_t)r * n_omega + w) * 2 + s) * n + b], acc);
    return acc;
  }
};

// One row (32 K values) of a three-slice block set [hi | lo | lo2] from FP64
// values times a power of two, with one FP64 subtraction and three conversions
// per value (the FP64 pipe bounds these packers): xf = x rounded to FP32 and
// xl = (x - xf) rounded, so xf + xl = x to 2^-47 |x|; hi = xf on the row's
// quantum (as umma::quant takes it from the row maximum), r = xf - hi and
// e = r - tf32(r) exact in FP32, lo = tf32(r), lo2 = tf32(e + xl).  The
// representation error stays within about 2^-31 of the row maximum, the bound
// of umma::store_row3.
__device__ __forceinline__ void store_row3_scaled(float *blk3, int row, const double (&v)[32], float scale) {
  float xf[32], xl[32];
  float m = 0.0f;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const float f = (float)v[k];
    xl[k] = (float)(v[k] - (double)f) * scale;
    xf[k] = f * scale;
    m = fmaxf(m, fabsf(xf[k]));
  }
  const umma::Quant u = umma::quant(m);
#pragma unroll
  for (int k4 = 0; k4 < 8; ++k4) {
    float h[4], l[4], l2[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float x = xf[4 * k4 + i];
      h[i] = rintf(x * u.inv) * u.q;
      const float r = x - h[i];
      l[i] = umma::tf32_rn(r);
      l2[i] = umma::tf32_rn((r - l[i]) + xl[4 * k4 + i]);
    }
    const uint32_t off = umma::kblock_off(row, 4 * k4) / 4;
    *(float4 *)(blk3 + off) = make_float4(h[0], h[1], h[2], h[3]);
    *(float4 *)(blk3 + umma::kBlockBytes / 4 + off) = make_float4(l[0], l[1], l[2], l[3]);
    *(float4 *)(blk3 + umma::kBlockBytes / 2 + off) = make_float4(l2[0], l2[1], l2[2], l2[3]);
  }
}

// Block (tile, kc) of a three-slice operand: rows tile*128 + m, K indices
// kc*32 + k, scale * f(m, k), zero outside rows x kdim, in the block layout the
// three-slice GEMM streams.  One thread per row.
template <class Fetch>
__global__ void __launch_bounds__(128) hf_pack3_kernel(Fetch f, int64_t rows, int64_t kdim, int64_t kchunks,
                                                       float scale, float *__restrict__ out) {
  const int64_t t = blockIdx.x / kchunks, kc = blockIdx.x % kchunks;
  const int64_t m = t * 128 + threadIdx.x;
  double v[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const int64_t kk = kc * 32 + k;
    v[k] = (m < rows && kk < kdim) ? f(m, kk) : 0.0;
  }
  store_row3_scaled(out + (size_t)blockIdx.x * 3 * (umma::kBlockBytes / 4), (int)threadIdx.x, v, scale);
}

// F[s][a][b] = sum_z part[z][a][s n + b], the splits in order.
__global__ void hf_fock_reduce_kernel(const double *__restrict__ part, int nsplit, int n, double *__restrict__ F) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nn = (size_t)n * n;
  if (i >= 2 * nn) return;
  const size_t s = i / nn;
  const size_t a = (i % nn) / n, b = i % n;
  const size_t src = a * 2 * n + s * n + b, stride = 2 * nn;
  double acc = 0.0;
  for (int z = 0; z < nsplit; ++z) acc += part[(size_t)z * stride + src];
  F[i] = acc;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

constexpr size_t kSet3Bytes = 3 * (size_t)umma::kBlockBytes;  // one 128 x 32 three-slice block set

// Workspace of the mixed form: [error word | energy-density or Fock buffers].
struct HfTcLayout {
  int64_t tiles_g, kc_ao, tiles_ao, tiles_j, rchunks, cps;
  int nsplit;
  size_t off_err, off_pa, off_pb, off_x, e_end;  // energy density: ao sets, D sets, X (n_grid x 2n)
  size_t off_fa, off_fb, off_part, f_end;          // Fock: ao^T sets, B sets, split partials
  size_t bytes;
};

HfTcLayout hf_tc_layout(int64_t n_grid, int n) {
  HfTcLayout L{};
  L.tiles_g = (n_grid + 127) / 128;
  L.kc_ao = (n + 31) / 32;
  L.tiles_ao = (n + 127) / 128;
  L.tiles_j = (2 * (int64_t)n + 127) / 128;
  L.rchunks = (n_grid + 31) / 32;
  // About one wave of the Fock GEMM's CTAs (one per SM) over its (orbital tile
  // x spin-orbital tile) grid, split along the points.
  const int64_t tiles = L.tiles_ao * L.tiles_j;
  int64_t ns = (152 + tiles - 1) / tiles;
  if (ns > L.rchunks) ns = L.rchunks;
  if (ns < 1) ns = 1;
  L.cps = (L.rchunks + ns - 1) / ns;
  L.nsplit = (int)((L.rchunks + L.cps - 1) / L.cps);
  L.off_err = 0;
  L.off_pa = 256;
  L.off_pb = L.off_pa + align256((size_t)L.tiles_g * L.kc_ao * kSet3Bytes);
  L.off_x = L.off_pb + align256((size_t)L.tiles_j * L.kc_ao * kSet3Bytes);
  L.e_end = L.off_x + align256((size_t)n_grid * 2 * n * sizeof(double));
  L.off_fa = 256;
  L.off_fb = L.off_fa + align256((size_t)L.tiles_ao * L.rchunks * kSet3Bytes);
  L.off_part = L.off_fb + align256((size_t)L.tiles_j * L.rchunks * kSet3Bytes);
  L.f_end = L.off_part + align256((size_t)L.nsplit * n * 2 * n * sizeof(double));
  L.bytes = L.e_end > L.f_end ? L.e_end : L.f_end;
  return L;
}

int hf_splits(int64_t n_grid) {
  int64_t s = n_grid / 2048;
  if (s < 1) s = 1;
  if (s > 148) s = 148;
  return (int)s;
}

int check_hf_args(const char *who, int form, const void *ao, const void *chi, int64_t n_grid, int n_ao, int n_omega,
                  const void *out, const void *ws, size_t ws_bytes) {
  if (form != GDFT_FP64 && form != GDFT_TF32X3) {
    set_error("%s: unknown form %d", who, form);
    return GDFT_ERR_INVALID;
  }
  if (ao == nullptr || chi == nullptr || out == nullptr || ws == nullptr) {
    set_error("%s: ao, chi, the output and the workspace are required", who);
    return GDFT_ERR_INVALID;
  }
  // The mixed form indexes points with 32-bit tile rows of 128.
  const int64_t max_grid = form == GDFT_FP64 ? (int64_t)INT32_MAX : ((int64_t)1 << 30);
  if (n_grid <= 0 || n_ao <= 0 || n_omega <= 0 || n_omega > 8 || n_grid > max_grid || n_ao > (1 << 20)) {
    set_error("%s: n_grid=%lld n_ao=%d n_omega=%d", who, (long long)n_grid, n_ao, n_omega);
    return GDFT_ERR_INVALID;
  }
  size_t need = 0;
  gdft_hf_workspace_bytes_form(n_grid, n_ao, n_omega, form, &need);
  if (ws_bytes < need) {
    set_error("%s: workspace of %zu bytes, %zu needed", who, ws_bytes, need);
    return GDFT_ERR_INVALID;
  }
  if (((uintptr_t)ao | (uintptr_t)chi | (uintptr_t)out | (uintptr_t)ws) & 7) {
    set_error("%s: device pointers must be 8-byte aligned", who);
    return GDFT_ERR_INVALID;
  }
  if (form == GDFT_TF32X3 && ((uintptr_t)ws & 255)) {
    set_error("%s: the mixed form needs a 256-byte aligned workspace", who);
    return GDFT_ERR_INVALID;
  }
  return GDFT_OK;
}

// Launch-size limits of the mixed form (grid x of each packer and GEMM).
int check_tc_sizes(const char *who, const HfTcLayout &L) {
  const int64_t lim = (int64_t)INT32_MAX;
  if (L.tiles_g * L.kc_ao > lim || L.tiles_j * L.kc_ao > lim || L.tiles_g * L.tiles_j > lim ||
      L.tiles_ao * L.rchunks > lim || L.tiles_j * L.rchunks > lim) {
    set_error("%s: problem too large for the mixed form", who);
    return GDFT_ERR_INVALID;
  }
  return GDFT_OK;
}

int hf_energy_density_tc(const double *ao, const double *rdm1, const double *chi, int64_t n_grid, int n, int n_omega,
                         double *ehf, char *ws, cudaStream_t st) {
  const HfTcLayout L = hf_tc_layout(n_grid, n);
  int rc = check_tc_sizes("gdft_hf_energy_density_form", L);
  if (rc) return rc;
  int *err = (int *)(ws + L.off_err);
  float *pa = (float *)(ws + L.off_pa), *pb = (float *)(ws + L.off_pb);
  double *X = (double *)(ws + L.off_x);
  if ((rc = check_cuda(cudaMemsetAsync(err, 0, sizeof(int), st), "hf err clear"))) return rc;
  hf_pack3_kernel<FetchRows><<<(unsigned)(L.tiles_g * L.kc_ao), 128, 0, st>>>(FetchRows{ao, n}, n_grid, n, L.kc_ao,
                                                                               1.0f, pa);
  hf_pack3_kernel<FetchDensity><<<(unsigned)(L.tiles_j * L.kc_ao), 128, 0, st>>>(FetchDensity{rdm1, n}, 2 * n, n,
                                                                                  L.kc_ao, 1.0f, pb);
  if ((rc = check_cuda(cudaGetLastError(), "hf pack ao, D"))) return rc;
  TcgArgs a{};
  a.a = pa;
  a.b = pb;
  a.m_tiles = (int)L.tiles_g;
  a.n_tiles = (int)L.tiles_j;
  a.a_chunks = a.b_chunks = a.k_chunks = a.chunks_per_split = L.kc_ao;
  a.out64 = X;  // one split: X[r][s n + c]
  a.m_valid = (int)n_grid;
  a.n_valid = 2 * n;
  a.err = err;
  if ((rc = check_cuda(launch_tcg3(a, 1, st), "hf ao.[D0|D1]"))) return rc;
  const int64_t threads = 2 * n_grid * 32;
  hf_rowdot_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(chi, X, n_grid, n, n_omega, 2 * (int64_t)n, n,
                                                                       ehf);
  return check_cuda(cudaGetLastError(), "hf rowdot");
}

int hf_fock_tc(const double *ao, const double *chi, const double *g, int64_t n_grid, int n, int n_omega, double *F,
               char *ws, cudaStream_t st) {
  const HfTcLayout L = hf_tc_layout(n_grid, n);
  int rc = check_tc_sizes("gdft_hf_fock_form", L);
  if (rc) return rc;
  int *err = (int *)(ws + L.off_err);
  float *fa = (float *)(ws + L.off_fa), *fb = (float *)(ws + L.off_fb);
  double *part = (double *)(ws + L.off_part);
  if ((rc = check_cuda(cudaMemsetAsync(err, 0, sizeof(int), st), "hf err clear"))) return rc;
  hf_pack3_kernel<FetchCols><<<(unsigned)(L.tiles_ao * L.rchunks), 128, 0, st>>>(FetchCols{ao, n}, n, n_grid,
                                                                                  L.rchunks, 1.0f, fa);
  hf_pack3_kernel<FetchHfB><<<(unsigned)(L.tiles_j * L.rchunks), 128, 0, st>>>(
      FetchHfB{chi, g, n_grid, n, n_omega}, 2 * n, n_grid, L.rchunks, -0.5f, fb);
  if ((rc = check_cuda(cudaGetLastError(), "hf pack ao^T, B"))) return rc;
  TcgArgs a{};
  a.a = fa;
  a.b = fb;
  a.m_tiles = (int)L.tiles_ao;
  a.n_tiles = (int)L.tiles_j;
  a.a_chunks = a.b_chunks = a.k_chunks = L.rchunks;
  a.chunks_per_split = L.cps;
  a.out64 = part;  // [split][a][s n + b]
  a.m_valid = n;
  a.n_valid = 2 * n;
  a.err = err;
  if ((rc = check_cuda(launch_tcg3(a, L.nsplit, st), "hf ao^T [B0|B1]"))) return rc;
  const size_t total = (size_t)2 * n * n;
  hf_fock_reduce_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(part, L.nsplit, n, F);
  return check_cuda(cudaGetLastError(), "hf fock reduce");
}

}  // namespace

}  // namespace gdft

using namespace gdft;

extern "C" {

int gdft_hf_workspace_bytes_form(int64_t n_grid, int32_t n_ao, int32_t n_omega, int32_t form, size_t *bytes) {
  (void)n_omega;
  if (bytes == nullptr || n_grid <= 0 || n_ao <= 0 || (form != GDFT_FP64 && form != GDFT_TF32X3)) {
    set_error("gdft_hf_workspace_bytes_form: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  if (form == GDFT_TF32X3) {
    *bytes = hf_tc_layout(n_grid, n_ao).bytes;
    return GDFT_OK;
  }
  // X or B: [2][n_grid][n_ao]; split partials of F: [nsplit][n_ao][n_ao].
  *bytes = align256((size_t)2 * n_grid * n_ao * sizeof(double)) +
           align256((size_t)hf_splits(n_grid) * n_ao * n_ao * sizeof(double));
  return GDFT_OK;
}

int gdft_hf_workspace_bytes(int64_t n_grid, int32_t n_ao, int32_t n_omega, size_t *bytes) {
  return gdft_hf_workspace_bytes_form(n_grid, n_ao, n_omega, GDFT_FP64, bytes);
}

int gdft_hf_energy_density_form(const double *d_ao, const double *d_rdm1, const double *d_chi, int64_t n_grid,
                                int32_t n_ao, int32_t n_omega, int32_t form, double *d_ehf, void *d_ws,
                                size_t ws_bytes, void *stream) {
  int rc = check_hf_args("gdft_hf_energy_density", form, d_ao, d_chi, n_grid, n_ao, n_omega, d_ehf, d_ws, ws_bytes);
  if (rc) return rc;
  if (d_rdm1 == nullptr) {
    set_error("gdft_hf_energy_density: rdm1 is required");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (form == GDFT_TF32X3) return hf_energy_density_tc(d_ao, d_rdm1, d_chi, n_grid, n_ao, n_omega, d_ehf,
                                                       (char *)d_ws, st);
  double *X = (double *)d_ws;
  for (int s = 0; s < 2; ++s)
    if ((rc = check_cuda(gemm<kNN>((int)n_grid, n_ao, n_ao, d_ao, n_ao, d_rdm1 + (size_t)s * n_ao * n_ao, n_ao,
                                   X + (size_t)s * n_grid * n_ao, n_ao, 0.0, st),
                         "hf ao.D")))
      return rc;
  const int64_t threads = 2 * n_grid * 32;
  hf_rowdot_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(d_chi, X, n_grid, n_ao, n_omega, n_ao,
                                                                       n_grid * n_ao, d_ehf);
  return check_cuda(cudaGetLastError(), "hf rowdot");
}

int gdft_hf_energy_density(const double *d_ao, const double *d_rdm1, const double *d_chi, int64_t n_grid,
                           int32_t n_ao, int32_t n_omega, double *d_ehf, void *d_ws, size_t ws_bytes, void *stream) {
  return gdft_hf_energy_density_form(d_ao, d_rdm1, d_chi, n_grid, n_ao, n_omega, GDFT_FP64, d_ehf, d_ws, ws_bytes,
                                     stream);
}

int gdft_hf_fock_form(const double *d_ao, const double *d_chi, const double *d_g, int64_t n_grid, int32_t n_ao,
                      int32_t n_omega, int32_t form, double *d_fock_hf, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_hf_args("gdft_hf_fock", form, d_ao, d_chi, n_grid, n_ao, n_omega, d_fock_hf, d_ws, ws_bytes);
  if (rc) return rc;
  if (d_g == nullptr) {
    set_error("gdft_hf_fock: g = dE/d ehf is required");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (form == GDFT_TF32X3) return hf_fock_tc(d_ao, d_chi, d_g, n_grid, n_ao, n_omega, d_fock_hf, (char *)d_ws, st);
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

int gdft_hf_fock(const double *d_ao, const double *d_chi, const double *d_g, int64_t n_grid, int32_t n_ao,
                 int32_t n_omega, double *d_fock_hf, void *d_ws, size_t ws_bytes, void *stream) {
  return gdft_hf_fock_form(d_ao, d_chi, d_g, n_grid, n_ao, n_omega, GDFT_FP64, d_fock_hf, d_ws, ws_bytes, stream);
}

int gdft_hf_device_status(void *d_ws, size_t ws_bytes, int32_t *status, void *stream) {
  if (d_ws == nullptr || status == nullptr || ws_bytes < sizeof(int)) {
    set_error("gdft_hf_device_status: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int h = 0;
  int rc;
  if ((rc = check_cuda(cudaMemcpyAsync(&h, d_ws, sizeof(int), cudaMemcpyDeviceToHost, st), "hf status read")))
    return rc;
  if ((rc = check_cuda(cudaStreamSynchronize(st), "hf status sync"))) return rc;
  *status = h;
  if (h != 0) {
    set_error("a device-side wait of the exchange GEMM expired (code %d); its results are invalid", h);
    return GDFT_ERR_DEVICE;
  }
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
