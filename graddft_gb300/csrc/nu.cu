// nu.cu - range-separated one-electron integrals on the grid and the chi tensor.
//
//   nu_ab(C) = int phi_a(r') phi_b(r') erf(omega |r' - C|) / |r' - C| dr'   (omega = 0: 1/|r' - C|)
//   chi[r][w][s][a] = sum_(b,d) D_s[b][d] phi_b(r) nu^w_da(r)
// (_evaluate_nu / _nu_chunk, external/_hf_density.py:17-120, which call PySCF's
// int1e_grids; generate_chi_tensor, interface/pyscf.py:1067-1126).
//
// Integrals by the McMurchie-Davidson scheme.  For primitives of exponents
// alpha (centre A) and beta (centre B), p = alpha + beta, P = (alpha A + beta B)/p:
//   G_a G_b = sum_tuv E^x_t E^y_u E^z_v Lambda_tuv(r; p, P)   (Hermite expansion, E^00_0 = exp(-alpha beta/p X_AB^2),
//     E^(i+1)j_t = E^ij_(t-1)/(2p) + X_PA E^ij_t + (t+1) E^ij_(t+1), likewise in j with X_PB),
//   int Lambda_tuv(r') erf(omega|r'-C|)/|r'-C| dr' = (2 pi / p) sqrt(mu/p) R_tuv(mu, P - C),
// with 1/mu = 1/p + 1/omega^2 (mu = p for the plain Coulomb operator): the
// attenuated operator acts as the Coulomb potential of a Gaussian charge of
// exponent omega^2, whose convolution with the product Gaussian is a Gaussian of
// exponent mu.  R^n_000 = (-2 mu)^n F_n(mu |P - C|^2) and
//   R^n_(t+1)uv = t R^(n+1)_(t-1)uv + X_PC R^(n+1)_tuv  (likewise in u and v).
// The Boys function F_n(T) = int_0^1 u^(2n) exp(-T u^2) du comes from a table of
// F_n on T = 0, 0.1, ..., 60 filled on the device from the positive series
// F_n(T) = exp(-T) sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1)), a 9-term Taylor
// expansion about the nearest tabulated T (F_n' = -F_(n+1)) for the highest n,
// and the downward recursion F_n = (2T F_(n+1) + exp(-T)) / (2n+1); beyond T = 60,
// F_0 = sqrt(pi/T)/2 and F_(n+1) = (2n+1) F_n / (2T).
//
// Work layout: one warp per shell pair and 32 grid points (lanes = points), so the
// shell pair's primitive data (set up once per pair and omega by
// nu_pair_setup_kernel) are uniform loads; templates on (l_a >= l_b) <= 3.
#include <vector>

#include "common.cuh"
#include "mlp_gemm.cuh"
#include "nu_kernels.cuh"

namespace gdft {

namespace {

using namespace nu_detail;

__global__ void boys_table_kernel(double *__restrict__ tab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kBoysPts * kBoysN) return;
  const int pt = i / kBoysN, n = i % kBoysN;
  const double T = pt * kBoysStep;
  double term = 1.0 / (2 * n + 1), sum = term;
  for (int k = 1; k < 1000; ++k) {
    term *= 2.0 * T / (2 * n + 2 * k + 1);
    sum += term;
    if (term < 1e-18 * sum) break;
  }
  tab[i] = exp(-T) * sum;
}

// One thread per shell pair: the primitive-pair records.  Besides mu and P,
// a record holds, for every pair of cartesian components (qa, qb) in PySCF's
// order and every (t, u, v) with t <= ia + ib, u <= ka + kb, v <= ma + mb, the
// product pref * E^x_t E^y_u E^z_v (pref = (2 pi / p) sqrt(mu / p)): the same for
// all grid points, so the per-point work is one FMA per term.
__global__ void nu_pair_setup_kernel(ShellView B, const int32_t *__restrict__ pairs, int n_pairs, double omega,
                                     double *__restrict__ pp, int64_t n_pp) {
  const int ip = blockIdx.x * blockDim.x + threadIdx.x;
  if (ip >= n_pairs) return;
  const int s1 = pairs[4 * ip], s2 = pairs[4 * ip + 1];
  const int64_t off = pairs[4 * ip + 2];
  shells_detail::ShellRec r1, r2;
  if (!shells_detail::load_shell(B, s1, r1) || !shells_detail::load_shell(B, s2, r2)) return;
  if (r1.l > kNuMaxL || r2.l > kNuMaxL) return;
  const int len = rec_len(r1.l, r2.l);
  if (off < 0 || off + (int64_t)r1.np * r2.np * len > n_pp) return;
  const double *A = B.centre + 3 * s1, *Bc = B.centre + 3 * s2;
  for (int i1 = 0; i1 < r1.np; ++i1) {
    for (int i2 = 0; i2 < r2.np; ++i2) {
      double *rec = pp + off + ((int64_t)i1 * r2.np + i2) * len;
      const double a = B.exps[r1.poff + i1], b = B.exps[r2.poff + i2];
      const double p = a + b, ip2 = 0.5 / p;
      const double mu = omega == 0.0 ? p : p * omega * omega / (p + omega * omega);
      const double pref = (2.0 * kPi / p) * sqrt(mu / p);
      rec[0] = mu;
      rec[5] = p;
      double E[3][kETab];
      for (int d = 0; d < 3; ++d) {
        const double P = (a * A[d] + b * Bc[d]) / p;
        rec[2 + d] = P;
        const double xab = A[d] - Bc[d], xpa = P - A[d], xpb = P - Bc[d];
        for (int q = 0; q < kETab; ++q) E[d][q] = 0.0;
        E[d][e_idx(0, 0, 0)] = exp(-a * b / p * xab * xab);
        for (int i = 0; i < r1.l; ++i)
          for (int t = 0; t <= i + 1; ++t)
            E[d][e_idx(i + 1, 0, t)] = (t > 0 ? ip2 * E[d][e_idx(i, 0, t - 1)] : 0.0) + xpa * E[d][e_idx(i, 0, t)] +
                                       (t + 1 <= i ? (t + 1) * E[d][e_idx(i, 0, t + 1)] : 0.0);
        for (int j = 0; j < r2.l; ++j)
          for (int i = 0; i <= r1.l; ++i)
            for (int t = 0; t <= i + j + 1; ++t)
              E[d][e_idx(i, j + 1, t)] = (t > 0 ? ip2 * E[d][e_idx(i, j, t - 1)] : 0.0) +
                                         xpb * E[d][e_idx(i, j, t)] +
                                         (t + 1 <= i + j ? (t + 1) * E[d][e_idx(i, j, t + 1)] : 0.0);
      }
      // screening: a Gaussian product of overlap prefactor below 1e-30 contributes
      // nothing at double precision to any point's integrals (the Hermite integrals
      // grow at most like (2 mu)^(L/2), far from closing the gap for l <= 3)
      rec[1] = E[0][0] * E[1][0] * E[2][0] < kScreen ? 1.0 : 0.0;
      double *E3 = rec + 8;
      int idx = 0;
      for (int ia = r1.l; ia >= 0; --ia)
        for (int ka = r1.l - ia; ka >= 0; --ka) {
          const int ma = r1.l - ia - ka;
          for (int ib = r2.l; ib >= 0; --ib)
            for (int kb = r2.l - ib; kb >= 0; --kb) {
              const int mb = r2.l - ib - kb;
              for (int t = 0; t <= ia + ib; ++t)
                for (int u = 0; u <= ka + kb; ++u)
                  for (int v = 0; v <= ma + mb; ++v)
                    if (idx < len - 8)
                      E3[idx++] = pref * E[0][e_idx(ia, ib, t)] * E[1][e_idx(ka, kb, u)] * E[2][e_idx(ma, mb, v)];
            }
        }
    }
  }
}

// chi[(p * n_omega + w) * 2 + s][a] = sum_d X_s[p][d] nu[d][a][p] for a chunk of points.
// CTA: 32 points (lanes) x 32 AOs (4 per warp); X staged through shared memory in 32-wide d tiles.
__global__ void __launch_bounds__(256) chi_kernel(const double *__restrict__ X, const double *__restrict__ nu,
                                                  int64_t n_pts, int64_t pc, int n, int n_omega, int w,
                                                  double *__restrict__ chi, int64_t p_begin) {
  __shared__ double xs[2][32][33];
  __shared__ double os[32][2][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t p0 = (int64_t)blockIdx.x * 32;
  const int a0 = blockIdx.y * 32;
  double acc[4][2];
#pragma unroll
  for (int j = 0; j < 4; ++j) acc[j][0] = acc[j][1] = 0.0;
  for (int d0 = 0; d0 < n; d0 += 32) {
    for (int i = threadIdx.x; i < 2 * 32 * 32; i += blockDim.x) {
      const int s = i / (32 * 32), pt = (i / 32) % 32, dd = i % 32;
      const int64_t p = p0 + pt;
      xs[s][pt][dd] = (p < n_pts && d0 + dd < n) ? X[((int64_t)s * pc + p) * n + d0 + dd] : 0.0;
    }
    __syncthreads();
    const int dn = min(32, n - d0);
    const int64_t p = p0 + lane;
    if (p < n_pts) {
      for (int dd = 0; dd < dn; ++dd) {
        const double x0 = xs[0][lane][dd], x1 = xs[1][lane][dd];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int a = a0 + 4 * warp + j;
          if (a < n) {
            const double v = nu[((int64_t)(d0 + dd) * n + a) * pc + p];
            acc[j][0] = fma(x0, v, acc[j][0]);
            acc[j][1] = fma(x1, v, acc[j][1]);
          }
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    os[lane][0][4 * warp + j] = acc[j][0];
    os[lane][1][4 * warp + j] = acc[j][1];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 32 * 2 * 32; i += blockDim.x) {
    const int pt = i / 64, s = (i / 32) % 2, aa = i % 32;
    const int64_t p = p0 + pt;
    if (p < n_pts && a0 + aa < n) chi[(((p_begin + p) * n_omega + w) * 2 + s) * n + a0 + aa] = os[pt][s][aa];
  }
}

size_t al256(size_t x) { return (x + 255) / 256 * 256; }

// Host-side pair list: shell pairs (s1, s2) with l(s1) >= l(s2), each unordered
// pair once, grouped by class (l1, l2); class_lo[c]..class_lo[c+1] for class c
// = l1 * (l1 + 1) / 2 + l2.
struct PairPlan {
  std::vector<int32_t> pairs;  // (n_pairs, 4): s1, s2, primitive-pair offset, 0
  int class_lo[11];
  int64_t n_pp = 0;  // doubles of the primitive-pair records of one omega
  int max_l = 0;
};

int make_plan(const gdft_basis *b, PairPlan &plan, const char *who) {
  std::vector<int32_t> sh((size_t)b->n_shell * kShellCols);
  cudaError_t e = cudaMemcpy(sh.data(), b->d_shell, sh.size() * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return check_cuda(e, who);
  std::vector<std::vector<int32_t>> cls(10);
  for (int i = 0; i < b->n_shell; ++i) {
    const int li = sh[(size_t)kShellCols * i];
    if (li < 0 || li > kNuMaxL) {
      set_error("%s: shell %d has l = %d; the integrals are built for l <= %d", who, i, li, kNuMaxL);
      return GDFT_ERR_UNSUPPORTED;
    }
    plan.max_l = li > plan.max_l ? li : plan.max_l;
  }
  for (int i = 0; i < b->n_shell; ++i)
    for (int j = 0; j <= i; ++j) {
      int s1 = i, s2 = j;
      if (sh[(size_t)kShellCols * s1] < sh[(size_t)kShellCols * s2]) {
        s1 = j;
        s2 = i;
      }
      const int l1 = sh[(size_t)kShellCols * s1], l2 = sh[(size_t)kShellCols * s2];
      auto &v = cls[l1 * (l1 + 1) / 2 + l2];
      v.push_back(s1);
      v.push_back(s2);
      v.push_back(0);
      v.push_back(0);
    }
  int n = 0;
  for (int c = 0; c < 10; ++c) {
    plan.class_lo[c] = n;
    for (size_t q = 0; q < cls[c].size(); q += 4) {
      const int s1 = cls[c][q], s2 = cls[c][q + 1];
      const int64_t np1 = sh[(size_t)kShellCols * s1 + 1], np2 = sh[(size_t)kShellCols * s2 + 1];
      const int64_t len = rec_len(sh[(size_t)kShellCols * s1], sh[(size_t)kShellCols * s2]);
      if (plan.n_pp + np1 * np2 * len > INT32_MAX) {
        set_error("%s: too many primitive pairs", who);
        return GDFT_ERR_INVALID;
      }
      plan.pairs.push_back(s1);
      plan.pairs.push_back(s2);
      plan.pairs.push_back((int32_t)plan.n_pp);
      plan.pairs.push_back(0);
      plan.n_pp += np1 * np2 * len;
      ++n;
    }
  }
  plan.class_lo[10] = n;
  return GDFT_OK;
}

struct NuWs {
  size_t off_boys, off_pairs, off_pp, off_nu, off_x, bytes;
};

NuWs nu_ws(const PairPlan &plan, int n_ao, int64_t chunk, bool want_chi, int n_omega) {
  NuWs W;
  size_t off = 0;
  W.off_boys = off;
  off = al256(off + (size_t)kBoysPts * kBoysN * sizeof(double));
  W.off_pairs = off;
  off = al256(off + plan.pairs.size() * sizeof(int32_t));
  W.off_pp = off;
  off = al256(off + (size_t)n_omega * plan.n_pp * sizeof(double));
  W.off_nu = off;
  W.off_x = off;
  if (want_chi) {
    off = al256(off + (size_t)n_ao * n_ao * chunk * sizeof(double));
    W.off_x = off;
    off = al256(off + (size_t)2 * chunk * n_ao * sizeof(double));
  }
  W.bytes = off;
  return W;
}

int check_nu_basis(const gdft_basis *b, const char *who, ShellView &B) {
  if (b == nullptr || b->d_shell == nullptr || b->d_centre == nullptr || b->d_exp == nullptr ||
      b->d_coef == nullptr || b->d_ao == nullptr || b->d_trans == nullptr || b->n_shell <= 0 || b->n_ao <= 0) {
    set_error("%s: a basis with all of its tables is required", who);
    return GDFT_ERR_INVALID;
  }
  B = ShellView{b->d_shell, b->d_centre, b->d_exp, b->d_coef, b->d_ao, b->d_trans,
                b->n_shell, b->n_ao,    b->n_prim, b->n_coef, b->n_trans};
  return GDFT_OK;
}

// Setup (Boys table, pair list, primitive pairs for omega) and the nu launches for points [p_begin, p_begin + n_pts).
int run_nu(const ShellView &B, const PairPlan &plan, const NuWs &W, char *ws, int w, const double *coords,
           int64_t p_begin, int64_t n_pts, NuOut out, const char *who, cudaStream_t st) {
  const double *boys_tab = (const double *)(ws + W.off_boys);
  const int32_t *pairs = (const int32_t *)(ws + W.off_pairs);
  const double *pp = (const double *)(ws + W.off_pp) + (size_t)w * plan.n_pp;
  int rc;
#define GDFT_NU_CLASS(LA, LB)                                                                                     \
  {                                                                                                               \
    const int c = LA * (LA + 1) / 2 + LB, lo = plan.class_lo[c], hi = plan.class_lo[c + 1];                        \
    if (hi > lo) {                                                                                                \
      if ((hi - lo + 7) / 8 > 65535) {                                                                            \
        set_error("%s: %d shell pairs of one class exceed one launch", who, hi - lo);                            \
        return GDFT_ERR_UNSUPPORTED;                                                                              \
      }                                                                                                           \
      const cudaError_t e = LA < 3 ? launch_nu_class<(LA < 3 ? LA : 0), (LA < 3 ? LB : 0)>(                      \
                                         B, pairs, lo, hi, pp, plan.n_pp, boys_tab, coords, p_begin, n_pts, out, st) \
                                   : launch_nu_f_class(LA, LB, B, pairs, lo, hi, pp, plan.n_pp, boys_tab, coords,    \
                                                       p_begin, n_pts, out, st);                                  \
      if ((rc = check_cuda(e, who))) return rc;                                                                   \
    }                                                                                                             \
  }
  GDFT_NU_CLASS(0, 0)
  GDFT_NU_CLASS(1, 0)
  GDFT_NU_CLASS(1, 1)
  GDFT_NU_CLASS(2, 0)
  GDFT_NU_CLASS(2, 1)
  GDFT_NU_CLASS(2, 2)
  GDFT_NU_CLASS(3, 0)
  GDFT_NU_CLASS(3, 1)
  GDFT_NU_CLASS(3, 2)
  GDFT_NU_CLASS(3, 3)
#undef GDFT_NU_CLASS
  return GDFT_OK;
}

int setup_nu(const ShellView &B, const PairPlan &plan, const NuWs &W, char *ws, int w, double omega, bool first,
             const char *who, cudaStream_t st) {
  int rc;
  if (first) {
    boys_table_kernel<<<(kBoysPts * kBoysN + 255) / 256, 256, 0, st>>>((double *)(ws + W.off_boys));
    if ((rc = check_cuda(cudaGetLastError(), who))) return rc;
    if ((rc = check_cuda(cudaMemcpyAsync(ws + W.off_pairs, plan.pairs.data(), plan.pairs.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, st),
                         who)))
      return rc;
  }
  const int np = (int)(plan.pairs.size() / 4);
  nu_pair_setup_kernel<<<(np + 127) / 128, 128, 0, st>>>(
      B, (const int32_t *)(ws + W.off_pairs), np, omega,
      (double *)(ws + W.off_pp) + (size_t)w * plan.n_pp, plan.n_pp);
  return check_cuda(cudaGetLastError(), who);
}

}  // namespace

}  // namespace gdft

using namespace gdft;

extern "C" {

int gdft_nu_workspace_bytes(const gdft_basis *basis, int64_t chunk, size_t *bytes) {
  const char *who = "gdft_nu_workspace_bytes";
  ShellView B;
  int rc = check_nu_basis(basis, who, B);
  if (rc) return rc;
  if (bytes == nullptr || chunk < 0) {
    set_error("%s: invalid arguments", who);
    return GDFT_ERR_INVALID;
  }
  PairPlan plan;
  if ((rc = make_plan(basis, plan, who))) return rc;
  *bytes = nu_ws(plan, basis->n_ao, chunk, chunk > 0, chunk > 0 ? kMaxOmega : 1).bytes;
  return GDFT_OK;
}

int gdft_nu_integrals(const gdft_basis *basis, const double *d_coords, int64_t n_grid, double omega, double *d_nu,
                      void *d_ws, size_t ws_bytes, void *stream) {
  const char *who = "gdft_nu_integrals";
  ShellView B;
  int rc = check_nu_basis(basis, who, B);
  if (rc) return rc;
  if (d_coords == nullptr || d_nu == nullptr || d_ws == nullptr || n_grid <= 0 || !(omega >= 0.0)) {
    set_error("%s: coords, nu and the workspace are required, n_grid > 0 and omega >= 0 (got %g)", who, omega);
    return GDFT_ERR_INVALID;
  }
  if ((((uintptr_t)d_coords | (uintptr_t)d_nu) & 7u) || ((uintptr_t)d_ws & 255u)) {
    set_error("%s: coords and nu must be 8-byte aligned, the workspace 256-byte aligned", who);
    return GDFT_ERR_ALIGNMENT;
  }
  PairPlan plan;
  if ((rc = make_plan(basis, plan, who))) return rc;
  const NuWs W = nu_ws(plan, basis->n_ao, 0, false, 1);
  if (ws_bytes < W.bytes) {
    set_error("%s: workspace of %zu bytes, %zu needed", who, ws_bytes, W.bytes);
    return GDFT_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = setup_nu(B, plan, W, (char *)d_ws, 0, omega, true, who, st))) return rc;
  const int n = basis->n_ao;
  const NuOut out{d_nu, 1, (int64_t)n * n, n};  // (grid, ao, ao)
  rc = run_nu(B, plan, W, (char *)d_ws, 0, d_coords, 0, n_grid, out, who, st);
  if (rc) return rc;
  // the pair list is copied from host memory that goes out of scope here
  return check_cuda(cudaStreamSynchronize(st), who);
}

int gdft_chi(const gdft_basis *basis, const double *d_coords, const double *d_ao, const double *d_rdm1,
             int64_t n_grid, const double *h_omegas, int32_t n_omega, int64_t chunk, double *d_chi, void *d_ws,
             size_t ws_bytes, void *stream) {
  const char *who = "gdft_chi";
  ShellView B;
  int rc = check_nu_basis(basis, who, B);
  if (rc) return rc;
  if (d_coords == nullptr || d_ao == nullptr || d_rdm1 == nullptr || d_chi == nullptr || d_ws == nullptr ||
      h_omegas == nullptr || n_grid <= 0 || n_omega <= 0 || n_omega > kMaxOmega || chunk <= 0) {
    set_error("%s: coords, ao, rdm1, omegas, chi and the workspace are required; n_grid, chunk > 0, "
              "1 <= n_omega <= %d", who, kMaxOmega);
    return GDFT_ERR_INVALID;
  }
  for (int w = 0; w < n_omega; ++w)
    if (!(h_omegas[w] >= 0.0)) {
      set_error("Range-separated parameter omega must be non-negative!");
      return GDFT_ERR_INVALID;
    }
  if ((((uintptr_t)d_coords | (uintptr_t)d_ao | (uintptr_t)d_rdm1 | (uintptr_t)d_chi) & 7u) ||
      ((uintptr_t)d_ws & 255u)) {
    set_error("%s: arrays must be 8-byte aligned, the workspace 256-byte aligned", who);
    return GDFT_ERR_ALIGNMENT;
  }
  PairPlan plan;
  if ((rc = make_plan(basis, plan, who))) return rc;
  const int n = basis->n_ao;
  const int64_t pc = chunk < n_grid ? chunk : n_grid;
  const NuWs W = nu_ws(plan, n, pc, true, n_omega);
  if (ws_bytes < W.bytes) {
    set_error("%s: workspace of %zu bytes, %zu needed", who, ws_bytes, W.bytes);
    return GDFT_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  double *nu = (double *)(ws + W.off_nu);
  double *X = (double *)(ws + W.off_x);
  for (int w = 0; w < n_omega; ++w)
    if ((rc = setup_nu(B, plan, W, ws, w, h_omegas[w], w == 0, who, st))) return rc;
  for (int64_t p0 = 0; p0 < n_grid; p0 += pc) {
    const int64_t np_ = n_grid - p0 < pc ? n_grid - p0 : pc;
    // X_s = ao[p0 : p0 + np_] D_s, shared by the omegas
    for (int s = 0; s < 2; ++s)
      if ((rc = check_cuda(gemm<kNN>((int)np_, n, n, d_ao + p0 * n, n, d_rdm1 + (size_t)s * n * n, n,
                                     X + (size_t)s * pc * n, n, 0.0, st),
                           who)))
        return rc;
    for (int w = 0; w < n_omega; ++w) {
      const NuOut out{nu, pc, 1, n};  // [a][b][point]
      if ((rc = run_nu(B, plan, W, ws, w, d_coords, p0, np_, out, who, st))) return rc;
      const dim3 grid((unsigned)((np_ + 31) / 32), (unsigned)((n + 31) / 32));
      chi_kernel<<<grid, 256, 0, st>>>(X, nu, np_, pc, n, n_omega, w, d_chi, p0);
      if ((rc = check_cuda(cudaGetLastError(), who))) return rc;
    }
  }
  return check_cuda(cudaStreamSynchronize(st), who);
}

}  // extern "C"
