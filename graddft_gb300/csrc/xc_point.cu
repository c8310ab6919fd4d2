// xc_point.cu - per-grid-point stage of the XC path.
//
// For every grid point it evaluates the functional's energy-density columns
// (compute_densities, functional.py:160-185), contracts them with the
// coefficients and clips (xc_energy, functional.py:219-253), weights them
// (_integrate, functional.py:316-342) and writes:
//   * a per-block partial sum of w_r * e_xc(r) (FP64; the blocks are summed
//     with Kahan compensation by reduce.cu);
//   * the adjoint coefficients of V_xc (the pointwise part of the transpose
//     that jax.value_and_grad builds at train.py:86), per spin:
//       C_RHO = dE/drho, C_GJ = 2 dE/d(d_j rho), C_LAP = 2 dE/d(lap rho),
//       C_KIN = 2 dE/d(lap rho) + 1/2 dE/dtau,
//     so that V_ab = sum_r phi_a (C_RHO phi_b + sum_j C_GJ d_j phi_b + C_LAP lap phi_b)
//                  + sum_r C_KIN sum_j d_j phi_a d_j phi_b;
//   * optionally, g_r = dE/d ehf[w][s][r] for a functional whose HF column is
//     the sum of ehf over omega and spin (b3lyp_combine): the gradient that
//     HF_density_grad_2_Fock takes (molecule.py:598-603), i.e. with the
//     other columns unclipped (energy_densities as predict passes them,
//     train.py:167-178): abs_clip(w_r) * [|sum_f c_f e_f| > clip] * c_HF.
#include "common.cuh"
#include "xc_functionals.cuh"
#include "kernels.cuh"

namespace gdft {

namespace {

constexpr int kBlock = 256;

// Dual variable indices: rho_a, rho_b, |grad rho_a|^2, |grad rho_b|^2, lap_a,
// lap_b and, for columns that read it (the w powers of the feature columns),
// tau_a, tau_b.  The kernel runs with K = 6 unless a column depends on tau.
enum { V_R0 = 0, V_R1 = 1, V_S0 = 2, V_S1 = 3, V_L0 = 4, V_L1 = 5, V_T0 = 6, V_T1 = 7 };

template <int K>
__device__ __forceinline__ Dual<K> seed(double v, int idx) {
  Dual<K> r = dconst<K>(v);
  if (idx < K) r.d[idx] = 1.0;
  return r;
}

// Fields of a GDFT_COL_DM21_UW / GDFT_COL_DENS_X code.
__host__ __device__ __forceinline__ bool is_uw_col(int col) { return (col & ~0xff) == 0x100 || (col & ~0x1ff) == 0x200; }
__host__ __device__ __forceinline__ int uw_i(int col) { return (col >> 4) & 15; }
__host__ __device__ __forceinline__ int uw_j(int col) { return col & 15; }

// The feature-power columns out of line: inlined beside the classical
// functionals they would raise every functional's register pressure.
template <class T>
__device__ __noinline__ T uw_column(int col, const T rho[2], const T s[2], const T tau[2], double clip) {
  if ((col & ~0xff) == 0x100) return dm21_uw(rho, s, tau, uw_i(col), uw_j(col), clip);
  const int sp = (col >> 8) & 1;  // densities(): one spin's exchange term
  return uw_term(rho[sp], s[sp], tau[sp], uw_i(col), uw_j(col), false, clip);
}

template <class T>
__device__ __forceinline__ T column(int col, const T rho[2], const T s[2], const T lap[2], const T tau[2], double hf,
                                    double hf0, double hf1, double clip, unsigned *poison) {
  if (is_uw_col(col)) return uw_column(col, rho, s, tau, clip);
  switch (col) {
    case GDFT_COL_LSDA: return lsda_x_e(rho, clip);
    case GDFT_COL_B88: return b88_x_e(rho, s, clip);
    case GDFT_COL_VWN: return vwn_c_e(rho, clip, poison);
    case GDFT_COL_LYP: return lyp_c_e(rho, s, lap, clip);
    case GDFT_COL_PW92: return pw92_c_e(rho, clip, poison);
    case GDFT_COL_DM21_LDA: return dm21_lda(rho, clip);
    case GDFT_COL_HF: return tconst(rho[0], hf);
    case GDFT_COL_HF_W0: return tconst(rho[0], hf0);
    case GDFT_COL_HF_W1: return tconst(rho[0], hf1);
    default: return tconst(rho[0], 0.0);  // GDFT_COL_ZERO
  }
}

template <int KV>
__global__ void __launch_bounds__(kBlock) xc_point_kernel(const double *__restrict__ feat, const double *__restrict__ w,
                                                          int64_t n_grid, int64_t np, gdft_functional fn,
                                                          const double *__restrict__ ehf, int n_omega,
                                                          double *__restrict__ coef, double *__restrict__ epart,
                                                          double *__restrict__ dens, double *__restrict__ ghf) {
  const int64_t p = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  double e_r = 0.0;
  if (p < np) {
    double c[2][kFeat];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int k = 0; k < kFeat; ++k) c[s][k] = 0.0;
    if (p < n_grid) {
      const double clip = fn.clip;
      double f[2][kFeat];
#pragma unroll
      for (int s = 0; s < 2; ++s)
#pragma unroll
        for (int k = 0; k < kFeat; ++k) f[s][k] = feat[((size_t)s * kFeat + k) * np + p];
      Dual<KV> rho[2], sg[2], lap[2], tau[2];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        rho[s] = seed<KV>(f[s][F_RHO], V_R0 + s);
        // jnp.sum(grad_rho**2, axis=-1)
        const double sv = (f[s][F_GX] * f[s][F_GX] + f[s][F_GY] * f[s][F_GY]) + f[s][F_GZ] * f[s][F_GZ];
        sg[s] = seed<KV>(sv, V_S0 + s);
        lap[s] = seed<KV>(f[s][F_LAP], V_L0 + s);
        tau[s] = seed<KV>(f[s][F_TAU], V_T0 + s);  // a constant when KV = 6 (no column reads tau)
      }
      double hf = 0.0, hf0 = 0.0, hf1 = 0.0;
      if (ehf != nullptr) {
        // ehf layout (omega, spin, grid).
        for (int o = 0; o < n_omega; ++o) {
          const double a = ehf[((size_t)o * 2 + 0) * n_grid + p];
          const double b = ehf[((size_t)o * 2 + 1) * n_grid + p];
          hf = o == 0 ? (a + b) : hf + (a + b);
          if (o == 0) hf0 = a + b;
          if (o == 1) hf1 = a + b;
        }
      }
      // Energy density: sum_f c_f * abs_clip(e_f), then abs_clip; weight abs_clip(w).
      Dual<KV> exc = dconst<KV>(0.0);
      double e_raw = 0.0, c_hf = 0.0;  // unclipped columns' sum; coefficient of the HF column
      unsigned poison = 0;  // spins whose rho gradient is NaN in the reference (see corr_pol)
      for (int i = 0; i < fn.n_cols; ++i) {
        Dual<KV> e = column<Dual<KV>>(fn.cols[i], rho, sg, lap, tau, hf, hf0, hf1, clip, &poison);
        if (dens != nullptr) dens[(size_t)p * fn.n_cols + i] = e.v;
        const double ci = fn.n_coeffs == 1 ? fn.coeffs[0] : fn.coeffs[i];
        e_raw += ci * e.v;
        if (fn.cols[i] == GDFT_COL_HF) c_hf += ci;
        if (!(fabs(e.v) > clip)) e = dconst<KV>(0.0);  // abs_clip(densities), functional.py:184
        exc = i == 0 ? ci * e : exc + ci * e;
      }
      if (!(fabs(exc.v) > clip)) exc = dconst<KV>(0.0);  // functional.py:252 and :342
      const double wr = w[p];
      const double W = fabs(wr) > clip ? wr : 0.0;      // abs_clip(gridweights), functional.py:342
      e_r = W * exc.v;
      if (ghf != nullptr) ghf[p] = fabs(e_raw) > clip ? W * c_hf : 0.0;
      // dE_r/dvar = W * d exc/dvar.
      double dv[KV];
#pragma unroll
      for (int k = 0; k < KV; ++k) dv[k] = W * exc.d[k];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const double dsig = dv[V_S0 + s];  // dE/d|grad rho_s|^2
        const double dlap = dv[V_L0 + s];
        c[s][C_RHO] = dv[V_R0 + s];
        c[s][C_GX] = 2.0 * (2.0 * f[s][F_GX] * dsig);
        c[s][C_GY] = 2.0 * (2.0 * f[s][F_GY] * dsig);
        c[s][C_GZ] = 2.0 * (2.0 * f[s][F_GZ] * dsig);
        c[s][C_LAP] = 2.0 * dlap;
        c[s][C_KIN] = 2.0 * dlap;
        if (KV > V_T0 + s) c[s][C_KIN] += 0.5 * dv[(KV > V_T0 + s) ? V_T0 + s : 0];  // tau = 1/2 sum_j D d_j phi d_j phi
        if (poison & (1u << s)) c[s][C_RHO] = __longlong_as_double(0x7ff8000000000000ll);
      }
    }
    if (coef != nullptr) {
#pragma unroll
      for (int s = 0; s < 2; ++s)
#pragma unroll
        for (int k = 0; k < kFeat; ++k) coef[((size_t)s * kFeat + k) * np + p] = c[s][k];
    }
  }
  // Block partial sum of the weighted energy density.
  __shared__ double red[kBlock / 32];
  double v = e_r;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < kBlock / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) epart[blockIdx.x] = v;
  }
}

}  // namespace

int xc_point_blocks(int64_t np) { return (int)((np + kBlock - 1) / kBlock); }

cudaError_t launch_xc_point(const double *feat, const double *w, int64_t n_grid, int64_t np,
                            const gdft_functional &fn, const double *ehf, int n_omega, double *coef,
                            double *epart, double *dens, cudaStream_t st, double *ghf) {
  const int blocks = xc_point_blocks(np);
  bool reads_tau = false;
  for (int i = 0; i < fn.n_cols; ++i) reads_tau |= is_uw_col(fn.cols[i]) && uw_j(fn.cols[i]) != 0;
  if (reads_tau)
    xc_point_kernel<8><<<blocks, kBlock, 0, st>>>(feat, w, n_grid, np, fn, ehf, n_omega, coef, epart, dens, ghf);
  else
    xc_point_kernel<6><<<blocks, kBlock, 0, st>>>(feat, w, n_grid, np, fn, ehf, n_omega, coef, epart, dens, ghf);
  return cudaGetLastError();
}

}  // namespace gdft
