// nu_kernels.cuh - device side of the range-separated integrals (nu.cu, nu_f.cu):
// constants, the Boys function, Hermite Coulomb integrals and the per-class
// integral kernel (one warp per shell pair, lanes = 32 grid points).
#pragma once

#include "common.cuh"
#include "shells.cuh"

namespace gdft {
namespace nu_detail {

constexpr int kNuMaxL = 3;                 // shells up to f
constexpr int kMaxOmega = 8;               // omegas of one gdft_chi call
constexpr int kBoysN = 17;                 // F_0 .. F_16 tabulated
constexpr int kBoysPts = 601;              // T = 0, 0.1, ..., 60
constexpr double kBoysStep = 0.1;
constexpr double kBoysTMax = 60.0;
constexpr int kETab = 4 * 4 * 7;           // E[i][j][t], i, j <= 3, t <= 6 (per dimension)

// Hermite products pref * E^x_t E^y_u E^z_v of a primitive pair of angular momenta
// (la, lb): for each pair of cartesian components, (ia+ib+1)(ka+kb+1)(ma+mb+1) terms.
__host__ __device__ constexpr int nprod(int la, int lb) {
  int n = 0;
  for (int ia = la; ia >= 0; --ia)
    for (int ka = la - ia; ka >= 0; --ka)
      for (int ib = lb; ib >= 0; --ib)
        for (int kb = lb - ib; kb >= 0; --kb) n += (ia + ib + 1) * (ka + kb + 1) * (la - ia - ka + lb - ib - kb + 1);
  return n;
}
// A primitive-pair record: mu, screened flag, P(3), p, 2 pad, then the products.
__host__ __device__ constexpr int rec_len(int la, int lb) { return 8 + nprod(la, lb); }
constexpr double kPi = 3.14159265358979323846;
constexpr double kScreen = 1e-30;          // product-overlap prefactor below which a primitive pair is skipped

// F_0 .. F_L at T.
template <int L>
__device__ __forceinline__ void boys(const double *__restrict__ tab, double T, double F[L + 1]) {
  if (T < kBoysTMax) {
    const int i = (int)(T * (1.0 / kBoysStep) + 0.5);
    const double md = i * kBoysStep - T;  // -(T - T_i)
    const double *row = tab + i * kBoysN + L;
    // sum_k F_(L+k)(T_i) (-(T - T_i))^k / k!, Horner from k = 8
    constexpr double inv_fact[9] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040,
                                    1.0 / 40320};
    double acc = row[8] * inv_fact[8];
#pragma unroll
    for (int k = 7; k >= 0; --k) acc = fma(acc, md, row[k] * inv_fact[k]);
    F[L] = acc;
    if (L > 0) {
      const double e = exp(-T);
#pragma unroll
      for (int n = L - 1; n >= 0; --n) F[n] = fma(2.0 * T, F[n + 1], e) * (1.0 / (2 * n + 1));
    }
  } else {
    F[0] = 0.5 * sqrt(kPi / T);
    const double h = 0.5 / T;
#pragma unroll
    for (int n = 0; n < L; ++n) F[n + 1] = F[n] * ((2 * n + 1) * h);
  }
}

__device__ __forceinline__ int e_idx(int i, int j, int t) { return (i * 4 + j) * 7 + t; }

template <int L>
struct CartPow {
  // exponents of the ncart(L) monomials in PySCF's order
  static constexpr int n = (L + 1) * (L + 2) / 2;
  static __device__ __forceinline__ constexpr int x(int q) {
    int idx = 0;
    for (int lx = L; lx >= 0; --lx)
      for (int ly = L - lx; ly >= 0; --ly) {
        if (idx == q) return lx;
        ++idx;
      }
    return 0;
  }
  static __device__ __forceinline__ constexpr int y(int q) {
    int idx = 0;
    for (int lx = L; lx >= 0; --lx)
      for (int ly = L - lx; ly >= 0; --ly) {
        if (idx == q) return ly;
        ++idx;
      }
    return 0;
  }
  static __device__ __forceinline__ constexpr int z(int q) { return L - x(q) - y(q); }
};

// Hermite Coulomb integrals R^0_tuv, t + u + v <= L.
template <int L>
__device__ __forceinline__ void hermite_r(const double F[L + 1], double mu, double X, double Y, double Z,
                                          double R[L + 1][L + 1][L + 1]) {
  double nxt[L + 1][L + 1][L + 1];
  double m2 = 1.0;
#pragma unroll
  for (int n = 0; n < L; ++n) m2 *= -2.0 * mu;
  nxt[0][0][0] = m2 * F[L];
#pragma unroll
  for (int n = L - 1; n >= 0; --n) {
    double cur[L + 1][L + 1][L + 1];
    const int top = L - n;
#pragma unroll
    for (int t = 0; t <= L; ++t)
#pragma unroll
      for (int u = 0; u <= L; ++u)
#pragma unroll
        for (int v = 0; v <= L; ++v) {
          if (t + u + v > top) continue;
          double val;
          if (t > 0)
            val = (t > 1 ? (t - 1) * nxt[t > 1 ? t - 2 : 0][u][v] : 0.0) + X * nxt[t - 1][u][v];
          else if (u > 0)
            val = (u > 1 ? (u - 1) * nxt[0][u > 1 ? u - 2 : 0][v] : 0.0) + Y * nxt[0][u - 1][v];
          else if (v > 0)
            val = (v > 1 ? (v - 1) * nxt[0][0][v > 1 ? v - 2 : 0] : 0.0) + Z * nxt[0][0][v - 1];
          else {
            double m = 1.0;
#pragma unroll
            for (int k = 0; k < n; ++k) m *= -2.0 * mu;
            val = m * F[n];
          }
          cur[t][u][v] = val;
        }
#pragma unroll
    for (int t = 0; t <= L; ++t)
#pragma unroll
      for (int u = 0; u <= L; ++u)
#pragma unroll
        for (int v = 0; v <= L; ++v)
          if (t + u + v <= top) nxt[t][u][v] = cur[t][u][v];
  }
#pragma unroll
  for (int t = 0; t <= L; ++t)
#pragma unroll
    for (int u = 0; u <= L; ++u)
#pragma unroll
      for (int v = 0; v <= L; ++v)
        if (t + u + v <= L) R[t][u][v] = nxt[t][u][v];
}

struct NuOut {
  double *nu;      // nu[(a * n + b) * s_ab + p * s_p]
  int64_t s_ab, s_p;
  int n;
};

// One warp per shell pair of class (LA, LB), lanes = 32 points from p0.
template <int LA, int LB>
__global__ void __launch_bounds__(256) nu_kernel(ShellView B, const int32_t *__restrict__ pairs, int pair_lo,
                                                 int pair_hi, const double *__restrict__ pp, int64_t n_pp,
                                                 const double *__restrict__ boys_tab,
                                                 const double *__restrict__ coords, int64_t p_begin, int64_t n_pts,
                                                 NuOut out) {
  constexpr int L = LA + LB;
  constexpr int NA = CartPow<LA>::n, NB = CartPow<LB>::n;
  const int lane = threadIdx.x & 31;
  const int ip = pair_lo + blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (ip >= pair_hi) return;  // whole warps leave together
  const int64_t pl = (int64_t)blockIdx.x * 32 + lane;  // point within the chunk
  const bool live = pl < n_pts;
  double Cx = 0.0, Cy = 0.0, Cz = 0.0;
  if (live) {
    const int64_t p = p_begin + pl;
    Cx = coords[3 * p];
    Cy = coords[3 * p + 1];
    Cz = coords[3 * p + 2];
  }
  const int s1 = pairs[4 * ip], s2 = pairs[4 * ip + 1];
  const int64_t off = pairs[4 * ip + 2];
  shells_detail::ShellRec r1, r2;
  if (!shells_detail::load_shell(B, s1, r1) || !shells_detail::load_shell(B, s2, r2)) return;
  constexpr int kLen = rec_len(LA, LB);
  if (r1.l != LA || r2.l != LB || off < 0 || off + (int64_t)r1.np * r2.np * kLen > n_pp) return;
  if (r1.ncomp > NA || r2.ncomp > NB) return;
  for (int c1 = 0; c1 < r1.nctr; ++c1) {
    for (int c2 = 0; c2 < r2.nctr; ++c2) {
      double cart[NA][NB];
#pragma unroll
      for (int qa = 0; qa < NA; ++qa)
#pragma unroll
        for (int qb = 0; qb < NB; ++qb) cart[qa][qb] = 0.0;
      for (int i1 = 0; i1 < r1.np; ++i1) {
        const double ca = B.coef[r1.coff + (int64_t)c1 * r1.np + i1];
        for (int i2 = 0; i2 < r2.np; ++i2) {
          const double *rec = pp + off + ((int64_t)i1 * r2.np + i2) * kLen;
          if (rec[1] != 0.0) continue;  // screened (uniform across the warp)
          const double cc = ca * B.coef[r2.coff + (int64_t)c2 * r2.np + i2];
          const double mu = rec[0];
          const double X = rec[2] - Cx, Y = rec[3] - Cy, Z = rec[4] - Cz;
          double F[L + 1];
          boys<L>(boys_tab, mu * (X * X + Y * Y + Z * Z), F);
          double R[L + 1][L + 1][L + 1];
          hermite_r<L>(F, mu, X, Y, Z, R);
          const double *E3 = rec + 8;
          int idx = 0;
#pragma unroll
          for (int qa = 0; qa < NA; ++qa) {
            const int ia = CartPow<LA>::x(qa), ka = CartPow<LA>::y(qa), ma = CartPow<LA>::z(qa);
#pragma unroll
            for (int qb = 0; qb < NB; ++qb) {
              const int ib = CartPow<LB>::x(qb), kb = CartPow<LB>::y(qb), mb = CartPow<LB>::z(qb);
              double s = 0.0;
#pragma unroll
              for (int t = 0; t <= L; ++t) {
                if (t > ia + ib) continue;
#pragma unroll
                for (int u = 0; u <= L; ++u) {
                  if (u > ka + kb) continue;
#pragma unroll
                  for (int v = 0; v <= L; ++v) {
                    if (v > ma + mb) continue;
                    s = fma(E3[idx], R[t][u][v], s);
                    ++idx;
                  }
                }
              }
              cart[qa][qb] = fma(cc, s, cart[qa][qb]);
            }
          }
        }
      }
      // angular rows on both sides, then the symmetric writes
      const double *T1 = B.trans + r1.toff, *T2 = B.trans + r2.toff;
      for (int k1 = 0; k1 < r1.ncomp; ++k1) {
        double h[NB];
#pragma unroll
        for (int qb = 0; qb < NB; ++qb) {
          double acc = 0.0;
#pragma unroll
          for (int qa = 0; qa < NA; ++qa) acc = fma(T1[k1 * NA + qa], cart[qa][qb], acc);
          h[qb] = acc;
        }
        const int a = r1.aoff + c1 * r1.ncomp + k1;
        for (int k2 = 0; k2 < r2.ncomp; ++k2) {
          double v = 0.0;
#pragma unroll
          for (int qb = 0; qb < NB; ++qb) v = fma(T2[k2 * NB + qb], h[qb], v);
          const int b = r2.aoff + c2 * r2.ncomp + k2;
          if (live) {
            out.nu[((int64_t)a * out.n + b) * out.s_ab + pl * out.s_p] = v;
            out.nu[((int64_t)b * out.n + a) * out.s_ab + pl * out.s_p] = v;
          }
        }
      }
    }
  }
}

// Launch the kernel of class (LA, LB) over pairs [lo, hi) and the points of a chunk.
template <int LA, int LB>
cudaError_t launch_nu_class(const ShellView &B, const int32_t *pairs, int lo, int hi, const double *pp, int64_t n_pp,
                            const double *boys_tab, const double *coords, int64_t p_begin, int64_t n_pts, NuOut out,
                            cudaStream_t st) {
  const dim3 grid((unsigned)((n_pts + 31) / 32), (unsigned)((hi - lo + 7) / 8));
  nu_kernel<LA, LB><<<grid, 256, 0, st>>>(B, pairs, lo, hi, pp, n_pp, boys_tab, coords, p_begin, n_pts, out);
  return cudaGetLastError();
}

// Classes with an f shell (nu_f.cu): class index LA * (LA + 1) / 2 + LB for LA = 3.
cudaError_t launch_nu_f_class(int la, int lb, const ShellView &B, const int32_t *pairs, int lo, int hi,
                              const double *pp, int64_t n_pp, const double *boys_tab, const double *coords,
                              int64_t p_begin, int64_t n_pts, NuOut out, cudaStream_t st);

// The f-d class (nu_fd.cu).
cudaError_t launch_nu_fd(const ShellView &B, const int32_t *pairs, int lo, int hi, const double *pp, int64_t n_pp,
                         const double *boys_tab, const double *coords, int64_t p_begin, int64_t n_pts, NuOut out,
                         cudaStream_t st);

// The f-f class (nu_ff.cu).
cudaError_t launch_nu_ff(const ShellView &B, const int32_t *pairs, int lo, int hi, const double *pp, int64_t n_pp,
                         const double *boys_tab, const double *coords, int64_t p_begin, int64_t n_pts, NuOut out,
                         cudaStream_t st);

}  // namespace nu_detail
}  // namespace gdft
