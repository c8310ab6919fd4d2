// kpoint.cu - the k-point (Solid) XC path on the real kernels.
//
// For crystal AOs phi_k = A + iB (complex, per k-point) and a complex density
// matrix D_k = X + iY, the reference's densities are bilinear forms without
// conjugation (solid.py:491-632), e.g.
//   rho_s(r) = Re sum_k w_k sum_ab D_s,k[a][b] phi_k,a(r) phi_k,b(r),
// and Re(D phi_a phi_b) = X (A_a A_b - B_a B_b) - Y (A_a B_b + B_a A_b).  So with
// the doubled real basis psi_k = [A | B] (2n functions) and the real matrix
//   M_s,k = w_k [[X, -Y], [-Y, -X]]   (2n x 2n)
// every density feature is the molecule formula on (psi_k, M_s,k), summed over k.
// jax.grad with respect to a complex D (train.py:86 with a Solid) returns
// dE/dX - i dE/dY; from the real V_s,k = dE/dM_s,k (blocks V11 V12 / V21 V22):
//   dE/dD_s,k = w_k ((V11 - V22) + i (V12 + V21)).
#include "common.cuh"
#include "kernels.cuh"

namespace gdft {

namespace {

// M (2, 2n, 2n) of k-point k from the interleaved complex rdm1 (2, K, n, n).
__global__ void kpt_build_m_kernel(const double *__restrict__ rdm1c, int K, int k, int n, double wk,
                                   double *__restrict__ M) {
  const int n2 = 2 * n;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)2 * n2 * n2) return;
  const int s = (int)(idx / ((size_t)n2 * n2));
  const int i = (int)((idx / n2) % n2), j = (int)(idx % n2);
  const int a = i % n, b = j % n, bi = i / n, bj = j / n;
  const double *z = rdm1c + 2 * ((((size_t)s * K + k) * n + a) * n + b);
  double v;
  if (bi == bj)
    v = bi == 0 ? z[0] : -z[0];
  else
    v = -z[1];
  M[idx] = wk * v;
}

__global__ void feat_add_kernel(const double *__restrict__ f, double *__restrict__ sum, size_t count, int first) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= count) return;
  sum[idx] = first ? f[idx] : sum[idx] + f[idx];
}

// Interleaved complex vxc (2, K, n, n) of k-point k from the real V (2, 2n, 2n).
__global__ void kpt_vxc_kernel(const double *__restrict__ V, int K, int k, int n, double wk,
                               double *__restrict__ vxc) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)2 * n * n) return;
  const int s = (int)(idx / ((size_t)n * n));
  const int a = (int)((idx / n) % n), b = (int)(idx % n);
  const int n2 = 2 * n;
  const double *Vs = V + (size_t)s * n2 * n2;
  const double v11 = Vs[(size_t)a * n2 + b], v22 = Vs[(size_t)(a + n) * n2 + b + n];
  const double v12 = Vs[(size_t)a * n2 + b + n], v21 = Vs[(size_t)(a + n) * n2 + b];
  double *z = vxc + 2 * ((((size_t)s * K + k) * n + a) * n + b);
  z[0] = wk * (v11 - v22);
  z[1] = wk * (v12 + v21);
}

// v_k[i][j] = w_k sum_(q,l,m) rep[k][q][i][j][l][m] D_q[m][l] with D = rdm1 summed over
// spin (solid.py:302-330, "k,kqijlm,qml->kij"); complex interleaved.  One thread per (k, i, j).
__global__ void kpt_coulomb_kernel(const double *__restrict__ rep, const double *__restrict__ rdm1c,
                                   const double *__restrict__ w, int K, int n, double *__restrict__ vj) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)K * n * n) return;
  const int k = (int)(idx / ((size_t)n * n)), i = (int)((idx / n) % n), j = (int)(idx % n);
  double re = 0.0, im = 0.0;
  const size_t nn = (size_t)n * n;
  for (int q = 0; q < K; ++q) {
    const double *r = rep + 2 * ((((size_t)k * K + q) * n + i) * n + j) * nn;
    const double *d0 = rdm1c + 2 * ((size_t)(0 * K + q) * nn);
    const double *d1 = rdm1c + 2 * ((size_t)(1 * K + q) * nn);
    for (int l = 0; l < n; ++l)
      for (int m = 0; m < n; ++m) {
        const size_t lm = (size_t)l * n + m, ml = (size_t)m * n + l;
        const double dr = d0[2 * ml] + d1[2 * ml], di = d0[2 * ml + 1] + d1[2 * ml + 1];
        const double rr = r[2 * lm], ri = r[2 * lm + 1];
        re = fma(rr, dr, fma(-ri, di, re));
        im = fma(rr, di, fma(ri, dr, im));
      }
  }
  vj[2 * idx] = w[k] * re;
  vj[2 * idx + 1] = w[k] * im;
}

// E_nuc + Re sum_k w_k tr(D_k h_k) + Re sum_k w_k tr(D_k v_k) / 2 (solid.py:272-411), one block, fixed order.
__global__ void __launch_bounds__(256) kpt_nonxc_kernel(const double *__restrict__ rdm1c,
                                                        const double *__restrict__ h1e,
                                                        const double *__restrict__ vj, const double *__restrict__ w,
                                                        int K, int n, double e_nuc, double *__restrict__ out) {
  __shared__ double red[256];
  const size_t nn = (size_t)n * n, total = (size_t)K * nn;
  double acc = 0.0;
  for (size_t idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int k = (int)(idx / nn), i = (int)((idx / n) % n), j = (int)(idx % n);
    const size_t ij = (size_t)k * nn + (size_t)i * n + j, ji = (size_t)k * nn + (size_t)j * n + i;
    const double dr = rdm1c[2 * ij] + rdm1c[2 * (total + ij)];
    const double di = rdm1c[2 * ij + 1] + rdm1c[2 * (total + ij) + 1];
    const double hr = h1e[2 * ji], hi = h1e[2 * ji + 1];
    const double vr = vj[2 * ji], vi = vj[2 * ji + 1];
    acc += w[k] * ((dr * hr - di * hi) + 0.5 * (dr * vr - di * vi));
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = e_nuc + red[0];
}

__device__ __forceinline__ void kclip(double &re, double &im, double clip) {
  if (!(sqrt(re * re + im * im) > clip)) re = im = 0.0;
}

// predict's Fock matrix for a Solid (train.py:147-163): F = h1e + vj + n_kpt vxc, abs_clip,
// (F + F^H)/2 over the orbital indices, abs_clip.  One thread per (spin, k, i, j).
__global__ void kpt_fock_kernel(const double *__restrict__ h1e, const double *__restrict__ vj,
                                const double *__restrict__ vxc, int K, int n, double scale, double clip,
                                double *__restrict__ fock) {
  const size_t nn = (size_t)n * n;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)2 * K * nn) return;
  const size_t sk = idx / nn;
  const int k = (int)(sk % K), i = (int)((idx / n) % n), j = (int)(idx % n);
  const size_t ij = (size_t)i * n + j, ji = (size_t)j * n + i;
  const size_t hk = (size_t)k * nn;
  double ar = h1e[2 * (hk + ij)] + vj[2 * (hk + ij)] + scale * vxc[2 * (sk * nn + ij)];
  double ai = h1e[2 * (hk + ij) + 1] + vj[2 * (hk + ij) + 1] + scale * vxc[2 * (sk * nn + ij) + 1];
  double br = h1e[2 * (hk + ji)] + vj[2 * (hk + ji)] + scale * vxc[2 * (sk * nn + ji)];
  double bi = h1e[2 * (hk + ji) + 1] + vj[2 * (hk + ji) + 1] + scale * vxc[2 * (sk * nn + ji) + 1];
  kclip(ar, ai, clip);
  kclip(br, bi, clip);
  double fr = 0.5 * (ar + br), fi = 0.5 * (ai - bi);
  kclip(fr, fi, clip);
  fock[2 * idx] = fr;
  fock[2 * idx + 1] = fi;
}

}  // namespace

cudaError_t launch_kpt_fock(const double *h1e, const double *vj, const double *vxc, int K, int n, double scale,
                            double clip, double *fock, cudaStream_t st) {
  const size_t total = (size_t)2 * K * n * n;
  kpt_fock_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(h1e, vj, vxc, K, n, scale, clip, fock);
  return cudaGetLastError();
}

cudaError_t launch_kpt_coulomb(const double *rep, const double *rdm1c, const double *w, int K, int n, double *vj,
                               cudaStream_t st) {
  const size_t total = (size_t)K * n * n;
  kpt_coulomb_kernel<<<(unsigned)((total + 127) / 128), 128, 0, st>>>(rep, rdm1c, w, K, n, vj);
  return cudaGetLastError();
}

cudaError_t launch_kpt_nonxc(const double *rdm1c, const double *h1e, const double *vj, const double *w, int K, int n,
                             double e_nuc, double *out, cudaStream_t st) {
  kpt_nonxc_kernel<<<1, 256, 0, st>>>(rdm1c, h1e, vj, w, K, n, e_nuc, out);
  return cudaGetLastError();
}

cudaError_t launch_kpt_build_m(const double *rdm1c, int K, int k, int n, double wk, double *M, cudaStream_t st) {
  const size_t total = (size_t)2 * 4 * n * n;
  kpt_build_m_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(rdm1c, K, k, n, wk, M);
  return cudaGetLastError();
}

cudaError_t launch_feat_add(const double *f, double *sum, size_t count, bool first, cudaStream_t st) {
  feat_add_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(f, sum, count, first ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_kpt_vxc(const double *V, int K, int k, int n, double wk, double *vxc, cudaStream_t st) {
  const size_t total = (size_t)2 * n * n;
  kpt_vxc_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(V, K, k, n, wk, vxc);
  return cudaGetLastError();
}

}  // namespace gdft
