// kernels.cuh - launchers shared between the translation units.
#pragma once

#include "common.cuh"
#include "shells.cuh"

namespace gdft {

// ao.cu
cudaError_t launch_load_tables(const double *ao, const double *grad_ao, const double *grad2_ao, const double *w,
                               int64_t n_grid, int n_ao, int64_t np, int ld, double *tab, double *wout,
                               cudaStream_t st);
cudaError_t launch_eval_basis(const double *basis, const double *coords, const double *w, int64_t n_grid, int n_ao,
                              int64_t np, int ld, double *tab, double *wout, cudaStream_t st);
// Contracted shells: reference layouts (eval_ao / ao_grads) and the FP64 planes.
cudaError_t launch_eval_ao(const ShellView &B, const double *coords, int64_t n_grid, int deriv, double *ao,
                           double *g1, double *g2, cudaStream_t st);
cudaError_t launch_eval_shell_tables(const ShellView &B, const double *coords, const double *w, int64_t n_grid,
                                     int64_t np, int ld, double *tab, double *wout, cudaStream_t st);

// dens_f64.cu: FP64 form of the density contraction -> feat[2][6][np].
cudaError_t launch_dens_f64(const double *tab, int64_t np, int ld, int n_ao, const double *rdm1, double *feat,
                            cudaStream_t st);

// vxc_f64.cu: FP64 form of the V_xc contraction -> vpart[nsplit][2][n][n].
int vxc_f64_splits(int64_t np, int n_ao);
cudaError_t launch_vxc_f64(const double *tab, int64_t np, int ld, int n_ao, const double *coef, int nsplit,
                           double *vpart, cudaStream_t st);

// tc_pack.cu / dens_tc.cu: TF32x3 form.
cudaError_t launch_pack_tables(const double *ao, const double *grad_ao, const double *grad2_ao, const double *basis,
                               const double *coords, const double *w, int64_t n_grid, int n_ao, int64_t np, int ldk,
                               float *pm, float *av, float *af, double *wout, cudaStream_t st,
                               const ShellView *shells = nullptr);
cudaError_t launch_pack_rdm1(const double *D, int n, int ldk, float *out, cudaStream_t st);
cudaError_t launch_dens_tc(const float *pm, const float *dpk, int64_t np, int ldk, double *feat, int *err,
                           cudaStream_t st);
// One persistent launch of the same kernel over several molecules' 128-point
// tiles (a device work queue, the molecules with the largest n_ao first): each
// molecule's features go to feat with row stride ldf.  d_scratch holds
// dens_ragged_scratch_bytes(n_mol) bytes (256-byte aligned).
struct DensMol {
  const float *pm;   // point-major resident tables
  const float *dpk;  // packed rdm1 (launch_pack_rdm1)
  int64_t np;        // padded grid points (multiple of 128)
  int ldk;           // n_ao rounded up to 128
  double *feat;      // [2][6][ldf]
  int64_t ldf;
};
size_t dens_ragged_scratch_bytes(int n_mol);
cudaError_t launch_dens_tc_ragged(const DensMol *mols, int n_mol, void *d_scratch, int *err, cudaStream_t st);

// vxc_q.cu: mixed V_xc as Q pre-pass + block-scaled three-slice tensor-core GEMM.
int vxc_q_splits(int64_t np, int n_ao);
size_t vxc_q_bytes(int64_t np, int n_ao);
cudaError_t launch_vxc_q_tc(const float *av, const float *af, const double *coef, int64_t np,
                            int ldk, int n_ao, float *q, int nsplit, double *vpart, double *vxc, int *err,
                            cudaStream_t st);

// kpoint.cu: the doubled real form of a k-point's complex density matrix and gradient.
cudaError_t launch_kpt_build_m(const double *rdm1c, int K, int k, int n, double wk, double *M, cudaStream_t st);
cudaError_t launch_feat_add(const double *f, double *sum, size_t count, bool first, cudaStream_t st);
cudaError_t launch_kpt_vxc(const double *V, int K, int k, int n, double wk, double *vxc, cudaStream_t st);
cudaError_t launch_kpt_coulomb(const double *rep, const double *rdm1c, const double *w, int K, int n, double *vj,
                               cudaStream_t st);
cudaError_t launch_kpt_fock(const double *h1e, const double *vj, const double *vxc, int K, int n, double scale,
                            double clip, double *fock, cudaStream_t st);
cudaError_t launch_kpt_nonxc(const double *rdm1c, const double *h1e, const double *vj, const double *w, int K, int n,
                             double e_nuc, double *out, cudaStream_t st);

// xc_point.cu
int xc_point_blocks(int64_t np);
cudaError_t launch_xc_point(const double *feat, const double *w, int64_t n_grid, int64_t np,
                            const gdft_functional &fn, const double *ehf, int n_omega, double *coef,
                            double *epart, double *dens, cudaStream_t st, double *ghf = nullptr);

// tc_selftest.cu: a bounded wait that runs out on purpose (failure-detection test).
cudaError_t launch_wait_expiry_probe(int *err, uint32_t limit, int code, cudaStream_t st);

// reduce.cu
int integrate_blocks(int64_t n_grid);
cudaError_t launch_pad_potentials(const double *pot, int64_t n_grid, int64_t np, double *coef, cudaStream_t st);
cudaError_t launch_integrate(int64_t n_grid, int n_cols, const gdft_functional &fn, const double *dens,
                             const double *w, double *epart, cudaStream_t st);
cudaError_t launch_energy_reduce(const double *epart, int n, double *exc, cudaStream_t st);
cudaError_t launch_err_fold(int *dst, int *src, cudaStream_t st);
cudaError_t launch_vxc_reduce(const double *vpart, int nsplit, int n_ao, double *vxc, cudaStream_t st);
cudaError_t launch_feat_to_reference(const double *feat, int64_t n_grid, int64_t np, double *rho, double *grad_rho,
                                     double *lapl, double *tau, cudaStream_t st);
cudaError_t launch_fock(int n_ao, const double *h1e, const double *vj, const double *vxc, double clip, double *fock,
                        cudaStream_t st);
cudaError_t launch_coulomb(int n_ao, const double *eri, const double *rdm1, const double *h1e, double enuc,
                           double *vj, double *enonxc, cudaStream_t st);

}  // namespace gdft
