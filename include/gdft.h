/*
 * gdft.h - C ABI of the GB300 XC grid path (libgdft_xc.so).
 *
 * The reference (Grad DFT) is pure Python/JAX and has no native interface;
 * each entry point below replaces one Python/JAX function of the XC path and
 * keeps its argument meaning.  Citations are file:line in the GradDFT tree.
 *
 * Conventions
 *  - Every pointer argument named d_* is DEVICE memory; h_* is host memory.
 *  - All floating-point inputs and outputs are IEEE float64 in the
 *    reference's own layouts (Molecule.ao (grid, ao), grad_ao (grid, ao, 3),
 *    grad_n_ao[2] (grid, ao, 3), rdm1 (2, ao, ao), row-major).
 *  - Work is enqueued on the caller's CUDA stream; nothing synchronises the
 *    host except where a function says so.
 *  - The library allocates no device memory: molecules live in a
 *    caller-provided buffer (gdft_molecule_bytes) and every call takes a
 *    caller-provided workspace (gdft_workspace_bytes).
 *  - Return value: GDFT_OK or an error code; gdft_last_error() gives the
 *    message of the calling thread's last failure.
 */
#ifndef GDFT_H_
#define GDFT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GDFT_ABI_VERSION 2

/* Status codes (the Python layer maps them to ValueError/TypeError/RuntimeError,
 * as the reference raises ValueError at functional.py:583, molecule.py:174-180). */
enum {
  GDFT_OK = 0,
  GDFT_ERR_INVALID = 1,     /* bad shape or argument                          */
  GDFT_ERR_ALIGNMENT = 2,   /* pointer not aligned as required                */
  GDFT_ERR_WORKSPACE = 3,   /* workspace or buffer too small                  */
  GDFT_ERR_CUDA = 4,        /* a CUDA runtime call failed                     */
  GDFT_ERR_DEVICE = 5,      /* a kernel reported an error word (bounded wait)  */
  GDFT_ERR_UNSUPPORTED = 6  /* functional/precision combination not built     */
};

/* Arithmetic forms of the path. */
enum {
  GDFT_FP64 = 0,    /* plain FP64 form: FP64 contractions and FP64 point work      */
  GDFT_TF32X3 = 1   /* mixed form: tcgen05 TF32 3-term split products, FP32
                       accumulation inside a K-chunk, FP64 across chunks       */
};

/* Energy-density columns (popular_functionals.py:29-326, functional.py:534-675). */
enum {
  GDFT_COL_LSDA = 0,     /* lsda_x_e               popular_functionals.py:29-50   */
  GDFT_COL_B88 = 1,      /* b88_x_e (correction)   popular_functionals.py:52-103  */
  GDFT_COL_VWN = 2,      /* vwn_c_e                popular_functionals.py:141-195 */
  GDFT_COL_LYP = 3,      /* lyp_c_e                popular_functionals.py:197-269 */
  GDFT_COL_PW92 = 4,     /* pw92_c_e               popular_functionals.py:105-139 */
  GDFT_COL_HF = 5,       /* sum_{omega,spin} ehf   popular_functionals.py:328-334 */
  GDFT_COL_DM21_LDA = 6, /* dm21_densities 'LDA'   functional.py:534-626          */
  GDFT_COL_HF_W0 = 7,    /* sum_spin ehf[0]        functional.py:652-675          */
  GDFT_COL_HF_W1 = 8,    /* sum_spin ehf[1]        functional.py:652-675          */
  GDFT_COL_ZERO = 9      /* the correlation features of densities() (functional.py:1146-1200):
                            e_PW92 < 0 is rounded to a multiple of 10^(-int(log10 clip)) and
                            compared with clip > 0 (:1188-1197), so they are identically 0 and
                            carry no gradient                                           */
};

/* Feature-power columns u^i w^j of dm21_densities and densities() for any
 * u_range / w_range (functional.py:534-626, 1048-1142), 0 <= i, j <= 15:
 *  - GDFT_COL_DM21_UW(i, j): sum over spin of 2^(4/3 log rho + i log u + j log w),
 *    times -2 pi (3/(4 pi))^(4/3) for i = j = 0 (dm21_densities, :616-624);
 *  - GDFT_COL_DENS_X(s, i, j): the same term for spin s alone with the MGGA
 *    variable of densities() (log 1/t = log tau - 5/3 log rho, :1119),
 *    unscaled (:1130-1134). */
#define GDFT_COL_DM21_UW(i, j) (0x100 | ((i) << 4) | (j))
#define GDFT_COL_DENS_X(s, i, j) (0x200 | ((s) << 8) | ((i) << 4) | (j))

#define GDFT_MAX_COLS 16

/* A functional with constant coefficients: Functional(coefficients=lambda: c,
 * energy_densities=stack of columns) (functional.py:128-141, popular_functionals.py:375-393).
 * A single coefficient broadcasts over all columns, as jnp.einsum("rf,rf->r")
 * broadcasts the [[1.0]] row in the reference. */
typedef struct gdft_functional {
  int32_t n_cols;
  int32_t cols[GDFT_MAX_COLS];
  int32_t n_coeffs;                 /* 1 (broadcast) or n_cols */
  double coeffs[GDFT_MAX_COLS];
  double clip;                      /* clip_cte, 1e-30 in the reference */
} gdft_functional;

/* A molecule resident on the device in the library's layout: the Molecule
 * fields the XC path reads (molecule.py:72-106: grid.weights, ao, grad_ao,
 * grad_n_ao[2]).  Filled by gdft_molecule_init; opaque beyond these fields. */
typedef struct gdft_molecule {
  int64_t n_grid;      /* grid points                                   */
  int64_t n_grid_pad;  /* grid points rounded up to the tile (128)      */
  int32_t n_ao;        /* atomic orbitals                               */
  int32_t ld;          /* AO leading dimension (n_ao rounded up to 32)  */
  int32_t precision;   /* GDFT_FP64 or GDFT_TF32X3                      */
  int32_t reserved;
  void *buffer;        /* device buffer of gdft_molecule_bytes bytes    */
  size_t buffer_bytes;
} gdft_molecule;

int gdft_abi_version(void);
const char *gdft_last_error(void);

/* Size of the device buffer that holds a molecule in the library's layout. */
int gdft_molecule_bytes(int64_t n_grid, int32_t n_ao, int32_t precision, size_t *bytes);

/* Bind a caller buffer to a molecule descriptor (no device work). */
int gdft_molecule_init(gdft_molecule *mol, int64_t n_grid, int32_t n_ao, int32_t precision,
                       void *d_buffer, size_t buffer_bytes);

/* Load Molecule.ao, grad_ao, grad_n_ao[2] and grid.weights (reference layouts,
 * molecule.py:72-106) into the molecule: the host-side analogue is
 * interface/pyscf.py:639-654 to_device_arrays.  d_grad2_ao may be NULL when
 * no functional needs the Laplacian. */
int gdft_molecule_load(const gdft_molecule *mol, const double *d_ao, const double *d_grad_ao,
                       const double *d_grad2_ao, const double *d_weights, void *stream);

/* Evaluate a Gaussian basis on the grid directly into the molecule (stands in
 * for numint.eval_ao, interface/pyscf.py:849-852, and ao_grads(order=2),
 * :677-705).  d_basis: (n_ao, 8) rows cx, cy, cz, alpha, norm, kind, comp, 0;
 * d_coords: (n_grid, 3) bohr. */
int gdft_molecule_eval_basis(const gdft_molecule *mol, const double *d_basis, const double *d_coords,
                             const double *d_weights, void *stream);

/* A contracted Gaussian basis on the device: the functions numint.eval_ao
 * evaluates (interface/pyscf.py:849-852).  Shell s (row s of d_shell: l,
 * nprim, exponent offset, coefficient offset, first AO, ncomp, nctr, row
 * offset) owns the nctr * ncomp consecutive AOs from its first AO on,
 * contraction-major; its AO for contraction c and component k is
 *   phi(r) = sum_p coef[coff + c*nprim + p] exp(-exp[poff + p] |r - R_s|^2)
 *            * sum_(i,j,k) trans[roff + k*ncart + q] x^i y^j z^k,   (x, y, z) = r - R_s,
 * q running over the ncart = (l+1)(l+2)/2 exponents (i, j, k) of degree l in
 * the order i = l..0, then j = l-i..0 (PySCF's cartesian order).  The
 * angular rows carry the convention (real solid harmonics or cartesians).
 * Shells follow each other in AO order.  d_ao row a: shell, contraction,
 * component, 0.  All pointers are device pointers; l <= 6.  An AO whose
 * entries fall outside the tables evaluates to NaN (the kernels never read
 * outside them). */
typedef struct gdft_basis {
  int32_t n_shell;
  int32_t n_ao;
  int64_t n_prim;          /* length of d_exp                                         */
  int64_t n_coef;          /* length of d_coef                                        */
  int64_t n_trans;         /* length of d_trans                                       */
  const int32_t *d_shell;  /* (n_shell, 8)                                            */
  const double *d_centre;  /* (n_shell, 3) bohr                                       */
  const double *d_exp;
  const double *d_coef;
  const int32_t *d_ao;     /* (n_ao, 4): shell, contraction, component, 0               */
  const double *d_trans;
} gdft_basis;

/* numint.eval_ao(mol, coords, deriv) for deriv 0 or 1 (interface/pyscf.py:849-852,
 * the derivative axis moved last as the Molecule stores it) and, for deriv 2,
 * the diagonal second derivatives of ao_grads(mol, coords, order=2)[2]
 * (interface/pyscf.py:677-705).  d_coords: (n_grid, 3) bohr; d_ao: (n_grid, n_ao);
 * d_grad_ao (deriv >= 1), d_grad2_ao (deriv 2): (n_grid, n_ao, 3). */
int gdft_eval_ao(const gdft_basis *basis, const double *d_coords, int64_t n_grid, int32_t deriv, double *d_ao,
                 double *d_grad_ao, double *d_grad2_ao, void *stream);

/* Evaluate a contracted basis on the grid directly into the molecule (both
 * arithmetic forms): phi, its gradient and Laplacian, with no reference-layout
 * tables in between.  basis->n_ao must equal the molecule's n_ao. */
int gdft_molecule_eval_shells(const gdft_molecule *mol, const gdft_basis *basis, const double *d_coords,
                              const double *d_weights, void *stream);

/* k-points (the Solid path, solid.py:100-260 and train.py:124-163 with a Solid).
 * Each k-point is a molecule of 2n "AOs": the real and imaginary parts of the
 * n crystal AOs, [Re phi_k | Im phi_k] (loaded with gdft_molecule_load from the
 * (grid, 2n) real and imaginary parts side by side); all k-points share the grid
 * and the form.  d_rdm1: (2, n_kpt, n, n) complex128 (interleaved re, im);
 * h_kweights: n_kpt host doubles (KPointInfo.weights).  The densities are the
 * reference's unconjugated bilinear forms, e.g.
 * rho = Re sum_k w_k D_k,ab phi_k,a phi_k,b (solid.py:491-632), summed over k. */
int gdft_kpoint_workspace_bytes(const gdft_molecule *mols, int32_t n_kpt, size_t *bytes);

/* density / grad_density / lapl_density / kinetic_density of a Solid (solid.py:491-632);
 * outputs as gdft_density (any may be NULL). */
int gdft_kpoint_density(const gdft_molecule *mols, int32_t n_kpt, const double *d_rdm1, const double *h_kweights,
                        double *d_rho, double *d_grad_rho, double *d_lapl, double *d_tau, void *d_ws,
                        size_t ws_bytes, void *stream);

/* xc_energy_and_grads (train.py:86-121) for a Solid and a functional with
 * constant coefficients: E_xc and d_vxc = jax.grad of E_xc with respect to the
 * complex rdm1 (JAX's convention dE/dRe - i dE/dIm), (2, n_kpt, n, n) complex128,
 * or NULL.  Columns needing HF densities are rejected (the reference's Solid
 * raises NotImplementedError for them, solid.py:228-256). */
int gdft_kpoint_xc_energy_and_grads(const gdft_molecule *mols, int32_t n_kpt, const double *d_rdm1,
                                    const double *h_kweights, const gdft_functional *fn, double *d_exc,
                                    double *d_vxc, void *d_ws, size_t ws_bytes, void *stream);

/* Coulomb potential and non-XC energy of a Solid (solid.py:272-411, complex128 interleaved):
 *   vj[k][i][j] = w_k sum_(q,l,m) rep[k][q][i][j][l][m] D_q[m][l]   (D = rdm1 summed over spin),
 *   enonxc = E_nuc + Re sum_k w_k tr(D_k h1e_k) + Re sum_k w_k tr(D_k vj_k) / 2.
 * d_rep (n_kpt, n_kpt, n, n, n, n); d_rdm1 (2, n_kpt, n, n); d_h1e (n_kpt, n, n);
 * d_kweights (n_kpt) device doubles; d_vj (n_kpt, n, n); d_enonxc one double or NULL. */
int gdft_kpoint_coulomb(int32_t n_kpt, int32_t n_ao, const double *d_rep, const double *d_rdm1, const double *d_h1e,
                        const double *d_kweights, double nuclear_repulsion, double *d_vj, double *d_enonxc,
                        void *stream);

/* predict's Fock matrix for a Solid (train.py:147-163): F = h1e + vj + n_kpt * vxc
 * (undoing the 1/n_kpt of the k-point weights in jax.grad), abs_clip, (F + F^H)/2
 * over the orbital indices, abs_clip.  d_h1e, d_vj (n_kpt, n, n), d_vxc and d_fock
 * (2, n_kpt, n, n), complex128 interleaved. */
int gdft_kpoint_fock(int32_t n_kpt, int32_t n_ao, const double *d_h1e, const double *d_vj, const double *d_vxc,
                     double clip, double *d_fock, void *stream);

/* nu integrals and the chi tensor (range-separated exact exchange inputs).
 *   nu_ab(r) = int phi_a(r') phi_b(r') erf(omega |r - r'|) / |r - r'| dr'  (omega = 0: 1/|r - r'|),
 * PySCF's int1e_grids as _evaluate_nu / _nu_chunk call it (external/_hf_density.py:17-120), and
 *   chi[r][w][s][a] = sum_(b,d) D_s[b][d] phi_b(r) nu^(omega_w)_da(r),
 * generate_chi_tensor (interface/pyscf.py:1067-1126).  Shells up to l = 3
 * (GDFT_ERR_UNSUPPORTED beyond).  Both calls read the basis's shell table back
 * to the host to plan the shell pairs and synchronise `stream` before returning. */

/* Workspace bytes: chunk = 0 for gdft_nu_integrals, the chunk of grid points
 * for gdft_chi (its nu buffer holds n_ao^2 * chunk doubles; up to 8 omegas). */
int gdft_nu_workspace_bytes(const gdft_basis *basis, int64_t chunk, size_t *bytes);

/* d_nu: (n_grid, n_ao, n_ao); omega >= 0. */
int gdft_nu_integrals(const gdft_basis *basis, const double *d_coords, int64_t n_grid, double omega, double *d_nu,
                      void *d_ws, size_t ws_bytes, void *stream);

/* d_ao: (n_grid, n_ao) phi on the grid; d_rdm1: (2, n_ao, n_ao); h_omegas: n_omega
 * host values >= 0; d_chi: (n_grid, n_omega, 2, n_ao). */
int gdft_chi(const gdft_basis *basis, const double *d_coords, const double *d_ao, const double *d_rdm1,
             int64_t n_grid, const double *h_omegas, int32_t n_omega, int64_t chunk, double *d_chi, void *d_ws,
             size_t ws_bytes, void *stream);

/* Workspace bytes for the calls below on this molecule. */
int gdft_workspace_bytes(const gdft_molecule *mol, size_t *bytes);

/* density / grad_density / lapl_density / kinetic_density (molecule.py:385-502)
 * in one pass.  Outputs (any may be NULL): rho (grid, 2), grad_rho (grid, 2, 3),
 * lapl (grid, 2), tau (grid, 2). */
int gdft_density(const gdft_molecule *mol, const double *d_rdm1, double *d_rho, double *d_grad_rho,
                 double *d_lapl, double *d_tau, void *d_ws, size_t ws_bytes, void *stream);

/* energy_predictor.xc_energy_and_grads (train.py:86-121) for a functional
 * with constant coefficients: E_xc = Functional.xc_energy (functional.py:219-253)
 * and V_xc = dE_xc/d rdm1 (raw, not symmetrised).
 * d_ehf: (n_omega, 2, grid) stop-gradient HF energy densities, needed by the
 * HF columns (NULL otherwise); n_omega its leading extent.
 * d_exc: one double; d_vxc: (2, ao, ao).  d_vxc may be NULL (energy only). */
int gdft_xc_energy_and_grads(const gdft_molecule *mol, const double *d_rdm1, const gdft_functional *fn,
                             const double *d_ehf, int32_t n_omega, double *d_exc, double *d_vxc,
                             void *d_ws, size_t ws_bytes, void *stream);

/* gdft_xc_energy_and_grads plus d_ghf (n_grid): dE_xc/d ehf[w][s][r] for a
 * functional whose HF column (GDFT_COL_HF) is ehf summed over omega and spin
 * (b3lyp_combine, popular_functionals.py:328-337), the same for every (w, s):
 * abs_clip(w_r) * [|sum_f c_f e_f(r)| > clip] * c_HF with the other columns
 * unclipped -- the gradient HF_density_grad_2_Fock takes (molecule.py:598-603)
 * with the energy densities as predict passes them (train.py:167-178). */
int gdft_xc_energy_grads_hf(const gdft_molecule *mol, const double *d_rdm1, const gdft_functional *fn,
                            const double *d_ehf, int32_t n_omega, double *d_exc, double *d_vxc, double *d_ghf,
                            void *d_ws, size_t ws_bytes, void *stream);

/* Exact-exchange terms from a supplied chi tensor (grid, omega, spin,
 * orbitals), FP64 device arrays in the reference's layouts; ao is (grid,
 * orbitals) row-major, rdm1 (2, n, n).  Workspace of
 * gdft_hf_workspace_bytes bytes (8-byte aligned).
 *   gdft_hf_energy_density: ehf (omega, 2, grid) =
 *       -1/2 einsum("rwsc,sac,ra->wsr", chi, rdm1, ao)   (molecule.py:507-541)
 *   gdft_hf_fock: fock_hf (2, n, n) =
 *       sum_w -1/2 einsum("rws,wsr,ra->wsab"...), i.e.
 *       F_s[a][b] = -1/2 sum_w sum_r ao[r][a] g[w][s][r] chi[r][w][s][b]
 *       with g = dE/d ehf (omega, 2, grid): HF_density_grad_2_Fock /
 *       HF_coefficient_input_grad_2_Fock (molecule.py:545-685) summed over
 *       omega as b3lyp_hfgrads and dm21_hfgrads_* do.
 *   gdft_fock_add_hf: fock (2, n, n) = abs_clip(fock + F + F^T, clip), the
 *       update of train.py:200-210. */
int gdft_hf_workspace_bytes(int64_t n_grid, int32_t n_ao, int32_t n_omega, size_t *bytes);
int gdft_hf_energy_density(const double *d_ao, const double *d_rdm1, const double *d_chi, int64_t n_grid,
                           int32_t n_ao, int32_t n_omega, double *d_ehf, void *d_ws, size_t ws_bytes, void *stream);
int gdft_hf_fock(const double *d_ao, const double *d_chi, const double *d_g, int64_t n_grid, int32_t n_ao,
                 int32_t n_omega, double *d_fock_hf, void *d_ws, size_t ws_bytes, void *stream);
int gdft_fock_add_hf(double *d_fock, const double *d_fock_hf, int32_t n_ao, double clip, void *stream);
/* The same two contractions in either arithmetic form (the three entries above
 * are the GDFT_FP64 form).  GDFT_TF32X3 runs both on the block-scaled
 * three-slice tcgen05 GEMM (FP64 inputs and outputs; the products are exact
 * in their high slices and compensated in the rest, about 1e-9 relative to
 * the largest term); it needs n_grid <= 2^30, a 256-byte aligned workspace of
 * gdft_hf_workspace_bytes_form bytes, and gdft_hf_device_status on that
 * workspace after the call to learn whether a bounded device wait expired. */
int gdft_hf_workspace_bytes_form(int64_t n_grid, int32_t n_ao, int32_t n_omega, int32_t form, size_t *bytes);
int gdft_hf_energy_density_form(const double *d_ao, const double *d_rdm1, const double *d_chi, int64_t n_grid,
                                int32_t n_ao, int32_t n_omega, int32_t form, double *d_ehf, void *d_ws,
                                size_t ws_bytes, void *stream);
int gdft_hf_fock_form(const double *d_ao, const double *d_chi, const double *d_g, int64_t n_grid, int32_t n_ao,
                      int32_t n_omega, int32_t form, double *d_fock_hf, void *d_ws, size_t ws_bytes, void *stream);
/* Reads (synchronising the stream) the device error word of a workspace last
 * used by a GDFT_TF32X3 exact-exchange call: GDFT_ERR_DEVICE with *status the
 * code when a bounded wait expired. */
int gdft_hf_device_status(void *d_ws, size_t ws_bytes, int32_t *status, void *stream);

/* The DM21-style coefficient network of a NeuralFunctional (DM21.default_nn,
 * functional.py:797-822, with NeuralFunctional.head :407-419):
 *   h0 = tanh(log(|x| + squash_offset) W0 + b0),
 *   h_i = elu(LayerNorm_i(h_{i-1} W_i + b_i + h_{i-1})), i = 1..n_layers,
 *   c = sigmoid_scale * sigmoid((h W_out + b_out) / sigmoid_scale).
 * Inputs x are the 11 DM21 features (dm21_coefficient_inputs :504-531 plus the
 * 4 HF columns of dm21_combine_cinputs :628-649); outputs multiply the 3
 * energy densities [dm21_densities 'LDA', sum_s ehf(w0), sum_s ehf(w1)]
 * (:534-626, :652-675). */
typedef struct gdft_network {
  int32_t n_in;          /* 11                                                  */
  int32_t width;         /* hidden width: 32, 64, 128 or 256                    */
  int32_t n_layers;      /* residual LayerNorm layers (6 in DM21.default_nn)    */
  int32_t n_out;         /* 3                                                   */
  int32_t precision;     /* GDFT_FP64                                           */
  int32_t reserved;
  double squash_offset;  /* 1e-4                                                */
  double sigmoid_scale;  /* 2.0                                                 */
  double ln_eps;         /* 1e-6 (flax LayerNorm default)                       */
  double clip;           /* clip_cte, 1e-30                                     */
} gdft_network;

/* Number of FP64 parameters in the flat layout the calls below take:
 * Dense_0 kernel (n_in x width, row-major as flax stores it) and bias; for
 * i = 1..n_layers, Dense_i kernel and bias followed by LayerNorm_{i-1} scale
 * and bias; Dense_{n_layers+1} kernel (width x n_out) and bias. */
int gdft_network_param_count(const gdft_network *net, size_t *count);

/* Workspace bytes of gdft_neural_xc_energy_and_grads on this molecule. */
int gdft_neural_workspace_bytes(const gdft_molecule *mol, const gdft_network *net, size_t *bytes);

/* xc_energy_and_grads (train.py:86-121) of a DM21-style NeuralFunctional with
 * stop-gradient HF inputs, plus dE_xc/dtheta (the gradient of
 * Functional.xc_energy with respect to params, as jax.grad gives it).
 * d_params / d_dparams: flat FP64 as gdft_network_param_count describes.
 * d_ehf: (2 omegas, 2 spins, grid).  d_vxc (2, ao, ao) and d_dparams may be
 * NULL. */
int gdft_neural_xc_energy_and_grads(const gdft_molecule *mol, const double *d_rdm1, const gdft_network *net,
                                    const double *d_params, const double *d_ehf, double *d_exc, double *d_vxc,
                                    double *d_dparams, void *d_ws, size_t ws_bytes, void *stream);

/* DM21 network (either network form, omegas 0 and 0.4) in one pass: E_xc into d_exc,
 * optionally V_xc = dE_xc/d rdm1 into d_vxc, and dE_xc/d ehf[w][s][r]
 * (2, 2, n_grid) through the HF energy-density columns (d_g_dens: the
 * gradient of HF_density_grad_2_Fock, molecule.py:598-603) and through the HF
 * coefficient inputs (d_g_cin: HF_coefficient_input_grad_2_Fock,
 * molecule.py:668-673); one of the two may be null.  Same workspace as
 * gdft_neural_xc_energy_and_grads. */
int gdft_neural_xc_hf_grads(const gdft_molecule *mol, const double *d_rdm1, const gdft_network *net,
                            const double *d_params, const double *d_ehf, double *d_exc, double *d_vxc,
                            double *d_g_dens, double *d_g_cin, void *d_ws, size_t ws_bytes, void *stream);


/* Workspace bytes of gdft_neural_xc_hvp on this molecule. */
int gdft_neural_hvp_workspace_bytes(const gdft_molecule *mol, const gdft_network *net, size_t *bytes);

/* Second-order adjoint of gdft_neural_xc_energy_and_grads: for a cotangent G
 * on V_xc (d_tangent, (2, ao, ao)), the gradients of L = <G, V_xc(D, theta)>
 * = sum_sab G_sab dE_xc/dD_sab: d_hrdm1 = dL/dD (2, ao, ao), d_hparams =
 * dL/dtheta (flat), d_value = L (each may be NULL).  This is the vector-
 * Jacobian product jax.grad forms when it differentiates through a Fock
 * matrix built from V_xc in the differentiable SCF loop (evaluate.py:314-344,
 * train.py:86-163).  No separate function in the reference (JAX derives it). */
int gdft_neural_xc_hvp(const gdft_molecule *mol, const double *d_rdm1, const gdft_network *net,
                       const double *d_params, const double *d_ehf, const double *d_tangent, double *d_value,
                       double *d_hrdm1, double *d_hparams, void *d_ws, size_t ws_bytes, void *stream);

/* Workspace bytes of gdft_neural_batch_xc for these molecules: a persistent
 * error word, ONE molecule region sized for the largest molecule (the
 * molecules' density and V_xc stages run one after another on the stream and
 * share it), the joint per-point arrays and the network's scratch. */
int gdft_neural_batch_workspace_bytes(int32_t n_mol, const gdft_molecule *mols, const gdft_network *net,
                                      size_t *bytes);

/* A batch of molecules of different sizes in one call (a training step over a
 * dataset, train.py:34-218 applied per molecule): every molecule's density
 * contraction, then ONE pass of the network over all molecules' grid points,
 * per-molecule energies E_m and the loss L = sum_m (E_m - e_ref_m)^2 (or
 * sum_m E_m when d_eref is NULL) formed on the device, the backward seeded with
 * dL/dE_m, and every molecule's V contraction.  Outputs: d_energies (n_mol),
 * d_loss (may be NULL), d_vxc[m] = dL/dD_m (2, ao_m, ao_m) (array of device
 * pointers; entries may be NULL), d_dparams = dL/dtheta.  h_rdm1 / h_ehf /
 * h_vxc are HOST arrays of n_mol device pointers.  The network must be the
 * TF32x3 form.  Nothing synchronises the host, so the call can be captured in
 * a CUDA graph.  No counterpart in the reference (JAX vmaps/loops over
 * molecules). */
int gdft_neural_batch_xc(int32_t n_mol, const gdft_molecule *mols, const double *const *h_rdm1,
                         const double *const *h_ehf, const gdft_network *net, const double *d_params,
                         const double *d_eref, double *d_energies, double *d_loss, double *const *h_vxc,
                         double *d_dparams, void *d_ws, size_t ws_bytes, void *stream);

/* Synchronises the stream and reads (then clears) the batch workspace's
 * persistent error word, where every molecule's and the network's expired
 * bounded waits of gdft_neural_batch_xc calls are folded; GDFT_ERR_DEVICE with
 * *status = the first code if one expired.  No counterpart in the reference. */
int gdft_neural_batch_status(void *d_ws, size_t ws_bytes, int32_t *status, void *stream);

/* The DM21 network inputs and energy densities of a molecule: d_cinputs
 * (grid, 11) = dm21_combine_cinputs(dm21_coefficient_inputs(...), ehf)
 * (functional.py:504-531, 628-649) and d_dens (grid, 3) =
 * dm21_combine_densities(dm21_densities('LDA'), ehf) before clipping
 * (:534-626, :652-675).  Either output may be NULL.  Workspace as for
 * gdft_neural_xc_energy_and_grads. */
int gdft_neural_inputs(const gdft_molecule *mol, const double *d_rdm1, const gdft_network *net, const double *d_ehf,
                       double *d_cinputs, double *d_dens, void *d_ws, size_t ws_bytes, void *stream);

/* Workspace bytes of gdft_network_apply for n_rows inputs. */
int gdft_network_apply_workspace_bytes(const gdft_network *net, int64_t n_rows, size_t *bytes);

/* The network alone on given inputs (NeuralFunctional.apply, the coefficients
 * of functional.py:797-822 + :407-419): d_x (n_rows, n_in) -> d_c (n_rows, n_out). */
int gdft_network_apply(const gdft_network *net, const double *d_params, int64_t n_rows, const double *d_x,
                       double *d_c, void *d_ws, size_t ws_bytes, void *stream);

/* The transposed density contraction on given per-point potentials (the part
 * of jax.grad at train.py:86 downstream of the pointwise functional):
 *   V_s[a][b] = sum_r  c[s][0] phi_a phi_b + sum_j c[s][1+j] phi_a d_j phi_b
 *                    + c[s][4] phi_a lap phi_b + c[s][5] sum_j d_j phi_a d_j phi_b
 * d_pot: (2, 6, grid) FP64; d_vxc: (2, ao, ao). */
int gdft_vxc_from_potentials(const gdft_molecule *mol, const double *d_pot, double *d_vxc, void *d_ws,
                             size_t ws_bytes, void *stream);

/* The functional's energy-density columns before clipping (the stacked output of
 * the energy_densities plugin, e.g. b88_density popular_functionals.py:277-284,
 * b3lyp_exhf_densities :306-326 plus the combine step :328-334).
 * d_dens: (grid, n_cols). */
int gdft_energy_densities(const gdft_molecule *mol, const double *d_rdm1, const gdft_functional *fn,
                          const double *d_ehf, int32_t n_omega, double *d_dens, void *d_ws, size_t ws_bytes,
                          void *stream);

/* Functional.xc_energy on given energy densities and constant coefficients
 * (functional.py:219-253 with _integrate :316-342):
 * E = sum_r abs_clip(w_r) * abs_clip(abs_clip(sum_f c_f dens_rf)), Kahan-compensated FP64.
 * d_dens (grid, n_cols); coeffs: n_coeffs (1 broadcasts) host doubles; d_exc one double. */
int gdft_integrate(int64_t n_grid, int32_t n_cols, const double *h_coeffs, int32_t n_coeffs, const double *d_dens,
                   const double *d_weights, double clip, double *d_exc, void *d_ws, size_t ws_bytes, void *stream);

/* Workspace bytes of gdft_integrate. */
int gdft_integrate_workspace_bytes(int64_t n_grid, size_t *bytes);

/* gdft_integrate without a workspace, for callers that cannot allocate device
 * memory when they need the energy (e.g. a JAX/XLA custom-call handler, which
 * must not allocate outside XLA's allocator, or a service whose device memory
 * is fully reserved at start-up).  No counterpart in the reference.
 * Its scratch is a fixed array in the library's device image (1 MiB, held by
 * every GPU that loads the library until exit), so n_grid is limited to
 * 33,554,432 points; larger grids are rejected with GDFT_ERR_INVALID.  The
 * first call on a device looks up the array's device address (make it before
 * any stream capture) and keeps it for the life of the process: do not use
 * this entry on a device after cudaDeviceReset, whose new context has the
 * array at another address.  Calls share the array: calls that overlap on the
 * GPU race.  Allocates nothing. */
int gdft_integrate_noalloc(int64_t n_grid, int32_t n_cols, const double *h_coeffs, int32_t n_coeffs,
                           const double *d_dens, const double *d_weights, double clip, double *d_exc, void *stream);

/* Fock assembly of predict (train.py:147-163):
 * F = abs_clip(1/2 (G + G^T)) with G = abs_clip(h1e + J + V_xc), both spins.
 * d_h1e (ao, ao), d_vj (ao, ao) Coulomb potential, d_vxc (2, ao, ao) -> d_fock (2, ao, ao). */
int gdft_fock(int32_t n_ao, const double *d_h1e, const double *d_vj, const double *d_vxc, double clip,
              double *d_fock, void *stream);

/* Coulomb potential J_pq = sum_rt (pq|rt) D_rt with D = rdm1 summed over spin
 * (molecule.py:783-811 coulomb_potential, :117 get_coulomb_potential), and the
 * non-XC energy E_nuc + tr(D h1e) + 1/2 tr(D J) (molecule.py:694-733 nonXC).
 * d_eri (ao, ao, ao, ao); d_vj (ao, ao); d_enonxc one double. */
int gdft_coulomb(int32_t n_ao, const double *d_eri, const double *d_rdm1, const double *d_h1e,
                 double nuclear_repulsion, double *d_vj, double *d_enonxc, void *stream);

/* Device-side status of the calls made with this workspace since the last
 * query: kernels never trap; a bounded wait that expired records a nonzero
 * code in the workspace.  Synchronises `stream`, returns GDFT_ERR_DEVICE (and
 * the code in *status) if set, and clears it.  No counterpart in the
 * reference (its errors are Python exceptions). */
int gdft_device_status(const gdft_molecule *mol, void *d_ws, size_t ws_bytes, int32_t *status, void *stream);

/* Grid-chunked evaluation: phi recomputed per chunk instead of held for the
 * whole grid.  Replaces holding Molecule.ao / grad_ao / grad_n_ao for all grid
 * points (interface/pyscf.py:849-852, molecule.py:72-106) when the basis is
 * known: the grid is processed in chunks of `chunk` points (a multiple of 256);
 * for each chunk the AO tables are evaluated from the basis (a contracted
 * gdft_basis, or the synthetic rows of gdft_molecule_eval_basis: exactly one
 * of the two) into a chunk buffer inside the workspace, then the density,
 * point and V_xc stages run on them and E_xc, V_xc (and dE/dtheta)
 * accumulate over the chunks on the device.  The result is
 * xc_energy_and_grads (train.py:86-121) of the whole grid; only the
 * summation order over grid points differs from the resident path.
 * d_coords (n_grid, 3) bohr, d_weights (n_grid,); d_ehf (omega, 2, n_grid)
 * with n_omega <= 4 where the functional reads it (the network: (2, 2,
 * n_grid)).  Workspace bytes from gdft_chunked_workspace_bytes (net NULL for
 * a constant-coefficient functional); an expired bounded wait is reported by
 * gdft_chunked_status. */
int gdft_chunked_workspace_bytes(int32_t n_ao, int64_t chunk, int32_t precision, const gdft_network *net,
                                 size_t *bytes);
int gdft_xc_energy_and_grads_chunked(const gdft_basis *shells, const double *d_basis_rows, int32_t n_ao,
                                     const double *d_coords, const double *d_weights, int64_t n_grid, int64_t chunk,
                                     int32_t precision, const double *d_rdm1, const gdft_functional *fn,
                                     const double *d_ehf, int32_t n_omega, double *d_exc, double *d_vxc, void *d_ws,
                                     size_t ws_bytes, void *stream);
/* The same for the DM21-style network (gdft_neural_xc_energy_and_grads per chunk; d_dparams may be NULL). */
int gdft_neural_xc_energy_and_grads_chunked(const gdft_basis *shells, const double *d_basis_rows, int32_t n_ao,
                                            const double *d_coords, const double *d_weights, int64_t n_grid,
                                            int64_t chunk, int32_t precision, const double *d_rdm1,
                                            const gdft_network *net, const double *d_params, const double *d_ehf,
                                            double *d_exc, double *d_vxc, double *d_dparams, void *d_ws,
                                            size_t ws_bytes, void *stream);
/* Status of the chunked calls made with this workspace since the last query
 * (as gdft_device_status: synchronises, returns GDFT_ERR_DEVICE with the code,
 * clears).  No counterpart in the reference. */
int gdft_chunked_status(void *d_ws, size_t ws_bytes, int32_t *status, void *stream);

/* Test of the failure path above: one kernel waits on an mbarrier that
 * nothing arrives on, with `limit` (1..65536) polls instead of the pipeline
 * kernels' limit, so the wait runs out; it records GDFT_WAIT_EXPIRY_PROBE in
 * the workspace's error word and returns (no trap; nothing else is in flight,
 * the context stays usable).  The next gdft_device_status reports it.  No
 * counterpart in the reference. */
#define GDFT_WAIT_EXPIRY_PROBE 99
int gdft_selftest_wait_expiry(const gdft_molecule *mol, void *d_ws, size_t ws_bytes, int32_t limit, void *stream);

/* Self-test of the tensor-core building blocks (TMA bulk copy, tcgen05.mma
 * kind::tf32, TMEM load) on one 128 x 128 x 32 product of small integers;
 * *max_abs_err is 0 on a correct device path.  Synchronous; allocates its own
 * small buffers.  No counterpart in the reference. */
int gdft_selftest_umma(double *max_abs_err);

/* D (128 x 128) = A (128 x 32) B (128 x 32)^T (host arrays, row-major, FP32
 * containers read as TF32) through the same tensor-core path, for
 * characterising its accumulation rounding.  Synchronous.  No counterpart in
 * the reference. */
int gdft_umma_probe(const float *h_a, const float *h_b, float *h_d);

/* D (M x N) = A (M x K) B (N x K)^T (host FP64 arrays, row-major) through the
 * packed TF32x3 tensor-core GEMM used by the network's mixed form (packing,
 * tcgen05, Kahan-folded FP32 sums; FP32 output for nsplit 1, FP64 split-K
 * partials otherwise).  Synchronous, allocates its own buffers.  No
 * counterpart in the reference. */
int gdft_tc_gemm_probe(int32_t M, int32_t N, int32_t K, int32_t nsplit, const double *h_a, const double *h_b,
                       double *h_d);

/* The same product through the block-scaled three-slice GEMM of the mixed
 * V_xc contraction (hi slices quantised per row and 32-wide K chunk so that
 * each chunk's hi*hi sum is exact in the FP32 accumulator; six products per
 * term; FP64 split-K partials summed on the host).  Synchronous, allocates its
 * own buffers.  No counterpart in the reference. */
int gdft_tc_gemm3_probe(int32_t M, int32_t N, int32_t K, int32_t nsplit, const double *h_a, const double *h_b,
                        double *h_d);

/* Stage timing (observability; no counterpart in the reference, whose only
 * tracing is jax.profiler.annotate_function at train.py:123).  When enabled,
 * the library records a CUDA event pair on the launching stream around every
 * kernel it launches, per stage.  Host-side state is process-wide and not
 * thread-safe; gdft_profile_read synchronises on the recorded events. */
enum {
  GDFT_STAGE_AO = 0,       /* AO table load / evaluation           */
  GDFT_STAGE_DENSITY = 1,  /* density contraction                  */
  GDFT_STAGE_POINT = 2,    /* energy densities + adjoint coefficients */
  GDFT_STAGE_VXC = 3,      /* V_xc contraction                     */
  GDFT_STAGE_REDUCE = 4,   /* energy / split-K reductions, assembly */
  GDFT_STAGE_MLP = 5,      /* coefficient network                  */
  GDFT_STAGE_COUNT = 8
};
int gdft_profile_enable(int32_t enable);
int gdft_profile_reset(void);
int gdft_profile_read(int32_t stage, double *total_ms, int64_t *launches);

#ifdef __cplusplus
}
#endif

#endif /* GDFT_H_ */
