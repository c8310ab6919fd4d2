// mlp.cuh - the DM21-style coefficient network on the grid (shape, scratch layout, launchers).
#pragma once

#include "common.cuh"

namespace gdft {

// Network inputs per point: 7 local features + 4 HF features (2 omegas x 2 spins).
constexpr int kDm21In = 11;
// Row stride of the squashed-input matrix u (and of dE/du): padded to 16 doubles.
constexpr int kDm21InPad = 16;
constexpr int kDm21Out = 3;
// Blocks of the LayerNorm backward (per-block parameter-gradient partials).
constexpr int kLnBlocks = 592;  // 4 x 148 SMs
// Blocks of the column-sum (bias gradient) first pass.
constexpr int kColBlocks = 296;
// Blocks of the head weight-gradient pass of the tensor-core forms (more row
// slices in flight: one thread per column walks its slice's rows).
constexpr int kHeadBlocks = 4 * kColBlocks;

struct MlpShape {
  int n_in, width, n_layers, n_out;
  double squash_offset, sigmoid_scale, ln_eps;
};

// Offsets (in doubles) of the network scratch inside its workspace region.
struct MlpLayout {
  size_t x, u, e, h, z, y, dy, de, d0, d1, du, kpart, lnpart, colpart, epart, doubles;
  int nsplit;   // split-K factor of the weight-gradient GEMMs
  int eblocks;  // energy partial sums
};

size_t mlp_param_count(const MlpShape &s);

// Per-point DM21 inputs x (np x 11), squashed u (np x 16), energy densities e
// (np x 3); and the V-contraction coefficients from dE/du and dE/de.
cudaError_t launch_dm21_features(const double *feat, const double *ehf, int64_t n_grid, int64_t np, double clip,
                                 double off, double *x, double *u, double *e, cudaStream_t st);
cudaError_t launch_dm21_potentials(const double *feat, const double *x, const double *du, const double *de,
                                   int64_t n_grid, int64_t np, double clip, double off, double *coef,
                                   cudaStream_t st);
MlpLayout mlp_layout(const MlpShape &s, int64_t np);
bool mlp_width_supported(int width);

// Forward (E into *exc), and when coef/dparams are non-null the backward:
// coef[2][6][np] = per-point adjoint coefficients for the V_xc contraction,
// dparams = dE/dtheta in the flat parameter order.
int mlp_run_f64(const MlpShape &S, const double *params, double *dparams, const double *feat, const double *ehf,
                const double *w, int64_t n_grid, int64_t np, double clip, double *ws, double *exc, double *coef,
                cudaStream_t st);
// After mlp_run_f64 with coef (the backward pass) on the same workspace:
// g_dens, g_cin (2 omegas, 2 spins, n_grid) = dE/d ehf through the HF
// energy-density columns and through the HF inputs (either may be null).
cudaError_t launch_dm21_hf_grads(const MlpShape &S, int64_t n_grid, int64_t np, const double *ws, double *g_dens,
                                 double *g_cin, cudaStream_t st);
// The same from the network pass's FP64 inputs x [np][11], input gradients du
// [np][16] and energy-density gradients de [np][3] (either network form).
cudaError_t launch_dm21_hf_grads_from(const double *x, const double *du, const double *de, int64_t n_grid,
                                      double squash_offset, double *g_dens, double *g_cin, cudaStream_t st);

// Scratch of the second-order pass (offsets in doubles).  Primal and tangent
// activations are stacked as [2][np][width] so one GEMM serves both.
struct MlpHvpLayout {
  size_t featp, x, xt, u, e, et, h, z, y, gy, ge, d0, d1, gu, kpart, lnpart, colpart, lpart, doubles;
  int nsplit;
  int eblocks;
};
MlpHvpLayout mlp_hvp_layout(const MlpShape &s, int64_t np);

// Second-order adjoint for L = <G, dE/dD>: from the density features of D
// (featp) and of the tangent G (featt), writes coef[2][6][np] (the per-point
// coefficients whose V contraction is dL/dD), dparams = dL/dtheta (may be
// null) and *lval = L (may be null).
int mlp_hvp_f64(const MlpShape &S, const double *params, double *dparams, const double *featp, const double *featt,
                const double *ehf, const double *w, int64_t n_grid, int64_t np, double clip, double *ws,
                double *lval, double *coef, cudaStream_t st);

// Mixed (TF32x3 tensor-core) form of mlp_run_f64: FP32 activations, FP64 row
// statistics, head, features and potentials; widths 128 and 256.
struct MlpTcLayout {
  size_t bytes;
  size_t x, u, e, dy, de, du, epart, kpart, lnpart, colpart, colpart2;            // FP64 regions (byte offsets)
  size_t pf, dyf, pu, wt, wr, zf, hf, ph, ch, gz, dhp, pg, cg;                   // FP32 regions (byte offsets)
  int nsplit;
};
MlpTcLayout mlp_tc_layout(const MlpShape &s, int64_t np);
bool mlp_tc_width_supported(int width);

// Several molecules' grid points in one network pass: segment m is rows
// [seg_off[m], seg_off[m + 1]) (multiples of 256).  After the forward, the
// per-segment energies E_m and the loss (sum_m (E_m - e_ref_m)^2, or sum_m E_m
// without references) are formed on the device, and the backward is seeded
// with dloss/dE_m per segment, so dparams = dloss/dtheta and coef carries
// dloss/dE_m for each molecule's points.
struct MlpSegments {
  int n_seg;
  const int64_t *d_seg_off;  // n_seg + 1 row offsets (device)
  const double *d_eref;      // n_seg reference energies or null
  double *d_energies;        // n_seg out
  double *d_loss;            // 1 out (may be null)
  double *d_cot;             // n_seg scratch: dloss/dE_m
};

int mlp_run_tc(const MlpShape &S, const double *params, double *dparams, const double *feat, const double *ehf,
               const double *w, int64_t n_grid, int64_t np, double clip, char *ws, double *exc, double *coef, int *err,
               cudaStream_t st, const MlpSegments *seg = nullptr);

// Per-point pieces of the second-order pass shared by its FP64 and mixed forms:
// primal/tangent inputs (u stacked [2][np][16]) and energy densities, and the
// V-contraction coefficients from [dL/du; dL/du~] (GU) and dL/de (ge [np][2]).
cudaError_t launch_features_tan(const double *featp, const double *featt, const double *ehf, int64_t n_grid,
                                int64_t np, double clip, double off, double *x, double *xt, double *u, double *e,
                                double *et, cudaStream_t st);
cudaError_t launch_hvp_potentials(const double *featp, const double *featt, const double *x, const double *xt,
                                  const double *GU, const double *ge, int64_t n_grid, int64_t np, double clip,
                                  double off, double *coef, cudaStream_t st);

// Mixed form of mlp_hvp_f64 (tensor-core GEMMs over the stacked 2 np rows,
// FP32 activations and row statistics, FP64 sums over grid points).
struct MlpHvpTcLayout {
  size_t bytes;
  size_t featp, x, xt, u, e, et, gy, ge, gu, lpart, kpart, lnpart, colpart, colpart2;  // FP64 (byte offsets)
  size_t pf, gyf, pu, wt, wr, z, h, ph, ch, gz, dhp, pg, cg;                        // FP32 (byte offsets)
  int nsplit;
};
MlpHvpTcLayout mlp_hvp_tc_layout(const MlpShape &s, int64_t np);
int mlp_hvp_tc(const MlpShape &S, const double *params, double *dparams, const double *featp, const double *featt,
               const double *ehf, const double *w, int64_t n_grid, int64_t np, double clip, char *ws, double *lval,
               double *coef, int *err, cudaStream_t st);

// The 11 network inputs (grid x 11) and the 3 energy densities (grid x 3) of
// the DM21 functional from the density features; scratch in ws.
int mlp_inputs_f64(const MlpShape &S, const double *feat, const double *ehf, int64_t n_grid, int64_t np,
                   double clip, double *ws, double *x_out, double *e_out, cudaStream_t st);

// Coefficients c (rows x n_out) of the network on given inputs x (rows x n_in).
int mlp_apply_f64(const MlpShape &S, const double *params, const double *x, int64_t rows, double *ws, double *c,
                  cudaStream_t st);

}  // namespace gdft
