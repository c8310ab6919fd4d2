// common.cuh - shared definitions for the XC grid path kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/gdft.h"

namespace gdft {

// Grid points are processed in tiles of this many rows; the resident tables
// are padded to a whole number of tiles (padded rows are zero and carry zero
// weight, and every kernel masks them explicitly).
constexpr int kPointTile = 128;
// AO leading dimension granularity (columns beyond n_ao are zero).
constexpr int kAoPad = 32;

// Number of per-point density quantities per spin: rho, d_x rho, d_y rho,
// d_z rho, laplacian, tau.
constexpr int kFeat = 6;
enum { F_RHO = 0, F_GX = 1, F_GY = 2, F_GZ = 3, F_LAP = 4, F_TAU = 5 };
// Adjoint coefficients per spin multiplying, in V_ab = sum_r ...:
//   C_RHO: phi_a phi_b, C_GJ: phi_a d_j phi_b, C_LAP: phi_a lap phi_b,
//   C_KIN: sum_j d_j phi_a d_j phi_b.
enum { C_RHO = 0, C_GX = 1, C_GY = 2, C_GZ = 3, C_LAP = 4, C_KIN = 5 };

// AO table planes.
enum { T_PHI = 0, T_DX = 1, T_DY = 2, T_DZ = 3, T_LAP = 4, kPlanes = 5 };

inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// Layout of the molecule buffer.
struct MolLayout {
  int64_t np;   // padded grid points
  int ld;       // AO leading dimension of the FP64 planes
  int ldk;      // AO extent of the TF32x3 tables (multiple of 128)
  size_t off_tab, off_w, off_pm, off_av, off_af, bytes;
  size_t plane_elems() const { return (size_t)np * ld; }
};

MolLayout mol_layout(int64_t n_grid, int n_ao, int precision);

// Layout of the per-call workspace.
struct WsLayout {
  size_t off_feat, off_coef, off_epart, off_vpart, off_dpk, off_q, off_err, bytes;
  int n_eblocks;   // blocks of the point kernel (energy partial sums)
  int n_vsplit;    // split-K factor of the V contraction
};

WsLayout ws_layout(const gdft_molecule *m);

// Thread-local last-error text.
void set_error(const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);

inline __host__ __device__ const double *plane(const double *tab, int p, size_t plane_elems) {
  return tab + (size_t)p * plane_elems;
}

// Kahan-compensated accumulation (FP64 grid sum of functional.py:342).
struct Kahan {
  double s, c;
  __device__ __forceinline__ void add(double x) {
    double y = x - c;
    double t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

}  // namespace gdft
