// api.cu - the C ABI (include/gdft.h): validation, layouts, launch order.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "common.cuh"
#include "kernels.cuh"
#include "mlp.cuh"

namespace gdft {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return GDFT_OK;
  set_error("%s: %s", what, cudaGetErrorString(e));
  return GDFT_ERR_CUDA;
}

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// ---- stage timing ---------------------------------------------------------
struct StageRec {
  cudaEvent_t a, b;
};
static bool g_prof = false;
static StageRec *g_recs[GDFT_STAGE_COUNT] = {nullptr};
static int g_nrec[GDFT_STAGE_COUNT] = {0}, g_cap[GDFT_STAGE_COUNT] = {0};

struct StageTimer {
  int stage;
  cudaStream_t st;
  StageRec *rec = nullptr;
  StageTimer(int s, cudaStream_t stream) : stage(s), st(stream) {
    if (!g_prof) return;
    if (g_nrec[s] == g_cap[s]) {
      const int cap = g_cap[s] ? 2 * g_cap[s] : 64;
      StageRec *n = new StageRec[cap];
      for (int i = 0; i < g_cap[s]; ++i) n[i] = g_recs[s][i];
      for (int i = g_cap[s]; i < cap; ++i) {
        cudaEventCreate(&n[i].a);
        cudaEventCreate(&n[i].b);
      }
      delete[] g_recs[s];
      g_recs[s] = n;
      g_cap[s] = cap;
    }
    rec = &g_recs[s][g_nrec[s]++];
    cudaEventRecord(rec->a, st);
  }
  ~StageTimer() {
    if (rec) cudaEventRecord(rec->b, st);
  }
};

MolLayout mol_layout(int64_t n_grid, int n_ao, int precision) {
  MolLayout L;
  L.np = round_up(n_grid, kPointTile);
  L.ld = (int)round_up(n_ao, kAoPad);
  L.ldk = (int)round_up(n_ao, 128);
  size_t off = 0;
  L.off_w = off;
  off = align256(off + (size_t)L.np * sizeof(double));
  L.off_tab = L.off_pm = L.off_av = L.off_af = off;
  if (precision == GDFT_FP64) {
    off = align256(off + (size_t)kPlanes * L.plane_elems() * sizeof(double));
  } else {
    // Point-major hi/lo of the five planes, AO-major block-scaled hi/lo/lo2
    // of four planes, and AO-major FP32 pairs (hi = fp32(x), lo = fp32(x - hi))
    // of the five planes.
    const size_t plane = (size_t)L.np * L.ldk * sizeof(float);
    L.off_pm = off;
    off = align256(off + kPlanes * 2 * plane);
    L.off_av = off;
    off = align256(off + 4 * 3 * plane);
    L.off_af = off;
    off = align256(off + kPlanes * 2 * plane);
  }
  L.bytes = off;
  return L;
}

WsLayout ws_layout(const gdft_molecule *m) {
  WsLayout W;
  const int64_t np = m->n_grid_pad;
  W.n_eblocks = xc_point_blocks(np);
  W.n_vsplit = m->precision == GDFT_FP64 ? vxc_f64_splits(np, m->n_ao) : vxc_q_splits(np, m->n_ao);
  size_t off = 0;
  W.off_feat = off;
  off = align256(off + (size_t)2 * kFeat * np * sizeof(double));
  W.off_coef = off;
  off = align256(off + (size_t)2 * kFeat * np * sizeof(double));
  W.off_epart = off;
  off = align256(off + (size_t)W.n_eblocks * sizeof(double));
  W.off_vpart = off;
  if (m->precision == GDFT_FP64) {
    off = align256(off + (size_t)W.n_vsplit * 2 * m->n_ao * m->n_ao * sizeof(double));
  } else {  // split-K partials of the packed GEMM: [split][n_ao][2 ldk]
    off = align256(off + (size_t)W.n_vsplit * m->n_ao * 2 * round_up(m->n_ao, 128) * sizeof(double));
  }
  W.off_dpk = off;
  W.off_q = off;
  if (m->precision == GDFT_TF32X3) {
    const size_t ldk = (size_t)round_up(m->n_ao, 128);
    off = align256(off + 2 * ldk * ldk * 2 * sizeof(float));
    W.off_q = off;
    off = align256(off + vxc_q_bytes(np, m->n_ao));
  }
  W.off_err = off;
  off = align256(off + 64);
  W.bytes = off;
  return W;
}

static int check_mol(const gdft_molecule *m) {
  if (m == nullptr || m->buffer == nullptr) {
    set_error("molecule is not initialised");
    return GDFT_ERR_INVALID;
  }
  if (m->n_grid <= 0 || m->n_ao <= 0) {
    set_error("molecule has n_grid=%lld n_ao=%d", (long long)m->n_grid, m->n_ao);
    return GDFT_ERR_INVALID;
  }
  const MolLayout L = mol_layout(m->n_grid, m->n_ao, m->precision);
  if (m->buffer_bytes < L.bytes || m->n_grid_pad != L.np || m->ld != L.ld ||
      (m->precision != GDFT_FP64 && m->precision != GDFT_TF32X3)) {
    set_error("molecule descriptor does not match its layout");
    return GDFT_ERR_INVALID;
  }
  return GDFT_OK;
}

static int check_ws(const gdft_molecule *m, void *ws, size_t ws_bytes) {
  const WsLayout W = ws_layout(m);
  if (ws == nullptr || ws_bytes < W.bytes) {
    set_error("workspace of %zu bytes is smaller than the %zu bytes required", ws_bytes, W.bytes);
    return GDFT_ERR_WORKSPACE;
  }
  if (((uintptr_t)ws & 255u) != 0) {
    set_error("workspace must be 256-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  return GDFT_OK;
}

static int check_aligned8(const void *p, const char *name) {
  if (((uintptr_t)p & 7u) != 0) {
    set_error("%s must be 8-byte aligned", name);
    return GDFT_ERR_ALIGNMENT;
  }
  return GDFT_OK;
}

static int check_functional(const gdft_functional *fn, const double *ehf, int n_omega) {
  if (fn == nullptr || fn->n_cols < 1 || fn->n_cols > GDFT_MAX_COLS) {
    set_error("functional must have 1..%d energy-density columns", GDFT_MAX_COLS);
    return GDFT_ERR_INVALID;
  }
  if (!(fn->n_coeffs == 1 || fn->n_coeffs == fn->n_cols)) {
    set_error("functional has %d coefficients for %d columns", fn->n_coeffs, fn->n_cols);
    return GDFT_ERR_INVALID;
  }
  for (int i = 0; i < fn->n_cols; ++i) {
    const int c = fn->cols[i];
    const bool uw = (c & ~0xff) == 0x100 || (c & ~0x1ff) == 0x200;  // GDFT_COL_DM21_UW / GDFT_COL_DENS_X
    if (!uw && (c < GDFT_COL_LSDA || c > GDFT_COL_ZERO)) {
      set_error("unknown energy-density column %d", c);
      return GDFT_ERR_INVALID;
    }
    const bool needs_hf = c == GDFT_COL_HF || c == GDFT_COL_HF_W0 || c == GDFT_COL_HF_W1;
    if (needs_hf && (ehf == nullptr || n_omega < (c == GDFT_COL_HF_W1 ? 2 : 1))) {
      set_error("energy-density column %d needs ehf with enough omegas (got n_omega=%d)", c, n_omega);
      return GDFT_ERR_INVALID;
    }
  }
  return GDFT_OK;
}

static const double *mol_tab(const gdft_molecule *m) {
  return (const double *)((const char *)m->buffer + mol_layout(m->n_grid, m->n_ao, m->precision).off_tab);
}
static const double *mol_w(const gdft_molecule *m) {
  return (const double *)((const char *)m->buffer + mol_layout(m->n_grid, m->n_ao, m->precision).off_w);
}

static const float *mol_pm(const gdft_molecule *m) {
  return (const float *)((const char *)m->buffer + mol_layout(m->n_grid, m->n_ao, m->precision).off_pm);
}
static const float *mol_av(const gdft_molecule *m) {
  return (const float *)((const char *)m->buffer + mol_layout(m->n_grid, m->n_ao, m->precision).off_av);
}
static const float *mol_af(const gdft_molecule *m) {
  return (const float *)((const char *)m->buffer + mol_layout(m->n_grid, m->n_ao, m->precision).off_af);
}

static int check_network(const gdft_network *net) {
  if (net == nullptr) {
    set_error("network descriptor is required");
    return GDFT_ERR_INVALID;
  }
  if (net->n_in != kDm21In || net->n_out != kDm21Out) {
    set_error("network must map the %d DM21 inputs to %d coefficients (got %d -> %d)", kDm21In, kDm21Out, net->n_in,
              net->n_out);
    return GDFT_ERR_INVALID;
  }
  if (!mlp_width_supported(net->width) || net->n_layers < 0 || net->n_layers > 64) {
    set_error("network width %d / layers %d not supported (width 32, 64, 128 or 256; 0..64 layers)", net->width,
              net->n_layers);
    return GDFT_ERR_INVALID;
  }
  if (net->precision != GDFT_FP64 && net->precision != GDFT_TF32X3) {
    set_error("network precision %d is not built", net->precision);
    return GDFT_ERR_UNSUPPORTED;
  }
  if (net->precision == GDFT_TF32X3 && (!mlp_tc_width_supported(net->width) || net->n_layers < 1)) {
    set_error("the TF32x3 network form needs width 128 or 256 and at least one residual layer (got %d, %d)",
              net->width, net->n_layers);
    return GDFT_ERR_UNSUPPORTED;
  }
  if (!(net->sigmoid_scale != 0.0) || !(net->ln_eps >= 0.0) || !(net->squash_offset >= 0.0)) {
    set_error("network constants out of range");
    return GDFT_ERR_INVALID;
  }
  return GDFT_OK;
}

static MlpShape net_shape(const gdft_network *net) {
  MlpShape S;
  S.n_in = net->n_in;
  S.width = net->width;
  S.n_layers = net->n_layers;
  S.n_out = net->n_out;
  S.squash_offset = net->squash_offset;
  S.sigmoid_scale = net->sigmoid_scale;
  S.ln_eps = net->ln_eps;
  return S;
}

// The network scratch follows the contraction workspace.
static size_t neural_ws_bytes(const gdft_molecule *mol, const gdft_network *net) {
  // The TF32x3 scratch also holds what gdft_neural_inputs writes there (the
  // FP64 layout's leading x, u, e arrays, 30 doubles per point).
  if (net->precision == GDFT_TF32X3) return ws_layout(mol).bytes + mlp_tc_layout(net_shape(net), mol->n_grid_pad).bytes;
  return ws_layout(mol).bytes + align256(mlp_layout(net_shape(net), mol->n_grid_pad).doubles * sizeof(double));
}
static size_t hvp_ws_bytes(const gdft_molecule *mol, const gdft_network *net) {
  if (net->precision == GDFT_TF32X3) return ws_layout(mol).bytes + mlp_hvp_tc_layout(net_shape(net), mol->n_grid_pad).bytes;
  return ws_layout(mol).bytes + align256(mlp_hvp_layout(net_shape(net), mol->n_grid_pad).doubles * sizeof(double));
}

// Segment offsets travel to the device as a kernel argument (captured by value
// in a CUDA graph, no host buffer involved).
constexpr int kBatchMax = 256;
struct SegTable {
  int64_t off[kBatchMax + 1];
};
__global__ void write_seg_kernel(const SegTable t, int n, int64_t *__restrict__ out) {
  for (int i = threadIdx.x; i <= n; i += blockDim.x) out[i] = t.off[i];
}

// Batch workspace: each molecule's own workspace, then the concatenated point
// arrays (segments padded to 256 rows) and the network scratch.
// Batch workspace: [256 B persistent error word][one molecule region, sized
// for the largest molecule and used by each molecule in turn: the density and
// V_xc stages run one molecule after another on the caller's stream][joint
// features, weights, ehf, coefficients, segments, cotangents][network].
struct BatchLayout {
  int64_t seg[kBatchMax + 1];
  int64_t npt;
  bool ragged;                  // every molecule in the mixed form: one ragged density launch
  size_t off_dpk[kBatchMax];    // ragged: each molecule's packed rdm1
  size_t off_mol, off_feat, off_w, off_ehf, off_coef, off_seg, off_cot, off_net, off_queue, bytes;
};

static int batch_layout(int n_mol, const gdft_molecule *mols, const gdft_network *net, BatchLayout *B) {
  if (n_mol < 1 || n_mol > kBatchMax || mols == nullptr) {
    set_error("batch of %d molecules (1..%d supported)", n_mol, kBatchMax);
    return GDFT_ERR_INVALID;
  }
  size_t off = 256, mol_bytes = 0;
  int64_t npt = 0;
  for (int m = 0; m < n_mol; ++m) {
    int rc = check_mol(&mols[m]);
    if (rc) return rc;
    const size_t b = align256(ws_layout(&mols[m]).bytes);
    mol_bytes = b > mol_bytes ? b : mol_bytes;
    B->seg[m] = npt;
    npt += round_up(mols[m].n_grid_pad, 256);
  }
  B->off_mol = off;
  off += mol_bytes;
  B->seg[n_mol] = npt;
  B->ragged = true;
  for (int m = 0; m < n_mol; ++m) B->ragged = B->ragged && mols[m].precision == GDFT_TF32X3;
  if (B->ragged) {
    for (int m = 0; m < n_mol; ++m) {
      const size_t ldk = (size_t)round_up(mols[m].n_ao, 128);
      B->off_dpk[m] = off;
      off += align256(2 * ldk * ldk * 2 * sizeof(float));
    }
    B->off_queue = off;
    off += align256(dens_ragged_scratch_bytes(n_mol));
  }
  B->npt = npt;
  B->off_feat = off;
  off += align256((size_t)2 * kFeat * npt * 8);
  B->off_w = off;
  off += align256((size_t)npt * 8);
  B->off_ehf = off;
  off += align256((size_t)4 * npt * 8);
  B->off_coef = off;
  off += align256((size_t)2 * kFeat * npt * 8);
  B->off_seg = off;
  off += align256((size_t)(n_mol + 1) * 8);
  B->off_cot = off;
  off += align256((size_t)n_mol * 8);
  B->off_net = off;
  off += mlp_tc_layout(net_shape(net), npt).bytes;
  B->bytes = off;
  return GDFT_OK;
}

// Density stage into ws.feat.
static int run_density(const gdft_molecule *m, const double *rdm1, char *ws, cudaStream_t st) {
  const WsLayout W = ws_layout(m);
  double *feat = (double *)(ws + W.off_feat);
  if (m->precision == GDFT_FP64) {
    StageTimer tm(GDFT_STAGE_DENSITY, st);
    return check_cuda(launch_dens_f64(mol_tab(m), m->n_grid_pad, m->ld, m->n_ao, rdm1, feat, st), "dens_f64");
  }
  const int ldk = (int)round_up(m->n_ao, 128);
  float *dpk = (float *)(ws + W.off_dpk);
  int rc;
  {
    StageTimer tm(GDFT_STAGE_REDUCE, st);
    if ((rc = check_cuda(launch_pack_rdm1(rdm1, m->n_ao, ldk, dpk, st), "pack_rdm1"))) return rc;
  }
  StageTimer tm(GDFT_STAGE_DENSITY, st);
  return check_cuda(launch_dens_tc(mol_pm(m), dpk, m->n_grid_pad, ldk, feat, (int *)(ws + W.off_err), st),
                    "dens_tc");
}

}  // namespace gdft

using namespace gdft;

// V_xc contraction of the adjoint coefficients in ws.coef into d_vxc.
static int run_vxc(const gdft_molecule *mol, const double *coef, double *d_vxc, char *ws, cudaStream_t st) {
  const WsLayout W = ws_layout(mol);
  int rc;
  double *vpart = (double *)(ws + W.off_vpart);
  if (mol->precision == GDFT_FP64) {
    {
      StageTimer tm(GDFT_STAGE_VXC, st);
      rc = check_cuda(launch_vxc_f64(mol_tab(mol), mol->n_grid_pad, mol->ld, mol->n_ao, coef, W.n_vsplit, vpart, st),
                      "vxc_f64");
      if (rc) return rc;
    }
    StageTimer tm(GDFT_STAGE_REDUCE, st);
    return check_cuda(launch_vxc_reduce(vpart, W.n_vsplit, mol->n_ao, d_vxc, st), "vxc_reduce");
  }
  StageTimer tm(GDFT_STAGE_VXC, st);
  return check_cuda(launch_vxc_q_tc(mol_av(mol), mol_af(mol), coef, mol->n_grid_pad, (int)round_up(mol->n_ao, 128),
                                    mol->n_ao, (float *)(ws + W.off_q), W.n_vsplit, vpart, d_vxc,
                                    (int *)(ws + W.off_err), st),
                    "vxc_q_tc");
}

// The error word at the start of a chunked or batch workspace: read, cleared,
// reported.
static int persistent_status(const char *name, void *d_ws, size_t ws_bytes, int32_t *status, void *stream) {
  if (d_ws == nullptr || ws_bytes < 256 || status == nullptr) {
    set_error("%s: invalid arguments", name);
    return GDFT_ERR_INVALID;
  }
  int h = 0;
  cudaStream_t st = (cudaStream_t)stream;
  int rc;
  if ((rc = check_cuda(cudaMemcpyAsync(&h, d_ws, sizeof(int), cudaMemcpyDeviceToHost, st), "status read"))) return rc;
  if ((rc = check_cuda(cudaStreamSynchronize(st), "status sync"))) return rc;
  if ((rc = check_cuda(cudaMemsetAsync(d_ws, 0, sizeof(int), st), "status clear"))) return rc;
  *status = h;
  if (h != 0) {
    set_error("a device-side wait expired (code %d); results of the last calls are invalid", h);
    return GDFT_ERR_DEVICE;
  }
  return GDFT_OK;
}

extern "C" {

int gdft_abi_version(void) { return GDFT_ABI_VERSION; }

int gdft_profile_enable(int32_t enable) {
  g_prof = enable != 0;
  return GDFT_OK;
}

int gdft_profile_reset(void) {
  for (int s = 0; s < GDFT_STAGE_COUNT; ++s) g_nrec[s] = 0;
  return GDFT_OK;
}

int gdft_profile_read(int32_t stage, double *total_ms, int64_t *launches) {
  if (stage < 0 || stage >= GDFT_STAGE_COUNT || total_ms == nullptr || launches == nullptr) {
    set_error("gdft_profile_read: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  double t = 0.0;
  for (int i = 0; i < g_nrec[stage]; ++i) {
    float ms = 0.0f;
    cudaError_t e = cudaEventSynchronize(g_recs[stage][i].b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, g_recs[stage][i].a, g_recs[stage][i].b);
    if (e != cudaSuccess) return check_cuda(e, "profile_read");
    t += ms;
  }
  *total_ms = t;
  *launches = g_nrec[stage];
  return GDFT_OK;
}

const char *gdft_last_error(void) { return g_err; }

int gdft_molecule_bytes(int64_t n_grid, int32_t n_ao, int32_t precision, size_t *bytes) {
  if (bytes == nullptr || n_grid <= 0 || n_ao <= 0) {
    set_error("gdft_molecule_bytes: n_grid and n_ao must be positive");
    return GDFT_ERR_INVALID;
  }
  if (precision != GDFT_FP64 && precision != GDFT_TF32X3) {
    set_error("unknown precision %d", precision);
    return GDFT_ERR_INVALID;
  }
  *bytes = mol_layout(n_grid, n_ao, precision).bytes;
  return GDFT_OK;
}

int gdft_molecule_init(gdft_molecule *mol, int64_t n_grid, int32_t n_ao, int32_t precision, void *d_buffer,
                       size_t buffer_bytes) {
  size_t need = 0;
  int rc = gdft_molecule_bytes(n_grid, n_ao, precision, &need);
  if (rc) return rc;
  if (mol == nullptr || d_buffer == nullptr) {
    set_error("gdft_molecule_init: null descriptor or buffer");
    return GDFT_ERR_INVALID;
  }
  if (buffer_bytes < need) {
    set_error("molecule buffer of %zu bytes is smaller than the %zu bytes required", buffer_bytes, need);
    return GDFT_ERR_WORKSPACE;
  }
  if (((uintptr_t)d_buffer & 255u) != 0) {
    set_error("molecule buffer must be 256-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  const MolLayout L = mol_layout(n_grid, n_ao, precision);
  mol->n_grid = n_grid;
  mol->n_grid_pad = L.np;
  mol->n_ao = n_ao;
  mol->ld = L.ld;
  mol->precision = precision;
  mol->reserved = 0;
  mol->buffer = d_buffer;
  mol->buffer_bytes = buffer_bytes;
  return GDFT_OK;
}

int gdft_molecule_load(const gdft_molecule *mol, const double *d_ao, const double *d_grad_ao,
                       const double *d_grad2_ao, const double *d_weights, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if (d_ao == nullptr || d_grad_ao == nullptr || d_weights == nullptr) {
    set_error("gdft_molecule_load: ao, grad_ao and weights are required");
    return GDFT_ERR_INVALID;
  }
  if ((rc = check_aligned8(d_ao, "ao")) || (rc = check_aligned8(d_grad_ao, "grad_ao")) ||
      (rc = check_aligned8(d_weights, "weights")))
    return rc;
  const MolLayout L = mol_layout(mol->n_grid, mol->n_ao, mol->precision);
  double *tab = (double *)((char *)mol->buffer + L.off_tab);
  double *w = (double *)((char *)mol->buffer + L.off_w);
  StageTimer tm(GDFT_STAGE_AO, (cudaStream_t)stream);
  if (mol->precision == GDFT_TF32X3)
    return check_cuda(launch_pack_tables(d_ao, d_grad_ao, d_grad2_ao, nullptr, nullptr, d_weights, mol->n_grid,
                                         mol->n_ao, L.np, L.ldk, (float *)((char *)mol->buffer + L.off_pm),
                                         (float *)((char *)mol->buffer + L.off_av),
                                         (float *)((char *)mol->buffer + L.off_af), w, (cudaStream_t)stream),
                      "pack_tables");
  return check_cuda(launch_load_tables(d_ao, d_grad_ao, d_grad2_ao, d_weights, mol->n_grid, mol->n_ao, L.np, L.ld,
                                       tab, w, (cudaStream_t)stream),
                    "load_tables");
}

int gdft_molecule_eval_basis(const gdft_molecule *mol, const double *d_basis, const double *d_coords,
                             const double *d_weights, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if (d_basis == nullptr || d_coords == nullptr || d_weights == nullptr) {
    set_error("gdft_molecule_eval_basis: basis, coords and weights are required");
    return GDFT_ERR_INVALID;
  }
  const MolLayout L = mol_layout(mol->n_grid, mol->n_ao, mol->precision);
  double *tab = (double *)((char *)mol->buffer + L.off_tab);
  double *w = (double *)((char *)mol->buffer + L.off_w);
  StageTimer tm(GDFT_STAGE_AO, (cudaStream_t)stream);
  if (mol->precision == GDFT_TF32X3)
    return check_cuda(launch_pack_tables(nullptr, nullptr, nullptr, d_basis, d_coords, d_weights, mol->n_grid,
                                         mol->n_ao, L.np, L.ldk, (float *)((char *)mol->buffer + L.off_pm),
                                         (float *)((char *)mol->buffer + L.off_av),
                                         (float *)((char *)mol->buffer + L.off_af), w, (cudaStream_t)stream),
                      "pack_tables");
  return check_cuda(launch_eval_basis(d_basis, d_coords, d_weights, mol->n_grid, mol->n_ao, L.np, L.ld, tab, w,
                                      (cudaStream_t)stream),
                    "eval_basis");
}

static int check_basis(const gdft_basis *b, const char *who, ShellView *out) {
  if (b == nullptr || b->d_shell == nullptr || b->d_centre == nullptr || b->d_exp == nullptr ||
      b->d_coef == nullptr || b->d_ao == nullptr || b->d_trans == nullptr) {
    set_error("%s: the basis and all of its tables are required", who);
    return GDFT_ERR_INVALID;
  }
  if (b->n_shell <= 0 || b->n_ao <= 0 || b->n_prim <= 0 || b->n_coef <= 0 || b->n_trans <= 0) {
    set_error("%s: basis sizes must be positive (n_shell=%d n_ao=%d)", who, b->n_shell, b->n_ao);
    return GDFT_ERR_INVALID;
  }
  int rc;
  if ((rc = check_aligned8(b->d_centre, "basis centres")) || (rc = check_aligned8(b->d_exp, "basis exponents")) ||
      (rc = check_aligned8(b->d_coef, "basis coefficients")) || (rc = check_aligned8(b->d_trans, "basis rows")))
    return rc;
  if (((uintptr_t)b->d_shell | (uintptr_t)b->d_ao) & 3u) {
    set_error("%s: the shell and AO tables must be 4-byte aligned", who);
    return GDFT_ERR_ALIGNMENT;
  }
  *out = ShellView{b->d_shell, b->d_centre, b->d_exp, b->d_coef, b->d_ao, b->d_trans,
                   b->n_shell, b->n_ao,   b->n_prim, b->n_coef, b->n_trans};
  return GDFT_OK;
}

int gdft_eval_ao(const gdft_basis *basis, const double *d_coords, int64_t n_grid, int32_t deriv, double *d_ao,
                 double *d_grad_ao, double *d_grad2_ao, void *stream) {
  ShellView B;
  int rc = check_basis(basis, "gdft_eval_ao", &B);
  if (rc) return rc;
  if (d_coords == nullptr || d_ao == nullptr || n_grid <= 0 || deriv < 0 || deriv > 2 ||
      (deriv >= 1 && d_grad_ao == nullptr) || (deriv >= 2 && d_grad2_ao == nullptr)) {
    set_error("gdft_eval_ao: coords, ao and the outputs of deriv=%d are required (n_grid=%lld)", deriv,
              (long long)n_grid);
    return GDFT_ERR_INVALID;
  }
  if ((size_t)n_grid * (size_t)basis->n_ao > ((size_t)1 << 38)) {  // grid of 256-thread blocks within 2^31
    set_error("gdft_eval_ao: n_grid * n_ao too large");
    return GDFT_ERR_INVALID;
  }
  if ((rc = check_aligned8(d_coords, "coords")) || (rc = check_aligned8(d_ao, "ao")) ||
      (rc = check_aligned8(d_grad_ao, "grad_ao")) || (rc = check_aligned8(d_grad2_ao, "grad2_ao")))
    return rc;
  StageTimer tm(GDFT_STAGE_AO, (cudaStream_t)stream);
  return check_cuda(launch_eval_ao(B, d_coords, n_grid, deriv, d_ao, deriv >= 1 ? d_grad_ao : nullptr,
                                   deriv >= 2 ? d_grad2_ao : nullptr, (cudaStream_t)stream),
                    "eval_ao");
}

int gdft_molecule_eval_shells(const gdft_molecule *mol, const gdft_basis *basis, const double *d_coords,
                              const double *d_weights, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  ShellView B;
  if ((rc = check_basis(basis, "gdft_molecule_eval_shells", &B))) return rc;
  if (basis->n_ao != mol->n_ao) {
    set_error("gdft_molecule_eval_shells: the basis has %d AOs, the molecule %d", basis->n_ao, mol->n_ao);
    return GDFT_ERR_INVALID;
  }
  if (d_coords == nullptr || d_weights == nullptr) {
    set_error("gdft_molecule_eval_shells: coords and weights are required");
    return GDFT_ERR_INVALID;
  }
  if ((rc = check_aligned8(d_coords, "coords")) || (rc = check_aligned8(d_weights, "weights"))) return rc;
  const MolLayout L = mol_layout(mol->n_grid, mol->n_ao, mol->precision);
  double *w = (double *)((char *)mol->buffer + L.off_w);
  StageTimer tm(GDFT_STAGE_AO, (cudaStream_t)stream);
  if (mol->precision == GDFT_TF32X3)
    return check_cuda(launch_pack_tables(nullptr, nullptr, nullptr, nullptr, d_coords, d_weights, mol->n_grid,
                                         mol->n_ao, L.np, L.ldk, (float *)((char *)mol->buffer + L.off_pm),
                                         (float *)((char *)mol->buffer + L.off_av),
                                         (float *)((char *)mol->buffer + L.off_af), w, (cudaStream_t)stream, &B),
                      "pack_tables (shells)");
  return check_cuda(launch_eval_shell_tables(B, d_coords, d_weights, mol->n_grid, L.np, L.ld,
                                             (double *)((char *)mol->buffer + L.off_tab), w, (cudaStream_t)stream),
                    "eval_shell_tables");
}

int gdft_workspace_bytes(const gdft_molecule *mol, size_t *bytes) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if (bytes == nullptr) {
    set_error("gdft_workspace_bytes: null output");
    return GDFT_ERR_INVALID;
  }
  *bytes = ws_layout(mol).bytes;
  return GDFT_OK;
}

int gdft_density(const gdft_molecule *mol, const double *d_rdm1, double *d_rho, double *d_grad_rho, double *d_lapl,
                 double *d_tau, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_ws(mol, d_ws, ws_bytes))) return rc;
  if (d_rdm1 == nullptr) {
    set_error("gdft_density: rdm1 is required");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = run_density(mol, d_rdm1, (char *)d_ws, st))) return rc;
  const WsLayout W = ws_layout(mol);
  StageTimer tm(GDFT_STAGE_REDUCE, st);
  return check_cuda(launch_feat_to_reference((const double *)((char *)d_ws + W.off_feat), mol->n_grid,
                                             mol->n_grid_pad, d_rho, d_grad_rho, d_lapl, d_tau, st),
                    "feat_to_reference");
}

static int xc_energy_and_grads(const char *who, const gdft_molecule *mol, const double *d_rdm1,
                               const gdft_functional *fn, const double *d_ehf, int32_t n_omega, double *d_exc,
                               double *d_vxc, double *d_ghf, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_ws(mol, d_ws, ws_bytes))) return rc;
  if ((rc = check_functional(fn, d_ehf, n_omega))) return rc;
  if (d_rdm1 == nullptr || d_exc == nullptr) {
    set_error("%s: rdm1 and exc are required", who);
    return GDFT_ERR_INVALID;
  }
  if (d_ghf != nullptr && ((uintptr_t)d_ghf & 7)) {
    set_error("%s: ghf must be 8-byte aligned", who);
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const WsLayout W = ws_layout(mol);
  if ((rc = run_density(mol, d_rdm1, ws, st))) return rc;
  double *feat = (double *)(ws + W.off_feat);
  double *coef = d_vxc ? (double *)(ws + W.off_coef) : nullptr;
  double *epart = (double *)(ws + W.off_epart);
  {
    StageTimer tm(GDFT_STAGE_POINT, st);
    rc = check_cuda(launch_xc_point(feat, mol_w(mol), mol->n_grid, mol->n_grid_pad, *fn, d_ehf, n_omega, coef, epart,
                                    nullptr, st, d_ghf),
                    "xc_point");
    if (rc) return rc;
  }
  {
    StageTimer tm(GDFT_STAGE_REDUCE, st);
    if ((rc = check_cuda(launch_energy_reduce(epart, W.n_eblocks, d_exc, st), "energy_reduce"))) return rc;
  }
  if (d_vxc == nullptr) return GDFT_OK;
  return run_vxc(mol, coef, d_vxc, ws, st);
}

int gdft_xc_energy_and_grads(const gdft_molecule *mol, const double *d_rdm1, const gdft_functional *fn,
                             const double *d_ehf, int32_t n_omega, double *d_exc, double *d_vxc, void *d_ws,
                             size_t ws_bytes, void *stream) {
  return xc_energy_and_grads("gdft_xc_energy_and_grads", mol, d_rdm1, fn, d_ehf, n_omega, d_exc, d_vxc, nullptr,
                             d_ws, ws_bytes, stream);
}

int gdft_xc_energy_grads_hf(const gdft_molecule *mol, const double *d_rdm1, const gdft_functional *fn,
                            const double *d_ehf, int32_t n_omega, double *d_exc, double *d_vxc, double *d_ghf,
                            void *d_ws, size_t ws_bytes, void *stream) {
  return xc_energy_and_grads("gdft_xc_energy_grads_hf", mol, d_rdm1, fn, d_ehf, n_omega, d_exc, d_vxc, d_ghf, d_ws,
                             ws_bytes, stream);
}


// ---- k-points (Solid) ------------------------------------------------------
// Workspace: one molecule's layout, then the doubled real matrix M, the real
// V of one k-point and the features summed over k-points.
struct KptWs {
  size_t off_m, off_v, off_fsum, bytes;
};

static KptWs kpt_ws(const gdft_molecule *m) {
  KptWs K;
  size_t off = align256(ws_layout(m).bytes);
  const size_t mat = (size_t)2 * m->n_ao * m->n_ao * sizeof(double);
  K.off_m = off;
  off += align256(mat);
  K.off_v = off;
  off += align256(mat);
  K.off_fsum = off;
  off += align256((size_t)2 * kFeat * m->n_grid_pad * sizeof(double));
  K.bytes = off;
  return K;
}

static int check_kpts(const gdft_molecule *mols, int32_t n_kpt, const double *h_kweights, const char *who) {
  if (mols == nullptr || n_kpt <= 0 || h_kweights == nullptr) {
    set_error("%s: k-point molecules and weights are required (n_kpt=%d)", who, n_kpt);
    return GDFT_ERR_INVALID;
  }
  for (int k = 0; k < n_kpt; ++k) {
    int rc = check_mol(&mols[k]);
    if (rc) return rc;
    if (mols[k].n_grid != mols[0].n_grid || mols[k].n_ao != mols[0].n_ao ||
        mols[k].precision != mols[0].precision || (mols[k].n_ao & 1)) {
      set_error("%s: every k-point needs the same grid, form and an even n_ao (2 x crystal AOs)", who);
      return GDFT_ERR_INVALID;
    }
  }
  return GDFT_OK;
}

// Features summed over k-points into ws + off_fsum.
static int kpt_density(const gdft_molecule *mols, int32_t K, const double *rdm1c, const double *h_kweights,
                       char *ws, cudaStream_t st) {
  const WsLayout W = ws_layout(&mols[0]);
  const KptWs KW = kpt_ws(&mols[0]);
  const int n = mols[0].n_ao / 2;
  double *M = (double *)(ws + KW.off_m), *fsum = (double *)(ws + KW.off_fsum);
  const size_t nf = (size_t)2 * kFeat * mols[0].n_grid_pad;
  int rc;
  for (int k = 0; k < K; ++k) {
    if ((rc = check_cuda(launch_kpt_build_m(rdm1c, K, k, n, h_kweights[k], M, st), "kpt_build_m"))) return rc;
    if ((rc = run_density(&mols[k], M, ws, st))) return rc;
    if ((rc = check_cuda(launch_feat_add((const double *)(ws + W.off_feat), fsum, nf, k == 0, st), "feat_add")))
      return rc;
  }
  return GDFT_OK;
}

int gdft_kpoint_workspace_bytes(const gdft_molecule *mols, int32_t n_kpt, size_t *bytes) {
  double one = 1.0;
  int rc = check_kpts(mols, n_kpt, &one, "gdft_kpoint_workspace_bytes");
  if (rc) return rc;
  if (bytes == nullptr) {
    set_error("gdft_kpoint_workspace_bytes: null output");
    return GDFT_ERR_INVALID;
  }
  *bytes = kpt_ws(&mols[0]).bytes;
  return GDFT_OK;
}

static int check_kpt_ws(const gdft_molecule *m, void *ws, size_t ws_bytes) {
  const size_t need = kpt_ws(m).bytes;
  if (ws == nullptr || ws_bytes < need) {
    set_error("workspace of %zu bytes is smaller than the %zu bytes required", ws_bytes, need);
    return GDFT_ERR_WORKSPACE;
  }
  if (((uintptr_t)ws & 255u) != 0) {
    set_error("workspace must be 256-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  return GDFT_OK;
}

int gdft_kpoint_density(const gdft_molecule *mols, int32_t n_kpt, const double *d_rdm1, const double *h_kweights,
                        double *d_rho, double *d_grad_rho, double *d_lapl, double *d_tau, void *d_ws,
                        size_t ws_bytes, void *stream) {
  const char *who = "gdft_kpoint_density";
  int rc = check_kpts(mols, n_kpt, h_kweights, who);
  if (rc) return rc;
  if ((rc = check_kpt_ws(&mols[0], d_ws, ws_bytes))) return rc;
  if (d_rdm1 == nullptr || ((uintptr_t)d_rdm1 & 7)) {
    set_error("%s: rdm1 (2, n_kpt, n, n) complex is required, 8-byte aligned", who);
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  if ((rc = kpt_density(mols, n_kpt, d_rdm1, h_kweights, ws, st))) return rc;
  StageTimer tm(GDFT_STAGE_REDUCE, st);
  return check_cuda(launch_feat_to_reference((const double *)(ws + kpt_ws(&mols[0]).off_fsum), mols[0].n_grid,
                                             mols[0].n_grid_pad, d_rho, d_grad_rho, d_lapl, d_tau, st),
                    "feat_to_reference");
}

int gdft_kpoint_xc_energy_and_grads(const gdft_molecule *mols, int32_t n_kpt, const double *d_rdm1,
                                    const double *h_kweights, const gdft_functional *fn, double *d_exc,
                                    double *d_vxc, void *d_ws, size_t ws_bytes, void *stream) {
  const char *who = "gdft_kpoint_xc_energy_and_grads";
  int rc = check_kpts(mols, n_kpt, h_kweights, who);
  if (rc) return rc;
  if ((rc = check_kpt_ws(&mols[0], d_ws, ws_bytes))) return rc;
  if ((rc = check_functional(fn, nullptr, 0))) return rc;
  if (d_rdm1 == nullptr || d_exc == nullptr || (((uintptr_t)d_rdm1 | (uintptr_t)d_vxc) & 7)) {
    set_error("%s: rdm1 and exc are required, 8-byte aligned", who);
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const WsLayout W = ws_layout(&mols[0]);
  const KptWs KW = kpt_ws(&mols[0]);
  if ((rc = kpt_density(mols, n_kpt, d_rdm1, h_kweights, ws, st))) return rc;
  double *coef = d_vxc ? (double *)(ws + W.off_coef) : nullptr;
  double *epart = (double *)(ws + W.off_epart);
  {
    StageTimer tm(GDFT_STAGE_POINT, st);
    rc = check_cuda(launch_xc_point((const double *)(ws + KW.off_fsum), mol_w(&mols[0]), mols[0].n_grid,
                                    mols[0].n_grid_pad, *fn, nullptr, 0, coef, epart, nullptr, st),
                    "xc_point");
    if (rc) return rc;
  }
  {
    StageTimer tm(GDFT_STAGE_REDUCE, st);
    if ((rc = check_cuda(launch_energy_reduce(epart, W.n_eblocks, d_exc, st), "energy_reduce"))) return rc;
  }
  if (d_vxc == nullptr) return GDFT_OK;
  const int n = mols[0].n_ao / 2;
  double *V = (double *)(ws + KW.off_v);
  for (int k = 0; k < n_kpt; ++k) {
    if ((rc = run_vxc(&mols[k], coef, V, ws, st))) return rc;
    if ((rc = check_cuda(launch_kpt_vxc(V, n_kpt, k, n, h_kweights[k], d_vxc, st), "kpt_vxc"))) return rc;
  }
  return GDFT_OK;
}

int gdft_kpoint_coulomb(int32_t n_kpt, int32_t n_ao, const double *d_rep, const double *d_rdm1, const double *d_h1e,
                        const double *d_kweights, double nuclear_repulsion, double *d_vj, double *d_enonxc,
                        void *stream) {
  if (n_kpt <= 0 || n_ao <= 0 || d_rep == nullptr || d_rdm1 == nullptr || d_kweights == nullptr || d_vj == nullptr ||
      (d_enonxc != nullptr && d_h1e == nullptr)) {
    set_error("gdft_kpoint_coulomb: rep_tensor, rdm1, k-point weights and vj are required (h1e with the energy)");
    return GDFT_ERR_INVALID;
  }
  if (((uintptr_t)d_rep | (uintptr_t)d_rdm1 | (uintptr_t)d_h1e | (uintptr_t)d_kweights | (uintptr_t)d_vj |
       (uintptr_t)d_enonxc) &
      7) {
    set_error("gdft_kpoint_coulomb: pointers must be 8-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc = check_cuda(launch_kpt_coulomb(d_rep, d_rdm1, d_kweights, n_kpt, n_ao, d_vj, st), "kpt_coulomb");
  if (rc || d_enonxc == nullptr) return rc;
  return check_cuda(launch_kpt_nonxc(d_rdm1, d_h1e, d_vj, d_kweights, n_kpt, n_ao, nuclear_repulsion, d_enonxc, st),
                    "kpt_nonxc");
}

int gdft_kpoint_fock(int32_t n_kpt, int32_t n_ao, const double *d_h1e, const double *d_vj, const double *d_vxc,
                     double clip, double *d_fock, void *stream) {
  if (n_kpt <= 0 || n_ao <= 0 || d_h1e == nullptr || d_vj == nullptr || d_vxc == nullptr || d_fock == nullptr) {
    set_error("gdft_kpoint_fock: h1e, vj, vxc and fock are required");
    return GDFT_ERR_INVALID;
  }
  if (((uintptr_t)d_h1e | (uintptr_t)d_vj | (uintptr_t)d_vxc | (uintptr_t)d_fock) & 7) {
    set_error("gdft_kpoint_fock: pointers must be 8-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  return check_cuda(launch_kpt_fock(d_h1e, d_vj, d_vxc, n_kpt, n_ao, (double)n_kpt, clip, d_fock,
                                    (cudaStream_t)stream),
                    "kpt_fock");
}

int gdft_network_param_count(const gdft_network *net, size_t *count) {
  int rc = check_network(net);
  if (rc) return rc;
  if (count == nullptr) {
    set_error("gdft_network_param_count: null output");
    return GDFT_ERR_INVALID;
  }
  *count = mlp_param_count(net_shape(net));
  return GDFT_OK;
}

int gdft_neural_workspace_bytes(const gdft_molecule *mol, const gdft_network *net, size_t *bytes) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_network(net))) return rc;
  if (bytes == nullptr) {
    set_error("gdft_neural_workspace_bytes: null output");
    return GDFT_ERR_INVALID;
  }
  *bytes = neural_ws_bytes(mol, net);
  return GDFT_OK;
}

int gdft_neural_xc_energy_and_grads(const gdft_molecule *mol, const double *d_rdm1, const gdft_network *net,
                                    const double *d_params, const double *d_ehf, double *d_exc, double *d_vxc,
                                    double *d_dparams, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_network(net))) return rc;
  const size_t need = neural_ws_bytes(mol, net);
  if (d_ws == nullptr || ws_bytes < need) {
    set_error("workspace of %zu bytes is smaller than the %zu bytes required", ws_bytes, need);
    return GDFT_ERR_WORKSPACE;
  }
  if (((uintptr_t)d_ws & 255u) != 0) {
    set_error("workspace must be 256-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  if (d_rdm1 == nullptr || d_params == nullptr || d_ehf == nullptr || d_exc == nullptr) {
    set_error("gdft_neural_xc_energy_and_grads: rdm1, params, ehf and exc are required");
    return GDFT_ERR_INVALID;
  }
  if ((rc = check_aligned8(d_params, "params")) || (rc = check_aligned8(d_ehf, "ehf")) ||
      (d_dparams && (rc = check_aligned8(d_dparams, "dparams"))))
    return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const WsLayout W = ws_layout(mol);
  if ((rc = run_density(mol, d_rdm1, ws, st))) return rc;
  double *feat = (double *)(ws + W.off_feat);
  double *coef = d_vxc ? (double *)(ws + W.off_coef) : nullptr;
  {
    StageTimer tm(GDFT_STAGE_MLP, st);
    if (net->precision == GDFT_TF32X3)
      rc = mlp_run_tc(net_shape(net), d_params, d_dparams, feat, d_ehf, mol_w(mol), mol->n_grid, mol->n_grid_pad,
                      net->clip, ws + W.bytes, d_exc, coef, (int *)(ws + W.off_err), st);
    else
      rc = mlp_run_f64(net_shape(net), d_params, d_dparams, feat, d_ehf, mol_w(mol), mol->n_grid, mol->n_grid_pad,
                       net->clip, (double *)(ws + W.bytes), d_exc, coef, st);
    if (rc) return rc;
  }
  if (d_vxc == nullptr) return GDFT_OK;
  return run_vxc(mol, coef, d_vxc, ws, st);
}

int gdft_neural_xc_hf_grads(const gdft_molecule *mol, const double *d_rdm1, const gdft_network *net,
                            const double *d_params, const double *d_ehf, double *d_exc, double *d_vxc,
                            double *d_g_dens, double *d_g_cin, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_network(net))) return rc;
  if (net->n_in != kDm21In || net->n_out != kDm21Out) {
    set_error("gdft_neural_xc_hf_grads: the HF gradients are built for the DM21 network (11 inputs, 3 outputs)");
    return GDFT_ERR_INVALID;
  }
  const size_t need = neural_ws_bytes(mol, net);
  if (d_ws == nullptr || ws_bytes < need) {
    set_error("workspace of %zu bytes is smaller than the %zu bytes required", ws_bytes, need);
    return GDFT_ERR_WORKSPACE;
  }
  if (((uintptr_t)d_ws & 255u) != 0) {
    set_error("workspace must be 256-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  if (d_rdm1 == nullptr || d_params == nullptr || d_ehf == nullptr || d_exc == nullptr ||
      (d_g_dens == nullptr && d_g_cin == nullptr)) {
    set_error("gdft_neural_xc_hf_grads: rdm1, params, ehf, exc and one of g_dens, g_cin are required");
    return GDFT_ERR_INVALID;
  }
  if ((rc = check_aligned8(d_params, "params")) || (rc = check_aligned8(d_ehf, "ehf")) ||
      (d_g_dens && (rc = check_aligned8(d_g_dens, "g_dens"))) || (d_g_cin && (rc = check_aligned8(d_g_cin, "g_cin"))))
    return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const WsLayout W = ws_layout(mol);
  if ((rc = run_density(mol, d_rdm1, ws, st))) return rc;
  double *feat = (double *)(ws + W.off_feat);
  double *coef = (double *)(ws + W.off_coef);
  double *mws = (double *)(ws + W.bytes);
  {
    StageTimer tm(GDFT_STAGE_MLP, st);
    if (net->precision == GDFT_TF32X3)
      rc = mlp_run_tc(net_shape(net), d_params, nullptr, feat, d_ehf, mol_w(mol), mol->n_grid, mol->n_grid_pad,
                      net->clip, ws + W.bytes, d_exc, coef, (int *)(ws + W.off_err), st);
    else
      rc = mlp_run_f64(net_shape(net), d_params, nullptr, feat, d_ehf, mol_w(mol), mol->n_grid, mol->n_grid_pad,
                       net->clip, mws, d_exc, coef, st);
    if (rc) return rc;
  }
  if (net->precision == GDFT_TF32X3) {
    const MlpTcLayout T = mlp_tc_layout(net_shape(net), mol->n_grid_pad);
    const char *nws = ws + W.bytes;
    rc = check_cuda(launch_dm21_hf_grads_from((const double *)(nws + T.x), (const double *)(nws + T.du),
                                              (const double *)(nws + T.de), mol->n_grid, net->squash_offset,
                                              d_g_dens, d_g_cin, st),
                    "dm21_hf_grads");
  } else {
    rc = check_cuda(launch_dm21_hf_grads(net_shape(net), mol->n_grid, mol->n_grid_pad, mws, d_g_dens, d_g_cin, st),
                    "dm21_hf_grads");
  }
  if (rc) return rc;
  if (d_vxc == nullptr) return GDFT_OK;
  return run_vxc(mol, coef, d_vxc, ws, st);
}

int gdft_neural_inputs(const gdft_molecule *mol, const double *d_rdm1, const gdft_network *net, const double *d_ehf,
                       double *d_cinputs, double *d_dens, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_network(net))) return rc;
  const size_t need = neural_ws_bytes(mol, net);
  if (d_ws == nullptr || ws_bytes < need) {
    set_error("workspace of %zu bytes is smaller than the %zu bytes required", ws_bytes, need);
    return GDFT_ERR_WORKSPACE;
  }
  if (((uintptr_t)d_ws & 255u) != 0) {
    set_error("workspace must be 256-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  if (d_rdm1 == nullptr || d_ehf == nullptr) {
    set_error("gdft_neural_inputs: rdm1 and ehf are required");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const WsLayout W = ws_layout(mol);
  if ((rc = run_density(mol, d_rdm1, ws, st))) return rc;
  StageTimer tm(GDFT_STAGE_MLP, st);
  return mlp_inputs_f64(net_shape(net), (const double *)(ws + W.off_feat), d_ehf, mol->n_grid, mol->n_grid_pad,
                        net->clip, (double *)(ws + W.bytes), d_cinputs, d_dens, st);
}

int gdft_network_apply_workspace_bytes(const gdft_network *net, int64_t n_rows, size_t *bytes) {
  int rc = check_network(net);
  if (rc) return rc;
  if (n_rows <= 0 || bytes == nullptr) {
    set_error("gdft_network_apply_workspace_bytes: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  *bytes = align256(mlp_layout(net_shape(net), n_rows).doubles * sizeof(double));
  return GDFT_OK;
}

int gdft_network_apply(const gdft_network *net, const double *d_params, int64_t n_rows, const double *d_x,
                       double *d_c, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_network(net);
  if (rc) return rc;
  if (n_rows <= 0 || d_params == nullptr || d_x == nullptr || d_c == nullptr) {
    set_error("gdft_network_apply: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  const size_t need = align256(mlp_layout(net_shape(net), n_rows).doubles * sizeof(double));
  if (d_ws == nullptr || ws_bytes < need) {
    set_error("workspace of %zu bytes is smaller than the %zu bytes required", ws_bytes, need);
    return GDFT_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  StageTimer tm(GDFT_STAGE_MLP, st);
  return mlp_apply_f64(net_shape(net), d_params, d_x, n_rows, (double *)d_ws, d_c, st);
}

int gdft_neural_hvp_workspace_bytes(const gdft_molecule *mol, const gdft_network *net, size_t *bytes) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_network(net))) return rc;
  if (bytes == nullptr) {
    set_error("gdft_neural_hvp_workspace_bytes: null output");
    return GDFT_ERR_INVALID;
  }
  *bytes = hvp_ws_bytes(mol, net);
  return GDFT_OK;
}

int gdft_neural_xc_hvp(const gdft_molecule *mol, const double *d_rdm1, const gdft_network *net,
                       const double *d_params, const double *d_ehf, const double *d_tangent, double *d_value,
                       double *d_hrdm1, double *d_hparams, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_network(net))) return rc;
  const size_t need = hvp_ws_bytes(mol, net);
  if (d_ws == nullptr || ws_bytes < need) {
    set_error("workspace of %zu bytes is smaller than the %zu bytes required", ws_bytes, need);
    return GDFT_ERR_WORKSPACE;
  }
  if (((uintptr_t)d_ws & 255u) != 0) {
    set_error("workspace must be 256-byte aligned");
    return GDFT_ERR_ALIGNMENT;
  }
  if (d_rdm1 == nullptr || d_params == nullptr || d_ehf == nullptr || d_tangent == nullptr) {
    set_error("gdft_neural_xc_hvp: rdm1, params, ehf and tangent are required");
    return GDFT_ERR_INVALID;
  }
  if ((rc = check_aligned8(d_params, "params")) || (rc = check_aligned8(d_ehf, "ehf")) ||
      (rc = check_aligned8(d_tangent, "tangent")))
    return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const WsLayout W = ws_layout(mol);
  const MlpShape S = net_shape(net);
  const bool tc = net->precision == GDFT_TF32X3;
  char *hws = ws + W.bytes;
  double *featp = (double *)(hws + (tc ? mlp_hvp_tc_layout(S, mol->n_grid_pad).featp
                                       : mlp_hvp_layout(S, mol->n_grid_pad).featp * sizeof(double)));
  double *feat = (double *)(ws + W.off_feat);
  // Features of D (kept in the second-order scratch), then of the tangent G.
  if ((rc = run_density(mol, d_rdm1, ws, st))) return rc;
  if ((rc = check_cuda(cudaMemcpyAsync(featp, feat, (size_t)2 * kFeat * mol->n_grid_pad * sizeof(double),
                                       cudaMemcpyDeviceToDevice, st),
                       "hvp feature copy")))
    return rc;
  if ((rc = run_density(mol, d_tangent, ws, st))) return rc;
  double *coef = d_hrdm1 ? (double *)(ws + W.off_coef) : nullptr;
  {
    StageTimer tm(GDFT_STAGE_MLP, st);
    if (tc)
      rc = mlp_hvp_tc(S, d_params, d_hparams, featp, feat, d_ehf, mol_w(mol), mol->n_grid, mol->n_grid_pad,
                      net->clip, hws, d_value, coef, (int *)(ws + W.off_err), st);
    else
      rc = mlp_hvp_f64(S, d_params, d_hparams, featp, feat, d_ehf, mol_w(mol), mol->n_grid, mol->n_grid_pad,
                       net->clip, (double *)hws, d_value, coef, st);
    if (rc) return rc;
  }
  if (d_hrdm1 == nullptr) return GDFT_OK;
  return run_vxc(mol, coef, d_hrdm1, ws, st);
}

int gdft_neural_batch_workspace_bytes(int32_t n_mol, const gdft_molecule *mols, const gdft_network *net,
                                      size_t *bytes) {
  int rc = check_network(net);
  if (rc) return rc;
  if (bytes == nullptr) {
    set_error("gdft_neural_batch_workspace_bytes: null output");
    return GDFT_ERR_INVALID;
  }
  static thread_local BatchLayout B;
  if ((rc = batch_layout(n_mol, mols, net, &B))) return rc;
  *bytes = B.bytes;
  return GDFT_OK;
}

int gdft_neural_batch_xc(int32_t n_mol, const gdft_molecule *mols, const double *const *h_rdm1,
                         const double *const *h_ehf, const gdft_network *net, const double *d_params,
                         const double *d_eref, double *d_energies, double *d_loss, double *const *h_vxc,
                         double *d_dparams, void *d_ws, size_t ws_bytes, void *stream) {
  int rc = check_network(net);
  if (rc) return rc;
  if (net->precision != GDFT_TF32X3) {
    set_error("gdft_neural_batch_xc needs the TF32x3 network form");
    return GDFT_ERR_UNSUPPORTED;
  }
  static thread_local BatchLayout B;
  if ((rc = batch_layout(n_mol, mols, net, &B))) return rc;
  if (d_ws == nullptr || ws_bytes < B.bytes || ((uintptr_t)d_ws & 255u) != 0) {
    set_error("batch workspace of %zu bytes (256-byte aligned) is smaller than the %zu bytes required", ws_bytes,
              B.bytes);
    return GDFT_ERR_WORKSPACE;
  }
  if (h_rdm1 == nullptr || h_ehf == nullptr || d_params == nullptr || d_energies == nullptr) {
    set_error("gdft_neural_batch_xc: rdm1, ehf, params and energies are required");
    return GDFT_ERR_INVALID;
  }
  for (int m = 0; m < n_mol; ++m)
    if (h_rdm1[m] == nullptr || h_ehf[m] == nullptr) {
      set_error("gdft_neural_batch_xc: molecule %d has no rdm1 or ehf", m);
      return GDFT_ERR_INVALID;
    }
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const int64_t npt = B.npt;
  double *feat = (double *)(ws + B.off_feat), *w = (double *)(ws + B.off_w), *ehf = (double *)(ws + B.off_ehf);
  double *coef = (double *)(ws + B.off_coef), *cot = (double *)(ws + B.off_cot);
  int64_t *seg = (int64_t *)(ws + B.off_seg);
  {
    SegTable t;
    for (int m = 0; m <= n_mol; ++m) t.off[m] = B.seg[m];
    write_seg_kernel<<<1, 256, 0, st>>>(t, n_mol, seg);
    if ((rc = check_cuda(cudaGetLastError(), "batch segments"))) return rc;
  }
  if ((rc = check_cuda(cudaMemsetAsync(feat, 0, (size_t)2 * kFeat * npt * 8, st), "batch clear")) ||
      (rc = check_cuda(cudaMemsetAsync(w, 0, (size_t)npt * 8, st), "batch clear")) ||
      (rc = check_cuda(cudaMemsetAsync(ehf, 0, (size_t)4 * npt * 8, st), "batch clear")))
    return rc;
  int *batch_err = (int *)ws;
  char *wsm = ws + B.off_mol;  // the shared molecule region
  // A molecule's error word sits where its own layout puts it in the shared
  // region: cleared before the molecule's stage (a previous molecule's data may
  // lie there) and folded into the batch's word after it.
  auto mol_err = [&](const gdft_molecule *mol) { return (int *)(wsm + ws_layout(mol).off_err); };
  if (B.ragged) {
    // Every molecule's density in one persistent launch over all their tiles,
    // straight into the joint feature array.
    DensMol dm[kBatchMax];
    {
      StageTimer tm(GDFT_STAGE_REDUCE, st);
      for (int m = 0; m < n_mol; ++m) {
        const gdft_molecule *mol = &mols[m];
        const int ldk = (int)round_up(mol->n_ao, 128);
        float *dpk = (float *)(ws + B.off_dpk[m]);
        if ((rc = check_cuda(launch_pack_rdm1(h_rdm1[m], mol->n_ao, ldk, dpk, st), "batch pack_rdm1"))) return rc;
        dm[m] = DensMol{mol_pm(mol), dpk, mol->n_grid_pad, ldk, feat + B.seg[m], npt};
      }
    }
    StageTimer tm(GDFT_STAGE_DENSITY, st);
    if ((rc = check_cuda(launch_dens_tc_ragged(dm, n_mol, ws + B.off_queue, batch_err, st), "batch dens_tc")))
      return rc;
  }
  for (int m = 0; m < n_mol; ++m) {
    const gdft_molecule *mol = &mols[m];
    const WsLayout W = ws_layout(mol);
    const int64_t np = mol->n_grid_pad, off = B.seg[m];
    if (B.ragged) {
      if ((rc = check_cuda(cudaMemcpyAsync(w + off, mol_w(mol), (size_t)np * 8, cudaMemcpyDeviceToDevice, st),
                           "batch weights")) ||
          (rc = check_cuda(cudaMemcpy2DAsync(ehf + off, (size_t)npt * 8, h_ehf[m], (size_t)mol->n_grid * 8,
                                             (size_t)mol->n_grid * 8, 4, cudaMemcpyDeviceToDevice, st),
                           "batch ehf")))
        return rc;
      continue;
    }
    if ((rc = check_cuda(cudaMemsetAsync(mol_err(mol), 0, sizeof(int), st), "batch error word"))) return rc;
    if ((rc = run_density(mol, h_rdm1[m], wsm, st))) return rc;
    if ((rc = check_cuda(launch_err_fold(batch_err, mol_err(mol), st), "batch error fold"))) return rc;
    if ((rc = check_cuda(cudaMemcpy2DAsync(feat + off, (size_t)npt * 8, wsm + W.off_feat, (size_t)np * 8,
                                           (size_t)np * 8, 2 * kFeat, cudaMemcpyDeviceToDevice, st),
                         "batch features")) ||
        (rc = check_cuda(cudaMemcpyAsync(w + off, mol_w(mol), (size_t)np * 8, cudaMemcpyDeviceToDevice, st),
                         "batch weights")) ||
        (rc = check_cuda(cudaMemcpy2DAsync(ehf + off, (size_t)npt * 8, h_ehf[m], (size_t)mol->n_grid * 8,
                                           (size_t)mol->n_grid * 8, 4, cudaMemcpyDeviceToDevice, st),
                         "batch ehf")))
      return rc;
  }
  MlpSegments sg{n_mol, seg, d_eref, d_energies, d_loss, cot};
  {
    StageTimer tm(GDFT_STAGE_MLP, st);
    rc = mlp_run_tc(net_shape(net), d_params, d_dparams, feat, ehf, w, npt, npt, net->clip, ws + B.off_net, nullptr,
                    coef, batch_err, st, &sg);
    if (rc) return rc;
  }
  for (int m = 0; m < n_mol; ++m) {
    if (h_vxc == nullptr || h_vxc[m] == nullptr) continue;
    const gdft_molecule *mol = &mols[m];
    const WsLayout W = ws_layout(mol);
    const int64_t np = mol->n_grid_pad, off = B.seg[m];
    if ((rc = check_cuda(cudaMemsetAsync(mol_err(mol), 0, sizeof(int), st), "batch error word")) ||
        (rc = check_cuda(cudaMemcpy2DAsync(wsm + W.off_coef, (size_t)np * 8, coef + off, (size_t)npt * 8,
                                           (size_t)np * 8, 2 * kFeat, cudaMemcpyDeviceToDevice, st),
                         "batch coefficients")))
      return rc;
    if ((rc = run_vxc(mol, (const double *)(wsm + W.off_coef), h_vxc[m], wsm, st))) return rc;
    if ((rc = check_cuda(launch_err_fold(batch_err, mol_err(mol), st), "batch error fold"))) return rc;
  }
  return GDFT_OK;
}

int gdft_neural_batch_status(void *d_ws, size_t ws_bytes, int32_t *status, void *stream) {
  return persistent_status("gdft_neural_batch_status", d_ws, ws_bytes, status, stream);
}

int gdft_vxc_from_potentials(const gdft_molecule *mol, const double *d_pot, double *d_vxc, void *d_ws,
                             size_t ws_bytes, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_ws(mol, d_ws, ws_bytes))) return rc;
  if (d_pot == nullptr || d_vxc == nullptr) {
    set_error("gdft_vxc_from_potentials: potentials and vxc are required");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const WsLayout W = ws_layout(mol);
  double *coef = (double *)(ws + W.off_coef);
  {
    StageTimer tm(GDFT_STAGE_REDUCE, st);
    if ((rc = check_cuda(launch_pad_potentials(d_pot, mol->n_grid, mol->n_grid_pad, coef, st), "pad_potentials")))
      return rc;
  }
  return run_vxc(mol, coef, d_vxc, ws, st);
}

int gdft_device_status(const gdft_molecule *mol, void *d_ws, size_t ws_bytes, int32_t *status, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_ws(mol, d_ws, ws_bytes))) return rc;
  if (status == nullptr) {
    set_error("gdft_device_status: null output");
    return GDFT_ERR_INVALID;
  }
  const WsLayout W = ws_layout(mol);
  int *err = (int *)((char *)d_ws + W.off_err);
  int h = 0;
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = check_cuda(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st), "status read"))) return rc;
  if ((rc = check_cuda(cudaStreamSynchronize(st), "status sync"))) return rc;
  if ((rc = check_cuda(cudaMemsetAsync(err, 0, sizeof(int), st), "status clear"))) return rc;
  *status = h;
  if (h != 0) {
    set_error("a device-side wait expired (code %d); results of the last calls are invalid", h);
    return GDFT_ERR_DEVICE;
  }
  return GDFT_OK;
}

int gdft_selftest_wait_expiry(const gdft_molecule *mol, void *d_ws, size_t ws_bytes, int32_t limit, void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_ws(mol, d_ws, ws_bytes))) return rc;
  if (limit < 1 || limit > 65536) {
    set_error("gdft_selftest_wait_expiry: limit %d outside 1..65536 polls", limit);
    return GDFT_ERR_INVALID;
  }
  int *err = (int *)((char *)d_ws + ws_layout(mol).off_err);
  return check_cuda(launch_wait_expiry_probe(err, (uint32_t)limit, GDFT_WAIT_EXPIRY_PROBE, (cudaStream_t)stream),
                    "wait expiry probe");
}

int gdft_energy_densities(const gdft_molecule *mol, const double *d_rdm1, const gdft_functional *fn,
                          const double *d_ehf, int32_t n_omega, double *d_dens, void *d_ws, size_t ws_bytes,
                          void *stream) {
  int rc = check_mol(mol);
  if (rc) return rc;
  if ((rc = check_ws(mol, d_ws, ws_bytes))) return rc;
  if ((rc = check_functional(fn, d_ehf, n_omega))) return rc;
  if (d_rdm1 == nullptr || d_dens == nullptr) {
    set_error("gdft_energy_densities: rdm1 and dens are required");
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *ws = (char *)d_ws;
  const WsLayout W = ws_layout(mol);
  if ((rc = run_density(mol, d_rdm1, ws, st))) return rc;
  return check_cuda(launch_xc_point((double *)(ws + W.off_feat), mol_w(mol), mol->n_grid, mol->n_grid_pad, *fn,
                                    d_ehf, n_omega, nullptr, (double *)(ws + W.off_epart), d_dens, st),
                    "xc_point");
}

// Largest grid whose block count (n_grid + 255) / 256 fits the int of integrate_blocks.
static constexpr int64_t kIntegrateMaxGrid = (int64_t)INT32_MAX * 256 - 255;

int gdft_integrate_workspace_bytes(int64_t n_grid, size_t *bytes) {
  if (n_grid <= 0 || n_grid > kIntegrateMaxGrid || bytes == nullptr) {
    set_error("gdft_integrate_workspace_bytes: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  *bytes = align256((size_t)integrate_blocks(n_grid) * sizeof(double));
  return GDFT_OK;
}

int gdft_integrate(int64_t n_grid, int32_t n_cols, const double *h_coeffs, int32_t n_coeffs, const double *d_dens,
                   const double *d_weights, double clip, double *d_exc, void *d_ws, size_t ws_bytes, void *stream) {
  if (n_grid <= 0 || n_cols < 1 || !(n_coeffs == 1 || n_coeffs == n_cols) || n_coeffs > GDFT_MAX_COLS ||
      h_coeffs == nullptr || d_dens == nullptr || d_weights == nullptr || d_exc == nullptr) {
    set_error("gdft_integrate: invalid arguments (n_cols=%d, n_coeffs=%d)", n_cols, n_coeffs);
    return GDFT_ERR_INVALID;
  }
  if (n_grid > kIntegrateMaxGrid) {  // block counts are int: checked before they are formed
    set_error("gdft_integrate: n_grid=%lld is beyond the supported %lld", (long long)n_grid,
              (long long)kIntegrateMaxGrid);
    return GDFT_ERR_INVALID;
  }
  const size_t need = align256((size_t)integrate_blocks(n_grid) * sizeof(double));
  if (d_ws == nullptr || ws_bytes < need) {
    set_error("gdft_integrate: workspace of %zu bytes is smaller than %zu", ws_bytes, need);
    return GDFT_ERR_WORKSPACE;
  }
  gdft_functional fn;
  memset(&fn, 0, sizeof(fn));
  fn.n_cols = n_cols;
  fn.n_coeffs = n_coeffs;
  for (int i = 0; i < n_coeffs; ++i) fn.coeffs[i] = h_coeffs[i];
  fn.clip = clip;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = check_cuda(launch_integrate(n_grid, n_cols, fn, d_dens, d_weights, (double *)d_ws, st), "integrate");
  if (rc) return rc;
  return check_cuda(launch_energy_reduce((const double *)d_ws, integrate_blocks(n_grid), d_exc, st), "energy_reduce");
}

int gdft_fock(int32_t n_ao, const double *d_h1e, const double *d_vj, const double *d_vxc, double clip,
              double *d_fock, void *stream) {
  if (n_ao <= 0 || !d_h1e || !d_vj || !d_vxc || !d_fock) {
    set_error("gdft_fock: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  return check_cuda(launch_fock(n_ao, d_h1e, d_vj, d_vxc, clip, d_fock, (cudaStream_t)stream), "fock");
}

int gdft_coulomb(int32_t n_ao, const double *d_eri, const double *d_rdm1, const double *d_h1e,
                 double nuclear_repulsion, double *d_vj, double *d_enonxc, void *stream) {
  if (n_ao <= 0 || !d_eri || !d_rdm1 || !d_vj || (d_enonxc && !d_h1e)) {
    set_error("gdft_coulomb: invalid arguments");
    return GDFT_ERR_INVALID;
  }
  return check_cuda(launch_coulomb(n_ao, d_eri, d_rdm1, d_h1e, nuclear_repulsion, d_vj, d_enonxc,
                                   (cudaStream_t)stream),
                    "coulomb");
}

}  // extern "C"

// ---- grid-chunked evaluation: phi recomputed per chunk ----------------------
// The AO tables of one chunk of grid points are evaluated from the basis into a
// chunk buffer, read by that chunk's density, point and V_xc stages, and
// overwritten by the next chunk: phi is recomputed where it is needed instead
// of being held for the whole grid.  E_xc, V_xc (and dE/dtheta) accumulate over
// the chunks on the device.  Workspace: [persistent error word (256 B)][chunk
// molecule buffer][chunk workspace][ehf slice][chunk E][chunk V][chunk dtheta].
constexpr int kChunkMaxOmega = 4;

struct ChunkWs {
  size_t off_mol, mol_bytes, off_ws, ws_bytes, off_ehf, off_e, off_v, off_dp, bytes;
};

static ChunkWs chunk_ws(int32_t n_ao, int64_t chunk, int32_t precision, const gdft_network *net) {
  ChunkWs C;
  size_t off = 256;  // the persistent error word
  const MolLayout L = mol_layout(chunk, n_ao, precision);
  C.off_mol = off;
  C.mol_bytes = L.bytes;
  off += align256(L.bytes);
  gdft_molecule m{chunk, L.np, n_ao, L.ld, precision, 0, nullptr, L.bytes};
  C.ws_bytes = net ? neural_ws_bytes(&m, net) : ws_layout(&m).bytes;
  C.off_ws = off;
  off += align256(C.ws_bytes);
  C.off_ehf = off;
  off += align256((size_t)kChunkMaxOmega * 2 * chunk * sizeof(double));
  C.off_e = off;
  off += 256;
  C.off_v = off;
  off += align256((size_t)2 * n_ao * n_ao * sizeof(double));
  C.off_dp = off;
  off += net ? align256(mlp_param_count(net_shape(net)) * sizeof(double)) : 0;
  C.bytes = off;
  return C;
}

static int check_chunked(const gdft_basis *shells, const double *rows, int32_t n_ao, const double *coords,
                         const double *weights, int64_t n_grid, int64_t chunk, int32_t precision, void *ws,
                         const char *who, ShellView *B) {
  if ((shells == nullptr) == (rows == nullptr)) {
    set_error("%s: give exactly one of a contracted basis and synthetic basis rows", who);
    return GDFT_ERR_INVALID;
  }
  int rc;
  if (shells != nullptr) {
    if ((rc = check_basis(shells, who, B))) return rc;
    if (shells->n_ao != n_ao) {
      set_error("%s: the basis has %d AOs, n_ao is %d", who, shells->n_ao, n_ao);
      return GDFT_ERR_INVALID;
    }
  }
  if (n_ao <= 0 || n_grid <= 0 || chunk < 128 || chunk % 256 != 0 || coords == nullptr || weights == nullptr ||
      !(precision == GDFT_FP64 || precision == GDFT_TF32X3)) {
    set_error("%s: n_ao %d, n_grid %lld, chunk %lld (a multiple of 256), precision %d", who, n_ao,
              (long long)n_grid, (long long)chunk, precision);
    return GDFT_ERR_INVALID;
  }
  if ((rc = check_aligned8(coords, "coords")) || (rc = check_aligned8(weights, "weights"))) return rc;
  if (((uintptr_t)ws & 255u) != 0) {
    set_error("%s: workspace must be 256-byte aligned", who);
    return GDFT_ERR_ALIGNMENT;
  }
  return GDFT_OK;
}

// AO tables of points [off, off + len) into the chunk molecule.
static int chunk_tables(const gdft_molecule *m, const ShellView *B, const double *rows, const double *coords,
                        const double *weights, int64_t off, cudaStream_t st) {
  const MolLayout L = mol_layout(m->n_grid, m->n_ao, m->precision);
  char *buf = (char *)m->buffer;
  double *w = (double *)(buf + L.off_w);
  const double *c = coords + 3 * off, *wt = weights + off;
  StageTimer tm(GDFT_STAGE_AO, st);
  if (m->precision == GDFT_TF32X3)
    return check_cuda(launch_pack_tables(nullptr, nullptr, nullptr, rows, c, wt, m->n_grid, m->n_ao, L.np, L.ldk,
                                         (float *)(buf + L.off_pm), (float *)(buf + L.off_av),
                                         (float *)(buf + L.off_af), w, st, B),
                      "chunk tables");
  if (B != nullptr)
    return check_cuda(launch_eval_shell_tables(*B, c, wt, m->n_grid, L.np, L.ld, (double *)(buf + L.off_tab), w, st),
                      "chunk tables");
  return check_cuda(launch_eval_basis(rows, c, wt, m->n_grid, m->n_ao, L.np, L.ld, (double *)(buf + L.off_tab), w,
                                      st),
                    "chunk tables");
}

// One chunk's stages; `net` selects the network pass, `fn` the constant-coefficient one.
static int chunk_pass(const gdft_molecule *m, char *ws, const ChunkWs &C, char *base, const double *rdm1,
                      const gdft_functional *fn, const gdft_network *net, const double *params, const double *ehf,
                      int n_omega, int64_t n_grid, int64_t off, bool first, double *exc, double *vxc,
                      double *dparams, cudaStream_t st) {
  const WsLayout W = ws_layout(m);
  int rc;
  // A shorter (last) chunk's layout puts its error word where the full chunks kept other data.
  if ((rc = check_cuda(cudaMemsetAsync(ws + W.off_err, 0, sizeof(int), st), "chunk status clear"))) return rc;
  if ((rc = run_density(m, rdm1, ws, st))) return rc;
  const double *ehf_c = nullptr;
  if (ehf != nullptr) {  // this chunk's columns of ehf (omega, spin, grid)
    double *dst = (double *)(base + C.off_ehf);
    if ((rc = check_cuda(cudaMemcpy2DAsync(dst, (size_t)m->n_grid * 8, ehf + off, (size_t)n_grid * 8,
                                           (size_t)m->n_grid * 8, (size_t)2 * n_omega, cudaMemcpyDeviceToDevice, st),
                         "chunk ehf")))
      return rc;
    ehf_c = dst;
  }
  double *feat = (double *)(ws + W.off_feat);
  double *coef = vxc ? (double *)(ws + W.off_coef) : nullptr;
  double *e_c = (double *)(base + C.off_e);
  double *dp_c = dparams ? (double *)(base + C.off_dp) : nullptr;
  if (net != nullptr) {
    StageTimer tm(GDFT_STAGE_MLP, st);
    if (net->precision == GDFT_TF32X3)
      rc = mlp_run_tc(net_shape(net), params, dp_c, feat, ehf_c, mol_w(m), m->n_grid, m->n_grid_pad, net->clip,
                      ws + W.bytes, e_c, coef, (int *)(ws + W.off_err), st);
    else
      rc = mlp_run_f64(net_shape(net), params, dp_c, feat, ehf_c, mol_w(m), m->n_grid, m->n_grid_pad, net->clip,
                       (double *)(ws + W.bytes), e_c, coef, st);
    if (rc) return rc;
  } else {
    double *epart = (double *)(ws + W.off_epart);
    {
      StageTimer tm(GDFT_STAGE_POINT, st);
      if ((rc = check_cuda(launch_xc_point(feat, mol_w(m), m->n_grid, m->n_grid_pad, *fn, ehf_c, n_omega, coef,
                                           epart, nullptr, st),
                           "xc_point")))
        return rc;
    }
    StageTimer tm(GDFT_STAGE_REDUCE, st);
    if ((rc = check_cuda(launch_energy_reduce(epart, W.n_eblocks, e_c, st), "energy_reduce"))) return rc;
  }
  {
    StageTimer tm(GDFT_STAGE_REDUCE, st);
    if ((rc = check_cuda(launch_feat_add(e_c, exc, 1, first, st), "chunk E"))) return rc;
    if (dparams &&
        (rc = check_cuda(launch_feat_add(dp_c, dparams, mlp_param_count(net_shape(net)), first, st), "chunk dtheta")))
      return rc;
  }
  if (vxc != nullptr) {
    double *v_c = (double *)(base + C.off_v);
    if ((rc = run_vxc(m, coef, v_c, ws, st))) return rc;
    StageTimer tm(GDFT_STAGE_REDUCE, st);
    if ((rc = check_cuda(launch_feat_add(v_c, vxc, (size_t)2 * m->n_ao * m->n_ao, first, st), "chunk V")))
      return rc;
  }
  return check_cuda(launch_err_fold((int *)base, (int *)(ws + W.off_err), st), "chunk status");
}

static int run_chunked(const char *who, const gdft_basis *shells, const double *rows, int32_t n_ao,
                       const double *coords, const double *weights, int64_t n_grid, int64_t chunk, int32_t precision,
                       const double *rdm1, const gdft_functional *fn, const gdft_network *net, const double *params,
                       const double *ehf, int32_t n_omega, double *exc, double *vxc, double *dparams, void *d_ws,
                       size_t ws_bytes, void *stream) {
  ShellView B;
  int rc = check_chunked(shells, rows, n_ao, coords, weights, n_grid, chunk, precision, d_ws, who, &B);
  if (rc) return rc;
  const ChunkWs C = chunk_ws(n_ao, chunk, precision, net);
  if (d_ws == nullptr || ws_bytes < C.bytes) {
    set_error("%s: workspace of %zu bytes is smaller than the %zu bytes required", who, ws_bytes, C.bytes);
    return GDFT_ERR_WORKSPACE;
  }
  if (rdm1 == nullptr || exc == nullptr) {
    set_error("%s: rdm1 and exc are required", who);
    return GDFT_ERR_INVALID;
  }
  if (ehf != nullptr && (n_omega < 1 || n_omega > kChunkMaxOmega)) {
    set_error("%s: n_omega %d outside 1..%d", who, n_omega, kChunkMaxOmega);
    return GDFT_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *base = (char *)d_ws;
  for (int64_t off = 0; off < n_grid; off += chunk) {
    const int64_t len = n_grid - off < chunk ? n_grid - off : chunk;
    gdft_molecule m;
    if ((rc = gdft_molecule_init(&m, len, n_ao, precision, base + C.off_mol, C.mol_bytes))) return rc;
    if ((rc = chunk_tables(&m, shells ? &B : nullptr, rows, coords, weights, off, st))) return rc;
    if ((rc = chunk_pass(&m, base + C.off_ws, C, base, rdm1, fn, net, params, ehf, n_omega, n_grid, off, off == 0,
                         exc, vxc, dparams, st)))
      return rc;
  }
  return GDFT_OK;
}

extern "C" {

int gdft_chunked_workspace_bytes(int32_t n_ao, int64_t chunk, int32_t precision, const gdft_network *net,
                                 size_t *bytes) {
  if (bytes == nullptr || n_ao <= 0 || chunk < 128 || chunk % 256 != 0 ||
      !(precision == GDFT_FP64 || precision == GDFT_TF32X3)) {
    set_error("gdft_chunked_workspace_bytes: n_ao %d, chunk %lld (a multiple of 256), precision %d", n_ao,
              (long long)chunk, precision);
    return GDFT_ERR_INVALID;
  }
  if (net != nullptr) {
    int rc = check_network(net);
    if (rc) return rc;
  }
  *bytes = chunk_ws(n_ao, chunk, precision, net).bytes;
  return GDFT_OK;
}

int gdft_xc_energy_and_grads_chunked(const gdft_basis *shells, const double *d_basis_rows, int32_t n_ao,
                                     const double *d_coords, const double *d_weights, int64_t n_grid, int64_t chunk,
                                     int32_t precision, const double *d_rdm1, const gdft_functional *fn,
                                     const double *d_ehf, int32_t n_omega, double *d_exc, double *d_vxc, void *d_ws,
                                     size_t ws_bytes, void *stream) {
  int rc = check_functional(fn, d_ehf, n_omega);
  if (rc) return rc;
  return run_chunked("gdft_xc_energy_and_grads_chunked", shells, d_basis_rows, n_ao, d_coords, d_weights, n_grid,
                     chunk, precision, d_rdm1, fn, nullptr, nullptr, d_ehf, n_omega, d_exc, d_vxc, nullptr, d_ws,
                     ws_bytes, stream);
}

int gdft_neural_xc_energy_and_grads_chunked(const gdft_basis *shells, const double *d_basis_rows, int32_t n_ao,
                                            const double *d_coords, const double *d_weights, int64_t n_grid,
                                            int64_t chunk, int32_t precision, const double *d_rdm1,
                                            const gdft_network *net, const double *d_params, const double *d_ehf,
                                            double *d_exc, double *d_vxc, double *d_dparams, void *d_ws,
                                            size_t ws_bytes, void *stream) {
  int rc = check_network(net);
  if (rc) return rc;
  if (d_params == nullptr || d_ehf == nullptr) {
    set_error("gdft_neural_xc_energy_and_grads_chunked: params and ehf (2, 2, grid) are required");
    return GDFT_ERR_INVALID;
  }
  if ((rc = check_aligned8(d_params, "params")) || (rc = check_aligned8(d_ehf, "ehf")) ||
      (d_dparams && (rc = check_aligned8(d_dparams, "dparams"))))
    return rc;
  return run_chunked("gdft_neural_xc_energy_and_grads_chunked", shells, d_basis_rows, n_ao, d_coords, d_weights,
                     n_grid, chunk, precision, d_rdm1, nullptr, net, d_params, d_ehf, 2, d_exc, d_vxc, d_dparams,
                     d_ws, ws_bytes, stream);
}

int gdft_chunked_status(void *d_ws, size_t ws_bytes, int32_t *status, void *stream) {
  return persistent_status("gdft_chunked_status", d_ws, ws_bytes, status, stream);
}

}  // extern "C"
