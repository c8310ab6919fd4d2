// noalloc.cu - an allocation-free variant of gdft_integrate.
//
// Some callers cannot allocate device memory at the point where they need
// the XC energy: a JAX/XLA custom-call handler (the natural way grad_dft
// would bind this library) runs inside XLA's execution and must not allocate
// outside XLA's own allocator, and long-running services that reserve their
// whole device-memory budget at start-up have nothing left to hand out later.
// gdft_integrate_noalloc serves them: instead of a caller workspace it uses a
// fixed scratch array that lives in the library's own device image.
//
// The scratch holds one FP64 partial sum per 256 grid points (the per-block
// sums of integrate_kernel, reduced by energy_reduce_kernel), so it bounds
// the grid size at kNoAllocMaxBlocks * 256 points.  Every block writes its
// partial sum before the reduction reads it, so nothing has to start at zero.
#include <string.h>

#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace gdft {
namespace {

constexpr int kNoAllocMaxBlocks = 131072;  // 1 MiB of FP64 partial sums: grids up to 33,554,432 points
constexpr int kMaxDevices = 64;

// Device-resident scratch: every GPU that loads this library holds it until
// the process exits.  All calls on a device share it (and it keeps the last
// call's contents), so two calls that overlap on the GPU race on it.
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks];

std::mutex g_setup_mutex;
double *g_partials_addr[kMaxDevices] = {nullptr};

// Device address of the scratch on the current device.  In host code the
// array's name is only a host-side stand-in, so the address comes from
// cudaGetSymbolAddress, once per device, with that device current.  The
// address belongs to the device's primary context; a cudaDeviceReset ends it,
// which is why gdft.h rules out this entry after a reset.
int partials_on_current_device(double **out) {
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "integrate_noalloc: cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("integrate_noalloc: device ordinal %d is beyond the %d supported", dev, kMaxDevices);
    return GDFT_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_partials_addr[dev] == nullptr) {
    void *p = nullptr;
    rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_partials), "integrate_noalloc: cudaGetSymbolAddress");
    if (rc) return rc;
    g_partials_addr[dev] = (double *)p;
  }
  *out = g_partials_addr[dev];
  return GDFT_OK;
}

}  // namespace
}  // namespace gdft

using namespace gdft;

extern "C" int gdft_integrate_noalloc(int64_t n_grid, int32_t n_cols, const double *h_coeffs, int32_t n_coeffs,
                                      const double *d_dens, const double *d_weights, double clip, double *d_exc,
                                      void *stream) {
  if (n_grid <= 0 || n_cols < 1 || !(n_coeffs == 1 || n_coeffs == n_cols) || n_coeffs > GDFT_MAX_COLS ||
      h_coeffs == nullptr || d_dens == nullptr || d_weights == nullptr || d_exc == nullptr) {
    set_error("gdft_integrate_noalloc: invalid arguments (n_cols=%d, n_coeffs=%d)", n_cols, n_coeffs);
    return GDFT_ERR_INVALID;
  }
  // The size check comes before any block arithmetic, so no grid size can overflow it.
  if (n_grid > (int64_t)kNoAllocMaxBlocks * 256) {
    set_error("gdft_integrate_noalloc: n_grid=%lld exceeds the fixed scratch limit of %lld grid points; "
              "use gdft_integrate with a caller workspace",
              (long long)n_grid, (long long)kNoAllocMaxBlocks * 256);
    return GDFT_ERR_INVALID;
  }
  const int blocks = integrate_blocks(n_grid);
  double *partials = nullptr;
  int rc = partials_on_current_device(&partials);
  if (rc) return rc;
  gdft_functional fn;
  memset(&fn, 0, sizeof(fn));
  fn.n_cols = n_cols;
  fn.n_coeffs = n_coeffs;
  for (int i = 0; i < n_coeffs; ++i) fn.coeffs[i] = h_coeffs[i];
  fn.clip = clip;
  cudaStream_t st = (cudaStream_t)stream;
  rc = check_cuda(launch_integrate(n_grid, n_cols, fn, d_dens, d_weights, partials, st), "integrate_noalloc");
  if (rc) return rc;
  return check_cuda(launch_energy_reduce(partials, blocks, d_exc, st), "integrate_noalloc reduce");
}
