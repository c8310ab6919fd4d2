// nu_f.cu - the integral classes with an f shell, compiled apart from nu.cu (their
// fully unrolled products dominate the build; f-d and f-f have units of their own,
// nu_fd.cu and nu_ff.cu).
#include "nu_kernels.cuh"

namespace gdft {
namespace nu_detail {

cudaError_t launch_nu_f_class(int la, int lb, const ShellView &B, const int32_t *pairs, int lo, int hi,
                              const double *pp, int64_t n_pp, const double *boys_tab, const double *coords,
                              int64_t p_begin, int64_t n_pts, NuOut out, cudaStream_t st) {
  if (la != 3) return cudaErrorInvalidValue;
  switch (lb) {
    case 0: return launch_nu_class<3, 0>(B, pairs, lo, hi, pp, n_pp, boys_tab, coords, p_begin, n_pts, out, st);
    case 1: return launch_nu_class<3, 1>(B, pairs, lo, hi, pp, n_pp, boys_tab, coords, p_begin, n_pts, out, st);
    case 2: return launch_nu_fd(B, pairs, lo, hi, pp, n_pp, boys_tab, coords, p_begin, n_pts, out, st);
    case 3: return launch_nu_ff(B, pairs, lo, hi, pp, n_pp, boys_tab, coords, p_begin, n_pts, out, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace nu_detail
}  // namespace gdft
