// nu_ff.cu - the f-f integral class in a translation unit of its own (1,920
// unrolled Hermite products per primitive pair).
#include "nu_kernels.cuh"

namespace gdft {
namespace nu_detail {

cudaError_t launch_nu_ff(const ShellView &B, const int32_t *pairs, int lo, int hi, const double *pp, int64_t n_pp,
                         const double *boys_tab, const double *coords, int64_t p_begin, int64_t n_pts, NuOut out,
                         cudaStream_t st) {
  return launch_nu_class<3, 3>(B, pairs, lo, hi, pp, n_pp, boys_tab, coords, p_begin, n_pts, out, st);
}

}  // namespace nu_detail
}  // namespace gdft
