// Placeholder launchers for the fast FP64 and mixed-precision kernels.
#include <cuda_runtime.h>

#include <vector>

#include "crs_internal.cuh"

namespace crs {

bool build_fast_tables(const std::vector<unsigned char> &, const ImgLayout &L,
                       std::vector<unsigned char> &extra, int, ImgLayout &out) {
  extra.clear();
  out = L;
  return true;
}

cudaError_t launch_wdot_fp64(const unsigned char *, const ImgLayout &,
                             const Batch &, int, int, cudaStream_t) {
  return cudaErrorNotSupported;
}

cudaError_t launch_wdot_mixed(const unsigned char *, const ImgLayout &,
                              const Batch &, int, int, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace crs
