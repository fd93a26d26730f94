// conv_tc.cu -- tcgen05 tensor-core convolutions (placeholder until the
// kernels land): report the geometry as unsupported so the dispatcher runs
// the FP32 CUDA-core kernels.
#include "common.cuh"

namespace owlgpu {
int tc_conv_fwd(int, const ConvGeom &, const float *, const float *, float *, cudaStream_t) {
  return kErrUnsupported;
}
int tc_conv_bwd_input(int, const ConvGeom &, float *, const float *, const float *, cudaStream_t) {
  return kErrUnsupported;
}
int tc_conv_bwd_kernel(int, const ConvGeom &, const float *, float *, const float *, cudaStream_t) {
  return kErrUnsupported;
}
}  // namespace owlgpu
