// Contraction of forward variables with an output adjoint
// (forwardVariablesToGradients, renderer/renderer_kernels.cuh:505-560).
#define DVR_FWDVARS_DEFINE
#include "dvr_fwdgrad.cuh"
#include "dvr_kernels.h"

namespace dvr {

cudaError_t launch_forward_variables_to_gradients(const FwdVarsParams& v, cudaStream_t s) {
  const int pixels = v.H * v.W;
  if (pixels == 0 || v.B == 0) return cudaSuccess;
  const dim3 grid((pixels + 255) / 256, v.B);
  const size_t smem = v.has_tf && v.R * v.C <= kFwdVarsSmemEntries ? size_t(v.R) * v.C * sizeof(float) : 0;
  forward_variables_to_gradients_kernel<<<grid, 256, smem, s>>>(v);
  return cudaGetLastError();
}

}  // namespace dvr
