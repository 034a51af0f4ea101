// Contraction of forward variables with an output adjoint
// (forwardVariablesToGradients, renderer/renderer_kernels.cuh:505-560).
#define DVR_FWDVARS_DEFINE
#include <algorithm>
#include "dvr_fwdgrad.cuh"
#include "dvr_kernels.h"

namespace dvr {

cudaError_t launch_forward_variables_to_gradients(const FwdVarsParams& v, const LaunchInfo& li, cudaStream_t s) {
  const int pixels = v.H * v.W;
  if (pixels == 0 || v.B == 0) return cudaSuccess;
  constexpr int nw = kFwdVarsThreads / 32;
  const int E = v.has_tf ? v.R * v.C : 0;
  const size_t smem = E > 0 && E * (nw + 1) <= kFwdVarsSmemFloats ? size_t(E) * (nw + 1) * sizeof(float) : 0;
  // about four blocks per SM in total, fewer when the image is small
  const int per_b = std::max(1, std::min((pixels + nw - 1) / nw, (4 * li.num_sms + v.B - 1) / v.B));
  const dim3 grid(per_b, v.B);
  forward_variables_to_gradients_kernel<<<grid, kFwdVarsThreads, smem, s>>>(v);
  return cudaGetLastError();
}

}  // namespace dvr
