// Forward-mode derivatives: Gaussian transfer function, all volume storage types.
#define DVR_FWDGRAD_DEFINE
#include <algorithm>
#include "dvr_fwdgrad.cuh"
#include "dvr_kernels.h"

namespace dvr {
template cudaError_t launch_forward_gradients<3>(const RenderParams&, const FwdGradParams&, int, int,
                                                   const LaunchInfo&, cudaStream_t);
}  // namespace dvr
