// Batched rendering of uneven instances in one launch (dvr_batch.cu).
#pragma once
#include <cuda_runtime.h>
#include "dvr_kernels.h"

namespace dvr {

// shapes: the tile shape (DvrTileShape) of each instance
cudaError_t launch_batched_forward(const RenderParams* instances, const unsigned char* shapes, int n, int filter,
                                   int tf_mode, int blend, int device, const LaunchInfo& li, cudaStream_t s);
cudaError_t launch_batched_adjoint(const RenderParams* instances, const AdjointParams* adjoints,
                                   const unsigned char* shapes, int n, int filter, int tf_mode, int blend, int device,
                                   const LaunchInfo& li, cudaStream_t s);

}  // namespace dvr
