// Entry-point helpers shared between the C-ABI translation units.
#pragma once
#include "diffdvr_gb300.h"
#include "dvr_kernels.h"

namespace dvr {

// Supplies the scratch of one call; called with `device` current.  Returns
// nullptr on success, else an error message (reported as DVR_E_CUDA).
using ScratchSource = const char* (*)(int device, CallerScratch* out);

// dvr_render_adjoint's validation and error reporting, then the optimized
// adjoint on the scratch that `source` supplies (the kernel-family switch
// does not apply).  Returns a DVR_* status code.
int render_adjoint_into(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs_from_forward,
                        const DvrTensor* adj_color, const DvrAdjointOutputs* adj_outputs, void* cuda_stream,
                        ScratchSource source);

}  // namespace dvr
