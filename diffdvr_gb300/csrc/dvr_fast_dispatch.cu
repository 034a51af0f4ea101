// Dispatch of the optimized family on the volume storage type.
#include "dvr_fast_launch.cuh"

namespace dvr {

template <int TF>
cudaError_t launch_fast_forward(const RenderParams& p, int filter, int blend, const LaunchInfo& li, cudaStream_t s) {
  switch (p.vol_storage) {
    case kF16: return launch_fast_forward_vt<TF, __half>(p, filter, blend, li, s);
    case kBF16: return launch_fast_forward_vt<TF, __nv_bfloat16>(p, filter, blend, li, s);
    default: return launch_fast_forward_vt<TF, float>(p, filter, blend, li, s);
  }
}

template <int TF>
cudaError_t launch_fast_adjoint(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                const LaunchInfo& li, cudaStream_t s) {
  switch (p.vol_storage) {
    case kF16: return launch_fast_adjoint_vt<TF, __half>(p, a, filter, blend, li, s);
    case kBF16: return launch_fast_adjoint_vt<TF, __nv_bfloat16>(p, a, filter, blend, li, s);
    default: return launch_fast_adjoint_vt<TF, float>(p, a, filter, blend, li, s);
  }
}

template <int TF>
cudaError_t launch_fast_adjoint_into(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                     const LaunchInfo& li, const CallerScratch& sc, cudaStream_t s) {
  switch (p.vol_storage) {
    case kF16: return launch_fast_adjoint_into_vt<TF, __half>(p, a, filter, blend, li, sc, s);
    case kBF16: return launch_fast_adjoint_into_vt<TF, __nv_bfloat16>(p, a, filter, blend, li, sc, s);
    default: return launch_fast_adjoint_into_vt<TF, float>(p, a, filter, blend, li, sc, s);
  }
}

#define DVR_DISPATCH(TF)                                                                                      \
  template cudaError_t launch_fast_forward<TF>(const RenderParams&, int, int, const LaunchInfo&, cudaStream_t); \
  template cudaError_t launch_fast_adjoint<TF>(const RenderParams&, const AdjointParams&, int, int,           \
                                               const LaunchInfo&, cudaStream_t);          \
  template cudaError_t launch_fast_adjoint_into<TF>(const RenderParams&, const AdjointParams&, int, int,      \
                                                    const LaunchInfo&, const CallerScratch&, cudaStream_t);
DVR_DISPATCH(0)
DVR_DISPATCH(1)
DVR_DISPATCH(2)
DVR_DISPATCH(3)

}  // namespace dvr
