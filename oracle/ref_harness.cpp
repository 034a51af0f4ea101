// Reference harness — TEST INFRASTRUCTURE ONLY.
//
// Exposes the reference's own CPU ray marcher (the DvrKernelForwardHost /
// DvrKernelAdjointHost templates of renderer/renderer_kernels.cuh:108-127 and
// :470-496) through the plain-C oracle interface of dvr_oracle.h.  It is
// compiled by oracle/Makefile straight from the reference's headers, with the
// declaration-only AD shim in oracle/ref_shim, into oracle/_ref/.  Nothing here
// is part of the product.
//
// The mode switch mirrors renderer/renderer_cpu.cpp:18-97 and :270-315; the
// accessors are built from raw pointers the way Renderer::checkInputs does
// (renderer/renderer.cpp:249-262).
#include <cuda_runtime.h>
#include "renderer_kernels.cuh"
#include "dvr_oracle.h"
#include "ref_image.h"

namespace {

template <typename Acc>
Acc make_acc(const OracleTensor& t) {
  using Ptr = typename Acc::PtrType;
  return Acc(static_cast<Ptr>(t.data), t.sizes, t.strides);
}

kernel::RendererInputs build_inputs(const OracleInputs* in) {
  kernel::RendererInputs r;
  r.screenSize = make_int2(in->width, in->height);
  r.volume = make_acc<kernel::Tensor4Read>(in->volume);
  r.volumeSize = make_int3(int(in->volume.sizes[1]), int(in->volume.sizes[2]), int(in->volume.sizes[3]));
  r.boxMin = make_acc<kernel::Tensor2Read>(in->box_min);
  r.boxSize = make_acc<kernel::Tensor2Read>(in->box_size);
  r.cameraRayStart = make_acc<kernel::Tensor4Read>(in->ray_start);
  r.cameraRayDir = make_acc<kernel::Tensor4Read>(in->ray_dir);
  r.cameraMatrix = make_acc<kernel::Tensor3Read>(in->camera_matrix);
  r.cameraFovYRadians = real_t(in->fov_y_radians);
  r.stepSize = make_acc<kernel::Tensor3Read>(in->step_size);
  r.tf = make_acc<kernel::Tensor3Read>(in->tf);
  r.blendingEarlyOut = real_t(in->blending_early_out);
  return r;
}

kernel::AdjointOutputs build_adjoint(const OracleAdjointOutputs* out) {
  kernel::AdjointOutputs o;
  if (out->has_volume) o.adj_volume = make_acc<kernel::BTensor4RW>(out->adj_volume);
  o.stepSizeHasBroadcasting = out->stepsize_broadcast != 0;
  if (out->has_stepsize) o.adj_stepSize = make_acc<kernel::BTensor3RW>(out->adj_stepsize);
  o.cameraHasBroadcasting = out->camera_broadcast != 0;
  if (out->has_camera) {
    o.adj_cameraRayStart = make_acc<kernel::BTensor4RW>(out->adj_ray_start);
    o.adj_cameraRayDir = make_acc<kernel::BTensor4RW>(out->adj_ray_dir);
  }
  if (out->has_tf) o.adj_tf = make_acc<kernel::BTensor3RW>(out->adj_tf);
  return o;
}

template <kernel::VolumeFilterMode F, kernel::CameraMode C, kernel::TFMode T, kernel::BlendMode B>
void fwd(dim3 vs, const kernel::RendererInputs& i, kernel::RendererOutputs& o) {
  kernel::DvrKernelForwardHost<F, C, T, B>(vs, i, o);
}

template <kernel::VolumeFilterMode F, kernel::CameraMode C, kernel::TFMode T, kernel::BlendMode B>
void adj(dim3 vs, const kernel::RendererInputs& i, const kernel::RendererOutputsAsInput& f,
         const kernel::AdjointColor_t& ac, const kernel::AdjointOutputs& o, int flags) {
  // flags: bit0 stepsize, bit1 camera, bit2 tf, bit3 volume
#define DVR_REF_ADJ(S, CA, TFD, V) \
  case (S) | ((CA) << 1) | ((TFD) << 2) | ((V) << 3): \
    kernel::DvrKernelAdjointHost<F, C, T, B, S, CA, TFD, V>(vs, i, f, ac, o); break;
  switch (flags) {
    DVR_REF_ADJ(0, 0, 0, 1) DVR_REF_ADJ(0, 0, 1, 0) DVR_REF_ADJ(0, 0, 1, 1)
    DVR_REF_ADJ(0, 1, 0, 0) DVR_REF_ADJ(0, 1, 0, 1) DVR_REF_ADJ(0, 1, 1, 0) DVR_REF_ADJ(0, 1, 1, 1)
    DVR_REF_ADJ(1, 0, 0, 0) DVR_REF_ADJ(1, 0, 0, 1) DVR_REF_ADJ(1, 0, 1, 0) DVR_REF_ADJ(1, 0, 1, 1)
    DVR_REF_ADJ(1, 1, 0, 0) DVR_REF_ADJ(1, 1, 0, 1) DVR_REF_ADJ(1, 1, 1, 0) DVR_REF_ADJ(1, 1, 1, 1)
    default: break;
  }
#undef DVR_REF_ADJ
}

// Dispatch over the 2 x 3 x 4 x 2 mode combinations, plus the pre-shaded
// filter/TF pair with its 3 x 2 camera and blend modes.
template <template <kernel::VolumeFilterMode, kernel::CameraMode, kernel::TFMode, kernel::BlendMode> class Fn,
          typename... Args>
int dispatch(int f, int c, int t, int b, Args&&... args) {
  using namespace kernel;
#define DVR_B(F_, C_, T_)                                                   \
  if (b == 0) { Fn<F_, C_, T_, BlendBeerLambert>::run(args...); return 0; } \
  if (b == 1) { Fn<F_, C_, T_, BlendAlpha>::run(args...); return 0; }       \
  return 2;
#define DVR_T(F_, C_)                                \
  switch (t) {                                       \
    case 0: { DVR_B(F_, C_, TFIdentity) }            \
    case 1: { DVR_B(F_, C_, TFTexture) }             \
    case 2: { DVR_B(F_, C_, TFLinear) }              \
    case 3: { DVR_B(F_, C_, TFGaussian) }            \
    default: return 2;                               \
  }
#define DVR_C(F_)                                      \
  switch (c) {                                         \
    case 0: { DVR_T(F_, CameraRayStartDir) }           \
    case 1: { DVR_T(F_, CameraInverseViewMatrix) }     \
    case 2: { DVR_T(F_, CameraReferenceFrame) }        \
    default: return 2;                                 \
  }
  if (f == 0) { DVR_C(FilterNearest) }
  if (f == 1) { DVR_C(FilterTrilinear) }
  if (f == 3 && t == 5) {
    // pre-shaded volume: the TF mode is pre-shaded too (renderer/renderer.cpp:72-74)
    switch (c) {
      case 0: { DVR_B(FilterPreshaded, CameraRayStartDir, TFPreshaded) }
      case 1: { DVR_B(FilterPreshaded, CameraInverseViewMatrix, TFPreshaded) }
      case 2: { DVR_B(FilterPreshaded, CameraReferenceFrame, TFPreshaded) }
      default: return 2;
    }
  }
  return 2;
#undef DVR_B
#undef DVR_T
#undef DVR_C
}

template <kernel::VolumeFilterMode F, kernel::CameraMode C, kernel::TFMode T, kernel::BlendMode B>
struct FwdFn {
  static void run(dim3 vs, const kernel::RendererInputs& i, kernel::RendererOutputs& o) { fwd<F, C, T, B>(vs, i, o); }
};
template <kernel::VolumeFilterMode F, kernel::CameraMode C, kernel::TFMode T, kernel::BlendMode B>
struct AdjFn {
  static void run(dim3 vs, const kernel::RendererInputs& i, const kernel::RendererOutputsAsInput& f,
                  const kernel::AdjointColor_t& ac, const kernel::AdjointOutputs& o, int flags) {
    adj<F, C, T, B>(vs, i, f, ac, o, flags);
  }
};

}  // namespace

extern "C" int oracle_real_size(void) { return int(sizeof(real_t)); }

extern "C" int oracle_forward(const OracleInputs* in, OracleTensor* color, OracleTensor* termination) {
  kernel::RendererInputs inputs = build_inputs(in);
  kernel::RendererOutputs outputs{make_acc<kernel::Tensor4RW>(*color), make_acc<kernel::ITensor3RW>(*termination)};
  dim3 vs(unsigned(in->width), unsigned(in->height), unsigned(in->batch));
  return dispatch<FwdFn>(in->filter_mode, in->camera_mode, in->tf_mode, in->blend_mode, vs, inputs, outputs);
}

extern "C" int oracle_adjoint(const OracleInputs* in, const OracleTensor* color, const OracleTensor* termination,
                              const OracleTensor* adj_color, OracleAdjointOutputs* out) {
  kernel::RendererInputs inputs = build_inputs(in);
  kernel::RendererOutputsAsInput fwd{make_acc<kernel::Tensor4Read>(*color),
                                     make_acc<kernel::ITensor3Read>(*termination)};
  kernel::AdjointColor_t ac = make_acc<kernel::AdjointColor_t>(*adj_color);
  kernel::AdjointOutputs o = build_adjoint(out);
  const int flags = (out->has_stepsize ? 1 : 0) | (out->has_camera ? 2 : 0) | (out->has_tf ? 4 : 0) |
                    (out->has_volume ? 8 : 0);
  if (flags == 0) return 3;
  dim3 vs(unsigned(in->width), unsigned(in->height), unsigned(in->batch));
  return dispatch<AdjFn>(in->filter_mode, in->camera_mode, in->tf_mode, in->blend_mode, vs, inputs, fwd, ac, o, flags);
}

// The parameter-block images of ref_image.h against the reference's own
// constructors: 0 when the constructors produce exactly what the images
// encode (so the GPU harness, which has no constructors, passes the
// reference's kernels the blocks its host code would), else the failing check.
extern "C" int oracle_ref_image_check(const OracleInputs* in, const OracleAdjointOutputs* out) {
  const kernel::RendererInputs by_ctor = build_inputs(in);
  if (!dvr_ref::inputs_match(by_ctor, *in)) return 1;
  alignas(kernel::RendererInputs) unsigned char ibuf[sizeof(kernel::RendererInputs)];
  auto* img = reinterpret_cast<kernel::RendererInputs*>(ibuf);
  dvr_ref::inputs_image(*in, img);
  if (!dvr_ref::inputs_match(*img, *in)) return 2;
  const kernel::AdjointOutputs o = build_adjoint(out);
  if (!dvr_ref::adjoint_match(o, *out)) return 3;
  alignas(kernel::AdjointOutputs) unsigned char obuf[sizeof(kernel::AdjointOutputs)];
  auto* oimg = reinterpret_cast<kernel::AdjointOutputs*>(obuf);
  dvr_ref::adjoint_image(*out, oimg);
  if (!dvr_ref::adjoint_match(*oimg, *out)) return 4;
  return 0;
}
