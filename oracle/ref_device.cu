// The reference's own CUDA ray marcher as a cubin — TEST INFRASTRUCTURE ONLY.
//
// Compiled by oracle/Makefile (target `ref`) from the reference's headers in
// place, with the declaration-only AD stand-in of ref_shim/ and the options
// the reference's runtime compiler uses (renderer/kernel_loader.cpp:218-230:
// C++17, fast math, line info), into oracle/_ref/.  oracle/ref_cuda.py loads
// it with the CUDA driver API and launches it as the reference's CUDA backend
// does (renderer/renderer_cuda.cpp:85-118, :251-317).
//
// * ref_fwd_<filter>_<camera>_<tf>_<blend>: the reference's forward kernel,
//   DvrKernelForwardDevice (renderer/renderer_kernels.cuh:92-106): its own
//   grid-stride loop KERNEL_3D_LOOP over its own per-pixel function
//   DvrKernelForwardImpl.
// * ref_adj_<filter>_<camera>_<tf>_<blend>_<S><C><T><D><V>: the adjoint
//   kernel DvrKernelAdjointDevice (:446-468) with the derivative switches
//   step size, camera, TF, delayed TF accumulation, volume.
// * ref_build_params: fills the parameter blocks those kernels take by value
//   from the plain-C structs of dvr_oracle.h (ref_image.h; the reference
//   builds them with host-only constructors) and reads them back through the
//   accessors' own getters, so the host can check them before any launch.
//
// Nothing here is part of the product.
#include <cuda_runtime.h>
#include "renderer_kernels.cuh"
#include "dvr_oracle.h"
#include "ref_image.h"

namespace {
// one slot per parameter block in ref_build_params' output buffer
constexpr int kSlot = 1024;
static_assert(sizeof(kernel::RendererInputs) <= kSlot, "slot size");
static_assert(sizeof(kernel::RendererOutputs) <= kSlot, "slot size");
static_assert(sizeof(kernel::RendererOutputsAsInput) <= kSlot, "slot size");
static_assert(sizeof(kernel::AdjointColor_t) <= kSlot, "slot size");
static_assert(sizeof(kernel::AdjointOutputs) <= kSlot, "slot size");
}  // namespace

// blobs: 5 slots of kSlot bytes (inputs, outputs, outputs as input, adjoint
// colour, adjoint outputs).  info[0..4]: the five block sizes; info[5]: 1 if
// every block reads back as intended; info[6]: sizeof(real_t).
extern "C" __global__ void ref_build_params(const OracleInputs in, const OracleTensor color,
                                            const OracleTensor term, const OracleTensor adj_color,
                                            const OracleAdjointOutputs adj, unsigned char* blobs,
                                            long long* info) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  auto* ri = reinterpret_cast<kernel::RendererInputs*>(blobs);
  auto* ro = reinterpret_cast<kernel::RendererOutputs*>(blobs + kSlot);
  auto* rf = reinterpret_cast<kernel::RendererOutputsAsInput*>(blobs + 2 * kSlot);
  auto* ac = reinterpret_cast<kernel::AdjointColor_t*>(blobs + 3 * kSlot);
  auto* ao = reinterpret_cast<kernel::AdjointOutputs*>(blobs + 4 * kSlot);
  dvr_ref::inputs_image(in, ri);
  memset(static_cast<void*>(ro), 0, sizeof(*ro));
  dvr_ref::put_acc(&ro->color, color);
  dvr_ref::put_acc(&ro->terminationIndex, term);
  memset(static_cast<void*>(rf), 0, sizeof(*rf));
  dvr_ref::put_acc(&rf->color, color);
  dvr_ref::put_acc(&rf->terminationIndex, term);
  memset(static_cast<void*>(ac), 0, sizeof(*ac));
  if (adj_color.data) dvr_ref::put_acc(ac, adj_color);
  dvr_ref::adjoint_image(adj, ao);
  info[0] = sizeof(kernel::RendererInputs);
  info[1] = sizeof(kernel::RendererOutputs);
  info[2] = sizeof(kernel::RendererOutputsAsInput);
  info[3] = sizeof(kernel::AdjointColor_t);
  info[4] = sizeof(kernel::AdjointOutputs);
  info[5] = dvr_ref::inputs_match(*ri, in) && dvr_ref::acc_matches(ro->color, color) &&
            dvr_ref::acc_matches(ro->terminationIndex, term) && dvr_ref::acc_matches(rf->color, color) &&
            dvr_ref::acc_matches(rf->terminationIndex, term) &&
            (!adj_color.data || dvr_ref::acc_matches(*ac, adj_color)) && dvr_ref::adjoint_match(*ao, adj);
  info[6] = sizeof(real_t);
}

#define DVR_REF_FWD(F, C, T, B)                                                                            \
  extern "C" __global__ void ref_fwd_##F##_##C##_##T##_##B(dim3 virtual_size, kernel::RendererInputs inputs, \
                                                           kernel::RendererOutputs outputs) {              \
    KERNEL_3D_LOOP(x, y, b, virtual_size) {                                                                \
      kernel::DvrKernelForwardImpl<kernel::F, kernel::C, kernel::T, kernel::B>(x, y, b, inputs, outputs);  \
    }                                                                                                      \
    KERNEL_3D_LOOP_END                                                                                     \
  }

// (one more macro level so that the flag arguments are expanded before they are pasted)
#define DVR_REF_ADJ(F, C, T, B, S, CA, TFD, DL, V) DVR_REF_ADJ_(F, C, T, B, S, CA, TFD, DL, V)
#define DVR_REF_ADJ_(F, C, T, B, S, CA, TFD, DL, V)                                                         \
  extern "C" __global__ void ref_adj_##F##_##C##_##T##_##B##_##S##CA##TFD##DL##V(                          \
      dim3 virtual_size, kernel::RendererInputs inputs, kernel::RendererOutputsAsInput outputsFromForward,  \
      kernel::AdjointColor_t adj_color, kernel::AdjointOutputs adj_outputs) {                              \
    KERNEL_3D_LOOP(x, y, b, virtual_size) {                                                                \
      kernel::DvrKernelAdjointImpl<kernel::F, kernel::C, kernel::T, kernel::B, S, CA, TFD, DL, V>(         \
          x, y, b, inputs, outputsFromForward, adj_color, adj_outputs);                                    \
    }                                                                                                      \
    KERNEL_3D_LOOP_END                                                                                     \
  }

// Forward: every filter x camera x TF x blend combination.  Adjoint: step
// size, TF and volume derivatives (plus camera derivatives for per-pixel
// rays, the only camera mode whose rays have gradients) with immediate TF
// atomics; for the TF-reconstruction modes also the TF-only kernel.
#define DVR_REF_MODE(F, C, T, B) DVR_REF_FWD(F, C, T, B)
#define DVR_REF_BLENDS(F, C, T)                 \
  DVR_REF_MODE(F, C, T, BlendBeerLambert)       \
  DVR_REF_MODE(F, C, T, BlendAlpha)             \
  DVR_REF_ADJ(F, C, T, BlendBeerLambert, 1, DVR_REF_CAM_##C, 1, 0, 1) \
  DVR_REF_ADJ(F, C, T, BlendAlpha, 1, DVR_REF_CAM_##C, 1, 0, 1)
#define DVR_REF_CAM_CameraRayStartDir 1
#define DVR_REF_CAM_CameraInverseViewMatrix 0
#define DVR_REF_CAM_CameraReferenceFrame 0
#define DVR_REF_TFS(F, C)                       \
  DVR_REF_BLENDS(F, C, TFIdentity)              \
  DVR_REF_BLENDS(F, C, TFTexture)               \
  DVR_REF_BLENDS(F, C, TFLinear)                \
  DVR_REF_BLENDS(F, C, TFGaussian)
#define DVR_REF_CAMS(F)                         \
  DVR_REF_TFS(F, CameraRayStartDir)             \
  DVR_REF_TFS(F, CameraInverseViewMatrix)       \
  DVR_REF_TFS(F, CameraReferenceFrame)

DVR_REF_CAMS(FilterNearest)
DVR_REF_CAMS(FilterTrilinear)

DVR_REF_ADJ(FilterTrilinear, CameraRayStartDir, TFTexture, BlendBeerLambert, 0, 0, 1, 0, 0)

// The adjoints that time the reference's CUDA path on the other workloads
// (oracle/ref_cuda.py, TIMED_ADJOINTS), each with exactly the derivatives its
// workload asks for: the volume only (identity TF, absorption
// reconstruction); rays, TF and volume (linear TF, large mixed
// configuration); TF and volume (linear TF, the small CPU-sized
// configuration).
//
// No kernel here uses the reference's delayed TF accumulation (its
// per-thread shared-memory TF gradient, the default of
// pytests/diffdvr/renderer.py:270): its warp reduction
// (renderer/cooperative_groups.cuh:161-212) passes the shuffle's value where
// the member mask belongs (:206) whenever the active threads of a warp are
// not a power of two in number, and kernels built with it raised "an
// illegal instruction was encountered" on the GB300.
DVR_REF_ADJ(FilterTrilinear, CameraRayStartDir, TFIdentity, BlendBeerLambert, 0, 0, 0, 0, 1)
DVR_REF_ADJ(FilterTrilinear, CameraRayStartDir, TFLinear, BlendBeerLambert, 0, 1, 1, 0, 1)
DVR_REF_ADJ(FilterTrilinear, CameraRayStartDir, TFLinear, BlendBeerLambert, 0, 0, 1, 0, 1)
