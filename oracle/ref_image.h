// Byte images of the reference's kernel parameter blocks — TEST INFRASTRUCTURE ONLY.
//
// The reference passes its parameter blocks (kernel::RendererInputs,
// RendererOutputs, RendererOutputsAsInput, AdjointOutputs of
// renderer/renderer_settings.cuh:150-244) to its CUDA kernels by value.
// Their tensor members are GenericPackedTensorAccessor objects
// (renderer/renderer_tensor.cuh:120-272) whose constructors exist on the host
// only, and only where the reference headers are compiled.  The functions
// here fill the same objects from the plain-C OracleTensor / OracleInputs
// structs of dvr_oracle.h without those constructors: an accessor is a data
// pointer followed by its N sizes and N strides (index_t = int32), and a
// broadcasting accessor stores stride 0 for a dimension of size 1
// (renderer/renderer_tensor.cuh:140-144).  They run on the host (where
// oracle_ref_image_check in ref_harness.cpp compares every field with the
// reference's constructors) and on the device (ref_device.cu, which builds
// the parameter blocks for the reference's kernels on the GPU).
#pragma once
#include <string.h>
#include "dvr_oracle.h"

namespace dvr_ref {

template <typename Acc>
struct AccShape;
template <typename T, size_t N, template <typename U> class PT, typename I, bool BC>
struct AccShape<kernel::GenericPackedTensorAccessor<T, N, PT, I, BC>> {
  static constexpr size_t dims = N;
  using index_t = I;
  static constexpr bool broadcast = BC;
};

template <size_t N, typename I>
struct AccImage {
  void* data;
  I sizes[N];
  I strides[N];
};

// expected (size, stride) of dimension i of accessor type Acc built from t
template <typename Acc>
__host__ __device__ inline void acc_dim(const OracleTensor& t, size_t i, int64_t& size, int64_t& stride) {
  using I = typename AccShape<Acc>::index_t;
  size = I(t.sizes[i]);
  stride = (AccShape<Acc>::broadcast && t.sizes[i] == 1) ? 0 : I(t.strides[i]);
}

template <typename Acc>
__host__ __device__ inline void put_acc(Acc* dst, const OracleTensor& t) {
  using S = AccShape<Acc>;
  AccImage<S::dims, typename S::index_t> img;
  static_assert(sizeof(img) == sizeof(Acc), "accessor layout: pointer + N sizes + N strides");
  static_assert(alignof(AccImage<S::dims, typename S::index_t>) == alignof(Acc), "accessor alignment");
  img.data = t.data;
  for (size_t i = 0; i < S::dims; ++i) {
    int64_t s, st;
    acc_dim<Acc>(t, i, s, st);
    img.sizes[i] = typename S::index_t(s);
    img.strides[i] = typename S::index_t(st);
  }
  memcpy(static_cast<void*>(dst), &img, sizeof img);
}

// 1 if accessor a, read through its own getters, holds what put_acc wrote for t
template <typename Acc>
__host__ __device__ inline int acc_matches(const Acc& a, const OracleTensor& t) {
  if (static_cast<const void*>(a.data()) != t.data) return 0;
  for (size_t i = 0; i < AccShape<Acc>::dims; ++i) {
    int64_t s, st;
    acc_dim<Acc>(t, i, s, st);
    if (int64_t(a.size(int(i))) != s || int64_t(a.stride(int(i))) != st) return 0;
  }
  return 1;
}

// The members the reference's host code sets (renderer/renderer.cpp:249-262;
// the same set as build_inputs in ref_harness.cpp).  *r is raw storage.
__host__ __device__ inline void inputs_image(const OracleInputs& in, kernel::RendererInputs* r) {
  memset(static_cast<void*>(r), 0, sizeof(*r));
  r->screenSize = make_int2(in.width, in.height);
  put_acc(&r->volume, in.volume);
  r->volumeSize = make_int3(int(in.volume.sizes[1]), int(in.volume.sizes[2]), int(in.volume.sizes[3]));
  put_acc(&r->boxMin, in.box_min);
  put_acc(&r->boxSize, in.box_size);
  put_acc(&r->cameraRayStart, in.ray_start);
  put_acc(&r->cameraRayDir, in.ray_dir);
  put_acc(&r->cameraMatrix, in.camera_matrix);
  r->cameraFovYRadians = real_t(in.fov_y_radians);
  put_acc(&r->stepSize, in.step_size);
  put_acc(&r->tf, in.tf);
  r->blendingEarlyOut = real_t(in.blending_early_out);
}

__host__ __device__ inline int inputs_match(const kernel::RendererInputs& r, const OracleInputs& in) {
  return r.screenSize.x == in.width && r.screenSize.y == in.height && acc_matches(r.volume, in.volume) &&
         r.volumeSize.x == int(in.volume.sizes[1]) && r.volumeSize.y == int(in.volume.sizes[2]) &&
         r.volumeSize.z == int(in.volume.sizes[3]) && acc_matches(r.boxMin, in.box_min) &&
         acc_matches(r.boxSize, in.box_size) && acc_matches(r.cameraRayStart, in.ray_start) &&
         acc_matches(r.cameraRayDir, in.ray_dir) && acc_matches(r.cameraMatrix, in.camera_matrix) &&
         r.cameraFovYRadians == real_t(in.fov_y_radians) && acc_matches(r.stepSize, in.step_size) &&
         acc_matches(r.tf, in.tf) && r.blendingEarlyOut == real_t(in.blending_early_out);
}

// AdjointOutputs as oracle_adjoint in ref_harness.cpp sets it; *o is raw storage
__host__ __device__ inline void adjoint_image(const OracleAdjointOutputs& a, kernel::AdjointOutputs* o) {
  memset(static_cast<void*>(o), 0, sizeof(*o));
  if (a.has_volume) put_acc(&o->adj_volume, a.adj_volume);
  o->stepSizeHasBroadcasting = a.stepsize_broadcast != 0;
  if (a.has_stepsize) put_acc(&o->adj_stepSize, a.adj_stepsize);
  o->cameraHasBroadcasting = a.camera_broadcast != 0;
  if (a.has_camera) {
    put_acc(&o->adj_cameraRayStart, a.adj_ray_start);
    put_acc(&o->adj_cameraRayDir, a.adj_ray_dir);
  }
  if (a.has_tf) put_acc(&o->adj_tf, a.adj_tf);
}

__host__ __device__ inline int adjoint_match(const kernel::AdjointOutputs& o, const OracleAdjointOutputs& a) {
  return (!a.has_volume || acc_matches(o.adj_volume, a.adj_volume)) &&
         o.stepSizeHasBroadcasting == (a.stepsize_broadcast != 0) &&
         (!a.has_stepsize || acc_matches(o.adj_stepSize, a.adj_stepsize)) &&
         o.cameraHasBroadcasting == (a.camera_broadcast != 0) &&
         (!a.has_camera || (acc_matches(o.adj_cameraRayStart, a.adj_ray_start) &&
                            acc_matches(o.adj_cameraRayDir, a.adj_ray_dir))) &&
         (!a.has_tf || acc_matches(o.adj_tf, a.adj_tf));
}

}  // namespace dvr_ref
