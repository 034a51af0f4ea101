// Host layer of the C ABI: validates the descriptors the way the reference's
// renderer::Renderer does (renderer/renderer.cpp:49-391 checkInputs /
// checkOutput / checkAdjointOutput, renderer/renderer.cpp:660-742 for the
// adjoint), flattens them into kernel parameter blocks and dispatches to the
// kernel families.  C++ internally, plain C at the boundary: nothing throws
// across it.
#include "diffdvr_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "dvr_kernels.h"
#include "dvr_batch.h"
#include "dvr_entry.h"

namespace dvr {
namespace {

thread_local std::string g_last_error;
std::atomic<int> g_family{DVR_KERNELS_OPTIMIZED};
std::atomic<int> g_window{0};
std::atomic<int> g_gather{DVR_GATHER_AUTO};
thread_local int g_adjoint_path = DVR_PATH_NONE;
std::atomic<int> g_sync{0};

struct DvrError : std::runtime_error {
  int code;
  DvrError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const std::string& msg) { throw DvrError(code, msg); }

std::string shape_str(const DvrTensor& t) {
  std::ostringstream os;
  os << "[";
  for (int i = 0; i < t.ndim; ++i) os << (i ? ", " : "") << t.sizes[i];
  os << "]";
  return os.str();
}

const char* dtype_name(int d) {
  switch (d) {
    case DVR_FLOAT32: return "float32";
    case DVR_FLOAT64: return "float64";
    case DVR_FLOAT16: return "float16";
    case DVR_BFLOAT16: return "bfloat16";
    case DVR_INT32: return "int32";
    default: return "unknown";
  }
}

// ---- the reference's CHECK_* macros (renderer/pytorch_utils.h:5-20) ----
void check_dim(const DvrTensor& t, const char* name, int d) {
  if (t.ndim < 0) fail(DVR_E_INVALID_ARGUMENT, std::string(name) + " is not defined!");
  if (t.ndim != d) {
    std::ostringstream os;
    os << name << " must be a tensor with " << d << " dimensions, but has shape " << shape_str(t);
    fail(DVR_E_INVALID_ARGUMENT, os.str());
  }
}
void check_size(const DvrTensor& t, const char* name, int d, int64_t s) {
  if (t.sizes[d] != s) {
    std::ostringstream os;
    os << name << " must have " << s << " entries at dimension " << d << ", but has " << t.sizes[d] << " entries";
    fail(DVR_E_INVALID_ARGUMENT, os.str());
  }
}
void check_dtype(const DvrTensor& t, const char* name, int dtype) {
  if (t.dtype != dtype) {
    std::ostringstream os;
    os << name << " must be of type " << dtype_name(dtype) << ", but is " << dtype_name(t.dtype);
    fail(DVR_E_INVALID_ARGUMENT, os.str());
  }
}
void check_device(const DvrTensor& t, const char* name, int device_index) {
  if (t.device_type != DVR_DEVICE_CUDA) {
    fail(DVR_E_INVALID_ARGUMENT, std::string(name) +
                                     " is a CPU tensor: diffdvr_gb300 renders on CUDA devices only, and all "
                                     "tensors must be on the same device");
  }
  if (t.device_index != device_index) {
    std::ostringstream os;
    os << "All tensors must be on the same device, but " << name << " is on cuda:" << t.device_index
       << " instead of cuda:" << device_index;
    fail(DVR_E_INVALID_ARGUMENT, os.str());
  }
}
int check_batch(const DvrTensor& t, const char* name, int B1, int batch_index = 0) {
  const int B2 = int(t.sizes[batch_index]);
  if (B2 == 1) return B1;
  if (B1 == 1) return B2;
  if (B1 != B2) {
    std::ostringstream os;
    os << name << " must be have the same batch size as other tensors, if batch>1. actual=" << B2
       << ", expected=" << B1;
    fail(DVR_E_INVALID_ARGUMENT, os.str());
  }
  return B1;
}

// broadcast-aware view: a dimension of size 1 gets stride 0
InView in_view(const DvrTensor& t) {
  InView v{};
  v.p = t.data;
  for (int i = 0; i < 4 && i < t.ndim; ++i) v.s[i] = t.sizes[i] == 1 ? 0 : t.strides[i];
  return v;
}
OutView out_view(const DvrTensor& t, bool broadcast) {
  OutView v{};
  v.p = t.data;
  for (int i = 0; i < 4 && i < t.ndim; ++i) v.s[i] = (broadcast && t.sizes[i] == 1) ? 0 : t.strides[i];
  return v;
}

struct DeviceInfo {
  bool valid = false;
  LaunchInfo li{};
};
std::mutex g_dev_mutex;
DeviceInfo g_dev[64];

LaunchInfo launch_info(int device) {
  std::lock_guard<std::mutex> lock(g_dev_mutex);
  if (device < 0 || device >= 64) fail(DVR_E_INVALID_ARGUMENT, "device index out of range");
  DeviceInfo& d = g_dev[device];
  if (!d.valid) {
    int sms = 0, smem = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) {
      cudaGetLastError();
      fail(DVR_E_CUDA, "cannot query CUDA device " + std::to_string(device));
    }
    d.li.num_sms = sms;
    d.li.max_smem_optin = smem;
    d.li.device = device;
    d.valid = true;
  }
  return d.li;
}

// Restores the caller's current device on scope exit.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int device) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      fail(DVR_E_CUDA, "no CUDA device available");
    }
    if (prev != device && cudaSetDevice(device) != cudaSuccess) {
      cudaGetLastError();
      fail(DVR_E_CUDA, "cannot select CUDA device " + std::to_string(device));
    }
  }
  ~DeviceGuard() {
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != prev && prev >= 0) cudaSetDevice(prev);
  }
};

// Resolved inputs of one render call.
struct Checked {
  RenderParams p{};
  int filter = 1, tf_mode = 1, blend = 0;
  int device = 0;
};

bool real_storage_ok(int dtype) { return dtype == DVR_FLOAT32 || dtype == DVR_FLOAT16 || dtype == DVR_BFLOAT16; }

// renderer::Renderer::checkInputs (renderer/renderer.cpp:49-263)
Checked check_inputs(const DvrRendererInputs& in) {
  Checked c;
  RenderParams& p = c.p;
  p.W = in.screen_width;
  p.H = in.screen_height;
  if (p.W < 0 || p.H < 0) fail(DVR_E_INVALID_ARGUMENT, "screen size must be non-negative");

  const DvrTensor& volume = in.volume;
  check_dim(volume, "volume", 4);
  c.device = volume.device_index;
  check_device(volume, "volume", c.device);
  if (!real_storage_ok(volume.dtype))
    fail(DVR_E_INVALID_ARGUMENT, std::string("volume must be of type float32 (or float16/bfloat16), but is ") +
                                     dtype_name(volume.dtype));
  int B = int(volume.sizes[0]);
  p.X = int(volume.sizes[1]);
  p.Y = int(volume.sizes[2]);
  p.Z = int(volume.sizes[3]);
  if (in.volume_filter_mode != DVR_FILTER_NEAREST && in.volume_filter_mode != DVR_FILTER_TRILINEAR &&
      in.volume_filter_mode != DVR_FILTER_PRESHADED)
    fail(DVR_E_INVALID_ARGUMENT, "unknown volume filter enum value");
  // renderer/renderer.cpp:72-80
  if ((in.volume_filter_mode == DVR_FILTER_PRESHADED) != (in.tf_mode == DVR_TF_PRESHADED))
    fail(DVR_E_INVALID_ARGUMENT, "if pre-shading is selected, both the filter mode and TF mode must be set to preshaded");
  if (in.volume_filter_mode == DVR_FILTER_PRESHADED) {
    if (volume.sizes[0] != 4)
      fail(DVR_E_INVALID_ARGUMENT,
           "In pre-shaded mode, the volume colors are encoded in the batch dimension of the volume. It must be 4, "
           "but is " + std::to_string(volume.sizes[0]));
    B = 1;
  }
  if (p.X < 1 || p.Y < 1 || p.Z < 1) fail(DVR_E_INVALID_ARGUMENT, "volume must have at least one voxel per axis");
  {
    // offsets inside one batch entry are 32-bit, as the reference's accessors
    const double span = double(p.X - 1) * std::fabs(double(volume.strides[1])) +
                        double(p.Y - 1) * std::fabs(double(volume.strides[2])) +
                        double(p.Z - 1) * std::fabs(double(volume.strides[3]));
    if (span >= 2147483647.0) fail(DVR_E_INVALID_ARGUMENT, "volume is too large: one batch entry must hold < 2^31 elements");
  }
  p.vol_storage = volume.dtype;
  p.volume = in_view(volume);
  c.filter = in.volume_filter_mode;

  auto vec3_input = [&](int kind, const DvrTensor& t, const double* val, const char* name, InView& out) {
    if (kind == DVR_KIND_TENSOR) {
      check_dim(t, name, 2);
      check_device(t, name, c.device);
      check_size(t, name, 1, 3);
      B = check_batch(t, name, B);
      check_dtype(t, name, DVR_FLOAT32);
      out = in_view(t);
    } else if (kind == DVR_KIND_VALUE) {
      out = InView{};
      out.p = nullptr;
      for (int i = 0; i < 3; ++i) out.val[i] = float(val[i]);
    } else {
      fail(DVR_E_INVALID_ARGUMENT, std::string("unknown kind for ") + name);
    }
  };
  vec3_input(in.box_min_kind, in.box_min, in.box_min_value, "boxMin", p.box_min);
  vec3_input(in.box_size_kind, in.box_size, in.box_size_value, "boxSize", p.box_size);

  p.camera_mode = in.camera_mode;
  switch (in.camera_mode) {
    case DVR_CAMERA_RAY_START_DIR: {
      if (in.camera_kind != DVR_CAMERA_PER_PIXEL_RAYS)
        fail(DVR_E_INVALID_ARGUMENT,
             "'CameraRayStartDir' specified in 'cameraMode', but 'camera' does not hold the first variant "
             "'CameraPerPixelRays'");
      const DvrTensor& rs = in.camera_ray_start;
      const DvrTensor& rd = in.camera_ray_dir;
      check_dim(rs, "cameraRayStart", 4);
      check_device(rs, "cameraRayStart", c.device);
      check_size(rs, "cameraRayStart", 1, p.H);
      check_size(rs, "cameraRayStart", 2, p.W);
      check_size(rs, "cameraRayStart", 3, 3);
      B = check_batch(rs, "cameraRayStart", B);
      check_dtype(rs, "cameraRayStart", DVR_FLOAT32);
      check_dim(rd, "cameraRayDir", 4);
      check_device(rd, "cameraRayDir", c.device);
      check_size(rd, "cameraRayDir", 1, p.H);
      check_size(rd, "cameraRayDir", 2, p.W);
      check_size(rd, "cameraRayDir", 3, 3);
      B = check_batch(rd, "cameraRayDir", B);
      check_dtype(rd, "cameraRayDir", DVR_FLOAT32);
      p.ray_start = in_view(rs);
      p.ray_dir = in_view(rd);
    } break;
    case DVR_CAMERA_INVERSE_VIEW_MATRIX: {
      if (in.camera_kind == DVR_CAMERA_INVERSE_VIEW_TENSOR) {
        const DvrTensor& m = in.camera_matrix;
        check_dim(m, "cameraMatrix", 3);
        check_device(m, "cameraMatrix", c.device);
        check_size(m, "cameraMatrix", 1, 4);
        check_size(m, "cameraMatrix", 2, 4);
        B = check_batch(m, "cameraMatrix", B);
        check_dtype(m, "cameraMatrix", DVR_FLOAT32);
        p.cam = in_view(m);
      } else if (in.camera_kind == DVR_CAMERA_INVERSE_VIEW_VALUE) {
        p.cam = InView{};
        for (int i = 0; i < 16; ++i) p.cam_value[i] = in.camera_matrix_value[i];
      } else {
        fail(DVR_E_INVALID_ARGUMENT,
             "'CameraInverseViewMatrix' specified in 'cameraMode', but 'camera' holds neither a B*4*4 tensor nor "
             "a mat4");
      }
    } break;
    case DVR_CAMERA_REFERENCE_FRAME: {
      if (in.camera_kind != DVR_CAMERA_REFERENCE_FRAME_KIND)
        fail(DVR_E_INVALID_ARGUMENT,
             "'CameraReferenceFrame' specified in 'cameraMode', but 'camera' does not hold the fourth variant "
             "'CameraReferenceFrame'");
      const DvrTensor& m = in.camera_matrix;
      check_dim(m, "cameraMatrix", 3);
      check_device(m, "cameraMatrix", c.device);
      check_size(m, "cameraMatrix", 1, 3);
      check_size(m, "cameraMatrix", 2, 3);
      B = check_batch(m, "cameraMatrix", B);
      check_dtype(m, "cameraMatrix", DVR_FLOAT32);
      p.cam = in_view(m);
      p.fov_y = float(in.camera_fov_y_radians);
    } break;
    default:
      fail(DVR_E_INVALID_ARGUMENT, "unknown camera enum value");
  }

  if (in.step_size_kind == DVR_KIND_TENSOR) {
    const DvrTensor& s = in.step_size;
    check_dim(s, "stepSize", 3);
    check_device(s, "stepSize", c.device);
    B = check_batch(s, "stepSize", B);
    check_batch(s, "stepSize-Height", p.H, 1);
    check_batch(s, "stepSize-Width", p.W, 2);
    check_dtype(s, "stepSize", DVR_FLOAT32);
    p.step = in_view(s);
  } else if (in.step_size_kind == DVR_KIND_VALUE) {
    p.step = InView{};
    p.step.val[0] = float(in.step_size_value);
  } else {
    fail(DVR_E_INVALID_ARGUMENT, "unknown kind for stepSize");
  }

  const DvrTensor& tf = in.tf;
  check_dim(tf, "tf", 3);
  check_device(tf, "tf", c.device);
  B = check_batch(tf, "tf", B);
  switch (in.tf_mode) {
    case DVR_TF_IDENTITY:
      check_size(tf, "tf", 1, 1);
      check_size(tf, "tf", 2, 2);
      break;
    case DVR_TF_TEXTURE:
      check_size(tf, "tf", 2, 4);
      break;
    case DVR_TF_LINEAR:
      check_size(tf, "tf", 2, 5);
      if (tf.sizes[1] <= 1) fail(DVR_E_INVALID_ARGUMENT, "tensor 'tf' must have at least two control points in TFLinear-mode");
      break;
    case DVR_TF_GAUSSIAN:
      check_size(tf, "tf", 2, 6);
      break;
    case DVR_TF_PRESHADED:
      break;  // any size, the TF is not read
    case DVR_TF_GAUSSIAN_LOG:
      fail(DVR_E_UNSUPPORTED, "TFGaussianLog is not supported by diffdvr_gb300");
    default:
      fail(DVR_E_INVALID_ARGUMENT, "unknown tf enum value");
  }
  if (tf.sizes[1] < 1) fail(DVR_E_INVALID_ARGUMENT, "tensor 'tf' must have at least one control point");
  if (!real_storage_ok(tf.dtype))
    fail(DVR_E_INVALID_ARGUMENT, std::string("tf must be of type float32 (or float16/bfloat16), but is ") +
                                     dtype_name(tf.dtype));
  p.tf = in_view(tf);
  p.tf_storage = tf.dtype;
  p.R = int(tf.sizes[1]);
  p.C = int(tf.sizes[2]);
  c.tf_mode = in.tf_mode;

  if (in.blend_mode != DVR_BLEND_BEER_LAMBERT && in.blend_mode != DVR_BLEND_ALPHA)
    fail(DVR_E_INVALID_ARGUMENT, "unknown blend enum value");
  c.blend = in.blend_mode;
  p.early_out = float(in.blending_early_out);
  p.B = B;
  // ray and pixel indices are 32-bit in the kernels
  if (int64_t(B) * p.H * p.W > 0x7fffffff)
    fail(DVR_E_INVALID_ARGUMENT, "batch x height x width must be below 2^31 rays");
  return c;
}

// renderer::Renderer::checkOutput (renderer/renderer.cpp:367-391)
void check_outputs(const DvrRendererOutputs& out, Checked& c, bool forward) {
  RenderParams& p = c.p;
  const DvrTensor& color = out.color;
  const char* cname = forward ? "color" : "output_color";
  check_dim(color, cname, 4);
  check_device(color, cname, c.device);
  check_size(color, cname, 0, p.B);
  check_size(color, cname, 1, p.H);
  check_size(color, cname, 2, p.W);
  check_size(color, cname, 3, 4);
  check_dtype(color, cname, DVR_FLOAT32);
  const DvrTensor& term = out.termination_index;
  check_dim(term, "terminationIndex", 3);
  check_device(term, "terminationIndex", c.device);
  check_size(term, "terminationIndex", 0, p.B);
  check_size(term, "terminationIndex", 1, p.H);
  check_size(term, "terminationIndex", 2, p.W);
  check_dtype(term, "terminationIndex", DVR_INT32);
  p.color = out_view(color, false);
  p.term = out_view(term, false);
  p.ckpt = OutView{};
  p.ckpt_slots = 0;
  p.ckpt_interval = out.checkpoint_interval > 0 ? out.checkpoint_interval : 32;
  if (out.checkpoints.ndim >= 0 && out.checkpoints.data != nullptr) {
    const DvrTensor& ck = out.checkpoints;
    check_dim(ck, "checkpoints", 4);
    check_device(ck, "checkpoints", c.device);
    check_size(ck, "checkpoints", 0, p.B);
    check_size(ck, "checkpoints", 1, p.H);
    check_size(ck, "checkpoints", 2, p.W);
    check_dtype(ck, "checkpoints", DVR_FLOAT32);
    if (ck.sizes[3] < 1) fail(DVR_E_INVALID_ARGUMENT, "checkpoints must hold at least one slot per ray");
    if (p.ckpt_interval < 1 || p.ckpt_interval > 64)
      fail(DVR_E_INVALID_ARGUMENT, "checkpoint_interval must be in [1, 64]");
    // the adjoint keeps one segment per thread in shared memory
    if (p.ckpt_interval > 32 && p.R * p.C > 1024)
      fail(DVR_E_INVALID_ARGUMENT, "checkpoint_interval above 32 needs a TF with at most 1024 entries");
    p.ckpt = out_view(ck, false);
    p.ckpt_slots = int(ck.sizes[3]);
  }
  p.dens = nullptr;
  p.dens_off = OutView{};
  p.dens_units = 0;
  const bool has_dens = out.sample_density.ndim >= 0 && out.sample_density.data != nullptr;
  const bool has_off = out.sample_offset.ndim >= 0 && out.sample_offset.data != nullptr;
  if (has_dens != has_off) fail(DVR_E_INVALID_ARGUMENT, "sample_density and sample_offset go together");
  if (has_dens) {
    // the density path re-marches unrecorded rays from checkpoints; pre-shaded rays invert the blend
    if (!p.ckpt.p && c.filter != DVR_FILTER_PRESHADED)
      fail(DVR_E_INVALID_ARGUMENT, "sample_density needs a checkpoint buffer");
    const DvrTensor& d = out.sample_density;
    check_dim(d, "sample_density", 1);
    check_device(d, "sample_density", c.device);
    check_dtype(d, "sample_density", DVR_FLOAT32);
    if (d.sizes[0] < 4 || (d.sizes[0] > 1 && d.strides[0] != 1) ||
        (reinterpret_cast<uintptr_t>(d.data) & 15u) != 0)
      fail(DVR_E_INVALID_ARGUMENT, "sample_density must be contiguous, 16-byte aligned and hold at least 4 values");
    const DvrTensor& o = out.sample_offset;
    check_dim(o, "sample_offset", 3);
    check_device(o, "sample_offset", c.device);
    check_size(o, "sample_offset", 0, p.B);
    check_size(o, "sample_offset", 1, p.H);
    check_size(o, "sample_offset", 2, p.W);
    check_dtype(o, "sample_offset", DVR_INT32);
    p.dens = static_cast<float*>(d.data);
    p.dens_off = out_view(o, false);
    p.dens_units = std::min<int64_t>(d.sizes[0] / 4, 0x7fffffff);
  }
}

// checkAdjointOutput (renderer/renderer.cpp:265-365) plus the forward-output
// and adj_color checks of renderAdjoint (renderer/renderer.cpp:670-717)
AdjointParams check_adjoint(const DvrTensor& adj_color, const DvrAdjointOutputs& o, const Checked& c) {
  const RenderParams& p = c.p;
  AdjointParams a{};
  check_dim(adj_color, "adj_color", 4);
  check_device(adj_color, "adj_color", c.device);
  check_size(adj_color, "adj_color", 0, p.B);
  check_size(adj_color, "adj_color", 1, p.H);
  check_size(adj_color, "adj_color", 2, p.W);
  check_size(adj_color, "adj_color", 3, 4);
  check_dtype(adj_color, "adj_color", DVR_FLOAT32);
  a.adj_color = in_view(adj_color);
  a.fwd_color = InView{p.color.p, {p.color.s[0], p.color.s[1], p.color.s[2], p.color.s[3]}, {0, 0, 0}, 0};
  a.fwd_term = InView{p.term.p, {p.term.s[0], p.term.s[1], p.term.s[2], 0}, {0, 0, 0}, 0};

  a.has_volume = o.has_volume_derivatives != 0;
  if (a.has_volume) {
    const DvrTensor& t = o.adj_volume;
    check_dim(t, "adj_volume", 4);
    check_device(t, "adj_volume", c.device);
    if (c.filter == DVR_FILTER_PRESHADED) check_size(t, "adj_volume", 0, 4);  // renderer/renderer.cpp:277-279
    else check_batch(t, "adj_volume", p.B);
    check_size(t, "adj_volume", 1, p.X);
    check_size(t, "adj_volume", 2, p.Y);
    check_size(t, "adj_volume", 3, p.Z);
    check_dtype(t, "adj_volume", DVR_FLOAT32);
    a.adj_volume = out_view(t, true);
  }
  a.has_stepsize = o.has_stepsize_derivatives != 0;
  if (a.has_stepsize) {
    const DvrTensor& t = o.adj_stepsize;
    check_dim(t, "adj_stepSize", 3);
    check_device(t, "adj_stepSize", c.device);
    check_batch(t, "adj_stepSize", p.B);
    check_batch(t, "adj_stepSize", p.H, 1);
    check_batch(t, "adj_stepSize", p.W, 2);
    check_dtype(t, "adj_stepSize", DVR_FLOAT32);
    a.adj_step = out_view(t, true);
    a.stepsize_broadcast = p.B != t.sizes[0] || p.H != t.sizes[1] || p.W != t.sizes[2];
  }
  a.has_camera = o.has_camera_derivatives != 0;
  if (a.has_camera) {
    const DvrTensor& ts = o.adj_camera_ray_start;
    check_dim(ts, "adj_cameraRayStart", 4);
    check_device(ts, "adj_cameraRayStart", c.device);
    check_batch(ts, "adj_cameraRayStart", p.B);
    check_size(ts, "adj_cameraRayStart", 1, p.H);
    check_size(ts, "adj_cameraRayStart", 2, p.W);
    check_size(ts, "adj_cameraRayStart", 3, 3);
    check_dtype(ts, "adj_cameraRayStart", DVR_FLOAT32);
    const DvrTensor& td = o.adj_camera_ray_dir;
    check_dim(td, "adj_cameraRayDir", 4);
    check_device(td, "adj_cameraRayDir", c.device);
    check_batch(td, "adj_cameraRayDir", p.B);
    check_size(td, "adj_cameraRayDir", 1, p.H);
    check_size(td, "adj_cameraRayDir", 2, p.W);
    check_size(td, "adj_cameraRayDir", 3, 3);
    check_dtype(td, "adj_cameraRayDir", DVR_FLOAT32);
    a.adj_start = out_view(ts, true);
    a.adj_dir = out_view(td, true);
    a.camera_broadcast = p.B != ts.sizes[0] || p.B != td.sizes[0];
    if (p.camera_mode != DVR_CAMERA_RAY_START_DIR)
      fail(DVR_E_INVALID_ARGUMENT, "camera derivatives require cameraMode == RayStartDir (per-pixel rays)");
  }
  a.has_tf = o.has_tf_derivatives != 0;
  a.tf_delayed = o.tf_delayed_accumulation != 0;
  if (a.has_tf) {
    const DvrTensor& t = o.adj_tf;
    check_dim(t, "adj_tf", 3);
    check_device(t, "adj_tf", c.device);
    check_batch(t, "adj_tf", p.B);
    check_size(t, "adj_tf", 1, p.R);
    check_size(t, "adj_tf", 2, p.C);
    check_dtype(t, "adj_tf", DVR_FLOAT32);
    a.adj_tf = out_view(t, true);
  }
  a.has_viewport = o.has_viewport_derivatives != 0;
  if (a.has_viewport) {
    const DvrTensor& t = o.adj_viewport;
    check_dim(t, "adj_viewport", 3);
    check_device(t, "adj_viewport", c.device);
    check_batch(t, "adj_viewport", p.B);
    check_size(t, "adj_viewport", 1, 3);
    check_size(t, "adj_viewport", 2, 3);
    check_dtype(t, "adj_viewport", DVR_FLOAT32);
    if (p.camera_mode != DVR_CAMERA_REFERENCE_FRAME)
      fail(DVR_E_INVALID_ARGUMENT, "viewport derivatives require cameraMode == ReferenceFrame");
    if (c.filter == DVR_FILTER_PRESHADED)
      fail(DVR_E_UNSUPPORTED, "viewport derivatives are not available for pre-shaded volumes");
    if (p.B > kMaxViewportBatch)
      fail(DVR_E_UNSUPPORTED, "viewport derivatives support batches of at most 256 views");
    a.adj_viewport = out_view(t, true);
  }
  if (!a.has_volume && !a.has_stepsize && !a.has_camera && !a.has_tf && !a.has_viewport)
    fail(DVR_E_NO_GRADIENT, "At least one adjoint variable must be activated!");
  return a;
}

void after_launch(cudaError_t e, cudaStream_t s, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(DVR_E_CUDA, std::string(what) + " launch failed: " + cudaGetErrorString(e));
  }
  if (g_sync.load()) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) fail(DVR_E_CUDA, std::string(what) + " failed: " + cudaGetErrorString(e));
  }
}

bool use_plain(const Checked& c, const AdjointParams* a = nullptr) {
  if (g_family.load() == DVR_KERNELS_PLAIN) {
    if (a && a->has_viewport)
      fail(DVR_E_UNSUPPORTED, "viewport derivatives are computed by the optimized kernel family only");
    if (c.p.vol_storage != DVR_FLOAT32 || c.p.tf_storage != DVR_FLOAT32)
      fail(DVR_E_UNSUPPORTED, "the plain kernel family renders float32 volumes and TFs only");
    if (c.p.dens)
      fail(DVR_E_UNSUPPORTED, "sample_density is recorded and read by the optimized kernel family only");
    return true;
  }
  return false;
}

template <typename F>
int guarded(F&& fn) {
  try {
    fn();
    g_last_error.clear();
    return DVR_OK;
  } catch (const DvrError& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return DVR_E_INVALID_ARGUMENT;
  }
}

cudaError_t dispatch_forward(const Checked& c, bool plain, const LaunchInfo& li, cudaStream_t s) {
  if (c.filter == DVR_FILTER_PRESHADED) return launch_preshaded_forward(c.p, c.blend, plain, li, s);
  switch (c.tf_mode) {
    case DVR_TF_IDENTITY:
      return plain ? launch_plain_forward<0>(c.p, c.filter, c.blend, li, s)
                   : launch_fast_forward<0>(c.p, c.filter, c.blend, li, s);
    case DVR_TF_TEXTURE:
      return plain ? launch_plain_forward<1>(c.p, c.filter, c.blend, li, s)
                   : launch_fast_forward<1>(c.p, c.filter, c.blend, li, s);
    case DVR_TF_LINEAR:
      return plain ? launch_plain_forward<2>(c.p, c.filter, c.blend, li, s)
                   : launch_fast_forward<2>(c.p, c.filter, c.blend, li, s);
    default:
      return plain ? launch_plain_forward<3>(c.p, c.filter, c.blend, li, s)
                   : launch_fast_forward<3>(c.p, c.filter, c.blend, li, s);
  }
}

cudaError_t dispatch_adjoint(const Checked& c, const AdjointParams& a, bool plain, const LaunchInfo& li,
                             cudaStream_t s) {
  // the plain family keeps the reference's position and step-size adjoints
  if (c.filter == DVR_FILTER_PRESHADED) return launch_preshaded_adjoint(c.p, a, c.blend, !plain, li, s);
  switch (c.tf_mode) {
    case DVR_TF_IDENTITY:
      return plain ? launch_plain_adjoint<0>(c.p, a, c.filter, c.blend, li, s)
                   : launch_fast_adjoint<0>(c.p, a, c.filter, c.blend, li, s);
    case DVR_TF_TEXTURE:
      return plain ? launch_plain_adjoint<1>(c.p, a, c.filter, c.blend, li, s)
                   : launch_fast_adjoint<1>(c.p, a, c.filter, c.blend, li, s);
    case DVR_TF_LINEAR:
      return plain ? launch_plain_adjoint<2>(c.p, a, c.filter, c.blend, li, s)
                   : launch_fast_adjoint<2>(c.p, a, c.filter, c.blend, li, s);
    default:
      return plain ? launch_plain_adjoint<3>(c.p, a, c.filter, c.blend, li, s)
                   : launch_fast_adjoint<3>(c.p, a, c.filter, c.blend, li, s);
  }
}

cudaError_t dispatch_adjoint_into(const Checked& c, const AdjointParams& a, const LaunchInfo& li,
                                  const CallerScratch& sc, cudaStream_t s) {
  switch (c.tf_mode) {
    case DVR_TF_IDENTITY: return launch_fast_adjoint_into<0>(c.p, a, c.filter, c.blend, li, sc, s);
    case DVR_TF_TEXTURE: return launch_fast_adjoint_into<1>(c.p, a, c.filter, c.blend, li, sc, s);
    case DVR_TF_LINEAR: return launch_fast_adjoint_into<2>(c.p, a, c.filter, c.blend, li, sc, s);
    default: return launch_fast_adjoint_into<3>(c.p, a, c.filter, c.blend, li, sc, s);
  }
}

// ---- forward-mode differentiation ----
// Derivative indices of DvrForwardDifferencesSettings (host values) checked
// against D; -1 (or any negative) = not traced.
int checked_index(int32_t i, int D, const char* name) {
  if (i < 0) return -1;
  if (i >= D) {
    std::ostringstream os;
    os << name << " = " << i << " is not a derivative index: the number of derivatives D is " << D;
    fail(DVR_E_INVALID_ARGUMENT, os.str());
  }
  return i;
}

void set_d_tf(const DvrForwardDifferencesSettings& fs, int device, const int32_t*& ptr, int64_t* strides) {
  ptr = nullptr;
  strides[0] = strides[1] = strides[2] = 0;
  if (!fs.has_tf_derivatives) return;
  const DvrTensor& t = fs.d_tf;
  if (t.ndim < 0 || t.data == nullptr)
    fail(DVR_E_INVALID_ARGUMENT, "d_tf not defined, hence hasTfDerivatives must be false but was set to true");
  check_dim(t, "d_tf", 3);
  check_device(t, "d_tf", device);
  check_dtype(t, "d_tf", DVR_INT32);
  ptr = static_cast<const int32_t*>(t.data);
  for (int i = 0; i < 3; ++i) strides[i] = t.sizes[i] == 1 ? 0 : t.strides[i];
}

cudaError_t dispatch_forward_gradients(const Checked& c, const FwdGradParams& g, const LaunchInfo& li,
                                       cudaStream_t s) {
  switch (c.tf_mode) {
    case DVR_TF_IDENTITY: return launch_forward_gradients<0>(c.p, g, c.filter, c.blend, li, s);
    case DVR_TF_TEXTURE: return launch_forward_gradients<1>(c.p, g, c.filter, c.blend, li, s);
    case DVR_TF_LINEAR: return launch_forward_gradients<2>(c.p, g, c.filter, c.blend, li, s);
    default: return launch_forward_gradients<3>(c.p, g, c.filter, c.blend, li, s);
  }
}

}  // namespace

int& last_adjoint_path() { return g_adjoint_path; }
bool window_adjoint_on() { return g_window.load() != 0; }
int forward_gather_mode() { return g_gather.load(); }

int render_adjoint_into(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs_from_forward,
                        const DvrTensor* adj_color, const DvrAdjointOutputs* adj_outputs, void* cuda_stream,
                        ScratchSource source) {
  return guarded([&] {
    if (!inputs || !outputs_from_forward || !adj_color || !adj_outputs)
      fail(DVR_E_INVALID_ARGUMENT, "arguments must not be NULL");
    Checked c = check_inputs(*inputs);
    if (c.filter == DVR_FILTER_PRESHADED)
      fail(DVR_E_UNSUPPORTED, "pre-shaded volumes take dvr_render_adjoint, which orders the rays in library scratch");
    check_outputs(*outputs_from_forward, c, false);
    const AdjointParams a = check_adjoint(*adj_color, *adj_outputs, c);
    DeviceGuard guard(c.device);
    const LaunchInfo li = launch_info(c.device);
    CallerScratch sc{};
    if (const char* msg = source(c.device, &sc)) fail(DVR_E_CUDA, msg);
    if (a.has_tf) {
      // one TF-gradient slice of R*C floats per block, at least one block per SM
      const size_t need = size_t(li.num_sms) * size_t(c.p.R) * size_t(c.p.C) * sizeof(float);
      if (need > sc.tf_bytes) {
        std::ostringstream m;
        m << "TF too large for the no-allocation adjoint: " << c.p.R << " control points x " << c.p.C
          << " channels need " << need << " bytes of TF-gradient scratch (" << li.num_sms
          << " SMs), the static scratch holds " << sc.tf_bytes << "; use dvr_render_adjoint";
        fail(DVR_E_INVALID_ARGUMENT, m.str());
      }
    }
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    after_launch(dispatch_adjoint_into(c, a, li, sc, s), s, "adjoint");
  });
}

}  // namespace dvr

using namespace dvr;

extern "C" int dvr_render_forward(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs,
                                  void* cuda_stream) {
  return guarded([&] {
    if (!inputs || !outputs) fail(DVR_E_INVALID_ARGUMENT, "inputs and outputs must not be NULL");
    Checked c = check_inputs(*inputs);
    check_outputs(*outputs, c, true);
    DeviceGuard guard(c.device);
    const LaunchInfo li = launch_info(c.device);
    const bool plain = use_plain(c);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    after_launch(dispatch_forward(c, plain, li, s), s, "forward");
  });
}

extern "C" int dvr_render_adjoint(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs_from_forward,
                                  const DvrTensor* adj_color, const DvrAdjointOutputs* adj_outputs,
                                  void* cuda_stream) {
  g_adjoint_path = DVR_PATH_NONE;
  return guarded([&] {
    if (!inputs || !outputs_from_forward || !adj_color || !adj_outputs)
      fail(DVR_E_INVALID_ARGUMENT, "arguments must not be NULL");
    Checked c = check_inputs(*inputs);
    check_outputs(*outputs_from_forward, c, false);
    const AdjointParams a = check_adjoint(*adj_color, *adj_outputs, c);
    DeviceGuard guard(c.device);
    const LaunchInfo li = launch_info(c.device);
    const bool plain = use_plain(c, &a);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    g_adjoint_path = c.filter == DVR_FILTER_PRESHADED ? DVR_PATH_PRESHADED : plain ? DVR_PATH_PLAIN : DVR_PATH_GENERAL;
    after_launch(dispatch_adjoint(c, a, plain, li, s), s, "adjoint");
  });
}

// Tile shape of each instance (DvrTileShape), default 16x8.
std::vector<unsigned char> tile_shapes(const int32_t* shapes, int n) {
  std::vector<unsigned char> out(n, 0);
  for (int i = 0; shapes && i < n; ++i) {
    if (shapes[i] < DVR_TILE_16x8 || shapes[i] > DVR_TILE_8x16) fail(DVR_E_INVALID_ARGUMENT, "unknown tile shape");
    out[i] = static_cast<unsigned char>(shapes[i]);
  }
  return out;
}

extern "C" int dvr_render_forward_batched(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs,
                                          int32_t n, void* cuda_stream) {
  return dvr_render_forward_batched_tiled(inputs, outputs, nullptr, n, cuda_stream);
}

extern "C" int dvr_render_forward_batched_tiled(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs,
                                                const int32_t* shapes, int32_t n, void* cuda_stream) {
  return guarded([&] {
    if (n < 0 || (n > 0 && (!inputs || !outputs))) fail(DVR_E_INVALID_ARGUMENT, "invalid instance list");
    if (n == 0) return;
    std::vector<Checked> cs(n);
    for (int i = 0; i < n; ++i) {
      cs[i] = check_inputs(inputs[i]);
      if (cs[i].filter == DVR_FILTER_PRESHADED)
        fail(DVR_E_UNSUPPORTED, "pre-shaded volumes are rendered by the single-instance entry points");
      check_outputs(outputs[i], cs[i], true);
      if (i > 0 && (cs[i].filter != cs[0].filter || cs[i].tf_mode != cs[0].tf_mode || cs[i].blend != cs[0].blend ||
                    cs[i].p.vol_storage != cs[0].p.vol_storage || cs[i].p.tf_storage != cs[0].p.tf_storage ||
                    cs[i].device != cs[0].device))
        fail(DVR_E_INVALID_ARGUMENT,
             "all instances of a batched call must share filter, TF and blend modes, storage types and device");
    }
    DeviceGuard guard(cs[0].device);
    const LaunchInfo li = launch_info(cs[0].device);
    std::vector<RenderParams> ps(n);
    for (int i = 0; i < n; ++i) ps[i] = cs[i].p;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    const std::vector<unsigned char> ts = tile_shapes(shapes, n);
    after_launch(launch_batched_forward(ps.data(), ts.data(), n, cs[0].filter, cs[0].tf_mode, cs[0].blend,
                                        cs[0].device, li, s),
                 s, "batched forward");
  });
}

extern "C" int dvr_render_adjoint_batched(const DvrRendererInputs* inputs,
                                          const DvrRendererOutputs* outputs_from_forward, const DvrTensor* adj_colors,
                                          const DvrAdjointOutputs* adj_outputs, int32_t n, void* cuda_stream) {
  return dvr_render_adjoint_batched_tiled(inputs, outputs_from_forward, adj_colors, adj_outputs, nullptr, n,
                                          cuda_stream);
}

extern "C" int dvr_render_adjoint_batched_tiled(const DvrRendererInputs* inputs,
                                                const DvrRendererOutputs* outputs_from_forward,
                                                const DvrTensor* adj_colors, const DvrAdjointOutputs* adj_outputs,
                                                const int32_t* shapes, int32_t n, void* cuda_stream) {
  return guarded([&] {
    if (n < 0 || (n > 0 && (!inputs || !outputs_from_forward || !adj_colors || !adj_outputs)))
      fail(DVR_E_INVALID_ARGUMENT, "invalid instance list");
    if (n == 0) return;
    std::vector<Checked> cs(n);
    std::vector<AdjointParams> as(n);
    for (int i = 0; i < n; ++i) {
      cs[i] = check_inputs(inputs[i]);
      if (cs[i].filter == DVR_FILTER_PRESHADED)
        fail(DVR_E_UNSUPPORTED, "pre-shaded volumes are rendered by the single-instance entry points");
      check_outputs(outputs_from_forward[i], cs[i], false);
      as[i] = check_adjoint(adj_colors[i], adj_outputs[i], cs[i]);
      if (as[i].has_viewport)
        fail(DVR_E_UNSUPPORTED, "the batched entry points do not compute viewport derivatives");
      if (i > 0 && (cs[i].filter != cs[0].filter || cs[i].tf_mode != cs[0].tf_mode || cs[i].blend != cs[0].blend ||
                    cs[i].p.vol_storage != cs[0].p.vol_storage || cs[i].p.tf_storage != cs[0].p.tf_storage ||
                    cs[i].device != cs[0].device || as[i].has_volume != as[0].has_volume ||
                    as[i].has_tf != as[0].has_tf))
        fail(DVR_E_INVALID_ARGUMENT,
             "all instances of a batched call must share modes, storage types, device and gradient selection");
    }
    DeviceGuard guard(cs[0].device);
    const LaunchInfo li = launch_info(cs[0].device);
    std::vector<RenderParams> ps(n);
    for (int i = 0; i < n; ++i) ps[i] = cs[i].p;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    const std::vector<unsigned char> ts = tile_shapes(shapes, n);
    after_launch(launch_batched_adjoint(ps.data(), as.data(), ts.data(), n, cs[0].filter, cs[0].tf_mode,
                                        cs[0].blend, cs[0].device, li, s),
                 s, "batched adjoint");
  });
}

// renderer::Renderer::renderForwardGradients (renderer/renderer.cpp:419-498)
extern "C" int dvr_render_forward_gradients(const DvrRendererInputs* inputs,
                                            const DvrForwardDifferencesSettings* settings,
                                            const DvrRendererOutputs* outputs, const DvrTensor* gradients_out,
                                            void* cuda_stream) {
  return guarded([&] {
    if (!inputs || !settings || !outputs || !gradients_out)
      fail(DVR_E_INVALID_ARGUMENT, "arguments must not be NULL");
    Checked c = check_inputs(*inputs);
    if (c.filter == DVR_FILTER_PRESHADED)
      fail(DVR_E_UNSUPPORTED, "forward derivatives are not available for pre-shaded volumes");
    const DvrForwardDifferencesSettings& fs = *settings;
    if (fs.D <= 0) fail(DVR_E_INVALID_ARGUMENT, "number of derivatives must be positive");
    FwdGradParams g{};
    g.D = fs.D;
    set_d_tf(fs, c.device, g.d_tf, g.dtf_s);
    if (g.d_tf) {
      check_size(fs.d_tf, "d_tf", 0, inputs->tf.sizes[0]);
      check_size(fs.d_tf, "d_tf", 1, c.p.R);
      check_size(fs.d_tf, "d_tf", 2, c.p.C);
    }
    g.has_tf = g.d_tf != nullptr;
    g.d_step = checked_index(fs.d_stepsize, fs.D, "d_stepsize");
    bool has_camera = false;
    for (int i = 0; i < 3; ++i) {
      g.d_start[i] = checked_index(fs.d_ray_start[i], fs.D, "d_rayStart");
      g.d_dir[i] = checked_index(fs.d_ray_dir[i], fs.D, "d_rayDir");
      has_camera |= g.d_start[i] >= 0 || g.d_dir[i] >= 0;
    }
    if (g.d_step < 0 && !has_camera && !g.has_tf) fail(DVR_E_INVALID_ARGUMENT, "at least one derivative must be activated");
    DvrRendererOutputs plain_out = *outputs;  // color and termination index only
    plain_out.checkpoints.ndim = -1;
    plain_out.sample_density.ndim = -1;
    plain_out.sample_offset.ndim = -1;
    check_outputs(plain_out, c, true);
    const DvrTensor& go = *gradients_out;
    check_dim(go, "gradientsOut", 5);
    check_device(go, "gradientsOut", c.device);
    check_size(go, "gradientsOut", 0, c.p.B);
    check_size(go, "gradientsOut", 1, c.p.H);
    check_size(go, "gradientsOut", 2, c.p.W);
    check_size(go, "gradientsOut", 3, fs.D);
    check_size(go, "gradientsOut", 4, 4);
    check_dtype(go, "gradientsOut", DVR_FLOAT32);
    g.grad = static_cast<float*>(go.data);
    for (int i = 0; i < 5; ++i) g.grad_s[i] = go.strides[i];
    DeviceGuard guard(c.device);
    const LaunchInfo li = launch_info(c.device);
    const int copies = c.p.tf.s[0] == 0 ? 1 : c.p.B;
    const size_t tf_bytes = size_t((int64_t(copies) * c.p.R * c.p.C + 3) / 4) * 16;
    int pass = kFwdMaxPass;
    while (pass > 32 && tf_bytes + size_t(kFwdThreads / 32) * pass * 16 > size_t(li.max_smem_optin)) pass /= 2;
    if (tf_bytes + size_t(kFwdThreads / 32) * pass * 16 > size_t(li.max_smem_optin))
      fail(DVR_E_UNSUPPORTED, "the TF (all batch entries) does not fit into shared memory for forward derivatives");
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    for (int d0 = 0; d0 < fs.D; d0 += pass) {
      g.d0 = d0;
      g.dn = std::min(pass, fs.D - d0);
      after_launch(dispatch_forward_gradients(c, g, li, s), s, "forward gradients");
    }
  });
}

// renderer::Renderer::forwardVariablesToGradients (renderer/renderer.cpp:500-558)
extern "C" int dvr_forward_variables_to_gradients(const DvrTensor* forward_variables, const DvrTensor* adj_color,
                                                  const DvrForwardDifferencesSettings* settings,
                                                  const DvrAdjointOutputs* adj_outputs, void* cuda_stream) {
  return guarded([&] {
    if (!forward_variables || !adj_color || !settings || !adj_outputs)
      fail(DVR_E_INVALID_ARGUMENT, "arguments must not be NULL");
    const DvrTensor& fv = *forward_variables;
    check_dim(fv, "forwardVariables", 5);
    if (fv.device_type != DVR_DEVICE_CUDA)
      fail(DVR_E_INVALID_ARGUMENT, "forwardVariables is a CPU tensor: diffdvr_gb300 runs on CUDA devices only");
    const int device = fv.device_index;
    check_size(fv, "forwardVariables", 4, 4);
    check_dtype(fv, "forwardVariables", DVR_FLOAT32);
    FwdVarsParams v{};
    v.B = int(fv.sizes[0]);
    v.H = int(fv.sizes[1]);
    v.W = int(fv.sizes[2]);
    v.D = int(fv.sizes[3]);
    v.fwd = static_cast<const float*>(fv.data);
    for (int i = 0; i < 5; ++i) v.fwd_s[i] = fv.strides[i];
    const DvrTensor& ac = *adj_color;
    check_dim(ac, "gradientOutputColor", 4);
    check_device(ac, "gradientOutputColor", device);
    check_size(ac, "gradientOutputColor", 0, v.B);
    check_size(ac, "gradientOutputColor", 1, v.H);
    check_size(ac, "gradientOutputColor", 2, v.W);
    check_size(ac, "gradientOutputColor", 3, 4);
    check_dtype(ac, "gradientOutputColor", DVR_FLOAT32);
    v.adj_color = static_cast<const float*>(ac.data);
    for (int i = 0; i < 4; ++i) v.adj_s[i] = ac.strides[i];
    const DvrForwardDifferencesSettings& fs = *settings;
    set_d_tf(fs, device, v.d_tf, v.dtf_s);
    v.d_step = checked_index(fs.d_stepsize, v.D, "d_stepsize");
    for (int i = 0; i < 3; ++i) {
      v.d_start[i] = checked_index(fs.d_ray_start[i], v.D, "d_rayStart");
      v.d_dir[i] = checked_index(fs.d_ray_dir[i], v.D, "d_rayDir");
    }
    const DvrAdjointOutputs& o = *adj_outputs;
    if (o.has_volume_derivatives)
      fail(DVR_E_INVALID_ARGUMENT, "volume derivatives are not supported with forward variables");
    if (o.has_viewport_derivatives)
      fail(DVR_E_INVALID_ARGUMENT, "viewport derivatives are not supported with forward variables");
    v.has_step = o.has_stepsize_derivatives != 0;
    if (v.has_step) {
      const DvrTensor& t = o.adj_stepsize;
      check_dim(t, "adj_stepSize", 3);
      check_device(t, "adj_stepSize", device);
      check_batch(t, "adj_stepSize", v.B);
      check_batch(t, "adj_stepSize", v.H, 1);
      check_batch(t, "adj_stepSize", v.W, 2);
      check_dtype(t, "adj_stepSize", DVR_FLOAT32);
      v.adj_step = static_cast<float*>(t.data);
      for (int i = 0; i < 3; ++i) v.step_s[i] = t.sizes[i] == 1 ? 0 : t.strides[i];
      v.step_broadcast = v.B != t.sizes[0] || v.H != t.sizes[1] || v.W != t.sizes[2];
    }
    v.has_camera = o.has_camera_derivatives != 0;
    if (v.has_camera) {
      const DvrTensor* ts[2] = {&o.adj_camera_ray_start, &o.adj_camera_ray_dir};
      const char* names[2] = {"adj_cameraRayStart", "adj_cameraRayDir"};
      for (int k = 0; k < 2; ++k) {
        const DvrTensor& t = *ts[k];
        check_dim(t, names[k], 4);
        check_device(t, names[k], device);
        check_batch(t, names[k], v.B);
        check_size(t, names[k], 1, v.H);
        check_size(t, names[k], 2, v.W);
        check_size(t, names[k], 3, 3);
        check_dtype(t, names[k], DVR_FLOAT32);
        v.camera_broadcast |= v.B != t.sizes[0];
      }
      v.adj_start = static_cast<float*>(o.adj_camera_ray_start.data);
      v.adj_dir = static_cast<float*>(o.adj_camera_ray_dir.data);
      for (int i = 0; i < 4; ++i) {
        v.start_s[i] = (i == 0 && o.adj_camera_ray_start.sizes[0] == 1) ? 0 : o.adj_camera_ray_start.strides[i];
        v.dir_s[i] = (i == 0 && o.adj_camera_ray_dir.sizes[0] == 1) ? 0 : o.adj_camera_ray_dir.strides[i];
      }
    }
    v.has_tf = o.has_tf_derivatives != 0 && v.d_tf != nullptr;
    if (o.has_tf_derivatives && !v.d_tf)
      fail(DVR_E_INVALID_ARGUMENT, "TF derivatives need the TF derivative indices (d_tf, has_tf_derivatives)");
    if (v.has_tf) {
      const DvrTensor& t = o.adj_tf;
      check_dim(t, "adj_tf", 3);
      check_device(t, "adj_tf", device);
      check_batch(t, "adj_tf", v.B);
      check_size(t, "adj_tf", 1, fs.d_tf.sizes[1]);
      check_size(t, "adj_tf", 2, fs.d_tf.sizes[2]);
      check_dtype(t, "adj_tf", DVR_FLOAT32);
      if (fs.d_tf.sizes[0] != 1 && fs.d_tf.sizes[0] != v.B)
        fail(DVR_E_INVALID_ARGUMENT, "d_tf must have batch size 1 or B");
      v.R = int(t.sizes[1]);
      v.C = int(t.sizes[2]);
      v.adj_tf = static_cast<float*>(t.data);
      for (int i = 0; i < 3; ++i) v.tf_s[i] = t.sizes[i] == 1 ? 0 : t.strides[i];
    }
    DeviceGuard guard(device);
    const LaunchInfo li = launch_info(device);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    after_launch(launch_forward_variables_to_gradients(v, li, s), s, "forward variables to gradients");
  });
}

// ---- TFUtils::preshadeVolume (renderer/tf_utils.cpp:173-249) ----
namespace dvr {
namespace {
PreshadeParams check_preshade(const DvrTensor& density, const DvrTensor& tf, int tf_mode, int& device) {
  PreshadeParams q{};
  check_dim(density, "densityVolume", 4);
  if (density.device_type != DVR_DEVICE_CUDA)
    fail(DVR_E_INVALID_ARGUMENT, "densityVolume is a CPU tensor: diffdvr_gb300 runs on CUDA devices only");
  device = density.device_index;
  check_dtype(density, "densityVolume", DVR_FLOAT32);
  check_size(density, "densityVolume", 0, 1);
  q.X = int(density.sizes[1]);
  q.Y = int(density.sizes[2]);
  q.Z = int(density.sizes[3]);
  check_dim(tf, "tf", 3);
  check_device(tf, "tf", device);
  check_size(tf, "tf", 0, 1);
  check_dtype(tf, "tf", DVR_FLOAT32);
  switch (tf_mode) {
    case DVR_TF_IDENTITY:
      check_size(tf, "tf", 1, 1);
      check_size(tf, "tf", 2, 2);
      break;
    case DVR_TF_TEXTURE:
      check_size(tf, "tf", 2, 4);
      break;
    case DVR_TF_LINEAR:
      check_size(tf, "tf", 2, 5);
      if (tf.sizes[1] <= 1) fail(DVR_E_INVALID_ARGUMENT, "tensor 'tf' must have at least two control points in TFLinear-mode");
      break;
    case DVR_TF_GAUSSIAN:
      check_size(tf, "tf", 2, 6);
      break;
    case DVR_TF_GAUSSIAN_LOG:
      fail(DVR_E_UNSUPPORTED, "TFGaussianLog is not supported by diffdvr_gb300");
    default:
      fail(DVR_E_INVALID_ARGUMENT, "unknown tf enum value: " + std::to_string(tf_mode));
  }
  if (tf.sizes[1] < 1) fail(DVR_E_INVALID_ARGUMENT, "tensor 'tf' must have at least one control point");
  q.R = int(tf.sizes[1]);
  q.C = int(tf.sizes[2]);
  q.density = static_cast<const float*>(density.data);
  for (int i = 0; i < 4; ++i) q.d_s[i] = density.strides[i];
  q.tf = static_cast<const float*>(tf.data);
  for (int i = 0; i < 3; ++i) q.tf_s[i] = tf.strides[i];
  return q;
}

void check_volume_like(const DvrTensor& t, const char* name, int channels, const PreshadeParams& q, int device) {
  check_dim(t, name, 4);
  check_device(t, name, device);
  check_size(t, name, 0, channels);
  check_size(t, name, 1, q.X);
  check_size(t, name, 2, q.Y);
  check_size(t, name, 3, q.Z);
  check_dtype(t, name, DVR_FLOAT32);
}
}  // namespace
}  // namespace dvr

extern "C" int dvr_preshade_volume(const DvrTensor* density, const DvrTensor* tf, int32_t tf_mode,
                                   const DvrTensor* color_out, void* cuda_stream) {
  return guarded([&] {
    if (!density || !tf || !color_out) fail(DVR_E_INVALID_ARGUMENT, "arguments must not be NULL");
    int device = 0;
    PreshadeParams q = check_preshade(*density, *tf, tf_mode, device);
    check_volume_like(*color_out, "color", 4, q, device);
    q.out = static_cast<float*>(color_out->data);
    for (int i = 0; i < 4; ++i) q.o_s[i] = color_out->strides[i];
    DeviceGuard guard(device);
    const LaunchInfo li = launch_info(device);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    after_launch(launch_preshade_volume(q, tf_mode, false, li, s), s, "preshade volume");
  });
}

extern "C" int dvr_preshade_volume_adjoint(const DvrTensor* density, const DvrTensor* tf, int32_t tf_mode,
                                           const DvrTensor* adj_color, const DvrTensor* adj_density,
                                           void* cuda_stream) {
  return guarded([&] {
    if (!density || !tf || !adj_color || !adj_density) fail(DVR_E_INVALID_ARGUMENT, "arguments must not be NULL");
    int device = 0;
    PreshadeParams q = check_preshade(*density, *tf, tf_mode, device);
    check_volume_like(*adj_color, "adj_color", 4, q, device);
    check_volume_like(*adj_density, "adj_density", 1, q, device);
    q.adj_color = static_cast<const float*>(adj_color->data);
    for (int i = 0; i < 4; ++i) q.a_s[i] = adj_color->strides[i];
    q.out = static_cast<float*>(adj_density->data);
    for (int i = 0; i < 4; ++i) q.o_s[i] = adj_density->strides[i];
    DeviceGuard guard(device);
    const LaunchInfo li = launch_info(device);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    after_launch(launch_preshade_volume(q, tf_mode, true, li, s), s, "preshade volume adjoint");
  });
}

extern "C" int64_t dvr_checkpoint_slots(double max_ray_length, double min_step_size, int32_t checkpoint_interval) {
  const int K = checkpoint_interval > 0 ? checkpoint_interval : 32;
  if (!(max_ray_length >= 0) || !(min_step_size > 0) || K > 64) {
    g_last_error = "dvr_checkpoint_slots: need max_ray_length >= 0, min_step_size > 0 and interval <= 64";
    return DVR_E_INVALID_ARGUMENT;
  }
  // samples k = 0..n-1 with t = tmin + k*step <= tmax: n <= floor(len/step) + 1
  const double n = std::floor(max_ray_length / min_step_size) + 2.0;
  const double slots = std::ceil(n / K);
  return slots < 1 ? 1 : int64_t(slots);
}

extern "C" const char* dvr_last_error(void) { return g_last_error.c_str(); }

extern "C" int dvr_set_kernel_family(int32_t family) {
  if (family != DVR_KERNELS_PLAIN && family != DVR_KERNELS_OPTIMIZED) {
    g_last_error = "unknown kernel family";
    return DVR_E_INVALID_ARGUMENT;
  }
  return g_family.exchange(family);
}
extern "C" int dvr_get_kernel_family(void) { return g_family.load(); }
extern "C" int dvr_set_sync_mode(int32_t sync) { return g_sync.exchange(sync ? 1 : 0); }
extern "C" int dvr_get_sync_mode(void) { return g_sync.load(); }
extern "C" int dvr_abi_version(void) { return DVR_ABI_VERSION; }
extern "C" int dvr_set_window_adjoint(int32_t enable) { return g_window.exchange(enable ? 1 : 0); }
extern "C" int dvr_get_window_adjoint(void) { return g_window.load(); }
extern "C" int dvr_set_forward_gather(int32_t mode) {
  if (mode < DVR_GATHER_AUTO || mode > DVR_GATHER_TEXTURE) return DVR_E_INVALID_ARGUMENT;
  return g_gather.exchange(mode);
}
extern "C" int dvr_get_forward_gather(void) { return g_gather.load(); }
extern "C" int dvr_last_adjoint_path(void) { return g_adjoint_path; }
