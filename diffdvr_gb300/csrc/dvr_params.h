// Kernel-side parameter blocks of the ray marcher (host and device).
//
// The host layer (dvr_host.cu) validates the C-ABI descriptors and flattens
// them into these PODs: element strides with the broadcast rule already
// applied (a dimension of size 1 gets stride 0, as the reference's
// BroadcastingTensorAccessor32 does, renderer/renderer_tensor.cuh:140-144),
// and scalar settings carried by value instead of as temporary tensors.
#pragma once
#include <stdint.h>

namespace dvr {

enum StorageType : int32_t { kF32 = 0, kF16 = 2, kBF16 = 3 };

// A (B) * ... real-valued input.  p == nullptr means "use val" (a setting
// given by value, broadcast over everything).
struct InView {
  const void* p;
  int64_t s[4];
  float val[3];
  int32_t pad_;
};

struct OutView {
  void* p;
  int64_t s[4];
};

struct RenderParams {
  int32_t W, H, B;              // screen size and resolved batch
  int32_t camera_mode;          // 0 rays, 1 inverse view matrix, 2 reference frame
  int32_t X, Y, Z;              // volume resolution
  int32_t R, C;                 // TF control points and channels
  int32_t vol_storage, tf_storage;
  float fov_y;                  // camera_mode 2
  float early_out;              // blendingEarlyOut
  int32_t pad0_;
  float cam_value[16];          // camera_mode 1 given by value: rows of the 4x4 matrix
  InView volume;                // [b][x][y][z]
  InView box_min, box_size;     // [b][i]
  InView ray_start, ray_dir;    // [b][y][x][i]
  InView cam;                   // [b][r][c]
  InView step;                  // [b][y][x]
  InView tf;                    // [b][r][c]
  OutView color;                // [b][y][x][c]
  OutView term;                 // [b][y][x] int32
  // checkpointed adjoint (optimized kernels); ckpt.p == nullptr when absent
  OutView ckpt;                 // [b][y][x][j] float, transmittance before sample (j+1)*K
  int32_t ckpt_slots;           // C slots per ray
  int32_t ckpt_interval;        // K
  // per-sample density record (optimized kernels); dens == nullptr when absent
  float* dens;                  // pool of dens_units groups of 4 floats, 16-byte aligned
  OutView dens_off;             // [b][y][x] int32: first group of the ray's densities, -1 = not recorded
  int64_t dens_units;
};

struct AdjointParams {
  InView fwd_color;             // [b][y][x][c]
  InView fwd_term;              // [b][y][x] int32 (read as int)
  InView adj_color;             // [b][y][x][c]
  int32_t has_volume, has_stepsize, has_camera, has_tf;
  int32_t stepsize_broadcast, camera_broadcast, tf_delayed;
  int32_t pad_;
  OutView adj_volume;           // [b][x][y][z]  (broadcast strides allowed)
  OutView adj_step;             // [b][y][x]
  OutView adj_start, adj_dir;   // [b][y][x][i]
  OutView adj_tf;               // [b][r][c]
  int32_t has_viewport, pad2_;
  OutView adj_viewport;         // [b][row][c], reference-frame camera (broadcast strides allowed)
  // Optional cell-corner volume gradient (general adjoint, trilinear): for
  // every volume batch entry of adj_volume and every cell (x, y, z), the
  // eight corner sums of the cell in the corner order of the trilinear
  // fetch, 8 floats per cell, z fastest; folded into adj_volume after the
  // launch.  nullptr: cells flush straight into adj_volume.
  float* cell_grad;
};

// Forward-mode derivatives (renderForwardGradients): derivative indices
// (-1 = not traced) and the forward-variable output of one launch, which
// covers the indices [d0, d0 + dn) of D.
struct FwdGradParams {
  int32_t D, d0, dn;
  int32_t d_step;
  int32_t d_start[3], d_dir[3];
  int32_t has_tf, pad_;
  const int32_t* d_tf;          // [b][r][c] (broadcast strides); nullptr when !has_tf
  int64_t dtf_s[3];
  float* grad;                  // [b][y][x][d][c]
  int64_t grad_s[5];
};

// forwardVariablesToGradients: forward variables and output adjoint in,
// enabled gradients out.  Indices are -1 or in [0, D).
constexpr int kFwdVarsThreads = 256;        // 8 warps, one pixel each at a time
constexpr int kFwdVarsSmemFloats = 12288;   // per-warp TF sums + entry indices in shared memory (48 KB), else global atomics
struct FwdVarsParams {
  int32_t B, H, W, D;
  int32_t R, C;
  int32_t has_step, has_camera, has_tf;
  int32_t step_broadcast, camera_broadcast;
  int32_t d_step, d_start[3], d_dir[3];
  int32_t pad_;
  const float* fwd;             // [b][y][x][d][c]
  int64_t fwd_s[5];
  const float* adj_color;       // [b][y][x][c]
  int64_t adj_s[4];
  float* adj_step;              // [b][y][x]
  int64_t step_s[3];
  float* adj_start;             // [b][y][x][i]
  int64_t start_s[4];
  float* adj_dir;
  int64_t dir_s[4];
  const int32_t* d_tf;          // [b][r][c]
  int64_t dtf_s[3];
  float* adj_tf;                // [b][r][c]
  int64_t tf_s[3];
};

// TFUtils::preshadeVolume: density [0][x][y][z] -> colour [c][x][y][z]
// (forward), or adj_color [c][x][y][z] -> d loss / d density [0][x][y][z]
// (adjoint, written to out).  TF [0][r][c] in float32.
struct PreshadeParams {
  int32_t X, Y, Z, R, C, pad_;
  const float* density;
  int64_t d_s[4];
  const float* tf;
  int64_t tf_s[3];
  const float* adj_color;
  int64_t a_s[4];
  float* out;
  int64_t o_s[4];
};

}  // namespace dvr
