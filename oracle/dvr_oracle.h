/*
 * Oracle interface — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of DiffDVR's forward and adjoint volume ray marcher, used
 * as the checker for the CUDA kernels of diffdvr_gb300.  Nothing in the
 * product links, imports or executes code from this directory; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
 *
 * Two libraries implement this interface:
 *   libdvr_oracle_{f32,f64}.so  our plain-C restatement (dvr_oracle.c), builds
 *                               anywhere (x86 container and the Arm GPU host);
 *   _ref/libdvr_ref_{f32,f64}.so  the reference's own DvrKernel*Host templates
 *                               compiled from its headers (ref_harness.cpp),
 *                               only where the reference sources are present.
 * Both take identical arguments so the Python wrapper (oracle.py) can call
 * either one and the tests can pin the restatement to the reference.  The
 * reference's CUDA kernels, compiled from the same headers into
 * _ref/ref_kernels_sm103a.cubin (ref_device.cu), take the same structs on
 * the GPU (ref_cuda.py).
 *
 * All real-valued buffers hold `real_t` = float (f32 build) or double (f64
 * build).  Tensors follow the reference memory layout
 * (renderer/renderer_settings.cuh:8-45); a dimension of size 1 is broadcast
 * (stride treated as 0), as BroadcastingTensorAccessor32 does
 * (renderer/renderer_tensor.cuh:140-144).
 */
#ifndef DVR_ORACLE_H
#define DVR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleTensor {
  void* data;          /* real_t* (or int32_t* for termination indices) */
  int32_t ndim;
  int32_t pad_;
  int64_t sizes[5];
  int64_t strides[5];  /* in elements */
} OracleTensor;

/* Enum values are those of renderer/renderer_settings.cuh:81-146; filter 3
 * (pre-shaded) goes with TF 5 (pre-shaded) and a 4 X Y Z volume. */
typedef struct OracleInputs {
  int32_t width, height;
  int32_t filter_mode;   /* 0 nearest, 1 trilinear, 3 pre-shaded */
  int32_t camera_mode;   /* 0 ray start/dir, 1 inverse view matrix, 2 reference frame */
  int32_t tf_mode;       /* 0 identity, 1 texture, 2 linear, 3 gaussian, 5 pre-shaded */
  int32_t blend_mode;    /* 0 Beer-Lambert, 1 alpha */
  OracleTensor volume;        /* (B) X Y Z */
  OracleTensor box_min;       /* (B) 3 */
  OracleTensor box_size;      /* (B) 3 */
  OracleTensor ray_start;     /* (B) H W 3   (camera_mode 0) */
  OracleTensor ray_dir;       /* (B) H W 3   (camera_mode 0) */
  OracleTensor camera_matrix; /* (B) 4 4 (mode 1) or (B) 3 3 (mode 2) */
  double fov_y_radians;       /* camera_mode 2 */
  OracleTensor step_size;     /* (B) (H) (W) */
  OracleTensor tf;            /* (B) R C */
  double blending_early_out;
  int32_t batch;              /* resolved broadcast batch size B */
  int32_t pad_;
} OracleInputs;

typedef struct OracleAdjointOutputs {
  int32_t has_volume, has_stepsize, has_camera, has_tf;
  int32_t stepsize_broadcast, camera_broadcast;
  OracleTensor adj_volume;     /* (B) X Y Z */
  OracleTensor adj_stepsize;   /* (B) (H) (W) */
  OracleTensor adj_ray_start;  /* (B) H W 3 */
  OracleTensor adj_ray_dir;    /* (B) H W 3 */
  OracleTensor adj_tf;         /* (B) R C */
} OracleAdjointOutputs;

/* Forward-mode derivative indices (renderer/renderer_settings.cuh:189-206):
 * -1 = not traced, else an index in [0, D). */
typedef struct OracleForwardSettings {
  int32_t D;
  int32_t d_stepsize;
  int32_t d_ray_start[3];
  int32_t d_ray_dir[3];
  int32_t has_tf;
  int32_t pad_;
  OracleTensor d_tf;           /* int32 (B) R C */
} OracleForwardSettings;

/* Returns 0 on success, nonzero for an unsupported mode combination. */
int oracle_forward(const OracleInputs* in, OracleTensor* color, OracleTensor* termination);
int oracle_adjoint(const OracleInputs* in, const OracleTensor* color,
                   const OracleTensor* termination, const OracleTensor* adj_color,
                   OracleAdjointOutputs* out);
/* Forward march with forward-mode derivatives: color, termination and
 * gradients B H W D 4 (d color / d variable) — renderForwardGradients. */
int oracle_forward_gradients(const OracleInputs* in, const OracleForwardSettings* fs, OracleTensor* color,
                             OracleTensor* termination, OracleTensor* gradients);
/* Contracts forward variables B H W D 4 with adj_color B H W 4 into the
 * enabled adjoint outputs (stepsize, camera, TF) — forwardVariablesToGradients. */
int oracle_forward_variables_to_gradients(const OracleTensor* forward_variables, const OracleTensor* adj_color,
                                          const OracleForwardSettings* fs, OracleAdjointOutputs* out);
/* Port only: pre-shading of a density volume (1 X Y Z) into a colour volume
 * (4 X Y Z) with the TF of batch entry 0, and its adjoint (d loss / d
 * density, written) — TFUtils::preshadeVolume. */
int oracle_preshade_volume(const OracleTensor* density, const OracleTensor* tf, int tf_mode, OracleTensor* color);
int oracle_preshade_volume_adjoint(const OracleTensor* density, const OracleTensor* tf, int tf_mode,
                                   const OracleTensor* adj_color, OracleTensor* adj_density);
/* Port only: the pre-shaded position adjoint follows the reference (0,
 * default) or is the exact trilinear derivative (1). */
void oracle_set_exact_preshaded(int exact);
/* Size of real_t in this build (4 or 8). */
int oracle_real_size(void);
int oracle_set_threads(int n);

#ifdef DVR_ORACLE_HAS_REAL_T
/* Port only: one step of each part of the march, as the march computes it,
 * for per-component adjoint tests.  Vectors are real_t[4] (r, g, b, opacity
 * or absorption) or real_t[3]; TFs and volumes are batch entry 0.
 * blend: the accumulator after compositing `cur` over `acc`.  Its adjoint
 * inverts the blend (acc_in, from acc_out) and maps the accumulator's adjoint
 * to those of acc_in, cur and the step size (the latter ASSIGNED, as the
 * reference's blend adjoint does). */
int oracle_blend_step(int mode, const real_t* acc, const real_t* cur, real_t step, real_t* out);
int oracle_blend_step_adjoint(int mode, const real_t* acc_out, const real_t* cur, real_t step, const real_t* adj_out,
                              real_t* acc_in, real_t* adj_acc_in, real_t* adj_cur, real_t* adj_step);
/* TF evaluation at one density, and its adjoint: d/d density returned in
 * *adj_density, TF gradient accumulated into adj_tf (skipped when null). */
int oracle_tf_step(const OracleTensor* tf, int tf_mode, real_t density, real_t* out);
int oracle_tf_step_adjoint(const OracleTensor* tf, int tf_mode, real_t density, const real_t* adj, OracleTensor* adj_tf,
                           real_t* adj_density);
/* One volume sample at a position in voxel coordinates (filter 0 nearest,
 * 1 trilinear), and its adjoint: d/d position written to adj_pos, volume
 * gradient accumulated into adj_volume (skipped when null). */
int oracle_sample_step(const OracleTensor* volume, int filter, const real_t* pos, real_t* density);
int oracle_sample_step_adjoint(const OracleTensor* volume, int filter, const real_t* pos, real_t adj_density,
                               real_t* adj_pos, OracleTensor* adj_volume);
/* The ray (start, direction; B H W 3 each) of every pixel, as the march
 * computes it for the inputs' camera mode. */
int oracle_camera_rays(const OracleInputs* in, OracleTensor* start, OracleTensor* dir);
/* The n sample positions (start + t*dir - box_min) / voxel, t = tmin + k*step,
 * of one ray (pos: n x 3), and their adjoint for the ray start, direction and
 * step size (tmin held fixed, as in the march). */
int oracle_ray_steps(const real_t* start, const real_t* dir, const real_t* box_min, const real_t* voxel, real_t tmin,
                     real_t step, int n, real_t* pos);
int oracle_ray_steps_adjoint(const real_t* start, const real_t* dir, const real_t* box_min, const real_t* voxel,
                             real_t tmin, real_t step, int n, const real_t* adj_pos, real_t* adj_start, real_t* adj_dir,
                             real_t* adj_step);
#endif

#ifdef __cplusplus
}
#endif
#endif
