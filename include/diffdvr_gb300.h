/*
 * diffdvr_gb300 — C ABI of the GB300 (sm_103a) differentiable volume ray marcher.
 *
 * Plain C: raw pointers, sizes and element strides; no torch types.  Every
 * entry point returns DVR_OK (0) or a negative DVR_E* code and never throws;
 * the message of the last failure on the calling thread is returned by
 * dvr_last_error().  Launches are asynchronous on the given CUDA stream
 * (NULL = legacy default stream), like the reference, which launches on the
 * PyTorch current stream (renderer/renderer_cuda.cpp:105, :304).
 *
 * Layout contract (renderer/renderer_settings.cuh:8-45); a bracketed leading
 * dimension may be 1 and is then broadcast over the batch:
 *   volume            (B) X Y Z            density
 *   box_min, box_size (B) 3
 *   camera            (B) H W 3 ray start + (B) H W 3 ray direction, or
 *                     (B) 4 4 inverse view-projection, or
 *                     (B) 3 3 reference frame (eye, right, up) + fovY
 *   step_size         (B) (H) (W)
 *   tf                (B) R C, C = 2 identity, 4 texture, 5 linear, 6 Gaussian
 *   pre-shaded volume 4 X Y Z              (filter and TF mode Preshaded: r, g,
 *                     b, absorption per voxel, shared by all batch entries;
 *                     the TF is not read; volume gradient 4 X Y Z)
 *   color             B H W 4              output (r, g, b, alpha)
 *   termination_index B H W int32          output
 * Gradient outputs are accumulated with atomics and must be zero-initialised
 * by the caller (renderer/renderer_settings.cuh:227-229).
 *
 * Storage types: every real-valued tensor is float32, except that the volume
 * and the TF may also be float16 or bfloat16 (sampled and blended in FP32);
 * gradients are always float32.  All tensors must live on the same CUDA device.
 */
#ifndef DIFFDVR_GB300_H
#define DIFFDVR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DVR_ABI_VERSION 6

/* ---- status codes ---- */
#define DVR_OK 0
#define DVR_E_INVALID_ARGUMENT (-1) /* a shape, dtype, device or mode check failed (TORCH_CHECK in the reference) */
#define DVR_E_NO_GRADIENT (-2)      /* adjoint with no gradient enabled (renderer/renderer.cpp:712-717) */
#define DVR_E_UNSUPPORTED (-3)      /* mode or dtype this build does not implement */
#define DVR_E_CUDA (-4)             /* a CUDA runtime call or launch failed */

/* ---- enums: values equal to the reference's (renderer/renderer_settings.cuh:81-146) ---- */
enum DvrVolumeFilterMode { DVR_FILTER_NEAREST = 0, DVR_FILTER_TRILINEAR = 1, DVR_FILTER_PRESHADED = 3 };
enum DvrCameraMode { DVR_CAMERA_RAY_START_DIR = 0, DVR_CAMERA_INVERSE_VIEW_MATRIX = 1, DVR_CAMERA_REFERENCE_FRAME = 2 };
enum DvrTFMode {
  DVR_TF_IDENTITY = 0, DVR_TF_TEXTURE = 1, DVR_TF_LINEAR = 2, DVR_TF_GAUSSIAN = 3,
  DVR_TF_PRESHADED = 5, DVR_TF_GAUSSIAN_LOG = 6
};
enum DvrBlendMode { DVR_BLEND_BEER_LAMBERT = 0, DVR_BLEND_ALPHA = 1 };

enum DvrDType { DVR_FLOAT32 = 0, DVR_FLOAT64 = 1, DVR_FLOAT16 = 2, DVR_BFLOAT16 = 3, DVR_INT32 = 4 };
enum DvrDeviceType { DVR_DEVICE_CPU = 0, DVR_DEVICE_CUDA = 1 };

/* Kernel family used by dvr_render_forward / dvr_render_adjoint.
 *  DVR_KERNELS_PLAIN:     one thread per ray, reference semantics throughout
 *                         (adjoint recovers the accumulator by inverting the
 *                         blend, renderer/renderer_blending.cuh:75-77).
 *  DVR_KERNELS_OPTIMIZED: tiled ray order, FP16/BF16 volume storage, TF in
 *                         shared memory, pre-aggregated gradient scatters and,
 *                         when the forward pass was given a checkpoint buffer,
 *                         a checkpointed adjoint that recomputes each segment
 *                         instead of inverting the blend.  Default. */
enum DvrKernelFamily { DVR_KERNELS_PLAIN = 0, DVR_KERNELS_OPTIMIZED = 1 };

/* A strided tensor view.  ndim < 0 marks an absent (undefined) tensor.
 * strides are in elements. */
typedef struct DvrTensor {
  void* data;
  int32_t ndim;
  int32_t dtype;         /* DvrDType */
  int32_t device_type;   /* DvrDeviceType */
  int32_t device_index;
  int64_t sizes[5];
  int64_t strides[5];
} DvrTensor;

/* Which alternative a host-side variant field holds. */
enum DvrValueKind { DVR_KIND_TENSOR = 0, DVR_KIND_VALUE = 1 };
enum DvrCameraKind {
  DVR_CAMERA_PER_PIXEL_RAYS = 0,           /* CameraPerPixelRays{ray_start, ray_dir} */
  DVR_CAMERA_INVERSE_VIEW_TENSOR = 1,      /* B*4*4 tensor */
  DVR_CAMERA_INVERSE_VIEW_VALUE = 2,       /* one 4x4 matrix by value (glm::mat4) */
  DVR_CAMERA_REFERENCE_FRAME_KIND = 3      /* CameraReferenceFrame{viewport B*3*3, fovY} */
};

/* Mirrors renderer::RendererInputsHost (renderer/renderer.h:20-64).  Each
 * std::variant of the reference becomes a kind tag plus both alternatives. */
typedef struct DvrRendererInputs {
  int32_t screen_width;          /* screenSize.x = W */
  int32_t screen_height;         /* screenSize.y = H */
  int32_t volume_filter_mode;    /* DvrVolumeFilterMode */
  int32_t camera_mode;           /* DvrCameraMode */
  int32_t tf_mode;               /* DvrTFMode */
  int32_t blend_mode;            /* DvrBlendMode */
  DvrTensor volume;
  int32_t box_min_kind;          /* DvrValueKind */
  int32_t box_size_kind;
  DvrTensor box_min;
  DvrTensor box_size;
  double box_min_value[3];
  double box_size_value[3];
  int32_t camera_kind;           /* DvrCameraKind */
  int32_t step_size_kind;        /* DvrValueKind */
  DvrTensor camera_ray_start;
  DvrTensor camera_ray_dir;
  DvrTensor camera_matrix;       /* B*4*4 or B*3*3 */
  float camera_matrix_value[16]; /* rows of the 4x4 matrix as the kernel reads them
                                    (= the column-major storage of a glm::mat4) */
  double camera_fov_y_radians;
  DvrTensor step_size;
  double step_size_value;
  DvrTensor tf;
  double blending_early_out;     /* default 1 - 1e-5 */
} DvrRendererInputs;

/* Mirrors renderer::RendererOutputsHost (renderer/renderer.h:67-71), plus
 * state the forward pass records for the optimized adjoint (ndim < 0 when
 * absent):
 *  - checkpoints: B*H*W*C float32, the accumulated opacity every
 *    `checkpoint_interval` samples.  C >= ceil(max samples per ray / interval) - 1.
 *  - sample_density + sample_offset (both or neither; need checkpoints,
 *    except with pre-shaded volumes): a
 *    1-D float32 pool of any size N (16-byte aligned, contiguous, N >= 4) and
 *    a B*H*W int32 tensor.  The forward stores, for every sample k of a ray,
 *    the density and the opacity accumulated in front of the sample as floats
 *    2k and 2k+1 of the ray's run in the pool (rays claim room in launch
 *    order, a multiple of 4 floats each) and writes the run's first float
 *    index / 4 to sample_offset, or -1 when the pool was full.  The adjoint
 *    then reads these instead of re-sampling the volume and re-marching from
 *    checkpoints; rays with offset -1 re-sample.  Checkpoints are written
 *    only for the rays without a record.  With pre-shaded volumes the first
 *    float of a pair is the sample's alpha (there is no density), and the
 *    adjoint reads the record when the image has few rays.  N = B*H*W*S with
 *    S = 4 * dvr_checkpoint_slots(length, step, 2) holds every ray.
 *    Written and read by the optimized entry points.  The batched entry
 *    points give every ray a fixed run of the pool instead of claiming room
 *    in launch order: pool / (B*H*W) groups of 4 floats, in pixel order;
 *    rays with more samples than that get offset -1; they write checkpoints
 *    for every ray. */
typedef struct DvrRendererOutputs {
  DvrTensor color;
  DvrTensor termination_index;
  DvrTensor checkpoints;
  int32_t checkpoint_interval;   /* samples between checkpoints; 0 = default (32) */
  int32_t pad_;
  DvrTensor sample_density;
  DvrTensor sample_offset;
} DvrRendererOutputs;

/* Mirrors renderer::AdjointOutputsHost (renderer/renderer.h:95-111). */
typedef struct DvrAdjointOutputs {
  int32_t has_volume_derivatives;
  int32_t has_stepsize_derivatives;
  int32_t has_camera_derivatives;
  int32_t has_tf_derivatives;
  int32_t tf_delayed_accumulation;
  int32_t pad_;
  DvrTensor adj_volume;          /* (B) X Y Z */
  DvrTensor adj_stepsize;        /* (B) (H) (W) */
  DvrTensor adj_camera_ray_start;/* (B) H W 3 */
  DvrTensor adj_camera_ray_dir;  /* (B) H W 3 */
  DvrTensor adj_tf;              /* (B) R C */
  /* Gradient of the reference-frame camera's viewport (rows eye, right, up),
   * (B) 3 3, accumulated: the rays are generated from the viewport inside the
   * kernel (renderer/camera_impl.cu:17-36) and each ray's start/direction
   * adjoint is carried back through that generation.  Needs cameraMode ==
   * ReferenceFrame and the optimized single-instance entry points; the
   * reference gets this gradient by materialising per-pixel rays and
   * differentiating their generation separately. */
  int32_t has_viewport_derivatives;
  int32_t pad2_;
  DvrTensor adj_viewport;
} DvrAdjointOutputs;

/* Forward rendering without gradients.
 * Replaces renderer::Renderer::renderForward (renderer/renderer.h:159-161,
 * renderer/renderer.cpp:393-417).
 * Library scratch: the optimized family takes work counters and, per
 * stream, a ray-order buffer (and, for trilinear filtering, the cell-corner
 * volume or the slab gather texture) from pools that
 * it grows with cudaMalloc when a call needs more than they hold;
 * dvr_render_adjoint does the same for its ray order, TF-gradient slices,
 * the gather texture of the rays it marches again and the cell-corner
 * volume-gradient buffer.  cudaMalloc is not allowed while a stream is being
 * captured into a CUDA graph, so make one call of the same sizes on the same
 * stream before capturing it; later calls reuse the pools and allocate
 * nothing. */
int dvr_render_forward(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs, void* cuda_stream);

/* Adjoint (backward) rendering: traces adj_color (B*H*W*4) back through the
 * march and accumulates into the enabled gradient outputs.
 * Replaces renderer::Renderer::renderAdjoint (renderer/renderer.h:264-268,
 * renderer/renderer.cpp:660-742). */
int dvr_render_adjoint(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs_from_forward,
                       const DvrTensor* adj_color, const DvrAdjointOutputs* adj_outputs, void* cuda_stream);

/* The optimized adjoint of dvr_render_adjoint (same arguments, validation,
 * errors and results) for callers that cannot let a library allocate device
 * memory: applications whose own allocator owns the device or that run under
 * a hard memory budget, and render loops that must not stall on cudaMalloc's
 * implicit synchronisation.  dvr_render_adjoint grows internal scratch pools
 * with cudaMalloc; this entry point allocates nothing and uses a static
 * 4 MiB device array per device instead (one work counter, zeroed on the
 * stream before each launch, and per-block TF-gradient slices that the kernel
 * zeroes itself).
 * Limit: with has_tf_derivatives, R x C x 4 bytes x (SM count) must fit in
 * 4 MiB - 256 bytes (R = TF control points, C = channels), i.e. R x C <= 6898
 * on a 152-SM GPU; larger TFs are rejected with DVR_E_INVALID_ARGUMENT.
 * Volume and image sizes are not limited.  The kernel-family switch does not
 * apply.  The first call on a device resolves the array's address and keeps
 * it for the life of the process; make it before capturing the stream into a
 * CUDA graph, and do not call this entry point on a device after
 * cudaDeviceReset there (the reset destroys the context the address belongs
 * to).  All calls on one device share the array: calls that may overlap
 * (other streams or host threads) race, so the caller serialises them.
 * No counterpart in the reference. */
int dvr_render_adjoint_noalloc(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs_from_forward,
                               const DvrTensor* adj_color, const DvrAdjointOutputs* adj_outputs,
                               void* cuda_stream);

/* Batched rendering of n independent instances, each with its own volume
 * size, image size, camera and TF, in ONE persistent launch over a work list
 * of (instance, view, tile) items.  All instances share the filter, TF and
 * blend modes and the volume storage dtype.  Extends the reference, whose
 * batches must share the volume and image sizes (renderer/renderer.cpp:59-70).
 * Up to 24 instances go into one launch whose kernel parameter carries their
 * descriptors (more instances: several launches); nothing is copied or
 * allocated, so the calls can be captured into a CUDA graph and replayed. */
int dvr_render_forward_batched(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs, int32_t n,
                               void* cuda_stream);
int dvr_render_adjoint_batched(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs_from_forward,
                               const DvrTensor* adj_colors, const DvrAdjointOutputs* adj_outputs, int32_t n,
                               void* cuda_stream);

/* Tile shapes of the batched launches: one block of 128 rays per tile, every
 * warp an 8x4 pixel patch, the four warps side by side (16x8: 2x2, 32x4: 4x1,
 * 8x16: 1x4). */
enum DvrTileShape { DVR_TILE_16x8 = 0, DVR_TILE_32x4 = 1, DVR_TILE_8x16 = 2 };
/* dvr_render_forward_batched / dvr_render_adjoint_batched with a tile shape
 * per instance: tile_shapes holds n DvrTileShape values (NULL = 16x8 for
 * every instance), for example chosen per size class by the autotuner of
 * the Python package (diffdvr_gb300.autotune).  No counterpart in the
 * reference, whose only launch tuning is an occupancy-based block size
 * (renderer/renderer_cuda.cpp:97-108). */
int dvr_render_forward_batched_tiled(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs,
                                     const int32_t* tile_shapes, int32_t n, void* cuda_stream);
int dvr_render_adjoint_batched_tiled(const DvrRendererInputs* inputs, const DvrRendererOutputs* outputs_from_forward,
                                     const DvrTensor* adj_colors, const DvrAdjointOutputs* adj_outputs,
                                     const int32_t* tile_shapes, int32_t n, void* cuda_stream);

/* Mirrors renderer::ForwardDifferencesSettingsHost (renderer/renderer.h:73-93):
 * which variables forward-mode differentiation traces, each given the index
 * of its derivative in [0, D); -1 = not traced. */
typedef struct DvrForwardDifferencesSettings {
  int32_t D;                     /* number of derivatives */
  int32_t d_stepsize;            /* the step size */
  int32_t d_ray_start[3];        /* ray start x, y, z (after ray generation, any camera mode) */
  int32_t d_ray_dir[3];          /* ray direction x, y, z */
  int32_t has_tf_derivatives;    /* nonzero: d_tf holds TF derivative indices */
  int32_t pad_;
  DvrTensor d_tf;                /* int32, the TF's shape (B) R C: index of each TF entry, -1 = not traced */
} DvrForwardDifferencesSettings;
/* Forward rendering with forward-mode derivatives: writes color, termination
 * index and gradients_out (B*H*W*D*4 float32, d color / d variable; no
 * zeroing needed).  Any D; volume derivatives are not available in forward
 * mode.  The checkpoint and sample-record fields of outputs are ignored.
 * Replaces renderer::Renderer::renderForwardGradients
 * (renderer/renderer.h:192-196, renderer/renderer.cpp:419-498). */
int dvr_render_forward_gradients(const DvrRendererInputs* inputs, const DvrForwardDifferencesSettings* settings,
                                 const DvrRendererOutputs* outputs, const DvrTensor* gradients_out,
                                 void* cuda_stream);
/* Contracts forward variables (B*H*W*D*4, from dvr_render_forward_gradients)
 * with the colour adjoint (B*H*W*4): per pixel, the gradient of each traced
 * variable is dot(adj_color, d color / d variable).  Step-size and camera
 * gradients are written per pixel (accumulated where the output broadcasts
 * over a dimension), TF gradients are accumulated (zero-initialise adj_tf).
 * Volume and viewport derivatives are rejected.
 * Replaces renderer::Renderer::forwardVariablesToGradients
 * (renderer/renderer.h:212-216, renderer/renderer.cpp:500-558). */
int dvr_forward_variables_to_gradients(const DvrTensor* forward_variables, const DvrTensor* adj_color,
                                       const DvrForwardDifferencesSettings* settings,
                                       const DvrAdjointOutputs* adj_outputs, void* cuda_stream);
/* Pre-shading: the colour volume color_out (4*X*Y*Z float32: r, g, b,
 * absorption) of a density volume (1*X*Y*Z float32) through the TF (1*R*C
 * float32) of mode tf_mode, for rendering with the pre-shaded filter and TF
 * modes (volume = color_out).  The adjoint writes d loss / d density
 * (1*X*Y*Z) for the colour-volume adjoint adj_color (4*X*Y*Z); there is no
 * TF gradient, as in the reference.
 * Replace renderer::TFUtils::preshadeVolume and its autograd backward
 * (renderer/tf_utils.h:125-140, renderer/tf_utils.cpp:173-249). */
int dvr_preshade_volume(const DvrTensor* density, const DvrTensor* tf, int32_t tf_mode, const DvrTensor* color_out,
                        void* cuda_stream);
int dvr_preshade_volume_adjoint(const DvrTensor* density, const DvrTensor* tf, int32_t tf_mode,
                                const DvrTensor* adj_color, const DvrTensor* adj_density, void* cuda_stream);
/* Number of checkpoint slots per ray (the C of DvrRendererOutputs.checkpoints)
 * for rays of at most max_ray_length world units inside the box (the box
 * diagonal bounds it) marched with steps of at least min_step_size, at the
 * given interval (0 = default).  Host-only; returns a negative DVR_E* code for
 * invalid arguments. */
int64_t dvr_checkpoint_slots(double max_ray_length, double min_step_size, int32_t checkpoint_interval);

/* Message of the last failed call on this thread ("" if none). */
const char* dvr_last_error(void);

/* Kernel family selection (process-wide).  Returns the previous value. */
int dvr_set_kernel_family(int32_t family);
int dvr_get_kernel_family(void);

/* Volume gradients from the sample record: nonzero = the window adjoint
 * (tiles of rays walked back to front in slabs of equal ray distance, each
 * slab's volume gradient accumulated in shared memory and added to global
 * memory once per touched group of four voxels, the volume staged in shared
 * memory by bulk copies where camera or step-size gradients need corner
 * densities), 0 = the general per-ray adjoint, which scatters with atomics on
 * every cell exit as the reference does.  Default 0: the window adjoint cuts
 * the L2 reduction traffic about eightfold but measured slower on GB300 (it
 * is latency-bound).  Process-wide.  Returns the previous value.  No
 * counterpart in the reference. */
int dvr_set_window_adjoint(int32_t enable);
int dvr_get_window_adjoint(void);

/* How the optimized single-instance forward reads the eight corners of a
 * trilinear sample (DvrForwardGather).  Process-wide.  Returns the previous
 * value, or DVR_E_INVALID_ARGUMENT for an unknown mode.  No counterpart in the
 * reference (its kernels load the corners directly). */
enum DvrForwardGather {
  DVR_GATHER_AUTO = 0,    /* the mode measured fastest for the volume's size:
                             CELLS when the cell records fit in 64 MB, else
                             TEXTURE (CELLS or DIRECT beyond its limits) */
  DVR_GATHER_DIRECT = 1,  /* eight loads from the volume */
  DVR_GATHER_CELLS = 2,   /* one 16-byte cell record per sample, built per call */
  DVR_GATHER_TEXTURE = 3  /* two tex2Dgather fetches per sample from the slab
                             texture, built per call; AUTO/DIRECT where the
                             slabs do not fit the texture's size limits */
};
int dvr_set_forward_gather(int32_t mode);
int dvr_get_forward_gather(void);

/* Which kernels the last dvr_render_adjoint call on the calling thread ran
 * (DvrAdjointPath).  No counterpart in the reference. */
enum DvrAdjointPath {
  DVR_PATH_NONE = 0,     /* no call yet, or the call failed before launching */
  DVR_PATH_PLAIN = 1,    /* plain family */
  DVR_PATH_GENERAL = 2,  /* general per-ray kernel (checkpoints or blend inversion) */
  DVR_PATH_RECORD = 3,   /* record kernel (TF gradient of a texture TF from the sample record) */
  DVR_PATH_WINDOW = 4,   /* window kernel (volume gradient from the sample record) */
  DVR_PATH_PRESHADED = 5, /* pre-shaded kernels */
  DVR_PATH_REMARCH = 6   /* re-march kernel (TF gradient of a texture TF from the
                            checkpoints alone: chunks re-marched into shared memory) */
};
int dvr_last_adjoint_path(void);

/* In sync mode every launch is followed by cudaStreamSynchronize and a launch
 * error check, for debugging (renderer::Renderer::setCudaSyncMode,
 * renderer/renderer.h:147-149).  Returns the previous value. */
int dvr_set_sync_mode(int32_t sync);
int dvr_get_sync_mode(void);

/* ABI version of the loaded library (DVR_ABI_VERSION). */
int dvr_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* DIFFDVR_GB300_H */
