// Launchers of the ray-marcher kernel families (host-callable, no torch).
// Each TF mode's kernels live in their own translation unit so the build
// compiles them in parallel; dvr_host.cu dispatches on the TF mode.
#pragma once
#include <cuda_runtime.h>
#include "diffdvr_gb300.h"
#include "dvr_params.h"

namespace dvr {

// Viewport derivatives are summed per batch entry in shared memory: at most
// this many entries (9 floats each).
constexpr int kMaxViewportBatch = 256;

// Which adjoint kernels the last call on this thread launched (DvrAdjointPath)
// and the window-adjoint switch (dvr_set_window_adjoint).
int& last_adjoint_path();
bool window_adjoint_on();
// The forward's corner-gather mode (DvrForwardGather, dvr_set_forward_gather).
int forward_gather_mode();

struct LaunchInfo {
  int num_sms;
  int max_smem_optin;  // cudaDevAttrMaxSharedMemoryPerBlockOptin
  int device;
};

// Zeroed counters for one persistent launch on stream s: 16 bytes, 16-byte
// aligned (int [0] = ray counter, bytes 8..15 = a 64-bit counter), from a
// per-device pool owned by the library (allocated on first use, so make the
// first call on a device before capturing a stream into a CUDA graph).
int* acquire_counter(int device, cudaStream_t s, cudaError_t& err);

// Scratch memory of at least `bytes` for launches on stream s, owned by the
// library and reused by later launches on the same stream (grown on demand;
// growing synchronises the stream).  Not zeroed.  Slots are independent
// buffers (0: ray order and TF-gradient slices, 1: cell-corner volume or the
// gather texture's staging image, 2: the adjoint's cell-corner gradient).
void* acquire_scratch(int device, cudaStream_t s, size_t bytes, cudaError_t& err, int slot = 0);

// A 2D CUDA array of W x H texels (format, TexelFormat of dvr_cells.cuh:
// 0 float, 1 half, 2 unsigned 16-bit) created with the gather flag, and its
// texture object (point filtering, clamped unnormalised coordinates, element
// reads: half texels arrive as float) and, where the array takes surface
// stores as well, its surface object (else surf = 0), owned by the library
// and reused by later launches on stream s while size and format stay the
// same (replacing it synchronises the stream).
cudaError_t acquire_gather_texture(int device, cudaStream_t s, int W, int H, int format, cudaArray_t& array,
                                   cudaTextureObject_t& tex, cudaSurfaceObject_t& surf);

// Scratch handed in by the caller instead of the library's pools: `counter`
// (one int, zeroed here on the stream before each launch) and `tf` (TF-gradient
// slices of R*C floats per block, zeroed by the kernel; tf_bytes bytes).
struct CallerScratch {
  int* counter;
  float* tf;
  size_t tf_bytes;
};

// Longest-first ray order for the persistent kernels: ray ids bucketed by
// descending sample count (the forward's termination index for the adjoint,
// a = its parameters; the sample bound of the ray for the forward, a =
// nullptr).  scratch holds work_order_ints(p) ints; the ordered list starts at
// scratch + work_order_list_offset, and scratch[work_order_count_offset] is
// the number of rays with samples, which come first.  The forward ordering
// also finishes the rays without samples (zero outputs).
constexpr size_t work_order_count_offset = 512;
constexpr size_t work_order_list_offset = 516;
size_t work_order_ints(const RenderParams& p);
cudaError_t order_rays_by_work(const RenderParams& p, const AdjointParams* a, int* scratch, const LaunchInfo& li,
                               cudaStream_t s);

// Adds the cell-corner volume gradient cell_grad (AdjointParams::cell_grad,
// vb volume batch entries of X*Y*Z cells) to adj_volume (dvr_cellgrad.cu).
cudaError_t fold_cell_grad(const float* cell_grad, const OutView& adj_volume, int X, int Y, int Z, int vb,
                           const LaunchInfo& li, cudaStream_t s);

// Plain family (reference semantics).
template <int TF>
cudaError_t launch_plain_forward(const RenderParams& p, int filter, int blend, const LaunchInfo& li, cudaStream_t s);
template <int TF>
cudaError_t launch_plain_adjoint(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                 const LaunchInfo& li, cudaStream_t s);

// Optimized family.
template <int TF>
cudaError_t launch_fast_forward(const RenderParams& p, int filter, int blend, const LaunchInfo& li, cudaStream_t s);
template <int TF>
cudaError_t launch_fast_adjoint(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                const LaunchInfo& li, cudaStream_t s);
// The optimized adjoint on caller-provided scratch: allocates nothing.  The
// persistent grid is capped to the blocks whose TF slices fit in sc.tf_bytes.
template <int TF>
cudaError_t launch_fast_adjoint_into(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                     const LaunchInfo& li, const CallerScratch& sc, cudaStream_t s);

// Pre-shaded volumes (4 x X x Y x Z colour/absorption).  Forward: the
// reference's one thread per ray (plain) or one warp per ray; adjoint: one
// thread per ray with blend inversion, the reference's position and
// step-size adjoints (exact = false) or the exact ones (exact = true).
cudaError_t launch_preshaded_forward(const RenderParams& p, int blend, bool plain, const LaunchInfo& li,
                                     cudaStream_t s);
cudaError_t launch_preshaded_adjoint(const RenderParams& p, const AdjointParams& a, int blend, bool exact,
                                     const LaunchInfo& li, cudaStream_t s);

cudaError_t launch_preshade_volume(const PreshadeParams& q, int tf_mode, bool adjoint, const LaunchInfo& li,
                                   cudaStream_t s);

// Forward-mode derivatives: blocks of kFwdThreads (one ray per warp at a
// time), one launch per range of at most kFwdMaxPass derivative indices
// (g.d0, g.dn); each warp holds its ray's dn x 4 Jacobian block in shared
// memory.
constexpr int kFwdThreads = 128;
constexpr int kFwdMaxPass = 1024;
template <int TF>
cudaError_t launch_forward_gradients(const RenderParams& p, const FwdGradParams& g, int filter, int blend,
                                     const LaunchInfo& li, cudaStream_t s);
cudaError_t launch_forward_variables_to_gradients(const FwdVarsParams& v, const LaunchInfo& li, cudaStream_t s);

}  // namespace dvr
