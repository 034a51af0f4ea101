// Batched rendering of uneven instances.
//
// Instances are ordered by decreasing estimated cost (samples per ray), so the
// block scheduler starts the longest tiles first and the tail of a launch is
// made of short ones.  Up to kBatchMax instances go into one launch whose
// kernel parameter carries their descriptors and item offsets
// (BatchForwardTable / BatchAdjointTable): no staging copy, no device
// workspace, nothing for a graph replay to go stale.  Also here: the
// library's pools of work counters and per-stream scratch for the persistent
// launches.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "dvr_batch.h"
#include "dvr_fast_launch.cuh"

namespace dvr {
namespace {

// Samples per ray, from the volume diagonal in voxels and the step in voxels
// (step given by value; a step-size tensor counts as one voxel).
double cost_per_ray(const RenderParams& p) {
  const double diag = std::sqrt(double(p.X) * p.X + double(p.Y) * p.Y + double(p.Z) * p.Z);
  double step_vox = 1.0;
  if (p.step.p == nullptr && p.box_size.p == nullptr) {
    const double vx = p.box_size.val[0] / std::max(1, p.X - 1);
    if (vx > 0 && p.step.val[0] > 0) step_vox = p.step.val[0] / vx;
  }
  return diag / std::max(step_vox, 1e-3);
}

// instances in decreasing cost order
std::vector<int> cost_order(const RenderParams* ps, int n) {
  std::vector<int> order(n);
  std::vector<double> cost(n);
  for (int i = 0; i < n; ++i) {
    order[i] = i;
    cost[i] = cost_per_ray(ps[i]);
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  return order;
}

// items (batch entries x tiles) of one instance
int64_t instance_items(const RenderParams& p, int shape) {
  const int tw = tile_w(shape), th = tile_h(shape);
  return int64_t(p.B) * ((p.W + tw - 1) / tw) * ((p.H + th - 1) / th);
}

template <int TF>
cudaError_t fwd_tf(const BatchForwardTable& t, int n_items, size_t smem, int vst, int filter, int blend,
                   cudaStream_t s) {
  switch (vst) {
    case kF16: return launch_fast_forward_batched_vt<TF, __half>(t, n_items, smem, filter, blend, s);
    case kBF16: return launch_fast_forward_batched_vt<TF, __nv_bfloat16>(t, n_items, smem, filter, blend, s);
    default: return launch_fast_forward_batched_vt<TF, float>(t, n_items, smem, filter, blend, s);
  }
}

template <int TF>
cudaError_t adj_tf(const BatchAdjointTable& t, int n_items, size_t smem, int vst, int filter, int blend, bool vg,
                   bool tg, cudaStream_t s) {
  switch (vst) {
    case kF16: return launch_fast_adjoint_batched_vt<TF, __half>(t, n_items, smem, filter, blend, vg, tg, s);
    case kBF16: return launch_fast_adjoint_batched_vt<TF, __nv_bfloat16>(t, n_items, smem, filter, blend, vg, tg, s);
    default: return launch_fast_adjoint_batched_vt<TF, float>(t, n_items, smem, filter, blend, vg, tg, s);
  }
}

std::mutex g_counter_mutex;
int* g_counters[64] = {};
unsigned g_counter_next[64] = {};
constexpr unsigned kCounters = 4096;
constexpr unsigned kCounterInts = 4;  // 16 bytes per launch

struct ScratchSlot {
  int device = -1;
  cudaStream_t stream = nullptr;
  int slot = 0;
  void* ptr = nullptr;
  size_t bytes = 0;
};
std::mutex g_scratch_mutex;
std::vector<ScratchSlot> g_scratch;

struct GatherTextureSlot {
  int device = -1;
  cudaStream_t stream = nullptr;
  int W = 0, H = 0, format = -1;
  cudaArray_t array = nullptr;
  cudaTextureObject_t tex = 0;
  cudaSurfaceObject_t surf = 0;  // 0 when the array could not take surface stores
};
std::mutex g_texture_mutex;
std::vector<GatherTextureSlot> g_textures;

}  // namespace

void* acquire_scratch(int device, cudaStream_t s, size_t bytes, cudaError_t& err, int which) {
  err = cudaSuccess;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  ScratchSlot* slot = nullptr;
  for (auto& e : g_scratch)
    if (e.device == device && e.stream == s && e.slot == which) slot = &e;
  if (!slot) {
    g_scratch.push_back(ScratchSlot{device, s, which, nullptr, 0});
    slot = &g_scratch.back();
  }
  if (slot->bytes < bytes) {
    if (slot->ptr) {
      // earlier launches on this stream may still use the old buffer
      err = cudaStreamSynchronize(s);
      if (err != cudaSuccess) return nullptr;
      cudaFree(slot->ptr);
      slot->ptr = nullptr;
      slot->bytes = 0;
    }
    const size_t want = std::max(bytes, size_t(1) << 20);
    err = cudaMalloc(&slot->ptr, want);
    if (err != cudaSuccess) return nullptr;
    slot->bytes = want;
  }
  return slot->ptr;
}

cudaError_t acquire_gather_texture(int device, cudaStream_t s, int W, int H, int format, cudaArray_t& array,
                                   cudaTextureObject_t& tex, cudaSurfaceObject_t& surf) {
  std::lock_guard<std::mutex> lock(g_texture_mutex);
  GatherTextureSlot* slot = nullptr;
  for (auto& e : g_textures)
    if (e.device == device && e.stream == s) slot = &e;
  if (!slot) {
    g_textures.push_back(GatherTextureSlot{device, s});
    slot = &g_textures.back();
  }
  if (slot->array && (slot->W != W || slot->H != H || slot->format != format)) {
    // earlier launches on this stream may still read the old texture
    const cudaError_t err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return err;
    cudaDestroyTextureObject(slot->tex);
    if (slot->surf) cudaDestroySurfaceObject(slot->surf);
    cudaFreeArray(slot->array);
    slot->array = nullptr;
    slot->tex = 0;
    slot->surf = 0;
  }
  if (!slot->array) {
    // texel formats of TexelFormat (dvr_cells.cuh): 0 float, 1 half, 2 raw 16-bit
    const cudaChannelFormatDesc desc = format == 0   ? cudaCreateChannelDesc<float>()
                                       : format == 1 ? cudaCreateChannelDescHalf()
                                                     : cudaCreateChannelDesc<unsigned short>();
    // with surface stores the slab image is written into the array
    // directly; where gather and surface flags do not combine, through a
    // staging image and a copy
    bool surface = true;
    cudaError_t err = cudaMallocArray(&slot->array, &desc, size_t(W), size_t(H),
                                      cudaArrayTextureGather | cudaArraySurfaceLoadStore);
    if (err != cudaSuccess) {
      (void)cudaGetLastError();  // the refused combination is not an error of the call
      surface = false;
      err = cudaMallocArray(&slot->array, &desc, size_t(W), size_t(H), cudaArrayTextureGather);
    }
    if (err != cudaSuccess) {
      slot->array = nullptr;
      return err;
    }
    cudaResourceDesc res{};
    res.resType = cudaResourceTypeArray;
    res.res.array.array = slot->array;
    if (surface && cudaCreateSurfaceObject(&slot->surf, &res) != cudaSuccess) {
      (void)cudaGetLastError();
      slot->surf = 0;
    }
    cudaTextureDesc td{};
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    err = cudaCreateTextureObject(&slot->tex, &res, &td, nullptr);
    if (err != cudaSuccess) {
      if (slot->surf) cudaDestroySurfaceObject(slot->surf);
      cudaFreeArray(slot->array);
      slot->array = nullptr;
      slot->tex = 0;
      slot->surf = 0;
      return err;
    }
    slot->W = W;
    slot->H = H;
    slot->format = format;
  }
  array = slot->array;
  tex = slot->tex;
  surf = slot->surf;
  return cudaSuccess;
}

int* acquire_counter(int device, cudaStream_t s, cudaError_t& err) {
  err = cudaSuccess;
  int* c = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_counter_mutex);
    const int d = device & 63;
    if (!g_counters[d]) {
      err = cudaMalloc(&g_counters[d], kCounters * kCounterInts * sizeof(int));
      if (err != cudaSuccess) return nullptr;
    }
    // launches in flight at the same time get different counters as long as
    // fewer than kCounters of them overlap
    c = g_counters[d] + (g_counter_next[d]++ % kCounters) * kCounterInts;
  }
  err = cudaMemsetAsync(c, 0, kCounterInts * sizeof(int), s);
  return err == cudaSuccess ? c : nullptr;
}

cudaError_t launch_batched_forward(const RenderParams* ps, const unsigned char* shapes, int n, int filter, int tf_mode,
                                   int blend, int, const LaunchInfo&, cudaStream_t s) {
  const std::vector<int> order = cost_order(ps, n);
  for (int first = 0; first < n; first += kBatchMax) {
    BatchForwardTable t{};
    t.n = std::min(kBatchMax, n - first);
    int64_t items = 0;
    size_t smem = 0;
    for (int j = 0; j < t.n; ++j) {
      const RenderParams& p = ps[order[first + j]];
      t.p[j] = p;
      t.shape[j] = shapes[order[first + j]];
      items += instance_items(p, t.shape[j]);
      if (items > 0x7fffffff) return cudaErrorInvalidConfiguration;
      t.item_end[j] = int(items);
      smem = std::max(smem, size_t(p.R) * p.C * sizeof(float));
    }
    if (items == 0) continue;
    cudaError_t e;
    switch (tf_mode) {
      case 0: e = fwd_tf<0>(t, int(items), smem, t.p[0].vol_storage, filter, blend, s); break;
      case 1: e = fwd_tf<1>(t, int(items), smem, t.p[0].vol_storage, filter, blend, s); break;
      case 2: e = fwd_tf<2>(t, int(items), smem, t.p[0].vol_storage, filter, blend, s); break;
      default: e = fwd_tf<3>(t, int(items), smem, t.p[0].vol_storage, filter, blend, s); break;
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_batched_adjoint(const RenderParams* ps, const AdjointParams* as, const unsigned char* shapes, int n,
                                   int filter, int tf_mode, int blend, int, const LaunchInfo&, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const std::vector<int> order = cost_order(ps, n);
  const bool tg = as[0].has_tf != 0, vg = as[0].has_volume != 0;
  for (int first = 0; first < n; first += kBatchMax) {
    BatchAdjointTable t{};
    t.n = std::min(kBatchMax, n - first);
    int64_t items = 0;
    size_t smem = 0;
    for (int j = 0; j < t.n; ++j) {
      const int i = order[first + j];
      t.p[j] = ps[i];
      t.a[j] = as[i];
      t.shape[j] = shapes[i];
      items += instance_items(ps[i], t.shape[j]);
      if (items > 0x7fffffff) return cudaErrorInvalidConfiguration;
      t.item_end[j] = int(items);
      const int seg = ps[i].ckpt.p ? ps[i].ckpt_interval : 0;
      smem = std::max(smem, fast_adjoint_smem(tf_mode, ps[i].R, ps[i].C, tg, seg));
    }
    if (items == 0) continue;
    cudaError_t e;
    switch (tf_mode) {
      case 0: e = adj_tf<0>(t, int(items), smem, t.p[0].vol_storage, filter, blend, vg, tg, s); break;
      case 1: e = adj_tf<1>(t, int(items), smem, t.p[0].vol_storage, filter, blend, vg, tg, s); break;
      case 2: e = adj_tf<2>(t, int(items), smem, t.p[0].vol_storage, filter, blend, vg, tg, s); break;
      default: e = adj_tf<3>(t, int(items), smem, t.p[0].vol_storage, filter, blend, vg, tg, s); break;
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace dvr
